/*
 * ORACLE / TEST INFRASTRUCTURE ONLY (see oracle/README.md).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load this; the
 * product never does.
 *
 * CPU restatement of the reference's photon transport for voxelized media
 * (bulk method 2) and of its two-phase fluorescence driver, written from the
 * reference's behaviour:
 *   launch_photon          LaunchPhoton          CUDAMCFLtransport.cu:460-562
 *   step                   MCd3D loop body       CUDAMCFLtransport.cu:286-447
 *   move_to_first_boundary MoveToFirstBoundary   CUDAMCFLtransport.cu:702-847
 *   reflect                Reflect (method 2)    CUDAMCFLtransport.cu:628-700
 *   spin                   Spin                  CUDAMCFLtransport.cu:585-625
 *   photon_survive         PhotonSurvive         CUDAMCFLtransport.cu:850-864
 *   Rng                    rand_MWC_co/oc        CUDAMCFLrng.cu:17-29
 *   init_rng_streams       init_RNG              CUDAMCFLrng.cu:31-90
 *   run_refstream          DoOneSimulation(Fl) + voxel loop  CUDAMCFLmain.cu:60-288,409-652
 *   step_layers            MCd loop body (bulk method 1: layers and one
 *                          spherical inclusion)  CUDAMCFLtransport.cu:73-233
 *
 * Every floating-point expression keeps the reference's operand order and
 * types (including its double-precision literals), so each rounding happens
 * where it happens in the reference.  The file is compiled without
 * contraction.  Two knobs:
 *   math   libm         __logf/__cosf/__sincosf as the C library computes them
 *                       (what the host build of the reference uses), or
 *          portable     the series of portable_math.h (what the CUDA engine's
 *                       exact-math kernel uses);
 *   rng    refstream    32768 per-thread streams and the reference's
 *                       relaunch schedule, or
 *          photon       one stream per photon index (the engine's scheme).
 * refstream+libm reproduces the host build of the reference bit for bit;
 * photon+portable reproduces the engine's exact-math kernel bit for bit.
 *
 * Where the reference indexes past an array when a coordinate rounds onto the
 * far edge of the grid or detector, the linear index is clamped to the last
 * element (the engine does the same); so is a time bin that rounds onto the
 * end of the histogram.  The reference converts time-of-flight increments
 * from double to unsigned long; a glass voxel's back-projection, and the
 * first step after it when it left the photon outside the slab, can make that
 * value negative, which C leaves undefined.  The GPU saturates it to 0 (the
 * engine does the same); the reference's x86-64 host build wraps it modulo
 * 2^64.  refstream+libm follows the host build (so that it stays bit-identical
 * to it), every other mode the GPU.
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

#include "oracle_api.h"
#include "portable_math.h"

namespace {

const unsigned kThreadsPerBlock = 256;   /* CUDAMCFL.h:18 */
const unsigned kBlocks = 128;            /* CUDAMCFL.h:19 */
const unsigned kThreads = kThreadsPerBlock * kBlocks;
const unsigned kStepsPerLaunch = 80000;  /* CUDAMCFL.h:21 */
const float kPi = 3.141592654f;          /* CUDAMCFL.h:22 */
const unsigned kWeightRoulette = 429497u; /* CUDAMCFL.h:33 */
const float kChance = 0.1f;              /* CUDAMCFL.h:34 */
const double kCcmfs = 2.99792E-5;        /* speed of light [cm/fs], CUDAMCFL.h:29 */

/* (unsigned long)(v) for a double: saturating as the GPU converts, or
 * wrapping negative values modulo 2^64 as the x86-64 host build does. */
inline uint64_t tof_u64(double v, int host_wrap) {
  if (host_wrap && v < 9223372036854775808.0) return (uint64_t)(int64_t)v;
  if (!(v > 0.0)) return 0;
  if (v >= 18446744073709551616.0) return 0xFFFFFFFFFFFFFFFFull;
  return (uint64_t)v;
}

struct LibmMath {
  static const int kHost = 1; /* the host build's library and conversions */
  static float log(float x) { return logf(x); }
  static float cos(float x) { return cosf(x); }
  static void sincos(float x, float *s, float *c) { *s = sinf(x); *c = cosf(x); }
};

struct PortableMath {
  static const int kHost = 0;
  static float log(float x) { return mcfl_plogf(x); }
  static float cos(float x) { return mcfl_pcosf(x); }
  static void sincos(float x, float *s, float *c) { mcfl_psincosf(x, s, c); }
};

struct Rng {
  uint64_t x;
  uint32_t a;
  float co() { /* [0,1) */
    x = (x & 0xffffffffull) * a + (x >> 32);
    return mcfl_u2f_rz((uint32_t)x) / 4294967296.0f;
  }
  float oc() { return 1.0f - co(); } /* (0,1] */
};

struct Prop {
  float mutr, mua, g, n;
};

struct Photon {
  float x, y, z, dx, dy, dz;
  uint32_t weight;
  uint32_t bulkpos;
  uint64_t tof; /* time of flight [fs] */
  /* voxel-boundary stepping: the photon's voxel (lateral indices beyond the
   * grid name virtual voxels of label 1) */
  int ix, iy, iz;
};

/* Everything one transport phase reads (the reference's __constant__ set). */
struct Phase {
  float esp;
  float hx, hy;     /* half lateral extents (2*esp in the reference) */
  float gx, gy, gz; /* voxels per cm (grid_size in the reference) */
  unsigned num_x, num_y, num_z;
  unsigned total;
  float size_x, size_y;
  float det_dx, det_dy, det_x0, det_y0;
  int det_nx;
  unsigned xy_size;
  unsigned last_bulk;
  Prop prop[ORACLE_MAX_BULKS + 2];
  const short *labels;
  /* voxel-boundary stepping: each voxel's free radius (see free_radius) */
  const unsigned char *free_r;
  int fhd_on;
  float xi, yi, zi, dir;
  uint32_t start_weight;
  int guard; /* reproduce the reference's non-atomic overflow guards */
  int launch_rng_reuse;
  /* time-resolved detectors (excitation phase) */
  int tof_wrap; /* host-build conversion of negative time increments (see the file comment) */
  int time_on;
  int tdet_face;
  unsigned tnx, tny;
  long tbins;
  uint64_t tmax;
  float tdet_r;
  const float *tposx, *tposy;
  /* bulk method 1: slabs 1..n_layers between the outer media 0 and
   * n_layers+1, one spherical inclusion; the photon's bulkpos is its layer */
  int method;
  unsigned n_layers;
  oracle_layer layers[ORACLE_MAX_LAYERS + 2];
  oracle_inclusion incl;
  uint32_t start_layer;
  int exact; /* voxel-boundary stepping (photon mode, voxelized media) */
};

inline unsigned voxel_index(const Phase &ph, float x, float y, float z) {
  unsigned idx = mcfl_f2u_rz((x + ph.hx) * ph.gx) +
                 ph.num_x * (mcfl_f2u_rz((y + ph.hy) * ph.gy) + ph.num_y * mcfl_f2u_rz(z * ph.gz));
  return idx < ph.total ? idx : ph.total - 1;
}

inline unsigned pixel_index(const Phase &ph, float x, float y) {
  unsigned idx = mcfl_f2u_rz((y - ph.det_y0 + ph.size_y) / ph.det_dy) * (unsigned)ph.det_nx +
                 mcfl_f2u_rz((x - ph.det_x0 + ph.size_x) / ph.det_dx);
  return idx < ph.xy_size ? idx : ph.xy_size - 1;
}

inline uint32_t start_label(const Phase &ph, const Photon &p) {
  if (p.z < ph.esp) {
    if (fabsf(p.x) < ph.hx && fabsf(p.y) < ph.hy) return (uint32_t)ph.labels[voxel_index(ph, p.x, p.y, p.z)];
    return 1;
  }
  return ph.last_bulk;
}

/* kSingle: the engine's all-single-precision isotropic launch (1 - 2u and
 * 2 PI u are bit-identical either way; the square root of 1 - cos^2 theta is
 * a single-precision square root instead of a rounded double one). */
template <class M, bool kSingle = false>
void launch_photon(Photon &p, Rng &r, const Phase &ph, float xi, float yi, float zi) {
  if (ph.dir == 0.0f) {
    p.x = xi + (0.999999f / ph.gx) * r.oc();
    p.y = yi + (0.999999f / ph.gy) * r.oc();
    p.z = zi + (0.999999f / ph.gz) * r.oc();
    float costheta, sintheta, psi;
    if (kSingle) {
      costheta = 1.0f - 2.0f * r.oc();
      sintheta = sqrtf(1.0f - costheta * costheta);
      psi = (2.0f * kPi) * r.oc();
    } else {
      costheta = (float)(1.0 - 2.0 * (double)r.oc());
      sintheta = (float)sqrt(1.0 - (double)(costheta * costheta));
      psi = (float)(2.0 * (double)kPi * (double)r.oc());
    }
    float cospsi = M::cos(psi);
    float sinpsi;
    const float sin2 = kSingle ? 1.0f - cospsi * cospsi : (float)(1.0 - (double)(cospsi * cospsi));
    if (psi < kPi)
      sinpsi = sqrtf(sin2);
    else
      sinpsi = -sqrtf(sin2);
    p.dx = sintheta * cospsi;
    p.dy = sintheta * sinpsi;
    p.dz = costheta;
    p.weight = 0xFFFFFFFFu;
  } else {
    const float input_fibre_diameter = (float)0.03;
    float sample_rad = input_fibre_diameter * sqrtf(-M::log(r.oc()));
    float sample_phi = 2 * kPi * r.oc();
    float sin_phi, cos_phi;
    M::sincos(sample_phi, &sin_phi, &cos_phi);
    p.x = xi + sample_rad * cos_phi;
    p.y = yi + sample_rad * sin_phi;
    p.z = zi;
    p.dx = 0.0f;
    p.dy = 0.0f;
    p.dz = 1.0f;
    p.weight = ph.start_weight;
  }
  p.bulkpos = ph.method == 1 ? ph.start_layer : start_label(ph, p);
  p.tof = 0;
}

template <class M>
void spin(Photon &p, float g, Rng &r) {
  float cost, sint, cosp, sinp, temp;
  float tempdir = p.dx;
  temp = (1.0f - g * g) / (1.0f - g + 2.0f * g * r.co());
  cost = (1.0f + g * g - temp * temp) / (2.0f * g);
  if (g == 0.0f) cost = 2.0f * r.co() - 1.0f;
  sint = sqrtf(1.0f - cost * cost);
  /* The reference passes (&cosp, &sinp) as (sin, cos) outputs
   * (CUDAMCFLtransport.cu:603): cosp holds sin(psi), sinp holds cos(psi). */
  M::sincos(2.0f * kPi * r.co(), &cosp, &sinp);
  temp = sqrtf(1.0f - p.dz * p.dz);
  if (temp == 0.0f) {
    p.dx = sint * cosp;
    p.dy = sint * sinp;
    p.dz = copysignf(cost, p.dz * cost);
  } else {
    p.dx = (sint * (p.dx * p.dz * cosp - p.dy * sinp)) / temp + p.dx * cost;
    p.dy = (sint * (p.dy * p.dz * cosp + tempdir * sinp)) / temp + p.dy * cost;
    p.dz = -sint * cosp * temp + p.dz * cost;
  }
  temp = 1.0f / sqrtf(p.dx * p.dx + p.dy * p.dy + p.dz * p.dz);
  p.dx = p.dx * temp;
  p.dy = p.dy * temp;
  p.dz = p.dz * temp;
}

/* Returns 1 when reflected. */
inline unsigned reflect(Photon &p, uint32_t newlb, Rng &r, const Phase &ph) {
  float n1 = ph.prop[p.bulkpos].n, n2 = ph.prop[newlb].n;
  float rr;
  float cos_angle_i = fabsf(p.dz);
  if (n1 == n2) {
    p.bulkpos = newlb;
    return 0u;
  }
  if (n2 * n2 < n1 * n1 * (1 - cos_angle_i * cos_angle_i)) {
    p.dz *= -1.0f;
    return 1u;
  }
  if (cos_angle_i == 1.0f) {
    rr = (n1 - n2) / (n1 + n2);
    if (r.co() <= rr * rr) {
      p.dz *= -1.0f;
      return 1u;
    }
    p.bulkpos = newlb;
    return 0u;
  }
  float e = (n1 * n1) / (n2 * n2) * (1.0f - cos_angle_i * cos_angle_i);
  rr = 2 * sqrtf((1.0f - cos_angle_i * cos_angle_i) * (1.0f - e) * e * cos_angle_i * cos_angle_i);
  e = e + (cos_angle_i * cos_angle_i) * (1.0f - 2.0f * e);
  rr = e * ((1.0f - e - rr) / ((1.0f - e + rr) * (e + rr)));
  if (r.co() <= rr) {
    p.dz *= -1.0f;
    return 1u;
  }
  rr = n1 / n2;
  e = rr * rr * (1.0f - cos_angle_i * cos_angle_i);
  p.dx *= rr;
  p.dy *= rr;
  p.dz = copysignf(sqrtf(1 - e), p.dz);
  p.bulkpos = newlb;
  return 0u;
}

/* Reflect of bulk method 1: the layers' refractive indices, the layer
 * changes on transmission.  Returns 1 when reflected. */
inline unsigned reflect_layers(Photon &p, uint32_t newl, Rng &r, const Phase &ph) {
  const float n1 = ph.layers[p.bulkpos].n, n2 = ph.layers[newl].n;
  float rr;
  float cos_angle_i = fabsf(p.dz);
  if (n1 == n2) {
    p.bulkpos = newl;
    return 0u;
  }
  if (n2 * n2 < n1 * n1 * (1 - cos_angle_i * cos_angle_i)) {
    p.dz *= -1.0f;
    return 1u;
  }
  if (cos_angle_i == 1.0f) {
    rr = (n1 - n2) / (n1 + n2);
    if (r.co() <= rr * rr) {
      p.dz *= -1.0f;
      return 1u;
    }
    p.bulkpos = newl;
    return 0u;
  }
  float e = (n1 * n1) / (n2 * n2) * (1.0f - cos_angle_i * cos_angle_i);
  rr = 2 * sqrtf((1.0f - cos_angle_i * cos_angle_i) * (1.0f - e) * e * cos_angle_i * cos_angle_i);
  e = e + (cos_angle_i * cos_angle_i) * (1.0f - 2.0f * e);
  rr = e * ((1.0f - e - rr) / ((1.0f - e + rr) * (e + rr)));
  if (r.co() <= rr) {
    p.dz *= -1.0f;
    return 1u;
  }
  rr = n1 / n2;
  e = rr * rr * (1.0f - cos_angle_i * cos_angle_i);
  p.dx *= rr;
  p.dy *= rr;
  p.dz = copysignf(sqrtf(1 - e), p.dz);
  p.bulkpos = newl;
  return 0u;
}

/* March through a scattering-free ("glass") voxel in half-voxel steps until
 * the label changes, then back-project onto the sphere of radius 0.707 voxel
 * around the centre of the voxel reached. */
inline uint32_t move_to_first_boundary(Photon &p, uint32_t old_bulk, const Phase &ph, float max_s) {
  const unsigned num_x = ph.num_x, num_y = ph.num_y;
  const float gf = ph.gx;
  float search_step = 1 / (2 * gf);
  float total_move = 0;
  int index = 1;
  uint32_t present_bulk = old_bulk;
  while (present_bulk == old_bulk && total_move < max_s) {
    p.x += p.dx * search_step;
    p.y += p.dy * search_step;
    p.z += p.dz * search_step;
    p.tof += tof_u64(search_step / kCcmfs, ph.tof_wrap);
    if (p.z + p.dz * search_step < 0.0f) {
      present_bulk = 0;
      index = -1;
      search_step = (-p.z) / p.dz;
    } else if (p.z + p.dz * search_step > ph.esp) {
      present_bulk = ph.last_bulk;
      index = -1;
      search_step = (ph.esp - p.z) / p.dz;
    } else if (fabsf(p.x + p.dx * search_step) >= ph.hx || fabsf(p.y + p.dy * search_step) >= ph.hy) {
      present_bulk = 1;
      index = -1;
    } else {
      index = (int)voxel_index(ph, p.x, p.y, p.z);
      present_bulk = (uint32_t)(unsigned short)ph.labels[index];
    }
    total_move += search_step;
  }
  if (index >= 0 && present_bulk != old_bulk) {
    unsigned uidx = (unsigned)index;
    unsigned z_grid = uidx / (num_x * num_y);
    uidx -= z_grid * num_x * num_y;
    unsigned y_grid = uidx / num_x;
    unsigned x_grid = uidx % num_x;
    const double half = 1. / (2. * (double)ph.gx);
    float y_voxel = (float)((double)(mcfl_i2f_rn((int)y_grid) / ph.gy - ph.hy) + half);
    float x_voxel = (float)((double)(mcfl_i2f_rn((int)x_grid) / ph.gx - ph.hx) + half);
    float z_voxel = (float)((double)(mcfl_i2f_rn((int)z_grid) / ph.gz) + half);
    const double rv = 0.707107 * (double)(1 / gf);
    float r_voxel2 = (float)(rv * rv);
    float pow_dx = p.dx * p.dx, pow_dy = p.dy * p.dy, pow_dz = p.dz * p.dz;
    float pow_px = p.x * p.x, pow_py = p.y * p.y, pow_pz = p.z * p.z;
    float pow_cx = x_voxel * x_voxel, pow_cy = y_voxel * y_voxel, pow_cz = z_voxel * z_voxel;
    float disc = 2 * x_voxel * y_voxel * p.dx * p.dy - (pow_cy + pow_cz) * pow_dx - (pow_cx + pow_cz) * pow_dy -
                 (pow_cx + pow_cy) * pow_dz - (pow_dy + pow_dz) * pow_px - (pow_dx + pow_dz) * pow_py -
                 (pow_dx + pow_dy) * pow_pz + (pow_dx + pow_dy + pow_dz) * r_voxel2 +
                 2 * (x_voxel * z_voxel * p.dx + y_voxel * z_voxel * p.dy) * p.dz -
                 2 * (y_voxel * p.dx * p.dy - x_voxel * pow_dy + z_voxel * p.dx * p.dz - x_voxel * pow_dz) * p.x +
                 2 * (y_voxel * pow_dx - x_voxel * p.dx * p.dy - z_voxel * p.dy * p.dz + y_voxel * pow_dz +
                      p.dx * p.dy * p.x) * p.y +
                 2 * (z_voxel * pow_dx + z_voxel * pow_dy + p.dx * p.dz * p.x + p.dy * p.dz * p.y -
                      (x_voxel * p.dx + y_voxel * p.dy) * p.dz) * p.z;
    float root = sqrtf(disc);
    float lin = x_voxel * p.dx + y_voxel * p.dy + z_voxel * p.dz - p.dx * p.x - p.dy * p.y - p.dz * p.z;
    float den = pow_dx + pow_dy + pow_dz;
    float back_step1 = -(lin + root) / den;
    float back_step2 = -(lin - root) / den;
    float new_px1 = p.x - p.dx * back_step1, new_py1 = p.y - p.dy * back_step1, new_pz1 = p.z - p.dz * back_step1;
    float new_px2 = p.x - p.dx * back_step2, new_py2 = p.y - p.dy * back_step2, new_pz2 = p.z - p.dz * back_step2;
    if (((new_px1 - x_voxel) * (new_px1 - x_voxel) + (new_py1 - y_voxel) * (new_py1 - y_voxel) +
         (new_pz1 - z_voxel) * (new_pz1 - z_voxel)) <
        ((new_px2 - x_voxel) * (new_px2 - x_voxel) + (new_py2 - y_voxel) * (new_py2 - y_voxel) +
         (new_pz2 - z_voxel) * (new_pz2 - z_voxel))) {
      p.x = new_px1; p.y = new_py1; p.z = new_pz1;
      p.tof -= tof_u64(back_step1 / kCcmfs, ph.tof_wrap);
    } else {
      p.x = new_px2; p.y = new_py2; p.z = new_pz2;
      p.tof -= tof_u64(back_step2 / kCcmfs, ph.tof_wrap);
    }
  }
  return present_bulk;
}

inline unsigned photon_survive(Photon &p, Rng &r, uint64_t *gain, uint64_t *loss) {
  if (p.weight > kWeightRoulette) return 1u;
  if (p.weight == 0u) return 0u;
  if (r.co() < kChance) {
    uint32_t w0 = p.weight;
    p.weight = mcfl_f2u_rn(mcfl_u2f_rn(p.weight) / kChance);
    *gain += (uint64_t)(p.weight - w0);
    return 1u;
  }
  *loss += p.weight;
  return 0u;
}

inline void add_guarded(unsigned long long *t, uint32_t w, int guard) {
  if (!guard) {
    __atomic_fetch_add(t, (unsigned long long)w, __ATOMIC_RELAXED);
  } else if (*t + w < (unsigned long long)LLONG_MAX) {
    __atomic_fetch_add(t, (unsigned long long)w, __ATOMIC_RELAXED);
  }
}

/* Where a phase's tallies go.  exit_img: image for an exit through the top
 * (R) or the bottom (T); the emission phase of the photon-indexed variant
 * weights exits with the emitting voxel's fixed-point factor instead. */
struct Sink {
  unsigned long long *Rd = nullptr, *Tt = nullptr, *fhd = nullptr, *time_xyt = nullptr;
  unsigned long long *R128 = nullptr, *T128 = nullptr; /* lo,hi pairs */
  uint64_t voxel_q = 0;
  uint64_t absorbed = 0, exit_top = 0, exit_bottom = 0, r_loss = 0, r_gain = 0, w0_loss = 0, steps = 0;
};

inline void add128(unsigned long long *acc, uint32_t w, uint64_t q) {
  unsigned __int128 prod = (unsigned __int128)w * q;
  uint64_t lo = (uint64_t)prod, hi = (uint64_t)(prod >> 64);
  uint64_t old = __atomic_fetch_add(&acc[0], lo, __ATOMIC_RELAXED);
  uint64_t carry = (old + lo < old) ? 1u : 0u;
  if (hi + carry) __atomic_fetch_add(&acc[1], hi + carry, __ATOMIC_RELAXED);
}

/* Time-resolved detectors at an exit through the detector array's face
 * (CUDAMCFLtransport.cu:379-390,406-417): every disc that contains the exit
 * point gets the weight in the photon's time bin. */
inline void tally_time(const Phase &ph, const Photon &p, Sink &sk) {
  if (!(p.tof < ph.tmax)) return;
  for (unsigned xpos = 0; xpos < ph.tnx; xpos++)
    for (unsigned ypos = 0; ypos < ph.tny; ypos++) {
      if (((p.x - ph.tposx[xpos]) * (p.x - ph.tposx[xpos]) + (p.y - ph.tposy[ypos]) * (p.y - ph.tposy[ypos])) <
          (ph.tdet_r * ph.tdet_r)) {
        unsigned bin = mcfl_f2u_rz(((float)p.tof / (float)ph.tmax) * (float)ph.tbins);
        if ((long)bin >= ph.tbins) bin = (unsigned)(ph.tbins - 1);
        const size_t idx = xpos + (size_t)ph.tnx * (ypos + (size_t)ph.tny * bin);
        add_guarded(&sk.time_xyt[idx], p.weight, ph.guard);
      }
    }
}

/* One pass of the MCd3D loop body up to the survival test.  Returns 1 while
 * the photon lives. */
template <class M>
unsigned step(Photon &p, Rng &r, const Phase &ph, Sink &sk) {
  float s;
  uint32_t new_bulk;
  const uint32_t last_bulk = ph.last_bulk;
  sk.steps++;
  if (ph.prop[p.bulkpos].mutr != FLT_MAX) {
    s = -M::log(r.oc()) * ph.prop[p.bulkpos].mutr;
    new_bulk = p.bulkpos;
    if (p.z + s * p.dz < 0.0f) {
      new_bulk = 0;
      s = (-p.z) / p.dz;
    }
    if (p.z + s * p.dz > ph.esp) {
      new_bulk = last_bulk;
      s = (ph.esp - p.z) / p.dz;
    }
    p.x += p.dx * s;
    p.y += p.dy * s;
    p.z += p.dz * s;
    p.tof += tof_u64((double)(s * ph.prop[p.bulkpos].n) / kCcmfs, ph.tof_wrap);
    if (new_bulk != 0 && new_bulk != last_bulk) {
      if (fabsf(p.x) < ph.hx && fabsf(p.y) < ph.hy && p.z < ph.esp)
        new_bulk = (uint32_t)(unsigned short)ph.labels[voxel_index(ph, p.x, p.y, p.z)];
      else
        new_bulk = 1;
    }
  } else {
    s = 100.0f;
    new_bulk = move_to_first_boundary(p, p.bulkpos, ph, s);
  }
  if (new_bulk != p.bulkpos) reflect(p, new_bulk, r, ph);
  if (fabsf(p.x) < ph.hx && fabsf(p.y) < ph.hy && p.z < ph.esp && ph.fhd_on == 1)
    add_guarded(&sk.fhd[voxel_index(ph, p.x, p.y, p.z)], p.weight, ph.guard);
  if (p.bulkpos == 0) {
    if (fabsf(p.x - ph.det_x0) < ph.size_x && fabsf(p.y - ph.det_y0) < ph.size_y) {
      unsigned idx = pixel_index(ph, p.x, p.y);
      if (sk.R128) add128(&sk.R128[2 * (size_t)idx], p.weight, sk.voxel_q);
      else add_guarded(&sk.Rd[idx], p.weight, ph.guard);
    }
    if (ph.time_on && ph.tdet_face == 0) tally_time(ph, p, sk);
    sk.exit_top += p.weight;
    p.weight = 0u;
    s = 0.0f;
  }
  if (p.bulkpos == last_bulk) {
    if (fabsf(p.x - ph.det_x0) < ph.size_x && fabsf(p.y - ph.det_y0) < ph.size_y) {
      unsigned idx = pixel_index(ph, p.x, p.y);
      if (sk.T128) add128(&sk.T128[2 * (size_t)idx], p.weight, sk.voxel_q);
      else add_guarded(&sk.Tt[idx], p.weight, ph.guard);
    }
    if (ph.time_on && ph.tdet_face == 1) tally_time(ph, p, sk);
    sk.exit_bottom += p.weight;
    p.weight = 0u;
    s = 0.0f;
  }
  if (s > 0.0f) {
    const Prop &pr = ph.prop[p.bulkpos];
    uint32_t w = mcfl_f2u_ru(pr.mua * pr.mutr * mcfl_u2f_rn(p.weight));
    if (w > 0) {
      p.weight -= w;
      sk.absorbed += w;
    } else {
      sk.w0_loss += p.weight;
      p.weight = 0u;
    }
    spin<M>(p, pr.g, r);
  }
  return photon_survive(p, r, &sk.r_gain, &sk.r_loss);
}

inline bool in_inclusion(const Phase &ph, const Photon &p) {
  const oracle_inclusion &c = ph.incl;
  return ((p.x - c.x) * (p.x - c.x) + (p.y - c.y) * (p.y - c.y) + (p.z - c.z) * (p.z - c.z)) <= (c.r * c.r);
}

/* One pass of the MCd loop body (bulk method 1).  Kept as the reference
 * runs it: outside the inclusion the step is 1/mu_t itself, not a sampled
 * -ln(u)/mu_t (CUDAMCFLtransport.cu:87-89); a scattering-free layer or
 * inclusion steps 2 cm; the weight drop rounds to nearest and never kills. */
template <class M>
unsigned step_layers(Photon &p, Rng &r, const Phase &ph, Sink &sk) {
  float s;
  const oracle_layer &L = ph.layers[p.bulkpos];
  sk.steps++;
  if (in_inclusion(ph, p)) {
    if (ph.incl.mutr != FLT_MAX) s = -M::log(r.oc()) * ph.incl.mutr;
    else s = 2.0f;
  } else {
    if (L.mutr != FLT_MAX) s = L.mutr;
    else s = 2.0f;
  }
  int new_layer = (int)p.bulkpos;
  if (p.z + s * p.dz < L.z_min) {
    new_layer--;
    s = (L.z_min - p.z) / p.dz;
  }
  if (p.z + s * p.dz >= L.z_max) {
    new_layer++;
    s = (L.z_max - p.z) / p.dz;
  }
  p.x += p.dx * s;
  p.y += p.dy * s;
  p.z += p.dz * s;
  p.tof += tof_u64((double)(s * L.n) / kCcmfs, ph.tof_wrap);
  if (p.z > L.z_max) p.z = L.z_max;
  if (p.z < L.z_min) p.z = L.z_min;
  if (ph.fhd_on == 1 && fabsf(p.x) < ph.hx && fabsf(p.y) < ph.hy && p.z < ph.esp)
    add_guarded(&sk.fhd[voxel_index(ph, p.x, p.y, p.z)], p.weight, ph.guard);
  if (new_layer != (int)p.bulkpos) {
    s = 0.0f;
    /* Reflect with the layers' indices (CUDAMCFLtransport.cu:636-638) */
    if (reflect_layers(p, (uint32_t)new_layer, r, ph) == 0u) {
      if (new_layer == 0) {
        if (fabsf(p.x - ph.det_x0) < ph.size_x && fabsf(p.y - ph.det_y0) < ph.size_y)
          add_guarded(&sk.Rd[pixel_index(ph, p.x, p.y)], p.weight, ph.guard);
        if (ph.time_on && ph.tdet_face == 0) tally_time(ph, p, sk);
        sk.exit_top += p.weight;
        p.weight = 0;
      }
      if (new_layer > (int)ph.n_layers) {
        if (fabsf(p.x - ph.det_x0) < ph.size_x && fabsf(p.y - ph.det_y0) < ph.size_y)
          add_guarded(&sk.Tt[pixel_index(ph, p.x, p.y)], p.weight, ph.guard);
        if (ph.time_on && ph.tdet_face == 1) tally_time(ph, p, sk);
        sk.exit_bottom += p.weight;
        p.weight = 0;
      }
    }
  }
  if (s > 0.0f) {
    if (in_inclusion(ph, p)) {
      const uint32_t w = mcfl_f2u_rn(ph.incl.mua * ph.incl.mutr * mcfl_u2f_rn(p.weight));
      p.weight -= w;
      sk.absorbed += w;
      spin<M>(p, ph.incl.g, r);
    } else {
      const oracle_layer &Lc = ph.layers[p.bulkpos];
      const uint32_t w = mcfl_f2u_rn(Lc.mua * Lc.mutr * mcfl_u2f_rn(p.weight));
      p.weight -= w;
      sk.absorbed += w;
      spin<M>(p, Lc.g, r);
    }
  }
  return photon_survive(p, r, &sk.r_gain, &sk.r_loss);
}

/* ------------------------- voxel-boundary stepping ------------------------ */

/* Largest free radius kept (the engine keeps the same). */
#define ORACLE_FREE_MAX 31

/* Voxel-boundary stepping: voxel (x, y) lies in the grid's lateral extent. */
inline bool in_grid(const Phase &ph, int x, int y) {
  return x >= 0 && x < (int)ph.num_x && y >= 0 && y < (int)ph.num_y;
}

/* The photon's voxel from its position, for voxel-boundary stepping: beyond
 * the grid's lateral extent the slab continues as virtual voxels of label 1
 * (the reference's medium there), so the lateral indices are any integers. */
inline void locate(Photon &p, const Phase &ph) {
  p.ix = (int)floorf((p.x + ph.hx) * ph.gx);
  p.iy = (int)floorf((p.y + ph.hy) * ph.gy);
  p.iz = std::min(std::max((int)floorf(p.z * ph.gz), 0), (int)ph.num_z - 1);
}

/* Label and free radius of voxel (x, y, z), z inside the slab: the grid's
 * map, or beyond the grid's lateral extent label 1 with the radius that keeps
 * its cube outside the grid. */
inline void region_of(const Phase &ph, int x, int y, int z, uint32_t &label, int &r) {
  if (in_grid(ph, x, y)) {
    const size_t q = (size_t)x + ph.num_x * ((size_t)y + ph.num_y * (size_t)z);
    label = (uint32_t)(unsigned short)ph.labels[q];
    r = ph.free_r[q];
  } else {
    const int dx = x < 0 ? -x : x - ((int)ph.num_x - 1);
    const int dy = y < 0 ? -y : y - ((int)ph.num_y - 1);
    label = 1;
    r = std::min(ORACLE_FREE_MAX, std::max(dx, dy) - 1);
  }
}

/* Fresnel reflection / refraction at a voxel face whose normal is axis a
 * (0, 1, 2 = x, y, z): the reference's Reflect with that axis in place of z.
 * Returns 1 when transmitted. */
inline unsigned refract_axis(Photon &p, int a, float n1, float n2, Rng &r) {
  float *d[3] = {&p.dx, &p.dy, &p.dz};
  float &dn = *d[a], &t1 = *d[(a + 1) % 3], &t2 = *d[(a + 2) % 3];
  float rr;
  const float cos_angle_i = fabsf(dn);
  if (n1 == n2) return 1u;
  if (n2 * n2 < n1 * n1 * (1 - cos_angle_i * cos_angle_i)) {
    dn *= -1.0f;
    return 0u;
  }
  if (cos_angle_i == 1.0f) {
    rr = (n1 - n2) / (n1 + n2);
    if (r.co() <= rr * rr) {
      dn *= -1.0f;
      return 0u;
    }
    return 1u;
  }
  float e = (n1 * n1) / (n2 * n2) * (1.0f - cos_angle_i * cos_angle_i);
  rr = 2 * sqrtf((1.0f - cos_angle_i * cos_angle_i) * (1.0f - e) * e * cos_angle_i * cos_angle_i);
  e = e + (cos_angle_i * cos_angle_i) * (1.0f - 2.0f * e);
  rr = e * ((1.0f - e - rr) / ((1.0f - e + rr) * (e + rr)));
  if (r.co() <= rr) {
    dn *= -1.0f;
    return 0u;
  }
  rr = n1 / n2;
  e = rr * rr * (1.0f - cos_angle_i * cos_angle_i);
  t1 *= rr;
  t2 *= rr;
  dn = copysignf(sqrtf(1 - e), dn);
  return 1u;
}

/* Distance along direction component d from coordinate c to plane b
 * (FLT_MAX when the photon does not move towards it), never negative. */
inline float plane_dist(float b, float c, float d) {
  if (d == 0.0f) return FLT_MAX;
  const float t = (b - c) / d;
  return t > 0.0f ? t : 0.0f;
}

/* Coordinate of face k of the grid along axis a (0, 1, 2 = x, y, z); the
 * z faces 0 and num_z are the slab faces themselves. */
inline float face_coord(const Phase &ph, int a, int k) {
  if (a == 0) return (float)k / ph.gx - ph.hx;
  if (a == 1) return (float)k / ph.gy - ph.hy;
  return k == 0 ? 0.0f : (k == (int)ph.num_z ? ph.esp : (float)k / ph.gz);
}

/* An exit through a slab face: the image tally. */
inline void exact_exit(Photon &p, const Phase &ph, Sink &sk, bool top) {
  if (fabsf(p.x - ph.det_x0) < ph.size_x && fabsf(p.y - ph.det_y0) < ph.size_y) {
    const unsigned idx = pixel_index(ph, p.x, p.y);
    if (top) {
      if (sk.R128) add128(&sk.R128[2 * (size_t)idx], p.weight, sk.voxel_q);
      else add_guarded(&sk.Rd[idx], p.weight, ph.guard);
    } else {
      if (sk.T128) add128(&sk.T128[2 * (size_t)idx], p.weight, sk.voxel_q);
      else add_guarded(&sk.Tt[idx], p.weight, ph.guard);
    }
  }
  if (ph.time_on && ph.tdet_face == (top ? 0 : 1)) tally_time(ph, p, sk);
  (top ? sk.exit_top : sk.exit_bottom) += p.weight;
  p.weight = 0u;
}

/* One pass with voxel-boundary stepping: an optical depth -ln(u) is spent
 * voxel by voxel with each voxel's mu_t, the label is taken where the photon
 * is, Fresnel acts at every face between different indices with that face's
 * normal, scattering-free voxels are crossed without interaction.  The pass
 * ends at the interaction (PHD tally, weight drop and spin as the reference's
 * pass) or at an exit.
 *
 * Inside the grid distances run along the ray from an origin o (the pass
 * start, or the face where the direction last changed).  Each step goes from
 * the photon's voxel straight to the face of its free cube (every voxel of
 * the grid within the free radius carries the same label; the voxel itself
 * when the radius is 0), or to the interaction inside it, and then across
 * that face; a run of voxels of one label is charged its optical depth once,
 * where the label changes (s0: where the run began).  Beyond the grid's
 * lateral extent the slab continues as virtual voxels of label 1 (the
 * reference's medium there, CUDAMCFLtransport.cu:331), walked the same way. */
template <class M>
unsigned step_exact(Photon &p, Rng &r, const Phase &ph, Sink &sk) {
  const uint32_t last = ph.last_bulk;
  sk.steps++;
  float tau = -M::log(r.oc());
  const int cap = 16 + 4 * (int)(ph.num_x + ph.num_y + ph.num_z);
  const int nx = (int)ph.num_x, ny = (int)ph.num_y, nz = (int)ph.num_z;
  int it = 0;
  for (;;) {
    /* one segment per iteration: from the photon's voxel straight to the
     * face of its free cube (radius cr, clipped to the grid for a voxel of
     * the grid; the voxel itself when cr = 0), or to the interaction inside
     * it; then across that face */
    const float ox = p.x, oy = p.y, oz = p.z;
    float s0 = 0.0f;
    uint32_t here; /* the photon's label, p.bulkpos */
    int cr;
    region_of(ph, p.ix, p.iy, p.iz, here, cr);
    (void)here;
    for (;;) {
      if (++it > cap) { /* a photon that cannot reach an interaction (e.g. glass all around) */
        sk.w0_loss += p.weight;
        p.weight = 0u;
        return photon_survive(p, r, &sk.r_gain, &sk.r_loss);
      }
      const Prop &pr = ph.prop[p.bulkpos];
      const bool in = in_grid(ph, p.ix, p.iy);
      const int lx = in ? std::max(p.ix - cr, 0) : p.ix - cr, ux = in ? std::min(p.ix + cr, nx - 1) : p.ix + cr;
      const int ly = in ? std::max(p.iy - cr, 0) : p.iy - cr, uy = in ? std::min(p.iy + cr, ny - 1) : p.iy + cr;
      const int lz = std::max(p.iz - cr, 0), uz = std::min(p.iz + cr, nz - 1);
      const float cx = plane_dist(face_coord(ph, 0, p.dx > 0.0f ? ux + 1 : lx), ox, p.dx);
      const float cy = plane_dist(face_coord(ph, 1, p.dy > 0.0f ? uy + 1 : ly), oy, p.dy);
      const float cz = plane_dist(face_coord(ph, 2, p.dz > 0.0f ? uz + 1 : lz), oz, p.dz);
      float db = cx;
      int axis = 0;
      if (cy < db) { db = cy; axis = 1; }
      if (cz < db) { db = cz; axis = 2; }
      float sj = db;
      bool hit = false;
      if (pr.mutr != FLT_MAX) {
        const float s_int = s0 + tau * pr.mutr;
        if (s_int <= db) {
          sj = s_int;
          hit = true;
        }
      }
      const float x = ox + p.dx * sj, y = oy + p.dy * sj, z = oz + p.dz * sj;
      /* the voxel there, inside the cube (its last layer along the exit axis) */
      const int fx = (!hit && axis == 0) ? (p.dx > 0.0f ? ux : lx)
                                         : std::min(std::max((int)floorf((x + ph.hx) * ph.gx), lx), ux);
      const int fy = (!hit && axis == 1) ? (p.dy > 0.0f ? uy : ly)
                                         : std::min(std::max((int)floorf((y + ph.hy) * ph.gy), ly), uy);
      const int fz = (!hit && axis == 2) ? (p.dz > 0.0f ? uz : lz)
                                         : std::min(std::max((int)floorf(z * ph.gz), lz), uz);
      if (hit) {
        p.ix = fx;
        p.iy = fy;
        p.iz = fz;
        p.x = x;
        p.y = y;
        p.z = z;
        p.tof += tof_u64((double)((sj - s0) * pr.n) / kCcmfs, ph.tof_wrap); /* the run's optical path */
        goto interaction;
      }
      /* the region across the face */
      int nix = fx, niy = fy, niz = fz;
      if (axis == 0) nix += p.dx > 0.0f ? 1 : -1;
      else if (axis == 1) niy += p.dy > 0.0f ? 1 : -1;
      else niz += p.dz > 0.0f ? 1 : -1;
      uint32_t next;
      int nr = 0;
      if (niz < 0) next = 0;
      else if (niz >= nz) next = last;
      else region_of(ph, nix, niy, niz, next, nr);
      if (next == p.bulkpos) { /* the same label: on, without a stop */
        p.ix = nix;
        p.iy = niy;
        p.iz = niz;
        cr = nr;
        continue;
      }
      /* the run of this label ends at the face */
      if (pr.mutr != FLT_MAX) {
        tau -= (db - s0) / pr.mutr;
        if (tau < 0.0f) tau = 0.0f;
      }
      p.tof += tof_u64((double)((db - s0) * pr.n) / kCcmfs, ph.tof_wrap);
      s0 = db;
      p.x = x;
      p.y = y;
      p.z = z;
      const float n_next = ph.prop[next].n;
      if (!refract_axis(p, axis, pr.n, n_next, r)) { /* reflected: the face voxel, a new direction */
        p.ix = fx;
        p.iy = fy;
        p.iz = fz;
        break;
      }
      const bool bent = pr.n != n_next; /* refracted: a new direction */
      p.bulkpos = next;
      p.ix = nix;
      p.iy = niy;
      p.iz = niz;
      if (next == 0 || next == last) {
        exact_exit(p, ph, sk, next == 0);
        return photon_survive(p, r, &sk.r_gain, &sk.r_loss);
      }
      if (bent) break;
      cr = nr;
    }
  }
interaction:
  if (ph.fhd_on == 1 && in_grid(ph, p.ix, p.iy))
    add_guarded(&sk.fhd[p.ix + ph.num_x * (p.iy + ph.num_y * p.iz)], p.weight, ph.guard);
  const Prop &pi = ph.prop[p.bulkpos];
  uint32_t w = mcfl_f2u_ru(pi.mua * pi.mutr * mcfl_u2f_rn(p.weight));
  if (w > 0) {
    p.weight -= w;
    sk.absorbed += w;
  } else {
    sk.w0_loss += p.weight;
    p.weight = 0u;
  }
  spin<M>(p, pi.g, r);
  return photon_survive(p, r, &sk.r_gain, &sk.r_loss);
}

template <class M>
inline unsigned step_any(Photon &p, Rng &r, const Phase &ph, Sink &sk) {
  if (ph.method == 1) return step_layers<M>(p, r, ph, sk);
  return ph.exact ? step_exact<M>(p, r, ph, sk) : step<M>(p, r, ph, sk);
}

/* ------------------------------------------------------------------------ */


/* Free radius of every voxel, for voxel-boundary stepping: the largest
 * r <= ORACLE_FREE_MAX such that every voxel of the grid within Chebyshev
 * distance r of it carries its label.  It is 0 next to a different label
 * (26 neighbours inside the grid), and otherwise the Chebyshev distance to
 * the nearest such voxel, capped: a chamfer transform, one forward and one
 * backward raster pass over the 13 neighbours already visited, which is
 * exact for the Chebyshev metric.  A free cube is clipped to the grid where
 * it is used. */
static void free_radius(const short *labels, unsigned nx, unsigned ny, unsigned nz, std::vector<unsigned char> &out) {
  const size_t n = (size_t)nx * ny * nz;
  out.assign(n, 0);
  std::vector<int> d(n);
  auto at = [&](long x, long y, long z) { return (size_t)x + nx * ((size_t)y + ny * (size_t)z); };
  for (long z = 0; z < (long)nz; ++z)
    for (long y = 0; y < (long)ny; ++y)
      for (long x = 0; x < (long)nx; ++x) {
        const size_t i = at(x, y, z);
        bool edge = false;
        for (int c = 0; c < 27 && !edge; ++c) {
          const long u = x + c % 3 - 1, v = y + (c / 3) % 3 - 1, w = z + c / 9 - 1;
          if (u < 0 || v < 0 || w < 0 || u >= (long)nx || v >= (long)ny || w >= (long)nz) continue;
          edge = labels[at(u, v, w)] != labels[i];
        }
        d[i] = edge ? 0 : INT_MAX / 2;
      }
  for (int pass = 0; pass < 2; ++pass) {
    const long s = pass == 0 ? 1 : -1;
    for (long zz = 0; zz < (long)nz; ++zz)
      for (long yy = 0; yy < (long)ny; ++yy)
        for (long xx = 0; xx < (long)nx; ++xx) {
          const long x = pass == 0 ? xx : (long)nx - 1 - xx, y = pass == 0 ? yy : (long)ny - 1 - yy,
                     z = pass == 0 ? zz : (long)nz - 1 - zz;
          const size_t i = at(x, y, z);
          if (d[i] == 0) continue;
          for (int c = 0; c < 13; ++c) { /* the neighbours before this voxel in the pass's order */
            const long dx = c % 3 - 1, dy = (c / 3) % 3 - 1, dz = c / 9 - 1;
            const long u = x + s * dx, v = y + s * dy, w = z + s * dz;
            if (u < 0 || v < 0 || w < 0 || u >= (long)nx || v >= (long)ny || w >= (long)nz) continue;
            d[i] = std::min(d[i], d[at(u, v, w)] + 1);
          }
        }
  }
  for (size_t i = 0; i < n; ++i) out[i] = (unsigned char)std::min(d[i], ORACLE_FREE_MAX);
}

/* one free-radius map per phase kind, rebuilt by make_phase */
static std::vector<unsigned char> g_free_r[2];

void make_phase(const oracle_sim *sim, Phase &ph, int emission) {
  memset(&ph, 0, sizeof(ph));
  ph.esp = sim->esp;
  if (sim->nx > 0) {
    ph.hx = sim->half_x;
    ph.hy = sim->half_y;
    ph.gx = sim->vox_per_cm[0];
    ph.gy = sim->vox_per_cm[1];
    ph.gz = sim->vox_per_cm[2];
    ph.num_x = (unsigned)sim->nx;
    ph.num_y = (unsigned)sim->ny;
    ph.num_z = (unsigned)sim->nz;
  } else {
    const float gf = mcfl_i2f_rn(sim->grid_size);
    ph.hx = ph.hy = 2 * ph.esp;
    ph.gx = ph.gy = ph.gz = gf;
    ph.num_x = mcfl_f2u_rn(4 * ph.esp * gf);
    ph.num_y = mcfl_f2u_rn(4 * ph.esp * gf);
    ph.num_z = (unsigned)(int)(sim->esp * (float)sim->grid_size);
  }
  ph.total = ph.num_x * ph.num_y * ph.num_z;
  ph.det_dx = sim->det_dx; ph.det_dy = sim->det_dy;
  ph.det_x0 = sim->det_x0; ph.det_y0 = sim->det_y0;
  ph.det_nx = sim->det_nx;
  ph.size_x = (sim->det_dx * mcfl_i2f_rn(sim->det_nx)) / 2.0f;
  ph.size_y = (sim->det_dy * mcfl_i2f_rn(sim->det_ny)) / 2.0f;
  ph.xy_size = (unsigned)(sim->det_nx + sim->det_ny * sim->det_nx);
  ph.last_bulk = sim->n_bulks + 1;
  for (unsigned i = 0; i < sim->n_bulks + 2; ++i) {
    const oracle_bulk &b = sim->bulks[i];
    ph.prop[i] = Prop{b.mutr, emission ? b.muaf : b.mua, b.g, b.n};
  }
  ph.method = sim->bulk_method == 1 ? 1 : 2;
  ph.exact = ph.method == 2 ? sim->exact_stepping : 0;
  if (ph.exact) /* mu_t of the phase's wavelength, fluorophore absorption included */
    for (unsigned i = 0; i < sim->n_bulks + 2; ++i) {
      const oracle_bulk &b = sim->bulks[i];
      const float mut = (emission ? b.muaf : b.mua) + b.mus;
      ph.prop[i].mutr = mut == 0.0f ? FLT_MAX : 1.0f / mut;
    }
  ph.labels = sim->bulk_info;
  if (ph.exact) {
    free_radius(ph.labels, ph.num_x, ph.num_y, ph.num_z, g_free_r[emission ? 1 : 0]);
    ph.free_r = g_free_r[emission ? 1 : 0].data();
  }
  if (ph.method == 1) {
    ph.n_layers = (unsigned)sim->n_layers;
    for (unsigned i = 0; i < ph.n_layers + 2 && i < ORACLE_MAX_LAYERS + 2; ++i) ph.layers[i] = sim->layers[i];
    ph.incl = sim->inclusion;
    ph.start_layer = 0;
    /* LaunchPhoton's search for the source's layer (CUDAMCFLtransport.cu:550-560) */
    for (unsigned nl = 1; nl <= ph.n_layers; ++nl)
      if (sim->zi < ph.layers[nl].z_max && sim->zi >= ph.layers[nl].z_min) {
        ph.start_layer = nl;
        break;
      }
  }
  ph.fhd_on = emission ? 0 : sim->fhd_activated;
  ph.xi = sim->xi; ph.yi = sim->yi; ph.zi = sim->zi;
  ph.dir = emission ? 0.0f : sim->dir;
  ph.start_weight = sim->start_weight;
  ph.launch_rng_reuse = sim->launch_rng_reuse;
  ph.time_on = (!emission && sim->do_temp_sim == 1 && sim->tdet_nx > 0 && sim->tdet_ny > 0 && sim->tdet_bins > 0)
                   ? 1 : 0;
  ph.tdet_face = sim->tdet_face;
  ph.tnx = (unsigned)sim->tdet_nx;
  ph.tny = (unsigned)sim->tdet_ny;
  ph.tbins = sim->tdet_bins;
  ph.tmax = sim->tdet_max;
  ph.tdet_r = sim->tdet_r;
}

/* Detector-array positions as DoOneSimulation computes them
 * (CUDAMCFLmain.cu:94-100), in single precision. */
void time_positions(const oracle_sim *sim, std::vector<float> &px, std::vector<float> &py) {
  px.resize(sim->tdet_nx > 0 ? sim->tdet_nx : 1);
  py.resize(sim->tdet_ny > 0 ? sim->tdet_ny : 1);
  for (int xi = 0; xi < sim->tdet_nx; xi++)
    px[xi] = xi * sim->tdet_sep_x - ((sim->tdet_nx - 1) * sim->tdet_sep_x) / 2 + sim->tdet_x0;
  for (int yi = 0; yi < sim->tdet_ny; yi++)
    py[yi] = yi * sim->tdet_sep_y - ((sim->tdet_ny - 1) * sim->tdet_sep_y) / 2 + sim->tdet_y0;
}

/* Allocates the time histogram of the result and points the phase at the
 * detector positions. */
void setup_time(const oracle_sim *sim, Phase &ph, std::vector<float> &px, std::vector<float> &py,
                oracle_result *res, Sink &sk) {
  if (!ph.time_on) return;
  time_positions(sim, px, py);
  ph.tposx = px.data();
  ph.tposy = py.data();
  res->time_size = (long)sim->tdet_nx * sim->tdet_ny * sim->tdet_bins;
  res->time_xyt = (unsigned long long *)calloc((size_t)res->time_size, 8);
  sk.time_xyt = res->time_xyt;
}

/* init_RNG (CUDAMCFLrng.cu:31-90) restated.  Returns 0 on success. */
int init_rng_streams(uint64_t *x, uint32_t *a, unsigned n, const char *path, uint64_t xinit) {
  FILE *fp = fopen(path, "r");
  if (!fp) return 1;
  unsigned begin = 0, fora, t1, t2;
  if (fscanf(fp, "%u %u %u", &begin, &t1, &t2) != 3) { fclose(fp); return 1; }
  if ((xinit == 0ull) | (((unsigned)(xinit >> 32)) >= (begin - 1)) | (((unsigned)xinit) >= 0xfffffffful)) {
    fclose(fp);
    return 1;
  }
  for (unsigned i = 0; i < n; i++) {
    if (fscanf(fp, "%u %u %u", &fora, &t1, &t2) != 3) { fclose(fp); return 1; }
    a[i] = fora;
    x[i] = 0;
    while ((x[i] == 0) | (((unsigned)(x[i] >> 32)) >= (fora - 1)) | (((unsigned)x[i]) >= 0xfffffffful)) {
      xinit = (xinit & 0xffffffffull) * (begin) + (xinit >> 32);
      x[i] = (unsigned)floor((((double)((unsigned)xinit)) / (double)0x100000000) * fora);
      x[i] = x[i] << 32;
      xinit = (xinit & 0xffffffffull) * (begin) + (xinit >> 32);
      x[i] += (unsigned)xinit;
    }
  }
  fclose(fp);
  return 0;
}

/* State of the 32768 virtual threads across relaunches. */
struct ThreadBank {
  std::vector<Photon> p;
  std::vector<uint32_t> active;
  std::vector<uint64_t> *x;
  std::vector<uint32_t> *a;
};

/* DoOneSimulation(Fl)'s launch loop with the MCd3D thread body restated:
 * one launch is 32768 virtual threads, each running up to 80000 passes; a
 * terminated photon is replaced while fewer than N - 32768 photons have
 * terminated.  Returns the number of terminated photons, 0 past the
 * relaunch cap. */
template <class M>
unsigned long long run_threads(const Phase &ph, unsigned long long nphot, std::vector<uint64_t> &x,
                               std::vector<uint32_t> &a, Sink &sk, int nthreads, long cap) {
  std::vector<Photon> P(kThreads);
  std::vector<uint32_t> active(kThreads, 1u);
  std::atomic<unsigned long long> terminated(0);
  /* LaunchPhoton_Global does not store the advanced RNG state back
   * (CUDAMCFLtransport.cu:574-581): the first transport pass of every thread
   * draws the same numbers its launch drew. */
  for (unsigned t = 0; t < kThreads; ++t) {
    Rng r{x[t], a[t]};
    launch_photon<M>(P[t], r, ph, ph.xi, ph.yi, ph.zi);
  }
  const unsigned long long limit = nphot - kThreads; /* unsigned, as the reference */
  auto body = [&](unsigned t, Sink &s) {
    Rng r{x[t], a[t]};
    Photon p = P[t];
    unsigned ii = active[t] ? 0 : kStepsPerLaunch;
    for (; ii < kStepsPerLaunch; ii++) {
      if (!step_any<M>(p, r, ph, s)) {
        if (terminated.fetch_add(1) < limit) {
          launch_photon<M>(p, r, ph, ph.xi, ph.yi, ph.zi);
        } else {
          active[t] = 0u;
          ii = kStepsPerLaunch;
        }
      }
    }
    P[t] = p;
    x[t] = r.x;
  };
  long launches = 0;
  for (;;) {
    ++launches;
    if (nthreads <= 1) {
      for (unsigned t = 0; t < kThreads; ++t) body(t, sk);
    } else {
      std::vector<Sink> local(nthreads);
      for (auto &l : local) {
        l.Rd = sk.Rd; l.Tt = sk.Tt; l.fhd = sk.fhd; l.R128 = sk.R128; l.T128 = sk.T128; l.time_xyt = sk.time_xyt;
      }
      std::vector<std::thread> pool;
      for (int w = 0; w < nthreads; ++w)
        pool.emplace_back([&, w] {
          for (unsigned b = (unsigned)w; b < kBlocks; b += (unsigned)nthreads)
            for (unsigned t = b * kThreadsPerBlock; t < (b + 1) * kThreadsPerBlock; ++t) body(t, local[w]);
        });
      for (auto &th : pool) th.join();
      for (auto &l : local) {
        sk.absorbed += l.absorbed; sk.exit_top += l.exit_top; sk.exit_bottom += l.exit_bottom;
        sk.r_loss += l.r_loss; sk.r_gain += l.r_gain; sk.w0_loss += l.w0_loss; sk.steps += l.steps;
      }
    }
    unsigned sum = 0;
    for (unsigned t = 0; t < kThreads; ++t) sum += active[t];
    if (sum == 0) break;
    if (cap > 0 && launches > cap) return 0;
  }
  return terminated.load();
}

template <class M>
int refstream_impl(const oracle_sim *sim, const char *sp, uint64_t seed_exc, uint64_t seed_fl, int nthreads,
                   oracle_result *res) {
  Phase ph;
  make_phase(sim, ph, 0);
  ph.guard = 1;
  ph.tof_wrap = M::kHost;
  const int nx2 = sim->det_nx, ny2 = sim->det_ny;
  const unsigned xy = ph.xy_size;
  res->grid[0] = (int)ph.num_x; res->grid[1] = (int)ph.num_y; res->grid[2] = (int)ph.num_z;
  res->image[0] = nx2; res->image[1] = ny2;
  res->number_of_photons = sim->number_of_photons;
  res->Rd = (unsigned long long *)calloc(xy, 8);
  res->Tt = (unsigned long long *)calloc(xy, 8);
  res->fhd = (unsigned long long *)calloc(ph.total ? ph.total : 1, 8);
  res->flR = (double *)calloc(xy, 8);
  res->flT = (double *)calloc(xy, 8);
  std::vector<uint64_t> x(kThreads);
  std::vector<uint32_t> a(kThreads);
  if (init_rng_streams(x.data(), a.data(), kThreads, sp, seed_exc)) return -2;
  Sink sk;
  sk.Rd = res->Rd; sk.Tt = res->Tt; sk.fhd = res->fhd;
  std::vector<float> tpx, tpy;
  setup_time(sim, ph, tpx, tpy, res, sk);
  const auto t_exc0 = std::chrono::steady_clock::now();
  unsigned long long done = run_threads<M>(ph, sim->number_of_photons, x, a, sk, nthreads, 0);
  const auto t_exc1 = std::chrono::steady_clock::now();
  res->seconds_exc = std::chrono::duration<double>(t_exc1 - t_exc0).count();
  res->photons_exc = done;
  res->steps_exc = sk.steps;
  res->balance[0] = sk.absorbed; res->balance[1] = sk.exit_top; res->balance[2] = sk.exit_bottom;
  res->balance[3] = sk.r_loss; res->balance[4] = sk.r_gain; res->balance[5] = sk.w0_loss;
  std::vector<double> Fx(ph.total ? ph.total : 1);
  for (unsigned v = 0; v < ph.total; v++) Fx[v] = ((double)res->fhd[v] / (0xFFFFFFFF * done));

  if (init_rng_streams(x.data(), a.data(), kThreads, sp, seed_fl)) return -2;
  if (sim->do_fl_sim == 0 || sim->bulk_method != 2) return 0;
  /* wall-clock of the emission phase, recorded when the voxel loop ends */
  struct FlClock {
    oracle_result *res;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    ~FlClock() { res->seconds_fl = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
  } fl_clock{res};
  Phase fl;
  make_phase(sim, fl, 1);
  fl.guard = 1;
  const double dx = sim->det_dx, dy = sim->det_dy;
  std::vector<unsigned long long> tR(xy), tT(xy);
  for (unsigned ix = 0; ix < ph.num_x; ix++)
    for (unsigned iy = 0; iy < ph.num_y; iy++)
      for (unsigned iz = 0; iz < ph.num_z; iz++) {
        unsigned index = ix + ph.num_x * (iy + iz * ph.num_y);
        short bd = sim->bulk_info[index];
        if (!(sim->bulks[bd].albedof < 1)) continue; /* adds 0 * image in the reference */
        /* With a fluorophore map (an input the reference does not have) a
         * voxel's weight is also multiplied by its map value, and voxels
         * whose weight rounds to zero in the engine's fixed point
         * (rint(w 2^40) = 0) are not simulated, as the engine's emission
         * list leaves them out; they add nothing to the images.  Without a
         * map every voxel of a fluorescent label runs, as in the reference. */
        if (sim->fluor_map) {
          const double w = (double)sim->bulks[bd].eY * (double)(1 - sim->bulks[bd].albedof) * Fx[index] *
                           (double)sim->fluor_map[index];
          if (nearbyint(w * 0x1p40) == 0.0) continue;
        }
        if (sim->max_fl_voxels > 0 && res->fl_voxels >= sim->max_fl_voxels) return 0;
        float xi = ((float)ix / ph.gx) - ph.hx;
        float yi = ((float)iy / ph.gy) - ph.hy;
        float zi = ((float)iz / ph.gz);
        fl.xi = xi; fl.yi = yi; fl.zi = zi;
        std::fill(tR.begin(), tR.end(), 0ull);
        std::fill(tT.begin(), tT.end(), 0ull);
        Sink s2;
        s2.Rd = tR.data(); s2.Tt = tT.data();
        std::vector<uint64_t> x_before = x; /* a capped run does not copy its RNG state back */
        unsigned long long st = run_threads<M>(fl, (unsigned long long)sim->number_of_photons_per_voxel, x, a, s2,
                                               nthreads, 10000);
        if (st == 0) x = x_before;
        res->steps_fl += s2.steps;
        res->fl_voxels += 1;
        if (st == 0) res->failed_voxels += 1;
        res->photons_fl += st;
        double voxelw = ((double)sim->bulks[bd].eY * (double)(1 - sim->bulks[bd].albedof) * Fx[index]) /
                        (double)(st * 0xFFFFFFFF);
        if (sim->fluor_map) voxelw *= (double)sim->fluor_map[index];
        for (unsigned ij = 0; ij < xy; ij++) {
          double tempvwR = voxelw * (double)tR[ij];
          double tempvwT = voxelw * (double)tT[ij];
          if (res->flR[ij] + tempvwR < DBL_MAX) res->flR[ij] += tempvwR / (dx * dy);
          if (res->flT[ij] + tempvwT < DBL_MAX) res->flT[ij] += tempvwT / (dx * dy);
        }
      }
  return 0;
}

/* ------------------------- photon-indexed variant ------------------------ */

template <class M>
void run_photon_range(const Phase &ph, uint64_t key, const uint32_t *table, uint64_t k0, uint64_t k1, Sink &sk,
                      const uint32_t *vox, const uint64_t *voxq, unsigned nv, uint64_t offset = 0) {
  for (uint64_t k = k0; k < k1; ++k) {
    Rng r;
    mcfl_photon_stream(key, offset + k, table, &r.x, &r.a);
    const uint64_t x_at_launch = r.x;
    /* the photon's index in its run: the stream index for the beam (a shard
     * of a run starts at its photon offset), the index within the voxel's
     * run for an emitting voxel */
    const uint64_t k_in_run = vox ? k % nv : offset + k;
    Photon p;
    if (vox) {
      uint32_t v = vox[k / nv];
      unsigned ix = v % ph.num_x, iy = (v / ph.num_x) % ph.num_y, iz = v / (ph.num_x * ph.num_y);
      float xi = ((float)ix / ph.gx) - ph.hx;
      float yi = ((float)iy / ph.gy) - ph.hy;
      float zi = ((float)iz / ph.gz);
      sk.voxel_q = voxq[k / nv];
      launch_photon<M, true>(p, r, ph, xi, yi, zi);
      p.ix = (int)ix;
      p.iy = (int)iy;
      p.iz = (int)iz;
    } else {
      launch_photon<M, true>(p, r, ph, ph.xi, ph.yi, ph.zi);
      locate(p, ph);
    }
    if (ph.launch_rng_reuse && k_in_run < kThreads) r.x = x_at_launch;
    while (step_any<M>(p, r, ph, sk)) {
    }
  }
}

/* Photon ranges dealt to host threads; integer tallies make the result
 * independent of the thread count. */
template <class M>
void run_photon_threads(const Phase &ph, uint64_t key, const uint32_t *table, uint64_t n, Sink &sk,
                        const uint32_t *vox, const uint64_t *voxq, unsigned nv, int nthreads, uint64_t offset = 0) {
  if (nthreads <= 1 || n < 4096) {
    run_photon_range<M>(ph, key, table, 0, n, sk, vox, voxq, nv, offset);
    return;
  }
  std::vector<Sink> local(nthreads, sk);
  for (auto &l : local) { l.absorbed = l.exit_top = l.exit_bottom = l.r_loss = l.r_gain = l.w0_loss = l.steps = 0; }
  std::vector<std::thread> pool;
  const uint64_t chunk = (n + nthreads - 1) / nthreads;
  for (int w = 0; w < nthreads; ++w)
    pool.emplace_back([&, w] {
      const uint64_t k0 = std::min<uint64_t>(n, (uint64_t)w * chunk), k1 = std::min<uint64_t>(n, k0 + chunk);
      run_photon_range<M>(ph, key, table, k0, k1, local[w], vox, voxq, nv, offset);
    });
  for (auto &t : pool) t.join();
  for (auto &l : local) {
    sk.absorbed += l.absorbed; sk.exit_top += l.exit_top; sk.exit_bottom += l.exit_bottom;
    sk.r_loss += l.r_loss; sk.r_gain += l.r_gain; sk.w0_loss += l.w0_loss; sk.steps += l.steps;
  }
}

template <class M>
int photon_impl(const oracle_sim *sim, const uint32_t *table, uint64_t seed_exc, uint64_t seed_fl,
                oracle_result *res, int nthreads) {
  Phase ph;
  make_phase(sim, ph, 0);
  ph.guard = 0;
  const unsigned xy = ph.xy_size;
  res->grid[0] = (int)ph.num_x; res->grid[1] = (int)ph.num_y; res->grid[2] = (int)ph.num_z;
  res->image[0] = sim->det_nx; res->image[1] = sim->det_ny;
  res->number_of_photons = sim->number_of_photons;
  res->Rd = (unsigned long long *)calloc(xy, 8);
  res->Tt = (unsigned long long *)calloc(xy, 8);
  res->fhd = (unsigned long long *)calloc(ph.total ? ph.total : 1, 8);
  res->flR = (double *)calloc(xy, 8);
  res->flT = (double *)calloc(xy, 8);
  res->flR128 = (unsigned long long *)calloc(2 * (size_t)xy, 8);
  res->flT128 = (unsigned long long *)calloc(2 * (size_t)xy, 8);
  Sink sk;
  sk.Rd = res->Rd; sk.Tt = res->Tt; sk.fhd = res->fhd;
  std::vector<float> tpx, tpy;
  setup_time(sim, ph, tpx, tpy, res, sk);
  const unsigned long long N = sim->number_of_photons;
  run_photon_threads<M>(ph, mcfl_stream_key(seed_exc, 0), table, N, sk, nullptr, nullptr, 1, nthreads,
                        sim->photon_offset);
  res->photons_exc = N;
  res->steps_exc = sk.steps;
  res->balance[0] = sk.absorbed; res->balance[1] = sk.exit_top; res->balance[2] = sk.exit_bottom;
  res->balance[3] = sk.r_loss; res->balance[4] = sk.r_gain; res->balance[5] = sk.w0_loss;
  if (sim->do_fl_sim == 0 || sim->bulk_method != 2) return 0;

  /* Emitting voxels in increasing linear index, with fixed-point weights
   * q_v = rint(eY (1 - albedof) PHD_v 2^40), PHD_v = fhd_v / ((2^32-1) N). */
  std::vector<uint32_t> vox;
  std::vector<uint64_t> q;
  for (unsigned v = 0; v < ph.total; ++v) {
    const oracle_bulk &b = sim->bulks[sim->bulk_info[v]];
    if (!(b.albedof < 1)) continue;
    double fx = (double)res->fhd[v] / (double)(0xFFFFFFFFull * N);
    double wv = (double)b.eY * (double)(1 - b.albedof) * fx;
    if (sim->fluor_map) wv = wv * (double)sim->fluor_map[v];
    double qs = nearbyint(wv * 0x1p40);
    uint64_t qv = qs >= 18446744073709551615.0 ? 0xFFFFFFFFFFFFFFFFull : (uint64_t)qs;
    if (qv == 0) continue;
    vox.push_back(v);
    q.push_back(qv);
  }
  Phase fl;
  make_phase(sim, fl, 1);
  fl.guard = 0;
  Sink s2;
  s2.R128 = res->flR128; s2.T128 = res->flT128;
  const unsigned nv = sim->number_of_photons_per_voxel;
  const uint64_t M_total = (uint64_t)vox.size() * nv;
  run_photon_threads<M>(fl, mcfl_stream_key(seed_fl, 1), table, M_total, s2, vox.data(), q.data(), nv, nthreads);
  res->steps_fl = s2.steps;
  res->fl_voxels = (long)vox.size();
  res->photons_fl = M_total;
  const double norm = ((double)nv * 4294967295.0) * ((double)sim->det_dx * (double)sim->det_dy);
  for (unsigned i = 0; i < xy; ++i) {
    double r = (double)res->flR128[2 * i + 1] * 18446744073709551616.0 + (double)res->flR128[2 * i];
    double t = (double)res->flT128[2 * i + 1] * 18446744073709551616.0 + (double)res->flT128[2 * i];
    res->flR[i] = r * 0x1p-40 / norm;
    res->flT[i] = t * 0x1p-40 / norm;
  }
  return 0;
}

} // namespace

extern "C" int oracle_run_refstream(const oracle_sim *sim, const char *safeprimes_path, unsigned long long seed_exc,
                                    unsigned long long seed_fl, int math_libm, int nthreads, oracle_result *res) {
  memset(res, 0, sizeof(*res));
  if ((sim->bulk_method != 1 && sim->bulk_method != 2) || sim->n_bulks > ORACLE_MAX_BULKS) return -1;
  if (sim->bulk_method == 1 && (sim->n_layers < 1 || sim->n_layers > ORACLE_MAX_LAYERS)) return -1;
  /* With N <= 32768 the reference's relaunch test compares against
   * N - 32768 computed in unsigned 64-bit arithmetic, which wraps: every
   * photon is replaced and the run never ends (the emission phase stops at
   * its 10000-launch cap only after ~2.6e12 passes).  Refuse such inputs. */
  if (sim->number_of_photons <= kThreads) return -4;
  if (sim->do_fl_sim != 0 && sim->bulk_method == 2 && sim->number_of_photons_per_voxel <= kThreads) return -4;
  return math_libm ? refstream_impl<LibmMath>(sim, safeprimes_path, seed_exc, seed_fl, nthreads, res)
                   : refstream_impl<PortableMath>(sim, safeprimes_path, seed_exc, seed_fl, nthreads, res);
}

extern "C" int oracle_run_photon(const oracle_sim *sim, const uint32_t *multipliers, unsigned int n_multipliers,
                                 unsigned long long seed_exc, unsigned long long seed_fl, int math_libm,
                                 int nthreads, oracle_result *res) {
  memset(res, 0, sizeof(*res));
  if ((sim->bulk_method != 1 && sim->bulk_method != 2) || sim->n_bulks > ORACLE_MAX_BULKS || n_multipliers != 32768)
    return -1;
  if (sim->bulk_method == 1 && (sim->n_layers < 1 || sim->n_layers > ORACLE_MAX_LAYERS)) return -1;
  return math_libm ? photon_impl<LibmMath>(sim, multipliers, seed_exc, seed_fl, res, nthreads)
                   : photon_impl<PortableMath>(sim, multipliers, seed_exc, seed_fl, res, nthreads);
}

/* ---------------------------------------------------------- test helpers */

/* The free-radius map of voxel-boundary stepping for labels (nz, ny, nx),
 * x fastest, into out (one byte per voxel). */
extern "C" void oracle_free_radius(const short *labels, unsigned nx, unsigned ny, unsigned nz, unsigned char *out) {
  std::vector<unsigned char> r;
  free_radius(labels, nx, ny, nz, r);
  memcpy(out, r.data(), r.size());
}

extern "C" float oracle_plogf(float x) { return mcfl_plogf(x); }
extern "C" void oracle_psincosf(float x, float *s, float *c) { mcfl_psincosf(x, s, c); }

/* The closed-form distances from p along d to the sphere (c, r) that
 * move_to_first_boundary back-projects with (CUDAMCFLtransport.cu:792-812),
 * evaluated with the same expression. */
extern "C" void oracle_sphere_back_steps(const float *pp, const float *dd, const float *cc, float r2, float *out) {
  const float px = pp[0], py = pp[1], pz = pp[2], dx = dd[0], dy = dd[1], dz = dd[2];
  const float x_voxel = cc[0], y_voxel = cc[1], z_voxel = cc[2];
  float pow_dx = dx * dx, pow_dy = dy * dy, pow_dz = dz * dz;
  float pow_px = px * px, pow_py = py * py, pow_pz = pz * pz;
  float pow_cx = x_voxel * x_voxel, pow_cy = y_voxel * y_voxel, pow_cz = z_voxel * z_voxel;
  float disc = 2 * x_voxel * y_voxel * dx * dy - (pow_cy + pow_cz) * pow_dx - (pow_cx + pow_cz) * pow_dy -
               (pow_cx + pow_cy) * pow_dz - (pow_dy + pow_dz) * pow_px - (pow_dx + pow_dz) * pow_py -
               (pow_dx + pow_dy) * pow_pz + (pow_dx + pow_dy + pow_dz) * r2 +
               2 * (x_voxel * z_voxel * dx + y_voxel * z_voxel * dy) * dz -
               2 * (y_voxel * dx * dy - x_voxel * pow_dy + z_voxel * dx * dz - x_voxel * pow_dz) * px +
               2 * (y_voxel * pow_dx - x_voxel * dx * dy - z_voxel * dy * dz + y_voxel * pow_dz + dx * dy * px) * py +
               2 * (z_voxel * pow_dx + z_voxel * pow_dy + dx * dz * px + dy * dz * py -
                    (x_voxel * dx + y_voxel * dy) * dz) * pz;
  float root = sqrtf(disc);
  float lin = x_voxel * dx + y_voxel * dy + z_voxel * dz - dx * px - dy * py - dz * pz;
  float den = pow_dx + pow_dy + pow_dz;
  out[0] = -(lin + root) / den;
  out[1] = -(lin - root) / den;
}

extern "C" int oracle_init_rng(uint64_t *x, uint32_t *a, unsigned n, const char *path, uint64_t seed) {
  return init_rng_streams(x, a, n, path, seed);
}
