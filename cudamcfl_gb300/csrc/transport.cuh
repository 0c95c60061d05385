/*
 * Persistent photon-transport kernel for voxelized (bulk-descriptor) turbid
 * media, sm_103a.
 *
 * Included by three translation units that differ only in floating-point
 * semantics (transport_f64.cu, the double-precision build of the same
 * kernel, states the single-precision error):
 *   transport_exact.cu  MCFL_EXACT_MATH=1, nvcc -fmad=false -prec-div=true
 *                       -prec-sqrt=true -ftz=false: every float operation is
 *                       rounded once, logarithm and sine/cosine come from
 *                       portable_math.h, so the tallies equal those of the
 *                       CPU oracle bit for bit;
 *   transport_fast.cu   MCFL_EXACT_MATH=0, --use_fast_math: the hardware
 *                       SFU intrinsics, i.e. the numerics of the reference's
 *                       own GPU build (Compile750:1 -use_fast_math).
 *
 * Physics follows the reference's voxelized transport step by step and keeps
 * its operand order (RefCompat):
 *   photon launch      LaunchPhoton           CUDAMCFLtransport.cu:460-562
 *   transport pass     MCd3D loop body        CUDAMCFLtransport.cu:286-447
 *   glass voxels       MoveToFirstBoundary    CUDAMCFLtransport.cu:702-847
 *   boundaries         Reflect                CUDAMCFLtransport.cu:628-700
 *   scattering         Spin                   CUDAMCFLtransport.cu:585-625
 *   roulette           PhotonSurvive          CUDAMCFLtransport.cu:850-864
 *   random numbers     rand_MWC_co/oc         CUDAMCFLrng.cu:17-29
 *
 * What is designed for the GPU instead of translated:
 *   - persistent threads draw photon tickets from one 64-bit counter, one
 *     warp-aggregated atomic per refill, instead of relaunching a fixed
 *     32768-thread grid from a host loop that copies 128 KB of flags back per
 *     launch (CUDAMCFLmain.cu:125-165);
 *   - each photon owns an MWC stream derived from (job key, photon index):
 *     results do not depend on the schedule, so any batch or slice of a batch
 *     reproduces the same tallies;
 *   - a job table lets one launch carry many sources, media and budgets; a
 *     step budget per launch lets a server slot new jobs in between slices
 *     while photons in flight are parked in HBM;
 *   - labels are uint8 in HBM (L2-resident: 4 MB for 200x200x100 voxels);
 *     each label's transport constants (a 32-byte record: 1/mu_t,
 *     mu_a/mu_t, 1-g^2, 1-g, 2g, 1+g^2, 1/(2g), n) sit in shared memory when
 *     the launch has one medium, or in registers for the photon's current
 *     label (reloaded on a label change) when it mixes media;
 *   - the photon-hitting-density tally is one fire-and-forget 64-bit
 *     atomic add per pass, resolved in L2 (the 32 MB tally of a 200 x 200 x
 *     100 grid stays resident), or, in the kPhdAgg variants the autotuner
 *     can pick, successive passes in one voxel summed in a register first
 *     (measured 4-5 % slower: the flush branch costs more than the atomics
 *     it saves);
 *   - per-job weight accounting (absorbed, left at each face, roulette) for
 *     an exact integer energy balance;
 *   - an optional voxel-boundary stepping (kMode 2, beyond the reference):
 *     the optical depth spent voxel by voxel, runs of equal labels crossed
 *     in free cubes of a label + free-radius map, one segment per loop
 *     iteration for every lane.
 */
#include <cuda_runtime.h>
#include <float.h>

#include <algorithm>
#include <stdint.h>
#include <string.h>

#include "engine_types.h"
#include "portable_math.h"

#ifndef MCFL_F64
#define MCFL_F64 0
#endif

#if MCFL_F64
/* Every transport quantity in double, IEEE double functions. */
typedef double real;
struct __align__(16) real4 {
  double x, y, z, w;
};
#define MCFL_C(c) (c)
#define MCFL_LOGF(x) log(x)
#define MCFL_SINCOSF(x, s, c) sincos((x), (s), (c))
#define MCFL_COSF(x) cos(x)
#define MCFL_RSQRTF(x) rsqrt(x)
#define MCFL_SQRT(x) sqrt(x)
#define MCFL_SQRT_RN(x) sqrt(x)
#define MCFL_FABS(x) fabs(x)
#define MCFL_COPYSIGN(a, b) copysign((a), (b))
#define MCFL_U2R_RZ(u) ((double)(u))
#define MCFL_U2R_RN(u) ((double)(u))
#define MCFL_I2R_RN(i) ((double)(i))
#define MCFL_R2U_RZ(x) __double2uint_rz(x)
#define MCFL_R2U_RU(x) __double2uint_ru(x)
#define MCFL_R2U_RN(x) __double2uint_rn(x)
#define MCFL_KERNEL_NAME mcfl_transport_f64
#define MCFL_LAUNCHER mcfl_launch_transport_f64
#define MCFL_ATTR_FN mcfl_attr_transport_f64
#else
typedef float real;
typedef float4 real4;
#define MCFL_C(c) (c##f)
#define MCFL_SQRT(x) sqrtf(x)
#define MCFL_SQRT_RN(x) __fsqrt_rn(x)
#define MCFL_FABS(x) fabsf(x)
#define MCFL_COPYSIGN(a, b) copysignf((a), (b))
#define MCFL_U2R_RZ(u) __uint2float_rz(u)
#define MCFL_U2R_RN(u) __uint2float_rn(u)
#define MCFL_I2R_RN(i) __int2float_rn(i)
#define MCFL_R2U_RZ(x) __float2uint_rz(x)
#define MCFL_R2U_RU(x) __float2uint_ru(x)
#define MCFL_R2U_RN(x) __float2uint_rn(x)
#if MCFL_EXACT_MATH
#define MCFL_LOGF(x) mcfl_plogf(x)
#define MCFL_SINCOSF(x, s, c) mcfl_psincosf((x), (s), (c))
#define MCFL_COSF(x) mcfl_pcosf(x)
#define MCFL_RSQRTF(x) (1.0f / sqrtf(x))
#define MCFL_KERNEL_NAME mcfl_transport_exact
#define MCFL_LAUNCHER mcfl_launch_transport_exact
#define MCFL_ATTR_FN mcfl_attr_transport_exact
#else
#define MCFL_LOGF(x) __logf(x)
#define MCFL_SINCOSF(x, s, c) __sincosf((x), (s), (c))
#define MCFL_COSF(x) __cosf(x)
#define MCFL_RSQRTF(x) rsqrtf(x)
#define MCFL_KERNEL_NAME mcfl_transport_fast
#define MCFL_LAUNCHER mcfl_launch_transport_fast
#define MCFL_ATTR_FN mcfl_attr_transport_fast
#endif
#endif

namespace {

constexpr real kPi = MCFL_C(3.141592654);        /* CUDAMCFL.h:22 */
constexpr uint32_t kWeightRoulette = 429497u; /* CUDAMCFL.h:33 */
constexpr real kChance = MCFL_C(0.1);            /* CUDAMCFL.h:34 */
constexpr unsigned kFull = 0xffffffffu;
/* shared-memory bytes of the label records (launches over one medium) */
__host__ __device__ constexpr size_t lab_bytes(bool uniform) {
  return uniform ? (size_t)MCFL_MAX_LABELS * MCFL_LAB_FLOATS * sizeof(real) : 0;
}

struct Rng {
  uint64_t x;
  uint32_t a;
  /* x <- lo(x) a + hi(x) (the MWC recurrence of CUDAMCFLrng.cu:17-29) as one
   * carry chain: low word lo(x) a + hi(x) with carry out, high word the high
   * half of lo(x) a plus the carry; returns the new low word */
  __device__ __forceinline__ uint32_t step() {
    const uint32_t lo = (uint32_t)x;
    uint32_t hi = (uint32_t)(x >> 32), nlo;
    asm("{\n\t.reg .u32 t;\n\tmad.lo.cc.u32 t, %2, %3, %1;\n\tmadc.hi.u32 %1, %2, %3, 0;\n\tmov.u32 %0, t;\n\t}"
        : "=r"(nlo), "+r"(hi)
        : "r"(lo), "r"(a));
    x = ((uint64_t)hi << 32) | nlo;
    return nlo;
  }
  __device__ __forceinline__ real co() { return MCFL_U2R_RZ(step()) * MCFL_C(0x1p-32); }
  __device__ __forceinline__ real oc() { return MCFL_C(1.0) - co(); }
  /* the next draw unscaled: co() = raw() * 2^-32 exactly (a power-of-two
   * scale), so a constant times co() equals (constant * 2^-32) times raw() */
  __device__ __forceinline__ real raw() { return MCFL_U2R_RZ(step()); }
};

struct Photon {
  real x, y, z, dx, dy, dz;
  uint32_t weight, label;
  uint64_t tof; /* time of flight [fs], time-of-flight kernels only */
  /* voxel-boundary stepping only: the photon's voxel (lateral indices beyond
   * the grid name virtual voxels of label 1) */
  int ix, iy, iz;
};

/* The GPU's global nanosecond clock (PTX %globaltimer). */
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

/* Time-of-flight increment (unsigned long)(v / c) of a path of optical
 * length v [cm] (CUDAMCFLtransport.cu:316,725,832,840; c = 2.99792e-5 cm/fs,
 * CUDAMCFL.h:29), converted with saturation (a negative value adds 0). */
#if MCFL_F64
__device__ __forceinline__ uint64_t tof_fs(double v) { return __double2ull_rz(v / 2.99792E-5); }
#elif MCFL_EXACT_MATH
__device__ __forceinline__ uint64_t tof_fs(float v) { return __double2ull_rz((double)v / 2.99792E-5); }
#else
__device__ __forceinline__ uint64_t tof_fs(float v) { return __float2ull_rz(v * 33356.4609375f); }
#endif

/* The current job's medium, held in registers. */
struct Med {
  const uint8_t *labels;
#if MCFL_F64
  const float4 *prop; /* (mutr, mu_a, g, n) per label; records are built from it in double */
#else
  const float4 *lab; /* label records, two float4 each */
#endif
  unsigned long long *fhd;
  real hx, hy, esp, gx, gy, gz;
  uint32_t nx, ny, total, last;
  uint32_t nz;            /* voxel-boundary stepping only */
  const uint16_t *lab16;  /* voxel-boundary stepping only: label | free radius << 8 */
};

__device__ __forceinline__ void load_med(const McflJob *J, Med &m) {
  m.labels = (const uint8_t *)__ldg((const unsigned long long *)&J->labels);
#if MCFL_F64
  m.prop = (const float4 *)__ldg((const unsigned long long *)&J->prop);
#else
  m.lab = (const float4 *)__ldg((const unsigned long long *)&J->lab);
#endif
  m.fhd = __ldg(&J->fhd_on) ? (unsigned long long *)__ldg((const unsigned long long *)&J->fhd) : nullptr;
  m.hx = __ldg(&J->hx);
  m.hy = __ldg(&J->hy);
  m.esp = __ldg(&J->esp);
  m.gx = __ldg(&J->gx);
  m.gy = __ldg(&J->gy);
  m.gz = __ldg(&J->gz);
  m.nx = __ldg(&J->nx);
  m.ny = __ldg(&J->ny);
  m.total = __ldg(&J->total);
  m.last = __ldg(&J->last_label);
  m.nz = __ldg(&J->nz);
  m.lab16 = (const uint16_t *)__ldg((const unsigned long long *)&J->lab16);
}

/* The label record: a = (mutr, mu_a*mutr, 1-g^2, 1-g), b = (2g, 1+g^2, 1/(2g), n). */
struct Rec {
  real4 a, b;
};

#if MCFL_F64
/* The record in double from a (mutr, mu_a, g, n) entry. */
__device__ __forceinline__ Rec make_rec(float4 q) {
  const double mutr = q.x, mua = q.y, g = q.z, n = q.w;
  Rec r;
  r.a = real4{mutr, mua * mutr, 1.0 - g * g, 1.0 - g};
  r.b = real4{2.0 * g, 1.0 + g * g, 1.0 / (2.0 * g), n};
  return r;
}

__device__ __forceinline__ Rec load_rec(const Med &m, uint32_t label) { return make_rec(__ldg(&m.prop[label])); }
#else
__device__ __forceinline__ Rec load_rec(const Med &m, uint32_t label) {
  Rec r;
  r.a = __ldg(&m.lab[2 * label]);
  r.b = __ldg(&m.lab[2 * label + 1]);
  return r;
}
#endif

/* The refractive index of a label (mixed-media launches, from global memory). */
__device__ __forceinline__ real label_n(const Med &m, uint32_t label) {
#if MCFL_F64
  return (real)__ldg(reinterpret_cast<const float *>(m.prop) + 4 * label + 3);
#else
  return __ldg(reinterpret_cast<const float *>(m.lab) + MCFL_LAB_FLOATS * label + 7);
#endif
}

__device__ __forceinline__ uint32_t voxel_index(const Med &m, real x, real y, real z) {
  uint32_t i = MCFL_R2U_RZ((x + m.hx) * m.gx) +
               m.nx * (MCFL_R2U_RZ((y + m.hy) * m.gy) + m.ny * MCFL_R2U_RZ(z * m.gz));
  return i < m.total ? i : m.total - 1u;
}

__device__ __forceinline__ uint32_t start_label(const Med &m, const Photon &p) {
  if (p.z < m.esp) {
    if (MCFL_FABS(p.x) < m.hx && MCFL_FABS(p.y) < m.hy) return (uint32_t)m.labels[voxel_index(m, p.x, p.y, p.z)];
    return 1u;
  }
  return m.last;
}

__device__ __forceinline__ uint32_t slot_at(const uint32_t *order, uint32_t i) { return order ? __ldg(&order[i]) : i; }

/* Locates the job slot owning ticket t of a queue (binary search over its
 * slots in ticket order). */
__device__ __forceinline__ uint32_t find_job(const McflJob *jobs, const uint32_t *order, uint32_t n_jobs, uint64_t t) {
  if (n_jobs == 0) return 0xffffffffu;
  uint32_t lo = 0, hi = n_jobs - 1;
  while (lo < hi) {
    uint32_t mid = (lo + hi + 1) >> 1;
    if (__ldg((const unsigned long long *)&jobs[slot_at(order, mid)].ticket_begin) <= t) lo = mid;
    else hi = mid - 1;
  }
  const uint32_t slot = slot_at(order, lo);
  const McflJob *J = &jobs[slot];
  const uint64_t b = __ldg((const unsigned long long *)&J->ticket_begin);
  const uint64_t n = __ldg((const unsigned long long *)&J->photons);
  return (t >= b && t - b < n) ? slot : 0xffffffffu;
}

/* Voxel-boundary stepping: voxel (x, y) lies in the grid's lateral extent. */
__device__ __forceinline__ bool in_grid(const Med &m, int x, int y) {
  return x >= 0 && x < (int)m.nx && y >= 0 && y < (int)m.ny;
}

__device__ __forceinline__ int vfloor(real v) { return (int)floor(v); }

/* The photon's voxel from its position, for voxel-boundary stepping: beyond
 * the grid's lateral extent the slab continues as virtual voxels of label 1
 * (the reference's medium there), so the lateral indices are any integers. */
__device__ __forceinline__ void locate(Photon &p, const Med &m) {
  p.ix = vfloor((p.x + m.hx) * m.gx);
  p.iy = vfloor((p.y + m.hy) * m.gy);
  p.iz = min(max(vfloor(p.z * m.gz), 0), (int)m.nz - 1);
}

/* Label and free radius of voxel (x, y, z), z inside the slab: the grid's
 * label + free-radius map, or beyond the grid's lateral extent label 1 with
 * the radius that keeps its cube outside the grid. */
__device__ __forceinline__ void region_of(const Med &m, int x, int y, int z, uint32_t &label, int &r) {
  if (in_grid(m, x, y)) {
    const uint32_t q = m.lab16[(uint32_t)x + m.nx * ((uint32_t)y + m.ny * (uint32_t)z)];
    label = q & 0xffu;
    r = (int)(q >> 8);
  } else {
    const int dx = x < 0 ? -x : x - ((int)m.nx - 1);
    const int dy = y < 0 ? -y : y - ((int)m.ny - 1);
    label = 1u;
    r = min(MCFL_FREE_MAX, max(dx, dy) - 1);
  }
}

template <int kMode, bool kVoxelSrc = true>
__device__ __forceinline__ void launch_photon(const McflJob *J, const Med &m, uint64_t k, const uint32_t *mult,
                                              Photon &p, Rng &r, uint32_t &src_idx) {
  const uint64_t stream = __ldg((const unsigned long long *)&J->rng_offset) + k;
  mcfl_photon_stream(__ldg((const unsigned long long *)&J->key), stream, mult, &r.x, &r.a);
  const uint64_t x_at_launch = r.x;
  const uint32_t kind = __ldg(&J->src_kind);
  /* the photon's index in its run: the stream index for a beam (a shard of a
   * run starts at its photon offset), the index within the voxel's run for
   * an emitting voxel */
  uint64_t k_in_run = stream;
  if (kVoxelSrc && kind == MCFL_SRC_VOXELS) {
    const uint32_t per = __ldg(&J->per_voxel);
    src_idx = (uint32_t)(k / per);
    k_in_run = k - (uint64_t)src_idx * per;
    const uint32_t v = __ldg(&J->src_vox[src_idx]);
    const uint32_t ix = v % m.nx, iy = (v / m.nx) % m.ny, iz = v / (m.nx * m.ny);
    const real xi = ((real)ix / m.gx) - m.hx;
    const real yi = ((real)iy / m.gy) - m.hy;
    const real zi = ((real)iz / m.gz);
    p.x = xi + (MCFL_C(0.999999) / m.gx) * r.oc();
    p.y = yi + (MCFL_C(0.999999) / m.gy) * r.oc();
    p.z = zi + (MCFL_C(0.999999) / m.gz) * r.oc();
    /* The reference evaluates these in double (CUDAMCFLtransport.cu:474-483).
     * 1 - 2u and 2*PI*u are exact in double, so their single-precision forms
     * round the same value once and are bit-identical; sqrt(1 - c^2) is taken
     * in single precision here (the reference rounds a double square root), so
     * no FP64 instruction runs in the single-precision kernels. */
    const real costheta = MCFL_C(1.0) - MCFL_C(2.0) * r.oc();
    const real sintheta = MCFL_SQRT_RN(MCFL_C(1.0) - costheta * costheta);
    const real psi = (MCFL_C(2.0) * kPi) * r.oc();
    const real cospsi = MCFL_COSF(psi);
    real sinpsi = MCFL_SQRT_RN(MCFL_C(1.0) - cospsi * cospsi);
    if (!(psi < kPi)) sinpsi = -sinpsi;
    p.dx = sintheta * cospsi;
    p.dy = sintheta * sinpsi;
    p.dz = costheta;
    p.weight = 0xFFFFFFFFu;
  } else if (kind == MCFL_SRC_WIDEFIELD) {
    p.x = __ldg(&J->sx) + (r.co() - MCFL_C(0.5)) * __ldg(&J->src_w);
    p.y = __ldg(&J->sy) + (r.co() - MCFL_C(0.5)) * __ldg(&J->src_h);
    p.z = __ldg(&J->sz);
    p.dx = MCFL_C(0.0);
    p.dy = MCFL_C(0.0);
    p.dz = MCFL_C(1.0);
    p.weight = __ldg(&J->start_weight);
  } else {
    const real input_fibre_diameter = MCFL_C(0.03);
    const real sample_rad = input_fibre_diameter * MCFL_SQRT_RN(-MCFL_LOGF(r.oc()));
    const real sample_phi = 2 * kPi * r.oc();
    real sin_phi, cos_phi;
    MCFL_SINCOSF(sample_phi, &sin_phi, &cos_phi);
    p.x = __ldg(&J->sx) + sample_rad * cos_phi;
    p.y = __ldg(&J->sy) + sample_rad * sin_phi;
    p.z = __ldg(&J->sz);
    p.dx = MCFL_C(0.0);
    p.dy = MCFL_C(0.0);
    p.dz = MCFL_C(1.0);
    p.weight = __ldg(&J->start_weight);
  }
  p.label = kMode == 1 ? __ldg(&J->start_layer) : start_label(m, p);
  p.tof = 0;
  if (kMode == 2) {
    if (kVoxelSrc && kind == MCFL_SRC_VOXELS) {
      const uint32_t v = __ldg(&J->src_vox[src_idx]);
      p.ix = (int)(v % m.nx);
      p.iy = (int)((v / m.nx) % m.ny);
      p.iz = (int)(v / (m.nx * m.ny));
    } else {
      locate(p, m);
    }
  }
  /* The reference's first photon on each of its 32768 threads draws its first
   * passes from the stream state its launch started from, because
   * LaunchPhoton_Global does not store the advanced state
   * (CUDAMCFLtransport.cu:574-581).  Reproduced on request for photons
   * 0..32767 of a run (of each emitting voxel's run). */
  if (__ldg(&J->launch_rng_reuse) && k_in_run < 32768u) r.x = x_at_launch;
}

/* The record of a (mutr, mu_a, g, n) entry, built on the device (layered
 * media). */
__device__ __forceinline__ Rec rec_of(float4 q) {
#if MCFL_F64
  return make_rec(q);
#else
  float t[MCFL_LAB_FLOATS];
  mcfl_label_record(q.x, q.y, q.z, q.w, t);
  Rec r;
  r.a = make_float4(t[0], t[1], t[2], t[3]);
  r.b = make_float4(t[4], t[5], t[6], t[7]);
  return r;
#endif
}

/* Henyey-Greenstein deflection and rotation of the direction
 * (CUDAMCFLtransport.cu:585-625).  The exact kernel keeps the reference's
 * expressions, with its per-label subexpressions (1-g^2, 1-g, 2g, 1+g^2)
 * taken from the label record: the same roundings.  The fast kernel uses
 * reciprocals and one reciprocal square root for the rotation instead of
 * divisions, and an isotropic label (g = 0) takes cos(theta) = 2u - 1 from
 * the uniform u already drawn for the Henyey-Greenstein form instead of a
 * second draw (the reference's g = 0 branch draws again): the same
 * distribution, one random number fewer, no predicated draw in every
 * pass. */
__device__ __forceinline__ void spin(Photon &p, const Rec &c, Rng &r) {
  real cost, sint, cosp, sinp;
  const real two_g = c.b.x;
#if MCFL_EXACT_MATH
  real temp;
  const real tempdir = p.dx;
  temp = c.a.z / (c.a.w + two_g * r.co());
  cost = (c.b.y - temp * temp) / two_g;
  if (two_g == MCFL_C(0.0)) cost = MCFL_C(2.0) * r.co() - MCFL_C(1.0);
  sint = MCFL_SQRT(MCFL_C(1.0) - cost * cost);
  /* sin goes to cosp and cos to sinp, as in CUDAMCFLtransport.cu:603 */
  MCFL_SINCOSF(MCFL_C(2.0) * kPi * r.co(), &cosp, &sinp);
  temp = MCFL_SQRT(MCFL_C(1.0) - p.dz * p.dz);
  if (temp == MCFL_C(0.0)) {
    p.dx = sint * cosp;
    p.dy = sint * sinp;
    p.dz = MCFL_COPYSIGN(cost, p.dz * cost);
  } else {
    p.dx = (sint * (p.dx * p.dz * cosp - p.dy * sinp)) / temp + p.dx * cost;
    p.dy = (sint * (p.dy * p.dz * cosp + tempdir * sinp)) / temp + p.dy * cost;
    p.dz = -sint * cosp * temp + p.dz * cost;
  }
  temp = MCFL_RSQRTF(p.dx * p.dx + p.dy * p.dy + p.dz * p.dz);
  p.dx = p.dx * temp;
  p.dy = p.dy * temp;
  p.dz = p.dz * temp;
#else
  const real u_hg = r.co();
  const real temp = c.a.z / (c.a.w + two_g * u_hg);
  cost = (c.b.y - temp * temp) * c.b.z;
  if (two_g == MCFL_C(0.0)) cost = MCFL_C(2.0) * u_hg - MCFL_C(1.0);
  sint = MCFL_SQRT(MCFL_C(1.0) - cost * cost);
  /* 2*pi*co() with the 2^-32 scale folded into the constant: the same value */
  __sincosf((MCFL_C(2.0) * kPi * MCFL_C(0x1p-32)) * r.raw(), &cosp, &sinp);
  const real q = MCFL_C(1.0) - p.dz * p.dz;
  real dx, dy, dz;
  if (q > MCFL_C(0.0)) {
    /* with st = sin(theta)/sin(theta_old), a = st cos(psi), b = st sin(psi):
     * dz' = -sin(theta) cos(psi) sin(theta_old) + dz cos(theta) = -a q + dz cos(theta) */
    const real rq = rsqrtf(q); /* 1/sin(theta_old) */
    const real st = sint * rq;
    const real a = st * cosp, b = st * sinp;
    dx = a * (p.dx * p.dz) - b * p.dy + p.dx * cost;
    dy = a * (p.dy * p.dz) + b * p.dx + p.dy * cost;
    dz = -a * q + p.dz * cost;
  } else {
    dx = sint * cosp;
    dy = sint * sinp;
    dz = MCFL_COPYSIGN(cost, p.dz * cost);
  }
  const real nrm = rsqrtf(dx * dx + dy * dy + dz * dz);
  p.dx = dx * nrm;
  p.dy = dy * nrm;
  p.dz = dz * nrm;
#endif
}

/* Fresnel reflection / refraction with z as the interface normal
 * (CUDAMCFLtransport.cu:628-700).  Returns true when the photon crosses into
 * the new label (the caller then changes its label). */
__device__ __forceinline__ bool reflect(Photon &p, real n1, real n2, Rng &r) {
  real rr;
  const real cos_angle_i = MCFL_FABS(p.dz);
  if (n1 == n2) return true;
  if (n2 * n2 < n1 * n1 * (1 - cos_angle_i * cos_angle_i)) {
    p.dz *= -MCFL_C(1.0);
    return false;
  }
  if (cos_angle_i == MCFL_C(1.0)) {
    rr = (n1 - n2) / (n1 + n2);
    if (r.co() <= rr * rr) {
      p.dz *= -MCFL_C(1.0);
      return false;
    }
    return true;
  }
  real e = (n1 * n1) / (n2 * n2) * (MCFL_C(1.0) - cos_angle_i * cos_angle_i);
  rr = 2 * MCFL_SQRT((MCFL_C(1.0) - cos_angle_i * cos_angle_i) * (MCFL_C(1.0) - e) * e * cos_angle_i * cos_angle_i);
  e = e + (cos_angle_i * cos_angle_i) * (MCFL_C(1.0) - MCFL_C(2.0) * e);
  rr = e * ((MCFL_C(1.0) - e - rr) / ((MCFL_C(1.0) - e + rr) * (e + rr)));
  if (r.co() <= rr) {
    p.dz *= -MCFL_C(1.0);
    return false;
  }
  rr = n1 / n2;
  e = rr * rr * (MCFL_C(1.0) - cos_angle_i * cos_angle_i);
  p.dx *= rr;
  p.dy *= rr;
  p.dz = MCFL_COPYSIGN(MCFL_SQRT(1 - e), p.dz);
  return true;
}

/* Voxel-boundary stepping: distance along direction component d from
 * coordinate c to plane b (FLT_MAX when the photon does not move towards it),
 * never negative. */
__device__ __forceinline__ real plane_dist(real b, real c, real d) {
  if (d == MCFL_C(0.0)) return FLT_MAX;
  const real t = (b - c) / d;
  return t > MCFL_C(0.0) ? t : MCFL_C(0.0);
}

/* Voxel-boundary stepping: coordinate of grid face k along x, y, z (the z
 * faces 0 and nz are the slab faces themselves). */
__device__ __forceinline__ real face_x(const Med &m, int k) { return (real)k / m.gx - m.hx; }
__device__ __forceinline__ real face_y(const Med &m, int k) { return (real)k / m.gy - m.hy; }
__device__ __forceinline__ real face_z(const Med &m, int k) {
  return k == 0 ? MCFL_C(0.0) : (k == (int)m.nz ? m.esp : (real)k / m.gz);
}

/* Fresnel reflection / refraction at a voxel face whose normal is axis a
 * (0, 1, 2 = x, y, z): reflect() with that axis in place of z.  Returns true
 * when the photon crosses. */
__device__ __forceinline__ bool refract_axis(Photon &p, int a, real n1, real n2, Rng &r) {
  /* the normal component and the two tangential ones, by value (no local
   * memory), written back below */
  real dn = a == 0 ? p.dx : (a == 1 ? p.dy : p.dz);
  real t1 = a == 0 ? p.dy : (a == 1 ? p.dz : p.dx);
  real t2 = a == 0 ? p.dz : (a == 1 ? p.dx : p.dy);
  bool cross;
  real rr;
  const real cos_angle_i = MCFL_FABS(dn);
  if (n1 == n2) return true;
  if (n2 * n2 < n1 * n1 * (1 - cos_angle_i * cos_angle_i)) {
    dn *= -MCFL_C(1.0);
    cross = false;
  } else if (cos_angle_i == MCFL_C(1.0)) {
    rr = (n1 - n2) / (n1 + n2);
    cross = !(r.co() <= rr * rr);
    if (!cross) dn *= -MCFL_C(1.0);
  } else {
    real e = (n1 * n1) / (n2 * n2) * (MCFL_C(1.0) - cos_angle_i * cos_angle_i);
    rr = 2 * MCFL_SQRT((MCFL_C(1.0) - cos_angle_i * cos_angle_i) * (MCFL_C(1.0) - e) * e * cos_angle_i * cos_angle_i);
    e = e + (cos_angle_i * cos_angle_i) * (MCFL_C(1.0) - MCFL_C(2.0) * e);
    rr = e * ((MCFL_C(1.0) - e - rr) / ((MCFL_C(1.0) - e + rr) * (e + rr)));
    cross = !(r.co() <= rr);
    if (!cross) {
      dn *= -MCFL_C(1.0);
    } else {
      rr = n1 / n2;
      e = rr * rr * (MCFL_C(1.0) - cos_angle_i * cos_angle_i);
      t1 *= rr;
      t2 *= rr;
      dn = MCFL_COPYSIGN(MCFL_SQRT(1 - e), dn);
    }
  }
  if (a == 0) {
    p.dx = dn; p.dy = t1; p.dz = t2;
  } else if (a == 1) {
    p.dy = dn; p.dz = t1; p.dx = t2;
  } else {
    p.dz = dn; p.dx = t1; p.dy = t2;
  }
  return cross;
}

/* Scattering-free voxels: march in half-voxel steps to the next label, then
 * back-project onto the sphere of radius 0.707 voxel around the centre of the
 * voxel reached.  The march is bounded by max_s. */
template <bool kTime>
__device__ __forceinline__ uint32_t move_to_first_boundary(Photon &p, const Med &m, real max_s) {
  real search_step = 1 / (2 * m.gx);
  real total_move = 0;
  int index = 1;
  const uint32_t old_bulk = p.label;
  uint32_t present_bulk = old_bulk;
  while (present_bulk == old_bulk && total_move < max_s) {
    p.x += p.dx * search_step;
    p.y += p.dy * search_step;
    p.z += p.dz * search_step;
    if (kTime) p.tof += tof_fs(search_step);
    if (p.z + p.dz * search_step < MCFL_C(0.0)) {
      present_bulk = 0;
      index = -1;
      search_step = (-p.z) / p.dz;
    } else if (p.z + p.dz * search_step > m.esp) {
      present_bulk = m.last;
      index = -1;
      search_step = (m.esp - p.z) / p.dz;
    } else if (MCFL_FABS(p.x + p.dx * search_step) >= m.hx || MCFL_FABS(p.y + p.dy * search_step) >= m.hy) {
      present_bulk = 1;
      index = -1;
    } else {
      index = (int)voxel_index(m, p.x, p.y, p.z);
      present_bulk = (uint32_t)m.labels[index];
    }
    total_move += search_step;
  }
  if (index >= 0 && present_bulk != old_bulk) {
    uint32_t uidx = (uint32_t)index;
    const uint32_t z_grid = uidx / (m.nx * m.ny);
    uidx -= z_grid * m.nx * m.ny;
    const uint32_t y_grid = uidx / m.nx;
    const uint32_t x_grid = uidx % m.nx;
    const double half = 1. / (2. * (double)m.gx);
    const real y_voxel = (real)((double)(MCFL_I2R_RN((int)y_grid) / m.gy - m.hy) + half);
    const real x_voxel = (real)((double)(MCFL_I2R_RN((int)x_grid) / m.gx - m.hx) + half);
    const real z_voxel = (real)((double)(MCFL_I2R_RN((int)z_grid) / m.gz) + half);
    const double rv = 0.707107 * (double)(1 / m.gx);
    const real r_voxel2 = (real)(rv * rv);
    const real pow_dx = p.dx * p.dx, pow_dy = p.dy * p.dy, pow_dz = p.dz * p.dz;
    const real pow_px = p.x * p.x, pow_py = p.y * p.y, pow_pz = p.z * p.z;
    const real pow_cx = x_voxel * x_voxel, pow_cy = y_voxel * y_voxel, pow_cz = z_voxel * z_voxel;
    const real disc =
        2 * x_voxel * y_voxel * p.dx * p.dy - (pow_cy + pow_cz) * pow_dx - (pow_cx + pow_cz) * pow_dy -
        (pow_cx + pow_cy) * pow_dz - (pow_dy + pow_dz) * pow_px - (pow_dx + pow_dz) * pow_py -
        (pow_dx + pow_dy) * pow_pz + (pow_dx + pow_dy + pow_dz) * r_voxel2 +
        2 * (x_voxel * z_voxel * p.dx + y_voxel * z_voxel * p.dy) * p.dz -
        2 * (y_voxel * p.dx * p.dy - x_voxel * pow_dy + z_voxel * p.dx * p.dz - x_voxel * pow_dz) * p.x +
        2 * (y_voxel * pow_dx - x_voxel * p.dx * p.dy - z_voxel * p.dy * p.dz + y_voxel * pow_dz + p.dx * p.dy * p.x) *
            p.y +
        2 * (z_voxel * pow_dx + z_voxel * pow_dy + p.dx * p.dz * p.x + p.dy * p.dz * p.y -
             (x_voxel * p.dx + y_voxel * p.dy) * p.dz) * p.z;
    const real root = MCFL_SQRT(disc);
    const real lin = x_voxel * p.dx + y_voxel * p.dy + z_voxel * p.dz - p.dx * p.x - p.dy * p.y - p.dz * p.z;
    const real den = pow_dx + pow_dy + pow_dz;
    const real back_step1 = -(lin + root) / den;
    const real back_step2 = -(lin - root) / den;
    const real npx1 = p.x - p.dx * back_step1, npy1 = p.y - p.dy * back_step1, npz1 = p.z - p.dz * back_step1;
    const real npx2 = p.x - p.dx * back_step2, npy2 = p.y - p.dy * back_step2, npz2 = p.z - p.dz * back_step2;
    if (((npx1 - x_voxel) * (npx1 - x_voxel) + (npy1 - y_voxel) * (npy1 - y_voxel) +
         (npz1 - z_voxel) * (npz1 - z_voxel)) <
        ((npx2 - x_voxel) * (npx2 - x_voxel) + (npy2 - y_voxel) * (npy2 - y_voxel) +
         (npz2 - z_voxel) * (npz2 - z_voxel))) {
      p.x = npx1; p.y = npy1; p.z = npz1;
      if (kTime) p.tof -= tof_fs(back_step1);
    } else {
      p.x = npx2; p.y = npy2; p.z = npz2;
      if (kTime) p.tof -= tof_fs(back_step2);
    }
  }
  return present_bulk;
}

/* 128-bit accumulate of weight x q: low word with carry detection. */
__device__ __forceinline__ void add128(unsigned long long *acc, uint32_t w, uint64_t q) {
  const uint64_t lo = (uint64_t)w * (uint32_t)q;
  const uint64_t mid = (uint64_t)w * (uint32_t)(q >> 32);
  const uint64_t plo = lo + (mid << 32);
  const uint64_t phi = (mid >> 32) + (plo < lo ? 1u : 0u);
  const unsigned long long old = atomicAdd(&acc[0], (unsigned long long)plo);
  const uint64_t carry = (old + plo < old) ? 1u : 0u;
  if (phi + carry) atomicAdd(&acc[1], (unsigned long long)(phi + carry));
}

/* Exit through a face: image tally when the exit point is inside the
 * detector.  top: R (z = 0), else T (z = esp). */
__device__ __noinline__ void tally_exit(const McflJob *J, real px, real py, uint32_t weight, bool top,
                                        uint32_t src_idx) {
  const real x0 = __ldg(&J->det_x0), y0 = __ldg(&J->det_y0);
  const real size_x = __ldg(&J->size_x), size_y = __ldg(&J->size_y);
  if (!(MCFL_FABS(px - x0) < size_x && MCFL_FABS(py - y0) < size_y)) return;
  uint32_t idx = MCFL_R2U_RZ((py - y0 + size_y) / __ldg(&J->det_dy)) * __ldg(&J->det_nx) +
                 MCFL_R2U_RZ((px - x0 + size_x) / __ldg(&J->det_dx));
  const uint32_t xy = __ldg(&J->xy_size);
  if (idx >= xy) idx = xy - 1u;
  if (__ldg(&J->src_kind) == MCFL_SRC_VOXELS) {
    unsigned long long *img =
        (unsigned long long *)__ldg((const unsigned long long *)(top ? &J->R128 : &J->T128));
    add128(&img[2 * (size_t)idx], weight, __ldg((const unsigned long long *)&J->src_q[src_idx]));
  } else {
    unsigned long long *img = (unsigned long long *)__ldg((const unsigned long long *)(top ? &J->R : &J->T));
    atomicAdd(&img[idx], (unsigned long long)weight);
  }
}

/* Time-resolved detectors at an exit (CUDAMCFLtransport.cu:379-390,406-417):
 * when the exit face is the array's and the time of flight is below the
 * range, every disc that contains the exit point gets the weight in the
 * photon's time bin (a bin that rounds onto the end of the range is the last
 * one). */
__device__ __noinline__ void tally_time(const McflJob *J, real px, real py, uint32_t weight, uint64_t tof, bool top) {
  if (!__ldg(&J->time_on) || __ldg(&J->tdet_face) != (top ? 0u : 1u)) return;
  const uint64_t tmax = __ldg((const unsigned long long *)&J->tmax);
  if (!(tof < tmax)) return;
  const uint32_t nx = __ldg(&J->tnx), ny = __ldg(&J->tny), bins = __ldg(&J->tbins);
  const float *tx = (const float *)__ldg((const unsigned long long *)&J->tpos_x);
  const float *ty = (const float *)__ldg((const unsigned long long *)&J->tpos_y);
  unsigned long long *hist = (unsigned long long *)__ldg((const unsigned long long *)&J->time_xyt);
  const real r = __ldg(&J->tdet_r);
#if MCFL_F64
  uint32_t bin = __double2uint_rz(((double)tof / (double)tmax) * (double)bins);
#elif MCFL_EXACT_MATH
  uint32_t bin = __float2uint_rz((__ull2float_rn(tof) / __ull2float_rn(tmax)) * __uint2float_rn(bins));
#else
  uint32_t bin = __float2uint_rz(__fdividef(__ull2float_rn(tof), __ull2float_rn(tmax)) * __uint2float_rn(bins));
#endif
  if (bin >= bins) bin = bins - 1u;
  for (uint32_t i = 0; i < nx; ++i) {
    const real dx = px - (real)__ldg(&tx[i]);
    for (uint32_t j = 0; j < ny; ++j) {
      const real dy = py - (real)__ldg(&ty[j]);
      if (dx * dx + dy * dy < r * r) atomicAdd(&hist[i + (size_t)nx * (j + (size_t)ny * bin)], (unsigned long long)weight);
    }
  }
}

} // namespace

/* One warp-synchronous persistent loop per thread; see the file comment.
 * kUniform: the medium comes from the launch parameters (constant bank)
 * instead of per-lane registers loaded from the job. */
/* kMode: 0 = the reference's voxelized transport (MCd3D), 1 = layered media
 * (MCd), 2 = voxel-boundary ("exact") stepping. */
/* kPhdAgg (single medium, reference stepping): the photon-hitting-density
 * tally sums the weights of a thread's successive passes in one voxel in a
 * register and adds them to HBM when the voxel changes (and at the end),
 * instead of one atomic add per pass; the autotuner picks the form. */
/* kGeneral (single medium, reference stepping): every test of the
 * reference's pass as its own branch (the form before the SIMT arrangement),
 * kept as an autotuner alternative. */
/* kPhdWarp (single medium, the SIMT-arranged pass): the hitting-density adds
 * of a warp's lanes aggregated per voxel, one add per distinct voxel. */
template <bool kUniform, bool kTime, int kMode, int kThreads, int kMinBlocks, bool kPhdAgg = false,
          bool kGeneral = false, bool kPhdWarp = false, bool kNoPhd = false>
__global__ void __launch_bounds__(kThreads, MCFL_F64 ? 1 : kMinBlocks) MCFL_KERNEL_NAME(McflLaunch L) {
  constexpr bool kLayered = kMode == 1;
  constexpr bool kExactStep = kMode == 2;
  /* the reference-stepping pass without the time of flight, arranged for
   * the SIMT warp (see the pass below) */
  constexpr bool kLean = kMode == 0 && !kTime && !kPhdAgg && !kGeneral;
  /* dynamic shared memory: (uniform medium) the label records of the
   * medium */
  extern __shared__ __align__(16) unsigned char s_mem[];
  real4 *s_lab = reinterpret_cast<real4 *>(s_mem);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned tib = threadIdx.x;
  const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (kLayered) {
    /* per layer (and, last, the inclusion): its record and its geometry */
    const float4 *tab = (const float4 *)L.med.layer_tab;
    for (uint32_t i = tib; i < L.med.n_layers + 3; i += blockDim.x) {
      const Rec q = rec_of(__ldg(&tab[2 * i]));
      const float4 g = __ldg(&tab[2 * i + 1]);
      s_lab[3 * i] = q.a;
      s_lab[3 * i + 1] = q.b;
      s_lab[3 * i + 2] = real4{g.x, g.y, g.z, g.w};
    }
    __syncthreads();
  } else if (kUniform) {
#if MCFL_F64
    for (uint32_t i = tib; i < L.med.n_labels; i += blockDim.x) {
      const Rec q = make_rec(__ldg((const float4 *)L.med.prop + i));
      s_lab[2 * i] = q.a;
      s_lab[2 * i + 1] = q.b;
    }
#else
    for (uint32_t i = tib; i < 2 * L.med.n_labels; i += blockDim.x) s_lab[i] = __ldg((const float4 *)L.med.lab + i);
#endif
    __syncthreads();
  }

  const uint64_t ticket_end = L.ticket_end_dev ? *L.ticket_end_dev : L.ticket_end;
  bool alive = false;
  /* lean single-medium pass: 1/mu_t and n of the photon's label */
  real mutr_c = MCFL_C(0.0), n_c = MCFL_C(0.0);
  /* the warp's ticket queue and which queues it found exhausted (warp-uniform;
   * a missing second queue counts as exhausted) */
  const bool two_queues = !kUniform && L.order2 != nullptr;
  const uint32_t period = L.express_period ? L.express_period : 4u;
  uint32_t q = two_queues ? (((uint32_t)(gtid >> 5) % period) != 0u ? 1u : 0u) : 0u;
  bool ex0 = false, ex1 = !two_queues;
  Photon p;
  Rng r;
  Med m = {};
  if (kUniform) {
    m.labels = L.med.labels;
#if MCFL_F64
    m.prop = (const float4 *)L.med.prop;
#else
    m.lab = (const float4 *)L.med.lab;
#endif
    m.fhd = L.med.fhd;
    m.hx = L.med.hx;
    m.hy = L.med.hy;
    m.esp = L.med.esp;
    m.gx = L.med.gx;
    m.gy = L.med.gy;
    m.gz = L.med.gz;
    m.nx = L.med.nx;
    m.ny = L.med.ny;
    m.total = L.med.total;
    m.last = L.med.last_label;
    if (kExactStep) {
      m.nz = m.total / (m.nx * m.ny);
      m.lab16 = L.med.lab16;
    }
  }
  Rec rc = {}; /* general kernel: the record of the photon's label, in registers */
  /* voxel-boundary stepping: the state of the photon's pass between
   * segments (remaining optical depth, ray origin, start of the label run,
   * free radius, segments so far; xbegin: the origin is to be set) */
  real xtau = MCFL_C(0.0), xox = MCFL_C(0.0), xoy = MCFL_C(0.0), xoz = MCFL_C(0.0), xs0 = MCFL_C(0.0);
  int xcr = 0, xit = 0;
  bool xmid = false, xbegin = false;
  /* kPhdAgg: the voxel and the weight summed there so far */
  uint32_t f_idx = 0;
  unsigned long long f_acc = 0ull;
  uint32_t job = 0xffffffffu, src_idx = 0, pst = 0, pst0 = 0, done = 0, steps = 0;
  uint64_t k = 0, absorbed = 0;
  const McflJob *J = nullptr;

  auto flush_stats = [&]() {
    if (J == nullptr) return;
    unsigned long long *st = (unsigned long long *)__ldg((const unsigned long long *)&J->stats);
    if (done) atomicAdd(&st[MCFL_ST_DONE], (unsigned long long)done);
    if (steps) atomicAdd(&st[MCFL_ST_STEPS], (unsigned long long)steps);
    if (absorbed) atomicAdd(&st[MCFL_ST_ABSORBED], (unsigned long long)absorbed);
    done = 0;
    steps = 0;
    absorbed = 0;
  };
  /* the events of a photon (exits, roulette, zero-drop kills, the pass cap:
   * a few per photon) go straight to the job's counters */
  auto ev_add = [&](int e, unsigned long long v) {
    if (v) atomicAdd((unsigned long long *)__ldg((const unsigned long long *)&J->stats) + e, v);
  };

  /* a slice of a served run: photons in flight are parked at its end and
   * resumed by the next slice */
  const bool sliced = !kUniform && (L.max_iters || L.slice_ns) && L.saved;
  uint32_t t_begin = 0; /* the low word of the clock: slices last under 2^32 ns */
  if (!kUniform && L.slice_ns) t_begin = __shfl_sync(kFull, (uint32_t)global_ns(), 0);
  if (sliced) {
    const McflSaved sv = L.saved[gtid];
    if (sv.alive) {
      job = sv.job;
      J = &L.jobs[job];
      if (!kUniform) load_med(J, m);
      p = Photon{sv.x, sv.y, sv.z, sv.dx, sv.dy, sv.dz, sv.weight, sv.label};
      p.tof = sv.tof;
      if (kExactStep) {
        p.ix = sv.ix;
        p.iy = sv.iy;
        p.iz = sv.iz;
        xtau = sv.xtau;
        xox = sv.xox;
        xoy = sv.xoy;
        xoz = sv.xoz;
        xs0 = sv.xs0;
        xcr = sv.xcr;
        xit = sv.xit;
        xmid = (sv.xflags & 1u) != 0u;
        xbegin = (sv.xflags & 2u) != 0u;
      }
      r.x = sv.rng_x;
      r.a = sv.rng_a;
      k = sv.k;
      pst = sv.steps;
      pst0 = pst;
      src_idx = sv.src_idx;
      if (!kUniform) rc = load_rec(m, p.label);
      alive = true;
    }
  }

  for (uint32_t it = 0;; ++it) {
    /* single-medium launches always run to the end of their tickets */
    if (!kUniform && L.max_iters && it >= L.max_iters) break;
    /* a served slice ends when its time is up or its stop flag is raised
     * (a request arrived, or one finished); the warps stop together,
     * whatever their pace (a warp-uniform test: lane 0 reads the clock and
     * the flag every 16 iterations) */
    if (!kUniform && (L.slice_ns || L.stop_flag) && (it & 63u) == 0u) {
      int stop = 0;
      if (lane == 0)
        stop = (L.slice_ns && (uint32_t)global_ns() - t_begin >= (uint32_t)L.slice_ns) ||
               (L.stop_flag && *(volatile const unsigned int *)L.stop_flag != 0u);
      if (__shfl_sync(kFull, stop, 0)) break;
    }
    /* one vote per pass while every lane carries a photon; live: the lanes
     * that run this pass (lanes without a photon skip it), the member mask
     * of any warp-wide operation inside the pass */
    unsigned live = kFull;
    const unsigned dead = __ballot_sync(kFull, !alive);
    if (dead) {
    /* lanes without a photon draw new ones together once at least
     * relaunch_min of them are free (0 or 1: at once), or every lane is;
     * until then they skip the pass below */
    if ((uint32_t)__popc(dead) >= L.relaunch_min || dead == kFull) {
    const bool need = !alive && !(ex0 && ex1);
    const unsigned nm = __ballot_sync(kFull, need);
    if (nm) {
      unsigned long long *ctr = L.ticket_counter;
      uint64_t end = ticket_end;
      if constexpr (!kUniform) {
        if (q ? ex1 : ex0) q ^= 1u;
        if (q) {
          ctr = L.ticket_counter2;
          end = L.ticket_end2;
        }
      }
      const int leader = __ffs(nm) - 1;
      unsigned long long base = 0ull;
      if ((int)lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(nm));
      base = __shfl_sync(kFull, base, leader);
      bool over = false;
      if (need) {
        const uint64_t t = base + (uint64_t)__popc(nm & ((1u << lane) - 1u));
        if (t < end) {
          const uint32_t j = (!kUniform && q) ? find_job(L.jobs, L.order2, L.n_jobs2, t)
                                              : find_job(L.jobs, L.order, L.n_jobs, t);
          if (j != 0xffffffffu) {
            if (j != job) {
              flush_stats();
              job = j;
              J = &L.jobs[j];
              if (!kUniform) load_med(J, m);
            }
            k = __ldg((const unsigned long long *)&J->photon_base) +
                (t - __ldg((const unsigned long long *)&J->ticket_begin));
            /* a mixed-media launch's jobs are beams (emission runs over
             * one medium) */
            launch_photon<kMode, kUniform>(J, m, k, L.mult, p, r, src_idx);
            if (!kUniform) rc = load_rec(m, p.label);
            if (kUniform && kLean) {
              mutr_c = s_lab[2 * p.label].x;
              n_c = s_lab[2 * p.label + 1].w;
            }
            pst = 0;
            pst0 = 0;
            alive = true;
          }
        } else {
          over = true;
        }
      }
      if (__any_sync(kFull, over)) {
        if (!kUniform && q) ex1 = true;
        else ex0 = true;
      }
    }
    if (__all_sync(kFull, !alive) && ex0 && ex1) break;
    }
    if constexpr (kPhdWarp) live = __ballot_sync(kFull, alive);
    if (!alive) continue; /* a lane without a photon never runs the pass */
    }

    if constexpr (!kExactStep) ++pst;
    if constexpr (kExactStep) {
      /* ---- voxel-boundary stepping, one segment per loop iteration: the
       * optical depth -ln(u) of a pass is spent voxel by voxel with each
       * voxel's mu_t, the label is the one where the photon is, Fresnel acts
       * at every face between different indices with that face's normal,
       * scattering-free voxels are crossed without interaction.  A pass ends
       * at the interaction (PHD tally, weight drop, spin, as the reference's
       * pass) or at an exit.  A segment goes from the photon's voxel
       * straight to the face of its free cube (radius xcr of the label +
       * free-radius map, clipped to the grid; the voxel itself when 0), or
       * to the interaction inside it, and then across that face; beyond the
       * grid's lateral extent the slab continues as virtual voxels of label 1
       * (the reference's medium there), walked by the same code.  Distances
       * run along the ray from an origin (xo*) — the pass start or the face
       * where the direction last changed — and a run of voxels of one label
       * is charged its optical depth once, where the label changes (xs0:
       * where the run began).  The pass state (xtau, xo*, xs0, xcr, xit)
       * lives across iterations, so every lane of a warp runs the same
       * segment code once per iteration, whatever number of segments its
       * pass needs. ---- */
      if (!xmid) { /* a new pass */
        ++pst;
        xtau = -MCFL_LOGF(r.oc());
        xit = 0;
        xmid = true;
        xbegin = true;
      }
      const int cap = 16 + 4 * (int)(m.nx + m.ny + m.nz);
      /* 0: the pass goes on, 1: interaction, 2: exit (tallied), 3: lost */
      int outcome = 0;
      if (xbegin) {
        xox = p.x;
        xoy = p.y;
        xoz = p.z;
        xs0 = MCFL_C(0.0);
        uint32_t here;
        region_of(m, p.ix, p.iy, p.iz, here, xcr);
        xbegin = false;
      }
      if (++xit > cap) {
        outcome = 3;
      } else {
        const real4 ca = kUniform ? s_lab[2 * p.label] : rc.a;
        const int cr = xcr;
        const bool in = in_grid(m, p.ix, p.iy);
        const int lx = in ? max(p.ix - cr, 0) : p.ix - cr, ux = in ? min(p.ix + cr, (int)m.nx - 1) : p.ix + cr;
        const int ly = in ? max(p.iy - cr, 0) : p.iy - cr, uy = in ? min(p.iy + cr, (int)m.ny - 1) : p.iy + cr;
        const int lz = max(p.iz - cr, 0), uz = min(p.iz + cr, (int)m.nz - 1);
        const real cx = plane_dist(face_x(m, p.dx > MCFL_C(0.0) ? ux + 1 : lx), xox, p.dx);
        const real cy = plane_dist(face_y(m, p.dy > MCFL_C(0.0) ? uy + 1 : ly), xoy, p.dy);
        const real cz = plane_dist(face_z(m, p.dz > MCFL_C(0.0) ? uz + 1 : lz), xoz, p.dz);
        real db = cx;
        int axis = 0;
        if (cy < db) { db = cy; axis = 1; }
        if (cz < db) { db = cz; axis = 2; }
        real sj = db;
        bool hit = false;
        if (ca.x != FLT_MAX) {
          const real s_int = xs0 + xtau * ca.x;
          if (s_int <= db) {
            sj = s_int;
            hit = true;
          }
        }
        const real x = xox + p.dx * sj, y = xoy + p.dy * sj, z = xoz + p.dz * sj;
        /* the voxel there, inside the cube (its last layer along the exit axis) */
        const int fx = (!hit && axis == 0) ? (p.dx > MCFL_C(0.0) ? ux : lx)
                                           : min(max(vfloor((x + m.hx) * m.gx), lx), ux);
        const int fy = (!hit && axis == 1) ? (p.dy > MCFL_C(0.0) ? uy : ly)
                                           : min(max(vfloor((y + m.hy) * m.gy), ly), uy);
        const int fz = (!hit && axis == 2) ? (p.dz > MCFL_C(0.0) ? uz : lz)
                                           : min(max(vfloor(z * m.gz), lz), uz);
        if (hit) {
          p.ix = fx;
          p.iy = fy;
          p.iz = fz;
          p.x = x;
          p.y = y;
          p.z = z;
          if (kTime) p.tof += tof_fs((sj - xs0) * (kUniform ? s_lab[2 * p.label + 1].w : rc.b.w)); /* the run's optical path */
          outcome = 1;
        } else {
          /* the region across the face */
          int nix = fx, niy = fy, niz = fz;
          if (axis == 0) nix += p.dx > MCFL_C(0.0) ? 1 : -1;
          else if (axis == 1) niy += p.dy > MCFL_C(0.0) ? 1 : -1;
          else niz += p.dz > MCFL_C(0.0) ? 1 : -1;
          uint32_t next;
          int nr = 0;
          if (niz < 0) next = 0u;
          else if (niz >= (int)m.nz) next = m.last;
          else region_of(m, nix, niy, niz, next, nr);
          if (next == p.label) { /* the same label: on, without a stop */
            p.ix = nix;
            p.iy = niy;
            p.iz = niz;
            xcr = nr;
          } else {
            /* the run of this label ends at the face */
            const real n_here = kUniform ? s_lab[2 * p.label + 1].w : rc.b.w;
            const real n_next = kUniform ? s_lab[2 * next + 1].w : label_n(m, next);
            if (ca.x != FLT_MAX) {
              xtau -= (db - xs0) / ca.x;
              if (xtau < MCFL_C(0.0)) xtau = MCFL_C(0.0);
            }
            if (kTime) p.tof += tof_fs((db - xs0) * n_here);
            xs0 = db;
            p.x = x;
            p.y = y;
            p.z = z;
            if (!refract_axis(p, axis, n_here, n_next, r)) { /* reflected: the face voxel, a new direction */
              p.ix = fx;
              p.iy = fy;
              p.iz = fz;
              xbegin = true;
            } else {
              p.label = next;
              if constexpr (!kUniform) rc = load_rec(m, next);
              p.ix = nix;
              p.iy = niy;
              p.iz = niz;
              if (next == 0u || next == m.last) {
                const bool top = next == 0u;
                tally_exit(J, p.x, p.y, p.weight, top, kUniform ? src_idx : 0u);
                if (kTime) tally_time(J, p.x, p.y, p.weight, p.tof, top);
                ev_add(top ? MCFL_ST_EXIT_TOP : MCFL_ST_EXIT_BOTTOM, p.weight);
                p.weight = 0u;
                outcome = 2;
              } else if (n_here != n_next) {
                xbegin = true; /* refracted: a new direction */
              } else {
                xcr = nr;
              }
            }
          }
        }
      }
      if (outcome == 0) continue; /* the pass goes on in the next iteration */
      xmid = false;
      if (outcome == 1) {
        if (m.fhd && in_grid(m, p.ix, p.iy))
          atomicAdd(&m.fhd[(uint32_t)p.ix + m.nx * ((uint32_t)p.iy + m.ny * (uint32_t)p.iz)],
                    (unsigned long long)p.weight);
        const Rec c2 = kUniform ? Rec{s_lab[2 * p.label], s_lab[2 * p.label + 1]} : rc;
        const uint32_t w = MCFL_R2U_RU(c2.a.y * MCFL_U2R_RN(p.weight));
        if (w > 0u) {
          p.weight -= w;
          absorbed += w;
        } else {
          ev_add(MCFL_ST_W0_LOSS, p.weight);
          p.weight = 0u;
        }
        spin(p, c2, r);
      } else if (outcome == 3 && p.weight) { /* cannot reach an interaction (cap or no face ahead) */
        ev_add(MCFL_ST_W0_LOSS, p.weight);
        p.weight = 0u;
      }
    } else if constexpr (kLayered) {
      /* ---- one transport pass of a layered medium (MCd loop body,
       * CUDAMCFLtransport.cu:73-233) ---- */
      const uint32_t nl = L.med.n_layers;
      const real4 ig = s_lab[3 * (nl + 2) + 2]; /* inclusion x, y, z, r */
      const real4 lg = s_lab[3 * p.label + 2];  /* z_min, z_max of the photon's layer */
      const real n_here = s_lab[3 * p.label + 1].w;
      auto inside = [&]() {
        return ((p.x - ig.x) * (p.x - ig.x) + (p.y - ig.y) * (p.y - ig.y) + (p.z - ig.z) * (p.z - ig.z)) <=
               (ig.w * ig.w);
      };
      real s;
      /* outside the inclusion the reference steps 1/mu_t itself, without
       * sampling (CUDAMCFLtransport.cu:87-89); scattering-free: 2 cm */
      if (inside()) {
        const real mutr = s_lab[3 * (nl + 2)].x;
        s = mutr != FLT_MAX ? -MCFL_LOGF(r.oc()) * mutr : MCFL_C(2.0);
      } else {
        const real mutr = s_lab[3 * p.label].x;
        s = mutr != FLT_MAX ? mutr : MCFL_C(2.0);
      }
      int new_layer = (int)p.label;
      if (p.z + s * p.dz < lg.x) {
        --new_layer;
        s = (lg.x - p.z) / p.dz;
      }
      if (p.z + s * p.dz >= lg.y) {
        ++new_layer;
        s = (lg.y - p.z) / p.dz;
      }
      p.x += p.dx * s;
      p.y += p.dy * s;
      p.z += p.dz * s;
      if (kTime) p.tof += tof_fs(s * n_here);
      if (p.z > lg.y) p.z = lg.y;
      if (p.z < lg.x) p.z = lg.x;
      if (m.fhd && MCFL_FABS(p.x) < m.hx && MCFL_FABS(p.y) < m.hy && p.z < m.esp)
        atomicAdd(&m.fhd[voxel_index(m, p.x, p.y, p.z)], (unsigned long long)p.weight);
      if (new_layer != (int)p.label) {
        s = MCFL_C(0.0);
        if (reflect(p, n_here, s_lab[3 * new_layer + 1].w, r)) {
          p.label = (uint32_t)new_layer;
          if (new_layer == 0 || new_layer > (int)nl) {
            const bool top = new_layer == 0;
            tally_exit(J, p.x, p.y, p.weight, top, kUniform ? src_idx : 0u);
            if (kTime) tally_time(J, p.x, p.y, p.weight, p.tof, top);
            ev_add(top ? MCFL_ST_EXIT_TOP : MCFL_ST_EXIT_BOTTOM, p.weight);
            p.weight = 0u;
          }
        }
      }
      if (s > MCFL_C(0.0)) {
        /* rounded to nearest, never a kill (CUDAMCFLtransport.cu:201-215) */
        const uint32_t e = inside() ? nl + 2 : p.label;
        const Rec c2 = Rec{s_lab[3 * e], s_lab[3 * e + 1]};
        const uint32_t w = MCFL_R2U_RN(c2.a.y * MCFL_U2R_RN(p.weight));
        p.weight -= w;
        absorbed += w;
        spin(p, c2, r);
      }
    } else if constexpr (kLean) {
      /* ---- one transport pass of a voxelized medium (MCd3D loop body,
       * CUDAMCFLtransport.cu:286-447), arranged for the SIMT warp.
       * Every test of the reference's pass compiled to a divergent branch of
       * its own.  Here the common pass — a positive step that stays inside
       * the slab in a scattering medium and ends in the same label or in
       * one of the same refractive index (where Reflect transmits without
       * drawing a number) — runs as straight-line code with the hitting
       * density tallied under a predicate, and every other case takes one
       * shared branch that runs the reference's sequence for it.  The same
       * operations run on the same values in the same order, so the tallies
       * equal the general pass's bit for bit; the weight drop and the spin
       * (the bulk of a pass) stay common to both.  A single-medium launch
       * reads the label records from shared memory; a mixed-media launch
       * holds the photon's record in registers and reloads it when the
       * label changes. ---- */
      const real mutr = kUniform ? mutr_c : rc.a.x;
      const uint64_t x_before = r.x;
      real s = -MCFL_LOGF(r.oc()) * mutr;
      const real zn = p.z + s * p.dz;
      const real xn = p.x + p.dx * s, yn = p.y + p.dy * s;
      const bool inside = MCFL_FABS(xn) < m.hx && MCFL_FABS(yn) < m.hy && zn < m.esp;
      const uint32_t vi = voxel_index(m, xn, yn, zn); /* clamped: always a voxel of the grid */
      /* the end point's label, kept in L1 ahead of other lines (evict-last
       * hint): the gather whose latency the excitation launch waits on */
      uint32_t g;
      asm("ld.global.nc.L1::evict_last.u8 %0, [%1];" : "=r"(g) : "l"(m.labels + vi));
      const uint32_t lab = inside ? g : 1u;
      const real n_old = kUniform ? n_c : rc.b.w;
      const real n_new = kUniform ? s_lab[2 * lab + 1].w : label_n(m, lab);
      const bool clip = zn < MCFL_C(0.0) || zn > m.esp;
      const bool rare = !(mutr != FLT_MAX) || clip || !(s > MCFL_C(0.0)) ||
                        (lab != p.label && (n_new != n_old || lab - 1u >= m.last - 1u));
      bool spin_now;
      /* the hitting-density add of the pass (made after both forms join, so
       * that the warp-aggregated form runs converged) */
      bool phd_on;
      uint32_t phd_idx = vi, phd_w = p.weight;
      if (!rare) {
        p.x = xn;
        p.y = yn;
        p.z = zn;
        if constexpr (!kUniform) {
          if (lab != p.label) rc = load_rec(m, lab);
        }
        p.label = lab;
        phd_on = !kNoPhd && m.fhd && inside;
        spin_now = true;
      } else {
        uint32_t new_bulk;
        uint32_t vr = 0xffffffffu;
        if (!(mutr != FLT_MAX)) { /* scattering-free voxel: it draws no step length */
          r.x = x_before;
          s = MCFL_C(100.0);
          new_bulk = move_to_first_boundary<false>(p, m, s);
        } else if (clip) { /* the step reaches a slab face */
          new_bulk = p.label;
          if (p.z + s * p.dz < MCFL_C(0.0)) {
            new_bulk = 0;
            s = (-p.z) / p.dz;
          }
          if (p.z + s * p.dz > m.esp) {
            new_bulk = m.last;
            s = (m.esp - p.z) / p.dz;
          }
          p.x += p.dx * s;
          p.y += p.dy * s;
          p.z += p.dz * s;
        } else { /* a zero step, a change of refractive index, or a label of the media outside */
          p.x = xn;
          p.y = yn;
          p.z = zn;
          new_bulk = lab;
          if (inside) vr = vi;
        }
        if (new_bulk != p.label &&
            reflect(p, n_old, kUniform ? s_lab[2 * new_bulk + 1].w : label_n(m, new_bulk), r)) {
          p.label = new_bulk;
          if constexpr (!kUniform) rc = load_rec(m, new_bulk);
        }
        phd_on = !kNoPhd && m.fhd &&
                 (vr != 0xffffffffu || (MCFL_FABS(p.x) < m.hx && MCFL_FABS(p.y) < m.hy && p.z < m.esp));
        if (phd_on) phd_idx = vr != 0xffffffffu ? vr : voxel_index(m, p.x, p.y, p.z);
        phd_w = p.weight; /* before an exit takes it */
        if (p.label == 0u || p.label == m.last) {
          const bool top = p.label == 0u;
          tally_exit(J, p.x, p.y, p.weight, top, kUniform ? src_idx : 0u);
          ev_add(top ? MCFL_ST_EXIT_TOP : MCFL_ST_EXIT_BOTTOM, p.weight);
          p.weight = 0u;
          s = MCFL_C(0.0);
        }
        spin_now = s > MCFL_C(0.0);
        if (kUniform) {
          mutr_c = s_lab[2 * p.label].x;
          n_c = s_lab[2 * p.label + 1].w;
        }
      }
      if constexpr (kPhdWarp) {
        /* Warp-aggregated: the lanes adding to the same voxel are grouped
         * (__match_any_sync), their weights summed in two 16-bit halves (a
         * sum of 32 weights of 32 bits needs 37 bits), and one lane of each
         * group adds the sum.  The tally is the same integer sum. */
        if (__any_sync(live, phd_on)) {
          const uint32_t key = phd_on ? phd_idx : 0xffffffffu;
          const unsigned peers = __match_any_sync(live, key);
          const uint32_t w = phd_on ? phd_w : 0u;
          const uint32_t lo = __reduce_add_sync(peers, w & 0xffffu);
          const uint32_t hi = __reduce_add_sync(peers, w >> 16);
          if (phd_on && lane == (unsigned)(__ffs(peers) - 1))
            atomicAdd(&m.fhd[phd_idx], ((unsigned long long)hi << 16) + lo);
        }
      } else {
        if (phd_on) atomicAdd(&m.fhd[phd_idx], (unsigned long long)phd_w);
      }
      if (spin_now) {
        const Rec c2 = kUniform ? Rec{s_lab[2 * p.label], s_lab[2 * p.label + 1]} : rc;
        if (kUniform) {
          mutr_c = c2.a.x;
          n_c = c2.b.w;
        }
        const uint32_t w = MCFL_R2U_RU(c2.a.y * MCFL_U2R_RN(p.weight));
        /* a zero drop kills the photon: its weight stays for the end branch
         * to count, flagged in the pass count's top bit (which also sends
         * the photon there: pst >= step_cap) */
        if (w > 0u) {
          p.weight -= w;
          absorbed += w;
        } else {
          pst |= 0x80000000u;
        }
        spin(p, c2, r);
      }
    } else {
    /* ---- one transport pass (MCd3D loop body) ---- */
    real s;
    uint32_t new_bulk;
    uint32_t vi = 0xffffffffu; /* voxel of the end point, when looked up */
    const Rec c = kUniform ? Rec{s_lab[2 * p.label], s_lab[2 * p.label + 1]} : rc;
    if (c.a.x != FLT_MAX) {
      s = -MCFL_LOGF(r.oc()) * c.a.x;
      new_bulk = p.label;
      if (p.z + s * p.dz < MCFL_C(0.0)) {
        new_bulk = 0;
        s = (-p.z) / p.dz;
      }
      if (p.z + s * p.dz > m.esp) {
        new_bulk = m.last;
        s = (m.esp - p.z) / p.dz;
      }
      p.x += p.dx * s;
      p.y += p.dy * s;
      p.z += p.dz * s;
      if (kTime) p.tof += tof_fs(s * c.b.w);
      if (new_bulk != 0u && new_bulk != m.last) {
        if (MCFL_FABS(p.x) < m.hx && MCFL_FABS(p.y) < m.hy && p.z < m.esp) {
          vi = voxel_index(m, p.x, p.y, p.z);
          new_bulk = (uint32_t)m.labels[vi];
        } else {
          new_bulk = 1u;
        }
      }
    } else {
      s = MCFL_C(100.0);
      new_bulk = move_to_first_boundary<kTime>(p, m, s);
    }
    Rec cur = c; /* the record of the photon's label after the boundary */
    if (new_bulk != p.label) {
      const Rec cn = kUniform ? Rec{s_lab[2 * new_bulk], s_lab[2 * new_bulk + 1]} : load_rec(m, new_bulk);
      if (reflect(p, c.b.w, cn.b.w, r)) {
        p.label = new_bulk;
        cur = cn;
        if (!kUniform) rc = cn;
      }
    }
    /* the hitting density is tallied at the end point, where the label was
     * looked up unless the pass was clipped to a face */
    if (m.fhd && (vi != 0xffffffffu || (MCFL_FABS(p.x) < m.hx && MCFL_FABS(p.y) < m.hy && p.z < m.esp))) {
      const uint32_t fi = vi != 0xffffffffu ? vi : voxel_index(m, p.x, p.y, p.z);
      if constexpr (kPhdAgg) {
        if (fi != f_idx) {
          if (f_acc) atomicAdd(&m.fhd[f_idx], f_acc);
          f_idx = fi;
          f_acc = 0ull;
        }
        f_acc += p.weight;
      } else {
        atomicAdd(&m.fhd[fi], (unsigned long long)p.weight);
      }
    }
    if (p.label == 0u || p.label == m.last) {
      const bool top = p.label == 0u;
      tally_exit(J, p.x, p.y, p.weight, top, kUniform ? src_idx : 0u);
      if (kTime) tally_time(J, p.x, p.y, p.weight, p.tof, top);
      ev_add(top ? MCFL_ST_EXIT_TOP : MCFL_ST_EXIT_BOTTOM, p.weight);
      p.weight = 0u;
      s = MCFL_C(0.0);
    }
    if (s > MCFL_C(0.0)) {
      const Rec c2 = cur;
      const uint32_t w = MCFL_R2U_RU(c2.a.y * MCFL_U2R_RN(p.weight));
      if (w > 0u) {
        p.weight -= w;
        absorbed += w;
      } else {
        ev_add(MCFL_ST_W0_LOSS, p.weight);
        p.weight = 0u;
      }
      spin(p, c2, r);
    }
    }
    /* PhotonSurvive, the pass cap and the photon's end: one branch for the
     * lean pass */
    if (!kLean || p.weight <= kWeightRoulette || pst >= L.step_cap) {
      if (kLean && (pst & 0x80000000u)) { /* the pass's zero weight drop */
        pst &= 0x7fffffffu;
        ev_add(MCFL_ST_W0_LOSS, p.weight);
        p.weight = 0u;
      }
      if (p.weight <= kWeightRoulette) {
        if (p.weight == 0u) {
          alive = false;
        } else if (r.co() < kChance) {
          const uint32_t w0 = p.weight;
          p.weight = MCFL_R2U_RN(MCFL_U2R_RN(p.weight) / kChance);
          ev_add(MCFL_ST_R_GAIN, (unsigned long long)(p.weight - w0));
        } else {
          ev_add(MCFL_ST_R_LOSS, p.weight);
          alive = false;
        }
      }
      if (alive && pst >= L.step_cap) {
        ev_add(MCFL_ST_CAPPED, 1ull);
        alive = false;
      }
      if (!alive) {
        steps += pst - pst0;
        if (!kUniform && L.stop_flag) {
          /* a served slice counts each finished photon at once, and the
           * request's last one raises the stop flag */
          const unsigned long long before =
              atomicAdd((unsigned long long *)__ldg((const unsigned long long *)&J->stats) + MCFL_ST_DONE, 1ull);
          if (before + 1ull == __ldg((const unsigned long long *)&J->photon_base) +
                                   __ldg((const unsigned long long *)&J->photons))
            *(volatile unsigned int *)L.stop_flag = 1u;
        } else {
          ++done;
        }
      }
    }
  }
  if (alive) steps += pst - pst0; /* passes of the photon parked by this slice */
  if (kPhdAgg && f_acc) atomicAdd(&m.fhd[f_idx], f_acc);

  if (sliced) {
    McflSaved sv;
    sv.alive = alive ? 1u : 0u;
    if (alive) {
      sv.x = (float)p.x; sv.y = (float)p.y; sv.z = (float)p.z;
      sv.dx = (float)p.dx; sv.dy = (float)p.dy; sv.dz = (float)p.dz;
      sv.weight = p.weight;
      sv.label = p.label;
      sv.rng_x = r.x;
      sv.rng_a = r.a;
      sv.job = job;
      sv.k = k;
      sv.steps = pst;
      sv.src_idx = src_idx;
      sv.tof = kTime ? p.tof : 0ull;
      if (kExactStep) {
        sv.ix = p.ix;
        sv.iy = p.iy;
        sv.iz = p.iz;
        sv.xtau = (float)xtau;
        sv.xox = (float)xox;
        sv.xoy = (float)xoy;
        sv.xoz = (float)xoz;
        sv.xs0 = (float)xs0;
        sv.xcr = xcr;
        sv.xit = xit;
        sv.xflags = (xmid ? 1u : 0u) | (xbegin ? 2u : 0u);
      }
    }
    L.saved[gtid] = sv;
  }
  flush_stats();
}

/* dynamic shared memory of a launch (threads: the variant's block size) */
static size_t smem_bytes(int threads, bool uniform) {
  (void)threads;
  return lab_bytes(uniform) + 16;
}

/* Kernel variants.  Single medium (occupancy variants: threads per block x
 * the blocks per SM the register budget is cut for): 0 = 256 x 4,
 * 1 = 256 x 5, 2 = 128 x 9, chosen by the autotuner, and 7, 8, 9 the same
 * with the photon-hitting-density sums held in a register, 11, 12, 13 the
 * same with the pass in its per-test branching form, 14, 15, 16 the same
 * with the hitting-density adds aggregated per warp, 17, 18, 19 the same
 * as 0, 1, 2 with no hitting-density code (the launcher runs them for
 * launches that tally none: emission, excitation without fluence); 3 = 256 x 3 carrying
 * the time of flight; layered medium 4 = 256 x 4, 5 = 256 x 3 with the time
 * of flight; voxel-boundary stepping 6 = 256 x 4, 10 = 256 x 3 with the time
 * of flight.  Mixed media: -1 = 256 x 3, -3 = 256 x 4, -4 = 128 x 7,
 * -5, -6, -7 the same with the per-test branching pass, -2 = 256 x 2 with
 * the time of flight; voxel-boundary stepping -8 = 256 x 3, -9 = 256 x 2 with
 * the time of flight. */
typedef void (*TransportKernel)(McflLaunch);

/* Mixed-media occupancy variants: 0 = 256 x 3, 1 = 256 x 4, 2 = 128 x 7;
 * 3, 4, 5 the same with the pass in its per-test branching form. */
static int mixed_variant_code(uint32_t v) {
  static const int code[6] = {-1, -3, -4, -5, -6, -7};
  return v < 6 ? code[v] : -1;
}

static TransportKernel kernel_of(int variant, int *threads) {
  switch (variant) {
  case -2: *threads = 256; return MCFL_KERNEL_NAME<false, true, 0, 256, 2>;
  case -1: *threads = 256; return MCFL_KERNEL_NAME<false, false, 0, 256, 3>;
  case -3: *threads = 256; return MCFL_KERNEL_NAME<false, false, 0, 256, 4>;
  case -4: *threads = 128; return MCFL_KERNEL_NAME<false, false, 0, 128, 7>;
  case -5: *threads = 256; return MCFL_KERNEL_NAME<false, false, 0, 256, 3, false, true>;
  case -6: *threads = 256; return MCFL_KERNEL_NAME<false, false, 0, 256, 4, false, true>;
  case -7: *threads = 128; return MCFL_KERNEL_NAME<false, false, 0, 128, 7, false, true>;
  case -8: *threads = 256; return MCFL_KERNEL_NAME<false, false, 2, 256, 3>;
  case -9: *threads = 256; return MCFL_KERNEL_NAME<false, true, 2, 256, 2>;
  case 0: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 4>;
  case 1: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 5>;
  case 2: *threads = 128; return MCFL_KERNEL_NAME<true, false, 0, 128, 9>;
  case 3: *threads = 256; return MCFL_KERNEL_NAME<true, true, 0, 256, 3>;
  case 4: *threads = 256; return MCFL_KERNEL_NAME<true, false, 1, 256, 4>;
  case 5: *threads = 256; return MCFL_KERNEL_NAME<true, true, 1, 256, 3>;
  case 6: *threads = 256; return MCFL_KERNEL_NAME<true, false, 2, 256, 4>;
  case 7: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 4, true>;
  case 8: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 5, true>;
  case 9: *threads = 128; return MCFL_KERNEL_NAME<true, false, 0, 128, 9, true>;
  case 10: *threads = 256; return MCFL_KERNEL_NAME<true, true, 2, 256, 3>;
  case 11: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 4, false, true>;
  case 12: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 5, false, true>;
  case 13: *threads = 128; return MCFL_KERNEL_NAME<true, false, 0, 128, 9, false, true>;
  case 14: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 4, false, false, true>;
  case 15: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 5, false, false, true>;
  case 16: *threads = 128; return MCFL_KERNEL_NAME<true, false, 0, 128, 9, false, false, true>;
  case 17: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 4, false, false, false, true>;
  case 18: *threads = 256; return MCFL_KERNEL_NAME<true, false, 0, 256, 5, false, false, false, true>;
  case 19: *threads = 128; return MCFL_KERNEL_NAME<true, false, 0, 128, 9, false, false, false, true>;
  default: *threads = 0; return nullptr;
  }
}

/* Launches the kernel the launch asks for (single medium: L->variant, or
 * variant 3 when it carries the time of flight; mixed media: -1 or -2); with
 * L->l2_bytes > 0 the launch carries a persisting-L2 access window (a launch
 * attribute, so it is recorded with the kernel node when captured). */
extern "C" cudaError_t MCFL_LAUNCHER(const McflLaunch *L, int grid, int block, cudaStream_t stream) {
  if (L->uniform_medium && L->med.n_labels > MCFL_MAX_LABELS) return cudaErrorInvalidValue;
#if MCFL_F64
  if (L->max_iters || L->slice_ns) return cudaErrorNotSupported; /* parked photons are stored in single precision */
#endif
  if ((L->max_iters || L->slice_ns) && L->uniform_medium) return cudaErrorNotSupported; /* slices run the mixed-media kernel */
  if (L->med.layered && (!L->uniform_medium || 3 * (L->med.n_layers + 3) > (MCFL_MAX_LABELS * MCFL_LAB_FLOATS) / 4))
    return cudaErrorInvalidValue;
  const int v = L->exact_step ? (!L->uniform_medium ? (L->time_on ? -9 : -8) : L->time_on ? 10 : 6)
                : L->med.layered ? (L->time_on ? 5 : 4)
                : L->uniform_medium ? (L->time_on ? 3 : (int)L->variant)
                : L->time_on        ? -2
                                    : mixed_variant_code(L->variant);
  int t = 0;
  /* variants 0..2 without a hitting-density tally: their instantiations
   * that compile none (17..19) */
  const int vk = (v >= 0 && v <= 2 && !L->med.fhd) ? v + 17 : v;
  const TransportKernel fn = kernel_of(vk, &t);
  if (!fn || block > t) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem_bytes(t, L->uniform_medium != 0);
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  if (L->l2_bytes) {
    memset(attr, 0, sizeof(attr));
    attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[0].val.accessPolicyWindow.base_ptr = const_cast<void *>(L->l2_base);
    attr[0].val.accessPolicyWindow.num_bytes = (size_t)L->l2_bytes;
    attr[0].val.accessPolicyWindow.hitRatio = L->l2_hit_ratio;
    attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, fn, *L);
}

/* Resident blocks per SM and registers of a kernel variant (see kernel_of)
 * at *block threads per block; *block <= 0 or above the variant's bound is
 * replaced by the bound. */
extern "C" cudaError_t MCFL_ATTR_FN(int variant, int *block, int *blocks_per_sm, int *regs) {
  int t = 0;
  const TransportKernel fn = kernel_of(variant, &t);
  if (!fn) return cudaErrorInvalidValue;
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, (const void *)fn);
  if (e != cudaSuccess) return e;
  if (regs) *regs = a.numRegs;
  if (*block <= 0 || *block > t) *block = t;
  const size_t smem = smem_bytes(t, variant >= 0);
  /* The L1/shared split: just the shared memory the blocks that the
   * registers allow need, the rest as L1 (the label gather of every pass
   * hits it).  Occupancy first with the whole shared memory available. */
  e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int bps = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void *)fn, *block, smem);
  if (e != cudaSuccess) return e;
  int dev = 0, max_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&max_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess) return e;
  if (bps > 0 && max_sm > 0) {
    const size_t need = (size_t)bps * (smem + a.sharedSizeBytes + 1024); /* 1 KB per block reserved by the system */
    const int pct = (int)std::min<size_t>(100, (need * 100 + (size_t)max_sm - 1) / (size_t)max_sm + 1);
    e = cudaFuncSetAttribute((const void *)fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    if (e != cudaSuccess) return e;
    if (variant >= 0 && variant <= 2) { /* the same split for its instantiation without the tally */
      int t2 = 0;
      e = cudaFuncSetAttribute((const void *)kernel_of(variant + 17, &t2), cudaFuncAttributePreferredSharedMemoryCarveout,
                               pct);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, (const void *)fn, *block, smem);
}
