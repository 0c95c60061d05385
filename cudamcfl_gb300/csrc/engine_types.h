/*
 * Device-side job and launch descriptors of the transport engine, shared by
 * the kernels and the host engine.
 *
 * A launch processes a list of jobs.  Every job owns a contiguous range of
 * global photon tickets [ticket_begin, ticket_begin + photons); persistent
 * threads draw tickets from one 64-bit counter, so jobs of any size, medium or
 * source mix freely inside one launch.  Photon k of a job draws its random
 * numbers from the MWC stream (key, rng_offset + k) of portable_math.h, so a
 * photon's trajectory does not depend on which thread, launch or batch
 * carries it, and the 64-bit integer tallies are therefore bit-identical for
 * any schedule.
 */
#ifndef MCFL_ENGINE_TYPES_H
#define MCFL_ENGINE_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
#define MCFL_ALIGN(n) alignas(n)
#else
#define MCFL_ALIGN(n)
#endif

/* Per-job statistics, 64-bit counters. */
enum {
  MCFL_ST_DONE = 0,        /* photons terminated */
  MCFL_ST_STEPS = 1,       /* transport passes */
  MCFL_ST_ABSORBED = 2,    /* weight deposited by absorption */
  MCFL_ST_EXIT_TOP = 3,    /* weight that left through z = 0 (inside or outside the detector) */
  MCFL_ST_EXIT_BOTTOM = 4, /* weight that left through z = thickness */
  MCFL_ST_R_LOSS = 5,      /* weight of photons that lost the roulette */
  MCFL_ST_R_GAIN = 6,      /* weight added to roulette survivors */
  MCFL_ST_W0_LOSS = 7,     /* weight of photons killed by a zero weight drop (mu_a = 0) */
  MCFL_ST_CAPPED = 8,      /* photons stopped by the per-photon pass cap */
  MCFL_ST_COUNT = 9
};

/* Source kinds. */
enum {
  MCFL_SRC_GAUSS_BEAM = 1, /* collimated beam, radius 0.03 sqrt(-ln u) (reference dir=1) */
  MCFL_SRC_VOXELS = 2,     /* isotropic, uniform inside voxels of a list (reference dir=0, per voxel) */
  MCFL_SRC_WIDEFIELD = 3   /* collimated, uniform over a rectangle */
};

typedef struct MCFL_ALIGN(16) McflJob {
  /* medium (bulk-descriptor voxel grid, x fastest) */
  const uint8_t *labels;
  const float *prop; /* 4 floats per label: 1/(mu_a+mu_s) (FLT_MAX = no scattering), mu_a, g, n */
  const float *lab;  /* MCFL_LAB_FLOATS per label, see mcfl_label_record */
  float hx, hy, esp; /* |x| < hx, |y| < hy, 0 <= z < esp */
  float gx, gy, gz;  /* voxels per cm */
  uint32_t nx, ny, nz, total;
  uint32_t last_label; /* label of the medium below the slab (labels + 1) */
  uint32_t src_kind;
  /* source */
  float sx, sy, sz;
  float src_w, src_h;
  uint32_t start_weight;
  const uint32_t *src_vox; /* MCFL_SRC_VOXELS: linear voxel indices */
  const uint64_t *src_q;   /* MCFL_SRC_VOXELS: fixed-point exit weights per voxel (2^-40 units) */
  uint32_t per_voxel;      /* MCFL_SRC_VOXELS: photons per voxel */
  uint32_t fhd_on;
  uint32_t launch_rng_reuse; /* 1: photons 0..32767 of a run (of each voxel) restart their stream after launch */
  uint32_t time_on;          /* 1: time-resolved detectors (the launch must run a time-of-flight kernel) */
  /* detector (R at z = 0, T at z = esp) */
  float det_x0, det_y0, det_dx, det_dy, size_x, size_y;
  uint32_t det_nx, xy_size;
  /* tallies */
  unsigned long long *R, *T;       /* 64-bit sums of 32-bit exit weights */
  unsigned long long *R128, *T128; /* (lo, hi) sums of weight x src_q, MCFL_SRC_VOXELS */
  unsigned long long *fhd;         /* photon hitting density, when fhd_on */
  unsigned long long *stats;       /* MCFL_ST_COUNT counters */
  /* time-resolved detectors: tnx x tny discs of radius tdet_r at (tpos_x[i],
   * tpos_y[j]) on face tdet_face (0: z = 0, 1: z = esp); tbins bins over
   * [0, tmax) fs; time_xyt[i + tnx*(j + tny*bin)] */
  const float *tpos_x, *tpos_y;
  unsigned long long *time_xyt;
  uint64_t tmax;
  float tdet_r;
  uint32_t tnx, tny, tbins, tdet_face;
  uint32_t start_layer; /* layered media: the layer holding the source */
  /* photons */
  uint64_t key;          /* stream family key */
  uint64_t rng_offset;   /* stream index of the job's photon 0 */
  uint64_t ticket_begin; /* first global ticket */
  uint64_t photon_base;  /* job photon index of ticket_begin (a server slice hands out a job's photons in parts) */
  uint64_t photons;      /* photons in the job */
  /* voxel-boundary stepping in a mixed-media launch: the medium's label |
   * free radius << 8 per voxel (McflMedium::lab16 of a single-medium launch) */
  const uint16_t *lab16;
  uint64_t pad_j;
} McflJob;

/* Photon state carried between slices of a budgeted launch. */
typedef struct MCFL_ALIGN(16) McflSaved {
  float x, y, z, dx, dy, dz;
  uint32_t weight, label;
  uint64_t rng_x;
  uint32_t rng_a, job;
  uint64_t k;        /* photon index within the job */
  uint32_t steps;    /* passes of this photon so far */
  uint32_t alive;
  uint32_t src_idx;  /* voxel-list entry (MCFL_SRC_VOXELS) */
  uint32_t pad;
  uint64_t tof;      /* time of flight [fs] (time-of-flight launches) */
  /* voxel-boundary stepping: the pass in progress (remaining optical depth,
   * ray origin, start of the label run), the photon's voxel, the free
   * radius and segment count, and flags (1: a pass in progress, 2: its
   * origin is to be set) */
  float xtau, xox, xoy, xoz, xs0;
  int32_t ix, iy, iz, xcr, xit;
  uint32_t xflags;
} McflSaved;

/* Per-label constants of the transport, derived once from
 * (mutr = 1/(mu_a+mu_s), mu_a, g, n) with the operations the reference
 * performs on every pass, so precomputing them changes no bit:
 *   [0] mutr   [1] mu_a*mutr   [2] 1-g*g   [3] 1-g
 *   [4] 2*g    [5] 1+g*g       [6] 1/(2*g) (fast-math kernel only)   [7] n  */
#define MCFL_LAB_FLOATS 8
#define MCFL_MAX_LABELS 256

/* Medium of a launch whose jobs all share it (kernel parameters). */
typedef struct McflMedium {
  const uint8_t *labels;
  const float *prop;
  const float *lab;     /* label records (MCFL_LAB_FLOATS each), staged in shared memory */
  uint32_t n_labels;    /* records in lab (<= MCFL_MAX_LABELS) */
  uint32_t pad0;
  unsigned long long *fhd; /* NULL when no job tallies the photon hitting density */
  float hx, hy, esp, gx, gy, gz;
  uint32_t nx, ny, total, last_label;
  /* Layered medium (the reference's bulk method 1): slabs 1..n_layers between
   * the media above (0) and below (n_layers+1) and one spherical inclusion.
   * layer_tab: n_layers+2 entries of two float4, (mutr, mu_a, g, n) and
   * (z_min, z_max, 0, 0), then the inclusion's (mutr, mu_a, g, n) and
   * (x, y, z, r).  The geometry above is then the photon-hitting-density
   * grid's. */
  const float *layer_tab;
  uint32_t layered, n_layers;
  /* voxel-boundary stepping: per voxel its label | free radius << 8, the
   * free radius being the largest r <= MCFL_FREE_MAX such that every voxel
   * of the grid within Chebyshev distance r carries the same label */
  const uint16_t *lab16;
} McflMedium;

#define MCFL_FREE_MAX 31

typedef struct McflLaunch {
  const McflJob *jobs;   /* job slots */
  const uint32_t *order; /* slots sorted by ticket_begin, or NULL: slots 0..n_jobs-1 in order */
  uint32_t n_jobs;       /* entries of order (or slots) */
  uint32_t max_iters; /* loop iterations per launch; 0 = run until no ticket is left */
  /* a slice (mixed-media launches with saved): every warp stops at the
   * first multiple of 16 iterations at least slice_ns after its start
   * (0: no time limit); with max_iters, whichever comes first */
  uint64_t slice_ns;
  /* a served slice (with saved): also ends once this word is nonzero; the
   * kernel sets it when a request's last photon finishes */
  unsigned int *stop_flag;
  unsigned long long *ticket_counter;
  uint64_t ticket_end;                       /* used when ticket_end_dev is NULL */
  const unsigned long long *ticket_end_dev; /* ticket end written by an earlier kernel */
  /* A second ticket queue (mixed-media launches): one warp in
   * express_period draws from the first queue, the others from the second,
   * each from the other once its own is exhausted.  NULL order2: one queue. */
  const uint32_t *order2;
  unsigned long long *ticket_counter2;
  uint64_t ticket_end2;
  uint32_t n_jobs2;
  uint32_t express_period; /* two queues: warp w draws from the first queue first when w % period == 0 (0: 4) */
  const uint32_t *mult; /* 32768 MWC multipliers */
  McflSaved *saved;     /* one per thread of the grid, when max_iters or slice_ns > 0 */
  uint32_t step_cap;    /* passes after which a photon is stopped and counted in MCFL_ST_CAPPED */
  uint32_t uniform_medium; /* 1: every job uses med (and fhd_on agrees with med.fhd) */
  uint32_t variant;        /* occupancy variant of the single-medium kernel */
  uint32_t time_on;        /* 1: carry the time of flight (some job has time-resolved detectors) */
  uint32_t exact_step;     /* 1: voxel-boundary stepping (single voxelized medium) */
  /* lanes of a warp without a photon wait until at least this many are
   * free (or every lane is), then draw new photons together (0: 1) */
  uint32_t relaunch_min;
  float l2_hit_ratio;      /* host side: persisting-L2 window over [l2_base, +l2_bytes) when l2_bytes > 0 */
  const void *l2_base;
  unsigned long long l2_bytes;
  McflMedium med;
} McflLaunch;


/* Builds one label record (host or device; IEEE single precision, no
 * contraction in the translation units that call it). */
#if defined(__CUDACC__)
__host__ __device__
#endif
static inline void mcfl_label_record(float mutr, float mua, float g, float n, float *out) {
  out[0] = mutr;
  out[1] = mua * mutr;
  out[2] = 1.0f - g * g;
  out[3] = 1.0f - g;
  out[4] = 2.0f * g;
  out[5] = 1.0f + g * g;
  out[6] = 1.0f / (2.0f * g);
  out[7] = n;
}

#endif
