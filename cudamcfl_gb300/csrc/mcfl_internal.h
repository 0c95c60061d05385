/*
 * Internal declarations of libmcfl shared by the host translation units.
 */
#ifndef MCFL_INTERNAL_H
#define MCFL_INTERNAL_H

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "engine_types.h"
#include "mcfl.h"

namespace mcfl {

constexpr size_t kMwcTableEntries = 32768;

/* safeprimes.cpp */
bool mwc_multiplier_valid(uint32_t a);
std::vector<uint32_t> mwc_multipliers(size_t count);
const std::vector<uint32_t> &mwc_table(); /* kMwcTableEntries + 1 entries */

/* errors (thread-local message) */
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *where);

#define MCFL_CUDA_TRY(call)                                    \
  do {                                                         \
    cudaError_t e__ = (call);                                  \
    if (e__ != cudaSuccess) return mcfl::cuda_fail(e__, #call); \
  } while (0)

/* Grow-only device buffer. */
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  cudaError_t reserve(size_t n);
  void release();
  template <class T> T *as() const { return static_cast<T *>(p); }
  ~DevBuf() { release(); }
};

/* engine_kernels.cu */
extern "C" cudaError_t mcfl_launch_emission_prep(const uint8_t *labels, const float2 *fl, const unsigned long long *fhd,
                                                 const float *fmap, uint32_t total, unsigned long long photons_exc,
                                                 uint32_t per_voxel, uint32_t *block_counts, uint32_t *vox,
                                                 uint64_t *q, unsigned long long *list_len,
                                                 McflJob *job, unsigned long long *ticket_end, cudaStream_t s);
size_t emission_prep_blocks(uint32_t total);
/* label | free radius << 8 per voxel (McflMedium::lab16); tmp: 2 * nx*ny*nz bytes */
extern "C" cudaError_t mcfl_launch_free_map(const uint8_t *labels, int nx, int ny, int nz, uint8_t *tmp,
                                           uint16_t *lab16, cudaStream_t s);
extern "C" cudaError_t mcfl_launch_normalize_u64(const unsigned long long *raw, double *out, size_t n, double scale,
                                                 cudaStream_t s);
extern "C" cudaError_t mcfl_launch_normalize_phd(const unsigned long long *raw, double *out, size_t n,
                                                 unsigned long long photons, cudaStream_t s);
extern "C" cudaError_t mcfl_launch_normalize_segments(const unsigned long long *raw, double *out, size_t seg_len,
                                                      size_t n_seg, const double *scales, cudaStream_t s);
extern "C" cudaError_t mcfl_launch_normalize_128(const unsigned long long *raw, double *out, size_t n, double norm,
                                                 cudaStream_t s);

/* transport kernels */
extern "C" cudaError_t mcfl_launch_transport_exact(const McflLaunch *L, int grid, int block, cudaStream_t s);
extern "C" cudaError_t mcfl_launch_transport_fast(const McflLaunch *L, int grid, int block, cudaStream_t s);
/* Occupancy of a kernel variant (variant < 0: mixed media; 0..MCFL_N_VARIANTS-1:
 * single medium) at *block threads (clamped to the variant's bound). */
extern "C" cudaError_t mcfl_attr_transport_exact(int variant, int *block, int *blocks_per_sm, int *regs);
extern "C" cudaError_t mcfl_attr_transport_fast(int variant, int *block, int *blocks_per_sm, int *regs);
extern "C" cudaError_t mcfl_launch_transport_f64(const McflLaunch *L, int grid, int block, cudaStream_t s);
extern "C" cudaError_t mcfl_attr_transport_f64(int variant, int *block, int *blocks_per_sm, int *regs);
typedef cudaError_t (*LaunchFn)(const McflLaunch *, int, int, cudaStream_t);
typedef cudaError_t (*AttrFn)(int, int *, int *, int *);
/* The transport kernel build of a math mode (MCFL_MATH_*). */
inline LaunchFn launch_fn(int math) {
  return math == MCFL_MATH_FAST  ? mcfl_launch_transport_fast
         : math == MCFL_MATH_F64 ? mcfl_launch_transport_f64
                                 : mcfl_launch_transport_exact;
}
inline AttrFn attr_fn(int math) {
  return math == MCFL_MATH_FAST  ? mcfl_attr_transport_fast
         : math == MCFL_MATH_F64 ? mcfl_attr_transport_f64
                                 : mcfl_attr_transport_exact;
}
constexpr int MCFL_N_VARIANTS = 3;

/* engine.cpp: one emission run from one voxel with the medium's excitation
 * table (DoOneSimulationFl), raw 64-bit images */
int run_single_voxel_emission(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run, unsigned int voxel,
                              unsigned long long *R, unsigned long long *T, unsigned long long *stats);

/* run.cpp: the label + free-radius map of voxel-boundary stepping, built on
 * the medium's first such run (synchronously on the context's stream) */
int ensure_free_map(mcfl_ctx *c, const mcfl_medium *m);

/* mci.cpp */
void simulation_geometry(const mcfl_simulation *sim, float *half_x, float *half_y, float *esp, float *g);
/* Detector-array positions of time-resolved detectors, as the reference
 * computes them (CUDAMCFLmain.cu:94-100, single precision). */
void time_positions(const mcfl_time_detectors &td, float *px, float *py);

} // namespace mcfl

unsigned long long next_medium_serial();

struct mcfl_medium {
  mcfl_ctx *ctx = nullptr;
  /* distinct for every medium a process creates: recorded graphs carry the
   * medium's geometry by value, and a freed medium's address can come back */
  unsigned long long serial = 0;
  mcfl::DevBuf labels, prop_exc, prop_emi, lab_exc, lab_emi, fl, fmap;
  /* voxel-boundary stepping: 1/mu_t with mu_t = mua + mus at excitation and
   * muaf + mus at emission (the fluorophore's absorption included) */
  mcfl::DevBuf prop_exc_x, prop_emi_x, lab_exc_x, lab_emi_x;
  /* voxel-boundary stepping: label | free radius << 8 per voxel, built on
   * the first such run (mcfl::ensure_free_map) */
  mutable mcfl::DevBuf lab16;
  const float *prop_of(bool emission, bool exact) const {
    return (exact ? (emission ? prop_emi_x : prop_exc_x) : (emission ? prop_emi : prop_exc)).as<float>();
  }
  const float *lab_of(bool emission, bool exact) const {
    return (exact ? (emission ? lab_emi_x : lab_exc_x) : (emission ? lab_emi : lab_exc)).as<float>();
  }
  int nx = 0, ny = 0, nz = 0;
  uint32_t total = 0;
  float hx = 0, hy = 0, esp = 0, gx = 0, gy = 0, gz = 0;
  int n_bulks = 0;
  bool has_fmap = false;
  std::vector<mcfl_bulk> bulks;
  size_t bytes = 0;
  /* layered medium (bulk method 1) */
  bool layered = false;
  int n_layers = 0;
  mcfl::DevBuf layer_tab;
  std::vector<float> z_min, z_max; /* per layer, host copies */
};

struct mcfl_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  mcfl::DevBuf mult;       /* 32768 multipliers */
  mcfl::DevBuf jobs;       /* job table */
  mcfl::DevBuf counters;   /* ticket counters and ticket ends */
  mcfl::DevBuf saved;      /* parked photons of budgeted launches */
  /* run workspace */
  mcfl::DevBuf R, T, fhd, R128, T128, stats, vox, q, block_counts, outd;
  mcfl::DevBuf tpos, tarr; /* time-resolved detector positions and tallies */
  /* pinned staging for job tables and results read back after a launch */
  McflJob *h_jobs = nullptr;
  size_t h_jobs_cap = 0;
  unsigned long long *h_out = nullptr;
  size_t h_out_cap = 0;
  /* recorded launch sequences replayed as CUDA graphs */
  cudaGraphExec_t graph_run = nullptr, graph_batch = nullptr;
  std::string graph_run_key, graph_batch_key;
  unsigned graph_run_kernels = 0, graph_batch_kernels = 0;
  int use_graphs = 1;
  std::string graph_error; /* why graphs were switched off, if they were */
  mcfl::DevBuf bR, bT, bstats, bcnt, seg_scale; /* batch workspace */
  int math = MCFL_MATH_EXACT;
  int block = 256;   /* threads per block, clamped to the variant's bound */
  int variant = 0;   /* occupancy variant of the single-medium kernel */
  /* photon-hitting-density tally: 0 one add per pass, 1 sums held in a
   * register (kernel variants 7..9), 2 adds aggregated per warp (14..16) */
  int phd_agg = 0;
  int pass_form = 0; /* 1: the pass with every test as its own branch (kernel variants 11..13) */
  /* the occupancy variant of the emission phase's launch (-1: variant) */
  int variant_fl = -1;
  /* the single-medium kernel variant the launches use (fl: an emission
   * launch, which tallies no hitting density) */
  int variant_code(bool fl = false) const {
    const int v = fl && variant_fl >= 0 ? variant_fl : variant;
    return v + (phd_agg == 1 ? 7 : phd_agg == 2 ? 14 : pass_form ? 11 : 0);
  }
  /* occupancy variant of the mixed-media kernel: 256 x 4 measured 2-4 %
   * faster than 128 x 7 on 24 requests of 5 media in one launch */
  int mixed_variant = 1;
  /* the mixed-media kernel variant the launches use (McflLaunch::variant) */
  int mixed_code() const { return mixed_variant + (pass_form ? 3 : 0); }
  int blocks_per_sm = 0;
  uint32_t step_cap = 1u << 24;
  uint32_t relaunch = 1; /* McflLaunch::relaunch_min */
  int l2_window = 0;            /* 1: persisting-L2 window over the medium's labels */
  size_t l2_persist_bytes = 0;  /* persisting set-aside this context asked for */
  size_t l2_max_window = 0;     /* cudaDevAttrMaxAccessPolicyWindowSize */
  unsigned long long launches = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

  /* Grid (SMs x resident blocks) and threads per block of the single-medium
   * (uniform) or mixed-media kernel under the current options. */
  int grid_for(bool uniform, int *block_out, int *bps_out = nullptr, bool time = false, bool exact = false,
               bool fl = false);
  int attr(bool uniform, int *block, int *bps, int *regs, bool time = false, bool exact = false, bool fl = false);
  cudaError_t launch_transport(const McflLaunch &L, int grid, int block_size);
};

#endif
