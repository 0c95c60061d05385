/*
 * Allocation-free batched excitation run (mcfl_batch_run_noalloc).
 *
 * Some callers cannot allocate device memory: code that runs inside another
 * framework's memory pool or arena, that must not trigger the implicit
 * synchronisation of cudaMalloc/cudaFree, or that is only handed device
 * buffers it may read and write.  This entry point serves them: the caller
 * passes the medium and the output images on the device, and the scratch the
 * persistent kernel needs (its ticket counter, its job table, the label
 * records and the MWC multiplier table) lives in one file-scope __device__ array of fixed size,
 * which every GPU that loads the library holds until the process exits.
 *
 * Limits and rules:
 *   - at most MCFL_NOALLOC_MAX_JOBS simulations per call (the job table's
 *     size); more is rejected with MCFL_E_RANGE;
 *   - the first call in a CUDA context (the device's primary context, or any
 *     context the caller made current), with that context current, resolves
 *     the array's device address (cudaGetSymbolAddress) and writes the
 *     multiplier table into it; make that first call before any stream
 *     capture (it is refused with MCFL_E_STATE while the stream captures).
 *     A new context on the device (after cudaDeviceReset, for instance) has
 *     its own copy of the array, which its first call sets up again;
 *   - every call shares the array and leaves its contents behind; the ticket
 *     counter is cleared at the start of each call, so calls that run one after
 *     another are independent, but calls that overlap on the GPU (other
 *     streams, other host threads) race on the array;
 *   - the job table travels to the GPU as a kernel parameter (by value), so
 *     nothing on the GPU refers to host memory of the call after it returns;
 *   - the output images and stats are cleared by the call, then accumulated
 *     by the kernel; the call is asynchronous on the given stream.
 * Nothing here calls cudaMalloc, cudaFree or any allocating library routine.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstring>
#include <map>
#include <mutex>

#include "mcfl_internal.h"
#include "portable_math.h"

using namespace mcfl;

namespace {

struct NoallocScratch {
  unsigned long long counter;
  unsigned long long pad[31]; /* jobs start 256 bytes in */
  McflJob jobs[MCFL_NOALLOC_MAX_JOBS];
  float lab[MCFL_MAX_LABELS * MCFL_LAB_FLOATS]; /* label records derived from the caller's table */
  uint32_t mult[32768];
};

/* A call's job table, passed by value (19.5 KB of kernel parameters). */
struct JobStage {
  McflJob jobs[MCFL_NOALLOC_MAX_JOBS];
};
static_assert(sizeof(JobStage) + 64 < 32764, "job table beyond the kernel parameter limit");

/* Writes the call's job table into the scratch, clears the ticket counter and
 * builds the label records from the caller's (mutr, mu_a, g, n) table. */
__global__ void noalloc_prepare(const __grid_constant__ JobStage t, uint32_t n_jobs, const float4 *prop,
                                uint32_t n_labels, NoallocScratch *sc) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nthreads = gridDim.x * blockDim.x;
  const uint4 *src = reinterpret_cast<const uint4 *>(t.jobs);
  uint4 *dst = reinterpret_cast<uint4 *>(sc->jobs);
  const uint32_t words = n_jobs * (uint32_t)(sizeof(McflJob) / sizeof(uint4));
  for (uint32_t i = tid; i < words; i += nthreads) dst[i] = src[i];
  for (uint32_t i = tid; i < n_labels; i += nthreads) {
    const float4 q = prop[i];
    mcfl_label_record(q.x, q.y, q.z, q.w, sc->lab + (size_t)i * MCFL_LAB_FLOATS);
  }
  if (tid == 0) sc->counter = 0ull;
}
static_assert(sizeof(McflJob) % sizeof(uint4) == 0, "job records are copied as 16-byte words");

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoallocScratch)];

typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

std::mutex g_mu;
/* set-up done, per CUDA context (by the context's process-unique ID) */
std::map<unsigned long long, NoallocScratch *> g_scratch;

/* The process-unique ID of the calling thread's current CUDA context (driver
 * entry points looked up through the runtime, so the library does not link
 * the driver library). */
int current_context_id(unsigned long long *id) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  if (!get_current || !get_id) {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = cudaDriverEntryPointSymbolNotFound;
    void *f1 = nullptr, *f2 = nullptr;
    MCFL_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault, &q1));
    MCFL_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return mcfl::fail(MCFL_E_STATE, "noalloc: driver entry points cuCtxGetCurrent/cuCtxGetId not found");
    get_current = (PfnCtxGetCurrent)f1;
    get_id = (PfnCtxGetId)f2;
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return mcfl::fail(MCFL_E_STATE, "noalloc: no current CUDA context");
  if (get_id(ctx, id) != CUDA_SUCCESS) return mcfl::fail(MCFL_E_STATE, "noalloc: cuCtxGetId failed");
  return MCFL_OK;
}

/* Device address of the scratch array in the current context, set up on the
 * context's first call (refused while stream s captures: the set-up copies
 * the multiplier table synchronously). */
int scratch_for_current_context(cudaStream_t s, NoallocScratch **out) {
  /* resolves (and, on a context's first use, creates) the current context */
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return mcfl::cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
  unsigned long long id = 0;
  int rc = current_context_id(&id);
  if (rc != MCFL_OK) return rc;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_scratch.find(id);
  if (it != g_scratch.end() && it->second == (NoallocScratch *)p) {
    *out = it->second;
    return MCFL_OK;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MCFL_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone)
    return mcfl::fail(MCFL_E_STATE, "noalloc: the first call in a CUDA context must come before stream capture");
  const std::vector<uint32_t> &tab = mcfl::mwc_table();
  if (tab.size() != mcfl::kMwcTableEntries + 1) return mcfl::fail(MCFL_E_STATE, "multiplier table incomplete");
  e = cudaMemcpy((char *)p + offsetof(NoallocScratch, mult), tab.data() + 1, mcfl::kMwcTableEntries * 4,
                 cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return mcfl::cuda_fail(e, "noalloc multiplier upload");
  g_scratch[id] = (NoallocScratch *)p;
  *out = (NoallocScratch *)p;
  return MCFL_OK;
}

} // namespace

extern "C" int mcfl_batch_run_noalloc(int math, const unsigned char *d_labels, const float *d_prop, int nx, int ny,
                                      int nz, float half_x, float half_y, float thickness, const float *vox_per_cm,
                                      int n_bulks, const mcfl_run_desc *runs, int n, unsigned long long *d_R,
                                      unsigned long long *d_T, unsigned long long *d_stats, void *stream) {
  using mcfl::fail;
  if (n < 1) return fail(MCFL_E_ARG, "noalloc: at least one simulation");
  if (n > MCFL_NOALLOC_MAX_JOBS) return fail(MCFL_E_RANGE, "noalloc: more than MCFL_NOALLOC_MAX_JOBS simulations");
  if (!d_labels || !d_prop || !runs || !d_R || !d_T || !d_stats || !vox_per_cm)
    return fail(MCFL_E_ARG, "noalloc: null pointer");
  if (math != MCFL_MATH_EXACT && math != MCFL_MATH_FAST) return fail(MCFL_E_ARG, "noalloc: unknown math");
  if (nx <= 0 || ny <= 0 || nz <= 0 || (unsigned long long)nx * ny * nz >= 0xFFFFFFFFull)
    return fail(MCFL_E_ARG, "noalloc: bad grid");
  if (n_bulks < 1 || n_bulks > MCFL_MAX_BULKS) return fail(MCFL_E_RANGE, "noalloc: n_bulks out of range");
  if ((uintptr_t)d_prop % 16 != 0) return fail(MCFL_E_ARG, "noalloc: d_prop must be 16-byte aligned");
  if ((uintptr_t)d_R % 8 != 0 || (uintptr_t)d_T % 8 != 0 || (uintptr_t)d_stats % 8 != 0)
    return fail(MCFL_E_ARG, "noalloc: d_R, d_T and d_stats must be 8-byte aligned");
  const mcfl_detector det = runs[0].det;
  for (int i = 0; i < n; ++i) {
    const mcfl_run_desc &r = runs[i];
    if (r.det.nx <= 0 || r.det.ny <= 0 || !(r.det.dx > 0) || !(r.det.dy > 0))
      return fail(MCFL_E_ARG, "noalloc: bad detector");
    if (r.photons == 0 || r.photons_per_voxel || r.fluence) return fail(MCFL_E_ARG, "noalloc: excitation images only");
    if (r.tdet.nx || r.exact_stepping) return fail(MCFL_E_ARG, "noalloc: the reference's stepping, no time detectors");
    if (r.start_weight == 0) return fail(MCFL_E_ARG, "noalloc: start_weight must be given");
    if (r.det.nx != det.nx || r.det.ny != det.ny) return fail(MCFL_E_ARG, "noalloc: detectors must share a size");
    if (r.source.kind != MCFL_SOURCE_GAUSS_BEAM && r.source.kind != MCFL_SOURCE_WIDEFIELD)
      return fail(MCFL_E_ARG, "noalloc: unknown source kind");
  }
  cudaStream_t s = (cudaStream_t)stream;
  NoallocScratch *sc = nullptr;
  int rc = scratch_for_current_context(s, &sc);
  if (rc != MCFL_OK) return rc;
  cudaGetLastError();
  const size_t xy = (size_t)det.nx + (size_t)det.nx * det.ny;
  JobStage stage;
  std::memset(&stage, 0, sizeof(stage));
  McflJob *jobs = stage.jobs;
  unsigned long long tickets = 0;
  for (int i = 0; i < n; ++i) {
    const mcfl_run_desc &r = runs[i];
    McflJob &j = jobs[i];
    j.labels = d_labels;
    j.prop = d_prop;
    j.lab = sc->lab;
    j.hx = half_x; j.hy = half_y; j.esp = thickness;
    j.gx = vox_per_cm[0]; j.gy = vox_per_cm[1]; j.gz = vox_per_cm[2];
    j.nx = (uint32_t)nx; j.ny = (uint32_t)ny; j.nz = (uint32_t)nz;
    j.total = (uint32_t)nx * (uint32_t)ny * (uint32_t)nz;
    j.last_label = (uint32_t)n_bulks + 1u;
    j.src_kind = r.source.kind == MCFL_SOURCE_WIDEFIELD ? MCFL_SRC_WIDEFIELD : MCFL_SRC_GAUSS_BEAM;
    j.sx = r.source.x; j.sy = r.source.y; j.sz = r.source.z;
    j.src_w = r.source.width; j.src_h = r.source.height;
    j.start_weight = r.start_weight;
    j.det_x0 = r.det.x0; j.det_y0 = r.det.y0; j.det_dx = r.det.dx; j.det_dy = r.det.dy;
    j.size_x = (r.det.dx * (float)r.det.nx) / 2.0f;
    j.size_y = (r.det.dy * (float)r.det.ny) / 2.0f;
    j.det_nx = (uint32_t)r.det.nx;
    j.xy_size = (uint32_t)xy;
    j.R = d_R + (size_t)i * xy;
    j.T = d_T + (size_t)i * xy;
    j.stats = d_stats + (size_t)i * MCFL_ST_COUNT;
    j.key = mcfl_stream_key(r.seed_exc, 0);
    j.rng_offset = r.photon_offset;
    j.launch_rng_reuse = r.launch_rng_reuse ? 1u : 0u;
    j.ticket_begin = tickets;
    j.photons = r.photons;
    tickets += r.photons;
  }
  MCFL_CUDA_TRY(cudaMemsetAsync(d_R, 0, (size_t)n * xy * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(d_T, 0, (size_t)n * xy * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(d_stats, 0, (size_t)n * MCFL_ST_COUNT * 8, s));
  const uint32_t n_labels = (uint32_t)n_bulks + 2u;
  noalloc_prepare<<<8, 256, 0, s>>>(stage, (uint32_t)n, (const float4 *)d_prop, n_labels, sc);
  MCFL_CUDA_TRY(cudaGetLastError());
  McflLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.jobs = sc->jobs;
  L.n_jobs = (uint32_t)n;
  L.ticket_counter = &sc->counter;
  L.ticket_end = tickets;
  L.mult = sc->mult;
  L.step_cap = 1u << 24;
  L.uniform_medium = 1;
  L.med.labels = d_labels;
  L.med.prop = d_prop;
  L.med.lab = sc->lab;
  L.med.n_labels = n_labels;
  L.med.fhd = nullptr;
  L.med.hx = half_x; L.med.hy = half_y; L.med.esp = thickness;
  L.med.gx = vox_per_cm[0]; L.med.gy = vox_per_cm[1]; L.med.gz = vox_per_cm[2];
  L.med.nx = (uint32_t)nx; L.med.ny = (uint32_t)ny; L.med.total = jobs[0].total;
  L.med.last_label = (uint32_t)n_bulks + 1u;
  int block = 0; /* variant 0's own: 256 threads */
  int dev = 0, sms = 0, bps = 0, regs = 0;
  MCFL_CUDA_TRY(cudaGetDevice(&dev));
  MCFL_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MCFL_CUDA_TRY(math == MCFL_MATH_FAST ? mcfl_attr_transport_fast(0, &block, &bps, &regs)
                                       : mcfl_attr_transport_exact(0, &block, &bps, &regs));
  if (bps < 1) bps = 1;
  MCFL_CUDA_TRY(math == MCFL_MATH_FAST ? mcfl_launch_transport_fast(&L, bps * sms, block, s)
                                       : mcfl_launch_transport_exact(&L, bps * sms, block, s));
  return MCFL_OK;
}
