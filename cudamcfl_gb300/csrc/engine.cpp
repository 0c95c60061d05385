/*
 * Host engine of libmcfl: GPU context, device-resident media and the
 * two-phase (excitation + emission) run.
 *
 * A run replaces the reference's DoOneSimulation / DoOneSimulationFl /
 * voxel-loop sequence (CUDAMCFLmain.cu:60-288,409-652) with four launches on
 * one stream and no host round trip between them:
 *   1. transport, excitation job (Gaussian beam or wide field), R/T images
 *      and the photon hitting density;
 *   2. emission-list build (engine_kernels.cu): every emitting voxel with its
 *      fixed-point weight, and the emission job's photon count;
 *   3. transport, one emission job over all emitting voxels;
 *   4. FP64 normalisation of the requested images.
 * All scratch lives in grow-only buffers of the context, so repeated runs
 * allocate nothing.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>

#include "mcfl_internal.h"
#include "portable_math.h"

namespace mcfl {

namespace {
thread_local std::string g_last_error;
}

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *where) {
  return fail(MCFL_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

cudaError_t DevBuf::reserve(size_t n) {
  if (n <= bytes && p) return cudaSuccess;
  release();
  cudaError_t e = cudaMalloc(&p, n ? n : 16);
  if (e != cudaSuccess) {
    p = nullptr;
    bytes = 0;
    return e;
  }
  bytes = n;
  return cudaSuccess;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

} // namespace mcfl

using namespace mcfl;

#define MCFL_CUDA_TRY(call)                                   \
  do {                                                        \
    cudaError_t e__ = (call);                                 \
    if (e__ != cudaSuccess) return cuda_fail(e__, #call);     \
  } while (0)

int mcfl_ctx::grid_for(int block_size, int *bps_out) {
  int bps = 0, regs = 0;
  cudaError_t e = math == MCFL_MATH_FAST ? mcfl_attr_transport_fast(block_size, &bps, &regs)
                                         : mcfl_attr_transport_exact(block_size, &bps, &regs);
  if (e != cudaSuccess || bps <= 0) bps = 1;
  if (blocks_per_sm > 0 && blocks_per_sm < bps) bps = blocks_per_sm;
  if (bps_out) *bps_out = bps;
  return bps * sm_count;
}

cudaError_t mcfl_ctx::launch_transport(const McflLaunch &L, int grid, int block_size) {
  ++launches;
  return math == MCFL_MATH_FAST ? mcfl_launch_transport_fast(&L, grid, block_size, stream)
                                : mcfl_launch_transport_exact(&L, grid, block_size, stream);
}

extern "C" const char *mcfl_last_error(void) { return g_last_error.c_str(); }

extern "C" int mcfl_create(int device, mcfl_ctx **out) {
  if (!out) return fail(MCFL_E_ARG, "mcfl_create: null output");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(MCFL_E_CUDA, "mcfl_create: no CUDA device");
  if (device < 0) MCFL_CUDA_TRY(cudaGetDevice(&device));
  if (device >= ndev) return fail(MCFL_E_ARG, "mcfl_create: device out of range");
  MCFL_CUDA_TRY(cudaSetDevice(device));
  mcfl_ctx *c = new mcfl_ctx();
  c->device = device;
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaGetDeviceProperties");
  }
  c->sm_count = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaStreamCreate");
  }
  c->stream = c->own_stream;
  for (auto &ev : c->ev) cudaEventCreate(&ev);
  const std::vector<uint32_t> &tab = mwc_table();
  if (tab.size() != kMwcTableEntries + 1) {
    mcfl_destroy(c);
    return fail(MCFL_E_STATE, "multiplier table incomplete");
  }
  e = c->mult.reserve(kMwcTableEntries * sizeof(uint32_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(c->mult.p, tab.data() + 1, kMwcTableEntries * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = c->counters.reserve(16 * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    mcfl_destroy(c);
    return cuda_fail(e, "mcfl_create");
  }
  *out = c;
  return MCFL_OK;
}

extern "C" void mcfl_destroy(mcfl_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->own_stream) cudaStreamSynchronize(c->own_stream);
  for (auto &ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

extern "C" int mcfl_set_option(mcfl_ctx *c, const char *key, long long v) {
  if (!c || !key) return fail(MCFL_E_ARG, "mcfl_set_option: null argument");
  const std::string k(key);
  if (k == "math") {
    if (v != MCFL_MATH_EXACT && v != MCFL_MATH_FAST) return fail(MCFL_E_ARG, "math: 0 (exact) or 1 (fast)");
    c->math = (int)v;
  } else if (k == "block") {
    if (v < 32 || v > 256 || (v % 32)) return fail(MCFL_E_ARG, "block: a multiple of 32 in [32, 256]");
    c->block = (int)v;
  } else if (k == "blocks_per_sm") {
    if (v < 0 || v > 64) return fail(MCFL_E_ARG, "blocks_per_sm: 0..64");
    c->blocks_per_sm = (int)v;
  } else if (k == "step_cap") {
    if (v < 1 || v > 0x7fffffffLL) return fail(MCFL_E_ARG, "step_cap: 1..2^31-1");
    c->step_cap = (uint32_t)v;
  } else if (k == "l2_window") {
    c->l2_window = v ? 1 : 0;
  } else {
    return fail(MCFL_E_ARG, "unknown option " + k);
  }
  return MCFL_OK;
}

extern "C" long long mcfl_get_option(mcfl_ctx *c, const char *key) {
  if (!c || !key) return -1;
  const std::string k(key);
  if (k == "math") return c->math;
  if (k == "block") return c->block;
  if (k == "blocks_per_sm") return c->blocks_per_sm;
  if (k == "step_cap") return c->step_cap;
  if (k == "l2_window") return c->l2_window;
  if (k == "sm_count") return c->sm_count;
  if (k == "grid") return c->grid_for(c->block);
  if (k == "regs") {
    int bps = 0, regs = 0;
    if (c->math == MCFL_MATH_FAST) mcfl_attr_transport_fast(c->block, &bps, &regs);
    else mcfl_attr_transport_exact(c->block, &bps, &regs);
    return regs;
  }
  return -1;
}

extern "C" int mcfl_set_stream(mcfl_ctx *c, void *stream) {
  if (!c) return fail(MCFL_E_ARG, "mcfl_set_stream: null context");
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return MCFL_OK;
}

extern "C" unsigned long long mcfl_launch_count(const mcfl_ctx *c) { return c ? c->launches : 0ull; }

/* ------------------------------------------------------------------ media */

extern "C" int mcfl_medium_create(mcfl_ctx *c, const mcfl_medium_desc *d, mcfl_medium **out) {
  if (!c || !d || !out || !d->labels || !d->bulks) return fail(MCFL_E_ARG, "mcfl_medium_create: null argument");
  *out = nullptr;
  if (d->nx <= 0 || d->ny <= 0 || d->nz <= 0) return fail(MCFL_E_ARG, "medium: non-positive grid");
  const unsigned long long total = (unsigned long long)d->nx * d->ny * d->nz;
  if (total >= 0xFFFFFFFFull) return fail(MCFL_E_RANGE, "medium: more than 2^32-1 voxels");
  if (d->n_bulks < 1 || d->n_bulks > MCFL_MAX_BULKS) return fail(MCFL_E_RANGE, "medium: n_bulks out of range");
  if (!(d->half_x > 0 && d->half_y > 0 && d->thickness > 0)) return fail(MCFL_E_ARG, "medium: non-positive extent");
  for (unsigned long long i = 0; i < total; ++i)
    if (d->labels[i] > (unsigned)d->n_bulks + 1u) return fail(MCFL_E_ARG, "medium: label beyond n_bulks+1");
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  mcfl_medium *m = new mcfl_medium();
  m->ctx = c;
  m->nx = d->nx;
  m->ny = d->ny;
  m->nz = d->nz;
  m->total = (uint32_t)total;
  m->hx = d->half_x;
  m->hy = d->half_y;
  m->esp = d->thickness;
  m->gx = d->vox_per_cm[0];
  m->gy = d->vox_per_cm[1];
  m->gz = d->vox_per_cm[2];
  m->n_bulks = d->n_bulks;
  m->bulks.assign(d->bulks, d->bulks + d->n_bulks + 2);
  const int nl = d->n_bulks + 2;
  std::vector<float> pe(4 * (size_t)nl), pm(4 * (size_t)nl), fl(2 * (size_t)nl);
  for (int i = 0; i < nl; ++i) {
    const mcfl_bulk &b = d->bulks[i];
    pe[4 * i + 0] = b.mutr; pe[4 * i + 1] = b.mua; pe[4 * i + 2] = b.g; pe[4 * i + 3] = b.n;
    pm[4 * i + 0] = b.mutr; pm[4 * i + 1] = b.muaf; pm[4 * i + 2] = b.g; pm[4 * i + 3] = b.n;
    fl[2 * i + 0] = b.eY; fl[2 * i + 1] = b.albedof;
  }
  cudaError_t e = m->labels.reserve(total);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->labels.p, d->labels, total, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = m->prop_exc.reserve(pe.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->prop_exc.p, pe.data(), pe.size() * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = m->prop_emi.reserve(pm.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->prop_emi.p, pm.data(), pm.size() * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = m->fl.reserve(fl.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->fl.p, fl.data(), fl.size() * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && d->fluor_map) {
    m->has_fmap = true;
    e = m->fmap.reserve(total * 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(m->fmap.p, d->fluor_map, total * 4, cudaMemcpyHostToDevice, c->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "mcfl_medium_create");
  }
  m->bytes = m->labels.bytes + m->prop_exc.bytes + m->prop_emi.bytes + m->fl.bytes + m->fmap.bytes;
  *out = m;
  return MCFL_OK;
}

extern "C" void mcfl_medium_free(mcfl_medium *m) {
  if (!m) return;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(m->ctx->stream);
  delete m;
}

extern "C" size_t mcfl_medium_bytes(const mcfl_medium *m) { return m ? m->bytes : 0; }

/* -------------------------------------------------------------------- run */

namespace {

unsigned int default_start_weight(const mcfl_medium *m) {
  /* CUDAMCFLio.cu:639-652: specular loss between the medium above and label 1 */
  const double n1 = m->bulks[0].n, n2 = m->bulks[1].n;
  double r = (n1 - n2) / (n1 + n2);
  r = r * r;
  return (unsigned int)((double)0xFFFFFFFF * (1 - r));
}

void fill_medium(McflJob &j, const mcfl_medium *m, bool emission) {
  j.labels = m->labels.as<uint8_t>();
  j.prop = emission ? m->prop_emi.as<float>() : m->prop_exc.as<float>();
  j.hx = m->hx;
  j.hy = m->hy;
  j.esp = m->esp;
  j.gx = m->gx;
  j.gy = m->gy;
  j.gz = m->gz;
  j.nx = (uint32_t)m->nx;
  j.ny = (uint32_t)m->ny;
  j.nz = (uint32_t)m->nz;
  j.total = m->total;
  j.last_label = (uint32_t)m->n_bulks + 1u;
}

void fill_detector(McflJob &j, const mcfl_detector &d) {
  j.det_x0 = d.x0;
  j.det_y0 = d.y0;
  j.det_dx = d.dx;
  j.det_dy = d.dy;
  j.size_x = (d.dx * (float)d.nx) / 2.0f; /* CUDAMCFLtransport.cu:259-260 */
  j.size_y = (d.dy * (float)d.ny) / 2.0f;
  j.det_nx = (uint32_t)d.nx;
  j.xy_size = (uint32_t)(d.nx + d.nx * d.ny);
}

} // namespace

extern "C" int mcfl_run(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run, mcfl_run_out *out) {
  if (!c || !m || !run) return fail(MCFL_E_ARG, "mcfl_run: null argument");
  if (m->ctx != c) return fail(MCFL_E_ARG, "mcfl_run: medium of another context");
  const mcfl_detector &det = run->det;
  if (det.nx <= 0 || det.ny <= 0 || !(det.dx > 0) || !(det.dy > 0)) return fail(MCFL_E_ARG, "mcfl_run: bad detector");
  if (run->photons == 0) return fail(MCFL_E_ARG, "mcfl_run: zero photons");
  if (run->source.kind != MCFL_SOURCE_GAUSS_BEAM && run->source.kind != MCFL_SOURCE_WIDEFIELD)
    return fail(MCFL_E_ARG, "mcfl_run: unknown source kind");
  const bool emission = run->photons_per_voxel > 0;
  const bool fluence = emission || run->fluence;
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  const size_t xy = (size_t)det.nx + (size_t)det.nx * det.ny;
  const size_t nv = m->total;

  MCFL_CUDA_TRY(c->R.reserve(xy * 8));
  MCFL_CUDA_TRY(c->T.reserve(xy * 8));
  MCFL_CUDA_TRY(c->stats.reserve(2 * MCFL_ST_COUNT * 8));
  MCFL_CUDA_TRY(c->jobs.reserve(2 * sizeof(McflJob)));
  if (fluence) MCFL_CUDA_TRY(c->fhd.reserve(nv * 8));
  if (emission) {
    MCFL_CUDA_TRY(c->R128.reserve(xy * 16));
    MCFL_CUDA_TRY(c->T128.reserve(xy * 16));
    MCFL_CUDA_TRY(c->vox.reserve(nv * 4));
    MCFL_CUDA_TRY(c->q.reserve(nv * 8));
    MCFL_CUDA_TRY(c->block_counts.reserve(emission_prep_blocks((uint32_t)nv) * 4 + 16));
  }
  MCFL_CUDA_TRY(cudaMemsetAsync(c->R.p, 0, xy * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->T.p, 0, xy * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->stats.p, 0, 2 * MCFL_ST_COUNT * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->counters.p, 0, 16 * 8, s));
  if (fluence) MCFL_CUDA_TRY(cudaMemsetAsync(c->fhd.p, 0, nv * 8, s));
  if (emission) {
    MCFL_CUDA_TRY(cudaMemsetAsync(c->R128.p, 0, xy * 16, s));
    MCFL_CUDA_TRY(cudaMemsetAsync(c->T128.p, 0, xy * 16, s));
  }

  McflJob jobs[2];
  std::memset(jobs, 0, sizeof(jobs));
  McflJob &je = jobs[0];
  fill_medium(je, m, false);
  fill_detector(je, det);
  je.src_kind = run->source.kind == MCFL_SOURCE_WIDEFIELD ? MCFL_SRC_WIDEFIELD : MCFL_SRC_GAUSS_BEAM;
  je.sx = run->source.x;
  je.sy = run->source.y;
  je.sz = run->source.z;
  je.src_w = run->source.width;
  je.src_h = run->source.height;
  je.start_weight = run->start_weight ? run->start_weight : default_start_weight(m);
  je.fhd_on = fluence ? 1u : 0u;
  je.R = c->R.as<unsigned long long>();
  je.T = c->T.as<unsigned long long>();
  je.fhd = fluence ? c->fhd.as<unsigned long long>() : nullptr;
  je.stats = c->stats.as<unsigned long long>();
  je.key = mcfl_stream_key(run->seed_exc, 0);
  je.rng_offset = 0;
  je.ticket_begin = 0;
  je.photons = run->photons;
  McflJob &jf = jobs[1];
  if (emission) {
    fill_medium(jf, m, true);
    fill_detector(jf, det);
    jf.src_kind = MCFL_SRC_VOXELS;
    jf.src_vox = c->vox.as<uint32_t>();
    jf.src_q = c->q.as<uint64_t>();
    jf.per_voxel = run->photons_per_voxel;
    jf.fhd_on = 0;
    jf.R128 = c->R128.as<unsigned long long>();
    jf.T128 = c->T128.as<unsigned long long>();
    jf.stats = c->stats.as<unsigned long long>() + MCFL_ST_COUNT;
    jf.key = mcfl_stream_key(run->seed_fl, 1);
    jf.rng_offset = 0;
    jf.ticket_begin = 0;
    jf.photons = 0; /* written by the list build */
  }
  MCFL_CUDA_TRY(cudaMemcpyAsync(c->jobs.p, jobs, sizeof(jobs), cudaMemcpyHostToDevice, s));

  unsigned long long *cnt = c->counters.as<unsigned long long>();
  const int grid = c->grid_for(c->block);
  McflLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.jobs = c->jobs.as<McflJob>();
  L.n_jobs = 1;
  L.max_iters = 0;
  L.ticket_counter = cnt + 0;
  L.ticket_end = run->photons;
  L.mult = c->mult.as<uint32_t>();
  L.step_cap = c->step_cap;
  MCFL_CUDA_TRY(cudaEventRecord(c->ev[0], s));
  MCFL_CUDA_TRY(c->launch_transport(L, grid, c->block));
  MCFL_CUDA_TRY(cudaEventRecord(c->ev[1], s));
  if (emission) {
    MCFL_CUDA_TRY(mcfl_launch_emission_prep(m->labels.as<uint8_t>(), m->fl.as<float2>(),
                                            c->fhd.as<unsigned long long>(), m->has_fmap ? m->fmap.as<float>() : nullptr,
                                            m->total, run->photons, run->photons_per_voxel,
                                            c->block_counts.as<uint32_t>(), c->vox.as<uint32_t>(), c->q.as<uint64_t>(),
                                            cnt + 2, c->jobs.as<McflJob>() + 1, cnt + 3, s));
    c->launches += 3;
    McflLaunch Lf = L;
    Lf.jobs = c->jobs.as<McflJob>() + 1;
    Lf.ticket_counter = cnt + 1;
    Lf.ticket_end_dev = cnt + 3;
    MCFL_CUDA_TRY(cudaEventRecord(c->ev[2], s));
    MCFL_CUDA_TRY(c->launch_transport(Lf, grid, c->block));
    MCFL_CUDA_TRY(cudaEventRecord(c->ev[3], s));
  }

  /* FP64 normalisation on the GPU, into one scratch block */
  size_t nd = 0;
  if (out) {
    nd += (out->R ? xy : 0) + (out->T ? xy : 0) + (out->phd && fluence ? nv : 0);
    nd += emission ? (out->flR ? xy : 0) + (out->flT ? xy : 0) : 0;
  }
  if (nd) MCFL_CUDA_TRY(c->outd.reserve(nd * 8));
  double *dd = c->outd.as<double>();
  const double scale2 = ((double)0xFFFFFFFF * (double)run->photons) * (double)det.dx * (double)det.dy;
  const double flnorm = ((double)run->photons_per_voxel * 4294967295.0) * ((double)det.dx * (double)det.dy);
  struct Pending { double *dev; double *host; size_t n; };
  std::vector<Pending> pend;
  if (out) {
    size_t off = 0;
    auto take = [&](size_t n) { double *p = dd + off; off += n; return p; };
    if (out->R) { double *p = take(xy); MCFL_CUDA_TRY(mcfl_launch_normalize_u64(c->R.as<unsigned long long>(), p, xy, scale2, s)); ++c->launches; pend.push_back({p, out->R, xy}); }
    if (out->T) { double *p = take(xy); MCFL_CUDA_TRY(mcfl_launch_normalize_u64(c->T.as<unsigned long long>(), p, xy, scale2, s)); ++c->launches; pend.push_back({p, out->T, xy}); }
    if (out->phd && fluence) { double *p = take(nv); MCFL_CUDA_TRY(mcfl_launch_normalize_phd(c->fhd.as<unsigned long long>(), p, nv, run->photons, s)); ++c->launches; pend.push_back({p, out->phd, nv}); }
    if (emission && out->flR) { double *p = take(xy); MCFL_CUDA_TRY(mcfl_launch_normalize_128(c->R128.as<unsigned long long>(), p, xy, flnorm, s)); ++c->launches; pend.push_back({p, out->flR, xy}); }
    if (emission && out->flT) { double *p = take(xy); MCFL_CUDA_TRY(mcfl_launch_normalize_128(c->T128.as<unsigned long long>(), p, xy, flnorm, s)); ++c->launches; pend.push_back({p, out->flT, xy}); }
  }
  if (out) {
    for (auto &pd : pend) MCFL_CUDA_TRY(cudaMemcpyAsync(pd.host, pd.dev, pd.n * 8, cudaMemcpyDeviceToHost, s));
    if (out->Rd) MCFL_CUDA_TRY(cudaMemcpyAsync(out->Rd, c->R.p, xy * 8, cudaMemcpyDeviceToHost, s));
    if (out->Tt) MCFL_CUDA_TRY(cudaMemcpyAsync(out->Tt, c->T.p, xy * 8, cudaMemcpyDeviceToHost, s));
    if (out->fhd && fluence) MCFL_CUDA_TRY(cudaMemcpyAsync(out->fhd, c->fhd.p, nv * 8, cudaMemcpyDeviceToHost, s));
    if (emission && out->flR128) MCFL_CUDA_TRY(cudaMemcpyAsync(out->flR128, c->R128.p, xy * 16, cudaMemcpyDeviceToHost, s));
    if (emission && out->flT128) MCFL_CUDA_TRY(cudaMemcpyAsync(out->flT128, c->T128.p, xy * 16, cudaMemcpyDeviceToHost, s));
  }
  unsigned long long st[2 * MCFL_ST_COUNT];
  unsigned long long cn[4];
  MCFL_CUDA_TRY(cudaMemcpyAsync(st, c->stats.p, sizeof(st), cudaMemcpyDeviceToHost, s));
  MCFL_CUDA_TRY(cudaMemcpyAsync(cn, c->counters.p, sizeof(cn), cudaMemcpyDeviceToHost, s));
  MCFL_CUDA_TRY(cudaStreamSynchronize(s));
  if (out) {
    std::memcpy(out->stats_exc, st, MCFL_ST_COUNT * 8);
    std::memcpy(out->stats_fl, st + MCFL_ST_COUNT, MCFL_ST_COUNT * 8);
    out->fl_voxels = emission ? (long long)cn[2] : 0;
    out->photons_fl = emission ? cn[3] : 0;
    const double launched = (double)run->photons * (double)je.start_weight;
    const double a = (double)st[MCFL_ST_ABSORBED], rt = (double)st[MCFL_ST_EXIT_TOP], tb = (double)st[MCFL_ST_EXIT_BOTTOM];
    const double lost = (double)st[MCFL_ST_R_LOSS] + (double)st[MCFL_ST_W0_LOSS] - (double)st[MCFL_ST_R_GAIN];
    out->energy_exc[0] = rt / launched;
    out->energy_exc[1] = tb / launched;
    out->energy_exc[2] = a / launched;
    out->energy_exc[3] = (launched - (a + rt + tb + lost)) / launched;
    cudaEventElapsedTime(&out->ms_exc, c->ev[0], c->ev[1]);
    out->ms_fl = 0.f;
    if (emission) cudaEventElapsedTime(&out->ms_fl, c->ev[2], c->ev[3]);
  }
  if (st[MCFL_ST_CAPPED] || st[MCFL_ST_COUNT + MCFL_ST_CAPPED])
    return fail(MCFL_E_CAPPED, "photons reached the per-photon pass cap");
  return MCFL_OK;
}

/* -------------------------------------------- one-voxel emission (plain) */

int mcfl::run_single_voxel_emission(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run, unsigned int voxel,
                                    unsigned long long *R, unsigned long long *T, unsigned long long *stats) {
  const mcfl_detector &det = run->det;
  const size_t xy = (size_t)det.nx + (size_t)det.nx * det.ny;
  cudaStream_t s = c->stream;
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  MCFL_CUDA_TRY(c->R128.reserve(xy * 16));
  MCFL_CUDA_TRY(c->T128.reserve(xy * 16));
  MCFL_CUDA_TRY(c->vox.reserve(64));
  MCFL_CUDA_TRY(c->q.reserve(64));
  MCFL_CUDA_TRY(c->stats.reserve(2 * MCFL_ST_COUNT * 8));
  MCFL_CUDA_TRY(c->jobs.reserve(2 * sizeof(McflJob)));
  const uint64_t one = 1;
  MCFL_CUDA_TRY(cudaMemcpyAsync(c->vox.p, &voxel, 4, cudaMemcpyHostToDevice, s));
  MCFL_CUDA_TRY(cudaMemcpyAsync(c->q.p, &one, 8, cudaMemcpyHostToDevice, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->R128.p, 0, xy * 16, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->T128.p, 0, xy * 16, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->stats.p, 0, MCFL_ST_COUNT * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->counters.p, 0, 8, s));
  McflJob j;
  std::memset(&j, 0, sizeof(j));
  fill_medium(j, m, false);
  fill_detector(j, det);
  j.src_kind = MCFL_SRC_VOXELS;
  j.src_vox = c->vox.as<uint32_t>();
  j.src_q = c->q.as<uint64_t>();
  j.per_voxel = (uint32_t)run->photons;
  j.R128 = c->R128.as<unsigned long long>();
  j.T128 = c->T128.as<unsigned long long>();
  j.stats = c->stats.as<unsigned long long>();
  j.key = mcfl_stream_key(run->seed_fl, 1);
  j.photons = run->photons;
  MCFL_CUDA_TRY(cudaMemcpyAsync(c->jobs.p, &j, sizeof(j), cudaMemcpyHostToDevice, s));
  McflLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.jobs = c->jobs.as<McflJob>();
  L.n_jobs = 1;
  L.ticket_counter = c->counters.as<unsigned long long>();
  L.ticket_end = run->photons;
  L.mult = c->mult.as<uint32_t>();
  L.step_cap = c->step_cap;
  MCFL_CUDA_TRY(c->launch_transport(L, c->grid_for(c->block), c->block));
  std::vector<unsigned long long> r(2 * xy), t(2 * xy);
  MCFL_CUDA_TRY(cudaMemcpyAsync(r.data(), c->R128.p, xy * 16, cudaMemcpyDeviceToHost, s));
  MCFL_CUDA_TRY(cudaMemcpyAsync(t.data(), c->T128.p, xy * 16, cudaMemcpyDeviceToHost, s));
  MCFL_CUDA_TRY(cudaMemcpyAsync(stats, c->stats.p, MCFL_ST_COUNT * 8, cudaMemcpyDeviceToHost, s));
  MCFL_CUDA_TRY(cudaStreamSynchronize(s));
  for (size_t i = 0; i < xy; ++i) {
    if (R) R[i] = r[2 * i];
    if (T) T[i] = t[2 * i];
  }
  return MCFL_OK;
}
