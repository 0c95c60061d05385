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
#include <atomic>
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


unsigned long long next_medium_serial() {
  static std::atomic<unsigned long long> counter{0};
  return ++counter;
}

int mcfl_ctx::attr(bool uniform, int *blk, int *bps, int *regs, bool time, bool exact, bool fl) {
  *blk = block;
  *bps = 0;
  *regs = 0;
  static const int mixed_codes[6] = {-1, -3, -4, -5, -6, -7};
  const int mixed = mixed_codes[mixed_code()];
  const int v = exact ? (uniform ? (time ? 10 : 6) : (time ? -9 : -8))
                : uniform ? (time ? 3 : variant_code(fl))
                          : (time ? -2 : mixed);
  return (int)attr_fn(math)(v, blk, bps, regs);
}

int mcfl_ctx::grid_for(bool uniform, int *block_out, int *bps_out, bool time, bool exact, bool fl) {
  int blk = 0, bps = 0, regs = 0;
  if (attr(uniform, &blk, &bps, &regs, time, exact, fl) != 0 || bps <= 0) bps = 1;
  if (blocks_per_sm > 0 && blocks_per_sm < bps) bps = blocks_per_sm;
  if (bps_out) *bps_out = bps;
  if (block_out) *block_out = blk;
  return bps * sm_count;
}

cudaError_t mcfl_ctx::launch_transport(const McflLaunch &L, int grid, int block_size) {
  ++launches;
  return launch_fn(math)(&L, grid, block_size, stream);
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
  if (c->l2_persist_bytes) { /* give the set-aside back to the process's other users */
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    cudaCtxResetPersistingL2Cache();
  }
  for (auto &ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  if (c->graph_run) cudaGraphExecDestroy(c->graph_run);
  if (c->graph_batch) cudaGraphExecDestroy(c->graph_batch);
  if (c->h_jobs) cudaFreeHost(c->h_jobs);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

extern "C" int mcfl_set_option(mcfl_ctx *c, const char *key, long long v) {
  if (!c || !key) return fail(MCFL_E_ARG, "mcfl_set_option: null argument");
  const std::string k(key);
  if (k == "math") {
    if (v != MCFL_MATH_EXACT && v != MCFL_MATH_FAST && v != MCFL_MATH_F64)
      return fail(MCFL_E_ARG, "math: 0 (exact), 1 (fast) or 2 (f64)");
    c->math = (int)v;
  } else if (k == "block") {
    if (v < 32 || v > 256 || (v % 32)) return fail(MCFL_E_ARG, "block: a multiple of 32 in [32, 256]");
    c->block = (int)v;
  } else if (k == "variant") {
    if (v < 0 || v >= MCFL_N_VARIANTS) return fail(MCFL_E_ARG, "variant: 0..2");
    c->variant = (int)v;
    c->variant_fl = -1;
  } else if (k == "variant_fl") {
    if (v < -1 || v >= MCFL_N_VARIANTS) return fail(MCFL_E_ARG, "variant_fl: -1 (as variant) or 0..2");
    c->variant_fl = (int)v;
  } else if (k == "phd_agg") {
    if (v < 0 || v > 2) return fail(MCFL_E_ARG, "phd_agg: 0 (one add per pass), 1 (register sums), 2 (warp sums)");
    c->phd_agg = (int)v;
  } else if (k == "pass_form") {
    c->pass_form = v ? 1 : 0;
  } else if (k == "mixed_variant") {
    if (v < 0 || v > 2) return fail(MCFL_E_ARG, "mixed_variant: 0..2");
    c->mixed_variant = (int)v;
  } else if (k == "blocks_per_sm") {
    if (v < 0 || v > 64) return fail(MCFL_E_ARG, "blocks_per_sm: 0..64");
    c->blocks_per_sm = (int)v;
  } else if (k == "step_cap") {
    if (v < 1 || v > 0x7fffffffLL) return fail(MCFL_E_ARG, "step_cap: 1..2^31-1");
    c->step_cap = (uint32_t)v;
  } else if (k == "relaunch") {
    if (v < 1 || v > 32) return fail(MCFL_E_ARG, "relaunch: 1..32");
    c->relaunch = (uint32_t)v;
  } else if (k == "l2_window") {
    MCFL_CUDA_TRY(cudaSetDevice(c->device));
    if (v) {
      int persist = 0, window = 0;
      MCFL_CUDA_TRY(cudaDeviceGetAttribute(&persist, cudaDevAttrMaxPersistingL2CacheSize, c->device));
      MCFL_CUDA_TRY(cudaDeviceGetAttribute(&window, cudaDevAttrMaxAccessPolicyWindowSize, c->device));
      if (persist <= 0 || window <= 0) return fail(MCFL_E_STATE, "l2_window: the device has no persisting L2");
      if (!c->l2_persist_bytes) MCFL_CUDA_TRY(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)persist));
      c->l2_persist_bytes = (size_t)persist;
      c->l2_max_window = (size_t)window;
    }
    c->l2_window = v ? 1 : 0;
  } else if (k == "graphs") {
    c->use_graphs = v ? 1 : 0;
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
  if (k == "variant") return c->variant;
  if (k == "variant_fl") return c->variant_fl;
  if (k == "phd_agg") return c->phd_agg;
  if (k == "pass_form") return c->pass_form;
  if (k == "mixed_variant") return c->mixed_variant;
  if (k == "step_cap") return c->step_cap;
  if (k == "l2_window") return c->l2_window;
  if (k == "relaunch") return c->relaunch;
  if (k == "graphs") return c->use_graphs;
  if (k == "graph_failed") return c->graph_error.empty() ? 0 : 1;
  if (k == "sm_count") return c->sm_count;
  if (k == "grid") return c->grid_for(true, nullptr);
  if (k == "grid_general") return c->grid_for(false, nullptr);
  if (k == "launch_block") {
    int blk = 0;
    c->grid_for(true, &blk);
    return blk;
  }
  if (k == "regs" || k == "regs_general") {
    int blk = 0, bps = 0, regs = 0;
    c->attr(k == "regs", &blk, &bps, &regs);
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
  m->serial = next_medium_serial();
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
  std::vector<float> le(MCFL_LAB_FLOATS * (size_t)nl), lm(MCFL_LAB_FLOATS * (size_t)nl);
  std::vector<float> pex(pe.size()), pmx(pm.size()), lex(le.size()), lmx(lm.size());
  /* voxel-boundary stepping spends the optical depth with the physical mu_t
   * of the phase's wavelength, the fluorophore's absorption included; the
   * reference's stepping keeps 1/(mua + mus) of the .mci column at both */
  auto inv_mut = [](float mua, float mus) {
    const float mut = mua + mus;
    return mut == 0.0f ? FLT_MAX : 1.0f / mut;
  };
  for (int i = 0; i < nl; ++i) {
    const mcfl_bulk &b = d->bulks[i];
    pe[4 * i + 0] = b.mutr; pe[4 * i + 1] = b.mua; pe[4 * i + 2] = b.g; pe[4 * i + 3] = b.n;
    pm[4 * i + 0] = b.mutr; pm[4 * i + 1] = b.muaf; pm[4 * i + 2] = b.g; pm[4 * i + 3] = b.n;
    fl[2 * i + 0] = b.eY; fl[2 * i + 1] = b.albedof;
    mcfl_label_record(b.mutr, b.mua, b.g, b.n, &le[MCFL_LAB_FLOATS * (size_t)i]);
    mcfl_label_record(b.mutr, b.muaf, b.g, b.n, &lm[MCFL_LAB_FLOATS * (size_t)i]);
    const float tx = inv_mut(b.mua, b.mus), tm = inv_mut(b.muaf, b.mus);
    pex[4 * i + 0] = tx; pex[4 * i + 1] = b.mua; pex[4 * i + 2] = b.g; pex[4 * i + 3] = b.n;
    pmx[4 * i + 0] = tm; pmx[4 * i + 1] = b.muaf; pmx[4 * i + 2] = b.g; pmx[4 * i + 3] = b.n;
    mcfl_label_record(tx, b.mua, b.g, b.n, &lex[MCFL_LAB_FLOATS * (size_t)i]);
    mcfl_label_record(tm, b.muaf, b.g, b.n, &lmx[MCFL_LAB_FLOATS * (size_t)i]);
  }
  cudaError_t e = m->labels.reserve(total);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->labels.p, d->labels, total, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = m->prop_exc.reserve(pe.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->prop_exc.p, pe.data(), pe.size() * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = m->prop_emi.reserve(pm.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->prop_emi.p, pm.data(), pm.size() * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = m->lab_exc.reserve(le.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->lab_exc.p, le.data(), le.size() * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = m->lab_emi.reserve(lm.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->lab_emi.p, lm.data(), lm.size() * 4, cudaMemcpyHostToDevice, c->stream);
  auto put = [&](mcfl::DevBuf &dst, const std::vector<float> &src) {
    cudaError_t r = dst.reserve(src.size() * 4);
    return r == cudaSuccess ? cudaMemcpyAsync(dst.p, src.data(), src.size() * 4, cudaMemcpyHostToDevice, c->stream) : r;
  };
  if (e == cudaSuccess) e = put(m->prop_exc_x, pex);
  if (e == cudaSuccess) e = put(m->prop_emi_x, pmx);
  if (e == cudaSuccess) e = put(m->lab_exc_x, lex);
  if (e == cudaSuccess) e = put(m->lab_emi_x, lmx);
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
  m->bytes = m->labels.bytes + m->prop_exc.bytes + m->prop_emi.bytes + m->lab_exc.bytes + m->lab_emi.bytes +
             m->prop_exc_x.bytes + m->prop_emi_x.bytes + m->lab_exc_x.bytes + m->lab_emi_x.bytes + m->fl.bytes +
             m->fmap.bytes;
  *out = m;
  return MCFL_OK;
}

extern "C" int mcfl_medium_create_layered(mcfl_ctx *c, const mcfl_layered_desc *d, mcfl_medium **out) {
  if (!c || !d || !out || !d->layers) return fail(MCFL_E_ARG, "mcfl_medium_create_layered: null argument");
  *out = nullptr;
  const int n = d->n_layers;
  if (n < 1 || n > MCFL_MAX_LAYERS) return fail(MCFL_E_RANGE, "layered medium: n_layers out of range");
  if (d->grid_size <= 0) return fail(MCFL_E_ARG, "layered medium: grid_size must be positive");
  for (int i = 1; i <= n; ++i) {
    const mcfl_layer &l = d->layers[i];
    if (!(l.z_max > l.z_min) || (i > 1 && l.z_min != d->layers[i - 1].z_max))
      return fail(MCFL_E_ARG, "layered medium: slabs must be contiguous with z_max > z_min");
  }
  if (d->layers[1].z_min != 0.0f) return fail(MCFL_E_ARG, "layered medium: the first slab starts at z = 0");
  if (!(d->inclusion.r >= 0.0f)) return fail(MCFL_E_ARG, "layered medium: negative inclusion radius");
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  mcfl_medium *m = new mcfl_medium();
  m->serial = next_medium_serial();
  m->ctx = c;
  m->layered = true;
  m->n_layers = n;
  const float esp = d->layers[n].z_max;
  const float g = (float)d->grid_size;
  /* the reference's photon-hitting-density grid (CUDAMCFLtransport.cu:44-45) */
  m->esp = esp;
  m->hx = m->hy = 2 * esp;
  m->gx = m->gy = m->gz = g;
  m->nx = m->ny = (int)(4 * esp * g); /* the size main allocates, CUDAMCFLmain.cu:340-342 */
  m->nz = (int)(esp * g);
  if (m->nx <= 0 || m->nz <= 0 || (unsigned long long)m->nx * m->ny * m->nz >= 0xFFFFFFFFull) {
    delete m;
    return fail(MCFL_E_RANGE, "layered medium: bad photon-hitting-density grid");
  }
  m->total = (uint32_t)((unsigned long long)m->nx * m->ny * m->nz);
  /* start weight: the medium above against the first slab (CUDAMCFLio.cu:638-652) */
  m->bulks.resize(2);
  std::memset(m->bulks.data(), 0, 2 * sizeof(mcfl_bulk));
  m->bulks[0].n = d->layers[0].n;
  m->bulks[1].n = d->layers[1].n;
  std::vector<float> tab(8 * (size_t)(n + 3), 0.0f);
  m->z_min.assign((size_t)n + 2, 0.0f);
  m->z_max.assign((size_t)n + 2, 0.0f);
  for (int i = 0; i < n + 2; ++i) {
    const mcfl_layer &l = d->layers[i];
    float *t = &tab[8 * (size_t)i];
    const bool slab = i >= 1 && i <= n;
    t[0] = slab ? l.mutr : 0.0f;
    t[1] = slab ? l.mua : 0.0f;
    t[2] = slab ? l.g : 0.0f;
    t[3] = l.n;
    t[4] = slab ? l.z_min : 0.0f;
    t[5] = slab ? l.z_max : 0.0f;
    m->z_min[i] = t[4];
    m->z_max[i] = t[5];
  }
  float *t = &tab[8 * (size_t)(n + 2)];
  const mcfl_inclusion &in = d->inclusion;
  t[0] = in.mutr; t[1] = in.mua; t[2] = in.g; t[3] = in.n;
  t[4] = in.x; t[5] = in.y; t[6] = in.z; t[7] = in.r;
  cudaError_t e = m->layer_tab.reserve(tab.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->layer_tab.p, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    delete m;
    return cuda_fail(e, "mcfl_medium_create_layered");
  }
  m->bytes = m->layer_tab.bytes;
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

