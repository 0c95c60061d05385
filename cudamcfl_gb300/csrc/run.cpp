/*
 * Runs, batches and the plain schedule.
 *
 *   mcfl_run        one two-phase simulation: excitation launch, emission-list
 *                   build, one emission launch over every emitting voxel,
 *                   recorded once and replayed as a CUDA graph;
 *   mcfl_batch_run  many excitation simulations (sources, budgets) on one
 *                   medium: BATCHED = one persistent launch over all of them
 *                   (graph replay), PLAIN = one launch per simulation;
 *   mcfl_run_plain  the two-phase simulation with the emission phase
 *                   scheduled the reference's way (CUDAMCFLmain.cu:471-594):
 *                   one launch per emitting voxel.
 * Photon k of a simulation always uses stream (key, rng_offset + k), so the
 * schedules give bit-identical tallies; only their speed differs.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "mcfl_internal.h"
#include "portable_math.h"

using namespace mcfl;

namespace {

unsigned int default_start_weight(const mcfl_medium *m) {
  /* CUDAMCFLio.cu:639-652: specular loss between the medium above and label 1 */
  const double n1 = m->bulks[0].n, n2 = m->bulks[1].n;
  double r = (n1 - n2) / (n1 + n2);
  r = r * r;
  return (unsigned int)((double)0xFFFFFFFF * (1 - r));
}

/* exact: the label records of voxel-boundary stepping (mu_t with the
 * fluorophore's absorption at the phase's wavelength) */
void fill_medium(McflJob &j, const mcfl_medium *m, bool emission, bool exact = false) {
  j.labels = m->labels.as<uint8_t>();
  j.lab16 = exact ? m->lab16.as<uint16_t>() : nullptr; /* built by ensure_free_map */
  j.prop = m->prop_of(emission, exact);
  j.lab = m->lab_of(emission, exact);
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

void fill_source(McflJob &j, const mcfl_run_desc &r, const mcfl_medium *m) {
  j.src_kind = r.source.kind == MCFL_SOURCE_WIDEFIELD ? MCFL_SRC_WIDEFIELD : MCFL_SRC_GAUSS_BEAM;
  j.sx = r.source.x;
  j.sy = r.source.y;
  j.sz = r.source.z;
  j.src_w = r.source.width;
  j.src_h = r.source.height;
  j.start_weight = r.start_weight ? r.start_weight : default_start_weight(m);
  if (m->layered) /* LaunchPhoton's search for the source's slab (CUDAMCFLtransport.cu:550-560) */
    for (int nl = 1; nl <= m->n_layers; ++nl)
      if (r.source.z < m->z_max[nl] && r.source.z >= m->z_min[nl]) {
        j.start_layer = (uint32_t)nl;
        break;
      }
}


int check_run(const mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run) {
  if (!c || !m || !run) return fail(MCFL_E_ARG, "null argument");
  if (m->ctx != c) return fail(MCFL_E_ARG, "medium of another context");
  const mcfl_detector &det = run->det;
  if (det.nx <= 0 || det.ny <= 0 || !(det.dx > 0) || !(det.dy > 0)) return fail(MCFL_E_ARG, "bad detector");
  if ((unsigned long long)det.nx * (unsigned long long)(det.ny + 1) >= 0xFFFFFFFFull)
    return fail(MCFL_E_RANGE, "detector too large");
  if (run->photons == 0) return fail(MCFL_E_ARG, "zero photons");
  if (run->source.kind != MCFL_SOURCE_GAUSS_BEAM && run->source.kind != MCFL_SOURCE_WIDEFIELD)
    return fail(MCFL_E_ARG, "unknown source kind");
  const mcfl_time_detectors &td = run->tdet;
  if (td.nx != 0) {
    if (td.nx < 0 || td.ny <= 0 || td.bins <= 0 || td.max_fs == 0 || (td.face != 0 && td.face != 1) ||
        !(td.radius > 0))
      return fail(MCFL_E_ARG, "bad time-resolved detectors");
    if ((unsigned long long)td.nx * (unsigned long long)td.ny * (unsigned long long)td.bins >= (1ull << 31))
      return fail(MCFL_E_RANGE, "time-resolved tally too large");
  }
  if (run->exact_stepping) {
    if (m->layered) return fail(MCFL_E_ARG, "exact stepping: voxelized media only");
  }
  if (m->layered) {
    if (run->photons_per_voxel) return fail(MCFL_E_ARG, "layered medium: excitation runs only");
    bool inside = false;
    for (int nl = 1; nl <= m->n_layers; ++nl)
      inside = inside || (run->source.z < m->z_max[nl] && run->source.z >= m->z_min[nl]);
    if (!inside) return fail(MCFL_E_ARG, "layered medium: the source z lies in no slab");
  }
  return MCFL_OK;
}

cudaError_t ensure_pinned(mcfl_ctx *c, size_t jobs, size_t outs) {
  if (jobs > c->h_jobs_cap) {
    if (c->h_jobs) cudaFreeHost(c->h_jobs);
    c->h_jobs = nullptr;
    c->h_jobs_cap = 0;
    cudaError_t e = cudaHostAlloc((void **)&c->h_jobs, jobs * sizeof(McflJob), cudaHostAllocDefault);
    if (e != cudaSuccess) return e;
    c->h_jobs_cap = jobs;
  }
  if (outs > c->h_out_cap) {
    if (c->h_out) cudaFreeHost(c->h_out);
    c->h_out = nullptr;
    c->h_out_cap = 0;
    cudaError_t e = cudaHostAlloc((void **)&c->h_out, outs * 8, cudaHostAllocDefault);
    if (e != cudaSuccess) return e;
    c->h_out_cap = outs;
  }
  return cudaSuccess;
}

/* Event record that becomes a timing node when the stream is being
 * captured into a graph. */
cudaError_t record_event(cudaEvent_t ev, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cs);
  if (e != cudaSuccess) return e;
  return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal)
                                             : cudaEventRecord(ev, s);
}

/* Replays a recorded launch sequence as a CUDA graph, recording it again when
 * the key (every pointer and size the sequence bakes in) changes.  On the
 * legacy default stream, with graphs off, or when a capture cannot be made,
 * the sequence runs directly. */
int replay(mcfl_ctx *c, cudaGraphExec_t *exec, std::string *cur_key, unsigned *kernels, const std::string &key,
           const std::function<cudaError_t(cudaStream_t, unsigned *)> &record) {
  cudaStream_t s = c->stream;
  auto direct = [&]() -> int {
    unsigned k = 0;
    cudaError_t e = record(s, &k);
    c->launches += k;
    return e == cudaSuccess ? MCFL_OK : cuda_fail(e, "launch sequence");
  };
  if (!c->use_graphs || s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread) return direct();
  if (*exec == nullptr || *cur_key != key) {
    if (*exec) cudaGraphExecDestroy(*exec);
    *exec = nullptr;
    cur_key->clear();
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    unsigned k = 0;
    cudaError_t er = record(s, &k);
    e = cudaStreamEndCapture(s, &g);
    if (er == cudaSuccess && e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (er != cudaSuccess || e != cudaSuccess) {
      /* not capturable here: keep the context working without graphs */
      cudaGetLastError();
      *exec = nullptr;
      c->use_graphs = 0;
      c->graph_error = std::string(cudaGetErrorString(er != cudaSuccess ? er : e));
      return direct();
    }
    *cur_key = key;
    *kernels = k;
  }
  c->launches += *kernels;
  cudaError_t e = cudaGraphLaunch(*exec, s);
  return e == cudaSuccess ? MCFL_OK : cuda_fail(e, "cudaGraphLaunch");
}

/* GPU time between two events; 0 when they hold no record.  Clears the
 * runtime's last-error slot so a failed query cannot leak into a later
 * launch check. */
float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    ms = 0.f;
  }
  return ms;
}

std::string ptr_key(std::initializer_list<const void *> ps, std::initializer_list<unsigned long long> vs) {
  std::string k;
  char buf[32];
  for (const void *p : ps) {
    snprintf(buf, sizeof(buf), "%p;", p);
    k += buf;
  }
  for (unsigned long long v : vs) {
    snprintf(buf, sizeof(buf), "%llu;", v);
    k += buf;
  }
  return k;
}

McflLaunch base_launch(mcfl_ctx *c) {
  McflLaunch L;
  std::memset(&L, 0, sizeof(L));
  L.mult = c->mult.as<uint32_t>();
  L.step_cap = c->step_cap;
  L.variant = (uint32_t)c->variant_code();
  L.relaunch_min = c->relaunch;
  return L;
}

/* Every job of the launch uses medium m with one photon-hitting-density
 * tally (or none): the medium travels in the kernel parameters. */
void set_uniform(const mcfl_ctx *c, McflLaunch &L, const mcfl_medium *m, bool emission, unsigned long long *fhd,
                 bool exact = false) {
  L.uniform_medium = 1;
  if (c->l2_window && c->l2_max_window) {
    const size_t bytes = std::min<size_t>(m->labels.bytes, c->l2_max_window);
    L.l2_base = m->labels.p;
    L.l2_bytes = bytes;
    L.l2_hit_ratio = (float)std::min(1.0, (double)c->l2_persist_bytes / (double)bytes);
  }
  McflMedium &u = L.med;
  u.labels = m->labels.as<uint8_t>();
  u.prop = m->prop_of(emission, exact);
  u.lab = m->lab_of(emission, exact);
  u.lab16 = exact ? m->lab16.as<uint16_t>() : nullptr;
  u.n_labels = (uint32_t)m->n_bulks + 2u;
  u.fhd = fhd;
  u.hx = m->hx;
  u.hy = m->hy;
  u.esp = m->esp;
  u.gx = m->gx;
  u.gy = m->gy;
  u.gz = m->gz;
  u.nx = (uint32_t)m->nx;
  u.ny = (uint32_t)m->ny;
  u.total = m->total;
  u.last_label = (uint32_t)m->n_bulks + 1u;
  if (m->layered) {
    u.layered = 1;
    u.n_layers = (uint32_t)m->n_layers;
    u.layer_tab = m->layer_tab.as<float>();
    u.n_labels = 0;
  }
}

} // namespace

/* The free-radius map of voxel-boundary stepping, built on the medium's
 * first such run (synchronously, before any recorded graph uses it). */
int mcfl::ensure_free_map(mcfl_ctx *c, const mcfl_medium *m) {
  if (m->lab16.p) return MCFL_OK;
  const size_t n = (size_t)m->total;
  mcfl::DevBuf tmp;
  MCFL_CUDA_TRY(tmp.reserve(2 * n));
  MCFL_CUDA_TRY(m->lab16.reserve(2 * n));
  cudaError_t e = mcfl_launch_free_map(m->labels.as<uint8_t>(), m->nx, m->ny, m->nz, tmp.as<uint8_t>(),
                                       m->lab16.as<uint16_t>(), c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    m->lab16.release();
    return cuda_fail(e, "free-radius map");
  }
  return MCFL_OK;
}

/* ------------------------------------------------------------------ run */

extern "C" int mcfl_run(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run, mcfl_run_out *out) {
  int rc = check_run(c, m, run);
  if (rc) return rc;
  cudaGetLastError();
  const mcfl_detector &det = run->det;
  const bool emission = run->photons_per_voxel > 0;
  const bool fluence = emission || run->fluence;
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  cudaGetLastError();
  if (run->exact_stepping && (rc = ensure_free_map(c, m)) != MCFL_OK) return rc;
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
  const size_t nout = 2 * MCFL_ST_COUNT + 4;
  MCFL_CUDA_TRY(ensure_pinned(c, 2, nout));
  const mcfl_time_detectors &td = run->tdet;
  const bool timed = td.nx > 0;
  const size_t tsize = timed ? (size_t)td.nx * td.ny * td.bins : 0;
  if (timed) {
    MCFL_CUDA_TRY(c->tpos.reserve((size_t)(td.nx + td.ny) * 4));
    MCFL_CUDA_TRY(c->tarr.reserve(tsize * 8));
    std::vector<float> pos((size_t)(td.nx + td.ny));
    time_positions(td, pos.data(), pos.data() + td.nx);
    MCFL_CUDA_TRY(cudaMemcpyAsync(c->tpos.p, pos.data(), pos.size() * 4, cudaMemcpyHostToDevice, s));
  }

  McflJob *jobs = c->h_jobs;
  std::memset(jobs, 0, 2 * sizeof(McflJob));
  McflJob &je = jobs[0];
  fill_medium(je, m, false, run->exact_stepping != 0);
  fill_detector(je, det);
  fill_source(je, *run, m);
  je.fhd_on = fluence ? 1u : 0u;
  je.R = c->R.as<unsigned long long>();
  je.T = c->T.as<unsigned long long>();
  je.fhd = fluence ? c->fhd.as<unsigned long long>() : nullptr;
  je.stats = c->stats.as<unsigned long long>();
  je.key = mcfl_stream_key(run->seed_exc, 0);
  je.rng_offset = run->photon_offset;
  je.photons = run->photons;
  je.launch_rng_reuse = run->launch_rng_reuse ? 1u : 0u;
  if (timed) {
    je.time_on = 1;
    je.tpos_x = c->tpos.as<float>();
    je.tpos_y = c->tpos.as<float>() + td.nx;
    je.time_xyt = c->tarr.as<unsigned long long>();
    je.tmax = td.max_fs;
    je.tdet_r = td.radius;
    je.tnx = (uint32_t)td.nx;
    je.tny = (uint32_t)td.ny;
    je.tbins = (uint32_t)td.bins;
    je.tdet_face = (uint32_t)td.face;
  }
  if (emission) {
    McflJob &jf = jobs[1];
    fill_medium(jf, m, true, run->exact_stepping != 0);
    fill_detector(jf, det);
    jf.src_kind = MCFL_SRC_VOXELS;
    jf.src_vox = c->vox.as<uint32_t>();
    jf.src_q = c->q.as<uint64_t>();
    jf.per_voxel = run->photons_per_voxel;
    jf.R128 = c->R128.as<unsigned long long>();
    jf.T128 = c->T128.as<unsigned long long>();
    jf.stats = c->stats.as<unsigned long long>() + MCFL_ST_COUNT;
    jf.key = mcfl_stream_key(run->seed_fl, 1);
    jf.photons = 0; /* written by the list build */
    jf.launch_rng_reuse = run->launch_rng_reuse ? 1u : 0u;
  }

  unsigned long long *cnt = c->counters.as<unsigned long long>();
  const bool exact = run->exact_stepping != 0;
  int block = 0, block_exc = 0;
  /* the emission launch may run its own occupancy variant */
  const int grid = c->grid_for(true, &block, nullptr, false, exact, true);
  const int grid_exc = c->grid_for(true, &block_exc, nullptr, timed, exact);
  const unsigned long long photons = run->photons;
  const unsigned per_voxel = run->photons_per_voxel;
  auto record = [&](cudaStream_t st, unsigned *k) -> cudaError_t {
    cudaError_t e;
#define REC(x)                   \
  if ((e = (x)) != cudaSuccess) \
    return e;
    REC(cudaMemsetAsync(c->R.p, 0, xy * 8, st));
    REC(cudaMemsetAsync(c->T.p, 0, xy * 8, st));
    REC(cudaMemsetAsync(c->stats.p, 0, 2 * MCFL_ST_COUNT * 8, st));
    REC(cudaMemsetAsync(c->counters.p, 0, 16 * 8, st));
    if (fluence) REC(cudaMemsetAsync(c->fhd.p, 0, nv * 8, st));
    if (timed) REC(cudaMemsetAsync(c->tarr.p, 0, tsize * 8, st));
    if (emission) {
      REC(cudaMemsetAsync(c->R128.p, 0, xy * 16, st));
      REC(cudaMemsetAsync(c->T128.p, 0, xy * 16, st));
    }
    REC(cudaMemcpyAsync(c->jobs.p, c->h_jobs, 2 * sizeof(McflJob), cudaMemcpyHostToDevice, st));
    McflLaunch L = base_launch(c);
    L.jobs = c->jobs.as<McflJob>();
    L.n_jobs = 1;
    L.ticket_counter = cnt + 0;
    L.ticket_end = photons;
    set_uniform(c, L, m, false, fluence ? c->fhd.as<unsigned long long>() : nullptr, exact);
    L.time_on = timed ? 1u : 0u;
    L.exact_step = exact ? 1u : 0u;
    REC(record_event(c->ev[0], st));
    REC(launch_fn(c->math)(&L, grid_exc, block_exc, st));
    ++*k;
    REC(record_event(c->ev[1], st));
    if (emission) {
      REC(mcfl_launch_emission_prep(m->labels.as<uint8_t>(), m->fl.as<float2>(), c->fhd.as<unsigned long long>(),
                                    m->has_fmap ? m->fmap.as<float>() : nullptr, m->total, photons, per_voxel,
                                    c->block_counts.as<uint32_t>(), c->vox.as<uint32_t>(), c->q.as<uint64_t>(),
                                    cnt + 2, c->jobs.as<McflJob>() + 1, cnt + 3, st));
      *k += 3;
      McflLaunch Lf = L;
      Lf.time_on = 0;
      Lf.jobs = c->jobs.as<McflJob>() + 1;
      Lf.ticket_counter = cnt + 1;
      Lf.ticket_end_dev = cnt + 3;
      set_uniform(c, Lf, m, true, nullptr, exact);
      Lf.variant = (uint32_t)c->variant_code(true);
      REC(record_event(c->ev[2], st));
      REC(launch_fn(c->math)(&Lf, grid, block, st));
      ++*k;
      REC(record_event(c->ev[3], st));
    }
    REC(cudaMemcpyAsync(c->h_out, c->stats.p, 2 * MCFL_ST_COUNT * 8, cudaMemcpyDeviceToHost, st));
    REC(cudaMemcpyAsync(c->h_out + 2 * MCFL_ST_COUNT, c->counters.p, 4 * 8, cudaMemcpyDeviceToHost, st));
#undef REC
    return cudaSuccess;
  };
  const std::string key = ptr_key({m, c->R.p, c->T.p, c->fhd.p, c->R128.p, c->T128.p, c->vox.p, c->q.p, c->jobs.p,
                                   c->h_jobs, c->h_out, c->stats.p, c->block_counts.p, (const void *)s,
                                   timed ? c->tarr.p : nullptr},
                                  {xy, nv, (unsigned long long)emission, (unsigned long long)fluence, photons,
                                   per_voxel, (unsigned long long)c->math, (unsigned long long)grid,
                                   (unsigned long long)block, c->step_cap, (unsigned long long)c->variant_code(),
                                   (unsigned long long)c->variant_code(true),
                                   (unsigned long long)c->l2_window, tsize, (unsigned long long)grid_exc,
                                   (unsigned long long)block_exc, (unsigned long long)exact, m->serial,
                                   c->relaunch});
  rc = replay(c, &c->graph_run, &c->graph_run_key, &c->graph_run_kernels, key, record);
  if (rc != MCFL_OK) return rc;

  /* FP64 normalisation of the requested images on the GPU */
  std::vector<std::pair<double *, std::pair<double *, size_t>>> pend;
  if (out) {
    size_t nd = (out->R ? xy : 0) + (out->T ? xy : 0) + (out->phd && fluence ? nv : 0) +
                (emission ? (out->flR ? xy : 0) + (out->flT ? xy : 0) : 0);
    if (nd) MCFL_CUDA_TRY(c->outd.reserve(nd * 8));
    double *dd = c->outd.as<double>();
    size_t off = 0;
    const double scale2 = ((double)0xFFFFFFFF * (double)photons) * (double)det.dx * (double)det.dy;
    const double flnorm = ((double)per_voxel * 4294967295.0) * ((double)det.dx * (double)det.dy);
    auto take = [&](size_t n, double *host) {
      double *p = dd + off;
      off += n;
      pend.push_back({p, {host, n}});
      ++c->launches;
      return p;
    };
    if (out->R) MCFL_CUDA_TRY(mcfl_launch_normalize_u64(c->R.as<unsigned long long>(), take(xy, out->R), xy, scale2, s));
    if (out->T) MCFL_CUDA_TRY(mcfl_launch_normalize_u64(c->T.as<unsigned long long>(), take(xy, out->T), xy, scale2, s));
    if (out->phd && fluence)
      MCFL_CUDA_TRY(mcfl_launch_normalize_phd(c->fhd.as<unsigned long long>(), take(nv, out->phd), nv, photons, s));
    if (emission && out->flR)
      MCFL_CUDA_TRY(mcfl_launch_normalize_128(c->R128.as<unsigned long long>(), take(xy, out->flR), xy, flnorm, s));
    if (emission && out->flT)
      MCFL_CUDA_TRY(mcfl_launch_normalize_128(c->T128.as<unsigned long long>(), take(xy, out->flT), xy, flnorm, s));
    for (auto &p : pend)
      MCFL_CUDA_TRY(cudaMemcpyAsync(p.second.first, p.first, p.second.second * 8, cudaMemcpyDeviceToHost, s));
    if (out->Rd) MCFL_CUDA_TRY(cudaMemcpyAsync(out->Rd, c->R.p, xy * 8, cudaMemcpyDeviceToHost, s));
    if (out->Tt) MCFL_CUDA_TRY(cudaMemcpyAsync(out->Tt, c->T.p, xy * 8, cudaMemcpyDeviceToHost, s));
    if (out->fhd && fluence) MCFL_CUDA_TRY(cudaMemcpyAsync(out->fhd, c->fhd.p, nv * 8, cudaMemcpyDeviceToHost, s));
    if (emission && out->flR128)
      MCFL_CUDA_TRY(cudaMemcpyAsync(out->flR128, c->R128.p, xy * 16, cudaMemcpyDeviceToHost, s));
    if (emission && out->flT128)
      MCFL_CUDA_TRY(cudaMemcpyAsync(out->flT128, c->T128.p, xy * 16, cudaMemcpyDeviceToHost, s));
    if (timed && out->time_xyt)
      MCFL_CUDA_TRY(cudaMemcpyAsync(out->time_xyt, c->tarr.p, tsize * 8, cudaMemcpyDeviceToHost, s));
  }
  MCFL_CUDA_TRY(cudaStreamSynchronize(s));
  const unsigned long long *st = c->h_out;
  const unsigned long long *cn = c->h_out + 2 * MCFL_ST_COUNT;
  if (out) {
    std::memcpy(out->stats_exc, st, MCFL_ST_COUNT * 8);
    std::memcpy(out->stats_fl, st + MCFL_ST_COUNT, MCFL_ST_COUNT * 8);
    out->fl_voxels = emission ? (long long)cn[2] : 0;
    out->photons_fl = emission ? cn[3] : 0;
    const double launched = (double)photons * (double)je.start_weight;
    const double a = (double)st[MCFL_ST_ABSORBED], rt = (double)st[MCFL_ST_EXIT_TOP],
                 tb = (double)st[MCFL_ST_EXIT_BOTTOM];
    const double lost = (double)st[MCFL_ST_R_LOSS] + (double)st[MCFL_ST_W0_LOSS] - (double)st[MCFL_ST_R_GAIN];
    out->energy_exc[0] = rt / launched;
    out->energy_exc[1] = tb / launched;
    out->energy_exc[2] = a / launched;
    out->energy_exc[3] = (launched - (a + rt + tb + lost)) / launched;
    out->ms_exc = elapsed_ms(c->ev[0], c->ev[1]);
    out->ms_fl = 0.f;
    if (emission) out->ms_fl = elapsed_ms(c->ev[2], c->ev[3]);
  }
  if (st[MCFL_ST_CAPPED] || st[MCFL_ST_COUNT + MCFL_ST_CAPPED])
    return fail(MCFL_E_CAPPED, "photons reached the per-photon pass cap");
  return MCFL_OK;
}

/* ---------------------------------------------------------------- batch */

extern "C" int mcfl_batch_run_media(mcfl_ctx *c, const mcfl_medium *const *media, const mcfl_run_desc *runs, int n,
                                    int schedule, mcfl_run_out *outs, float *gpu_ms) {
  if (n <= 0 || !runs || !media) return fail(MCFL_E_ARG, "mcfl_batch_run: empty batch");
  if (schedule != MCFL_SCHEDULE_BATCHED && schedule != MCFL_SCHEDULE_PLAIN)
    return fail(MCFL_E_ARG, "mcfl_batch_run: unknown schedule");
  const mcfl_detector det = runs[0].det;
  /* one medium for every run: the single-medium kernel; several: the
   * mixed-media kernel, each job carrying its medium */
  const mcfl_medium *m = media[0];
  bool uniform = true;
  for (int i = 0; i < n; ++i) uniform = uniform && media[i] == m;
  const bool exact = runs[0].exact_stepping != 0;
  for (int i = 0; i < n; ++i)
    if ((runs[i].exact_stepping != 0) != exact)
      return fail(MCFL_E_ARG, "mcfl_batch_run: the runs of a batch share the stepping");
  for (int i = 0; i < n; ++i) {
    if (!media[i]) return fail(MCFL_E_ARG, "mcfl_batch_run: null medium");
    if (!uniform && media[i]->layered)
      return fail(MCFL_E_ARG, "mcfl_batch_run: layered media batch with their own medium only");
    int rc = check_run(c, media[i], &runs[i]);
    if (rc) return rc;
    if (runs[i].photons_per_voxel || runs[i].fluence)
      return fail(MCFL_E_ARG, "mcfl_batch_run: excitation images and time detectors only (no fluence or emission)");
    if (runs[i].tdet.nx && media[i]->layered && !uniform)
      return fail(MCFL_E_ARG, "mcfl_batch_run: time detectors on layered media batch with their own medium only");
    const mcfl_detector &d = runs[i].det;
    if (d.nx != det.nx || d.ny != det.ny) return fail(MCFL_E_ARG, "mcfl_batch_run: detectors must share a size");
  }
  if (exact) {
    MCFL_CUDA_TRY(cudaSetDevice(c->device));
    for (int i = 0; i < n; ++i) {
      const int rcm = ensure_free_map(c, media[i]);
      if (rcm != MCFL_OK) return rcm;
    }
  }
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  cudaGetLastError();
  cudaStream_t s = c->stream;
  const size_t xy = (size_t)det.nx + (size_t)det.nx * det.ny;
  const size_t N = (size_t)n;
  MCFL_CUDA_TRY(c->bR.reserve(N * xy * 8));
  MCFL_CUDA_TRY(c->bT.reserve(N * xy * 8));
  MCFL_CUDA_TRY(c->bstats.reserve(N * MCFL_ST_COUNT * 8));
  MCFL_CUDA_TRY(c->bcnt.reserve(N * 8 + 8));
  MCFL_CUDA_TRY(c->jobs.reserve(N * sizeof(McflJob) + sizeof(McflJob)));
  MCFL_CUDA_TRY(ensure_pinned(c, N, N * MCFL_ST_COUNT + N + 8));
  /* time-resolved detectors: each timed run's histogram and disc positions
   * at its own offset in one buffer */
  std::vector<size_t> toff(N + 1, 0), poff(N + 1, 0);
  for (int i = 0; i < n; ++i) {
    const mcfl_time_detectors &td = runs[i].tdet;
    toff[i + 1] = toff[i] + (td.nx ? (size_t)td.nx * td.ny * td.bins : 0);
    poff[i + 1] = poff[i] + (td.nx ? (size_t)(td.nx + td.ny) : 0);
  }
  const size_t tsize = toff[N];
  const bool timed = tsize > 0;
  if (timed) {
    MCFL_CUDA_TRY(c->tarr.reserve(tsize * 8));
    MCFL_CUDA_TRY(c->tpos.reserve(poff[N] * 4));
    std::vector<float> pos(poff[N]);
    for (int i = 0; i < n; ++i)
      if (runs[i].tdet.nx) time_positions(runs[i].tdet, pos.data() + poff[i], pos.data() + poff[i] + runs[i].tdet.nx);
    MCFL_CUDA_TRY(cudaMemcpyAsync(c->tpos.p, pos.data(), pos.size() * 4, cudaMemcpyHostToDevice, s));
  }
  McflJob *jobs = c->h_jobs;
  std::memset(jobs, 0, N * sizeof(McflJob));
  unsigned long long tickets = 0;
  for (int i = 0; i < n; ++i) {
    McflJob &j = jobs[i];
    fill_medium(j, media[i], false, exact);
    fill_detector(j, runs[i].det);
    fill_source(j, runs[i], media[i]);
    j.R = c->bR.as<unsigned long long>() + i * xy;
    j.T = c->bT.as<unsigned long long>() + i * xy;
    j.stats = c->bstats.as<unsigned long long>() + i * (size_t)MCFL_ST_COUNT;
    j.key = mcfl_stream_key(runs[i].seed_exc, 0);
    j.rng_offset = runs[i].photon_offset;
    j.launch_rng_reuse = runs[i].launch_rng_reuse ? 1u : 0u;
    j.ticket_begin = schedule == MCFL_SCHEDULE_BATCHED ? tickets : 0;
    j.photons = runs[i].photons;
    tickets += runs[i].photons;
    const mcfl_time_detectors &td = runs[i].tdet;
    if (td.nx) {
      j.time_on = 1;
      j.tpos_x = c->tpos.as<float>() + poff[i];
      j.tpos_y = c->tpos.as<float>() + poff[i] + td.nx;
      j.time_xyt = c->tarr.as<unsigned long long>() + toff[i];
      j.tmax = td.max_fs;
      j.tdet_r = td.radius;
      j.tnx = (uint32_t)td.nx;
      j.tny = (uint32_t)td.ny;
      j.tbins = (uint32_t)td.bins;
      j.tdet_face = (uint32_t)td.face;
    }
  }
  int block = 0, block_one = 0;
  const int grid = c->grid_for(uniform, &block, nullptr, timed, exact);
  float ms = 0.f;
  if (schedule == MCFL_SCHEDULE_BATCHED) {
    auto record = [&](cudaStream_t st, unsigned *k) -> cudaError_t {
      cudaError_t e;
      if ((e = cudaMemsetAsync(c->bR.p, 0, N * xy * 8, st))) return e;
      if ((e = cudaMemsetAsync(c->bT.p, 0, N * xy * 8, st))) return e;
      if ((e = cudaMemsetAsync(c->bstats.p, 0, N * MCFL_ST_COUNT * 8, st))) return e;
      if ((e = cudaMemsetAsync(c->bcnt.p, 0, 8, st))) return e;
      if (timed && (e = cudaMemsetAsync(c->tarr.p, 0, tsize * 8, st))) return e;
      if ((e = cudaMemcpyAsync(c->jobs.p, c->h_jobs, N * sizeof(McflJob), cudaMemcpyHostToDevice, st))) return e;
      McflLaunch L = base_launch(c);
      L.jobs = c->jobs.as<McflJob>();
      L.n_jobs = (uint32_t)n;
      L.ticket_counter = c->bcnt.as<unsigned long long>();
      L.ticket_end = tickets;
      if (uniform) set_uniform(c, L, m, false, nullptr, exact);
      else L.variant = (uint32_t)c->mixed_code();
      L.exact_step = exact ? 1u : 0u;
      L.time_on = timed ? 1u : 0u;
      if ((e = record_event(c->ev[0], st))) return e;
      if ((e = launch_fn(c->math)(&L, grid, block, st)))
        return e;
      ++*k;
      if ((e = record_event(c->ev[1], st))) return e;
      return cudaMemcpyAsync(c->h_out, c->bstats.p, N * MCFL_ST_COUNT * 8, cudaMemcpyDeviceToHost, st);
    };
    std::string key =
        ptr_key({m, c->bR.p, c->bT.p, c->bstats.p, c->bcnt.p, c->jobs.p, c->h_jobs, c->h_out, (const void *)s,
                 timed ? c->tarr.p : nullptr},
                {N, xy, tickets, (unsigned long long)c->math, (unsigned long long)grid, (unsigned long long)block,
                 c->step_cap, (unsigned long long)c->variant_code(), (unsigned long long)c->l2_window,
                 (unsigned long long)uniform, (unsigned long long)exact, m->serial, tsize,
                 (unsigned long long)c->mixed_code(), c->relaunch});
    const int rcb = replay(c, &c->graph_batch, &c->graph_batch_key, &c->graph_batch_kernels, key, record);
    if (rcb != MCFL_OK) return rcb;
    MCFL_CUDA_TRY(cudaStreamSynchronize(s));
    ms = elapsed_ms(c->ev[0], c->ev[1]);
  } else {
    MCFL_CUDA_TRY(cudaMemsetAsync(c->bR.p, 0, N * xy * 8, s));
    MCFL_CUDA_TRY(cudaMemsetAsync(c->bT.p, 0, N * xy * 8, s));
    MCFL_CUDA_TRY(cudaMemsetAsync(c->bstats.p, 0, N * MCFL_ST_COUNT * 8, s));
    MCFL_CUDA_TRY(cudaMemsetAsync(c->bcnt.p, 0, N * 8, s));
    if (timed) MCFL_CUDA_TRY(cudaMemsetAsync(c->tarr.p, 0, tsize * 8, s));
    MCFL_CUDA_TRY(cudaMemcpyAsync(c->jobs.p, c->h_jobs, N * sizeof(McflJob), cudaMemcpyHostToDevice, s));
    MCFL_CUDA_TRY(cudaEventRecord(c->ev[0], s));
    for (int i = 0; i < n; ++i) {
      /* plain schedule: one medium per launch */
      const bool timed_i = runs[i].tdet.nx > 0;
      const int grid_one = c->grid_for(true, &block_one, nullptr, timed_i, exact);
      McflLaunch L = base_launch(c);
      L.jobs = c->jobs.as<McflJob>() + i;
      L.n_jobs = 1;
      L.ticket_counter = c->bcnt.as<unsigned long long>() + i;
      L.ticket_end = runs[i].photons;
      set_uniform(c, L, media[i], false, nullptr, exact);
      L.exact_step = exact ? 1u : 0u;
      L.time_on = timed_i ? 1u : 0u;
      MCFL_CUDA_TRY(c->launch_transport(L, grid_one, block_one));
      MCFL_CUDA_TRY(cudaStreamSynchronize(s)); /* one simulation per call, as DoOneSimulation */
    }
    MCFL_CUDA_TRY(cudaEventRecord(c->ev[1], s));
    MCFL_CUDA_TRY(cudaMemcpyAsync(c->h_out, c->bstats.p, N * MCFL_ST_COUNT * 8, cudaMemcpyDeviceToHost, s));
    MCFL_CUDA_TRY(cudaStreamSynchronize(s));
    ms = elapsed_ms(c->ev[0], c->ev[1]);
  }
  if (gpu_ms) *gpu_ms = ms;
  bool capped = false;
  if (outs) {
    bool any_norm = false;
    for (int i = 0; i < n; ++i) any_norm |= (outs[i].R || outs[i].T);
    std::vector<double> scales(N);
    if (any_norm) {
      MCFL_CUDA_TRY(c->seg_scale.reserve(N * 8));
      MCFL_CUDA_TRY(c->outd.reserve(2 * N * xy * 8));
      for (int i = 0; i < n; ++i)
        scales[i] = ((double)0xFFFFFFFF * (double)runs[i].photons) * (double)runs[i].det.dx * (double)runs[i].det.dy;
      MCFL_CUDA_TRY(cudaMemcpyAsync(c->seg_scale.p, scales.data(), N * 8, cudaMemcpyHostToDevice, s));
      double *dd = c->outd.as<double>();
      MCFL_CUDA_TRY(mcfl_launch_normalize_segments(c->bR.as<unsigned long long>(), dd, xy, N,
                                                   c->seg_scale.as<double>(), s));
      MCFL_CUDA_TRY(mcfl_launch_normalize_segments(c->bT.as<unsigned long long>(), dd + N * xy, xy, N,
                                                   c->seg_scale.as<double>(), s));
      c->launches += 2;
    }
    for (int i = 0; i < n; ++i) {
      mcfl_run_out &o = outs[i];
      if (o.Rd) MCFL_CUDA_TRY(cudaMemcpyAsync(o.Rd, c->bR.as<unsigned long long>() + i * xy, xy * 8, cudaMemcpyDeviceToHost, s));
      if (o.Tt) MCFL_CUDA_TRY(cudaMemcpyAsync(o.Tt, c->bT.as<unsigned long long>() + i * xy, xy * 8, cudaMemcpyDeviceToHost, s));
      if (o.R) MCFL_CUDA_TRY(cudaMemcpyAsync(o.R, c->outd.as<double>() + i * xy, xy * 8, cudaMemcpyDeviceToHost, s));
      if (o.T) MCFL_CUDA_TRY(cudaMemcpyAsync(o.T, c->outd.as<double>() + (N + i) * xy, xy * 8, cudaMemcpyDeviceToHost, s));
      if (o.time_xyt && toff[i + 1] > toff[i])
        MCFL_CUDA_TRY(cudaMemcpyAsync(o.time_xyt, c->tarr.as<unsigned long long>() + toff[i],
                                      (toff[i + 1] - toff[i]) * 8, cudaMemcpyDeviceToHost, s));
    }
    MCFL_CUDA_TRY(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i) {
      std::memcpy(outs[i].stats_exc, c->h_out + i * (size_t)MCFL_ST_COUNT, MCFL_ST_COUNT * 8);
      std::memset(outs[i].stats_fl, 0, sizeof(outs[i].stats_fl));
      outs[i].ms_exc = ms;
      capped |= outs[i].stats_exc[MCFL_ST_CAPPED] != 0;
    }
  }
  if (capped) return fail(MCFL_E_CAPPED, "photons reached the per-photon pass cap");
  return MCFL_OK;
}

extern "C" int mcfl_batch_run(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *runs, int n, int schedule,
                              mcfl_run_out *outs, float *gpu_ms) {
  if (n <= 0 || !runs) return fail(MCFL_E_ARG, "mcfl_batch_run: empty batch");
  std::vector<const mcfl_medium *> media((size_t)n, m);
  return mcfl_batch_run_media(c, media.data(), runs, n, schedule, outs, gpu_ms);
}

/* ---------------------------------------------------------------- plain */

extern "C" int mcfl_run_plain(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run, long long max_voxels,
                              mcfl_run_out *out) {
  int rc = check_run(c, m, run);
  if (rc) return rc;
  if (run->photons_per_voxel == 0) return mcfl_run(c, m, run, out);
  const mcfl_detector &det = run->det;
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  cudaGetLastError();
  if (run->exact_stepping && (rc = ensure_free_map(c, m)) != MCFL_OK) return rc;
  cudaStream_t s = c->stream;
  const size_t xy = (size_t)det.nx + (size_t)det.nx * det.ny;
  const size_t nv = m->total;
  /* excitation with the photon hitting density, then the emission list,
   * exactly as mcfl_run builds them */
  mcfl_run_desc exc = *run;
  exc.photons_per_voxel = 0;
  exc.fluence = 1;
  rc = mcfl_run(c, m, &exc, nullptr);
  if (rc != MCFL_OK) return rc;
  MCFL_CUDA_TRY(c->vox.reserve(nv * 4));
  MCFL_CUDA_TRY(c->q.reserve(nv * 8));
  MCFL_CUDA_TRY(c->block_counts.reserve(emission_prep_blocks((uint32_t)nv) * 4 + 16));
  MCFL_CUDA_TRY(c->R128.reserve(xy * 16));
  MCFL_CUDA_TRY(c->T128.reserve(xy * 16));
  MCFL_CUDA_TRY(mcfl_launch_emission_prep(m->labels.as<uint8_t>(), m->fl.as<float2>(), c->fhd.as<unsigned long long>(),
                                          m->has_fmap ? m->fmap.as<float>() : nullptr, m->total, run->photons,
                                          run->photons_per_voxel, c->block_counts.as<uint32_t>(),
                                          c->vox.as<uint32_t>(), c->q.as<uint64_t>(),
                                          c->counters.as<unsigned long long>() + 2, c->jobs.as<McflJob>() + 1,
                                          c->counters.as<unsigned long long>() + 3, s));
  c->launches += 3;
  unsigned long long cn[4];
  MCFL_CUDA_TRY(cudaMemcpyAsync(cn, c->counters.p, sizeof(cn), cudaMemcpyDeviceToHost, s));
  MCFL_CUDA_TRY(cudaStreamSynchronize(s));
  long long nlist = (long long)cn[2];
  if (max_voxels > 0 && max_voxels < nlist) nlist = max_voxels;
  /* the exc launch's stats stay in c->stats[0..]; emission stats restart */
  MCFL_CUDA_TRY(cudaMemsetAsync(c->R128.p, 0, xy * 16, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->T128.p, 0, xy * 16, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->stats.as<unsigned long long>() + MCFL_ST_COUNT, 0, MCFL_ST_COUNT * 8, s));
  const size_t NL = (size_t)(nlist > 0 ? nlist : 0);
  MCFL_CUDA_TRY(c->jobs.reserve((NL + 2) * sizeof(McflJob)));
  MCFL_CUDA_TRY(c->bcnt.reserve(NL * 8 + 8));
  MCFL_CUDA_TRY(ensure_pinned(c, NL + 2, 2 * MCFL_ST_COUNT + 8));
  McflJob t;
  std::memset(&t, 0, sizeof(t));
  fill_medium(t, m, true, run->exact_stepping != 0);
  fill_detector(t, det);
  t.src_kind = MCFL_SRC_VOXELS;
  t.per_voxel = run->photons_per_voxel;
  t.R128 = c->R128.as<unsigned long long>();
  t.T128 = c->T128.as<unsigned long long>();
  t.stats = c->stats.as<unsigned long long>() + MCFL_ST_COUNT;
  t.key = mcfl_stream_key(run->seed_fl, 1);
  t.photons = run->photons_per_voxel;
  t.launch_rng_reuse = run->launch_rng_reuse ? 1u : 0u;
  for (size_t i = 0; i < NL; ++i) {
    McflJob &j = c->h_jobs[i];
    j = t;
    j.src_vox = c->vox.as<uint32_t>() + i;
    j.src_q = c->q.as<uint64_t>() + i;
    j.rng_offset = (uint64_t)i * run->photons_per_voxel;
  }
  MCFL_CUDA_TRY(cudaMemcpyAsync(c->jobs.p, c->h_jobs, NL * sizeof(McflJob), cudaMemcpyHostToDevice, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(c->bcnt.p, 0, NL * 8 + 8, s));
  int block = 0;
  const int grid = c->grid_for(true, &block, nullptr, false, run->exact_stepping != 0);
  MCFL_CUDA_TRY(cudaEventRecord(c->ev[2], s));
  for (size_t i = 0; i < NL; ++i) {
    McflLaunch L = base_launch(c);
    L.jobs = c->jobs.as<McflJob>() + i;
    L.n_jobs = 1;
    L.ticket_counter = c->bcnt.as<unsigned long long>() + i;
    L.ticket_end = run->photons_per_voxel;
    set_uniform(c, L, m, true, nullptr, run->exact_stepping != 0);
    L.exact_step = run->exact_stepping ? 1u : 0u;
    MCFL_CUDA_TRY(c->launch_transport(L, grid, block));
    MCFL_CUDA_TRY(cudaStreamSynchronize(s)); /* one simulation per call, as DoOneSimulationFl */
  }
  MCFL_CUDA_TRY(cudaEventRecord(c->ev[3], s));
  MCFL_CUDA_TRY(cudaMemcpyAsync(c->h_out, c->stats.p, 2 * MCFL_ST_COUNT * 8, cudaMemcpyDeviceToHost, s));
  if (out) {
    if (out->Rd) MCFL_CUDA_TRY(cudaMemcpyAsync(out->Rd, c->R.p, xy * 8, cudaMemcpyDeviceToHost, s));
    if (out->Tt) MCFL_CUDA_TRY(cudaMemcpyAsync(out->Tt, c->T.p, xy * 8, cudaMemcpyDeviceToHost, s));
    if (out->fhd) MCFL_CUDA_TRY(cudaMemcpyAsync(out->fhd, c->fhd.p, nv * 8, cudaMemcpyDeviceToHost, s));
    if (out->flR128) MCFL_CUDA_TRY(cudaMemcpyAsync(out->flR128, c->R128.p, xy * 16, cudaMemcpyDeviceToHost, s));
    if (out->flT128) MCFL_CUDA_TRY(cudaMemcpyAsync(out->flT128, c->T128.p, xy * 16, cudaMemcpyDeviceToHost, s));
  }
  MCFL_CUDA_TRY(cudaStreamSynchronize(s));
  if (out) {
    std::memcpy(out->stats_exc, c->h_out, MCFL_ST_COUNT * 8);
    std::memcpy(out->stats_fl, c->h_out + MCFL_ST_COUNT, MCFL_ST_COUNT * 8);
    out->fl_voxels = (long long)NL;
    out->photons_fl = (unsigned long long)NL * run->photons_per_voxel;
    out->ms_exc = elapsed_ms(c->ev[0], c->ev[1]);
    out->ms_fl = elapsed_ms(c->ev[2], c->ev[3]);
  }
  return MCFL_OK;
}

/* ------------------------------------------------- one-voxel emission */

int mcfl::run_single_voxel_emission(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run, unsigned int voxel,
                                    unsigned long long *R, unsigned long long *T, unsigned long long *stats) {
  if (m->layered) return fail(MCFL_E_ARG, "layered medium: no emission runs");
  const mcfl_detector &det = run->det;
  const size_t xy = (size_t)det.nx + (size_t)det.nx * det.ny;
  cudaStream_t s = c->stream;
  MCFL_CUDA_TRY(cudaSetDevice(c->device));
  cudaGetLastError();
  if (run->exact_stepping) {
    const int rcm = ensure_free_map(c, m);
    if (rcm != MCFL_OK) return rcm;
  }
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
  fill_medium(j, m, false, run->exact_stepping != 0);
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
  j.launch_rng_reuse = run->launch_rng_reuse ? 1u : 0u;
  MCFL_CUDA_TRY(cudaMemcpyAsync(c->jobs.p, &j, sizeof(j), cudaMemcpyHostToDevice, s));
  McflLaunch L = base_launch(c);
  L.jobs = c->jobs.as<McflJob>();
  L.n_jobs = 1;
  L.ticket_counter = c->counters.as<unsigned long long>();
  L.ticket_end = run->photons;
  set_uniform(c, L, m, false, nullptr, run->exact_stepping != 0);
  L.exact_step = run->exact_stepping ? 1u : 0u;
  int block = 0;
  const int grid = c->grid_for(true, &block, nullptr, false, run->exact_stepping != 0);
  MCFL_CUDA_TRY(c->launch_transport(L, grid, block));
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
