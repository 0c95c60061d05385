/*
 * Continuous-batching server.
 *
 * Requests (a medium and an excitation run) arrive on any thread.  A server
 * thread owns the GPU context and loops:
 *   1. admission: queued requests are admitted in arrival order while their
 *      HBM footprint (labels, fluorophore map, property tables, R/T images,
 *      photon hitting density) fits the budget and a job slot is free; the
 *      medium is uploaded and the request becomes a job whose photon tickets
 *      start where the running jobs' tickets end;
 *   2. one slice: the persistent transport kernel runs a bounded number of
 *      passes over every admitted job at once, drawing tickets from all of
 *      them, and parks the photons still in flight in HBM when the budget is
 *      spent;
 *   3. completion: jobs whose photons have all terminated are copied out and
 *      their memory and slot are released.
 * New work therefore joins the running batch at the next slice (every few
 * milliseconds) while earlier requests are still in flight, and a request's
 * photons draw the same random streams whatever else shares the GPU, so its
 * tallies equal those of running it alone bit for bit.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "mcfl_internal.h"
#include "portable_math.h"

using namespace mcfl;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
  unsigned long long id = 0;
  mcfl_medium_desc desc{};
  std::vector<mcfl_bulk> bulks;
  mcfl_run_desc run{};
  Clock::time_point t_submit, t_admit, t_done;
  size_t footprint = 0;
  /* device state while admitted */
  mcfl_medium *medium = nullptr;
  DevBuf R, T, fhd, stats, tpos, tarr;
  unsigned mode = 0;         /* bit 0: voxel-boundary stepping, bit 1: time-resolved detectors */
  int slot = -1;
  uint64_t ticket_begin = 0; /* in the current slice */
  uint64_t started = 0;      /* photons handed to the GPU so far */
  unsigned queue = 0;        /* ticket queue of the current slice */
  /* results */
  bool done = false;
  int status = MCFL_OK;
  std::vector<unsigned long long> Rd, Tt, fhd_host, time_host;
  unsigned long long st[MCFL_ST_COUNT] = {0};
};

size_t footprint_of(const mcfl_medium_desc &d, const mcfl_run_desc &r) {
  const size_t nv = (size_t)d.nx * d.ny * d.nz;
  const size_t xy = (size_t)r.det.nx + (size_t)r.det.nx * r.det.ny;
  size_t b = nv + (d.fluor_map ? nv * 4 : 0) + 3 * 16 * (size_t)(d.n_bulks + 2);
  b += 2 * xy * 8 + MCFL_ST_COUNT * 8;
  if (r.fluence) b += nv * 8;
  if (r.tdet.nx) b += (size_t)r.tdet.nx * r.tdet.ny * r.tdet.bins * 8 + (size_t)(r.tdet.nx + r.tdet.ny) * 4;
  if (r.exact_stepping) b += 6 * 16 * (size_t)(d.n_bulks + 2) + 2 * nv; /* its tables and free-radius map */
  return b;
}

} // namespace

struct mcfl_server {
  mcfl_ctx *ctx = nullptr;
  size_t budget = 0, used = 0;
  unsigned slots = 64;
  /* a slice's limits: passes per thread (0: none) and nanoseconds; a slice
   * also ends at once when a request arrives that can be admitted (the
   * submitting thread raises the stop word) or when a request's last photon
   * finishes (the kernel raises it) */
  uint32_t slice_iters = 0;
  uint64_t slice_ns = 32000000;
  uint32_t express_period = 4, express_ratio = 8; /* see mcfl_server_opts */
  std::mutex mu;
  std::condition_variable cv, cv_done;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<unsigned long long, std::shared_ptr<Request>> all;
  std::vector<std::shared_ptr<Request>> active; /* by slot */
  unsigned long long next_id = 1;
  bool stop = false;
  int fatal = MCFL_OK;
  std::thread worker;
  /* device state */
  DevBuf slot_jobs, order, counter, stats_all;
  DevBuf stop_word;              /* the running slice's stop flag */
  cudaStream_t sig = nullptr;    /* the submitting threads' stop signals */
  cudaEvent_t ev_reset = nullptr; /* the stop word's reset before the running slice */
  unsigned int *h_one = nullptr; /* pinned 1 */
  bool in_slice = false;         /* a slice is running (under mu) */
  /* Modes: bit 0 voxel-boundary stepping, bit 1 time of flight.  A launch
   * runs the requests of one mode with that mode's kernel variant; each mode
   * keeps one launch shape and its own photons in flight (parked per
   * thread), so slices of different modes take turns. */
  static constexpr unsigned kModes = 4;
  DevBuf parked[kModes];
  int grid_m[kModes] = {0, 0, 0, 0}, block_m[kModes] = {256, 256, 256, 256};
  unsigned next_mode = 0;
  McflJob *h_jobs = nullptr;
  uint32_t *h_order = nullptr;
  unsigned long long *h_read = nullptr;
  uint64_t tickets_end = 0;
  int grid = 0;
  int block = 256;
  /* metrics */
  std::vector<double> latencies_ms;
  unsigned long long photons_done = 0, slices = 0, max_inflight = 0, inflight_sum = 0;
  double busy_s = 0, upload_s = 0, finish_s = 0, kernel_s = 0;
  cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr; /* around each slice's launch */
  Clock::time_point t_first, t_last;
  bool any = false;

  void loop();
  int admit_locked(std::vector<std::shared_ptr<Request>> &to_upload);
  int upload(Request &r);
  void release(Request &r);
};

int mcfl_server::upload(Request &r) {
  mcfl_medium *m = nullptr;
  int rc = mcfl_medium_create(ctx, &r.desc, &m);
  if (rc != MCFL_OK) return rc;
  r.medium = m;
  const size_t xy = (size_t)r.run.det.nx + (size_t)r.run.det.nx * r.run.det.ny;
  const size_t nv = m->total;
  cudaStream_t s = ctx->stream;
  MCFL_CUDA_TRY(r.R.reserve(xy * 8));
  MCFL_CUDA_TRY(r.T.reserve(xy * 8));
  MCFL_CUDA_TRY(r.stats.reserve(MCFL_ST_COUNT * 8));
  MCFL_CUDA_TRY(cudaMemsetAsync(r.R.p, 0, xy * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(r.T.p, 0, xy * 8, s));
  MCFL_CUDA_TRY(cudaMemsetAsync(r.stats.p, 0, MCFL_ST_COUNT * 8, s));
  if (r.run.fluence) {
    MCFL_CUDA_TRY(r.fhd.reserve(nv * 8));
    MCFL_CUDA_TRY(cudaMemsetAsync(r.fhd.p, 0, nv * 8, s));
  }
  McflJob &j = h_jobs[r.slot];
  std::memset(&j, 0, sizeof(j));
  const bool exact = r.run.exact_stepping != 0;
  if (exact) {
    const int rcm = ensure_free_map(ctx, m);
    if (rcm != MCFL_OK) return rcm;
  }
  j.labels = m->labels.as<uint8_t>();
  j.prop = m->prop_of(false, exact);
  j.lab = m->lab_of(false, exact);
  j.lab16 = exact ? m->lab16.as<uint16_t>() : nullptr;
  j.hx = m->hx; j.hy = m->hy; j.esp = m->esp;
  j.gx = m->gx; j.gy = m->gy; j.gz = m->gz;
  j.nx = (uint32_t)m->nx; j.ny = (uint32_t)m->ny; j.nz = (uint32_t)m->nz; j.total = m->total;
  j.last_label = (uint32_t)m->n_bulks + 1u;
  j.src_kind = r.run.source.kind == MCFL_SOURCE_WIDEFIELD ? MCFL_SRC_WIDEFIELD : MCFL_SRC_GAUSS_BEAM;
  j.sx = r.run.source.x; j.sy = r.run.source.y; j.sz = r.run.source.z;
  j.src_w = r.run.source.width; j.src_h = r.run.source.height;
  if (r.run.start_weight) {
    j.start_weight = r.run.start_weight;
  } else {
    const double n1 = m->bulks[0].n, n2 = m->bulks[1].n;
    double q = (n1 - n2) / (n1 + n2);
    q = q * q;
    j.start_weight = (unsigned int)((double)0xFFFFFFFF * (1 - q));
  }
  const mcfl_detector &d = r.run.det;
  j.det_x0 = d.x0; j.det_y0 = d.y0; j.det_dx = d.dx; j.det_dy = d.dy;
  j.size_x = (d.dx * (float)d.nx) / 2.0f;
  j.size_y = (d.dy * (float)d.ny) / 2.0f;
  j.det_nx = (uint32_t)d.nx;
  j.xy_size = (uint32_t)xy;
  j.R = r.R.as<unsigned long long>();
  j.T = r.T.as<unsigned long long>();
  j.fhd_on = r.run.fluence ? 1u : 0u;
  j.fhd = r.run.fluence ? r.fhd.as<unsigned long long>() : nullptr;
  j.stats = r.stats.as<unsigned long long>();
  j.key = mcfl_stream_key(r.run.seed_exc, 0);
  j.launch_rng_reuse = r.run.launch_rng_reuse ? 1u : 0u;
  j.rng_offset = r.run.photon_offset;
  j.ticket_begin = r.ticket_begin;
  j.photons = r.run.photons;
  const mcfl_time_detectors &td = r.run.tdet;
  if (td.nx) {
    const size_t tsize = (size_t)td.nx * td.ny * td.bins;
    MCFL_CUDA_TRY(r.tpos.reserve((size_t)(td.nx + td.ny) * 4));
    MCFL_CUDA_TRY(r.tarr.reserve(tsize * 8));
    std::vector<float> pos((size_t)(td.nx + td.ny));
    time_positions(td, pos.data(), pos.data() + td.nx);
    MCFL_CUDA_TRY(cudaMemcpyAsync(r.tpos.p, pos.data(), pos.size() * 4, cudaMemcpyHostToDevice, s));
    MCFL_CUDA_TRY(cudaMemsetAsync(r.tarr.p, 0, tsize * 8, s));
    j.time_on = 1;
    j.tpos_x = r.tpos.as<float>();
    j.tpos_y = r.tpos.as<float>() + td.nx;
    j.time_xyt = r.tarr.as<unsigned long long>();
    j.tmax = td.max_fs;
    j.tdet_r = td.radius;
    j.tnx = (uint32_t)td.nx;
    j.tny = (uint32_t)td.ny;
    j.tbins = (uint32_t)td.bins;
    j.tdet_face = (uint32_t)td.face;
  }
  r.mode = (exact ? 1u : 0u) | (td.nx ? 2u : 0u);
  return MCFL_OK;
}

void mcfl_server::release(Request &r) {
  if (r.medium) mcfl_medium_free(r.medium);
  r.medium = nullptr;
  r.R.release();
  r.T.release();
  r.fhd.release();
  r.stats.release();
  r.tpos.release();
  r.tarr.release();
}

int mcfl_server::admit_locked(std::vector<std::shared_ptr<Request>> &to_upload) {
  while (!queue.empty()) {
    auto r = queue.front();
    if (r->footprint > budget) {
      r->status = MCFL_E_RANGE;
      r->done = true;
      queue.pop_front();
      cv_done.notify_all();
      continue;
    }
    if (used + r->footprint > budget) break;
    int slot = -1;
    for (unsigned i = 0; i < slots; ++i)
      if (!active[i]) {
        slot = (int)i;
        break;
      }
    if (slot < 0) break;
    queue.pop_front();
    r->slot = slot;
    active[slot] = r;
    used += r->footprint;
    to_upload.push_back(r);
  }
  return MCFL_OK;
}

void mcfl_server::loop() {
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  for (;;) {
    std::vector<std::shared_ptr<Request>> fresh;
    {
      std::unique_lock<std::mutex> lk(mu);
      bool have_active = false;
      for (auto &a : active) have_active |= (bool)a;
      if (!have_active && queue.empty()) {
        if (stop) return;
        cv.wait_for(lk, std::chrono::milliseconds(2));
        continue;
      }
      admit_locked(fresh);
    }
    const auto t_up0 = Clock::now();
    for (auto &r : fresh) {
      r->t_admit = Clock::now();
      r->started = 0;
      int rc = upload(*r);
      if (rc != MCFL_OK) {
        std::lock_guard<std::mutex> lk(mu);
        r->status = rc;
        r->done = true;
        active[r->slot] = nullptr;
        used -= r->footprint;
        release(*r);
        cv_done.notify_all();
      }
    }
    upload_s += std::chrono::duration<double>(Clock::now() - t_up0).count();
    /* Tickets of this slice, in two queues.  The head queue: the oldest
     * admitted request (the head), then the other requests larger than
     * 1/express_ratio of the head's remaining photons, in admission order,
     * which take over the warps as the head's tickets run out (no warp idles
     * while its last photons finish).  The express queue: the requests at
     * most 1/express_ratio of the head's remaining, shortest remaining
     * first, drawn first by one warp in express_period; every warp turns to
     * the other queue once its own is exhausted.  So a small request
     * arriving behind a large one starts at once on a share of the GPU, and
     * large requests keep their admission order and the rest of the GPU.
     * Photon k of a request still draws the stream of index k, whatever
     * slice or queue hands it out. */
    unsigned n = 0, n_active = 0;
    int head = -1;
    std::vector<uint32_t> h_stat_slot;
    /* the mode of this slice: the next one, in turn, with admitted requests */
    unsigned have = 0;
    for (unsigned i = 0; i < slots; ++i)
      if (active[i]) have |= 1u << active[i]->mode;
    if (!have) continue;
    unsigned mode = next_mode;
    while (!(have & (1u << mode))) mode = (mode + 1) % kModes;
    next_mode = (mode + 1) % kModes;
    auto older = [&](uint32_t a, uint32_t b) {
      return active[a]->t_admit != active[b]->t_admit ? active[a]->t_admit < active[b]->t_admit
                                                      : active[a]->id < active[b]->id;
    };
    for (unsigned i = 0; i < slots; ++i)
      if (active[i]) {
        ++n_active;
        h_stat_slot.push_back(i);
        if (active[i]->mode == mode && active[i]->started < active[i]->run.photons) {
          h_order[n++] = i;
          if (head < 0 || older(i, (uint32_t)head)) head = (int)i;
        }
      }
    if (n_active == 0) continue;
    unsigned n0 = n, n2 = 0;
    if (n > 1) {
      auto left = [&](uint32_t a) { return active[a]->run.photons - active[a]->started; };
      const uint64_t head_left = left((uint32_t)head);
      std::vector<uint32_t> express, main_q{(uint32_t)head}, rest;
      for (unsigned i = 0; i < n; ++i) {
        if ((int)h_order[i] == head) continue;
        (left(h_order[i]) * express_ratio <= head_left ? express : rest).push_back(h_order[i]);
      }
      std::sort(express.begin(), express.end(),
                [&](uint32_t a, uint32_t b) { return left(a) != left(b) ? left(a) < left(b) : a < b; });
      std::sort(rest.begin(), rest.end(), older);
      main_q.insert(main_q.end(), rest.begin(), rest.end());
      /* the first queue (express, if any) and the second (the head queue) */
      unsigned w = 0;
      for (uint32_t x : express) h_order[w++] = x;
      for (uint32_t x : main_q) h_order[w++] = x;
      n0 = express.empty() ? (unsigned)main_q.size() : (unsigned)express.size();
      n2 = express.empty() ? 0u : (unsigned)main_q.size();
    }
    uint64_t tickets = 0, tickets2 = 0;
    for (unsigned i = 0; i < n0 + n2; ++i) {
      Request &r = *active[h_order[i]];
      McflJob &j = h_jobs[h_order[i]];
      uint64_t &tk = i < n0 ? tickets : tickets2;
      r.ticket_begin = tk;
      r.queue = i < n0 ? 0 : 1;
      j.ticket_begin = tk;
      j.photon_base = r.started;
      j.photons = r.run.photons - r.started;
      tk += j.photons;
    }
    tickets_end = tickets;
    const uint64_t tickets_end2 = tickets2;
    const auto t0 = Clock::now();
    cudaMemsetAsync(counter.p, 0, 16, s);
    cudaMemcpyAsync(slot_jobs.p, h_jobs, slots * sizeof(McflJob), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(order.p, h_order, (size_t)(n0 + n2) * 4, cudaMemcpyHostToDevice, s);
    McflLaunch L;
    std::memset(&L, 0, sizeof(L));
    L.jobs = slot_jobs.as<McflJob>();
    L.order = order.as<uint32_t>();
    L.n_jobs = n0;
    if (n2) {
      L.order2 = order.as<uint32_t>() + n0;
      L.n_jobs2 = n2;
      L.ticket_counter2 = counter.as<unsigned long long>() + 1;
      L.ticket_end2 = tickets_end2;
    }
    L.max_iters = slice_iters;
    L.slice_ns = slice_ns;
    L.stop_flag = stop_word.as<unsigned int>();
    L.express_period = express_period;
    L.variant = (uint32_t)ctx->mixed_code();
    L.exact_step = (mode & 1u) ? 1u : 0u;
    L.time_on = (mode & 2u) ? 1u : 0u;
    L.ticket_counter = counter.as<unsigned long long>();
    L.ticket_end = tickets_end;
    L.mult = ctx->mult.as<uint32_t>();
    L.saved = parked[mode].as<McflSaved>();
    L.step_cap = ctx->step_cap;
    L.relaunch_min = ctx->relaunch;
    cudaMemsetAsync(stop_word.p, 0, 4, s);
    cudaEventRecord(ev_reset, s);
    {
      std::lock_guard<std::mutex> lk(mu);
      in_slice = true;
    }
    cudaEventRecord(ev_k0, s);
    cudaError_t e = ctx->launch_transport(L, grid_m[mode], block_m[mode]);
    cudaEventRecord(ev_k1, s);
    cudaMemcpyAsync(h_read, counter.p, 16, cudaMemcpyDeviceToHost, s);
    for (unsigned i = 0; i < n_active; ++i) {
      Request &r = *active[h_stat_slot[i]];
      cudaMemcpyAsync(h_read + 2 + (size_t)i * MCFL_ST_COUNT, r.stats.p, MCFL_ST_COUNT * 8, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    {
      std::lock_guard<std::mutex> lk(mu);
      in_slice = false;
    }
    const auto t1 = Clock::now();
    float k_ms = 0.f;
    if (e == cudaSuccess && cudaEventElapsedTime(&k_ms, ev_k0, ev_k1) == cudaSuccess) kernel_s += 1e-3 * k_ms;
    busy_s += std::chrono::duration<double>(t1 - t0).count();
    ++slices;
    inflight_sum += n_active;
    max_inflight = std::max<unsigned long long>(max_inflight, n_active);
    if (e != cudaSuccess) {
      std::lock_guard<std::mutex> lk(mu);
      fatal = cuda_fail(e, "server slice");
      for (auto &a : active)
        if (a) {
          a->status = MCFL_E_CUDA;
          a->done = true;
          a = nullptr;
        }
      for (auto &q : queue) {
        q->status = MCFL_E_CUDA;
        q->done = true;
      }
      queue.clear();
      cv_done.notify_all();
      return;
    }
    /* warps may draw past a queue's end */
    const uint64_t drawn[2] = {std::min<uint64_t>(h_read[0], tickets_end), std::min<uint64_t>(h_read[1], tickets_end2)};
    for (unsigned i = 0; i < n0 + n2; ++i) {
      Request &r = *active[h_order[i]];
      const uint64_t c = drawn[r.queue];
      const uint64_t handed = c > r.ticket_begin ? c - r.ticket_begin : 0;
      r.started += std::min<uint64_t>(handed, r.run.photons - r.started);
    }
    const auto t_fin0 = Clock::now();
    for (unsigned i = 0; i < n_active; ++i) {
      const uint32_t slot = h_stat_slot[i];
      std::shared_ptr<Request> r = active[slot];
      const unsigned long long *st = h_read + 2 + (size_t)i * MCFL_ST_COUNT;
      if (st[MCFL_ST_DONE] < r->run.photons) continue;
      const size_t xy = (size_t)r->run.det.nx + (size_t)r->run.det.nx * r->run.det.ny;
      r->Rd.resize(xy);
      r->Tt.resize(xy);
      cudaMemcpyAsync(r->Rd.data(), r->R.p, xy * 8, cudaMemcpyDeviceToHost, s);
      cudaMemcpyAsync(r->Tt.data(), r->T.p, xy * 8, cudaMemcpyDeviceToHost, s);
      if (r->run.fluence) {
        r->fhd_host.resize(r->medium->total);
        cudaMemcpyAsync(r->fhd_host.data(), r->fhd.p, (size_t)r->medium->total * 8, cudaMemcpyDeviceToHost, s);
      }
      if (r->run.tdet.nx) {
        const size_t tsize = (size_t)r->run.tdet.nx * r->run.tdet.ny * r->run.tdet.bins;
        r->time_host.resize(tsize);
        cudaMemcpyAsync(r->time_host.data(), r->tarr.p, tsize * 8, cudaMemcpyDeviceToHost, s);
      }
      std::memcpy(r->st, st, sizeof(r->st));
      cudaStreamSynchronize(s);
      release(*r);
      std::lock_guard<std::mutex> lk(mu);
      r->t_done = Clock::now();
      r->status = r->st[MCFL_ST_CAPPED] ? MCFL_E_CAPPED : MCFL_OK;
      r->done = true;
      const double lat = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
      latencies_ms.push_back(lat);
      photons_done += r->run.photons;
      if (!any) t_first = r->t_submit;
      any = true;
      t_last = r->t_done;
      active[slot] = nullptr;
      used -= r->footprint;
      cv_done.notify_all();
    }
    finish_s += std::chrono::duration<double>(Clock::now() - t_fin0).count();
  }
}

extern "C" int mcfl_server_create(mcfl_ctx *ctx, const mcfl_server_opts *opts, mcfl_server **out) {
  if (!ctx || !out) return fail(MCFL_E_ARG, "mcfl_server_create: null argument");
  *out = nullptr;
  if (ctx->math == MCFL_MATH_F64)
    return fail(MCFL_E_ARG, "mcfl_server_create: the f64 build runs whole launches only (no parked photons)");
  auto *sv = new mcfl_server();
  sv->ctx = ctx;
  size_t free_b = 0, total_b = 0;
  cudaSetDevice(ctx->device);
  cudaMemGetInfo(&free_b, &total_b);
  sv->budget = opts && opts->hbm_budget_bytes ? (size_t)opts->hbm_budget_bytes : free_b / 2;
  sv->slots = opts && opts->max_jobs ? (unsigned)opts->max_jobs : 64u;
  sv->slice_iters = opts ? (uint32_t)opts->slice_passes : 0u;
  if (opts && opts->slice_us) sv->slice_ns = std::min<uint64_t>((uint64_t)opts->slice_us * 1000u, 4000000000ull);
  if (opts && opts->express_period) sv->express_period = opts->express_period;
  if (opts && opts->express_ratio) sv->express_ratio = opts->express_ratio;
  if (sv->slots > 4096) {
    delete sv;
    return fail(MCFL_E_RANGE, "max_jobs above 4096");
  }
  sv->active.assign(sv->slots, nullptr);
  sv->grid = ctx->grid_for(false, &sv->block);
  cudaError_t e = sv->slot_jobs.reserve(sv->slots * sizeof(McflJob));
  if (!e) e = sv->order.reserve(sv->slots * 4);
  if (!e) e = sv->counter.reserve(16); /* the two queues' ticket counters */
  if (!e) e = cudaMemset(sv->counter.p, 0, 8);
  if (!e) e = sv->stop_word.reserve(4);
  if (!e) e = cudaMemset(sv->stop_word.p, 0, 4);
  if (!e) e = cudaStreamCreateWithFlags(&sv->sig, cudaStreamNonBlocking);
  if (!e) e = cudaEventCreateWithFlags(&sv->ev_reset, cudaEventDisableTiming);
  if (!e) e = cudaEventCreate(&sv->ev_k0);
  if (!e) e = cudaEventCreate(&sv->ev_k1);
  for (unsigned mode = 0; mode < mcfl_server::kModes && !e; ++mode) {
    sv->grid_m[mode] = ctx->grid_for(false, &sv->block_m[mode], nullptr, (mode & 2u) != 0, (mode & 1u) != 0);
    const size_t threads = (size_t)sv->grid_m[mode] * sv->block_m[mode];
    e = sv->parked[mode].reserve(threads * sizeof(McflSaved));
    if (!e) e = cudaMemset(sv->parked[mode].p, 0, threads * sizeof(McflSaved));
  }
  if (!e) e = cudaHostAlloc((void **)&sv->h_jobs, sv->slots * sizeof(McflJob), cudaHostAllocDefault);
  if (!e) e = cudaHostAlloc((void **)&sv->h_order, sv->slots * 4, cudaHostAllocDefault);
  if (!e) e = cudaHostAlloc((void **)&sv->h_read, (2 + (size_t)sv->slots * MCFL_ST_COUNT) * 8, cudaHostAllocDefault);
  if (!e) e = cudaHostAlloc((void **)&sv->h_one, 4, cudaHostAllocDefault);
  if (!e) *sv->h_one = 1u;
  if (e) {
    mcfl_server_destroy(sv);
    return cuda_fail(e, "mcfl_server_create");
  }
  std::memset(sv->h_jobs, 0, sv->slots * sizeof(McflJob));
  sv->worker = std::thread([sv] { sv->loop(); });
  *out = sv;
  return MCFL_OK;
}

extern "C" int mcfl_server_submit(mcfl_server *sv, const mcfl_medium_desc *medium, const mcfl_run_desc *run,
                                  unsigned long long *id) {
  if (!sv || !medium || !run || !id) return fail(MCFL_E_ARG, "mcfl_server_submit: null argument");
  if (run->photons_per_voxel) return fail(MCFL_E_ARG, "server requests are excitation runs (photons_per_voxel = 0)");
  const mcfl_time_detectors &td = run->tdet;
  if (td.nx < 0 || (td.nx && (td.ny <= 0 || td.bins <= 0 || td.max_fs == 0 || !(td.radius > 0) ||
                             (td.face != 0 && td.face != 1))))
    return fail(MCFL_E_ARG, "bad time-resolved detectors");
  if (run->photons == 0 || run->det.nx <= 0 || run->det.ny <= 0) return fail(MCFL_E_ARG, "bad run");
  if (!medium->labels || !medium->bulks || medium->n_bulks < 1 || medium->n_bulks > MCFL_MAX_BULKS)
    return fail(MCFL_E_ARG, "bad medium");
  auto r = std::make_shared<Request>();
  r->desc = *medium;
  r->bulks.assign(medium->bulks, medium->bulks + medium->n_bulks + 2);
  r->desc.bulks = r->bulks.data();
  r->run = *run;
  r->footprint = footprint_of(*medium, *run);
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->fatal != MCFL_OK) return fail(MCFL_E_STATE, "server stopped after a CUDA error");
  r->id = sv->next_id++;
  sv->queue.push_back(r);
  sv->all[r->id] = r;
  *id = r->id;
  sv->cv.notify_all();
  /* a running slice ends early when this request can join the next one (a
   * free slot and room in the budget); the signal is ordered after that
   * slice's reset of its stop word.  It only shortens a slice: if it is lost
   * (a failed call) or lands after the slice ended (the next one then stops
   * at once), results are unchanged */
  if (sv->in_slice && sv->queue.size() == 1 && sv->used + r->footprint <= sv->budget) {
    unsigned used_slots = 0;
    for (auto &a : sv->active) used_slots += a ? 1u : 0u;
    if (used_slots < sv->slots) {
      int dev_old = -1;
      cudaGetDevice(&dev_old);
      if (dev_old != sv->ctx->device) cudaSetDevice(sv->ctx->device);
      cudaStreamWaitEvent(sv->sig, sv->ev_reset, 0);
      cudaMemcpyAsync(sv->stop_word.p, sv->h_one, 4, cudaMemcpyHostToDevice, sv->sig);
      if (dev_old >= 0 && dev_old != sv->ctx->device) cudaSetDevice(dev_old);
    }
  }
  return MCFL_OK;
}

extern "C" int mcfl_server_wait(mcfl_server *sv, unsigned long long id, int timeout_ms) {
  if (!sv) return fail(MCFL_E_ARG, "null server");
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->all.find(id);
  if (it == sv->all.end()) return fail(MCFL_E_ARG, "unknown request");
  auto r = it->second;
  auto pred = [&] { return r->done; };
  if (timeout_ms < 0) sv->cv_done.wait(lk, pred);
  else if (!sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
    return fail(MCFL_E_TIMEOUT, "request not finished");
  return r->status;
}

extern "C" int mcfl_server_result(mcfl_server *sv, unsigned long long id, mcfl_run_out *out, double *latency_ms) {
  if (!sv) return fail(MCFL_E_ARG, "null server");
  std::shared_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->all.find(id);
    if (it == sv->all.end()) return fail(MCFL_E_ARG, "unknown request");
    r = it->second;
    if (!r->done) return fail(MCFL_E_STATE, "request not finished");
    sv->all.erase(it);
  }
  if (r->status != MCFL_OK) return fail(r->status, "request failed");
  if (out) {
    if (out->Rd) std::memcpy(out->Rd, r->Rd.data(), r->Rd.size() * 8);
    if (out->Tt) std::memcpy(out->Tt, r->Tt.data(), r->Tt.size() * 8);
    if (out->fhd && !r->fhd_host.empty()) std::memcpy(out->fhd, r->fhd_host.data(), r->fhd_host.size() * 8);
    if (out->time_xyt && !r->time_host.empty())
      std::memcpy(out->time_xyt, r->time_host.data(), r->time_host.size() * 8);
    std::memcpy(out->stats_exc, r->st, sizeof(r->st));
  }
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  return MCFL_OK;
}

extern "C" int mcfl_server_metrics(mcfl_server *sv, mcfl_server_metrics_t *m) {
  if (!sv || !m) return fail(MCFL_E_ARG, "null argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  std::memset(m, 0, sizeof(*m));
  std::vector<double> l = sv->latencies_ms;
  std::sort(l.begin(), l.end());
  auto pct = [&](double p) {
    if (l.empty()) return 0.0;
    const double pos = p * (double)(l.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < l.size() ? l[i] * (1 - f) + l[i + 1] * f : l[i];
  };
  m->completed = l.size();
  m->p50_ms = pct(0.50);
  m->p99_ms = pct(0.99);
  m->max_ms = l.empty() ? 0.0 : l.back();
  m->photons = sv->photons_done;
  m->slices = sv->slices;
  m->busy_s = sv->busy_s;
  m->mean_inflight = sv->slices ? (double)sv->inflight_sum / (double)sv->slices : 0.0;
  m->max_inflight = sv->max_inflight;
  m->span_s = sv->any ? std::chrono::duration<double>(sv->t_last - sv->t_first).count() : 0.0;
  m->hbm_used = sv->used;
  m->hbm_budget = sv->budget;
  m->upload_s = sv->upload_s;
  m->finish_s = sv->finish_s;
  m->kernel_s = sv->kernel_s;
  return MCFL_OK;
}

extern "C" void mcfl_server_destroy(mcfl_server *sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
    sv->cv.notify_all();
  }
  if (sv->worker.joinable()) sv->worker.join();
  for (auto &a : sv->active)
    if (a) sv->release(*a);
  if (sv->h_jobs) cudaFreeHost(sv->h_jobs);
  if (sv->h_order) cudaFreeHost(sv->h_order);
  if (sv->h_read) cudaFreeHost(sv->h_read);
  if (sv->h_one) cudaFreeHost(sv->h_one);
  if (sv->ev_reset) cudaEventDestroy(sv->ev_reset);
  if (sv->ev_k0) cudaEventDestroy(sv->ev_k0);
  if (sv->ev_k1) cudaEventDestroy(sv->ev_k1);
  if (sv->sig) cudaStreamDestroy(sv->sig);
  delete sv;
}
