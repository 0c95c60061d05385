/*
 * Launch-shape autotuner (mcfl_autotune).
 *
 * The reference fixes its launch shape at compile time (128 blocks of 256
 * threads, CUDAMCFL.h:18-20).  The persistent kernel here is compiled in
 * several occupancy variants of the single-medium kernel (threads per block x
 * the blocks per SM the register budget is cut for), each with two forms of
 * the pass (arranged for the SIMT warp, or every test of the reference's
 * pass as its own branch) and two forms of the photon-hitting-density tally
 * (one atomic add per pass, or the sums of successive passes in one voxel
 * held in a register, a form of the branching pass), and can put a
 * persisting L2 access window on the labels and tallies; the SIMT-arranged
 * pass is also timed with the free lanes of a warp starting new photons in
 * pairs (option "relaunch" 2).  Which combination is fastest
 * depends on the medium (how often photons change label, how deep they go)
 * and on the emission/excitation mix, so the tuner times every combination on
 * a sample of the caller's own run and keeps the fastest in the context,
 * with its own occupancy variant for the excitation and the emission phase
 * (the excitation launch, which waits on its label loads, can prefer fewer
 * registers or more warps than the issue-bound emission launch).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "mcfl_internal.h"

using namespace mcfl;

extern "C" int mcfl_autotune(mcfl_ctx *c, const mcfl_medium *m, const mcfl_run_desc *run,
                             unsigned long long sample_photons, int *variant_out, double *rate_out) {
  if (!c || !m || !run) return fail(MCFL_E_ARG, "mcfl_autotune: null argument");
  if (sample_photons == 0) return fail(MCFL_E_ARG, "mcfl_autotune: sample_photons must be positive");
  mcfl_run_desc r = *run;
  r.photons = std::min<unsigned long long>(sample_photons, run->photons ? run->photons : sample_photons);
  if (run->photons_per_voxel) {
    /* keep the run's emission/excitation proportion */
    const double f = (double)r.photons / (double)(run->photons ? run->photons : r.photons);
    r.photons_per_voxel = (unsigned)std::max(1.0, (double)run->photons_per_voxel * f);
  }
  const int old_variant = c->variant, old_variant_fl = c->variant_fl, old_l2 = c->l2_window, old_agg = c->phd_agg,
            old_form = c->pass_form;
  const uint32_t old_relaunch = c->relaunch;
  /* forms: 0 SIMT-arranged pass, 1 branching pass, and when the run tallies
   * the hitting density 2 the branching pass with the register-held sums,
   * 3 the SIMT-arranged pass with the warp-aggregated adds; last, form 0
   * with relaunch 2.  Each with and without the L2 window. */
  const int n_forms = (r.fluence || r.photons_per_voxel) ? 5 : 3;
  const int n_cfg = 2 * n_forms;
  auto apply = [&](int cfg) {
    const int form = cfg >> 1;
    const bool pairs = form == n_forms - 1;
    c->l2_window = cfg & 1;
    c->phd_agg = pairs ? 0 : form == 2 ? 1 : form == 3 ? 2 : 0;
    c->pass_form = form == 1 ? 1 : 0;
    c->relaunch = pairs ? 2u : 1u;
  };
  /* per (variant, configuration): the best excitation and emission launch
   * times of the sample runs; each phase then takes its fastest variant */
  std::vector<double> ms_exc((size_t)MCFL_N_VARIANTS * n_cfg, 1e30), ms_fl((size_t)MCFL_N_VARIANTS * n_cfg, 1e30);
  double photons = 0.0;
  for (int v = 0; v < MCFL_N_VARIANTS; ++v) {
    for (int cfg = 0; cfg < n_cfg; ++cfg) {
      c->variant = v;
      c->variant_fl = -1;
      apply(cfg);
      for (int rep = 0; rep < 3; ++rep) { /* the first run records the graph */
        mcfl_run_out o;
        std::memset(&o, 0, sizeof(o));
        const int rc = mcfl_run(c, m, &r, &o);
        if (rc != MCFL_OK) {
          c->variant = old_variant;
          c->variant_fl = old_variant_fl;
          c->l2_window = old_l2;
          c->phd_agg = old_agg;
          c->pass_form = old_form;
          c->relaunch = old_relaunch;
          return rc;
        }
        photons = (double)o.stats_exc[0] + (double)o.stats_fl[0];
        if (rep > 0) {
          const size_t i = (size_t)v * n_cfg + cfg;
          ms_exc[i] = std::min(ms_exc[i], (double)o.ms_exc);
          ms_fl[i] = std::min(ms_fl[i], (double)o.ms_fl);
        }
      }
    }
  }
  int best_cfg = 0, best_v = 0, best_vf = 0;
  double best = 1e300;
  for (int cfg = 0; cfg < n_cfg; ++cfg) {
    int ve = 0, vf = 0;
    for (int v = 1; v < MCFL_N_VARIANTS; ++v) {
      if (ms_exc[(size_t)v * n_cfg + cfg] < ms_exc[(size_t)ve * n_cfg + cfg]) ve = v;
      if (ms_fl[(size_t)v * n_cfg + cfg] < ms_fl[(size_t)vf * n_cfg + cfg]) vf = v;
    }
    const double t = ms_exc[(size_t)ve * n_cfg + cfg] + (r.photons_per_voxel ? ms_fl[(size_t)vf * n_cfg + cfg] : 0.0);
    if (t < best) {
      best = t;
      best_cfg = cfg;
      best_v = ve;
      best_vf = r.photons_per_voxel ? vf : ve;
    }
  }
  c->variant = best_v;
  c->variant_fl = best_vf;
  apply(best_cfg);
  const double rate = best > 0 && best < 1e299 ? photons / (best * 1e-3) : 0.0;
  if (variant_out) *variant_out = best_v;
  if (rate_out) *rate_out = rate;
  return MCFL_OK;
}
