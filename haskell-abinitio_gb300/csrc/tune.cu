// Autotuner of the task budgets of the direct J/K and gradient builds.
//
// A task of a quartet-class list is (bra pair, up to task_kets kets of one
// segment, a range of bra primitives); lane_prims bounds the primitive
// quartets one lane evaluates in one task (see build_task_lists in jk.cu).
// Both set the granularity of a persistent class launch: small tasks balance
// the SMs and shorten the tail, large ones amortise the per-task bra loads and
// the scatter.  The best values depend on the basis (primitives per shell),
// the molecule sizes and the screening, so the tuner measures them on the
// caller's basis and density.
//
// Method: every class has its own launch and its own budgets, so the launch
// time of a class depends on its budgets alone.  The tuner therefore runs
// whole builds with the per-class launches serialised and timed by CUDA
// events, once per candidate (all classes at once), and keeps per class the
// fastest candidate when it beats the default by more than 3%.  Two sweeps:
// lane_prims x {1/4, 1/2, 1, 2, 4}, then, for the warp-per-quartet classes,
// kets per task in {1, 2, 4, 8}.  Each candidate is the minimum of `reps`
// builds after one warm-up build.  The context's profile counters are left as
// they were apart from the launch count.
#include "gbhf_internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace gbhf {

namespace {

struct TuneTarget {
  int which, ncls;
  int* lp;
  int* tk;
};

// One timed build of the target; per-class milliseconds (both precisions) into ms.
gbhf_status timed_build(gbhf_ctx* c, const TuneTarget& t, const double* d_D, double* d_out, int precision,
                        double schwarz, double mixed_cutoff, std::vector<double>& ms) {
  ms.assign(t.ncls, 0.0);
  if (t.which == 0) {
    double before[NCOMBO][2];
    for (int k = 0; k < NCOMBO; ++k)
      for (int p = 0; p < 2; ++p) before[k][p] = c->prof.cls[k][p][3];
    c->tasks.thr_all = -1;   // rebuild the lists with the current budgets
    GBHF_CUDA(c, cudaMemsetAsync(d_out, 0, (size_t)c->basis.stacked * sizeof(double), c->stream));
    GBHF_TRY(jk_build(c, d_D, d_out, precision, schwarz, mixed_cutoff, 1.0));
    for (int k = 0; k < NCOMBO; ++k)
      for (int p = 0; p < 2; ++p) ms[k] += c->prof.cls[k][p][3] - before[k][p];
  } else {
    double before[NCOMBO_MAX][2];
    for (int k = 0; k < NCOMBO_MAX; ++k)
      for (int p = 0; p < 2; ++p) before[k][p] = c->prof.gcls_ms[k][p];
    GBHF_CUDA(c, cudaMemsetAsync(d_out, 0, 3 * (size_t)std::max(c->basis.natoms, 1) * sizeof(double), c->stream));
    GBHF_TRY(grad_2e(c, d_D, schwarz, mixed_cutoff, precision, d_out));
    for (int k = 0; k < NCOMBO_MAX; ++k)
      for (int p = 0; p < 2; ++p) ms[k] += c->prof.gcls_ms[k][p] - before[k][p];
  }
  GBHF_CUDA(c, cudaStreamSynchronize(c->stream));
  return GBHF_OK;
}

gbhf_status min_of(gbhf_ctx* c, const TuneTarget& t, const double* d_D, double* d_out, int precision,
                   double schwarz, double mixed_cutoff, int reps, std::vector<double>& best) {
  std::vector<double> ms;
  best.assign(t.ncls, 1e300);
  for (int r = 0; r < reps; ++r) {
    GBHF_TRY(timed_build(c, t, d_D, d_out, precision, schwarz, mixed_cutoff, ms));
    for (int k = 0; k < t.ncls; ++k) best[k] = std::min(best[k], ms[k]);
  }
  return GBHF_OK;
}

// Per class: take the candidate if it beats the incumbent by more than 3%.
void keep_faster(int ncls, const std::vector<double>& cand_ms, const std::vector<int>& cand, std::vector<double>& inc_ms,
                 std::vector<int>& inc) {
  for (int k = 0; k < ncls; ++k)
    if (inc_ms[k] > 0.02 && cand_ms[k] < 0.97 * inc_ms[k]) {
      inc_ms[k] = cand_ms[k];
      inc[k] = cand[k];
    }
}

}  // namespace

gbhf_status autotune_dev(gbhf_ctx* c, int which, const double* d_D, int precision, double schwarz,
                         double mixed_cutoff, int reps, double* class_ms) {
  TuneTarget t{which, which == 0 ? NCOMBO : NCOMBO_MAX, which == 0 ? c->jk_lp : c->gr_lp,
               which == 0 ? c->jk_tk : c->gr_tk};
  reps = std::max(1, reps);
  const Profile saved = c->prof;
  c->prof.events = true;
  DBuf<double> out;
  const size_t nout = which == 0 ? (size_t)c->basis.stacked : 3 * (size_t)std::max(c->basis.natoms, 1);
  gbhf_status st = GBHF_OK;
  std::vector<double> ms, base_ms, cur_ms;
  std::vector<int> lp0(t.lp, t.lp + t.ncls), tk0(t.tk, t.tk + t.ncls);
  auto body = [&]() -> gbhf_status {
    GBHF_CUDA(c, out.alloc(std::max<size_t>(nout, 1)));
    GBHF_TRY(timed_build(c, t, d_D, out.p, precision, schwarz, mixed_cutoff, ms));   // warm-up
    GBHF_TRY(min_of(c, t, d_D, out.p, precision, schwarz, mixed_cutoff, reps, base_ms));
    // sweep 1: primitive quartets per lane and task
    std::vector<int> best_lp = lp0;
    cur_ms = base_ms;
    static const double mult[] = {0.25, 0.5, 2.0, 4.0};
    for (double m : mult) {
      std::vector<int> cand(t.ncls);
      for (int k = 0; k < t.ncls; ++k) cand[k] = std::max(1, (int)std::lround(lp0[k] * m));
      std::copy(cand.begin(), cand.end(), t.lp);
      GBHF_TRY(min_of(c, t, d_D, out.p, precision, schwarz, mixed_cutoff, reps, ms));
      keep_faster(t.ncls, ms, cand, cur_ms, best_lp);
    }
    std::copy(best_lp.begin(), best_lp.end(), t.lp);
    // sweep 2: kets per task of the warp-per-quartet classes
    bool any_warp = false;
    for (int k = 0; k < t.ncls; ++k) any_warp |= !lane_per_ket(which, k) && cur_ms[k] > 0.02;
    if (any_warp) {
      std::vector<int> best_tk = tk0;
      static const int kets[] = {1, 2, 4, 8};
      for (int q : kets) {
        std::vector<int> cand = tk0;
        bool differs = false;
        for (int k = 0; k < t.ncls; ++k)
          if (!lane_per_ket(which, k)) {
            differs |= cand[k] != q;
            cand[k] = q;
          }
        if (!differs) continue;
        std::copy(cand.begin(), cand.end(), t.tk);
        GBHF_TRY(min_of(c, t, d_D, out.p, precision, schwarz, mixed_cutoff, reps, ms));
        keep_faster(t.ncls, ms, cand, cur_ms, best_tk);
      }
      std::copy(best_tk.begin(), best_tk.end(), t.tk);
    }
    return GBHF_OK;
  };
  st = body();
  const long long launches = c->prof.launches;
  c->prof = saved;
  c->prof.launches = launches;
  if (which == 0) c->tasks.thr_all = -1;   // lists of the old budgets are stale
  if (st != GBHF_OK) {
    std::copy(lp0.begin(), lp0.end(), t.lp);
    std::copy(tk0.begin(), tk0.end(), t.tk);
    return st;
  }
  c->tuned[which] = true;
  if (class_ms) {
    for (int k = 0; k < t.ncls; ++k) {
      class_ms[2 * k] = base_ms[k];
      class_ms[2 * k + 1] = cur_ms[k];
    }
  }
  return GBHF_OK;
}

}  // namespace gbhf
