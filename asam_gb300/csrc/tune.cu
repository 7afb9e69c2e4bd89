// Autotuner of the refined mode's inner solver.
//
// The settings that decide the speed of an FP32-refined stage solve do not
// change its result beyond the refinement tolerance: the preconditioner
// (Gauss-Seidel sweeps or a line solve along z, x or y), the number of inner
// Gauss-Seidel sweeps, their schedule (persistent tile scheduler or one launch
// per tile level) and the components per CTA.  Which combination is fastest
// depends on the block's size (how many tiles a wavefront level has against
// the SM count), its component count and its wind (how many Krylov iterations
// each preconditioner needs).  The tuner times complete refined stage solves
// of the block's own first stage (its Jacobian and flux RHS at the given
// state) and keeps the fastest setting, searching one setting at a time
// (component group, then sweeps, then schedule, then preconditioner, then
// the CUDA-graph capture of the iterations; an FP64 context only has the
// last to choose).
#include <algorithm>
#include <vector>

#include "context.h"

using namespace asam;

namespace {

struct Setting {
  int inner_precond, inner_gs_iter, gs_schedule, gs_group, graphs;
};

void apply(asam_ctx* h, const Setting& s) {
  h->cfg.inner_precond = s.inner_precond;
  h->cfg.inner_gs_iter = s.inner_gs_iter;
  h->cfg.gs_schedule = s.gs_schedule;
  h->cfg.gs_group = s.gs_group;
  h->use_graphs = s.graphs != 0;
}

int install(asam_ctx* h, const Setting& s) {
  apply(h, s);
  graphs_reset(h);
  if (h->cfg.precision != ASAM_PREC_FP32_REFINED) return kOk;
  if (s.inner_precond == 0 && s.gs_schedule == 0) return gs_schedule_init(h, 1 + s.inner_gs_iter);
  gs_schedule_free(h);
  return kOk;
}

// time of one refined solve of the stage system (after two untimed solves:
// the first runs every half-iteration eagerly, the second captures its graph)
int time_solve(asam_ctx* h, const double* rhs, double* x, cudaEvent_t e0, cudaEvent_t e1, double* ms) {
  for (int rep = 0; rep < 3; ++rep) {
    CK(cudaMemsetAsync(x, 0, h->len * sizeof(double), h->L.stream));
    int it = h->cfg.bicgstab_maxiter;
    double tol = h->cfg.bicgstab_tol;
    CK(cudaEventRecord(e0, h->L.stream));
    const int rc = solve_dev(h, x, rhs, &it, &tol, true);
    CK(cudaEventRecord(e1, h->L.stream));
    CK(cudaEventSynchronize(e1));
    if (rc == kNotConverged || rc == kBreakdown) {
      *ms = 1e30;  // not a candidate
      return kOk;
    }
    if (rc != kOk) return rc;
  }
  float t = 0;
  CK(cudaEventElapsedTime(&t, e0, e1));
  *ms = t;
  return kOk;
}

}  // namespace

extern "C" int asam_autotune(asam_ctx* h, const double* c, double dt, int* choice, double* best_ms) {
  if (!h || !c || !choice) return kBadArg;
  const Setting start{h->cfg.inner_precond, h->cfg.inner_gs_iter, h->cfg.gs_schedule, h->cfg.gs_group,
                      h->use_graphs ? 1 : 0};
  const bool refined = h->cfg.precision == ASAM_PREC_FP32_REFINED;
  const Launch& L = h->L;
  const double* dc;
  int rc = stage_in(h, c, h->len, h->stage_a, &dc);
  if (rc) return rc;
  // the first stage of a step from c: exchanged state, Jacobian, dt*F(c)
  double* cs = h->stage_b;
  CK(cudaMemcpyAsync(cs, dc, h->len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  launch_exchange_cell(L, h->d, h->cfg.ncomp, cs);
  launch_bound_cond(L, h->d, h->cfg.ncomp, 0, h->bc, cs);
  if ((rc = jac_dev(h, cs, dt)) || (rc = fcn_dev(h, cs, h->rhs))) return rc;
  launch_scale_host(L, h->len, dt, h->rhs);
  double* x = h->incr;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  struct Ev {
    cudaEvent_t a, b;
    ~Ev() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } ev{e0, e1};
  Setting best = start;
  if (refined) {
    best.inner_precond = 0;
    best.gs_schedule = 0;
    if (best.gs_group <= 0) best.gs_group = 5;
  }
  best.graphs = 1;
  double best_t = 1e30;
  auto trial = [&](const Setting& s) -> int {
    int r = install(h, s);
    if (r) return r;
    double t = 0;
    if ((r = time_solve(h, h->rhs, x, e0, e1, &t))) return r;
    if (t < best_t) {
      best_t = t;
      best = s;
    }
    return kOk;
  };
  const int nc = h->cfg.ncomp;
  if (!refined) {  // the FP64 path: only the graph capture of its iterations to choose
    if ((rc = trial(best))) return rc;
    Setting s = best;
    s.graphs = 0;
    if ((rc = trial(s))) return rc;
  }
  // 1. components per CTA
  if (refined) {
    std::vector<int> groups;
    for (int g : {1, 2, 4, 5, 8, nc})
      if (g >= 1 && g <= nc && g <= 16 && std::find(groups.begin(), groups.end(), g) == groups.end())
        groups.push_back(g);
    Setting s = best;
    for (int g : groups) {
      s.gs_group = g;
      if ((rc = trial(s))) return rc;
    }
  }
  // 2. inner sweeps
  if (refined) {
    Setting s = best;
    for (int it : {0, 1, 2, 3}) {
      if (it == best.inner_gs_iter) continue;
      s.inner_gs_iter = it;
      if ((rc = trial(s))) return rc;
    }
  }
  // 3. schedule
  if (refined) {
    Setting s = best;
    s.gs_schedule = 1;
    if ((rc = trial(s))) return rc;
  }
  // 4. preconditioner: the line solves along z, x and y
  if (refined) {
    Setting s = best;
    for (int p : {1, 2, 3}) {
      s.inner_precond = p;
      if ((rc = trial(s))) return rc;
    }
  }
  // 5. graph capture of the iterations
  if (refined) {
    Setting s = best;
    s.graphs = 0;
    if ((rc = trial(s))) return rc;
  }
  if ((rc = install(h, best))) return rc;
  choice[0] = best.inner_precond;
  choice[1] = best.inner_gs_iter;
  choice[2] = best.gs_schedule;
  choice[3] = best.gs_group;
  choice[4] = best.graphs;
  if (best_ms) *best_ms = best_t;
  return check_launch();
}
