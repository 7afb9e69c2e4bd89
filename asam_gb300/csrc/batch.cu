// Batched ensemble: many independent blocks (domains of their own size,
// orography and wind) advanced together on one GPU.
//
// Each member is a complete context with its own CUDA stream.  Host worker
// threads take members largest-first from a shared queue and drive their
// Rosenbrock steps; the Krylov exit decisions of one member (a small
// device-to-host read twice per BiCGStab iteration) then stall only that
// member's thread while the other members' kernels keep the GPU busy, so
// members of very different sizes overlap instead of queueing behind one
// another.  Nothing is shared between members except the device.
//
// One-graph mode (asam_batch_set_graph, FP64 members): the whole run --
// nsteps steps of every member -- is recorded into one CUDA graph, one
// branch per member forked from and joined to a batch stream, each branch
// the member's device-driven steps (BiCGStab loops as WHILE/IF nodes, exit
// decisions on the device) with its per-stage scalars copied into a history
// buffer after every step.  A call is then one graph launch and one read of
// the histories; the kernels are the members' own, so the states are bitwise
// those of the members run alone.
#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "context.h"

using namespace asam;

struct asam_batch {
  std::vector<asam_ctx*> members;
  std::vector<int> order;  // members by decreasing cell count
  int nthreads = 1;
  // one-graph mode
  bool use_graph = false;
  cudaStream_t stream = nullptr;     // fork/join stream of the graph
  std::vector<cudaEvent_t> ev;       // [0] fork, [1+m] join of member m
  cudaGraphExec_t exec = nullptr;
  std::vector<double*> g_c;          // recorded for these device states ...
  std::vector<double> g_dt, g_tol;   // ... step sizes and tolerances
  std::vector<unsigned long long> g_gen;  // ... and members' configurations (graph_gen)
  int g_nsteps = 0;
  std::vector<KrylovScalars*> hist;  // per member: nsteps x 4 stage scalars (device)
  KrylovScalars* hist_host = nullptr;
  size_t hist_cap = 0;               // steps the history buffers hold
  std::vector<long long> n_fixed, n_h1, n_h2, n_outer;  // per member, per recorded step
};

namespace {

int run_member(asam_ctx* h, double* state, double dt, int nsteps, int* iters, double* resid) {
  if (cudaSetDevice(h->device) != cudaSuccess) return kCudaError;
  double* dc;
  int rc = stage_out_begin(h, state, h->len, h->c, &dc, true);
  if (rc) return rc;
  int status = kOk;
  for (int s = 0; s < nsteps; ++s) {
    int it[4] = {0, 0, 0, 0};
    double rs[4] = {0, 0, 0, 0};
    const int st = ros_step_dev(h, dc, dt, it, rs);
    if (st != kOk && st != kNotConverged && st != kBreakdown) return st;
    if (st != kOk && status == kOk) status = st;
    for (int q = 0; q < 4; ++q) {
      if (iters) iters[(size_t)s * 4 + q] = it[q];
      if (resid) resid[(size_t)s * 4 + q] = rs[q];
    }
  }
  rc = stage_out_end(h, state, h->len, dc);
  if (!rc) rc = check_launch();
  if (!rc) {
    CK(cudaStreamSynchronize(h->L.stream));
  }
  return rc ? rc : status;
}

void graph_free(asam_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->g_c.clear();
}

void graph_release(asam_batch* b) {
  graph_free(b);
  for (auto e : b->ev) cudaEventDestroy(e);
  b->ev.clear();
  for (auto p : b->hist) cudaFree(p);
  b->hist.clear();
  if (b->hist_host) cudaFreeHost(b->hist_host);
  b->hist_host = nullptr;
  b->hist_cap = 0;
  if (b->stream) cudaStreamDestroy(b->stream);
  b->stream = nullptr;
}

// Records every member's nsteps device-driven steps into one graph.
int graph_record(asam_batch* b, const std::vector<double*>& dc, const double* dt, int nsteps) {
  const int n = (int)b->members.size();
  if (b->hist_cap < (size_t)nsteps) {
    for (auto p : b->hist) cudaFree(p);
    b->hist.assign(n, nullptr);
    if (b->hist_host) cudaFreeHost(b->hist_host);
    b->hist_host = nullptr;
    b->hist_cap = 0;
    for (int m = 0; m < n; ++m) CK(cudaMalloc((void**)&b->hist[m], (size_t)nsteps * 4 * sizeof(KrylovScalars)));
    CK(cudaMallocHost((void**)&b->hist_host, (size_t)n * nsteps * 4 * sizeof(KrylovScalars)));
    b->hist_cap = nsteps;
  }
  graph_free(b);
  b->n_fixed.assign(n, 0);
  b->n_h1.assign(n, 0);
  b->n_h2.assign(n, 0);
  b->n_outer.assign(n, 0);
  CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = kOk;
  cudaError_t e = cudaEventRecord(b->ev[0], b->stream);
  // branches in decreasing member size, the order the host threads take them:
  // the longest chains start first
  for (int q = 0; q < n && rc == kOk && e == cudaSuccess; ++q) {
    const int m = b->order[q];
    asam_ctx* h = b->members[m];
    e = cudaStreamWaitEvent(h->L.stream, b->ev[0], 0);  // the member's stream joins the capture
    for (int st = 0; st < nsteps && rc == kOk && e == cudaSuccess; ++st) {
      rc = step_record(h, dc[m], dt[m], &b->n_fixed[m], &b->n_h1[m], &b->n_h2[m], &b->n_outer[m]);
      if (rc == kOk)
        e = cudaMemcpyAsync(b->hist[m] + (size_t)st * 4, h->stage_sc, 4 * sizeof(KrylovScalars),
                            cudaMemcpyDeviceToDevice, h->L.stream);
    }
    if (rc == kOk && e == cudaSuccess) e = cudaEventRecord(b->ev[1 + m], h->L.stream);
    if (rc == kOk && e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->ev[1 + m], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
  if (rc == kOk && e == cudaSuccess) e = e2;
  if (rc == kOk && e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (rc) return rc;
  if (e != cudaSuccess) {
    b->exec = nullptr;
    cudaGetLastError();
    set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return kCudaError;
  }
  b->g_c = dc;
  b->g_dt.assign(dt, dt + n);
  b->g_tol.resize(n);
  for (int m = 0; m < n; ++m) b->g_tol[m] = b->members[m]->cfg.bicgstab_tol;
  b->g_gen.assign(n, 0);
  for (int m = 0; m < n; ++m) b->g_gen[m] = b->members[m]->graph_gen;
  b->g_nsteps = nsteps;
  return kOk;
}

// asam_batch_ros_step in one-graph mode.
int graph_run(asam_batch* b, double* const* states, const double* dt, int nsteps, int* iters, double* resid,
              int* status) {
  const int n = (int)b->members.size();
  std::vector<double*> dc(n);
  for (int m = 0; m < n; ++m) {
    asam_ctx* h = b->members[m];
    if (int rc = stage_out_begin(h, states[m], h->len, h->c, &dc[m], true)) return rc;
    CK(cudaStreamSynchronize(h->L.stream));  // copies in (host states) before the launch
  }
  bool same = b->exec && b->g_c == dc && b->g_nsteps == nsteps;
  for (int m = 0; same && m < n; ++m)
    same = b->g_dt[m] == dt[m] && b->g_tol[m] == b->members[m]->cfg.bicgstab_tol &&
           b->g_gen[m] == b->members[m]->graph_gen;  // wall rules, their data, diffusion, ... unchanged
  if (!same) {
    if (int rc = graph_record(b, dc, dt, nsteps)) return rc;
  }
  CK(cudaGraphLaunch(b->exec, b->stream));
  for (int m = 0; m < n; ++m)
    CK(cudaMemcpyAsync(b->hist_host + (size_t)m * nsteps * 4, b->hist[m], (size_t)nsteps * 4 * sizeof(KrylovScalars),
                       cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  int worst = kOk;
  long long ran = 0;
  for (int m = 0; m < n; ++m) {
    asam_ctx* h = b->members[m];
    int st_m = kOk;
    for (int st = 0; st < nsteps; ++st) {
      int it[4] = {0, 0, 0, 0};
      double rs[4] = {0, 0, 0, 0};
      long long r = 0;
      const int st1 = step_outputs(h, b->hist_host + ((size_t)m * nsteps + st) * 4, b->n_fixed[m], b->n_h1[m],
                                   b->n_h2[m], b->n_outer[m], it, rs, &r);
      ran += r;
      if (st1 != kOk && st_m == kOk) st_m = st1;
      for (int q = 0; q < 4; ++q) {
        if (iters) iters[((size_t)m * nsteps + st) * 4 + q] = it[q];
        if (resid) resid[((size_t)m * nsteps + st) * 4 + q] = rs[q];
      }
    }
    if (int rc = stage_out_end(h, states[m], h->len, dc[m])) return rc;
    CK(cudaStreamSynchronize(h->L.stream));
    if (status) status[m] = st_m;
    if (st_m == kCudaError || st_m == kNanDetected) {
      if (worst == kOk || worst == kNotConverged || worst == kBreakdown) worst = st_m;
    } else if (worst == kOk) {
      worst = st_m;
    }
  }
  count_launches(ran);
  const int rc = check_launch();
  return rc ? rc : worst;
}

}  // namespace

extern "C" {

int asam_batch_set_graph(asam_batch* b, int on) {
  if (!b || on < 0 || on > 1) return kBadArg;
  if (!on) {
    graph_release(b);
    b->use_graph = false;
    return kOk;
  }
  for (asam_ctx* h : b->members)
    if (h->L.stream == nullptr || h->device != b->members[0]->device) {
      set_last_error("asam_batch_set_graph: every member must have its own stream, all on one device", __FILE__,
                     __LINE__);
      return kBadArg;
    }
  CK(cudaSetDevice(b->members[0]->device));
  for (asam_ctx* h : b->members)
    if (int rc = step_graph_prepare(h)) return rc;
  if (!b->stream) CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  if (b->ev.empty()) {
    b->ev.resize(b->members.size() + 1, nullptr);
    for (auto& e : b->ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  b->use_graph = true;
  return kOk;
}

int asam_batch_create(int nmember, asam_ctx* const* members, int nthreads, asam_batch** out) {
  if (nmember < 1 || !members || !out || nthreads < 0) return kBadArg;
  *out = nullptr;
  auto* b = new asam_batch();
  for (int m = 0; m < nmember; ++m) {
    if (!members[m]) {
      delete b;
      return kBadArg;
    }
    for (int q = 0; q < m; ++q)
      if (members[q] == members[m]) {  // a context drives one member at a time
        delete b;
        return kBadArg;
      }
    b->members.push_back(members[m]);
    b->order.push_back(m);
  }
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int x, int y) { return b->members[x]->npad > b->members[y]->npad; });
  if (nthreads == 0) nthreads = std::min(nmember, 64);
  b->nthreads = std::min(nthreads, nmember);
  *out = b;
  return kOk;
}

int asam_batch_destroy(asam_batch* b) {
  if (b) graph_release(b);
  delete b;
  return kOk;
}

int asam_batch_ros_step(asam_batch* b, double* const* states, const double* dt, int nsteps, int* iters,
                        double* resid, int* status) {
  if (!b || !states || !dt || nsteps < 1) return kBadArg;
  const int n = (int)b->members.size();
  for (int m = 0; m < n; ++m)
    if (!states[m]) return kBadArg;
  if (b->use_graph) {
    CK(cudaSetDevice(b->members[0]->device));
    return graph_run(b, states, dt, nsteps, iters, resid, status);
  }
  std::atomic<int> next{0};
  std::vector<int> rcs(n, kOk);
  std::vector<std::string> msgs(n);
  auto worker = [&]() {
    for (;;) {
      const int q = next.fetch_add(1);
      if (q >= n) return;
      const int m = b->order[q];
      rcs[m] = run_member(b->members[m], states[m], dt[m], nsteps, iters ? iters + (size_t)m * nsteps * 4 : nullptr,
                          resid ? resid + (size_t)m * nsteps * 4 : nullptr);
      if (rcs[m] != kOk && rcs[m] != kNotConverged && rcs[m] != kBreakdown) msgs[m] = asam_last_error();
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < b->nthreads; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  int worst = kOk;
  bool failed = false;
  for (int m = 0; m < n; ++m) {
    if (status) status[m] = rcs[m];
    const int r = rcs[m];
    if (r != kOk && r != kNotConverged && r != kBreakdown) {  // a failure: report the first
      if (!failed) {
        const std::string msg = "member " + std::to_string(m) + ": " + msgs[m];
        set_last_error(msg.c_str(), __FILE__, __LINE__);
      }
      failed = true;
      worst = r;
    } else if (!failed && worst == kOk) {
      worst = r;
    }
  }
  return worst;
}

}  // extern "C"
