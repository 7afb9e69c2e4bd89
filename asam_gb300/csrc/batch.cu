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

}  // namespace

extern "C" {

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
  delete b;
  return kOk;
}

int asam_batch_ros_step(asam_batch* b, double* const* states, const double* dt, int nsteps, int* iters,
                        double* resid, int* status) {
  if (!b || !states || !dt || nsteps < 1) return kBadArg;
  const int n = (int)b->members.size();
  for (int m = 0; m < n; ++m)
    if (!states[m]) return kBadArg;
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
