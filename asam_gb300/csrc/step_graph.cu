// Device-driven Rosenbrock step (FP64): the whole step -- stages, Jacobian,
// flux RHS and every BiCGStab solve -- is one CUDA graph, and the BiCGStab
// iteration loop is a graph WHILE node whose condition a kernel sets from the
// device-resident Krylov scalars (converged, broken down, or the iteration
// limit reached: the loop always ends).  The second half of an iteration is an
// IF node that runs only while nothing has ended the solve.  The host launches
// the step once and reads the per-stage MaxIter/Tol outputs once.
//
// The kernels and their order are those of the host-driven solver
// (bicgstab_dev, capi.cu), so the results are bit-identical; only the exit
// decisions move from the host to a condition kernel.
#include <cmath>

#include "context.h"
#include "kernels.cuh"

using namespace asam;

namespace {

__global__ void k_ks_init(KrylovScalars* sc, double tol, int maxiter) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  KrylovScalars z = {};
  z.tol = tol;
  z.maxiter = maxiter;
  *sc = z;
}

// p = r on the first iteration, else beta = (rho/rho_old)*(alpha/omega) and
// p = beta*(p - omega*v) + r (the operations of k_beta + k_pupdate)
// ---- the refined solve's outer FP64 refinement (bicgstab_refined, capi.cu)
// as device kernels with the host driver's arithmetic: outer scalars in `so`
// (rnorm0, rnorm, tol = the target |r0|*Tol, iter = outer passes, out_*),
// the inner BiCGStab's in `sc`.
constexpr int kMaxOuter = 8;  // the host driver's refinement limit

__global__ void k_ref_init(cudaGraphConditionalHandle hnd, KrylovScalars* so, const KrylovScalars* sc, double tol) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double rr0 = sc->dot_a;
  KrylovScalars z = {};
  z.rnorm0 = sqrt(rr0);
  z.rnorm = z.rnorm0;
  z.tol = tol * z.rnorm0;
  if (isnan(rr0)) {
    z.rnorm0 = rr0;  // NaN: the decoder reports it
  } else if (z.rnorm0 == 0.0) {
    z.done = 2;
    z.out_iters = 1;
    z.out_tol = 0.0;
  }
  *so = z;
  cudaGraphSetConditional(hnd, (z.done == 0 && !isnan(rr0)) ? 1u : 0u);
}

// b32 = (float)((1/|r|) * r): the inner system's right-hand side at unit scale
__global__ void k_ref_scale(size_t len, const double* __restrict__ r, const KrylovScalars* so, float* __restrict__ y) {
  const double s = 1.0 / so->rnorm;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = (float)(s * r[q]);
}

// the inner solve's scalars: tolerance 0.5*target/|r| clamped to [1e-6, 1e-2]
__global__ void k_ref_inner_init(KrylovScalars* sc, const KrylovScalars* so, int maxiter) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double tin = 0.5 * so->tol / so->rnorm;
  if (tin < 1e-6) tin = 1e-6;
  if (tin > 1e-2) tin = 1e-2;
  KrylovScalars z = {};
  z.tol = tin;
  z.maxiter = maxiter;
  *sc = z;
}

// after the inner solve: its iteration count into the total (the host
// driver's rule for the half-step and limit sentinels), its passes for the
// launch count, a give-up of the persistent schedule
__global__ void k_ref_accum(KrylovScalars* so, const KrylovScalars* sc, int maxiter) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int it = sc->out_iters;
  so->out_iters += it < 0 ? -it : (it > maxiter ? it / 2 : it);
  so->passes1 += sc->iter;
  const int seconds = (sc->done == 1 || sc->done == 3) ? sc->iter - 1 : sc->iter;
  so->passes2 += seconds > 0 ? seconds : 0;
  if (sc->gs_err) so->gs_err = 1;
}

// x += |r| * correction
__global__ void k_ref_add(size_t len, const float* __restrict__ x32, const KrylovScalars* so, double* __restrict__ y) {
  const double s = so->rnorm;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = y[q] + s * (double)x32[q];
}

// the FP64 residual's norm decides: converged, another pass, or the limit
__global__ void k_ref_check(cudaGraphConditionalHandle hnd, KrylovScalars* so, const KrylovScalars* sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double rr = sc->dot_a;
  const int pass = so->iter + 1;
  so->iter = pass;
  if (isnan(rr)) {
    so->rnorm0 = rr;  // NaN: the decoder reports it
    cudaGraphSetConditional(hnd, 0u);
    return;
  }
  const double rnorm = sqrt(rr);
  so->rnorm = rnorm;
  so->out_tol = rnorm;
  if (rnorm <= so->tol) {
    so->done = 2;
  } else if (pass == kMaxOuter) {
    so->out_iters = 2 * so->out_iters;  // the limit's sentinel
  }
  cudaGraphSetConditional(hnd, (so->done == 0 && pass < kMaxOuter) ? 1u : 0u);
}

// enter a WHILE loop: its handle's default is applied once per graph launch
// only, and a loop nested in another runs once per outer pass
__global__ void k_cond_enter(cudaGraphConditionalHandle hnd) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(hnd, 1u);
}

__global__ void k_cond_running(cudaGraphConditionalHandle hnd, const KrylovScalars* sc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(hnd, sc->done == 0 ? 1u : 0u);
}

// end of an iteration: count it, write the reference's outputs, continue?
__global__ void k_cond_next(cudaGraphConditionalHandle hnd, KrylovScalars* sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int it = sc->iter + 1;
  sc->iter = it;
  const int done = sc->done;
  if (done == 1) {
    sc->out_iters = -it;
    sc->out_tol = sc->rnorm;
  } else if (done == 2) {
    sc->out_iters = it;
    sc->out_tol = sc->rnorm;
  } else if (done == 3) {
    sc->out_iters = it;
    sc->out_tol = 0.0;
  } else {
    sc->out_iters = 2 * it;  // the limit's sentinel, replaced if the loop goes on
    sc->out_tol = sc->rnorm;
  }
  cudaGraphSetConditional(hnd, (done == 0 && it < sc->maxiter) ? 1u : 0u);
}

constexpr int kB = 256;
inline int grid_of(const Launch& L, size_t n) {
  size_t g = (n + kB - 1) / kB, cap = (size_t)L.sm_count * 16;
  return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

// A conditional handle of the graph being captured on stream s.
int make_handle(cudaStream_t s, unsigned dflt, cudaGraphConditionalHandle* hnd) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, nullptr, nullptr, nullptr));
  if (st != cudaStreamCaptureStatusActive || !g) return kCudaError;
  CK(cudaGraphConditionalHandleCreate(hnd, g, dflt, cudaGraphCondAssignDefault));
  return kOk;
}

// Adds a conditional node with handle hnd after the current capture position of
// stream s and starts capturing its body on stream body_s.
int begin_conditional(cudaStream_t s, cudaStream_t body_s, cudaGraphConditionalNodeType type,
                      cudaGraphConditionalHandle hnd) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CK(cudaStreamGetCaptureInfo(s, &st, nullptr, &g, &deps, nullptr, &ndeps));
  if (st != cudaStreamCaptureStatusActive || !g) return kCudaError;
  cudaGraphNodeParams prm = {};
  prm.type = cudaGraphNodeTypeConditional;
  prm.conditional.handle = hnd;
  prm.conditional.type = type;
  prm.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &prm));
  cudaGraph_t body = prm.conditional.phGraph_out[0];
  CK(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  CK(cudaStreamBeginCaptureToGraph(body_s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  return kOk;
}

int end_conditional(cudaStream_t body_s) {
  cudaGraph_t body = nullptr;
  CK(cudaStreamEndCapture(body_s, &body));
  return kOk;
}

// kernels per pass of the loop body (first half) and of the IF body (second
// half), counted while recording, to report how many kernels a step launched
struct BodyCounts {
  long long h1 = 0, h2 = 0;
  long long outer = 0;  // refined solve: kernels per outer pass outside the inner loop
};

// Records the iterations of one device-driven BiCGStab solve of A x = b
// (x = 0 on entry, the scalars in h->sc initialised by the caller) into the
// capture of h->L.stream.  The bodies are recorded on the context's two
// capture streams (h->L.stream is switched to them while their kernels are
// emitted).
template <typename T>
int record_bicgstab(asam_ctx* h, const T* val, T* x, const T* b, Work<T>& w, BodyCounts* bc) {
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  const size_t len = h->len;
  const cudaStream_t s0 = h->L.stream, s1 = h->cap_stream[0], s2 = h->cap_stream[1];
  CK(cudaMemcpyAsync(w.r, b, len * sizeof(T), cudaMemcpyDeviceToDevice, s0));
  CK(cudaMemcpyAsync(w.rt, w.r, len * sizeof(T), cudaMemcpyDeviceToDevice, s0));
  launch_dot(h->L, d, nc, w.r, w.r, h->partial, h->sc, OP_RNORM0, nullptr);
  // WHILE: one iteration per pass; the host-driven solver always enters it
  cudaGraphConditionalHandle wh, ih;
  int rc;
  if ((rc = make_handle(s0, 1u, &wh))) return rc;
  k_cond_enter<<<1, 1, 0, s0>>>(wh);
  count_launches(1);
  if ((rc = begin_conditional(s0, s1, cudaGraphCondTypeWhile, wh))) return rc;
  h->L.stream = s1;
  const long long n1 = thread_launches();
  launch_dot(h->L, d, nc, w.rt, w.r, h->partial, h->sc, OP_RHO, nullptr);
  launch_pupdate_auto(h->L, len, h->sc, w.r, w.v, w.p);
  psolve_dev<T>(h, val, w.p, w.ph, w);
  launch_matvec_dot(h->L, d, nc, val, w.ph, w.v, w.rt, h->partial, h->sc, OP_ALPHA);
  launch_axpy_dot(h->L, d, nc, h->sc, SEL_ALPHA, -1.0, w.v, w.r, h->partial, OP_RNORM_HALF);
  launch_xupdate_half(h->L, len, h->sc, w.ph, x);
  // IF nothing ended the solve: the second half
  if ((rc = make_handle(s1, 0u, &ih))) return rc;
  k_cond_running<<<1, 1, 0, s1>>>(ih, h->sc);
  count_launches(1);
  if ((rc = begin_conditional(s1, s2, cudaGraphCondTypeIf, ih))) return rc;
  h->L.stream = s2;
  const long long n2 = thread_launches();
  psolve_dev<T>(h, val, w.r, w.rh, w);
  launch_matvec_dot2(h->L, d, nc, val, w.rh, w.t, w.r, h->partial, h->sc, OP_STORE_A, OP_OMEGA);
  launch_axpy_dot(h->L, d, nc, h->sc, SEL_OMEGA, -1.0, w.t, w.r, h->partial, OP_RNORM_FULL);
  launch_xupdate(h->L, len, h->sc, 1, w.ph, w.rh, x);
  bc->h2 = thread_launches() - n2;
  if ((rc = end_conditional(s2))) return rc;
  h->L.stream = s1;
  k_cond_next<<<1, 1, 0, s1>>>(wh, h->sc);
  count_launches(1);
  bc->h1 = thread_launches() - n1 - bc->h2;
  if ((rc = end_conditional(s1))) return rc;
  h->L.stream = s0;
  return check_launch();
}

// FP64 (the drop-in): its outputs land in h->sc
int record_solve(asam_ctx* h, double* x, const double* b, int maxiter, double tol, BodyCounts* bc) {
  k_ks_init<<<1, 1, 0, h->L.stream>>>(h->sc, tol, maxiter);
  count_launches(1);
  return record_bicgstab<double>(h, h->val, x, b, h->w64, bc);
}

// The refined solve (bicgstab_refined): r = b, |r0|; WHILE the FP64
// residual is above Tol*|r0| and fewer than 8 passes ran: the inner FP32
// BiCGStab on A d = r/|r| (its own WHILE/IF loop), x += |r| d, r = b - A x
// (FP64) and its norm.  The outputs land in h->ref_sc.
int record_refined(asam_ctx* h, double* x, const double* b, int maxiter, double tol, BodyCounts* bc) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  const size_t len = h->len;
  const cudaStream_t s0 = L.stream;
  double* r = h->w64.r;
  CK(cudaMemcpyAsync(r, b, len * sizeof(double), cudaMemcpyDeviceToDevice, s0));  // r = b - A*0
  launch_dot(L, d, nc, r, r, h->partial, h->sc, OP_STORE_A, nullptr);
  prepare_inner(h);  // the x-line factors of this matrix, once (they depend on the matrix only)
  cudaGraphConditionalHandle oh;
  int rc;
  if ((rc = make_handle(s0, 0u, &oh))) return rc;
  k_ref_init<<<1, 1, 0, s0>>>(oh, h->ref_sc, h->sc, tol);
  count_launches(1);
  // the outer body is recorded on a stream of its own; the inner loop's
  // bodies use the context's two capture streams
  cudaStream_t so_s = h->cap_stream[2];
  if ((rc = begin_conditional(s0, so_s, cudaGraphCondTypeWhile, oh))) return rc;
  h->L.stream = so_s;
  const long long n0 = thread_launches();
  k_ref_scale<<<grid_of(h->L, len), kB, 0, so_s>>>(len, r, h->ref_sc, h->b32);
  CK(cudaMemsetAsync(h->x32, 0, len * sizeof(float), so_s));
  k_ref_inner_init<<<1, 1, 0, so_s>>>(h->sc, h->ref_sc, maxiter);
  count_launches(2);
  BodyCounts ib;
  if ((rc = record_bicgstab<float>(h, h->val32, h->x32, h->b32, h->w32, &ib))) return rc;
  h->L.stream = so_s;
  k_ref_accum<<<1, 1, 0, so_s>>>(h->ref_sc, h->sc, maxiter);
  k_ref_add<<<grid_of(h->L, len), kB, 0, so_s>>>(len, h->x32, h->ref_sc, x);
  count_launches(2);
  asam_fma::launch_resid_dot(h->L, d, nc, h->val, x, b, r, h->partial, h->sc, OP_STORE_A, nullptr);
  k_ref_check<<<1, 1, 0, so_s>>>(oh, h->ref_sc, h->sc);
  count_launches(1);
  const long long nin = thread_launches() - n0;  // outer body with one pass of each inner body recorded
  bc->h1 = ib.h1;
  bc->h2 = ib.h2;
  bc->outer = nin - ib.h1 - ib.h2;
  if ((rc = end_conditional(so_s))) return rc;
  h->L.stream = s0;
  return check_launch();
}

// Records the whole step (ros_step_dev's operations with device-driven solves).
int record_step(asam_ctx* h, double* c, double dt, BodyCounts* bc) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  const size_t len = h->len;
  CK(cudaMemcpyAsync(h->cold, c, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  for (int is = 0; is < h->nstage; ++is) {
    launch_exchange_cell(L, d, nc, c);
    launch_bound_cond(L, d, nc, 0, h->bc, c);
    int rc;
    if (is == 0 && (rc = jac_dev(h, c, dt))) return rc;
    if ((rc = fcn_dev(h, c, h->rhs))) return rc;
    launch_scale_host(L, len, dt, h->rhs);
    for (int js = 0; js < is; ++js) launch_axpy_host(L, len, h->beta[is * 4 + js], h->incr + (size_t)js * len, h->rhs);
    double* x = h->incr + (size_t)is * len;
    CK(cudaMemsetAsync(x, 0, len * sizeof(double), L.stream));
    const bool refined = h->cfg.precision == ASAM_PREC_FP32_REFINED;
    rc = refined ? record_refined(h, x, h->rhs, h->cfg.bicgstab_maxiter, h->cfg.bicgstab_tol, bc)
                 : record_solve(h, x, h->rhs, h->cfg.bicgstab_maxiter, h->cfg.bicgstab_tol, bc);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->stage_sc + is, refined ? h->ref_sc : h->sc, sizeof(KrylovScalars),
                       cudaMemcpyDeviceToDevice, L.stream));
    launch_exchange_cell(L, d, nc, x);
    launch_exchange_cell(L, d, nc, x);
    CK(cudaMemcpyAsync(c, h->cold, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    for (int js = 0; js <= is; ++js) launch_axpy_host(L, len, h->alpha[is * 4 + js], h->incr + (size_t)js * len, c);
  }
  return check_launch();
}

// after a failed recording: end the captures still open on the body streams
void abandon_bodies(asam_ctx* h) {
  for (cudaStream_t s : h->cap_stream) {
    cudaStreamCaptureStatus st;
    if (s && cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(s, &g);
    }
  }
  cudaGetLastError();
}

}  // namespace

namespace asam {

void step_graph_free(asam_ctx* h) {
  if (h->step_exec) cudaGraphExecDestroy(h->step_exec);
  h->step_exec = nullptr;
  h->step_c = nullptr;
}

// The per-context resources of recorded steps: the stage scalars and the two
// capture streams of the loop bodies.
int step_graph_prepare(asam_ctx* h) {
  if (!h->stage_sc) {
    CK(cudaMalloc((void**)&h->stage_sc, 4 * sizeof(KrylovScalars)));
    CK(cudaMalloc((void**)&h->ref_sc, sizeof(KrylovScalars)));
    CK(cudaMallocHost((void**)&h->stage_sc_host, 4 * sizeof(KrylovScalars)));
    for (auto& s : h->cap_stream) CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  }
  return kOk;
}

// Records one device-driven step of h into the capture running on
// h->L.stream; kernels outside the loops and per pass of each loop body are
// returned for the launch count.  On failure the body captures are closed.
int step_record(asam_ctx* h, double* c, double dt, long long* n_fixed, long long* n_h1, long long* n_h2,
                long long* n_outer) {
  const cudaStream_t s0 = h->L.stream;
  const long long t0 = thread_launches();
  BodyCounts bc;
  const int rc = record_step(h, c, dt, &bc);
  h->L.stream = s0;
  const long long nrec = thread_launches() - t0;
  count_launches(-nrec);  // recorded, not run
  if (rc) {
    abandon_bodies(h);
    return rc;
  }
  *n_h1 = bc.h1;
  *n_h2 = bc.h2;
  *n_outer = bc.outer;
  *n_fixed = nrec - h->nstage * (bc.outer + bc.h1 + bc.h2);
  return kOk;
}

// Decodes the stage scalars of one recorded step (host copies) into the
// reference's per-stage MaxIter/Tol outputs and a status; *ran receives the
// kernels the step ran (fixed part plus the passes of its loops).
int step_outputs(const asam_ctx* h, const KrylovScalars* ks, long long n_fixed, long long n_h1, long long n_h2,
                 long long n_outer, int* iters, double* resid, long long* ran) {
  int status = kOk;
  long long nr = n_fixed;
  const bool refined = h->cfg.precision == ASAM_PREC_FP32_REFINED;
  for (int is = 0; is < h->nstage; ++is) {
    const KrylovScalars& k = ks[is];
    if (refined) {  // outer passes, each with its inner loop's passes
      nr += k.iter * n_outer + (long long)k.passes1 * n_h1 + (long long)k.passes2 * n_h2;
    } else {
      const int passes = k.iter;                                           // first halves
      const int seconds = (k.done == 1 || k.done == 3) ? passes - 1 : passes;  // second halves
      nr += passes * n_h1 + (seconds > 0 ? seconds : 0) * n_h2;
    }
    if (k.gs_err) {
      set_last_error("persistent Gauss-Seidel schedule: a dependency wait gave up", __FILE__, __LINE__);
      return kCudaError;
    }
    if (std::isnan(k.rnorm0) || (k.done != 3 && std::isnan(k.rnorm))) {
      set_last_error("NaN in the stage system", __FILE__, __LINE__);
      return kNanDetected;
    }
    if (iters) iters[is] = k.out_iters;
    if (resid) resid[is] = k.out_tol;
    int st = kOk;
    if (k.done == 3 && k.rnorm0 > 0.0) st = kBreakdown;
    if (k.done == 0) st = kNotConverged;
    if (st != kOk && status == kOk) status = st;
  }
  *ran = nr;
  return status;
}

// One Rosenbrock step as one graph launch (captured on first use for this
// state pointer, step size and tolerance); the per-stage BiCGStab outputs are
// read once.
int ros_step_graph(asam_ctx* h, double* c, double dt, int* iters, double* resid) {
  if (int rc = step_graph_prepare(h)) return rc;
  const cudaStream_t s0 = h->L.stream;
  if (!h->step_exec || h->step_c != c || h->step_dt != dt || h->step_tol != h->cfg.bicgstab_tol) {
    step_graph_free(h);
    CK(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
    const int rc = step_record(h, c, dt, &h->step_n_fixed, &h->step_n_h1, &h->step_n_h2, &h->step_n_outer);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s0, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&h->step_exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      h->step_exec = nullptr;
      set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
      return kCudaError;
    }
    h->step_c = c;
    h->step_dt = dt;
    h->step_tol = h->cfg.bicgstab_tol;
  }
  CK(cudaGraphLaunch(h->step_exec, s0));
  CK(cudaMemcpyAsync(h->stage_sc_host, h->stage_sc, h->nstage * sizeof(KrylovScalars), cudaMemcpyDeviceToHost, s0));
  CK(cudaStreamSynchronize(s0));
  long long ran = 0;
  const int status = step_outputs(h, h->stage_sc_host, h->step_n_fixed, h->step_n_h1, h->step_n_h2,
                                  h->step_n_outer, iters, resid, &ran);
  if (status == kCudaError || status == kNanDetected) return status;
  count_launches(ran);
  const int rc = check_launch();
  return rc ? rc : status;
}

}  // namespace asam
