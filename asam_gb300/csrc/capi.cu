// C-ABI of the GB300 transport-stage library: context, staging of host
// pointers, and the host-side drivers of BiCGStab, the preconditioner and the
// Rosenbrock stage.  The drivers keep every Krylov scalar on the device; the
// host only reads the convergence flag twice per iteration.
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include <string>

#include "context.h"

#include <atomic>
#include <mutex>

namespace asam {
static std::atomic<long long> g_launches{0};
static thread_local long long t_launches = 0;  // this thread's share (capture bookkeeping)
void count_launches(long long n) {
  g_launches.fetch_add(n, std::memory_order_relaxed);
  t_launches += n;
}
long long thread_launches() { return t_launches; }
static thread_local std::string g_last_error;
void set_last_error(const char* msg, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s (%s:%d)", msg, file, line);
  g_last_error = buf;
}
}  // namespace asam

using namespace asam;

namespace {

// Host restatement of InitRos3MetC's coefficient tables (ADVECT/Int_Mod.f90:78-261).
int ros_coeffs(int method, double* beta0_out, double alpha[16], double beta[16], double gamma1[5]) {
  double a[4][4] = {{0}}, b[4][4] = {{0}}, gm[5] = {0};
  double beta0 = 0;
  int nStage = 0;
  auto scale_all = [&]() {
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        a[i][j] *= beta0;
        b[i][j] *= beta0;
      }
  };
  switch (method) {
    case ASAM_ROS3AMF:
      nStage = 2;
      beta0 = (double)(0.5f + sqrtf(3.0f) / 6.0f);  // single-precision literals in the Fortran
      a[0][0] = 2.0 / 3.0;
      a[1][0] = 5.0 / 4.0;
      a[1][1] = 3.0 / 4.0;
      b[1][0] = -4.0 / 3.0;
      gm[1] = 0.666666666666667;
      gm[2] = 1.0;
      break;
    case ASAM_ROSRK32: {
      nStage = 3;
      double theta = 1.0 / 3.0 * atan(sqrt(2.0) / 4.0);
      beta0 = 1.0 - 0.5 * sqrt(2.0) * cos(theta) + 0.5 * sqrt(6.0) * sin(theta);
      double g32 = 0.5 - 3.0 * beta0;
      double g31 = -(6.0 * beta0 * beta0 * beta0 - 12.0 * beta0 * beta0 + 6.0 * (1.0 + g32) * beta0 + 2.0 * g32 * g32 - 0.5) /
                   (1.0 + 2.0 * g32);
      double g21 = -(3.0 * beta0 + g31 + g32);
      double tt[3][3] = {{1.0, 0, 0}, {-g21 / beta0, 1.0, 0}, {-g31 / beta0 + g32 * g21 / (beta0 * beta0), -g32 / beta0, 1.0}};
      double al[3][3] = {{0.5, 0, 0}, {0.5, 0.5, 0}, {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0}};
      double be[3][3] = {{0, 0, 0}, {g21 / beta0, 0, 0}, {g31 / beta0, g32 / beta0, 0}};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double s = 0.0, s2 = 0.0;
          for (int k = 0; k < 3; ++k) {
            s = s + al[i][k] * tt[k][j];
            s2 = s2 + be[i][k] * tt[k][j];
          }
          a[i][j] = s;
          b[i][j] = s2;
        }
      gm[2] = 1.0;
      break;
    }
    case ASAM_ROSEUL:
      beta0 = 1.0;
      nStage = 1;
      a[0][0] = 1.0;
      gm[1] = 1.0;
      break;
    case ASAM_ROS3P:
      nStage = 3;
      beta0 = 7.886751345948129e-1;
      a[0][0] = 1.267949192431123;
      a[1][0] = 1.267949192431123;
      a[2][0] = 2.0;
      a[2][1] = 5.773502691896258e-1;
      a[2][2] = 4.226497308103742e-1;
      b[1][0] = -1.607695154586736;
      b[2][0] = -3.464101615137755;
      b[2][1] = -1.732050807568877;
      scale_all();
      break;
    case ASAM_ROS3PW:
      nStage = 3;
      beta0 = 7.88675134594812865529e-01;
      a[0][0] = 2.0;
      a[1][0] = 6.33974596215561403412e-01;
      a[2][0] = 1.63397459621556140341e+00;
      a[2][1] = 2.94228634059947813384e-01;
      a[2][2] = 1.07179676972449078320e+00;
      b[1][0] = -2.53589838486224561365e+00;
      b[2][0] = -1.62740473580835520728e+00;
      b[2][1] = -2.74519052838329002952e-01;
      scale_all();
      break;
    case ASAM_ROSRK3:
      nStage = 3;
      beta0 = 1.0;
      a[0][0] = 1.0 / (3.0 * beta0);
      a[1][0] = (-1.0 + 12.0 * pow(beta0, 2.0)) / (18.0 * pow(beta0, 2.0) * (-1.0 + 4.0 * beta0));
      a[1][1] = 1.0 / (2.0 * beta0);
      a[2][0] = (1.0 - 3.0 * beta0 * (7.0 + 16.0 * beta0 * (-2.0 + 3.0 * beta0))) / (36.0 * pow(beta0, 3.0) * (-1.0 + 4.0 * beta0));
      a[2][1] = (-1.0 + 12.0 * beta0) / (4.0 * pow(beta0, 2.0));
      a[2][2] = 1.0 / beta0;
      b[1][0] = (1.0 - 12.0 * pow(beta0, 2.0)) / (pow(beta0, 2.0) * (-9.0 + 36.0 * beta0));
      b[2][0] = (-1.0 + 3.0 * beta0 * (7.0 + 16.0 * beta0 * (-2.0 + 3.0 * beta0))) / (36. * pow(beta0, 3.0) * (-1.0 + 4.0 * beta0));
      b[2][1] = (0.250 - 3.0 * beta0) / pow(beta0, 2.0);
      scale_all();
      gm[1] = 1.0 / 3.0;
      gm[2] = 1.0 / 2.0;
      gm[3] = 1.0;
      break;
    case ASAM_ROSTVD:
      nStage = 3;
      beta0 = 0.5;
      a[0][0] = 1.0 / beta0;
      a[1][0] = (1.0 + beta0 * (-9.0 + 16.0 * beta0)) / (4. * pow(beta0, 2.0) * (-1.0 + 4.0 * beta0));
      a[1][1] = 1.0 / (4.0 * beta0);
      a[2][0] = (1.0 + beta0 * (-3.0 + 2.0 * beta0 * (-17.0 + 44.0 * beta0))) / (12. * pow(beta0, 3.0) * (-1.0 + 4.0 * beta0));
      a[2][1] = (1.0 + 6.0 * beta0) / (12.0 * pow(beta0, 2.0));
      a[2][2] = 2.0 / (3. * beta0);
      b[1][0] = pow(beta0, -2.0) - 4.0 / beta0 + 4.0 / (-1.0 + 4.0 * beta0);
      b[2][0] = (-1.0 + beta0 * (5.0 + 8.0 * (2.0 - 7.0 * beta0) * beta0)) / (8.0 * pow(beta0, 3.0) * (-1.0 + 4.0 * beta0));
      b[2][1] = -(1.0 + 4.0 * beta0) / (8. * pow(beta0, 2.0));
      scale_all();
      break;
    case ASAM_ROSRK4:
      nStage = 4;
      beta0 = 1.0 / 4.0;
      a[0][0] = 2.0;
      a[1][0] = 2.0;
      a[1][1] = 2.0;
      a[2][0] = 6.0;
      a[2][1] = 10.0;
      a[2][2] = 4.0;
      a[3][0] = 14.0 / 3.0;
      a[3][1] = 20.0 / 3.0;
      a[3][2] = 4.0 / 3.0;
      a[3][3] = 2.0 / 3.0;
      b[1][0] = -4.0;
      b[2][0] = -6.0;
      b[2][1] = -10.0;
      b[3][0] = -4.0;
      b[3][1] = -12.0;
      scale_all();
      break;
    default:
      return 0;
  }
  *beta0_out = beta0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      alpha[i * 4 + j] = a[i][j];
      beta[i * 4 + j] = b[i][j];
    }
  for (int i = 0; i < 5; ++i) gamma1[i] = gm[i];
  return nStage;
}

}  // namespace

namespace asam {
bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Without a CUDA driver every array is a host array, and the CUDA runtime is
// not touched at all (the host-only file routines run on machines without a
// GPU).
bool device_array(const void* p) {
  static const bool driver = [] {
    void* d = dlopen("libcuda.so.1", RTLD_LAZY | RTLD_LOCAL);
    if (d) dlclose(d);
    return d != nullptr;
  }();
  return p && driver && is_device_ptr(p);
}

}  // namespace asam


namespace asam {

int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return kCudaError;
  }
  return kOk;
}

int read_scalars(asam_ctx* h) {
  CK(cudaMemcpyAsync(h->sc_host, h->sc, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, h->L.stream));
  CK(cudaStreamSynchronize(h->L.stream));
  if (h->sc_host->gs_err) {
    set_last_error("persistent Gauss-Seidel schedule: a dependency wait gave up", __FILE__, __LINE__);
    return kCudaError;
  }
  // a NaN in the residual norms of a running iteration means a NaN in the
  // system (the reference's driver stops on ISNAN(DOT(VecMet,VecMet)),
  // ADVECT/MainProg.f90:975-980); after a breakdown (rho = 0, done = 3) the
  // norms are 0/0 by construction and the breakdown exit is taken instead
  if (std::isnan(h->sc_host->rnorm0) || (h->sc_host->done != 3 && std::isnan(h->sc_host->rnorm))) {
    set_last_error("NaN in the stage system", __FILE__, __LINE__);
    return kNanDetected;
  }
  return kOk;
}

int reduce_to_host(asam_ctx* h, double* out) {
  CK(cudaMemcpyAsync(h->red_host, h->red_out, sizeof(double), cudaMemcpyDeviceToHost, h->L.stream));
  CK(cudaStreamSynchronize(h->L.stream));
  *out = *h->red_host;
  return kOk;
}

// Tiles of the Gauss-Seidel wavefront (32 x 4 x 4 cells of the padded box) and
// component groups of its FP32 variants (two components per CTA).
static int gs_tile_count(const Dims& d) {
  return ((d.NX() + 31) / 32) * ((d.NY() + 3) / 4) * ((d.NZ() + 3) / 4);
}
static int gs_ngroups_host(int ncomp, int group) { return (ncomp + group - 1) / group; }

// Components per CTA of the FP32 Gauss-Seidel (asam_config.gs_group; 0 picks
// the library default).
static int gs_group_of(const asam_config& c) {
  const int g = c.gs_group > 0 ? c.gs_group : 5;
  return g < c.ncomp ? g : c.ncomp;
}

// Ticket table of the persistent schedule: (I, J, K, sweep*ngroups + group)
// ordered by level + 2*sweep, so that every dependency of a ticket has a
// smaller ticket.
int gs_schedule_init(asam_ctx* h, int nsweep) {
  const Dims& d = h->d;
  const int ntx = (d.NX() + 31) / 32, nty = (d.NY() + 3) / 4, ntz = (d.NZ() + 3) / 4;
  const int nlev = ntx + nty + ntz - 2;
  const int ngroups = gs_ngroups_host(h->cfg.ncomp, gs_group_of(h->cfg));
  std::vector<int4> order;
  order.reserve((size_t)ntx * nty * ntz * nsweep * ngroups);
  for (int tau = 0; tau < nlev + 2 * (nsweep - 1); ++tau)
    for (int s = 0; s < nsweep; ++s) {
      const int L = tau - 2 * s;
      if (L < 0 || L >= nlev) continue;
      for (int K = 0; K < ntz; ++K)
        for (int J = 0; J < nty; ++J) {
          const int I = L - J - K;
          if (I < 0 || I >= ntx) continue;
          for (int g = 0; g < ngroups; ++g) order.push_back(make_int4(I, J, K, s * ngroups + g));
        }
    }
  gs_schedule_free(h);
  h->gs_nticket = (int)order.size();
  h->gs_nflags = (size_t)gs_tile_count(d) * ngroups;
  CK(cudaMalloc((void**)&h->gs_order, order.size() * sizeof(int4)));
  CK(cudaMalloc((void**)&h->gs_flags, h->gs_nflags * sizeof(int)));
  CK(cudaMalloc((void**)&h->gs_counter, 2 * sizeof(int)));
  CK(cudaMemcpy(h->gs_order, order.data(), order.size() * sizeof(int4), cudaMemcpyHostToDevice));
  CK(cudaMemsetAsync(h->gs_flags, 0, h->gs_nflags * sizeof(int), h->L.stream));
  CK(cudaMemsetAsync(h->gs_counter, 0, 2 * sizeof(int), h->L.stream));
  return kOk;
}

void gs_schedule_free(asam_ctx* h) {
  graphs_reset(h);
  if (h->gs_order) cudaFree(h->gs_order);
  if (h->gs_flags) cudaFree(h->gs_flags);
  if (h->gs_counter) cudaFree(h->gs_counter);
  h->gs_order = nullptr;
  h->gs_flags = nullptr;
  h->gs_counter = nullptr;
  h->gs_nticket = 0;
}

// PSolve_Vec4CellSp: copy, exchange, 1+IterG Gauss-Seidel sweeps (one
// pipelined wavefront), zero halo, exchange.  The FP32 inner solver of the
// refined mode may use the vertical-column line solve instead of the sweeps.
template <typename T>
void psolve_dev(asam_ctx* h, const T* val, const T* in, T* out, Work<T>& w) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  cudaMemcpyAsync(w.bbuf, in, h->len * sizeof(T), cudaMemcpyDeviceToDevice, L.stream);
  launch_exchange_cell(L, d, nc, w.bbuf);
  const bool inner = sizeof(T) == sizeof(float);  // FP32 inner solver of the refined mode
  const int nsweep = 1 + (inner ? h->cfg.inner_gs_iter : h->cfg.gs_iter);
  if (inner && h->cfg.inner_precond != 0) {  // 1: z lines, 2: x lines, 3: y lines
    const int axis = h->cfg.inner_precond == 1 ? 2 : h->cfg.inner_precond == 2 ? 0 : 1;
    launch_line_psolve(L, d, nc, val, w.bbuf, out, w.tbuf, axis, (const T*)h->xl_w, (const T*)h->xl_r);
  } else if (inner && h->gs_order) {
    const GsTileSched sch{h->gs_order,
                          h->gs_nticket,
                          h->gs_flags,
                          h->gs_counter,
                          &h->sc->gs_err,
                          reinterpret_cast<unsigned*>(h->gs_counter + 1),
                          gs_group_of(h->cfg),
                          h->gs_spin > 0 ? h->gs_spin : kGsSpinLimit};
    launch_gs_persist(L, d, nc, val, w.bbuf, out, w.tbuf, nsweep, sch);
  } else {
    launch_gs_sweeps(L, d, nc, val, w.bbuf, out, w.tbuf, nsweep, gs_group_of(h->cfg));
  }
  launch_zero_halo(L, d, nc, out);
  launch_exchange_cell(L, d, nc, out);
}

// CUDA graphs of the two half-iterations of BiCGStab, per context and
// precision: [0] first half of iteration 1, [1] first half of later
// iterations, [2] second half.  A half runs eagerly the first time (so that
// every one-time setting of its kernels is done outside a capture), is
// captured the second time, and is replayed from then on.  The bodies touch
// only the context's own buffers; the caller's x is updated outside them.
void graphs_reset(asam_ctx* h) {
  ++h->graph_gen;  // graphs recorded elsewhere (an ensemble's) compare it before a replay
  step_graph_free(h);
  for (auto& kg : h->kg) {
    for (int q = 0; q < 3; ++q) {
      if (kg.exec[q]) cudaGraphExecDestroy(kg.exec[q]);
      kg.exec[q] = nullptr;
      kg.warm[q] = false;
      kg.n[q] = 0;
    }
  }
}

template <typename Body>
static int run_half(asam_ctx* h, int prec, int q, Body&& body) {
  KrylovGraphs& kg = h->kg[prec];
  const Launch& L = h->L;
  if (!h->use_graphs || L.stream == nullptr) {  // the legacy default stream cannot be captured
    body();
    return check_launch();
  }
  if (!kg.exec[q]) {
    if (!kg.warm[q]) {
      kg.warm[q] = true;
      body();
      return check_launch();
    }
    const long long t0 = thread_launches();
    CK(cudaStreamBeginCapture(L.stream, cudaStreamCaptureModeThreadLocal));
    body();
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(L.stream, &g);
    const long long nl = thread_launches() - t0;
    count_launches(-nl);  // captured, not run
    if (e == cudaSuccess) e = cudaGraphInstantiate(&kg.exec[q], g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      kg.exec[q] = nullptr;
      set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
      return kCudaError;
    }
    kg.n[q] = nl;
  }
  CK(cudaGraphLaunch(kg.exec[q], L.stream));
  count_launches(kg.n[q]);
  return kOk;
}

// x-line factors of the current stage matrix for the FP32 inner line solve
// (outside any captured half-iteration: they change with the matrix only)
void prepare_inner(asam_ctx* h) {
  if (h->cfg.inner_precond == 2 && !h->xline_ready) {
    launch_xline_factor(h->L, h->d, h->val32, h->xl_w, h->xl_r);
    h->xline_ready = true;
  }
}

// BiCGStabMet_Vec4CellSp (MODULE/SpMatrix4CellPar_Mod.f90:245-348) on the device.
template <typename T>
int bicgstab_dev(asam_ctx* h, const T* val, T* x, const T* b, int* maxiter, double* tol, Work<T>& w,
                 bool x_is_zero) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  const size_t len = h->len;
  memset(h->sc_host, 0, sizeof(KrylovScalars));
  h->sc_host->tol = *tol;
  CK(cudaMemcpyAsync(h->sc, h->sc_host, sizeof(KrylovScalars), cudaMemcpyHostToDevice, L.stream));
  if (x_is_zero) {  // r = b - A*0 = b exactly
    CK(cudaMemcpyAsync(w.r, b, len * sizeof(T), cudaMemcpyDeviceToDevice, L.stream));
  } else {
    launch_matvec(L, d, nc, val, x, w.r, 0);
    launch_xpay_host(L, len, b, (T)-1, w.r);
  }
  CK(cudaMemcpyAsync(w.rt, w.r, len * sizeof(T), cudaMemcpyDeviceToDevice, L.stream));
  launch_dot(L, d, nc, w.r, w.r, h->partial, h->sc, OP_RNORM0, nullptr);
  if (sizeof(T) == sizeof(float)) prepare_inner(h);
  const int prec = sizeof(T) == sizeof(float) ? 1 : 0;
  auto half1 = [&](bool first) {
    launch_dot(L, d, nc, w.rt, w.r, h->partial, h->sc, OP_RHO, nullptr);
    if (first) {
      cudaMemcpyAsync(w.p, w.r, len * sizeof(T), cudaMemcpyDeviceToDevice, L.stream);
    } else {
      launch_beta(L, h->sc);
      launch_pupdate(L, len, h->sc, w.r, w.v, w.p);
    }
    psolve_dev<T>(h, val, w.p, w.ph, w);
    launch_matvec_dot(L, d, nc, val, w.ph, w.v, w.rt, h->partial, h->sc, OP_ALPHA);  // v = A ph, (r~, v)
    launch_axpy_dot(L, d, nc, h->sc, SEL_ALPHA, -1.0, w.v, w.r, h->partial, OP_RNORM_HALF);  // r -= alpha v, (r, r)
  };
  // second half without the update of x (launched after it: x is the
  // caller's array, and nothing in the half reads alpha/omega after it)
  auto half2 = [&]() {
    psolve_dev<T>(h, val, w.r, w.rh, w);
    // t = A rh with (t, r) and (t, t); r -= omega t with (r, r)
    launch_matvec_dot2(L, d, nc, val, w.rh, w.t, w.r, h->partial, h->sc, OP_STORE_A, OP_OMEGA);
    launch_axpy_dot(L, d, nc, h->sc, SEL_OMEGA, -1.0, w.t, w.r, h->partial, OP_RNORM_FULL);
  };
  const int MaxIter = *maxiter;
  for (int it = 1; it <= MaxIter; ++it) {
    int rc = run_half(h, prec, it == 1 ? 0 : 1, [&] { half1(it == 1); });
    if (rc) return rc;
    rc = read_scalars(h);
    if (rc) return rc;
    if (h->sc_host->done == 3) {
      *maxiter = it;
      *tol = 0.0;
      return h->sc_host->rnorm0 > 0.0 ? kBreakdown : kOk;
    }
    if (h->sc_host->done == 1) {
      launch_xupdate(L, len, h->sc, 0, w.ph, (const T*)nullptr, x);
      *maxiter = -it;
      *tol = h->sc_host->rnorm;
      return check_launch();
    }
    if ((rc = run_half(h, prec, 2, half2))) return rc;
    launch_xupdate(L, len, h->sc, 1, w.ph, w.rh, x);
    rc = check_launch();
    if (rc) return rc;
    rc = read_scalars(h);
    if (rc) return rc;
    if (h->sc_host->done == 2) {
      *maxiter = it;
      *tol = h->sc_host->rnorm;
      return kOk;
    }
    if (it == MaxIter) {
      *maxiter = 2 * it;
      *tol = h->sc_host->rnorm;
      return kNotConverged;
    }
  }
  *tol = 0.0;
  return kOk;
}

// FP32-refined solve: outer FP64 iterative refinement, FP32 inner BiCGStab
// with the FP32 Gauss-Seidel preconditioner, FP64 residual recomputation and
// the reference's stopping test ||r|| <= Tol*||r0|| on the FP64 residual.
int bicgstab_refined(asam_ctx* h, double* x, const double* b, int* maxiter, double* tol, bool x_is_zero) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  const size_t len = h->len;
  double* r = h->w64.r;
  if (x_is_zero) {  // r = b - A*0 = b
    CK(cudaMemcpyAsync(r, b, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  } else {
    launch_matvec(L, d, nc, h->val, x, r, 0);
    launch_xpay_host(L, len, b, -1.0, r);
  }
  launch_dot(L, d, nc, r, r, h->partial, h->sc, OP_STORE_A, h->red_out);
  double rr0 = 0;
  int rc = reduce_to_host(h, &rr0);
  if (rc) return rc;
  if (std::isnan(rr0)) {
    set_last_error("NaN in the stage system", __FILE__, __LINE__);
    return kNanDetected;
  }
  const double rnorm0 = sqrt(rr0);
  const double target = *tol * rnorm0;
  if (rnorm0 == 0.0) {
    *maxiter = 1;
    *tol = 0.0;
    return kOk;
  }
  double rnorm = rnorm0;
  int total_inner = 0;
  const int max_outer = 8;
  for (int outer = 0; outer < max_outer; ++outer) {
    // the inner system is A d = r/|r| (unit scale in FP32); x += |r| d
    launch_convert_f64_to_f32_scaled(L, len, r, 1.0 / rnorm, h->b32);
    CK(cudaMemsetAsync(h->x32, 0, len * sizeof(float), L.stream));
    int it = h->cfg.bicgstab_maxiter;
    double tin = 0.5 * target / rnorm;
    if (tin < 1e-6) tin = 1e-6;
    if (tin > 1e-2) tin = 1e-2;
    rc = bicgstab_dev<float>(h, h->val32, h->x32, h->b32, &it, &tin, h->w32, true);
    // an inner breakdown or iteration limit still leaves a usable correction:
    // the outer FP64 residual decides
    if (rc != kOk && rc != kNotConverged && rc != kBreakdown) return rc;
    total_inner += it < 0 ? -it : (it > h->cfg.bicgstab_maxiter ? it / 2 : it);
    launch_add_f32_to_f64(L, len, h->x32, rnorm, x);                             // x += |r| * correction
    asam_fma::launch_resid_dot(L, d, nc, h->val, x, b, r, h->partial, h->sc, OP_STORE_A, h->red_out);  // r, r.r
    double rr = 0;
    rc = reduce_to_host(h, &rr);
    if (rc) return rc;
    if (std::isnan(rr)) {
      set_last_error("NaN in the stage system", __FILE__, __LINE__);
      return kNanDetected;
    }
    rnorm = sqrt(rr);
    if (rnorm <= target) {
      *maxiter = total_inner;
      *tol = rnorm;
      return kOk;
    }
  }
  *maxiter = 2 * total_inner;
  *tol = rnorm;
  return kNotConverged;
}

int fcn_dev(asam_ctx* h, const double* c, double* f) {
  const Launch& L = h->L;
  DiffSrc<double> tmp;
  const DiffSrc<double>* df = h->diff_src(tmp);
  if (h->cfg.precision == ASAM_PREC_FP32_REFINED) {  // contracted FP64 (the refined mode's 1e-10 contract)
    asam_fma::launch_fcn(L, h->d, h->geom(), h->cfg.ncomp, h->cfg.rho_pos, c, h->coef_x, h->coef_y, h->coef_z,
                         h->mask_x, h->mask_y, h->mask_z, h->phi, h->gx, h->gy, h->gz, h->rvol, f, df);
    return check_launch();
  }
  launch_phi(L, h->d, h->cfg.ncomp, h->cfg.rho_pos, c, h->phi);
  launch_face_flux(L, h->d, h->geom(), h->cfg.ncomp, h->coef_x, h->coef_y, h->coef_z, h->mask_x, h->mask_y,
                   h->mask_z, h->phi, h->gx, h->gy, h->gz);
  launch_flux_gather(L, h->d, h->geom(), h->cfg.ncomp, h->gx, h->gy, h->gz, h->rvol, f, df,
                     WallIn<double>{c, c + (size_t)h->cfg.rho_pos * h->npad});
  return check_launch();
}

int jac_dev(asam_ctx* h, const double* c, double dt) {
  const double* rho = c + (size_t)h->cfg.rho_pos * h->npad;
  const bool jd = h->dkx && h->jac_diff;
  const double *kx = jd ? h->dkx : nullptr, *ky = jd ? h->dky : nullptr, *kz = jd ? h->dkz : nullptr;
  if (h->cfg.precision == ASAM_PREC_FP32_REFINED)
    asam_fma::launch_jac(h->L, h->d, h->geom(), rho, h->rvol, h->beta0 * dt, h->val, kx, ky, kz);
  else
    launch_jac(h->L, h->d, h->geom(), rho, h->rvol, h->beta0 * dt, h->val, kx, ky, kz);
  if (h->cfg.precision == ASAM_PREC_FP32_REFINED) launch_convert_f64_to_f32(h->L, 8 * h->npad, h->val, h->val32);
  h->jac_ready = true;
  h->xline_ready = false;
  return check_launch();
}

int solve_dev(asam_ctx* h, double* x, const double* b, int* maxiter, double* tol, bool x_is_zero) {
  if (h->cfg.precision == ASAM_PREC_FP32_REFINED) return bicgstab_refined(h, x, b, maxiter, tol, x_is_zero);
  return bicgstab_dev<double>(h, h->val, x, b, maxiter, tol, h->w64, x_is_zero);
}

// Ros3MetC + StageRos, transport part (ADVECT/Int_Mod.f90:263-374, 1059-1122).
int ros_step_dev(asam_ctx* h, double* c, double dt, int* iters, double* resid) {
  if (h->step_graphs && h->L.stream != nullptr)
    return ros_step_graph(h, c, dt, iters, resid);  // the whole step as one device-driven graph
  const Launch& L = h->L;
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  const size_t len = h->len;
  int status = kOk;
  CK(cudaMemcpyAsync(h->cold, c, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  for (int is = 0; is < h->nstage; ++is) {
    launch_exchange_cell(L, d, nc, c);
    launch_bound_cond(L, d, nc, 0, h->bc, c);
    if (is == 0) {
      int rc = jac_dev(h, c, dt);
      if (rc) return rc;
    }
    int rc = fcn_dev(h, c, h->rhs);
    if (rc) return rc;
    launch_scale_host(L, len, dt, h->rhs);
    for (int js = 0; js < is; ++js) launch_axpy_host(L, len, h->beta[is * 4 + js], h->incr + (size_t)js * len, h->rhs);
    double* x = h->incr + (size_t)is * len;
    CK(cudaMemsetAsync(x, 0, len * sizeof(double), L.stream));
    int it = h->cfg.bicgstab_maxiter;
    double tol = h->cfg.bicgstab_tol;
    rc = solve_dev(h, x, h->rhs, &it, &tol, true);
    if (rc != kOk && rc != kNotConverged && rc != kBreakdown) return rc;
    if (rc != kOk && status == kOk) status = rc;
    if (iters) iters[is] = it;
    if (resid) resid[is] = tol;
    launch_exchange_cell(L, d, nc, x);
    launch_exchange_cell(L, d, nc, x);
    CK(cudaMemcpyAsync(c, h->cold, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    for (int js = 0; js <= is; ++js) launch_axpy_host(L, len, h->alpha[is * 4 + js], h->incr + (size_t)js * len, c);
  }
  int rc = check_launch();
  return rc ? rc : status;
}

// Staging of a caller pointer: device pointers are used in place, host
// pointers are copied through the context's staging buffers.
int stage_in(asam_ctx* h, const double* p, size_t n, double* buf, const double** dev) {
  if (is_device_ptr(p)) {
    *dev = p;
    return kOk;
  }
  CK(cudaMemcpyAsync(buf, p, n * sizeof(double), cudaMemcpyHostToDevice, h->L.stream));
  *dev = buf;
  return kOk;
}
int stage_out_begin(asam_ctx* h, double* p, size_t n, double* buf, double** dev, bool copy_in) {
  if (is_device_ptr(p)) {
    *dev = p;
    return kOk;
  }
  if (copy_in) CK(cudaMemcpyAsync(buf, p, n * sizeof(double), cudaMemcpyHostToDevice, h->L.stream));
  *dev = buf;
  return kOk;
}
int stage_out_end(asam_ctx* h, double* p, size_t n, double* dev) {
  if (dev != p) {
    CK(cudaMemcpyAsync(p, dev, n * sizeof(double), cudaMemcpyDeviceToHost, h->L.stream));
    CK(cudaStreamSynchronize(h->L.stream));
  }
  return kOk;
}

template void psolve_dev<double>(asam_ctx*, const double*, const double*, double*, Work<double>&);
template void psolve_dev<float>(asam_ctx*, const float*, const float*, float*, Work<float>&);
template int bicgstab_dev<double>(asam_ctx*, const double*, double*, const double*, int*, double*, Work<double>&,
                                  bool);
template int bicgstab_dev<float>(asam_ctx*, const float*, float*, const float*, int*, double*, Work<float>&, bool);

}  // namespace asam

namespace {
int validate(const asam_config* c) {
  if (!c) return kBadArg;
  if (c->nx < 1 || c->ny < 1 || c->nz < 1) return kBadArg;
  if (c->ncomp < 1 || c->ncomp > kMaxComp) return kBadArg;
  if (c->rho_pos < 0 || c->rho_pos >= c->ncomp) return kBadArg;
  if (c->bicgstab_maxiter < 1 || c->gs_iter < 0) return kBadArg;
  if (c->precision != ASAM_PREC_FP64 && c->precision != ASAM_PREC_FP32_REFINED) return kBadArg;
  if (c->inner_precond < 0 || c->inner_precond > 3) return kBadArg;
  if (c->inner_gs_iter < 0) return kBadArg;
  if (c->gs_schedule != 0 && c->gs_schedule != 1) return kBadArg;
  if (c->gs_group < 0 || c->gs_group > 16) return kBadArg;
  return kOk;
}

// Device workspace of the host-array column entries (asam_tri_solve,
// asam_tri_matvec), one per device, grown to the largest call and kept until
// the process exits, so that a call does not pay cudaMalloc/cudaFree (each
// synchronises the device).  The entries are synchronous and serialised by
// g_col_mu, so one workspace per device suffices.  A workspace whose memory
// no longer belongs to the device (the device was reset) is replaced.
std::mutex g_col_mu;
std::vector<std::pair<double*, size_t>> g_col_ws;  // per device ordinal

int col_workspace(size_t n, double** out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if ((int)g_col_ws.size() <= dev) g_col_ws.resize(dev + 1, {nullptr, 0});
  auto& ws = g_col_ws[dev];
  if (ws.first) {
    cudaPointerAttributes a;
    const bool valid = cudaPointerGetAttributes(&a, ws.first) == cudaSuccess && a.type == cudaMemoryTypeDevice &&
                       a.device == dev;
    if (!valid) {
      cudaGetLastError();
      ws = {nullptr, 0};
    }
  }
  if (ws.second < n) {
    if (ws.first) cudaFree(ws.first);
    ws = {nullptr, 0};
    CK(cudaMalloc((void**)&ws.first, n * sizeof(double)));
    ws.second = n;
  }
  *out = ws.first;
  return kOk;
}

}  // namespace

// Scalar FP64 FMA throughput probe: 8 independent chains per thread.
__global__ void k_probe_fp64(int iters, double seed, double* out) {
  double a[8];
  for (int q = 0; q < 8; ++q) a[q] = seed + q + threadIdx.x;
  const double m = 0.999999, c = 1e-7;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int q = 0; q < 8; ++q) a[q] = __fma_rn(a[q], m, c);
  double s = 0;
  for (int q = 0; q < 8; ++q) s += a[q];
  if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

// Cost of a dependent FP64 chain: the first `lanes` threads of the first
// `warps` warps of one block each run iters dependent FMAs; the slowest
// warp's clock64 cycles per FMA go to cyc[0].
__global__ void k_probe_fp64_chain(int iters, int lanes, int warps, double* out, long long* cyc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp >= warps || lane >= lanes) return;
  double x = 1.0 + threadIdx.x * 1e-3;
  const double m = 0.999999, c = 1e-7;
  const long long t0 = clock64();
  for (int i = 0; i < iters; ++i) x = __fma_rn(x, m, c);
  const long long t1 = clock64();
  if (x == 12345.0) out[0] = x;  // keeps the chain alive
  if (lane == 0) atomicMax((unsigned long long*)cyc, (unsigned long long)(t1 - t0));
}

// Check of the FMA-corrected quotient (kernels.cuh div_rn) against the IEEE
// quotient on pseudo-random operands spanning many binades.
__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}
__device__ __forceinline__ double rand_double(unsigned long long h, int span) {
  // mantissa from the hash, exponent in [-span, span], random sign
  const double m = 1.0 + (double)(h >> 12) * 0x1.0p-52;
  const int e = (int)((h >> 3) % (unsigned long long)(2 * span + 1)) - span;
  return ((h & 1) ? -1.0 : 1.0) * ldexp(m, e);
}
__global__ void k_probe_div(unsigned long long n, unsigned long long seed, int span, unsigned long long* bad) {
  unsigned long long cnt = 0;
  for (unsigned long long q = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; q < n;
       q += (unsigned long long)gridDim.x * blockDim.x) {
    const double x = rand_double(splitmix(seed ^ (2 * q)), span);
    const double dd = rand_double(splitmix(seed ^ (2 * q + 1)), span);
    const double r = 1.0 / dd;
    const double q0 = __dmul_rn(x, r);
    const double e = __fma_rn(-q0, dd, x);
    const double qq = __fma_rn(e, r, q0);
    if (qq != x / dd) ++cnt;
  }
  if (cnt) atomicAdd(bad, cnt);
}

// ---------------------------------------------------------------------------
extern "C" {

int asam_probe_div(long long n, long long seed, int span, long long* mismatches) {
  if (n < 1 || !mismatches || span < 0 || span > 500) return kBadArg;
  unsigned long long* d;
  CK(cudaMalloc((void**)&d, sizeof(unsigned long long)));
  CK(cudaMemset(d, 0, sizeof(unsigned long long)));
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  k_probe_div<<<sms * 8, 256>>>((unsigned long long)n, (unsigned long long)seed, span, d);
  unsigned long long h = 0;
  cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return kCudaError;
  }
  *mismatches = (long long)h;
  return check_launch();
}

int asam_probe_fp64_chain(int warps, int lanes, int iters, double* cycles_per_op) {
  if (warps < 1 || warps > 32 || lanes < 1 || lanes > 32 || iters < 1 || !cycles_per_op) return kBadArg;
  double* out;
  long long* cyc;
  CK(cudaMalloc((void**)&out, sizeof(double)));
  CK(cudaMalloc((void**)&cyc, sizeof(long long)));
  long long h = 0;
  for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
    CK(cudaMemset(cyc, 0, sizeof(long long)));
    k_probe_fp64_chain<<<1, 32 * warps>>>(iters, lanes, warps, out, cyc);
    CK(cudaMemcpy(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost));
  }
  cudaFree(out);
  cudaFree(cyc);
  *cycles_per_op = (double)h / iters;
  return check_launch();
}

int asam_probe_fp64_fma(int iters, double* gflops) {
  if (iters < 1 || !gflops) return kBadArg;
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* out;
  CK(cudaMalloc((void**)&out, sizeof(double)));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int blocks = sms * 8, threads = 256;
  k_probe_fp64<<<blocks, threads>>>(iters / 10 + 1, 1.0, out);  // warm-up
  CK(cudaEventRecord(e0));
  k_probe_fp64<<<blocks, threads>>>(iters, 1.0, out);
  CK(cudaEventRecord(e1));
  CK(cudaEventSynchronize(e1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  *gflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e9;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return check_launch();
}

const char* asam_last_error(void) { return g_last_error.c_str(); }

long long asam_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

long long asam_npad(const asam_config* cfg) {
  if (!cfg) return -1;
  return (long long)(cfg->nx + 2) * (cfg->ny + 2) * (cfg->nz + 2);
}

int asam_ros_coeffs(int method, double* beta0, double* alpha, double* beta, double* gamma1) {
  return ros_coeffs(method, beta0, alpha, beta, gamma1);
}

int asam_destroy(asam_ctx* h) {
  if (!h) return kOk;
  double* dptrs[] = {h->volc, h->fu,     h->fv,     h->fw,     h->uf,     h->vf,      h->wf,      h->c,
                     h->cold, h->rhs,    h->incr,   h->phi,    h->gx,     h->gy,      h->gz,      h->val,
                     h->partial, h->red_out, h->stage_a, h->stage_b, h->coef_x, h->coef_y, h->coef_z,
                     h->rvol};
  unsigned char* bptrs[] = {h->mask_x, h->mask_y, h->mask_z};
  for (unsigned char* p : bptrs)
    if (p) cudaFree(p);
  for (double* p : dptrs)
    if (p) cudaFree(p);
  if (h->val32) cudaFree(h->val32);
  for (double* p : {h->bc_mean, h->bc_fval, h->bc_amb})
    if (p) cudaFree(p);
  if (h->xl_w) cudaFree(h->xl_w);
  if (h->xl_r) cudaFree(h->xl_r);
  if (h->x32) cudaFree(h->x32);
  if (h->b32) cudaFree(h->b32);
  if (h->sc) cudaFree(h->sc);
  if (h->sc_host) cudaFreeHost(h->sc_host);
  if (h->red_host) cudaFreeHost(h->red_host);
  free_work(h->w64);
  free_work(h->w32);
  gs_schedule_free(h);  // and the graphs
  proj_free(h);
  dyn_free(h);
  double* dk[] = {h->dkx, h->dky, h->dkz};
  for (double* q : dk)
    if (q) cudaFree(q);
  for (auto st : h->cap_stream)
    if (st) cudaStreamDestroy(st);
  if (h->stage_sc) cudaFree(h->stage_sc);
  if (h->ref_sc) cudaFree(h->ref_sc);
  if (h->stage_sc_host) cudaFreeHost(h->stage_sc_host);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return kOk;
}

int asam_create(const asam_config* cfg, const double* volc, const double* fu, const double* fv, const double* fw,
                asam_ctx** out) {
  if (!out || validate(cfg) != kOk || !volc || !fu || !fv || !fw) {
    set_last_error("invalid configuration or null geometry", __FILE__, __LINE__);
    return kBadArg;
  }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_last_error("no CUDA device", __FILE__, __LINE__);
    return kNoDevice;
  }
  asam_ctx* h = new asam_ctx();
  h->cfg = *cfg;
  h->d = Dims{cfg->nx, cfg->ny, cfg->nz, cfg->periodic_x ? 1 : 0, cfg->periodic_y ? 1 : 0, cfg->periodic_z ? 1 : 0};
  h->npad = h->d.npad();
  h->len = h->npad * (size_t)cfg->ncomp;
  h->nstage = ros_coeffs(cfg->method, &h->beta0, h->alpha, h->beta, h->gamma1);
  for (int ic = 0; ic < kMaxComp; ++ic)
    for (int sd = 0; sd < 6; ++sd) h->bc.k[ic][sd] = kBcZeroGrad;
  if (h->nstage <= 0) {
    delete h;
    set_last_error("unknown Rosenbrock method", __FILE__, __LINE__);
    return kBadArg;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&h->L.sm_count, cudaDevAttrMultiProcessorCount, dev);
  h->device = dev;
  auto fail = [&](cudaError_t e) {
    set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    asam_destroy(h);
    return (int)kCudaError;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  h->L.stream = h->own_stream;
  const Dims& d = h->d;
  struct A {
    double** p;
    size_t n;
  } allocs[] = {{&h->volc, h->npad},      {&h->fu, d.n_fu()},        {&h->fv, d.n_fv()},        {&h->fw, d.n_fw()},
                {&h->uf, d.n_uf()},       {&h->vf, d.n_vf()},        {&h->wf, d.n_wf()},        {&h->c, h->len},
                {&h->cold, h->len},       {&h->rhs, h->len},         {&h->incr, h->len * h->nstage},
                {&h->phi, h->len},        {&h->gx, d.n_uf() * cfg->ncomp}, {&h->gy, d.n_vf() * cfg->ncomp},
                {&h->gz, d.n_wf() * cfg->ncomp}, {&h->val, 8 * h->npad}, {&h->partial, 2 * (size_t)kFusedGridMax},
                {&h->red_out, 1},         {&h->stage_a, h->len},     {&h->stage_b, h->len},
                {&h->coef_x, 4 * d.n_uf()}, {&h->coef_y, 4 * d.n_vf()}, {&h->coef_z, 4 * d.n_wf()},
                {&h->rvol, h->npad}};
  for (auto& a : allocs)
    if ((e = cudaMalloc((void**)a.p, a.n * sizeof(double))) != cudaSuccess) return fail(e);
  h->bc.uf = h->uf;  // InFlowOutFlow tests the sign of the context's face velocities
  h->bc.vf = h->vf;
  h->bc.rho = cfg->rho_pos;
  if ((e = cudaMalloc((void**)&h->mask_x, d.n_uf())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc((void**)&h->mask_y, d.n_vf())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc((void**)&h->mask_z, d.n_wf())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc((void**)&h->sc, sizeof(KrylovScalars))) != cudaSuccess) return fail(e);
  if ((e = cudaMallocHost((void**)&h->sc_host, sizeof(KrylovScalars))) != cudaSuccess) return fail(e);
  if ((e = cudaMallocHost((void**)&h->red_host, sizeof(double))) != cudaSuccess) return fail(e);
  if ((e = alloc_work(h->w64, h->len)) != cudaSuccess) return fail(e);
  if (cfg->precision == ASAM_PREC_FP32_REFINED) {
    if ((e = alloc_work(h->w32, h->len)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&h->val32, 8 * h->npad * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&h->x32, h->len * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&h->b32, h->len * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&h->xl_w, h->npad * sizeof(float))) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&h->xl_r, h->npad * sizeof(float))) != cudaSuccess) return fail(e);
    if (cfg->inner_precond == 0 && cfg->gs_schedule == 0 && gs_schedule_init(h, 1 + cfg->inner_gs_iter) != kOk) {
      asam_destroy(h);
      return (int)kCudaError;
    }
  }
  struct C {
    double* dst;
    const double* src;
    size_t n;
  } copies[] = {{h->volc, volc, h->npad}, {h->fu, fu, d.n_fu()}, {h->fv, fv, d.n_fv()}, {h->fw, fw, d.n_fw()}};
  for (auto& c : copies)
    if ((e = cudaMemcpy(c.dst, c.src, c.n * sizeof(double), cudaMemcpyDefault)) != cudaSuccess) return fail(e);
  double* zero[] = {h->uf, h->vf, h->wf};
  size_t nz[] = {d.n_uf(), d.n_vf(), d.n_wf()};
  for (int q = 0; q < 3; ++q)
    if ((e = cudaMemsetAsync(zero[q], 0, nz[q] * sizeof(double), h->L.stream)) != cudaSuccess) return fail(e);
  if ((e = cudaMemsetAsync(h->c, 0, h->len * sizeof(double), h->L.stream)) != cudaSuccess) return fail(e);
  launch_recip_eps(h->L, h->npad, h->volc, h->rvol);
  launch_face_coef(h->L, d, h->geom(), h->coef_x, h->coef_y, h->coef_z, h->mask_x, h->mask_y, h->mask_z);
  if ((e = cudaStreamSynchronize(h->L.stream)) != cudaSuccess) return fail(e);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  *out = h;
  return kOk;
}

int asam_set_graphs(asam_ctx* h, int on) {
  if (!h || on < 0 || on > 2) return kBadArg;
  graphs_reset(h);
  h->use_graphs = on != 0;
  h->step_graphs = on == 2;
  return kOk;
}

int asam_set_wait_limit(asam_ctx* h, int polls) {
  if (!h || polls < 0) return kBadArg;
  graphs_reset(h);  // captured launches carry the limit
  h->gs_spin = polls;
  return kOk;
}

int asam_set_stream(asam_ctx* h, void* stream) {
  if (!h) return kBadArg;
  h->L.stream = (cudaStream_t)stream;  // NULL: the legacy default stream
  return kOk;
}

int asam_state_device_ptr(asam_ctx* h, double** dptr) {
  if (!h || !dptr) return kBadArg;
  *dptr = h->c;
  return kOk;
}

int asam_synchronize(asam_ctx* h) {
  if (!h) return kBadArg;
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

int asam_set_velocity(asam_ctx* h, const double* uf, const double* vf, const double* wf) {
  if (!h || !uf || !vf || !wf) return kBadArg;
  const Dims& d = h->d;
  CK(cudaMemcpyAsync(h->uf, uf, d.n_uf() * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaMemcpyAsync(h->vf, vf, d.n_vf() * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaMemcpyAsync(h->wf, wf, d.n_wf() * sizeof(double), cudaMemcpyDefault, h->L.stream));
  launch_face_coef(h->L, d, h->geom(), h->coef_x, h->coef_y, h->coef_z, h->mask_x, h->mask_y, h->mask_z);
  CK(cudaStreamSynchronize(h->L.stream));
  return check_launch();
}

int asam_exchange_cell(asam_ctx* h, int ncomp, double* c) {
  if (!h || !c || ncomp < 1 || ncomp > h->cfg.ncomp) return kBadArg;
  double* dc;
  size_t n = h->npad * (size_t)ncomp;
  int rc = stage_out_begin(h, c, n, h->stage_a, &dc, true);
  if (rc) return rc;
  launch_exchange_cell(h->L, h->d, ncomp, dc);
  rc = check_launch();
  if (rc) return rc;
  return stage_out_end(h, c, n, dc);
}

int asam_set_boundary(asam_ctx* h, const int* kinds) {
  if (!h || !kinds) return kBadArg;
  bool open = false;
  for (int q = 0; q < 6 * h->cfg.ncomp; ++q) {
    if (kinds[q] < ASAM_BC_NONE || kinds[q] > ASAM_BC_EXTRAPOLATION) return kBadArg;
    const char* missing = kinds[q] == ASAM_BC_MEAN_VALUE && !h->bc_mean ? "MeanValue needs its profile"
                          : kinds[q] == ASAM_BC_FUNCTION && !h->bc_fval ? "Function needs its halo values"
                          : kinds[q] == ASAM_BC_INFLOW_OUTFLOW && !h->bc_amb ? "InFlowOutFlow needs the ambient state"
                                                                              : nullptr;
    if (missing) {
      set_last_error((std::string("asam_set_boundary: ") + missing + " (asam_set_boundary_data first)").c_str(),
                     __FILE__, __LINE__);
      return kBadArg;
    }
    open = open || kinds[q] > ASAM_BC_ZERO_VALUE;
  }
  if (open && h->dyn) {
    set_last_error("asam_set_boundary: the open-boundary kinds are built for the transport stage only", __FILE__,
                   __LINE__);
    return kBadArg;
  }
  for (int ic = 0; ic < h->cfg.ncomp; ++ic)
    for (int sd = 0; sd < 6; ++sd) h->bc.k[ic][sd] = (signed char)kinds[6 * ic + sd];
  graphs_reset(h);  // a captured step holds the old rule
  return kOk;
}

int asam_set_boundary_data(asam_ctx* h, const double* mean_profile, const double* function_values,
                           const double* ambient) {
  if (!h) return kBadArg;
  const size_t sizes[3] = {(size_t)h->cfg.ncomp * h->cfg.nz, h->len, h->len};
  const double* src[3] = {mean_profile, function_values, ambient};
  double** dst[3] = {&h->bc_mean, &h->bc_fval, &h->bc_amb};
  const signed char kind[3] = {kBcMeanValue, kBcFunction, kBcInflowOutflow};
  for (int q = 0; q < 3; ++q) {
    if (src[q]) continue;
    for (int ic = 0; ic < h->cfg.ncomp; ++ic)
      for (int sd = 0; sd < 6; ++sd)
        if (h->bc.k[ic][sd] == kind[q]) {
          set_last_error("asam_set_boundary_data: a kind in use needs this array", __FILE__, __LINE__);
          return kBadArg;
        }
  }
  for (int q = 0; q < 3; ++q) {
    if (!src[q]) {
      if (*dst[q]) cudaFree(*dst[q]);
      *dst[q] = nullptr;
      continue;
    }
    if (!*dst[q]) CK(cudaMalloc((void**)dst[q], sizes[q] * sizeof(double)));
    CK(cudaMemcpyAsync(*dst[q], src[q], sizes[q] * sizeof(double), cudaMemcpyDefault, h->L.stream));
  }
  CK(cudaStreamSynchronize(h->L.stream));
  h->bc.mean = h->bc_mean;
  h->bc.fval = h->bc_fval;
  h->bc.amb = h->bc_amb;
  graphs_reset(h);  // a captured step holds the old pointers
  return kOk;
}

int asam_set_diffusion(asam_ctx* h, const double* dh, const double* dv, int jac) {
  if (!h) return kBadArg;
  const Dims& d = h->d;
  if (!dh) {  // off
    double* p[] = {h->dkx, h->dky, h->dkz};
    for (double* q : p)
      if (q) cudaFree(q);
    h->dkx = h->dky = h->dkz = nullptr;
    h->jac_diff = false;
    h->jac_ready = false;
    graphs_reset(h);
    return kOk;
  }
  if (!dv) dv = dh;
  if (!h->dkx) {
    CK(cudaMalloc((void**)&h->dkx, d.n_uf() * sizeof(double)));
    CK(cudaMalloc((void**)&h->dky, d.n_vf() * sizeof(double)));
    CK(cudaMalloc((void**)&h->dkz, d.n_wf() * sizeof(double)));
  }
  const double *ddh, *ddv;
  int rc;
  if ((rc = stage_in(h, dh, h->npad, h->stage_a, &ddh))) return rc;
  if ((rc = stage_in(h, dv, h->npad, h->stage_b, &ddv))) return rc;
  launch_diff_coef(h->L, d, h->geom(), ddh, ddv, h->dkx, h->dky, h->dkz);
  CK(cudaStreamSynchronize(h->L.stream));
  h->jac_diff = jac != 0;
  h->jac_ready = false;
  graphs_reset(h);  // a captured step holds the old flux
  return check_launch();
}

int asam_boundary_condition(asam_ctx* h, double* c) {
  if (!h || !c) return kBadArg;
  double* dc;
  int rc = stage_out_begin(h, c, h->len, h->stage_a, &dc, true);
  if (rc) return rc;
  launch_bound_cond(h->L, h->d, h->cfg.ncomp, 0, h->bc, dc);
  rc = check_launch();
  if (rc) return rc;
  return stage_out_end(h, c, h->len, dc);
}

int asam_fcn(asam_ctx* h, const double* c, double* f) {
  if (!h || !c || !f) return kBadArg;
  const double* dc;
  double* df;
  int rc = stage_in(h, c, h->len, h->stage_a, &dc);
  if (rc) return rc;
  rc = stage_out_begin(h, f, h->len, h->stage_b, &df, false);
  if (rc) return rc;
  rc = fcn_dev(h, dc, df);
  if (rc) return rc;
  return stage_out_end(h, f, h->len, df);
}

int asam_div(asam_ctx* h, double* rhs) {
  if (!h || !rhs) return kBadArg;
  double* dr;
  int rc = stage_out_begin(h, rhs, h->npad, h->stage_a, &dr, true);
  if (rc) return rc;
  launch_div(h->L, h->d, h->geom(), dr);
  rc = check_launch();
  if (rc) return rc;
  return stage_out_end(h, rhs, h->npad, dr);
}

int asam_jac(asam_ctx* h, const double* c, double dt) {
  if (!h || !c) return kBadArg;
  const double* dc;
  int rc = stage_in(h, c, h->len, h->stage_a, &dc);
  if (rc) return rc;
  rc = jac_dev(h, dc, dt);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

int asam_get_jac(asam_ctx* h, double* val) {
  if (!h || !val) return kBadArg;
  CK(cudaMemcpyAsync(val, h->val, 7 * h->npad * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

int asam_set_jac(asam_ctx* h, const double* val) {
  if (!h || !val) return kBadArg;
  CK(cudaMemcpyAsync(h->val, val, 7 * h->npad * sizeof(double), cudaMemcpyDefault, h->L.stream));
  launch_recip_diag(h->L, h->npad, h->val);
  if (h->cfg.precision == ASAM_PREC_FP32_REFINED) launch_convert_f64_to_f32(h->L, 8 * h->npad, h->val, h->val32);
  CK(cudaStreamSynchronize(h->L.stream));
  h->jac_ready = true;
  h->xline_ready = false;
  return check_launch();
}

int asam_matvec(asam_ctx* h, const double* x, double* y) {
  if (!h || !x || !y) return kBadArg;
  const double* dx;
  double* dy;
  int rc = stage_in(h, x, h->len, h->stage_a, &dx);
  if (rc) return rc;
  rc = stage_out_begin(h, y, h->len, h->stage_b, &dy, false);
  if (rc) return rc;
  launch_matvec(h->L, h->d, h->cfg.ncomp, h->val, dx, dy, 0);
  rc = check_launch();
  if (rc) return rc;
  return stage_out_end(h, y, h->len, dy);
}

int asam_psolve(asam_ctx* h, const double* x, double* px) {
  if (!h || !x || !px) return kBadArg;
  const double* dx;
  double* dp;
  int rc = stage_in(h, x, h->len, h->stage_a, &dx);
  if (rc) return rc;
  rc = stage_out_begin(h, px, h->len, h->stage_b, &dp, false);
  if (rc) return rc;
  psolve_dev<double>(h, h->val, dx, dp, h->w64);
  rc = check_launch();
  if (rc) return rc;
  return stage_out_end(h, px, h->len, dp);
}

int asam_inner_psolve(asam_ctx* h, const double* x, double* px) {
  if (!h || !x || !px) return kBadArg;
  if (h->cfg.precision != ASAM_PREC_FP32_REFINED) {
    set_last_error("the FP32 inner preconditioner exists in the refined precision only", __FILE__, __LINE__);
    return kBadArg;
  }
  const Launch& L = h->L;
  const double* dx;
  double* dp;
  int rc = stage_in(h, x, h->len, h->stage_a, &dx);
  if (rc) return rc;
  rc = stage_out_begin(h, px, h->len, h->stage_b, &dp, false);
  if (rc) return rc;
  CK(cudaMemsetAsync(&h->sc->gs_err, 0, sizeof(int), L.stream));
  prepare_inner(h);
  launch_convert_f64_to_f32(L, h->len, dx, h->b32);
  psolve_dev<float>(h, h->val32, h->b32, h->x32, h->w32);
  launch_convert_f32_to_f64(L, h->len, h->x32, dp);
  if ((rc = check_launch()) || (rc = read_scalars(h))) return rc;
  return stage_out_end(h, px, h->len, dp);
}

int asam_bicgstab(asam_ctx* h, double* x, const double* b, int* maxiter, double* tol) {
  if (!h || !x || !b || !maxiter || !tol || *maxiter < 1) return kBadArg;
  const double* db;
  double* dx;
  int rc = stage_in(h, b, h->len, h->stage_a, &db);
  if (rc) return rc;
  rc = stage_out_begin(h, x, h->len, h->stage_b, &dx, true);
  if (rc) return rc;
  int st = solve_dev(h, dx, db, maxiter, tol, false);
  if (st != kOk && st != kNotConverged && st != kBreakdown) return st;
  rc = stage_out_end(h, x, h->len, dx);
  return rc ? rc : st;
}

int asam_ros_step(asam_ctx* h, double* c, double dt, int* iters, double* resid) {
  if (!h || !c) return kBadArg;
  double* dc;
  int rc = stage_out_begin(h, c, h->len, h->c, &dc, true);
  if (rc) return rc;
  int st = ros_step_dev(h, dc, dt, iters, resid);
  if (st != kOk && st != kNotConverged && st != kBreakdown) return st;
  rc = stage_out_end(h, c, h->len, dc);
  return rc ? rc : st;
}

int asam_state_dot(asam_ctx* h, const double* c, double* out) {
  if (!h || !c || !out) return kBadArg;
  const double* dc;
  int rc = stage_in(h, c, h->len, h->stage_a, &dc);
  if (rc) return rc;
  launch_dot(h->L, h->d, h->cfg.ncomp, dc, dc, h->partial, h->sc, OP_STORE_B, h->red_out);
  if ((rc = check_launch())) return rc;
  if ((rc = reduce_to_host(h, out))) return rc;
  if (std::isnan(*out)) {
    set_last_error("NaN in the state", __FILE__, __LINE__);
    return kNanDetected;
  }
  return kOk;
}

int asam_total_scalar(asam_ctx* h, const double* c, int comp, double* out) {
  if (!h || !c || !out || comp < 0 || comp >= h->cfg.ncomp) return kBadArg;
  const double* dc;
  int rc = stage_in(h, c, h->len, h->stage_a, &dc);
  if (rc) return rc;
  launch_mass(h->L, h->d, dc + (size_t)comp * h->npad, h->volc, h->partial, h->red_out);
  rc = check_launch();
  if (rc) return rc;
  return reduce_to_host(h, out);
}

int asam_tri_solve(int ncol, int n1, const double* d, const double* u, const double* l, double* b) {
  if (ncol < 1 || n1 < 1 || !d || !b || (n1 > 1 && (!u || !l))) return kBadArg;
  const size_t nd = (size_t)ncol * n1, no = (size_t)ncol * (n1 - 1);
  std::lock_guard<std::mutex> lock(g_col_mu);
  double* ws = nullptr;
  if (int rc = col_workspace(3 * nd + 2 * no, &ws)) return rc;
  double *dd = ws, *db = ws + nd, *dw = ws + 2 * nd;
  double *du = no ? ws + 3 * nd : nullptr, *dl = no ? ws + 3 * nd + no : nullptr;
  if (no) {
    CK(cudaMemcpy(du, u, no * sizeof(double), cudaMemcpyDefault));
    CK(cudaMemcpy(dl, l, no * sizeof(double), cudaMemcpyDefault));
  }
  CK(cudaMemcpy(dd, d, nd * sizeof(double), cudaMemcpyDefault));
  CK(cudaMemcpy(db, b, nd * sizeof(double), cudaMemcpyDefault));
  Launch L{0, 1};
  launch_tri_solve(L, ncol, n1, dd, du, dl, db, dw);
  if (int rc = check_launch()) return rc;
  CK(cudaMemcpy(b, db, nd * sizeof(double), cudaMemcpyDefault));
  return kOk;
}

int asam_tri_matvec(int ncol, int n1, const double* d, const double* u, const double* l, const double* x, double* y) {
  if (ncol < 1 || n1 < 1 || !d || !x || !y || (n1 > 1 && (!u || !l))) return kBadArg;
  const size_t nd = (size_t)ncol * n1, no = (size_t)ncol * (n1 - 1);
  std::lock_guard<std::mutex> lock(g_col_mu);
  double* ws = nullptr;
  if (int rc = col_workspace(3 * nd + 2 * no, &ws)) return rc;
  double *dd = ws, *dx = ws + nd, *dy = ws + 2 * nd;
  double *du = no ? ws + 3 * nd : nullptr, *dl = no ? ws + 3 * nd + no : nullptr;
  if (no) {
    CK(cudaMemcpy(du, u, no * sizeof(double), cudaMemcpyDefault));
    CK(cudaMemcpy(dl, l, no * sizeof(double), cudaMemcpyDefault));
  }
  CK(cudaMemcpy(dd, d, nd * sizeof(double), cudaMemcpyDefault));
  CK(cudaMemcpy(dx, x, nd * sizeof(double), cudaMemcpyDefault));
  Launch L{0, 1};
  launch_tri_matvec(L, ncol, n1, dd, du, dl, dx, dy);
  if (int rc = check_launch()) return rc;
  CK(cudaMemcpy(y, dy, nd * sizeof(double), cudaMemcpyDefault));
  return kOk;
}

}  // extern "C"
