// Context of one block on the device and the internal host drivers shared by
// the C-ABI translation units (capi.cu, adjoint.cu).
#pragma once
#include "asam_common.cuh"
#include "asam_gb300.h"
#include "launch.h"

namespace asam {

template <typename T>
struct Work {
  T *r = nullptr, *rt = nullptr, *rh = nullptr, *p = nullptr, *ph = nullptr, *t = nullptr, *v = nullptr;
  T *bbuf = nullptr, *tbuf = nullptr;
};

template <typename T>
inline cudaError_t alloc_work(Work<T>& w, size_t len) {
  T** ptrs[] = {&w.r, &w.rt, &w.rh, &w.p, &w.ph, &w.t, &w.v, &w.bbuf, &w.tbuf};
  for (T** q : ptrs) {
    cudaError_t e = cudaMalloc((void**)q, len * sizeof(T));
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
template <typename T>
inline void free_work(Work<T>& w) {
  T* ptrs[] = {w.r, w.rt, w.rh, w.p, w.ph, w.t, w.v, w.bbuf, w.tbuf};
  for (T* q : ptrs)
    if (q) cudaFree(q);
  w = Work<T>();
}

struct ProjState;
struct DynState;

}  // namespace asam

// CUDA graphs of the BiCGStab half-iterations of one precision
struct KrylovGraphs {
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
  bool warm[3] = {false, false, false};
  long long n[3] = {0, 0, 0};  // kernel launches per replay
};

struct asam_ctx {
  using Launch = asam::Launch;
  using Dims = asam::Dims;
  template <typename T> using Work = asam::Work<T>;
  template <typename T> using GeomT = asam::GeomT<T>;
  using KrylovScalars = asam::KrylovScalars;
  asam_config cfg;
  Dims d;
  Launch L;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  size_t npad = 0, len = 0;
  int nstage = 0;
  double beta0 = 0, alpha[16], beta[16], gamma1[5];
  // geometry + velocities (device)
  double *volc = nullptr, *fu = nullptr, *fv = nullptr, *fw = nullptr, *uf = nullptr, *vf = nullptr, *wf = nullptr;
  // stage storage
  double *c = nullptr, *cold = nullptr, *rhs = nullptr, *incr = nullptr, *phi = nullptr;
  double *gx = nullptr, *gy = nullptr, *gz = nullptr;
  double *coef_x = nullptr, *coef_y = nullptr, *coef_z = nullptr;  // per-face flux coefficients
  unsigned char *mask_x = nullptr, *mask_y = nullptr, *mask_z = nullptr;
  double* rvol = nullptr;  // 1/(VolC+Eps)
  double* val = nullptr;
  float* val32 = nullptr;
  Work<double> w64;
  Work<float> w32;
  float *x32 = nullptr, *b32 = nullptr;
  KrylovScalars* sc = nullptr;
  KrylovScalars* sc_host = nullptr;
  double* partial = nullptr;
  double* red_out = nullptr;
  double* red_host = nullptr;
  double *stage_a = nullptr, *stage_b = nullptr;
  bool jac_ready = false;
  KrylovGraphs kg[2];     // [0] FP64, [1] FP32 inner solver
  unsigned long long graph_gen = 0;  // bumped whenever captured work goes stale (graphs_reset)
  bool use_graphs = true;  // capture the half-iterations (when the stream allows it)
  // device-driven whole-step graphs (FP64): every BiCGStab loop is a graph
  // WHILE node, so a Rosenbrock step is one graph launch and one host read
  bool step_graphs = false;
  cudaGraphExec_t step_exec = nullptr;
  const double* step_c = nullptr;  // state, step and tolerance the graph was captured for
  double step_dt = 0.0, step_tol = 0.0;
  long long step_n_fixed = 0, step_n_h1 = 0, step_n_h2 = 0, step_n_outer = 0;  // kernels outside / per pass of the loops
  cudaStream_t cap_stream[3] = {nullptr, nullptr, nullptr};  // capture streams of the loop bodies
  KrylovScalars* stage_sc = nullptr;                // scalars of each stage's solve (4)
  KrylovScalars* ref_sc = nullptr;                  // outer scalars of a device-driven refined solve
  KrylovScalars* stage_sc_host = nullptr;
  // x-line factors of the FP32 inner line solve (w and 1/den per cell), valid
  // for the current stage matrix while xline_ready is set
  float *xl_w = nullptr, *xl_r = nullptr;
  bool xline_ready = false;
  // persistent Gauss-Seidel schedule of the FP32 inner sweeps
  int4* gs_order = nullptr;
  int gs_nticket = 0;
  int* gs_flags = nullptr;  // one completion counter per tile and component group
  size_t gs_nflags = 0;
  int* gs_counter = nullptr;  // [0] ticket counter; [1] epoch base (unsigned)
  int gs_spin = 0;            // polls per dependency wait; 0 = the default (2^21)

  asam::ProjState* proj = nullptr;  // pressure projection (proj.cu), set up on demand
  asam::DynState* dyn = nullptr;    // dynamical-core stage (dyn.cu), set up on demand
  // halo rule of each component on the outer walls, applied to the state at
  // the start of every stage (default ZeroGrad, BoundaryCond_Mod.f90:240-247)
  asam::BcKinds bc{};
  // device copies of the open-boundary rules' data (asam_set_boundary_data)
  double *bc_mean = nullptr, *bc_fval = nullptr, *bc_amb = nullptr;
  bool bc_open() const {  // a kind beyond ZeroGrad/ZeroValue is set
    for (int ic = 0; ic < cfg.ncomp; ++ic)
      for (int sd = 0; sd < 6; ++sd)
        if (bc.k[ic][sd] > asam::kBcZeroValue) return true;
    return false;
  }
  // diffusion (asam_set_diffusion): face coefficients of DiffusionCompute,
  // nullptr while diffusion is off; jac_diff adds the diffusion Jacobian
  double *dkx = nullptr, *dky = nullptr, *dkz = nullptr;
  bool jac_diff = false;
  const asam::DiffSrc<double>* diff_src(asam::DiffSrc<double>& tmp) const {
    if (!dkx) return nullptr;
    tmp = asam::DiffSrc<double>{dkx, dky, dkz, phi};
    return &tmp;
  }

  GeomT<double> geom() const { return GeomT<double>{volc, fu, fv, fw, uf, vf, wf}; }
};

namespace asam {

void count_launches(long long n);
void set_last_error(const char* msg, const char* file, int line);
int check_launch();
int read_scalars(asam_ctx* h);
int reduce_to_host(asam_ctx* h, double* out);
bool is_device_ptr(const void* p);
bool device_array(const void* p);  // device memory, false without a CUDA driver
template <typename T>
void psolve_dev(asam_ctx* h, const T* val, const T* in, T* out, Work<T>& w);
template <typename T>
int bicgstab_dev(asam_ctx* h, const T* val, T* x, const T* b, int* maxiter, double* tol, Work<T>& w,
                 bool x_is_zero);
int fcn_dev(asam_ctx* h, const double* c, double* f);
int jac_dev(asam_ctx* h, const double* c, double dt);
int solve_dev(asam_ctx* h, double* x, const double* b, int* maxiter, double* tol, bool x_is_zero);
int ros_step_dev(asam_ctx* h, double* c, double dt, int* iters, double* resid);
int stage_in(asam_ctx* h, const double* p, size_t n, double* buf, const double** dev);
int stage_out_begin(asam_ctx* h, double* p, size_t n, double* buf, double** dev, bool copy_in);
int stage_out_end(asam_ctx* h, double* p, size_t n, double* dev);
int gs_schedule_init(asam_ctx* h, int nsweep);
void gs_schedule_free(asam_ctx* h);
void graphs_reset(asam_ctx* h);
int ros_step_graph(asam_ctx* h, double* c, double dt, int* iters, double* resid);
void step_graph_free(asam_ctx* h);
int step_graph_prepare(asam_ctx* h);
void prepare_inner(asam_ctx* h);
int step_record(asam_ctx* h, double* c, double dt, long long* n_fixed, long long* n_h1, long long* n_h2,
                long long* n_outer);
int step_outputs(const asam_ctx* h, const KrylovScalars* ks, long long n_fixed, long long n_h1, long long n_h2,
                 long long n_outer, int* iters, double* resid, long long* ran);
long long thread_launches();
void proj_free(asam_ctx* h);
// device arrays of the projection's grid (valid after asam_proj_setup)
struct ProjGrid {
  const double *dx, *dy, *dz, *mxy, *myx;
};
bool proj_grid(asam_ctx* h, ProjGrid* out);
void dyn_free(asam_ctx* h);

}  // namespace asam

#define CK(expr) ASAM_CUDA_OK(expr)
