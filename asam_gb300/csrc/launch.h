// Host-side launch wrappers of the transport-stage kernels.  Each function is
// defined twice: in k64.cu for double (exact FP64 rounding, no FMA
// contraction) and in k32.cu for float (inner solver of the refined mode).
#pragma once
#include "asam_common.cuh"

namespace asam {

struct Launch {
  cudaStream_t stream;
  int sm_count;
};

#define ASAM_DECLARE_LAUNCHERS(T, TM)                                                                            \
  void launch_phi(const Launch&, const Dims&, int ncomp, int rho_pos, const T* c, T* phi);                      \
  void launch_face_coef(const Launch&, const Dims&, const GeomT<T>&, T* coef_x, T* coef_y, T* coef_z,           \
                        unsigned char* mask_x, unsigned char* mask_y, unsigned char* mask_z);                    \
  void launch_face_flux(const Launch&, const Dims&, const GeomT<T>&, int ncomp, const T* coef_x, const T* coef_y, \
                        const T* coef_z, const unsigned char* mask_x, const unsigned char* mask_y,               \
                        const unsigned char* mask_z, const T* phi, T* gx, T* gy, T* gz);                         \
  void launch_flux_gather(const Launch&, const Dims&, const GeomT<T>&, int ncomp, const T* gx, const T* gy,      \
                          const T* gz, const T* rvol, T* f, const DiffSrc<T>* df,                                \
                          const WallIn<T>& wl = WallIn<T>{});                                                    \
  void launch_diff_coef(const Launch&, const Dims&, const GeomT<T>&, const T* dh, const T* dv, T* kx, T* ky,    \
                        T* kz);                                                                                  \
  void launch_recip_eps(const Launch&, size_t len, const T* v, T* rv);                                          \
  void launch_div(const Launch&, const Dims&, const GeomT<T>&, T* rhs);                                          \
  void launch_jac(const Launch&, const Dims&, const GeomT<T>&, const T* rho, const T* rvol, T bdt, T* val,      \
                  const T* dkx, const T* dky, const T* dkz);                                                     \
  void launch_matvec(const Launch&, const Dims&, int ncomp, const TM* val, const T* x, T* y, int plain_spmv);    \
  void launch_gs_sweeps(const Launch&, const Dims&, int ncomp, const TM* val, const T* b, T* out, T* work,       \
                        int nsweep, int group);                                                                  \
  void launch_gs_persist(const Launch&, const Dims&, int ncomp, const TM* val, const T* b, T* out, T* work,      \
                         int nsweep, const GsTileSched& sch);                                                    \
  void launch_line_psolve(const Launch&, const Dims&, int ncomp, const TM* val, const T* b, T* x, T* w,         \
                          int axis, const T* fw, const T* fr);                                                   \
  void launch_xline_factor(const Launch&, const Dims&, const TM* val, T* fw, T* fr);                            \
  void launch_zero_halo(const Launch&, const Dims&, int ncomp, T* x);                                           \
  void launch_exchange_cell(const Launch&, const Dims&, int ncomp, T* c);                                       \
  void launch_bound_cond(const Launch&, const Dims&, int ncomp, int comp0, const BcKinds& bc, T* c);            \
  void launch_dot(const Launch&, const Dims&, int ncomp, const T* x, const T* y, double* partial,               \
                  KrylovScalars* sc, int op, double* out);                                                       \
  void launch_axpy_sc(const Launch&, size_t len, const KrylovScalars* sc, int sel, double sign, const T* x,      \
                      T* y);                                                                                     \
  void launch_matvec_dot(const Launch&, const Dims&, int ncomp, const TM* val, const T* x, T* y, const T* a,     \
                         double* partial, KrylovScalars* sc, int op);                                            \
  void launch_matvec_dot2(const Launch&, const Dims&, int ncomp, const TM* val, const T* x, T* y, const T* a,    \
                          double* partial, KrylovScalars* sc, int op1, int op2);                                 \
  void launch_axpy_dot(const Launch&, const Dims&, int ncomp, KrylovScalars* sc, int sel, double sign,          \
                       const T* x, T* y, double* partial, int op);                                               \
  void launch_pupdate(const Launch&, size_t len, const KrylovScalars* sc, const T* r, const T* v, T* p);         \
  void launch_pupdate_auto(const Launch&, size_t len, const KrylovScalars* sc, const T* r, const T* v, T* p);    \
  void launch_xupdate_half(const Launch&, size_t len, const KrylovScalars* sc, const T* ph, T* x);              \
  void launch_xupdate(const Launch&, size_t len, const KrylovScalars* sc, int with_omega, const T* ph,          \
                      const T* rh, T* x);                                                                        \
  void launch_axpy_host(const Launch&, size_t len, T a, const T* x, T* y);                                      \
  void launch_xpay_host(const Launch&, size_t len, const T* x, T a, T* y);                                      \
  void launch_scale_host(const Launch&, size_t len, T a, T* y);                                                 \
  void launch_tri_solve(const Launch&, int ncol, int n1, const T* d, const T* u, const T* l, T* b, T* w);        \
  void launch_tri_matvec(const Launch&, int ncol, int n1, const T* d, const T* u, const T* l, const T* x, T* y);

ASAM_DECLARE_LAUNCHERS(double, double)
ASAM_DECLARE_LAUNCHERS(float, float)

void launch_beta(const Launch&, KrylovScalars* sc);
void launch_recip_diag(const Launch&, size_t npad, double* val);
void launch_mass(const Launch&, const Dims&, const double* c, const double* volc, double* partial, double* out);
void launch_convert_f64_to_f32(const Launch&, size_t len, const double* x, float* y);
void launch_convert_f32_to_f64(const Launch&, size_t len, const float* x, double* y);
void launch_add_f32_to_f64(const Launch&, size_t len, const float* x, double s, double* y);
void launch_convert_f64_to_f32_scaled(const Launch&, size_t len, const double* x, double s, float* y);
void launch_resid_dot(const Launch&, const Dims&, int ncomp, const double* val, const double* x, const double* b,
                      double* r, double* partial, KrylovScalars* sc, int op, double* out);

constexpr int kRedGrid = 1024;  // number of partial sums of the reductions
// blocks of the fused SpMV + dot kernels (at most; the matvec's grid, whose
// every thread keeps many cells' loads in flight), and the partials they need
constexpr int kFusedGridMax = 4096;

}  // namespace asam

// FP64 launchers of the refined mode with FMA contraction (k64fma.cu)
namespace asam_fma {
void launch_fcn(const asam::Launch&, const asam::Dims&, const asam::GeomT<double>& g, int ncomp, int rho_pos,
                const double* c, const double* cx, const double* cy, const double* cz, const unsigned char* mx,
                const unsigned char* my, const unsigned char* mz, double* phi, double* gx, double* gy, double* gz,
                const double* rvol, double* f, const asam::DiffSrc<double>* df);
// the same flux with the momentum sources of the dynamical stage
void launch_fcn_mom(const asam::Launch&, const asam::Dims&, const asam::GeomT<double>& g, int ncomp, int rho_pos,
                    const double* c, const double* cx, const double* cy, const double* cz, const unsigned char* mx,
                    const unsigned char* my, const unsigned char* mz, double* phi, double* gx, double* gy, double* gz,
                    const double* rvol, double* f, const asam::MomSrc<double>& ms, const asam::DiffSrc<double>* df);
void launch_jac(const asam::Launch&, const asam::Dims&, const asam::GeomT<double>&, const double* rho,
                const double* rvol, double bdt, double* val, const double* dkx, const double* dky, const double* dkz);
void launch_resid_dot(const asam::Launch&, const asam::Dims&, int ncomp, const double* val, const double* x,
                      const double* b, double* r, double* partial, asam::KrylovScalars* sc, int op, double* out);
}  // namespace asam_fma
