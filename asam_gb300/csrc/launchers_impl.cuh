// Definitions of the launch wrappers declared in launch.h for one scalar type.
// Included once per precision translation unit after kernels.cuh.
#pragma once
#include "kernels.cuh"

namespace asam {
void count_launches(long long n);
}
namespace {
constexpr int kBlock = 256;
inline int fused_grid(const asam::Launch& L, size_t n) {
  size_t g = (n + RED_BLOCK - 1) / RED_BLOCK, cap = (size_t)L.sm_count * 16;
  if (cap > (size_t)asam::kFusedGridMax) cap = asam::kFusedGridMax;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}
inline int gs_grid(const asam::Launch& L, size_t n) {
  size_t g = (n + kBlock - 1) / kBlock;
  size_t cap = (size_t)L.sm_count * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}
}  // namespace

#define ASAM_DEFINE_LAUNCHERS(T, TM)                                                                               \
  namespace asam {                                                                                                 \
  void launch_phi(const Launch& L, const Dims& d, int ncomp, int rho_pos, const T* c, T* phi) {                   \
    k_phi<T><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, ncomp, rho_pos, c, phi); count_launches(1);                            \
  }                                                                                                                \
  void launch_face_coef(const Launch& L, const Dims& d, const GeomT<T>& g, T* cx, T* cy, T* cz, unsigned char* mx,  \
                        unsigned char* my, unsigned char* mz) {                                                    \
    k_face_coef<T, 0><<<gs_grid(L, d.n_uf()), kBlock, 0, L.stream>>>(d, g, cx, mx);                               \
    k_face_coef<T, 1><<<gs_grid(L, d.n_vf()), kBlock, 0, L.stream>>>(d, g, cy, my);                               \
    k_face_coef<T, 2><<<gs_grid(L, d.n_wf()), kBlock, 0, L.stream>>>(d, g, cz, mz);                               \
    count_launches(3);                                                                                             \
  }                                                                                                                \
  void launch_face_flux(const Launch& L, const Dims& d, const GeomT<T>& g, int ncomp, const T* cx, const T* cy,    \
                        const T* cz, const unsigned char* mx, const unsigned char* my, const unsigned char* mz,    \
                        const T* phi, T* gx, T* gy, T* gz) {                                                       \
    k_face_flux<T, 0><<<gs_grid(L, d.n_uf()), kBlock, 0, L.stream>>>(d, g, ncomp, cx, mx, phi, gx);               \
    k_face_flux<T, 1><<<gs_grid(L, d.n_vf()), kBlock, 0, L.stream>>>(d, g, ncomp, cy, my, phi, gy);               \
    k_face_flux<T, 2><<<gs_grid(L, d.n_wf()), kBlock, 0, L.stream>>>(d, g, ncomp, cz, mz, phi, gz);               \
    count_launches(3);                                                                                             \
  }                                                                                                                \
  void launch_flux_gather(const Launch& L, const Dims& d, const GeomT<T>& g, int ncomp, const T* gx, const T* gy,  \
                          const T* gz, const T* rvol, T* f, const DiffSrc<T>* df, const WallIn<T>& wl) {           \
    if (df)                                                                                                        \
      k_flux_gather<T, false, true><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, ncomp, gx, gy, gz, rvol,  \
                                                                                   f, MomSrc<T>{}, *df, wl);       \
    else                                                                                                           \
      k_flux_gather<T><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, ncomp, gx, gy, gz, rvol, f,            \
                                                                      MomSrc<T>{}, DiffSrc<T>{}, wl);              \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_diff_coef(const Launch& L, const Dims& d, const GeomT<T>& g, const T* dh, const T* dv, T* kx, T* ky,  \
                        T* kz) {                                                                                   \
    k_diff_coef<T><<<gs_grid(L, d.n_uf() + d.n_vf() + d.n_wf()), kBlock, 0, L.stream>>>(d, g, dh, dv, kx, ky, kz);  \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_recip_eps(const Launch& L, size_t len, const T* v, T* rv) {                                          \
    k_recip_eps<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, v, rv);                                          \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_div(const Launch& L, const Dims& d, const GeomT<T>& g, T* rhs) {                                     \
    k_div<T><<<gs_grid(L, (size_t)d.nx * d.ny * d.nz), kBlock, 0, L.stream>>>(d, g, rhs); count_launches(1);                          \
  }                                                                                                                \
  void launch_jac(const Launch& L, const Dims& d, const GeomT<T>& g, const T* rho, const T* rvol, T bdt,         \
                  T* val, const T* dkx, const T* dky, const T* dkz) {                                              \
    k_jac<T><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, rho, rvol, bdt, val, dkx, dky, dkz);            \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_matvec(const Launch& L, const Dims& d, int ncomp, const TM* val, const T* x, T* y, int plain) {      \
    k_matvec<TM, T><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, ncomp, val, x, y, plain);                    \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_gs_sweeps(const Launch& L, const Dims& d, int ncomp, const TM* val, const T* b, T* out, T* work,     \
                        int nsweep, int group) {                                                                   \
    const int ntx = (d.NX() + GS_TX - 1) / GS_TX;                                                                  \
    const int nty = (d.NY() + GS_TY - 1) / GS_TY;                                                                  \
    const int ntz = (d.NZ() + GS_TZ - 1) / GS_TZ;                                                                  \
    const int nlev = ntx + nty + ntz - 2;                                                                          \
    const bool staged = sizeof(T) == sizeof(float);                                                               \
    /* whole warps (the sweep shuffles); the staged variant runs one component group per CTA */                 \
    const int threads = (GS_TY * GS_TZ * (staged ? group : ncomp) + 31) / 32 * 32;                                \
    const dim3 grid(ntx, ntz, nsweep * (staged ? gs_ngroups(ncomp, group) : 1));                                   \
    const size_t smem = staged ? gs_smem_elems(group) * sizeof(T) : 0;                                             \
    thread_local size_t smem_set = 0;                                                                              \
    if (staged && smem > smem_set) {                                                                               \
      cudaFuncSetAttribute(k_gs_pipe_smem<TM, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);         \
      smem_set = smem;                                                                                             \
    }                                                                                                              \
    for (int tau = 0; tau < nlev + 2 * (nsweep - 1); ++tau) {                                                      \
      if (staged)                                                                                                  \
        k_gs_pipe_smem<TM, T><<<grid, threads, smem, L.stream>>>(d, ncomp, group, val, b, out, work, tau, nsweep,  \
                                                                 ntx, nty, ntz, nlev);                             \
      else                                                                                                         \
        k_gs_pipe_reg<TM, T><<<grid, threads, 0, L.stream>>>(d, ncomp, val, b, out, work, tau, nsweep, ntx, nty,  \
                                                             ntz, nlev);                                           \
      count_launches(1);                                                                                           \
    }                                                                                                              \
  }                                                                                                                \
  void launch_gs_persist(const Launch& L, const Dims& d, int ncomp, const TM* val, const T* b, T* out, T* work,    \
                         int nsweep, const GsTileSched& sch) {                                                     \
    const int ntx = (d.NX() + GS_TX - 1) / GS_TX;                                                                  \
    const int nty = (d.NY() + GS_TY - 1) / GS_TY;                                                                  \
    const int ntz = (d.NZ() + GS_TZ - 1) / GS_TZ;                                                                  \
    const int threads = (GS_TY * GS_TZ * sch.group + 31) / 32 * 32;                                                \
    const size_t smem = gs_smem_elems(sch.group) * sizeof(T);                                                      \
    /* per host thread: the attribute and the occupancy of the last shared-memory size */                       \
    thread_local size_t smem_set = 0;                                                                              \
    thread_local int per_sm = 0;                                                                                   \
    if (smem != smem_set) { /* smem determines threads */                                                         \
      cudaFuncSetAttribute(k_gs_persist<TM, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);           \
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gs_persist<TM, T>, threads, smem);                  \
      if (per_sm < 1) per_sm = 1;                                                                                  \
      smem_set = smem;                                                                                             \
    }                                                                                                              \
    int grid = per_sm * L.sm_count;                                                                                \
    if (grid > sch.nticket) grid = sch.nticket;                                                                    \
    cudaMemsetAsync(sch.counter, 0, sizeof(int), L.stream);                                                        \
    k_gs_persist<TM, T><<<grid, threads, smem, L.stream>>>(d, ncomp, val, b, out, work, nsweep, ntx, nty, ntz,    \
                                                            sch);                                                  \
    k_gs_advance<<<1, 32, 0, L.stream>>>(sch.base, nsweep);                                                        \
    count_launches(2);                                                                                             \
  }                                                                                                                \
  void launch_line_psolve(const Launch& L, const Dims& d, int ncomp, const TM* val, const T* b, T* x, T* w,       \
                          int axis, const T* fw, const T* fr) {                                                    \
    if (axis == 0) {                                                                                               \
      const int wpb = xl_warps<T>();                                                                               \
      const long long tasks = (long long)((d.NY() * d.NZ() + 31) / 32) * ncomp;                                   \
      k_xline_solve<TM, T><<<(unsigned)((tasks + wpb - 1) / wpb), 32 * wpb, 0, L.stream>>>(d, ncomp, val, fw, fr,  \
                                                                                             b, x);                \
    } else {                                                                                                       \
      const size_t ncols = (size_t)d.NX() * (axis == 2 ? d.NY() : d.NZ());                                         \
      k_line_psolve<TM, T><<<(unsigned)((ncols + 127) / 128), 128, 0, L.stream>>>(d, ncomp, axis, val, b, x, w);   \
    }                                                                                                              \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_xline_factor(const Launch& L, const Dims& d, const TM* val, T* fw, T* fr) {                          \
    const int wpb = xl_warps<T>();                                                                                 \
    const long long groups = (d.NY() * d.NZ() + 31) / 32;                                                         \
    k_xline_factor<TM, T><<<(unsigned)((groups + wpb - 1) / wpb), 32 * wpb, 0, L.stream>>>(d, val, fw, fr);        \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_zero_halo(const Launch& L, const Dims& d, int ncomp, T* x) {                                         \
    k_zero_halo<T><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, ncomp, x); count_launches(1);                                    \
  }                                                                                                                \
  void launch_exchange_cell(const Launch& L, const Dims& d, int ncomp, T* c) {                                     \
    size_t tot = (d.per_x ? (size_t)d.ny * d.nz : 0) + (d.per_y ? (size_t)d.nx * d.nz : 0) +                       \
                 (d.per_z ? (size_t)d.nx * d.ny : 0);                                                              \
    if (tot == 0) return;                                                                                          \
    k_exchange_cell<T><<<gs_grid(L, tot), kBlock, 0, L.stream>>>(d, ncomp, c); count_launches(1);                                     \
  }                                                                                                                \
  void launch_bound_cond(const Launch& L, const Dims& d, int ncomp, int comp0, const BcKinds& bc, T* c) {        \
    size_t tot = (d.per_x ? 0 : (size_t)d.ny * d.nz) + (d.per_y ? 0 : (size_t)d.nx * d.nz) +                       \
                 (d.per_z ? 0 : (size_t)d.nx * d.ny);                                                              \
    bool any = false;                                                                                              \
    for (int ic = comp0; ic < comp0 + ncomp; ++ic)                                                                 \
      for (int s = 0; s < 6; ++s) any = any || bc.k[ic][s] != kBcNone;                                            \
    if (tot == 0 || !any) return;                                                                                  \
    k_bound_cond<T><<<gs_grid(L, tot), kBlock, 0, L.stream>>>(d, ncomp, comp0, bc, c); count_launches(1);         \
  }                                                                                                                \
  void launch_dot(const Launch& L, const Dims& d, int ncomp, const T* x, const T* y, double* partial,              \
                  KrylovScalars* sc, int op, double* out) {                                                        \
    k_dot_partial<T><<<RED_GRID, RED_BLOCK, 0, L.stream>>>(d, ncomp, x, y, partial); count_launches(1);                               \
    k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial, RED_GRID, sc, op, out); count_launches(1);                                    \
  }                                                                                                                \
  void launch_axpy_sc(const Launch& L, size_t len, const KrylovScalars* sc, int sel, double sign, const T* x,       \
                      T* y) {                                                                                      \
    k_axpy_sc<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, sc, sel, sign, x, y); count_launches(1);                              \
  }                                                                                                                \
  void launch_matvec_dot(const Launch& L, const Dims& d, int ncomp, const TM* val, const T* x, T* y, const T* a,  \
                         double* partial, KrylovScalars* sc, int op) {                                             \
    if (sizeof(T) == sizeof(float)) { /* FP32: product and dot product apart, measured faster */               \
      launch_matvec(L, d, ncomp, val, x, y, 0);                                                                    \
      launch_dot(L, d, ncomp, a, y, partial, sc, op, nullptr);                                                     \
      return;                                                                                                      \
    }                                                                                                              \
    const int g = fused_grid(L, d.npad());                                                                         \
    k_matvec_dot<TM, T, false><<<g, RED_BLOCK, 0, L.stream>>>(d, ncomp, val, x, y, a, partial, nullptr);           \
    k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial, g, sc, op, nullptr);                                       \
    count_launches(2);                                                                                             \
  }                                                                                                                \
  /* two dot products of the product: partial holds 2*RED_GRID values; op1 is final first */                      \
  void launch_matvec_dot2(const Launch& L, const Dims& d, int ncomp, const TM* val, const T* x, T* y, const T* a, \
                          double* partial, KrylovScalars* sc, int op1, int op2) {                                  \
    if (sizeof(T) == sizeof(float)) {                                                                              \
      launch_matvec(L, d, ncomp, val, x, y, 0);                                                                    \
      launch_dot(L, d, ncomp, y, a, partial, sc, op1, nullptr);                                                    \
      launch_dot(L, d, ncomp, y, y, partial, sc, op2, nullptr);                                                    \
      return;                                                                                                      \
    }                                                                                                              \
    const int g = fused_grid(L, d.npad());                                                                         \
    k_matvec_dot<TM, T, true><<<g, RED_BLOCK, 0, L.stream>>>(d, ncomp, val, x, y, a, partial, partial + g);        \
    k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial, g, sc, op1, nullptr);                                      \
    k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial + g, g, sc, op2, nullptr);                                  \
    count_launches(3);                                                                                             \
  }                                                                                                                \
  void launch_axpy_dot(const Launch& L, const Dims& d, int ncomp, KrylovScalars* sc, int sel, double sign,        \
                       const T* x, T* y, double* partial, int op) {                                                \
    k_axpy_dot<T><<<RED_GRID, RED_BLOCK, 0, L.stream>>>(d, ncomp, sc, sel, sign, x, y, partial);                  \
    k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial, RED_GRID, sc, op, nullptr);                                \
    count_launches(2);                                                                                             \
  }                                                                                                                \
  void launch_pupdate_auto(const Launch& L, size_t len, const KrylovScalars* sc, const T* r, const T* v, T* p) {    \
    k_pupdate_auto<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, sc, r, v, p); count_launches(1);              \
  }                                                                                                                \
  void launch_xupdate_half(const Launch& L, size_t len, const KrylovScalars* sc, const T* ph, T* x) {              \
    k_xupdate_half<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, sc, ph, x); count_launches(1);                \
  }                                                                                                                \
  void launch_pupdate(const Launch& L, size_t len, const KrylovScalars* sc, const T* r, const T* v, T* p) {         \
    k_pupdate<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, sc, r, v, p); count_launches(1);                                      \
  }                                                                                                                \
  void launch_xupdate(const Launch& L, size_t len, const KrylovScalars* sc, int with_omega, const T* ph,           \
                      const T* rh, T* x) {                                                                         \
    k_xupdate<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, sc, with_omega, ph, rh, x); count_launches(1);                        \
  }                                                                                                                \
  void launch_axpy_host(const Launch& L, size_t len, T a, const T* x, T* y) {                                      \
    if (a == (T)0) return;                                                                                         \
    k_axpy_host<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, a, x, y); count_launches(1);                                        \
  }                                                                                                                \
  void launch_xpay_host(const Launch& L, size_t len, const T* x, T a, T* y) {                                      \
    k_xpay_host<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, x, a, y); count_launches(1);                                        \
  }                                                                                                                \
  void launch_scale_host(const Launch& L, size_t len, T a, T* y) {                                                 \
    k_scale_host<T><<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, a, y); count_launches(1);                                          \
  }                                                                                                                \
  void launch_tri_solve(const Launch& L, int ncol, int n1, const T* dd, const T* uu, const T* ll, T* bb, T* ww) {  \
    k_tri_solve_w<T><<<(ncol + 32 * kTriWarps - 1) / (32 * kTriWarps), 32 * kTriWarps, 0, L.stream>>>(             \
        ncol, n1, dd, uu, ll, bb, ww);                                                                             \
    count_launches(1);                                                                                             \
  }                                                                                                                \
  void launch_tri_matvec(const Launch& L, int ncol, int n1, const T* dd, const T* uu, const T* ll, const T* xx,    \
                         T* yy) {                                                                                  \
    size_t tot = (size_t)ncol * n1;                                                                                \
    k_tri_matvec<T><<<(unsigned)((tot + 255) / 256), 256, 0, L.stream>>>(ncol, n1, dd, uu, ll, xx, yy); count_launches(1);            \
  }                                                                                                                \
  }
