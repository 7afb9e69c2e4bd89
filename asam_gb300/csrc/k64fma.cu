// FP64 kernels of the refined mode with FMA contraction allowed: the flux
// right-hand side (with the momentum sources of the dynamical stage), the
// stage matrix and the refinement residual.  The refined
// mode is held to 1e-10 against the FP64 oracle, not to bit parity, so these
// may fuse multiply-adds (fewer instructions on the scarce FP64 pipe); the
// drop-in path keeps its own copies compiled without contraction (k64.cu).
#include "launchers_impl.cuh"

namespace asam_fma {
using asam::count_launches;
using asam::Dims;
using asam::GeomT;
using asam::KrylovScalars;
using asam::Launch;

void launch_fcn(const Launch& L, const Dims& d, const GeomT<double>& g, int ncomp, int rho_pos, const double* c,
                const double* cx, const double* cy, const double* cz, const unsigned char* mx,
                const unsigned char* my, const unsigned char* mz, double* phi, double* gx, double* gy, double* gz,
                const double* rvol, double* f, const asam::DiffSrc<double>* df) {
  k_phi<double><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, ncomp, rho_pos, c, phi);
  k_face_flux<double, 0><<<gs_grid(L, d.n_uf()), kBlock, 0, L.stream>>>(d, g, ncomp, cx, mx, phi, gx);
  k_face_flux<double, 1><<<gs_grid(L, d.n_vf()), kBlock, 0, L.stream>>>(d, g, ncomp, cy, my, phi, gy);
  k_face_flux<double, 2><<<gs_grid(L, d.n_wf()), kBlock, 0, L.stream>>>(d, g, ncomp, cz, mz, phi, gz);
  const asam::WallIn<double> wl{c, c + (size_t)rho_pos * d.npad()};
  if (df)
    k_flux_gather<double, false, true><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, ncomp, gx, gy, gz, rvol, f,
                                                                                        MomSrc<double>{}, *df, wl);
  else
    k_flux_gather<double><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, ncomp, gx, gy, gz, rvol, f,
                                                                          MomSrc<double>{}, asam::DiffSrc<double>{},
                                                                          wl);
  count_launches(5);
}

void launch_fcn_mom(const Launch& L, const Dims& d, const GeomT<double>& g, int ncomp, int rho_pos, const double* c,
                    const double* cx, const double* cy, const double* cz, const unsigned char* mx,
                    const unsigned char* my, const unsigned char* mz, double* phi, double* gx, double* gy,
                    double* gz, const double* rvol, double* f, const asam::MomSrc<double>& ms,
                    const asam::DiffSrc<double>* df) {
  k_phi<double><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, ncomp, rho_pos, c, phi);
  k_face_flux<double, 0><<<gs_grid(L, d.n_uf()), kBlock, 0, L.stream>>>(d, g, ncomp, cx, mx, phi, gx);
  k_face_flux<double, 1><<<gs_grid(L, d.n_vf()), kBlock, 0, L.stream>>>(d, g, ncomp, cy, my, phi, gy);
  k_face_flux<double, 2><<<gs_grid(L, d.n_wf()), kBlock, 0, L.stream>>>(d, g, ncomp, cz, mz, phi, gz);
  const asam::WallIn<double> wl{c, c + (size_t)rho_pos * d.npad()};
  if (df)
    k_flux_gather<double, true, true><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, ncomp, gx, gy, gz, rvol, f,
                                                                                       ms, *df, wl);
  else
    k_flux_gather<double, true><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, ncomp, gx, gy, gz, rvol, f, ms,
                                                                                asam::DiffSrc<double>{}, wl);
  count_launches(5);
}

void launch_jac(const Launch& L, const Dims& d, const GeomT<double>& g, const double* rho, const double* rvol,
                double bdt, double* val, const double* dkx, const double* dky, const double* dkz) {
  k_jac<double><<<gs_grid(L, d.npad()), kBlock, 0, L.stream>>>(d, g, rho, rvol, bdt, val, dkx, dky, dkz);
  count_launches(1);
}

void launch_resid_dot(const Launch& L, const Dims& d, int ncomp, const double* val, const double* x, const double* b,
                      double* r, double* partial, KrylovScalars* sc, int op, double* out) {
  k_resid_dot<double><<<RED_GRID, RED_BLOCK, 0, L.stream>>>(d, ncomp, val, x, b, r, partial);
  k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial, RED_GRID, sc, op, out);
  count_launches(2);
}
}  // namespace asam_fma
