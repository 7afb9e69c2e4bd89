// Dynamical-core stage of one block (closed sides, or periodic in x and/or y)
// on the device: the momentum branch
// (uPosL>0) of the Rosenbrock stage around the transport solve and the
// pressure projection.
//   * VelocityFaceToCellLR (ADVECT/VelocityCellFace_Mod.f90:72-95, 541-654)
//     with ShiftVel1 / ShiftNoSlip at the boundary cells (:820-909),
//   * VelocityCellToFaceLR (:27-52, 1369-1894),
//   * AbsTCompute 'Density' and PreCompute (ADVECT/Diagnostic_Mod.f90:593-615,
//     710-865),
//   * FcnMet with the pressure gradient and the buoyancy of the momentum
//     components (ADVECT/Function_Mod.f90:989-1506; the sources are fused into
//     the flux gather, kernels.cuh MomSrc),
//   * the stage driver (ADVECT/Int_Mod.f90:263-374, 1059-1122): JacAccGrav at
//     the first stage, the transport BiCGStab, ProjectVelFace, the face
//     velocity update.
// FP64 without FMA contraction (-fmad=false): every value except the
// temperature (pow) is the oracle's bit for bit.  A context in the refined
// precision takes its flux from the contracted copy (k64fma.cu), like the
// transport step.
#include <cmath>
#include <vector>

#include "context.h"
#include "kernels.cuh"

namespace asam {

struct DynState {
  asam_dyn_config cfg{};
  int* bound = nullptr;  // BoundCell list, (ix,iy,iz) per cell
  int nbound = 0;
  std::vector<int> scalars;
  double *tabs = nullptr, *pre = nullptr;  // padded TAbsCell, PreCell
  double* vold = nullptr;                  // VelFOld: uF, vF, wF back to back
  double* incrf = nullptr;                 // VecIncrF of each stage, same layout
  double* facef = nullptr;                 // face staging for host callers
  size_t nu = 0, nv = 0, nw = 0;
};

namespace dyn {

// MODULE/Parameter_Mod.f90:20-36
constexpr double kCpd = 1004.0, kCvd = 717.0, kRd = kCpd - kCvd, kCpv = 1885.0, kRv = 461.0, kCpl = 4186.0,
                 kCpi = 2110.0, kP0 = 1.0e5;
constexpr int kB = 256;

struct Pos6 {
  int p[6];
};

inline int grid_of(const Launch& L, size_t n) {
  size_t g = (n + kB - 1) / kB, cap = (size_t)L.sm_count * 16;
  return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

// VelFaceToCellComputeLR: every interior cell takes its face values (the
// loop's first assignment block is overwritten by the second, :621-626).
__global__ void k_face_to_cell(Dims d, Pos6 pos, const double* __restrict__ uf, const double* __restrict__ vf,
                               const double* __restrict__ wf, double* __restrict__ c) {
  const int nx = d.nx, ny = d.ny;
  const size_t n = d.npad(), nint = (size_t)nx * ny * d.nz;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nint; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx) + 1, j = (int)((q / nx) % ny) + 1, k = (int)(q / ((size_t)nx * ny)) + 1;
    const size_t P = d.P(i, j, k);
    c[pos.p[0] * n + P] = uf[d.UF(i - 1, j, k)];
    c[pos.p[1] * n + P] = uf[d.UF(i, j, k)];
    c[pos.p[2] * n + P] = vf[d.VF(i, j - 1, k)];
    c[pos.p[3] * n + P] = vf[d.VF(i, j, k)];
    c[pos.p[4] * n + P] = wf[d.WF(i, j, k - 1)];
    c[pos.p[5] * n + P] = wf[d.WF(i, j, k)];
  }
}

// ShiftVel1 (FreeSlip, ADVECT/VelocityCellFace_Mod.f90:820-855) or
// ShiftNoSlip (:880-909) of the cells of the BoundCell list.
__device__ __forceinline__ void shift_pair(bool free_slip, double FL, double FR, double l, double r, double& cl,
                                           double& cr) {
  const double e = kEps;
  if (free_slip) {
    if (FL > FR) {
      cl = l;
      cr = (FR * r + (FL - FR) * l) / (FL + e);
    } else {
      cl = (FL * l + (FR - FL) * r) / (FR + e);
      cr = r;
    }
  } else {
    const double m = FR > FL ? FR : FL;
    cl = FL * l / m;
    cr = FR * r / m;
  }
}
__global__ void k_shift_bound(Dims d, GeomT<double> g, Pos6 pos, const int* __restrict__ cells, int ncell,
                              int free_slip, const double* __restrict__ uf, const double* __restrict__ vf,
                              const double* __restrict__ wf, double* __restrict__ c) {
  const size_t n = d.npad();
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ncell; q += gridDim.x * blockDim.x) {
    const int i = cells[3 * q], j = cells[3 * q + 1], k = cells[3 * q + 2];
    const size_t P = d.P(i, j, k);
    double a, b;
    shift_pair(free_slip, g.fu[d.FU(i - 1, j, k)], g.fu[d.FU(i, j, k)], uf[d.UF(i - 1, j, k)], uf[d.UF(i, j, k)], a,
               b);
    c[pos.p[0] * n + P] = a;
    c[pos.p[1] * n + P] = b;
    shift_pair(free_slip, g.fv[d.FV(i, j - 1, k)], g.fv[d.FV(i, j, k)], vf[d.VF(i, j - 1, k)], vf[d.VF(i, j, k)], a,
               b);
    c[pos.p[2] * n + P] = a;
    c[pos.p[3] * n + P] = b;
    shift_pair(free_slip, g.fw[d.FW(i, j, k - 1)], g.fw[d.FW(i, j, k)], wf[d.WF(i, j, k - 1)], wf[d.WF(i, j, k)], a,
               b);
    c[pos.p[4] * n + P] = a;
    c[pos.p[5] * n + P] = b;
  }
}

// VelCellToFaceComputeLR (ADVECT/VelocityCellFace_Mod.f90:1692-1722 interior,
// the 'iw'/'pw' neighbour branches :1384-1689 for periodic sides, and the
// outer-wall branches :1723-1892): one thread per face of uF, vF, wF.
__global__ void k_cell_to_face(Dims d, GeomT<double> g, Pos6 pos, BcKinds bc, const double* __restrict__ c,
                               double* __restrict__ uf, double* __restrict__ vf, double* __restrict__ wf) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t n = d.npad();
  const size_t nu = d.n_uf(), nv = d.n_vf(), nw = d.n_wf();
  const double e = kEps;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nu + nv + nw;
       q += (size_t)gridDim.x * blockDim.x) {
    if (q < nu) {
      const int i = (int)(q % (nx + 1)), j = (int)((q / (nx + 1)) % ny) + 1, k = (int)(q / ((size_t)(nx + 1) * ny)) + 1;
      double val;
      if ((i >= 1 && i <= nx - 1) || d.per_x) {
        const double F = g.fu[d.FU(i, j, k)];
        const double VR = g.volc[d.P(i + 1, j, k)] * F / (F + g.fu[d.FU(i + 1, j, k)] + e);
        const double VL = g.volc[d.P(i, j, k)] * F / (F + g.fu[d.FU(i - 1, j, k)] + e);
        val = (VR * c[pos.p[0] * n + d.P(i + 1, j, k)] + VL * c[pos.p[1] * n + d.P(i, j, k)]) / (VL + VR + e) * F /
              (F + e);
      } else if (i == 0) {
        val = bc.k[pos.p[0]][0] == kBcZeroGrad ? c[pos.p[0] * n + d.P(1, j, k)] : 0.0;
      } else {
        val = bc.k[pos.p[1]][1] == kBcZeroGrad ? c[pos.p[1] * n + d.P(nx, j, k)] : 0.0;
      }
      uf[q] = val;
    } else if (q < nu + nv) {
      const size_t r = q - nu;
      const int i = (int)(r % nx) + 1, j = (int)((r / nx) % (ny + 1)), k = (int)(r / ((size_t)nx * (ny + 1))) + 1;
      double val;
      if ((j >= 1 && j <= ny - 1) || d.per_y) {
        const double F = g.fv[d.FV(i, j, k)];
        const double VR = g.volc[d.P(i, j + 1, k)] * F / (F + g.fv[d.FV(i, j + 1, k)] + e);
        const double VL = g.volc[d.P(i, j, k)] * F / (F + g.fv[d.FV(i, j - 1, k)] + e);
        val = (VR * c[pos.p[2] * n + d.P(i, j + 1, k)] + VL * c[pos.p[3] * n + d.P(i, j, k)]) / (VL + VR + e) * F /
              (F + e);
      } else if (j == 0) {
        val = bc.k[pos.p[2]][2] == kBcZeroGrad ? c[pos.p[2] * n + d.P(i, 1, k)] : 0.0;
      } else {
        val = bc.k[pos.p[3]][3] == kBcZeroGrad ? c[pos.p[3] * n + d.P(i, ny, k)] : 0.0;
      }
      vf[r] = val;
    } else {
      const size_t r = q - nu - nv;
      const int i = (int)(r % nx) + 1, j = (int)((r / nx) % ny) + 1, k = (int)(r / ((size_t)nx * ny));
      double val;
      if ((k >= 1 && k <= nz - 1) || d.per_z) {
        const double F = g.fw[d.FW(i, j, k)];
        const double VR = g.volc[d.P(i, j, k + 1)] * F / (F + g.fw[d.FW(i, j, k + 1)] + e);
        const double VL = g.volc[d.P(i, j, k)] * F / (F + g.fw[d.FW(i, j, k - 1)] + e);
        val = (VR * c[pos.p[4] * n + d.P(i, j, k + 1)] + VL * c[pos.p[5] * n + d.P(i, j, k)]) / (VL + VR + e) * F /
              (F + e);
      } else if (k == 0) {
        val = bc.k[pos.p[4]][4] == kBcZeroGrad ? c[pos.p[4] * n + d.P(i, j, 1)] : 0.0;
      } else {
        val = bc.k[pos.p[5]][5] == kBcZeroGrad ? c[pos.p[5] * n + d.P(i, j, nz)] : 0.0;
      }
      wf[r] = val;
    }
  }
}

// AbsTCompute, ThetaKind='Density' (ADVECT/Diagnostic_Mod.f90:602-615), and
// the default branch of PreCompute (:805-811) over the padded box.  Absent
// moisture components (nullptr) are the reference's zero component.
__global__ void k_thermo(size_t n, const double* __restrict__ rho, const double* __restrict__ th,
                         const double* __restrict__ rv, const double* __restrict__ rc, const double* __restrict__ rr,
                         const double* __restrict__ ri, double* __restrict__ t, double* __restrict__ p) {
  const double e = kEps;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const double RhoLoc = rho[P];
    const double RhoVLoc = rv ? rv[P] : 0.0;
    const double rl = rc ? rc[P] : 0.0, rrr = rr ? rr[P] : 0.0;
    const double RhoLLoc = rl + rrr;
    const double RhoILoc = ri ? ri[P] : 0.0;
    const double RhoDLoc = RhoLoc - RhoVLoc - RhoLLoc - RhoILoc + e;
    const double Rm = kRd * RhoDLoc + kRv * RhoVLoc + e;
    const double Cpml = kCpd * RhoDLoc + kCpv * RhoVLoc + kCpl * RhoLLoc + kCpi * RhoILoc + e;
    const double KappaLoc = Rm / Cpml;
    const double T = pow(kRd * th[P] / pow(kP0, KappaLoc), 1.0 / (1.0 - KappaLoc)) / Rm + e;
    t[P] = T;
    p[P] = (kRd * (RhoLoc - rl - rrr) + (kRv - kRd) * RhoVLoc) * T;
  }
}

__global__ void k_axpy3(size_t n, double a, const double* __restrict__ x, double* __restrict__ u,
                        double* __restrict__ v, double* __restrict__ w, size_t nu, size_t nv) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    double* y = q < nu ? u + q : q < nu + nv ? v + (q - nu) : w + (q - nu - nv);
    *y = *y + a * x[q];
  }
}

Pos6 pos6(const DynState* s) {
  Pos6 p;
  for (int q = 0; q < 6; ++q) p.p[q] = s->cfg.mom_pos[q];
  return p;
}

const double* comp_of(const asam_ctx* h, const double* c, int pos) {
  return pos >= 0 ? c + (size_t)pos * h->npad : nullptr;
}

// VelocityFaceToCellLR into state-like c (device): faces -> momentum
// components, boundary-cell shift, ExchangeCell
void face_to_cell_dev(asam_ctx* h, const double* uf, const double* vf, const double* wf, double* c) {
  const Launch& L = h->L;
  const DynState* s = h->dyn;
  const Dims& d = h->d;
  k_face_to_cell<<<grid_of(L, (size_t)d.nx * d.ny * d.nz), kB, 0, L.stream>>>(d, pos6(s), uf, vf, wf, c);
  count_launches(1);
  if (s->nbound > 0) {
    k_shift_bound<<<grid_of(L, (size_t)s->nbound), kB, 0, L.stream>>>(d, h->geom(), pos6(s), s->bound, s->nbound,
                                                                      s->cfg.free_slip, uf, vf, wf, c);
    count_launches(1);
  }
  launch_exchange_cell(L, d, h->cfg.ncomp, c);
}

void cell_to_face_dev(asam_ctx* h, const double* c, double* uf, double* vf, double* wf) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  k_cell_to_face<<<grid_of(L, d.n_uf() + d.n_vf() + d.n_wf()), kB, 0, L.stream>>>(d, h->geom(), pos6(h->dyn), h->bc,
                                                                                   c, uf, vf, wf);
  count_launches(1);
}

// PrepareF's AbsTCompute + PreCompute with the outer-wall copies of the
// pressure (:816-862) and the ExchangeCell of both (ADVECT/Function_Mod.f90:252-263)
void thermo_dev(asam_ctx* h, const double* c, double* t, double* p) {
  const Launch& L = h->L;
  const DynState* s = h->dyn;
  const asam_dyn_config& k = s->cfg;
  k_thermo<<<grid_of(L, h->npad), kB, 0, L.stream>>>(h->npad, comp_of(h, c, h->cfg.rho_pos), comp_of(h, c, k.th_pos),
                                                      comp_of(h, c, k.rv_pos), comp_of(h, c, k.rc_pos),
                                                      comp_of(h, c, k.rr_pos), comp_of(h, c, k.ri_pos), t, p);
  count_launches(1);
  BcKinds zg{};
  for (int sd = 0; sd < 6; ++sd) zg.k[0][sd] = kBcZeroGrad;
  launch_bound_cond(L, h->d, 1, 0, zg, p);
  launch_exchange_cell(L, h->d, 1, p);
  launch_exchange_cell(L, h->d, 1, t);
}

// FcnMet with the momentum sources: advection of all components with the
// face coefficients of the context's velocity, then the gather with the
// pressure gradient (before AdvectionScale) and the buoyancy (after it).
void fcn_dyn_dev(asam_ctx* h, const double* c, const double* p, double* f) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const DynState* s = h->dyn;
  ProjGrid pg{};
  proj_grid(h, &pg);
  MomSrc<double> ms{};
  ms.p = p;
  ms.rho = c + (size_t)h->cfg.rho_pos * h->npad;
  ms.dx = pg.dx;
  ms.dy = pg.dy;
  ms.dz = pg.dz;
  ms.mxy = pg.mxy;
  ms.myx = pg.myx;
  for (int q = 0; q < 6; ++q) ms.pos[q] = s->cfg.mom_pos[q];
  ms.pgrad = s->cfg.pgradient;
  ms.buoy = s->cfg.buoyancy;
  ms.grav = s->cfg.grav;
  DiffSrc<double> tmp;
  const DiffSrc<double>* df = h->diff_src(tmp);
  if (h->cfg.precision == ASAM_PREC_FP32_REFINED) {  // contracted FP64, the refined mode's 1e-10 contract
    asam_fma::launch_fcn_mom(L, d, h->geom(), h->cfg.ncomp, h->cfg.rho_pos, c, h->coef_x, h->coef_y, h->coef_z,
                             h->mask_x, h->mask_y, h->mask_z, h->phi, h->gx, h->gy, h->gz, h->rvol, f, ms, df);
    return;
  }
  launch_phi(L, d, h->cfg.ncomp, h->cfg.rho_pos, c, h->phi);
  launch_face_flux(L, d, h->geom(), h->cfg.ncomp, h->coef_x, h->coef_y, h->coef_z, h->mask_x, h->mask_y, h->mask_z,
                   h->phi, h->gx, h->gy, h->gz);
  const int grid = grid_of(L, h->npad);
  const WallIn<double> wl{c, c + (size_t)h->cfg.rho_pos * h->npad};
  if (df)
    k_flux_gather<double, true, true><<<grid, kB, 0, L.stream>>>(d, h->geom(), h->cfg.ncomp, h->gx, h->gy, h->gz,
                                                                 h->rvol, f, ms, *df, wl);
  else
    k_flux_gather<double, true><<<grid, kB, 0, L.stream>>>(d, h->geom(), h->cfg.ncomp, h->gx, h->gy, h->gz, h->rvol,
                                                             f, ms, DiffSrc<double>{}, wl);
  count_launches(1);
}

int need_dyn(asam_ctx* h) {
  if (!h || !h->dyn || !h->proj) {
    set_last_error("call asam_proj_setup and asam_dyn_setup first", __FILE__, __LINE__);
    return kBadArg;
  }
  return kOk;
}

// Ros3MetC + StageRos of the dynamical core (ADVECT/Int_Mod.f90:1059-1122, 263-374)
int ros_step_dyn(asam_ctx* h, double* c, double dt, int* iters, double* resid, int* psteps, double* presid) {
  DynState* s = h->dyn;
  const Launch& L = h->L;
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  const size_t len = h->len, nu = s->nu, nv = s->nv, nw = s->nw, nf = nu + nv + nw;
  const asam_dyn_config& k = s->cfg;
  int status = kOk;
  CK(cudaMemcpyAsync(h->cold, c, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));  // VecMetOld
  CK(cudaMemcpyAsync(s->vold, h->uf, nu * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));  // VelFOld
  CK(cudaMemcpyAsync(s->vold + nu, h->vf, nv * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  CK(cudaMemcpyAsync(s->vold + nu + nv, h->wf, nw * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  for (int is = 0; is < h->nstage; ++is) {
    launch_exchange_cell(L, d, nc, c);
    face_to_cell_dev(h, h->uf, h->vf, h->wf, c);  // VelocityFaceToCellLR(VelF, VecMet)
    launch_bound_cond(L, d, nc, 0, h->bc, c);     // BoundaryVelocity + BoundaryCondition
    launch_face_coef(L, d, h->geom(), h->coef_x, h->coef_y, h->coef_z, h->mask_x, h->mask_y, h->mask_z);
    thermo_dev(h, c, s->tabs, s->pre);  // PrepareF
    int rc;
    if (is == 0) {
      if ((rc = jac_dev(h, c, dt))) return rc;
      // JacAccGrav: WeightDiagCompute with RhoV => Vec(RhoCPos)
      // (MULTI/JacAccGrav_Mod.f90:313-315), then LaplTFullCompute
      if ((rc = asam_proj_weights_density(h, c, k.th_pos, h->cfg.rho_pos, k.rc_pos, k.rc_pos, k.rr_pos, s->tabs)))
        return rc;
      if ((rc = asam_lapl_compute(h, h->beta0, dt))) return rc;
    }
    fcn_dyn_dev(h, c, s->pre, h->rhs);
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
    double* fu = s->incrf + (size_t)is * nf;
    double *fv = fu + nu, *fw = fv + nv;
    cell_to_face_dev(h, x, fu, fv, fw);  // VelocityCellToFaceLR(VecIncrMetC, VecIncrF)
    int ps = 0;
    double pr = 0.0;
    rc = asam_project_vel_face(h, fu, fv, fw, x, h->cold, k.th_pos, h->cfg.rho_pos, s->scalars.data(),
                               (int)s->scalars.size(), nullptr, &ps, &pr);
    if (rc != kOk && rc != kNotConverged) return rc;
    if (psteps) psteps[is] = ps;
    if (presid) presid[is] = pr;
    face_to_cell_dev(h, fu, fv, fw, x);  // VelocityFaceToCellLR(VecIncrF, VecIncrMetC)
    // VelF = VelFOld + sum_j alpha(is,j) VecIncrF(j)
    CK(cudaMemcpyAsync(h->uf, s->vold, nu * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    CK(cudaMemcpyAsync(h->vf, s->vold + nu, nv * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    CK(cudaMemcpyAsync(h->wf, s->vold + nu + nv, nw * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    for (int js = 0; js <= is; ++js) {
      k_axpy3<<<grid_of(L, nf), kB, 0, L.stream>>>(nf, h->alpha[is * 4 + js], s->incrf + (size_t)js * nf, h->uf,
                                                   h->vf, h->wf, nu, nv);
      count_launches(1);
    }
    launch_exchange_cell(L, d, nc, x);
    CK(cudaMemcpyAsync(c, h->cold, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    for (int js = 0; js <= is; ++js) launch_axpy_host(L, len, h->alpha[is * 4 + js], h->incr + (size_t)js * len, c);
  }
  // the transport operators of later calls see the new velocity
  launch_face_coef(L, d, h->geom(), h->coef_x, h->coef_y, h->coef_z, h->mask_x, h->mask_y, h->mask_z);
  h->jac_ready = false;
  int rc = check_launch();
  return rc ? rc : status;
}

}  // namespace dyn

void dyn_free(asam_ctx* h) {
  DynState* s = h->dyn;
  if (!s) return;
  double* p[] = {s->tabs, s->pre, s->vold, s->incrf, s->facef};
  for (double* q : p)
    if (q) cudaFree(q);
  if (s->bound) cudaFree(s->bound);
  delete s;
  h->dyn = nullptr;
}

}  // namespace asam

using namespace asam;
using namespace asam::dyn;

extern "C" {

int asam_dyn_setup(asam_ctx* h, const asam_dyn_config* cfg, const int* bound_cells, int nbound, const int* scalars,
                   int nscalar) {
  if (!h || !cfg || nbound < 0 || nscalar < 0 || (nbound > 0 && !bound_cells) || (nscalar > 0 && !scalars))
    return kBadArg;
  if (!h->proj) {
    set_last_error("asam_dyn_setup: call asam_proj_setup first", __FILE__, __LINE__);
    return kBadArg;
  }
  if (h->bc_open()) {  // BoundaryVelocity and the projection of open boundaries are not built
    set_last_error("asam_dyn_setup: the open-boundary wall rules are built for the transport stage only", __FILE__,
                   __LINE__);
    return kBadArg;
  }
  if (h->d.per_z) {  // the buoyancy's 'ib'/'it' neighbour terms are not built
    set_last_error("asam_dyn_setup: a block periodic in z is not supported by the dynamical core", __FILE__,
                   __LINE__);
    return kBadArg;
  }
  const int nc = h->cfg.ncomp;
  auto in = [&](int p) { return p >= 0 && p < nc; };
  auto opt = [&](int p) { return p == -1 || in(p); };
  bool ok = in(cfg->th_pos) && opt(cfg->rv_pos) && opt(cfg->rc_pos) && opt(cfg->rr_pos) && opt(cfg->ri_pos) &&
            cfg->th_pos != h->cfg.rho_pos;
  for (int q = 0; q < 6 && ok; ++q) {
    ok = in(cfg->mom_pos[q]) && cfg->mom_pos[q] != h->cfg.rho_pos && cfg->mom_pos[q] != cfg->th_pos;
    for (int r = 0; r < q && ok; ++r) ok = cfg->mom_pos[r] != cfg->mom_pos[q];
  }
  for (int q = 0; q < nscalar && ok; ++q) ok = in(scalars[q]);
  const Dims& d = h->d;
  for (int q = 0; q < nbound && ok; ++q) {
    const int i = bound_cells[3 * q], j = bound_cells[3 * q + 1], k = bound_cells[3 * q + 2];
    ok = i >= 1 && i <= d.nx && j >= 1 && j <= d.ny && k >= 1 && k <= d.nz;
  }
  if (!ok) {
    set_last_error("asam_dyn_setup: component position or boundary cell out of range", __FILE__, __LINE__);
    return kBadArg;
  }
  dyn_free(h);
  DynState* s = new DynState();
  h->dyn = s;
  s->cfg = *cfg;
  s->scalars.assign(scalars, scalars + nscalar);
  s->nu = d.n_uf();
  s->nv = d.n_vf();
  s->nw = d.n_wf();
  const size_t nf = s->nu + s->nv + s->nw;
  auto fail = [&](cudaError_t e) {
    set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    dyn_free(h);
    return (int)kCudaError;
  };
  cudaError_t e;
  struct A {
    double** p;
    size_t n;
  } al[] = {{&s->tabs, h->npad}, {&s->pre, h->npad}, {&s->vold, nf}, {&s->incrf, nf * h->nstage}, {&s->facef, nf}};
  for (auto& a : al) {
    if ((e = cudaMalloc((void**)a.p, a.n * sizeof(double))) != cudaSuccess) return fail(e);
    if ((e = cudaMemsetAsync(*a.p, 0, a.n * sizeof(double), h->L.stream)) != cudaSuccess) return fail(e);
  }
  s->nbound = nbound;
  if (nbound > 0) {
    if ((e = cudaMalloc((void**)&s->bound, (size_t)3 * nbound * sizeof(int))) != cudaSuccess) return fail(e);
    if ((e = cudaMemcpyAsync(s->bound, bound_cells, (size_t)3 * nbound * sizeof(int), cudaMemcpyHostToDevice,
                             h->L.stream)) != cudaSuccess)
      return fail(e);
  }
  // walls of the momentum components from BCVel (FreeSlip: the normal
  // components ZeroValue; NoSlip: all six ZeroValue), the rest ZeroGrad
  for (int q = 0; q < 6; ++q)
    for (int sd = 0; sd < 6; ++sd) {
      const bool normal = (q / 2) == (sd / 2);
      h->bc.k[cfg->mom_pos[q]][sd] = (normal || cfg->wall_no_slip) ? kBcZeroValue : kBcZeroGrad;
    }
  graphs_reset(h);
  if ((e = cudaStreamSynchronize(h->L.stream)) != cudaSuccess) return fail(e);
  return kOk;
}

int asam_face_to_cell(asam_ctx* h, const double* uf, const double* vf, const double* wf, double* c) {
  if (int rc = need_dyn(h)) return rc;
  if (!uf || !vf || !wf || !c) return kBadArg;
  DynState* s = h->dyn;
  const double *du, *dv, *dw;
  double* dc;
  int rc;
  if ((rc = stage_in(h, uf, s->nu, s->facef, &du)) || (rc = stage_in(h, vf, s->nv, s->facef + s->nu, &dv)) ||
      (rc = stage_in(h, wf, s->nw, s->facef + s->nu + s->nv, &dw)))
    return rc;
  if ((rc = stage_out_begin(h, c, h->len, h->stage_a, &dc, true))) return rc;
  face_to_cell_dev(h, du, dv, dw, dc);
  if ((rc = check_launch())) return rc;
  return stage_out_end(h, c, h->len, dc);
}

int asam_cell_to_face(asam_ctx* h, const double* c, double* uf, double* vf, double* wf) {
  if (int rc = need_dyn(h)) return rc;
  if (!uf || !vf || !wf || !c) return kBadArg;
  DynState* s = h->dyn;
  const double* dc;
  int rc;
  if ((rc = stage_in(h, c, h->len, h->stage_a, &dc))) return rc;
  cell_to_face_dev(h, dc, s->facef, s->facef + s->nu, s->facef + s->nu + s->nv);
  if ((rc = check_launch())) return rc;
  CK(cudaMemcpyAsync(uf, s->facef, s->nu * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaMemcpyAsync(vf, s->facef + s->nu, s->nv * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaMemcpyAsync(wf, s->facef + s->nu + s->nv, s->nw * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

int asam_thermo(asam_ctx* h, const double* c, double* tabs, double* pre) {
  if (int rc = need_dyn(h)) return rc;
  if (!c) return kBadArg;
  DynState* s = h->dyn;
  const double* dc;
  int rc;
  if ((rc = stage_in(h, c, h->len, h->stage_a, &dc))) return rc;
  thermo_dev(h, dc, s->tabs, s->pre);
  if ((rc = check_launch())) return rc;
  if (tabs) CK(cudaMemcpyAsync(tabs, s->tabs, h->npad * sizeof(double), cudaMemcpyDefault, h->L.stream));
  if (pre) CK(cudaMemcpyAsync(pre, s->pre, h->npad * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

int asam_fcn_dyn(asam_ctx* h, const double* c, const double* pre, double* f) {
  if (int rc = need_dyn(h)) return rc;
  if (!c || !pre || !f) return kBadArg;
  DynState* s = h->dyn;
  const double *dc, *dp;
  double* df;
  int rc;
  if ((rc = stage_in(h, c, h->len, h->stage_a, &dc))) return rc;
  if ((rc = stage_in(h, pre, h->npad, s->pre, &dp))) return rc;
  if ((rc = stage_out_begin(h, f, h->len, h->stage_b, &df, false))) return rc;
  fcn_dyn_dev(h, dc, dp, df);
  if ((rc = check_launch())) return rc;
  return stage_out_end(h, f, h->len, df);
}

int asam_ros_step_dyn(asam_ctx* h, double* c, double dt, int* iters, double* resid, int* psteps, double* presid) {
  if (int rc = need_dyn(h)) return rc;
  if (!c) return kBadArg;
  double* dc;
  int rc = stage_out_begin(h, c, h->len, h->c, &dc, true);
  if (rc) return rc;
  int st = ros_step_dyn(h, dc, dt, iters, resid, psteps, presid);
  if (st != kOk && st != kNotConverged && st != kBreakdown) return st;
  rc = stage_out_end(h, c, h->len, dc);
  return rc ? rc : st;
}

int asam_get_velocity(asam_ctx* h, double* uf, double* vf, double* wf) {
  if (!h || !uf || !vf || !wf) return kBadArg;
  const Dims& d = h->d;
  CK(cudaMemcpyAsync(uf, h->uf, d.n_uf() * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaMemcpyAsync(vf, h->vf, d.n_vf() * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaMemcpyAsync(wf, h->wf, d.n_wf() * sizeof(double), cudaMemcpyDefault, h->L.stream));
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

}  // extern "C"
