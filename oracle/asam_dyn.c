/*
 * CPU oracle of the dynamical-core stage of one block with closed or
 * periodic sides.
 *
 * TEST INFRASTRUCTURE ONLY.  The parity tests and the CPU-baseline leg of the
 * benchmark call it as the checker; the CUDA library never links or calls it.
 *
 * It restates, loop for loop and in the same floating-point operation order,
 * the momentum branch of the Rosenbrock stage of ASAM (OsKnoth/ASAM) with the
 * configuration's switches (GradFull, ThetaKind='Density', no Anelastic /
 * PseudoIn, no diffusion, cloud physics or Coriolis):
 *
 *   StageRos (uPosL>0)         ADVECT/Int_Mod.f90:263-374
 *   Ros3MetC (fixed dt)        ADVECT/Int_Mod.f90:1059-1122
 *   VelocityFaceToCellLR       ADVECT/VelocityCellFace_Mod.f90:72-95, 541-654
 *     ShiftVel1 / ShiftNoSlip  :820-909 (FreeSlip / no-slip boundary cells)
 *   VelocityCellToFaceLR       :27-52, 1369-1894 (closed and periodic sides)
 *   AbsTCompute 'Density'      ADVECT/Diagnostic_Mod.f90:593-615
 *   PreCompute (default)       :710-865
 *   PGradComputeCFull          ADVECT/PressureGrad_Mod.f90:245-276
 *   AuftriebDryComputeLRFull   ADVECT/Buoyancy_Mod.f90:43-63
 *   FcnMet                     ADVECT/Function_Mod.f90:989-1506 (advection,
 *                              diffusion, pressure gradient, AdvectionScale,
 *                              buoyancy)
 *   JacAccGrav, ProjectVelFace through the projection oracle (asam_proj.c)
 *
 * The BoundCell list of the grid (cells that hold a piece of the terrain
 * surface) is an input: triples (ix,iy,iz) of interior cells, 1-based.
 *
 * Build with -O2 -ffp-contract=off.  Parity with the Fortran binary itself is
 * unpinned (no Fortran compiler is available).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "asam_oracle.h"

/* MODULE/Parameter_Mod.f90:20-36 */
#define CPD 1004.0
#define CVD 717.0
#define RD (CPD - CVD)
#define CPV 1885.0
#define RV 461.0
#define CPL 4186.0
#define CPI 2110.0
#define P0 1.0e5

/* projection oracle (asam_proj.c) */
void ora_weights_density(void *hv, const double *rth, const double *rho, const double *rv, const double *rc,
                         const double *rr, const double *t, double *dtu, double *dtv, double *dtw, double *duu,
                         double *duv, double *duw, double *dut, double *dtt);
void ora_proj_set_weights(void *hv, const double *dtu, const double *dtv, const double *dtw, const double *duu,
                          const double *duv, const double *duw, const double *dut, const double *dtt);
void ora_lapl_compute(void *hv, double beta0, double dtp);
void ora_proj_rhs(void *hv, const double *u, const double *v, const double *w, const double *incr_th, double *b);
int ora_fgmres(void *hv, double *x, const double *b, int maxiter, double tol, int step, double *rho_out,
               double *rho0_out);
void ora_proj_update(void *hv, double *x, double *u, double *v, double *w, double *incr_th, double *incr_rho, int ncs,
                     double *const *incr_c, const double *const *c, const double *rho_pad);
long ora_proj_nvec(void *hv);

/* positions of the six LR momentum components: uL, uR, vL, vR, wL, wR */
typedef struct {
  int p[6];
} pos6;

static double *comp(double *c, const ora_geom *g, int pos) { return pos >= 0 ? c + (size_t)pos * NPAD(g) : NULL; }

/* ------------------------------------------------------------------ */
/* VelFaceToCellComputeLR (ADVECT/VelocityCellFace_Mod.f90:541-654): the
 * first assignment block of the loop is overwritten by the second, so every
 * interior cell takes the face values; then ShiftVel1 (FreeSlip, :820-855)
 * or ShiftNoSlip (:880-909) at the boundary cells.  The ExchangeCell of
 * VelocityFaceToCellLR (:94) follows. */
/* ------------------------------------------------------------------ */
void ora_face_to_cell(const ora_geom *g, int ncomp, const int *pos, const double *uf, const double *vf,
                      const double *wf, const int *bound, int nbound, int free_slip, double *c) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  double *uL = comp(c, g, pos[0]), *uR = comp(c, g, pos[1]), *vL = comp(c, g, pos[2]);
  double *vR = comp(c, g, pos[3]), *wL = comp(c, g, pos[4]), *wR = comp(c, g, pos[5]);
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j)
      for (int k = 1; k <= nz; ++k) {
        const size_t P = PIDX(g, i, j, k);
        uL[P] = uf[UFI(g, i - 1, j, k)];
        uR[P] = uf[UFI(g, i, j, k)];
        vL[P] = vf[VFI(g, i, j - 1, k)];
        vR[P] = vf[VFI(g, i, j, k)];
        wL[P] = wf[WFI(g, i, j, k - 1)];
        wR[P] = wf[WFI(g, i, j, k)];
      }
  for (int q = 0; q < nbound; ++q) {
    const int i = bound[3 * q], j = bound[3 * q + 1], k = bound[3 * q + 2];
    const size_t P = PIDX(g, i, j, k);
    const double FUL = g->fu[FUI(g, i - 1, j, k)], FUR = g->fu[FUI(g, i, j, k)];
    const double FVL = g->fv[FVI(g, i, j - 1, k)], FVR = g->fv[FVI(g, i, j, k)];
    const double FWL = g->fw[FWI(g, i, j, k - 1)], FWR = g->fw[FWI(g, i, j, k)];
    const double ul = uf[UFI(g, i - 1, j, k)], ur = uf[UFI(g, i, j, k)];
    const double vl = vf[VFI(g, i, j - 1, k)], vr = vf[VFI(g, i, j, k)];
    const double wl = wf[WFI(g, i, j, k - 1)], wr = wf[WFI(g, i, j, k)];
    if (free_slip) {
      if (FUL > FUR) {
        uL[P] = ul;
        uR[P] = (FUR * ur + (FUL - FUR) * ul) / (FUL + EPS);
      } else {
        uL[P] = (FUL * ul + (FUR - FUL) * ur) / (FUR + EPS);
        uR[P] = ur;
      }
      if (FVL > FVR) {
        vL[P] = vl;
        vR[P] = (FVR * vr + (FVL - FVR) * vl) / (FVL + EPS);
      } else {
        vL[P] = (FVL * vl + (FVR - FVL) * vr) / (FVR + EPS);
        vR[P] = vr;
      }
      if (FWL > FWR) {
        wL[P] = wl;
        wR[P] = (FWR * wr + (FWL - FWR) * wl) / (FWL + EPS);
      } else {
        wL[P] = (FWL * wl + (FWR - FWL) * wr) / (FWR + EPS);
        wR[P] = wr;
      }
    } else {
      const double mu = FUR > FUL ? FUR : FUL, mv = FVR > FVL ? FVR : FVL, mw = FWR > FWL ? FWR : FWL;
      uL[P] = FUL * ul / mu;
      uR[P] = FUR * ur / mu;
      vL[P] = FVL * vl / mv;
      vR[P] = FVR * vr / mv;
      wL[P] = FWL * wl / mw;
      wR[P] = FWR * wr / mw;
    }
  }
  ora_exchange_cell(g, ncomp, c);
}

/* ------------------------------------------------------------------ */
/* VelCellToFaceComputeLR (ADVECT/VelocityCellFace_Mod.f90:1369-1894):
 * volume-weighted faces from the LR cell values; a periodic side uses the
 * same formula with the exchanged halo cells (the 'iw'/'pw' neighbour
 * branches, :1384-1689); an outer wall ('o', :1723-1892) takes the adjacent
 * cell value where the normal component's rule is ZeroGrad and 0 otherwise.
 * bc: the halo rules of the state's components (may be NULL: ZeroGrad). */
/* ------------------------------------------------------------------ */
void ora_cell_to_face(const ora_geom *g, const int *pos, const double *c, double *uf, double *vf, double *wf) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const double *V = g->volc;
  double *cc = (double *)c;
  const double *uL = comp(cc, g, pos[0]), *uR = comp(cc, g, pos[1]), *vL = comp(cc, g, pos[2]);
  const double *vR = comp(cc, g, pos[3]), *wL = comp(cc, g, pos[4]), *wR = comp(cc, g, pos[5]);
#define KIND(ic, side) (g->bc ? g->bc[6 * (ic) + (side)] : 1)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        double val;
        if ((i >= 1 && i <= nx - 1) || g->per_x) {
          const double F = g->fu[FUI(g, i, j, k)];
          const double VR = V[PIDX(g, i + 1, j, k)] * F / (F + g->fu[FUI(g, i + 1, j, k)] + EPS);
          const double VL = V[PIDX(g, i, j, k)] * F / (F + g->fu[FUI(g, i - 1, j, k)] + EPS);
          val = (VR * uL[PIDX(g, i + 1, j, k)] + VL * uR[PIDX(g, i, j, k)]) / (VL + VR + EPS) * F / (F + EPS);
        } else if (i == 0) {
          val = KIND(pos[0], 0) == 1 ? uL[PIDX(g, 1, j, k)] : 0.0;
        } else {
          val = KIND(pos[1], 1) == 1 ? uR[PIDX(g, nx, j, k)] : 0.0;
        }
        uf[UFI(g, i, j, k)] = val;
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double val;
        if ((j >= 1 && j <= ny - 1) || g->per_y) {
          const double F = g->fv[FVI(g, i, j, k)];
          const double VR = V[PIDX(g, i, j + 1, k)] * F / (F + g->fv[FVI(g, i, j + 1, k)] + EPS);
          const double VL = V[PIDX(g, i, j, k)] * F / (F + g->fv[FVI(g, i, j - 1, k)] + EPS);
          val = (VR * vL[PIDX(g, i, j + 1, k)] + VL * vR[PIDX(g, i, j, k)]) / (VL + VR + EPS) * F / (F + EPS);
        } else if (j == 0) {
          val = KIND(pos[2], 2) == 1 ? vL[PIDX(g, i, 1, k)] : 0.0;
        } else {
          val = KIND(pos[3], 3) == 1 ? vR[PIDX(g, i, ny, k)] : 0.0;
        }
        vf[VFI(g, i, j, k)] = val;
      }
  for (int k = 0; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double val;
        if ((k >= 1 && k <= nz - 1) || g->per_z) {
          const double F = g->fw[FWI(g, i, j, k)];
          const double VR = V[PIDX(g, i, j, k + 1)] * F / (F + g->fw[FWI(g, i, j, k + 1)] + EPS);
          const double VL = V[PIDX(g, i, j, k)] * F / (F + g->fw[FWI(g, i, j, k - 1)] + EPS);
          val = (VR * wL[PIDX(g, i, j, k + 1)] + VL * wR[PIDX(g, i, j, k)]) / (VL + VR + EPS) * F / (F + EPS);
        } else if (k == 0) {
          val = KIND(pos[4], 4) == 1 ? wL[PIDX(g, i, j, 1)] : 0.0;
        } else {
          val = KIND(pos[5], 5) == 1 ? wR[PIDX(g, i, j, nz)] : 0.0;
        }
        wf[WFI(g, i, j, k)] = val;
      }
#undef KIND
}

/* ------------------------------------------------------------------ */
/* AbsTCompute, ThetaKind='Density' (ADVECT/Diagnostic_Mod.f90:602-615), and
 * the default branch of PreCompute (:805-811) over the padded box, then the
 * outer-wall copies of PreCompute (:816-862) and the ExchangeCell of PreCell
 * and TAbsCell in PrepareF (ADVECT/Function_Mod.f90:252-263).  th is rho
 * theta; absent moisture components (NULL) are the zero component. */
/* ------------------------------------------------------------------ */
void ora_thermo(const ora_geom *g, const double *rho, const double *th, const double *rv, const double *rc,
                const double *rr, const double *ri, double *t, double *p) {
  const size_t n = NPAD(g);
  for (size_t P = 0; P < n; ++P) {
    const double RhoLoc = rho[P];
    const double RhoVLoc = rv ? rv[P] : 0.0;
    const double rl = rc ? rc[P] : 0.0, rrr = rr ? rr[P] : 0.0;
    const double RhoLLoc = rl + rrr;
    const double RhoILoc = ri ? ri[P] : 0.0;
    const double RhoDLoc = RhoLoc - RhoVLoc - RhoLLoc - RhoILoc + EPS;
    const double Rm = RD * RhoDLoc + RV * RhoVLoc + EPS;
    const double Cpml = CPD * RhoDLoc + CPV * RhoVLoc + CPL * RhoLLoc + CPI * RhoILoc + EPS;
    const double KappaLoc = Rm / Cpml;
    t[P] = pow(RD * th[P] / pow(P0, KappaLoc), 1.0 / (1.0 - KappaLoc)) / Rm + EPS;
    p[P] = (RD * (rho[P] - rl - rrr) + (RV - RD) * RhoVLoc) * t[P];
  }
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  if (!g->per_x)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        p[PIDX(g, 0, j, k)] = p[PIDX(g, 1, j, k)];
        p[PIDX(g, nx + 1, j, k)] = p[PIDX(g, nx, j, k)];
      }
  if (!g->per_y)
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        p[PIDX(g, i, 0, k)] = p[PIDX(g, i, 1, k)];
        p[PIDX(g, i, ny + 1, k)] = p[PIDX(g, i, ny, k)];
      }
  if (!g->per_z)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        p[PIDX(g, i, j, 0)] = p[PIDX(g, i, j, 1)];
        p[PIDX(g, i, j, nz + 1)] = p[PIDX(g, i, j, nz)];
      }
  ora_exchange_cell(g, 1, p);
  ora_exchange_cell(g, 1, t);
}

/* ------------------------------------------------------------------ */
/* FcnMet with the momentum sources (ADVECT/Function_Mod.f90:989-1506):
 * advection of every component, PGradComputeCFull (:1267-1297,
 * ADVECT/PressureGrad_Mod.f90:252-276 with DUU = F/(F+Eps),
 * MULTI/JacAccGrav_Mod.f90:297), ExchangeFlux, AdvectionScale, then
 * AuftriebDryComputeLRFull on wL/wR (:1389-1393, ADVECT/Buoyancy_Mod.f90:51-63).
 * p: padded pressure; dx[nx], dy[ny], dz[nz]; mxy = MetrXY[ny], myx =
 * MetrYX[nx]. */
/* ------------------------------------------------------------------ */
void ora_fcn_dyn(const ora_geom *g, int ncomp, int rho_pos, const int *pos, int pgrad, int buoy, double grav,
                 const double *c, const double *uf, const double *vf, const double *wf, const double *p,
                 const double *dx, const double *dy, const double *dz, const double *mxy, const double *myx,
                 double *f) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = NPAD(g);
  const double *V = g->volc;
  memset(f, 0, sizeof(double) * n * (size_t)ncomp);
  const double *rho = c + (size_t)rho_pos * n;
  for (int ic = 0; ic < ncomp; ++ic) ora_advection(g, c + ic * n, rho, uf, vf, wf, f + ic * n);
  ora_diffusion(g, ncomp, rho_pos, c, f); /* Function_Mod.f90:1106-1239 (no-op without coefficients) */
  if (pgrad) {
    double *uRhsL = comp(f, g, pos[0]), *uRhsR = comp(f, g, pos[1]), *vRhsL = comp(f, g, pos[2]);
    double *vRhsR = comp(f, g, pos[3]), *wRhsL = comp(f, g, pos[4]), *wRhsR = comp(f, g, pos[5]);
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx - 1; ++i) {
          const double F = g->fu[FUI(g, i, j, k)];
          const double DUU = F / (F + EPS);
          const double Grad = DUU * F / (F + EPS) * (p[PIDX(g, i + 1, j, k)] - p[PIDX(g, i, j, k)]) /
                              (mxy[j - 1] * (dx[i] + dx[i - 1] + EPS));
          uRhsL[PIDX(g, i + 1, j, k)] = uRhsL[PIDX(g, i + 1, j, k)] - 2.0 * V[PIDX(g, i + 1, j, k)] * Grad;
          uRhsR[PIDX(g, i, j, k)] = uRhsR[PIDX(g, i, j, k)] - 2.0 * V[PIDX(g, i, j, k)] * Grad;
        }
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny - 1; ++j)
        for (int i = 1; i <= nx; ++i) {
          const double F = g->fv[FVI(g, i, j, k)];
          const double DUV = F / (F + EPS);
          const double Grad = DUV * F / (F + EPS) * (p[PIDX(g, i, j + 1, k)] - p[PIDX(g, i, j, k)]) /
                              (myx[i - 1] * (dy[j] + dy[j - 1] + EPS));
          vRhsL[PIDX(g, i, j + 1, k)] = vRhsL[PIDX(g, i, j + 1, k)] - 2.0 * V[PIDX(g, i, j + 1, k)] * Grad;
          vRhsR[PIDX(g, i, j, k)] = vRhsR[PIDX(g, i, j, k)] - 2.0 * V[PIDX(g, i, j, k)] * Grad;
        }
    for (int k = 1; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const double F = g->fw[FWI(g, i, j, k)];
          const double DUW = F / (F + EPS);
          const double Grad =
              DUW * F / (F + EPS) * (p[PIDX(g, i, j, k + 1)] - p[PIDX(g, i, j, k)]) / (dz[k] + dz[k - 1] + EPS);
          wRhsL[PIDX(g, i, j, k + 1)] = wRhsL[PIDX(g, i, j, k + 1)] - 2.0 * V[PIDX(g, i, j, k + 1)] * Grad;
          wRhsR[PIDX(g, i, j, k)] = wRhsR[PIDX(g, i, j, k)] - 2.0 * V[PIDX(g, i, j, k)] * Grad;
        }
    /* the periodic sides: the neighbour loop of PGradComputeCFull
     * ('iw'/'ie'/'is'/'in' with equal refinement, PressureGrad_Mod.f90:307-313,
     * 340-346, 373-379, 406-412): no DUU factor, and the partner cell's width dLoc (the last
     * cell of the block for 'iw', the first for 'ie', ReadWeights_Mod.f90:
     * 903-960) in the denominator */
    if (g->per_x)
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) {
          const double FW0 = g->fu[FUI(g, 0, j, k)], FE0 = g->fu[FUI(g, nx, j, k)];
          const double GW = FW0 / (FW0 + EPS) * (p[PIDX(g, 1, j, k)] - p[PIDX(g, 0, j, k)]) /
                            (mxy[j - 1] * (dx[0] + dx[nx - 1] + EPS));
          uRhsL[PIDX(g, 1, j, k)] = uRhsL[PIDX(g, 1, j, k)] - 2.0 * V[PIDX(g, 1, j, k)] * GW;
          const double GE = FE0 / (FE0 + EPS) * (p[PIDX(g, nx + 1, j, k)] - p[PIDX(g, nx, j, k)]) /
                            (mxy[j - 1] * (dx[nx - 1] + dx[0] + EPS));
          uRhsR[PIDX(g, nx, j, k)] = uRhsR[PIDX(g, nx, j, k)] - 2.0 * V[PIDX(g, nx, j, k)] * GE;
        }
    if (g->per_y)
      for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
          const double FS0 = g->fv[FVI(g, i, 0, k)], FN0 = g->fv[FVI(g, i, ny, k)];
          const double GS = FS0 / (FS0 + EPS) * (p[PIDX(g, i, 1, k)] - p[PIDX(g, i, 0, k)]) /
                            (myx[i - 1] * (dy[0] + dy[ny - 1] + EPS));
          vRhsL[PIDX(g, i, 1, k)] = vRhsL[PIDX(g, i, 1, k)] - 2.0 * V[PIDX(g, i, 1, k)] * GS;
          const double GN = FN0 / (FN0 + EPS) * (p[PIDX(g, i, ny + 1, k)] - p[PIDX(g, i, ny, k)]) /
                            (myx[i - 1] * (dy[0] + dy[ny - 1] + EPS));
          vRhsR[PIDX(g, i, ny, k)] = vRhsR[PIDX(g, i, ny, k)] - 2.0 * V[PIDX(g, i, ny, k)] * GN;
        }
  }
  ora_exchange_flux(g, ncomp, f);
  for (int ic = 0; ic < ncomp; ++ic) {
    double *a = f + ic * n;
    for (size_t P = 0; P < n; ++P) a[P] = a[P] / (V[P] + EPS);
  }
  if (buoy) {
    double *fL = comp(f, g, pos[4]), *fR = comp(f, g, pos[5]);
    for (int k = 1; k <= nz - 1; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const double F = g->fw[FWI(g, i, j, k)];
          const double RhoLoc = F / (F + EPS) * (dz[k - 1] * rho[PIDX(g, i, j, k)] + dz[k] * rho[PIDX(g, i, j, k + 1)]) /
                                (dz[k - 1] + dz[k] + EPS);
          fL[PIDX(g, i, j, k + 1)] = fL[PIDX(g, i, j, k + 1)] - RhoLoc * grav;
          fR[PIDX(g, i, j, k)] = fR[PIDX(g, i, j, k)] - RhoLoc * grav;
        }
  }
}

/* ------------------------------------------------------------------ */
/* One Rosenbrock step of the dynamical core of one block
 * (Ros3MetC + StageRos with uPosL>0, ADVECT/Int_Mod.f90:1059-1122, 263-374).
 * c: state (ncomp padded fields, in/out); uf, vf, wf: face velocities VelF
 * (in/out).  proj: the projection oracle of this block (ora_proj_create).
 * ipar: ncomp, rho_pos, th_pos, rv_pos, rc_pos, rr_pos, ri_pos, uL, uR, vL,
 *       vR, wL, wR, pgradient, buoyancy, free_slip, method, bicg_maxiter,
 *       iterg, proj_maxiter, proj_step
 * dpar: grav, bicg_tol, proj_tol
 * Outputs per stage: BiCGStab MaxIter/Tol and FGMRES steps / relative residual. */
/* ------------------------------------------------------------------ */
int ora_ros_step_dyn(const ora_geom *g, void *proj, const int *ipar, const double *dpar, double *c, double *uf,
                     double *vf, double *wf, const double *dx, const double *dy, const double *dz, const double *mxy,
                     const double *myx, const int *bound, int nbound, const int *scalars, int nscalar, double dt,
                     int *iters, double *resid, int *psteps, double *presid) {
  const int ncomp = ipar[0], rho_pos = ipar[1], th_pos = ipar[2];
  const int rv_pos = ipar[3], rc_pos = ipar[4], rr_pos = ipar[5], ri_pos = ipar[6];
  const int *pos = ipar + 7;
  const int pgrad = ipar[13], buoy = ipar[14], free_slip = ipar[15], method = ipar[16];
  const int bicg_maxiter = ipar[17], iterg = ipar[18], proj_maxiter = ipar[19], proj_step = ipar[20];
  const double grav = dpar[0], bicg_tol = dpar[1], proj_tol = dpar[2];
  double beta0, alpha[16], beta[16], gamma1[5];
  const int nStage = ora_ros_coeffs(method, &beta0, alpha, beta, gamma1);
  if (nStage <= 0) return -1;
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = NPAD(g), len = n * (size_t)ncomp, nc = (size_t)nx * ny * nz;
  const size_t nu = (size_t)(nx + 1) * ny * nz, nv = (size_t)nx * (ny + 1) * nz, nw = (size_t)nx * ny * (nz + 1);
  const size_t nf = nu + nv + nw;
  double *cold = (double *)malloc(sizeof(double) * len);
  double *rhs = (double *)malloc(sizeof(double) * len);
  double *incr = (double *)calloc(len * (size_t)nStage, sizeof(double));
  double *incrf = (double *)calloc(nf * (size_t)nStage, sizeof(double));
  double *vold = (double *)malloc(sizeof(double) * nf);
  double *val = (double *)malloc(sizeof(double) * 7 * n);
  double *t = (double *)malloc(sizeof(double) * n);
  double *p = (double *)malloc(sizeof(double) * n);
  double *w8 = (double *)malloc(sizeof(double) * (3 * nu + 3 * nv + 3 * nw + 2 * nc));
  const size_t nvec = (size_t)ora_proj_nvec(proj); /* pressure + boundary face unknowns */
  double *xp = (double *)malloc(sizeof(double) * nvec), *bp = (double *)malloc(sizeof(double) * nvec);
  double **ic_ptr = (double **)malloc(sizeof(double *) * (nscalar > 0 ? nscalar : 1));
  const double **c_ptr = (const double **)malloc(sizeof(double *) * (nscalar > 0 ? nscalar : 1));
  memcpy(cold, c, sizeof(double) * len); /* Copy(VecMet,VecMetOld) */
  memcpy(vold, uf, sizeof(double) * nu); /* Copy(VelF,VelFOld) */
  memcpy(vold + nu, vf, sizeof(double) * nv);
  memcpy(vold + nu + nv, wf, sizeof(double) * nw);
  for (int is = 0; is < nStage; ++is) {
    ora_exchange_cell(g, ncomp, c);
    ora_face_to_cell(g, ncomp, pos, uf, vf, wf, bound, nbound, free_slip, c);
    ora_bound_cond(g, ncomp, 0, c); /* BoundaryVelocity + BoundaryCondition */
    ora_thermo(g, c + (size_t)rho_pos * n, c + (size_t)th_pos * n, comp(c, g, rv_pos), comp(c, g, rc_pos),
               comp(c, g, rr_pos), comp(c, g, ri_pos), t, p); /* PrepareF */
    if (is == 0) {
      ora_jac(g, c + (size_t)rho_pos * n, uf, vf, wf, beta0, dt, val);
      /* JacAccGrav: WeightDiagCompute with RhoV => Vec(RhoCPos)
       * (MULTI/JacAccGrav_Mod.f90:313-315), then LaplTFullCompute */
      double *W = w8;
      double *dtu = W, *duu = W + nu, *dtv = W + 2 * nu, *duv = W + 2 * nu + nv, *dtw = W + 2 * nu + 2 * nv;
      double *duw = dtw + nw, *dut = duw + nw, *dtt = dut + nc;
      ora_weights_density(proj, c + (size_t)th_pos * n, c + (size_t)rho_pos * n, comp(c, g, rc_pos),
                          comp(c, g, rc_pos), comp(c, g, rr_pos), t, dtu, dtv, dtw, duu, duv, duw, dut, dtt);
      ora_proj_set_weights(proj, dtu, dtv, dtw, duu, duv, duw, dut, dtt);
      ora_lapl_compute(proj, beta0, dt);
    }
    ora_fcn_dyn(g, ncomp, rho_pos, pos, pgrad, buoy, grav, c, uf, vf, wf, p, dx, dy, dz, mxy, myx, rhs);
    for (size_t q = 0; q < len; ++q) rhs[q] = dt * rhs[q]; /* ScaleV */
    for (int js = 0; js < is; ++js) {
      const double b = beta[is * 4 + js];
      const double *k = incr + (size_t)js * len;
      for (size_t q = 0; q < len; ++q) rhs[q] = rhs[q] + b * k[q];
    }
    double *x = incr + (size_t)is * len;
    memset(x, 0, sizeof(double) * len);
    int it = bicg_maxiter;
    double tol = bicg_tol;
    ora_bicgstab(g, ncomp, val, x, rhs, &it, &tol, iterg);
    if (iters) iters[is] = it;
    if (resid) resid[is] = tol;
    ora_exchange_cell(g, ncomp, x);
    double *fu = incrf + (size_t)is * nf, *fv = fu + nu, *fw = fv + nv;
    ora_cell_to_face(g, pos, x, fu, fv, fw); /* VelocityCellToFaceLR */
    /* ProjectVelFace(dt, VecIncrF, VecIncrMetC, VecMetOld) */
    ora_proj_rhs(proj, fu, fv, fw, x + (size_t)th_pos * n, bp);
    memset(xp, 0, sizeof(double) * nvec);
    double rr = 0.0, rr0 = 0.0;
    const int steps = ora_fgmres(proj, xp, bp, proj_maxiter, proj_tol, proj_step, &rr, &rr0);
    if (psteps) psteps[is] = steps;
    if (presid) presid[is] = rr0 > 0.0 ? rr / rr0 : 0.0;
    for (int q = 0; q < nscalar; ++q) {
      ic_ptr[q] = x + (size_t)scalars[q] * n;
      c_ptr[q] = cold + (size_t)scalars[q] * n;
    }
    ora_proj_update(proj, xp, fu, fv, fw, x + (size_t)th_pos * n, x + (size_t)rho_pos * n, nscalar, ic_ptr, c_ptr,
                    cold + (size_t)rho_pos * n);
    ora_face_to_cell(g, ncomp, pos, fu, fv, fw, bound, nbound, free_slip, x); /* VelocityFaceToCellLR */
    /* VelF = VelFOld + sum alpha VecIncrF */
    memcpy(uf, vold, sizeof(double) * nu);
    memcpy(vf, vold + nu, sizeof(double) * nv);
    memcpy(wf, vold + nu + nv, sizeof(double) * nw);
    for (int js = 0; js <= is; ++js) {
      const double a = alpha[is * 4 + js];
      const double *k = incrf + (size_t)js * nf;
      for (size_t q = 0; q < nu; ++q) uf[q] = uf[q] + a * k[q];
      for (size_t q = 0; q < nv; ++q) vf[q] = vf[q] + a * k[nu + q];
      for (size_t q = 0; q < nw; ++q) wf[q] = wf[q] + a * k[nu + nv + q];
    }
    ora_exchange_cell(g, ncomp, x);
    memcpy(c, cold, sizeof(double) * len);
    for (int js = 0; js <= is; ++js) {
      const double a = alpha[is * 4 + js];
      const double *k = incr + (size_t)js * len;
      for (size_t q = 0; q < len; ++q) c[q] = c[q] + a * k[q];
    }
  }
  free(cold); free(rhs); free(incr); free(incrf); free(vold); free(val); free(t); free(p); free(w8);
  free(xp); free(bp); free(ic_ptr); free(c_ptr);
  return nStage;
}
