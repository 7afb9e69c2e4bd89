/*
 * CPU oracle for the ASAM implicit Rosenbrock transport stage.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it.  The
 * product (the CUDA library) never links or calls it.
 *
 * It restates, loop for loop and in the same floating-point operation order,
 * the Fortran routines of ASAM (OsKnoth/ASAM) that make up the transport
 * part of one Rosenbrock stage.  Every function cites the routine it follows
 * (paths relative to the ASAM source tree).  The reference itself cannot be
 * compiled here (Fortran + MPI + MUMPS), so this restatement is the oracle;
 * parity with the Fortran binary is unpinned and the restatement is checked
 * against analytic known answers and an independent Python restatement.
 *
 * Conventions (identical to the Fortran memory layout, 0-based):
 *   padded cell (i,j,k), i in [0,nx+1] (0 = ix0 halo), j in [0,ny+1],
 *   k in [0,nz+1]:  P = i + NX*(j + NY*k),  NX=nx+2, NY=ny+2, NZ=nz+2.
 *   FU(ix0-1:ix1+1, iy0+1:iy1, iz0+1:iz1)  -> fu[(i+1) + (nx+3)*((j-1) + ny*(k-1))]
 *   FV(ix0+1:ix1, iy0-1:iy1+1, iz0+1:iz1)  -> fv[(i-1) + nx*((j+1) + (ny+3)*(k-1))]
 *   FW(ix0+1:ix1, iy0+1:iy1, iz0-1:iz1+1)  -> fw[(i-1) + nx*((j-1) + ny*(k+1))]
 *   uF(ix0:ix1, iy0+1:iy1, iz0+1:iz1)      -> uf[i + (nx+1)*((j-1) + ny*(k-1))]
 *   vF(ix0+1:ix1, iy0:iy1, iz0+1:iz1)      -> vf[(i-1) + nx*(j + (ny+1)*(k-1))]
 *   wF(ix0+1:ix1, iy0+1:iy1, iz0:iz1)      -> wf[(i-1) + nx*((j-1) + ny*k)]
 *   DIA matrix Val(m,7) column-major -> val[d*m + P], offsets of
 *   MODULE/Vector4Cell_Mod.f90:1030-1036.
 *
 * Boundary handling covered: periodic sides ('iw'/'ie'/'is'/'in' neighbours
 * that are the block itself) and outer walls ('ow'...'ot'), closed or with
 * flow through them (the first-order inflow of AdvectionComputeP and the
 * outflow term of JacAdvectionCompute), whose halo cells the stage driver
 * sets with the rules of BoundaryCompute (ZeroGrad, ZeroValue, MeanValue,
 * Function, InFlowOutFlow, Extrapolation).  Refined-neighbour branches are
 * not restated.
 *
 * Build with -O2 -ffp-contract=off (no FMA contraction, like gfortran on
 * x86-64 without -march).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "asam_oracle.h"

/* ------------------------------------------------------------------ */
/* Halo exchange for a single periodic block:                          */
/* MODULE/Vector4CellPar_Mod.f90:611-659 RandCopyCell_VecCell (EqualEqual
 * copy of MODULE/Exchange_Mod.f90:501) -- face halos, interior tangential
 * ranges only.                                                          */
/* ------------------------------------------------------------------ */
void ora_exchange_cell(const ora_geom *g, int ncomp, double *c) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = NPAD(g);
  for (int ic = 0; ic < ncomp; ++ic) {
    double *a = c + ic * n;
    if (g->per_x)
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) {
          a[PIDX(g, 0, j, k)] = a[PIDX(g, nx, j, k)];
          a[PIDX(g, nx + 1, j, k)] = a[PIDX(g, 1, j, k)];
        }
    if (g->per_y)
      for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
          a[PIDX(g, i, 0, k)] = a[PIDX(g, i, ny, k)];
          a[PIDX(g, i, ny + 1, k)] = a[PIDX(g, i, 1, k)];
        }
    if (g->per_z)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          a[PIDX(g, i, j, 0)] = a[PIDX(g, i, j, nz)];
          a[PIDX(g, i, j, nz + 1)] = a[PIDX(g, i, j, 1)];
        }
  }
}

/* ------------------------------------------------------------------ */
/* Halo rule of the outer walls at the start of a stage, BoundaryCondition /
 * BoundaryCompute (ADVECT/BoundaryCondition_Mod.f90:1143-1221, 70-346) and
 * BoundaryVelocityCellCompute (:424-970) for the ZeroGrad and ZeroValue
 * kinds: face halos of the non-periodic sides, tangential interior ranges.
 * Kinds of BoundaryCompute beyond those, per component and side in the order
 * W, E, S, N, B, T (a side without the kind's branch leaves its halo alone):
 *   3 MeanValue      halo = 2*MeanProfile(ic,iz) - interior; the bottom and
 *                    top take the profile's first and last level (:102-107)
 *   4 Function       halo = 2*F - interior, F the caller's value of Val
 *                    (RhoFun*Val for the non-number components) at the halo
 *                    cell (:108-120)
 *   5 InFlowOutFlow  W/E/S/N only: inflow (uF(ix0) >= 0 on the west,
 *                    uF(ix1) <= 0 on the east, vF likewise) halo =
 *                    Rho(halo)*VecAmb(halo), else the interior value (:86-95)
 *   6 Extrapolation  B/T only: halo = 2*c(iz0+1) - c(iz0+2) (:276-281)
 * Components are processed in order, so the density halo an InFlowOutFlow
 * rule reads is already updated for the components after the density.
 * comp0 is the index of the first of the ncomp fields in g->bc. */
/* ------------------------------------------------------------------ */
static int bc_kind(const ora_geom *g, int ic, int side) { return g->bc ? g->bc[6 * ic + side] : 1; }
typedef struct {
  const ora_geom *g;
  const double *uf, *vf, *rho;
  size_t n;
  int q; /* component index in g->bc and the data arrays */
} bc_ctx;
/* one halo cell h from its interior neighbour src (src2 the next one inward);
 * side 0-5, level iz of the profile, vel the InFlowOutFlow face velocity */
static void bc_set(const bc_ctx *x, double *a, size_t h, size_t src, size_t src2, int side, int iz, double vel) {
  const ora_geom *g = x->g;
  const int kind = bc_kind(g, x->q, side);
  if (kind == 1) a[h] = a[src];
  else if (kind == 2) a[h] = -a[src];
  else if (kind == 3) a[h] = 2.0 * g->bc_mean[(size_t)x->q * g->nz + (size_t)(iz - 1)] - a[src];
  else if (kind == 4) a[h] = 2.0 * g->bc_fval[(size_t)x->q * x->n + h] - a[src];
  else if (kind == 5 && side < 4) {
    const int in = (side & 1) ? vel <= 0.0 : vel >= 0.0;
    a[h] = in ? x->rho[h] * g->bc_amb[(size_t)x->q * x->n + h] : a[src];
  } else if (kind == 6 && side >= 4) a[h] = 2.0 * a[src] - a[src2];
}
static void bound_cond(const ora_geom *g, int ncomp, int comp0, double *c, const double *uf, const double *vf,
                       int rho_pos) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = NPAD(g);
  for (int ic = 0; ic < ncomp; ++ic) {
    double *a = c + ic * n;
    bc_ctx x = {g, uf, vf, c + (size_t)(rho_pos - comp0) * n, n, comp0 + ic};
    if (!g->per_x)
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) {
          bc_set(&x, a, PIDX(g, 0, j, k), PIDX(g, 1, j, k), PIDX(g, 2, j, k), 0, k, uf ? uf[UFI(g, 0, j, k)] : 0.0);
          bc_set(&x, a, PIDX(g, nx + 1, j, k), PIDX(g, nx, j, k), PIDX(g, nx - 1, j, k), 1, k,
                 uf ? uf[UFI(g, nx, j, k)] : 0.0);
        }
    if (!g->per_y)
      for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
          bc_set(&x, a, PIDX(g, i, 0, k), PIDX(g, i, 1, k), PIDX(g, i, 2, k), 2, k, vf ? vf[VFI(g, i, 0, k)] : 0.0);
          bc_set(&x, a, PIDX(g, i, ny + 1, k), PIDX(g, i, ny, k), PIDX(g, i, ny - 1, k), 3, k,
                 vf ? vf[VFI(g, i, ny, k)] : 0.0);
        }
    if (!g->per_z)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          bc_set(&x, a, PIDX(g, i, j, 0), PIDX(g, i, j, 1), PIDX(g, i, j, 2), 4, 1, 0.0);
          bc_set(&x, a, PIDX(g, i, j, nz + 1), PIDX(g, i, j, nz), PIDX(g, i, j, nz - 1), 5, nz, 0.0);
        }
  }
}
void ora_bound_cond(const ora_geom *g, int ncomp, int comp0, double *c) {
  bound_cond(g, ncomp, comp0, c, g->bc_uf, g->bc_vf, g->bc_rho);
}

/* ADVECT/Advection_Mod.f90:2118-2125 k1F / k2F */
static double k1f(double hL, double hC, double hR) {
  return (hC / (hC + hR + EPS)) * ((hL + hC) / (hL + hC + hR + EPS));
}
static double k2f(double hL, double hC, double hR) {
  return (hC / (hL + hC + EPS)) * (hR / (hL + hC + hR + EPS));
}
/* ADVECT/Advection_Mod.f90:2127-2134 PhiLim, MethAdv='Koren' (default,
 * MODULE/Control_Mod.f90:591).  cC/cR are the formal arguments. */
static double philim_koren(double r, double k1, double k2, double cC, double cR) {
  double a = k1 * r + k2;
  double m = a < 1.0 ? a : 1.0;     /* MIN(k1*r+k2,One) */
  m = r < m ? r : m;                /* MIN(r,...) */
  m = 0.0 > m ? 0.0 : m;            /* MAX(Zero,...) */
  return m * (cC - cR);
}

/* ------------------------------------------------------------------ */
/* Flux RHS of one component: ADVECT/Advection_Mod.f90:737-1054
 * AdvectionComputeP (main loop :854-974, zero-volume mask :1045-1051).
 * rho = density component (Rho(:,:,:,1)), c = component, f = output
 * (accumulated; caller zeroes).  No outflow sides, no fall speed.        */
/* ------------------------------------------------------------------ */
static void advection_compute_p(const ora_geom *g, const double *c, const double *rho,
                                const double *uf, const double *vf, const double *wf,
                                double *f) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const double *V = g->volc;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t P = PIDX(g, i, j, k);
        double cC = c[P] / (rho[P] + EPS);
        double VC = V[P];
        double cL, cR, VL, VR, FL, FR, k1, k2, cDiff, r, Flux;
        /* x-direction */
        {
          size_t PL = PIDX(g, i - 1, j, k), PR = PIDX(g, i + 1, j, k);
          cL = c[PL] / (rho[PL] + EPS);
          cR = c[PR] / (rho[PR] + EPS);
          VL = V[PL];
          VR = V[PR];
          FR = g->fu[FUI(g, i, j, k)];
          FL = g->fu[FUI(g, i - 1, j, k)];
          if (VL < VC) cL = ((VC - VL) * cC + VL * cL) / VC;
          if (VR < VC) cR = ((VC - VR) * cC + VR * cR) / VC;
          if (FL < FR) cL = ((FR - FL) * cC + FL * cL) / FR;
          if (FR < FL) cR = ((FL - FR) * cC + FR * cR) / FL;
          /* left boundary */
          k1 = k1f(VR, VC, VL);
          k2 = k2f(VR, VC, VL);
          cDiff = cR - cC;
          r = (cC - cL + EPS) / (cDiff + EPS);
          {
            double uu = uf[UFI(g, i - 1, j, k)];
            Flux = HALF * (fabs(uu) - uu) * FL * (cC + FR / (FR + EPS) * philim_koren(r, k1, k2, cC, cR));
          }
          f[PL] = f[PL] + Flux;
          f[P] = f[P] - Flux;
          /* right boundary */
          k1 = k1f(VL, VC, VR);
          k2 = k2f(VL, VC, VR);
          cDiff = cC - cL;
          r = (cR - cC + EPS) / (cDiff + EPS);
          {
            double uu = uf[UFI(g, i, j, k)];
            Flux = HALF * (fabs(uu) + uu) * FR * (cC + FL / (FL + EPS) * philim_koren(r, k1, k2, cC, cL));
          }
          f[PR] = f[PR] + Flux;
          f[P] = f[P] - Flux;
        }
        /* y-direction (no volume blend, :903-904) */
        {
          size_t PL = PIDX(g, i, j - 1, k), PR = PIDX(g, i, j + 1, k);
          cL = c[PL] / (rho[PL] + EPS);
          cR = c[PR] / (rho[PR] + EPS);
          VL = V[PL];
          VR = V[PR];
          FR = g->fv[FVI(g, i, j, k)];
          FL = g->fv[FVI(g, i, j - 1, k)];
          if (FL < FR) cL = ((FR - FL) * cC + FL * cL) / FR;
          if (FR < FL) cR = ((FL - FR) * cC + FR * cR) / FL;
          k1 = k1f(VR, VC, VL);
          k2 = k2f(VR, VC, VL);
          cDiff = cR - cC;
          r = (cC - cL + EPS) / (cDiff + EPS);
          {
            double vv = vf[VFI(g, i, j - 1, k)];
            Flux = HALF * (fabs(vv) - vv) * FL * (cC + FR / (FR + EPS) * philim_koren(r, k1, k2, cC, cR));
          }
          f[PL] = f[PL] + Flux;
          f[P] = f[P] - Flux;
          k1 = k1f(VL, VC, VR);
          k2 = k2f(VL, VC, VR);
          cDiff = cC - cL;
          r = (cR - cC + EPS) / (cDiff + EPS);
          {
            double vv = vf[VFI(g, i, j, k)];
            Flux = HALF * (fabs(vv) + vv) * FR * (cC + FL / (FL + EPS) * philim_koren(r, k1, k2, cC, cL));
          }
          f[PR] = f[PR] + Flux;
          f[P] = f[P] - Flux;
        }
        /* z-direction (no fall speed: wFLoc = wF) */
        {
          size_t PL = PIDX(g, i, j, k - 1), PR = PIDX(g, i, j, k + 1);
          cL = c[PL] / (rho[PL] + EPS);
          cR = c[PR] / (rho[PR] + EPS);
          VL = V[PL];
          VR = V[PR];
          FR = g->fw[FWI(g, i, j, k)];
          FL = g->fw[FWI(g, i, j, k - 1)];
          if (FL < FR) cL = ((FR - FL) * cC + FL * cL) / FR;
          if (FR < FL) cR = ((FL - FR) * cC + FR * cR) / FL;
          k1 = k1f(VR, VC, VL);
          k2 = k2f(VR, VC, VL);
          cDiff = cR - cC;
          r = (cC - cL + EPS) / (cDiff + EPS);
          {
            double ww = wf[WFI(g, i, j, k - 1)];
            Flux = HALF * (fabs(ww) - ww) * FL * (cC + FR / (FR + EPS) * philim_koren(r, k1, k2, cC, cR));
          }
          f[PL] = f[PL] + Flux;
          f[P] = f[P] - Flux;
          k1 = k1f(VL, VC, VR);
          k2 = k2f(VL, VC, VR);
          cDiff = cC - cL;
          r = (cR - cC + EPS) / (cDiff + EPS);
          {
            double ww = wf[WFI(g, i, j, k)];
            Flux = HALF * (fabs(ww) + ww) * FR * (cC + FL / (FL + EPS) * philim_koren(r, k1, k2, cC, cL));
          }
          f[PR] = f[PR] + Flux;
          f[P] = f[P] - Flux;
        }
      }
  /* inflow through the faces of the outer walls, first-order upwind from
   * the halo cell (:975-1044); the bottom divides by the interior density */
  if (!g->per_x)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        size_t H = PIDX(g, 0, j, k);
        double u = uf[UFI(g, 0, j, k)];
        double Flux = HALF * (fabs(u) + u) * c[H] / (rho[H] + EPS) * g->fu[FUI(g, 0, j, k)];
        f[PIDX(g, 1, j, k)] = f[PIDX(g, 1, j, k)] + Flux;
        f[H] = 0.0;
      }
  if (!g->per_x)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        size_t H = PIDX(g, nx + 1, j, k);
        double u = uf[UFI(g, nx, j, k)];
        double Flux = HALF * (fabs(u) - u) * c[H] / (rho[H] + EPS) * g->fu[FUI(g, nx, j, k)];
        f[PIDX(g, nx, j, k)] = f[PIDX(g, nx, j, k)] + Flux;
        f[H] = 0.0;
      }
  if (!g->per_y)
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        size_t H = PIDX(g, i, 0, k);
        double v = vf[VFI(g, i, 0, k)];
        double Flux = HALF * (fabs(v) + v) * c[H] / (rho[H] + EPS) * g->fv[FVI(g, i, 0, k)];
        f[PIDX(g, i, 1, k)] = f[PIDX(g, i, 1, k)] + Flux;
        f[H] = 0.0;
      }
  if (!g->per_y)
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        size_t H = PIDX(g, i, ny + 1, k);
        double v = vf[VFI(g, i, ny, k)];
        double Flux = HALF * (fabs(v) - v) * c[H] / (rho[H] + EPS) * g->fv[FVI(g, i, ny, k)];
        f[PIDX(g, i, ny, k)] = f[PIDX(g, i, ny, k)] + Flux;
        f[H] = 0.0;
      }
  if (!g->per_z)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t H = PIDX(g, i, j, 0), P = PIDX(g, i, j, 1);
        double w = wf[WFI(g, i, j, 0)];
        double Flux = HALF * (fabs(w) + w) * c[H] / (rho[P] + EPS) * g->fw[FWI(g, i, j, 0)];
        f[P] = f[P] + Flux;
        f[H] = 0.0;
      }
  if (!g->per_z)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t H = PIDX(g, i, j, nz + 1);
        double w = wf[WFI(g, i, j, nz)];
        double Flux = HALF * (fabs(w) - w) * c[H] / (rho[H] + EPS) * g->fw[FWI(g, i, j, nz)];
        f[PIDX(g, i, j, nz)] = f[PIDX(g, i, j, nz)] + Flux;
        f[H] = 0.0;
      }
  /* zero-volume mask over the padded box, :1045-1051 */
  const size_t n = NPAD(g);
  for (size_t P = 0; P < n; ++P) f[P] = f[P] * V[P] / (V[P] + EPS);
}

/* ExchangeFlux for a single periodic block: MODULE/Vector4CellPar_Mod.f90:359-417
 * RandCopyFlux_VecCell with CopyFlux EqualEqual (MODULE/Exchange_Mod.f90:257-324):
 * the interior cell next to a periodic side receives the flux deposited in the
 * opposite halo.  Neighbour order W, E, S, N, B, T.                           */
void ora_exchange_flux(const ora_geom *g, int ncomp, double *f) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = NPAD(g);
  for (int ic = 0; ic < ncomp; ++ic) {
    double *a = f + ic * n;
    if (g->per_x) {
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) a[PIDX(g, 1, j, k)] = a[PIDX(g, 1, j, k)] + a[PIDX(g, nx + 1, j, k)];
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) a[PIDX(g, nx, j, k)] = a[PIDX(g, nx, j, k)] + a[PIDX(g, 0, j, k)];
    }
    if (g->per_y) {
      for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) a[PIDX(g, i, 1, k)] = a[PIDX(g, i, 1, k)] + a[PIDX(g, i, ny + 1, k)];
      for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) a[PIDX(g, i, ny, k)] = a[PIDX(g, i, ny, k)] + a[PIDX(g, i, 0, k)];
    }
    if (g->per_z) {
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) a[PIDX(g, i, j, 1)] = a[PIDX(g, i, j, 1)] + a[PIDX(g, i, j, nz + 1)];
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) a[PIDX(g, i, j, nz)] = a[PIDX(g, i, j, nz)] + a[PIDX(g, i, j, 0)];
    }
  }
}

/* ------------------------------------------------------------------ */
/* FcnMet advection part for all components:
 *   ADVECT/Function_Mod.f90:1032-1099 (AdvectionCompute per component, the
 *   density component advected with c=>Rho), :1312-1314 BoundaryFluxCondition
 *   (no-op without chemistry) and ExchangeFlux, :1338-1345 AdvectionScale
 *   (ADVECT/Advection_Mod.f90:2888-2898).
 * c: ncomp padded fields; comp rho_pos is the density.  f: output (zeroed here). */
/* ------------------------------------------------------------------ */
/* ------------------------------------------------------------------ */
/* DiffusionCompute (ADVECT/Diffusion_Mod.f90:11-275) of one component with
 * DH/DV = g->dh/g->dv and DF the arithmetic face mean
 * (ADVECT/Operator_Mod.f90:49-53).  Sides that are not outer walls (the
 * periodic neighbour) carry half the flux from each side, completed by
 * ExchangeFlux; an outer wall takes the interior cell's coefficient and
 * updates the interior cell only.  Ends with f = f*VolC/(VolC+Eps) over the
 * padded box. */
/* ------------------------------------------------------------------ */
static double df_mean(double DL, double VL, double DR, double VR) { return (DL * VR + DR * VL) / (VL + VR + EPS); }
static void diffusion_compute(const ora_geom *g, const double *c, const double *rho, double *f) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const double *V = g->volc, *DH = g->dh, *DV = g->dv;
  const size_t n = NPAD(g);
#define CF(P) (c[P] / (rho[P] + EPS))
  /* x */
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      const size_t L = PIDX(g, 0, j, k), R = PIDX(g, 1, j, k);
      const double FF = g->fu[FUI(g, 0, j, k)], VL = V[L], VR = V[R];
      if (g->per_x) {
        const double Flux = df_mean(DH[L], VL, DH[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      } else {
        const double Flux = 2.0 * DH[R] * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
      }
    }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        const size_t L = PIDX(g, i, j, k), R = PIDX(g, i + 1, j, k);
        const double FF = g->fu[FUI(g, i, j, k)], VL = V[L], VR = V[R];
        const double Flux = 2.0 * df_mean(DH[L], VL, DH[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      const size_t L = PIDX(g, nx, j, k), R = PIDX(g, nx + 1, j, k);
      const double FF = g->fu[FUI(g, nx, j, k)], VL = V[L], VR = V[R];
      if (g->per_x) {
        const double Flux = df_mean(DH[L], VL, DH[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      } else {
        const double Flux = 2.0 * DH[L] * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[L] = f[L] + Flux;
      }
    }
  /* y */
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) {
      const size_t L = PIDX(g, i, 0, k), R = PIDX(g, i, 1, k);
      const double FF = g->fv[FVI(g, i, 0, k)], VL = V[L], VR = V[R];
      if (g->per_y) {
        const double Flux = df_mean(DH[L], VL, DH[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      } else {
        const double Flux = 2.0 * DH[R] * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
      }
    }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t L = PIDX(g, i, j, k), R = PIDX(g, i, j + 1, k);
        const double FF = g->fv[FVI(g, i, j, k)], VL = V[L], VR = V[R];
        const double Flux = 2.0 * df_mean(DH[L], VL, DH[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      }
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) {
      const size_t L = PIDX(g, i, ny, k), R = PIDX(g, i, ny + 1, k);
      const double FF = g->fv[FVI(g, i, ny, k)], VL = V[L], VR = V[R];
      if (g->per_y) {
        const double Flux = df_mean(DH[L], VL, DH[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      } else {
        const double Flux = 2.0 * DH[L] * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[L] = f[L] + Flux;
      }
    }
  /* z */
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const size_t L = PIDX(g, i, j, 0), R = PIDX(g, i, j, 1);
      const double FF = g->fw[FWI(g, i, j, 0)], VL = V[L], VR = V[R];
      if (g->per_z) {
        const double Flux = df_mean(DV[L], VL, DV[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      } else {
        const double Flux = 2.0 * DV[R] * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
      }
    }
  for (int k = 1; k <= nz - 1; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t L = PIDX(g, i, j, k), R = PIDX(g, i, j, k + 1);
        const double FF = g->fw[FWI(g, i, j, k)], VL = V[L], VR = V[R];
        const double Flux = 2.0 * df_mean(DV[L], VL, DV[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const size_t L = PIDX(g, i, j, nz), R = PIDX(g, i, j, nz + 1);
      const double FF = g->fw[FWI(g, i, j, nz)], VL = V[L], VR = V[R];
      if (g->per_z) {
        const double Flux = df_mean(DV[L], VL, DV[R], VR) * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[R] = f[R] - Flux;
        f[L] = f[L] + Flux;
      } else {
        const double Flux = 2.0 * DV[L] * FF * FF / (VL + VR + EPS) * (CF(R) - CF(L));
        f[L] = f[L] + Flux;
      }
    }
#undef CF
  for (size_t P = 0; P < n; ++P) f[P] = f[P] * V[P] / (V[P] + EPS);
}

/* the diffusion terms of FcnMet for every component (Function_Mod.f90:1112-1239;
 * CrossDiff off, Prandtl number 1, one coefficient pair for all components) */
void ora_diffusion(const ora_geom *g, int ncomp, int rho_pos, const double *c, double *f) {
  if (!g->dh) return;
  const size_t n = NPAD(g);
  const double *rho = c + (size_t)rho_pos * n;
  for (int ic = 0; ic < ncomp; ++ic) diffusion_compute(g, c + ic * n, rho, f + ic * n);
}

/* AdvectionComputeP of one component (accumulates into f, unscaled). */
void ora_advection(const ora_geom *g, const double *c, const double *rho, const double *uf, const double *vf,
                   const double *wf, double *f) {
  advection_compute_p(g, c, rho, uf, vf, wf, f);
}

void ora_fcn(const ora_geom *g, int ncomp, int rho_pos, const double *c, const double *uf,
             const double *vf, const double *wf, double *f) {
  const size_t n = NPAD(g);
  memset(f, 0, sizeof(double) * n * (size_t)ncomp);
  const double *rho = c + (size_t)rho_pos * n;
  for (int ic = 0; ic < ncomp; ++ic) advection_compute_p(g, c + ic * n, rho, uf, vf, wf, f + ic * n);
  ora_diffusion(g, ncomp, rho_pos, c, f);
  ora_exchange_flux(g, ncomp, f);
  for (int ic = 0; ic < ncomp; ++ic) {
    double *a = f + ic * n;
    for (size_t P = 0; P < n; ++P) a[P] = a[P] / (g->volc[P] + EPS);
  }
}

/* DivCompute: ADVECT/Advection_Mod.f90:2901-2916 (accumulates into rhs). */
void ora_div(const ora_geom *g, const double *uf, const double *vf, const double *wf, double *rhs) {
  for (int k = 1; k <= g->nz; ++k)
    for (int j = 1; j <= g->ny; ++j)
      for (int i = 1; i <= g->nx; ++i) {
        size_t P = PIDX(g, i, j, k);
        rhs[P] = rhs[P] - (uf[UFI(g, i, j, k)] * g->fu[FUI(g, i, j, k)] - uf[UFI(g, i - 1, j, k)] * g->fu[FUI(g, i - 1, j, k)] +
                           vf[VFI(g, i, j, k)] * g->fv[FVI(g, i, j, k)] - vf[VFI(g, i, j - 1, k)] * g->fv[FVI(g, i, j - 1, k)] +
                           wf[WFI(g, i, j, k)] * g->fw[FWI(g, i, j, k)] - wf[WFI(g, i, j, k - 1)] * g->fw[FWI(g, i, j, k - 1)]);
      }
}

/* ------------------------------------------------------------------ */
/* Jacobian: ADVECT/Advection_Mod.f90:2220-2872 JacAdvectionCompute (interior
 * loops :2244-2318; periodic-neighbour branches, non-refined, :2320-2870), then
 * ADVECT/Function_Mod.f90:1782-1862 JacScaleCompute (boundary fold + scale to
 * I - beta0*dt*J).  val: 7*NPAD, overwritten.                                  */
/* ------------------------------------------------------------------ */
static void jac_face(double *val, size_t n, size_t iL, size_t iR, int dUp, int dDn, double vel, double F,
                     double VL, double VR, double rhoL, double rhoR) {
  /* one face between padded cells iL (left) and iR (right):
   * "uF > 0" part then "uF < 0" part, exactly as in the Fortran loops */
  val[(size_t)dUp * n + iL] = val[(size_t)dUp * n + iL] + HALF * (fabs(vel) + vel) * F / VR / (rhoL + EPS);
  val[3 * n + iL] = val[3 * n + iL] - HALF * (fabs(vel) + vel) * F / VL / (rhoL + EPS);
  val[(size_t)dDn * n + iR] = val[(size_t)dDn * n + iR] + HALF * (fabs(vel) - vel) * F / VL / (rhoR + EPS);
  val[3 * n + iR] = val[3 * n + iR] - HALF * (fabs(vel) - vel) * F / VR / (rhoR + EPS);
}

/* JacDiffusionCompute (ADVECT/Diffusion_Mod.f90:1504-1708): per face with a
 * neighbour (interior faces, and the boundary faces of periodic sides; an
 * outer wall adds nothing) Temp = Two*DF*F*F/(VL+VR+Eps) enters the two
 * off-diagonals and the two diagonals of the face's cells, divided by the
 * row cell's VolC+Eps and by the column cell's Rho+Eps.  Slots: off-diagonal
 * of the left column d_lo (x: 2, y: 1, z: 0), of the right column d_hi. */
static void jac_diff_face(double *val, size_t n, size_t L, size_t R, int d_lo, int d_hi, double DL, double DR,
                          double VL, double VR, double FF, const double *rho) {
  const double Temp = 2.0 * df_mean(DL, VL, DR, VR) * FF * FF / (VL + VR + EPS);
  val[(size_t)d_lo * n + L] = val[(size_t)d_lo * n + L] + Temp / (VR + EPS) / (rho[L] + EPS);
  val[3 * n + L] = val[3 * n + L] - Temp / (VL + EPS) / (rho[L] + EPS);
  val[(size_t)d_hi * n + R] = val[(size_t)d_hi * n + R] + Temp / (VL + EPS) / (rho[R] + EPS);
  val[3 * n + R] = val[3 * n + R] - Temp / (VR + EPS) / (rho[R] + EPS);
}
static void jac_diffusion(const ora_geom *g, const double *rho, double *val) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = NPAD(g);
  const double *V = g->volc, *DH = g->dh, *DV = g->dv;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = g->per_x ? 0 : 1; i <= (g->per_x ? nx : nx - 1); ++i) {
        const size_t L = PIDX(g, i, j, k), R = PIDX(g, i + 1, j, k);
        jac_diff_face(val, n, L, R, 2, 4, DH[L], DH[R], V[L], V[R], g->fu[FUI(g, i, j, k)], rho);
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = g->per_y ? 0 : 1; j <= (g->per_y ? ny : ny - 1); ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t L = PIDX(g, i, j, k), R = PIDX(g, i, j + 1, k);
        jac_diff_face(val, n, L, R, 1, 5, DH[L], DH[R], V[L], V[R], g->fv[FVI(g, i, j, k)], rho);
      }
  for (int k = g->per_z ? 0 : 1; k <= (g->per_z ? nz : nz - 1); ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t L = PIDX(g, i, j, k), R = PIDX(g, i, j, k + 1);
        jac_diff_face(val, n, L, R, 0, 6, DV[L], DV[R], V[L], V[R], g->fw[FWI(g, i, j, k)], rho);
      }
}

void ora_jac(const ora_geom *g, const double *rho, const double *uf, const double *vf, const double *wf,
             double beta0, double dt, double *val) {
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  const size_t n = NPAD(g);
  const double *V = g->volc;
  memset(val, 0, sizeof(double) * 7 * n);
  /* JacTransportX, interior faces */
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        size_t iL = PIDX(g, i, j, k), iR = PIDX(g, i + 1, j, k);
        jac_face(val, n, iL, iR, 2, 4, uf[UFI(g, i, j, k)], g->fu[FUI(g, i, j, k)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t iL = PIDX(g, i, j, k), iR = PIDX(g, i, j + 1, k);
        jac_face(val, n, iL, iR, 1, 5, vf[VFI(g, i, j, k)], g->fv[FVI(g, i, j, k)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
  for (int k = 1; k <= nz - 1; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t iL = PIDX(g, i, j, k), iR = PIDX(g, i, j, k + 1);
        jac_face(val, n, iL, iR, 0, 6, wf[WFI(g, i, j, k)], g->fw[FWI(g, i, j, k)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
  /* neighbour branches in order W, E, S, N, B, T ('iw'/'ie'/... of a
   * periodic single block; walls have no neighbour entry) */
  if (g->per_x) {
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        size_t iL = PIDX(g, 0, j, k), iR = PIDX(g, 1, j, k);
        jac_face(val, n, iL, iR, 2, 4, uf[UFI(g, 0, j, k)], g->fu[FUI(g, 0, j, k)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        size_t iL = PIDX(g, nx, j, k), iR = PIDX(g, nx + 1, j, k);
        jac_face(val, n, iL, iR, 2, 4, uf[UFI(g, nx, j, k)], g->fu[FUI(g, nx, j, k)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
  }
  else { /* 'ow', 'oe' (:2390-2410 and the east twin): the outflow diagonal of the interior cell */
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        size_t P = PIDX(g, 1, j, k);
        double u = uf[UFI(g, 0, j, k)], F = g->fu[FUI(g, 0, j, k)];
        val[3 * n + P] = val[3 * n + P] - HALF * (fabs(u) - u) * F / (V[P] + EPS) / (rho[P] + EPS);
      }
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j) {
        size_t P = PIDX(g, nx, j, k);
        double u = uf[UFI(g, nx, j, k)], F = g->fu[FUI(g, nx, j, k)];
        val[3 * n + P] = val[3 * n + P] - HALF * (fabs(u) + u) * F / (V[P] + EPS) / (rho[P] + EPS);
      }
  }
  if (g->per_y) {
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        size_t iL = PIDX(g, i, 0, k), iR = PIDX(g, i, 1, k);
        jac_face(val, n, iL, iR, 1, 5, vf[VFI(g, i, 0, k)], g->fv[FVI(g, i, 0, k)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        size_t iL = PIDX(g, i, ny, k), iR = PIDX(g, i, ny + 1, k);
        jac_face(val, n, iL, iR, 1, 5, vf[VFI(g, i, ny, k)], g->fv[FVI(g, i, ny, k)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
  }
  else { /* 'os', 'on' */
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        size_t P = PIDX(g, i, 1, k);
        double v = vf[VFI(g, i, 0, k)], F = g->fv[FVI(g, i, 0, k)];
        val[3 * n + P] = val[3 * n + P] - HALF * (fabs(v) - v) * F / (V[P] + EPS) / (rho[P] + EPS);
      }
    for (int k = 1; k <= nz; ++k)
      for (int i = 1; i <= nx; ++i) {
        size_t P = PIDX(g, i, ny, k);
        double v = vf[VFI(g, i, ny, k)], F = g->fv[FVI(g, i, ny, k)];
        val[3 * n + P] = val[3 * n + P] - HALF * (fabs(v) + v) * F / (V[P] + EPS) / (rho[P] + EPS);
      }
  }
  if (g->per_z) {
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t iL = PIDX(g, i, j, 0), iR = PIDX(g, i, j, 1);
        jac_face(val, n, iL, iR, 0, 6, wf[WFI(g, i, j, 0)], g->fw[FWI(g, i, j, 0)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t iL = PIDX(g, i, j, nz), iR = PIDX(g, i, j, nz + 1);
        jac_face(val, n, iL, iR, 0, 6, wf[WFI(g, i, j, nz)], g->fw[FWI(g, i, j, nz)], V[iL] + EPS, V[iR] + EPS, rho[iL], rho[iR]);
      }
  }
  else { /* 'ob', 'ot' */
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t P = PIDX(g, i, j, 1);
        double w = wf[WFI(g, i, j, 0)], F = g->fw[FWI(g, i, j, 0)];
        val[3 * n + P] = val[3 * n + P] - HALF * (fabs(w) - w) * F / (V[P] + EPS) / (rho[P] + EPS);
      }
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        size_t P = PIDX(g, i, j, nz);
        double w = wf[WFI(g, i, j, nz)], F = g->fw[FWI(g, i, j, nz)];
        val[3 * n + P] = val[3 * n + P] - HALF * (fabs(w) + w) * F / (V[P] + EPS) / (rho[P] + EPS);
      }
  }
  if (g->dh && g->jac_diff) jac_diffusion(g, rho, val);
  /* JacScaleCompute fold (no side is outflow): Function_Mod.f90:1791-1856 */
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      size_t P = PIDX(g, 0, j, k);
      val[3 * n + P] = val[3 * n + P] - val[2 * n + P];
    }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      size_t P = PIDX(g, nx + 1, j, k);
      val[3 * n + P] = val[3 * n + P] - val[4 * n + P];
    }
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) {
      size_t P = PIDX(g, i, 0, k);
      val[3 * n + P] = val[3 * n + P] - val[1 * n + P];
    }
  for (int k = 1; k <= nz; ++k)
    for (int i = 1; i <= nx; ++i) {
      size_t P = PIDX(g, i, ny + 1, k);
      val[3 * n + P] = val[3 * n + P] - val[5 * n + P];
    }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t P = PIDX(g, i, j, 0);
      val[3 * n + P] = val[3 * n + P] - val[0 * n + P];
    }
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      size_t P = PIDX(g, i, j, nz + 1);
      val[3 * n + P] = val[3 * n + P] - val[6 * n + P];
    }
  /* scale: Function_Mod.f90:1857-1862 */
  const double bdt = beta0 * dt;
  for (size_t P = 0; P < n; ++P) val[3 * n + P] = 1.0 - bdt * val[3 * n + P];
  for (int d = 0; d < 7; ++d) {
    if (d == 3) continue;
    for (size_t P = 0; P < n; ++P) val[(size_t)d * n + P] = -(bdt * val[(size_t)d * n + P]);
  }
}

/* DIA shifts, MODULE/Vector4Cell_Mod.f90:1030-1036 */
static void dia_shifts(const ora_geom *g, long sh[7]) {
  long NX = NXP(g), NXY = (long)NXP(g) * NYP(g);
  sh[0] = -NXY; sh[1] = -NX; sh[2] = -1; sh[3] = 0; sh[4] = 1; sh[5] = NX; sh[6] = NXY;
}

/* y = A*x, CG/MatSpDiag_Mod.f90:87-108 SpAVec_SpDiag (column oriented) */
void ora_spmv(const ora_geom *g, const double *val, const double *x, double *y) {
  const long n = (long)NPAD(g);
  long sh[7];
  dia_shifts(g, sh);
  for (long i = 0; i < n; ++i) y[i] = 0.0;
  for (int d = 0; d < 7; ++d) {
    long s = sh[d];
    long lo = s > 0 ? s : 0, hi = n + (s < 0 ? s : 0);
    for (long i = lo; i < hi; ++i) y[i - s] = y[i - s] + val[(size_t)d * n + i] * x[i];
  }
}

/* x = GS(b), CG/MatSpDiag_Mod.f90:191-235 GaussSeidel_SpDiag (1 forward
 * solve + IterG=5 forward sweeps).  x and b may alias. */
void ora_gauss_seidel(const ora_geom *g, const double *val, const double *b, double *x, int iterg) {
  const long n = (long)NPAD(g);
  long sh[7];
  dia_shifts(g, sh);
  const long pad = -sh[0];
  double *T = (double *)malloc(sizeof(double) * (size_t)(n + 2 * pad));
  double *tmp = T + pad; /* Temp(1+DiagPtr(1) : n-DiagPtr(1)) */
  double *bb = (double *)malloc(sizeof(double) * (size_t)n);
  memcpy(bb, b, sizeof(double) * (size_t)n);
  memset(T, 0, sizeof(double) * (size_t)(n + 2 * pad));
  for (long i = 0; i < n; ++i) tmp[i] = bb[i];
  for (long i = 0; i < n; ++i) {
    tmp[i] = tmp[i] / val[3 * n + i];
    for (int d = 0; d < 3; ++d) tmp[i - sh[d]] = tmp[i - sh[d]] - val[(size_t)d * n + i] * tmp[i];
  }
  for (int it = 0; it < iterg; ++it) {
    for (long i = 0; i < n; ++i) {
      for (int d = 4; d < 7; ++d) tmp[i - sh[d]] = tmp[i - sh[d]] - val[(size_t)d * n + i] * tmp[i];
      tmp[i] = bb[i];
    }
    for (long i = 0; i < n; ++i) {
      tmp[i] = tmp[i] / val[3 * n + i];
      for (int d = 0; d < 3; ++d) tmp[i - sh[d]] = tmp[i - sh[d]] - val[(size_t)d * n + i] * tmp[i];
    }
  }
  memcpy(x, tmp, sizeof(double) * (size_t)n);
  free(T);
  free(bb);
}

/* PSolve_Vec4CellSp: MODULE/SpMatrix4CellPar_Mod.f90:86-102 with PSolveSp
 * (MODULE/Vector4Cell_Mod.f90:694-740): copy, exchange, per-component GS,
 * halo zeroed, exchange. */
void ora_psolve(const ora_geom *g, int ncomp, const double *val, const double *x, double *px, int iterg) {
  const size_t n = NPAD(g);
  const int nx = g->nx, ny = g->ny, nz = g->nz;
  memcpy(px, x, sizeof(double) * n * (size_t)ncomp);
  ora_exchange_cell(g, ncomp, px);
  for (int ic = 0; ic < ncomp; ++ic) {
    double *a = px + ic * n;
    ora_gauss_seidel(g, val, a, a, iterg);
    for (int j = 0; j <= ny + 1; ++j)
      for (int i = 0; i <= nx + 1; ++i) {
        a[PIDX(g, i, j, 0)] = 0.0;
        a[PIDX(g, i, j, nz + 1)] = 0.0;
      }
    for (int k = 0; k <= nz + 1; ++k)
      for (int i = 0; i <= nx + 1; ++i) {
        a[PIDX(g, i, 0, k)] = 0.0;
        a[PIDX(g, i, ny + 1, k)] = 0.0;
      }
    for (int k = 0; k <= nz + 1; ++k)
      for (int j = 0; j <= ny + 1; ++j) {
        a[PIDX(g, 0, j, k)] = 0.0;
        a[PIDX(g, nx + 1, j, k)] = 0.0;
      }
  }
  ora_exchange_cell(g, ncomp, px);
}

/* MatVecMet_Vec4CellSp: MODULE/SpMatrix4CellPar_Mod.f90:70-84 with
 * MatVecMetSp (MODULE/Vector4Cell_Mod.f90:605-644).  The per-cell source block
 * of the transport-only stage is the identity, so PSolve(JacSMetLU) leaves its
 * argument unchanged; Axpy(-1,x,Ax) and Xpy(x,Ax) are kept for the rounding. */
void ora_matvec(const ora_geom *g, int ncomp, const double *val, const double *x, double *ax) {
  const size_t n = NPAD(g);
  for (int ic = 0; ic < ncomp; ++ic) {
    const double *xa = x + ic * n;
    double *ya = ax + ic * n;
    ora_spmv(g, val, xa, ya);
    for (size_t P = 0; P < n; ++P) ya[P] = -1.0 * xa[P] + ya[P];
    for (size_t P = 0; P < n; ++P) ya[P] = xa[P] + ya[P];
  }
}

/* Dot_VectorCell (MODULE/Vector4Cell_Mod.f90:1120-1132): interior only, per
 * component SUM in array-element order, then summed over components. */
double ora_dot(const ora_geom *g, int ncomp, const double *x, const double *y) {
  const size_t n = NPAD(g);
  double tot = 0.0;
  for (int ic = 0; ic < ncomp; ++ic) {
    double s = 0.0;
    for (int k = 1; k <= g->nz; ++k)
      for (int j = 1; j <= g->ny; ++j)
        for (int i = 1; i <= g->nx; ++i) {
          size_t P = PIDX(g, i, j, k);
          s = s + x[ic * n + P] * y[ic * n + P];
        }
    tot = tot + s;
  }
  return tot;
}

/* Axpy_VectorCell (:1237-1250): y = alpha*x + y, skipped if alpha == 0 */
static void axpy(size_t len, double alpha, const double *x, double *y) {
  if (alpha == 0.0) return;
  for (size_t i = 0; i < len; ++i) y[i] = alpha * x[i] + y[i];
}
/* Xpay_VectorCell (:1316-1326): y = alpha*y + x */
static void xpay(size_t len, const double *x, double alpha, double *y) {
  for (size_t i = 0; i < len; ++i) y[i] = alpha * y[i] + x[i];
}

/* BiCGStabMet_Vec4CellSp: MODULE/SpMatrix4CellPar_Mod.f90:245-348.
 * x: in/out (initial guess), b: rhs.  *maxiter and *tol in/out with the
 * reference's conventions (negative = converged at the half step, 2*Iter =
 * iteration limit hit; tol returns the final residual norm). */
/* stop_half > 0 (tests only): leave after exactly that many half-steps, the
 * way the solver leaves when the tolerance is met there (the comparison of a
 * GPU run whose iteration count differs by one from the tolerance-driven
 * run); 0: the reference's exits only. */
static void bicgstab_core(const ora_geom *g, int ncomp, const double *val, double *x, const double *b, int *maxiter,
                          double *tol, int iterg, int stop_half);
void ora_bicgstab(const ora_geom *g, int ncomp, const double *val, double *x, const double *b, int *maxiter,
                  double *tol, int iterg) {
  bicgstab_core(g, ncomp, val, x, b, maxiter, tol, iterg, 0);
}
void ora_bicgstab_halfsteps(const ora_geom *g, int ncomp, const double *val, double *x, const double *b, int nhalf,
                            int iterg) {
  int maxiter = (nhalf + 1) / 2;
  double tol = 0.0;
  bicgstab_core(g, ncomp, val, x, b, &maxiter, &tol, iterg, nhalf);
}
static void bicgstab_core(const ora_geom *g, int ncomp, const double *val, double *x, const double *b, int *maxiter,
                          double *tol, int iterg, int stop_half) {
  const size_t len = NPAD(g) * (size_t)ncomp;
  double *r = (double *)calloc(len, sizeof(double));
  double *rt = (double *)calloc(len, sizeof(double));
  double *rh = (double *)calloc(len, sizeof(double));
  double *p = (double *)calloc(len, sizeof(double));
  double *ph = (double *)calloc(len, sizeof(double));
  double *t = (double *)calloc(len, sizeof(double));
  double *v = (double *)calloc(len, sizeof(double));
  double alpha = 0, beta, omega = 0, rho = 0, rhoOld, rNorm, rNorm0;
  int MaxIter = *maxiter;
  double Tol = *tol;
  ora_matvec(g, ncomp, val, x, r); /* MatVecChem with the identity source block */
  xpay(len, b, -1.0, r);
  memcpy(rt, r, sizeof(double) * len);
  rNorm0 = sqrt(ora_dot(g, ncomp, r, r));
  for (int Iter = 1; Iter <= MaxIter; ++Iter) {
    rhoOld = rho;
    rho = ora_dot(g, ncomp, rt, r);
    if (rho == 0.0) {
      *maxiter = Iter;
      *tol = 0.0;
      goto done;
    }
    if (Iter == 1) {
      memcpy(p, r, sizeof(double) * len);
    } else {
      beta = (rho / rhoOld) * (alpha / omega);
      axpy(len, -omega, v, p);
      xpay(len, r, beta, p);
    }
    ora_psolve(g, ncomp, val, p, ph, iterg);
    ora_matvec(g, ncomp, val, ph, v);
    alpha = rho / ora_dot(g, ncomp, rt, v);
    axpy(len, -alpha, v, r);
    rNorm = sqrt(ora_dot(g, ncomp, r, r));
    if (rNorm <= Tol * rNorm0 || stop_half == 2 * Iter - 1) {
      axpy(len, alpha, ph, x);
      *maxiter = -Iter;
      *tol = rNorm;
      goto done;
    }
    ora_psolve(g, ncomp, val, r, rh, iterg);
    ora_matvec(g, ncomp, val, rh, t);
    omega = ora_dot(g, ncomp, t, r) / ora_dot(g, ncomp, t, t);
    axpy(len, alpha, ph, x);
    axpy(len, omega, rh, x);
    axpy(len, -omega, t, r);
    rNorm = sqrt(ora_dot(g, ncomp, r, r));
    if (rNorm <= Tol * rNorm0 || stop_half == 2 * Iter) {
      *maxiter = Iter;
      *tol = rNorm;
      goto done;
    }
    if (Iter == MaxIter) {
      *maxiter = 2 * Iter;
      *tol = rNorm;
      goto done;
    }
  }
done:
  free(r); free(rt); free(rh); free(p); free(ph); free(t); free(v);
}

/* ------------------------------------------------------------------ */
/* Rosenbrock coefficients: ADVECT/Int_Mod.f90:78-261 InitRos3MetC.
 * method: 0 Ros3AMF, 1 RosRK32, 2 RosEul, 3 Ros3P, 4 Ros3Pw, 5 RosRK3,
 *         6 RosTVD, 7 RosRK4.  alpha/beta are 4x4 row-major [i][j] (1-based
 * i,j of the Fortran mapped to [i-1][j-1]), gamma1[0..4].  Returns nStage.  */
/* ------------------------------------------------------------------ */
int ora_ros_coeffs(int method, double *beta0_out, double alpha[16], double beta[16], double gamma1[5]) {
  double a[4][4] = {{0}}, b[4][4] = {{0}}, gm[5] = {0};
  double beta0 = 0;
  int nStage = 0;
  if (method == 0) { /* Ros3AMF (single-precision literals in the Fortran) */
    nStage = 2;
    beta0 = (double)(0.5f + sqrtf(3.0f) / 6.0f);
    a[0][0] = 2.0 / 3.0; a[0][1] = 0.0; a[1][0] = 5.0 / 4.0; a[1][1] = 3.0 / 4.0;
    b[1][0] = -4.0 / 3.0;
    gm[0] = 0.0; gm[1] = 0.666666666666667; gm[2] = 1.0;
  } else if (method == 1) { /* RosRK32 */
    nStage = 3;
    double theta = 1.0 / 3.0 * atan(sqrt(2.0) / 4.0);
    beta0 = 1.0 - 0.5 * sqrt(2.0) * cos(theta) + 0.5 * sqrt(6.0) * sin(theta);
    double gamma32 = 0.5 - 3.0 * beta0;
    double gamma31 = -(6.0 * beta0 * beta0 * beta0 - 12.0 * beta0 * beta0 + 6.0 * (1.0 + gamma32) * beta0 +
                       2.0 * gamma32 * gamma32 - 0.5) / (1.0 + 2.0 * gamma32);
    double gamma21 = -(3.0 * beta0 + gamma31 + gamma32);
    double tt[3][3] = {{0}};
    tt[0][0] = 1.0;
    tt[1][0] = -gamma21 / beta0; tt[1][1] = 1.0;
    tt[2][0] = -gamma31 / beta0 + gamma32 * gamma21 / (beta0 * beta0); tt[2][1] = -gamma32 / beta0; tt[2][2] = 1.0;
    double al[3][3] = {{0.5, 0, 0}, {0.5, 0.5, 0}, {1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0}};
    double be[3][3] = {{0, 0, 0}, {gamma21 / beta0, 0, 0}, {gamma31 / beta0, gamma32 / beta0, 0}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = 0.0, s2 = 0.0;
        for (int k = 0; k < 3; ++k) { s = s + al[i][k] * tt[k][j]; s2 = s2 + be[i][k] * tt[k][j]; }
        a[i][j] = s; b[i][j] = s2;
      }
    gm[0] = 0; gm[1] = 0; gm[2] = 1.0;
  } else if (method == 2) { /* RosEul */
    beta0 = 1.0; nStage = 1; a[0][0] = 1.0; gm[0] = 0.0; gm[1] = 1.0;
  } else if (method == 3) { /* Ros3P */
    nStage = 3;
    beta0 = 7.886751345948129e-1;
    a[0][0] = 1.267949192431123; a[1][0] = 1.267949192431123; a[2][0] = 2.0; a[2][1] = 5.773502691896258e-1;
    a[2][2] = 4.226497308103742e-1;
    b[1][0] = -1.607695154586736; b[2][0] = -3.464101615137755; b[2][1] = -1.732050807568877;
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) { a[i][j] *= beta0; b[i][j] *= beta0; }
  } else if (method == 4) { /* Ros3Pw */
    nStage = 3;
    beta0 = 7.88675134594812865529e-01;
    a[0][0] = 2.0; a[1][0] = 6.33974596215561403412e-01; a[2][0] = 1.63397459621556140341e+00;
    a[2][1] = 2.94228634059947813384e-01; a[2][2] = 1.07179676972449078320e+00;
    b[1][0] = -2.53589838486224561365e+00; b[2][0] = -1.62740473580835520728e+00; b[2][1] = -2.74519052838329002952e-01;
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) { a[i][j] *= beta0; b[i][j] *= beta0; }
  } else if (method == 5) { /* RosRK3 */
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
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) { a[i][j] *= beta0; b[i][j] *= beta0; }
    gm[0] = 0.0; gm[1] = 1.0 / 3.0; gm[2] = 1.0 / 2.0; gm[3] = 1.0;
  } else if (method == 6) { /* RosTVD */
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
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) { a[i][j] *= beta0; b[i][j] *= beta0; }
  } else if (method == 7) { /* RosRK4 */
    nStage = 4;
    beta0 = 1.0 / 4.0;
    a[0][0] = 2.0; a[1][0] = 2.0; a[1][1] = 2.0; a[2][0] = 6.0; a[2][1] = 10.0; a[2][2] = 4.0;
    a[3][0] = 14.0 / 3.0; a[3][1] = 20.0 / 3.0; a[3][2] = 4.0 / 3.0; a[3][3] = 2.0 / 3.0;
    b[1][0] = -4.0; b[2][0] = -6.0; b[2][1] = -10.0; b[3][0] = -4.0; b[3][1] = -12.0;
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) { a[i][j] *= beta0; b[i][j] *= beta0; }
  } else {
    return 0;
  }
  *beta0_out = beta0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) { alpha[i * 4 + j] = a[i][j]; beta[i * 4 + j] = b[i][j]; }
  for (int i = 0; i < 5; ++i) gamma1[i] = gm[i];
  return nStage;
}

/* ------------------------------------------------------------------ */
/* One Rosenbrock step of the transport-only stage (prognostic velocity
 * absent, face velocities prescribed and steady):
 *   ADVECT/Int_Mod.f90:1059-1122 Ros3MetC (ErrControl=.FALSE.) and
 *   :263-374 StageRos.  c: ncomp padded fields (in/out).
 * iters/resid: per stage BiCGStab MaxIter/Tol outputs (nStage entries). */
/* ------------------------------------------------------------------ */
int ora_ros_step(const ora_geom *g, int ncomp, int rho_pos, double *c, const double *uf, const double *vf,
                 const double *wf, double dt, int method, double bicg_tol, int bicg_maxiter, int iterg,
                 int *iters, double *resid) {
  double beta0, alpha[16], beta[16], gamma1[5];
  int nStage = ora_ros_coeffs(method, &beta0, alpha, beta, gamma1);
  if (nStage <= 0) return -1;
  const size_t n = NPAD(g), len = n * (size_t)ncomp;
  double *cold = (double *)malloc(sizeof(double) * len);
  double *rhs = (double *)malloc(sizeof(double) * len);
  double *incr = (double *)calloc(len * (size_t)nStage, sizeof(double));
  double *val = (double *)malloc(sizeof(double) * 7 * n);
  memcpy(cold, c, sizeof(double) * len);
  for (int is = 0; is < nStage; ++is) {
    ora_exchange_cell(g, ncomp, c);
    bound_cond(g, ncomp, 0, c, uf, vf, rho_pos); /* StageRos :287 BoundaryCondition */
    if (is == 0) ora_jac(g, c + (size_t)rho_pos * n, uf, vf, wf, beta0, dt, val);
    ora_fcn(g, ncomp, rho_pos, c, uf, vf, wf, rhs);
    for (size_t i = 0; i < len; ++i) rhs[i] = dt * rhs[i]; /* ScaleV */
    for (int js = 0; js < is; ++js) axpy(len, beta[is * 4 + js], incr + (size_t)js * len, rhs);
    double *x = incr + (size_t)is * len;
    memset(x, 0, sizeof(double) * len);
    int it = bicg_maxiter;
    double tol = bicg_tol;
    ora_bicgstab(g, ncomp, val, x, rhs, &it, &tol, iterg);
    if (iters) iters[is] = it;
    if (resid) resid[is] = tol;
    ora_exchange_cell(g, ncomp, x);
    ora_exchange_cell(g, ncomp, x);
    memcpy(c, cold, sizeof(double) * len);
    for (int js = 0; js <= is; ++js) axpy(len, alpha[is * 4 + js], incr + (size_t)js * len, c);
  }
  free(cold); free(rhs); free(incr); free(val);
  return nStage;
}

/* TotalScalar: ADVECT/Diagnostic_Mod.f90:13-31, SUM(c*VolB) over the interior. */
double ora_total_scalar(const ora_geom *g, const double *c) {
  double s = 0.0;
  for (int k = 1; k <= g->nz; ++k)
    for (int j = 1; j <= g->ny; ++j)
      for (int i = 1; i <= g->nx; ++i) {
        size_t P = PIDX(g, i, j, k);
        s = s + c[P] * g->volc[P];
      }
  return s;
}

/* ------------------------------------------------------------------ */
/* Vertical-column tridiagonal kernels: MULTI/TriDiagT_Mod.f90:113-133
 * MatVecT_1D and :135-155 Solve_1D (Thomas), applied to ncol independent
 * columns of length n1 (column-contiguous: d[col*n1 + i], u/l[col*(n1-1)+i]). */
/* ------------------------------------------------------------------ */
void ora_tri_solve(int ncol, int n1, const double *d, const double *u, const double *l, double *b) {
  double *w = (double *)malloc(sizeof(double) * (size_t)(n1 > 1 ? n1 : 1));
  for (int col = 0; col < ncol; ++col) {
    const double *dd = d + (size_t)col * n1;
    const double *uu = u + (size_t)col * (n1 - 1);
    const double *ll = l + (size_t)col * (n1 - 1);
    double *bb = b + (size_t)col * n1;
    double t = dd[0];
    bb[0] = bb[0] / t;
    for (int i = 1; i < n1; ++i) {
      w[i - 1] = uu[i - 1] / t;
      t = dd[i] - ll[i - 1] * w[i - 1];
      bb[i] = (bb[i] - ll[i - 1] * bb[i - 1]) / t;
    }
    for (int i = n1 - 2; i >= 0; --i) bb[i] = bb[i] - w[i] * bb[i + 1];
  }
  free(w);
}

void ora_tri_matvec(int ncol, int n1, const double *d, const double *u, const double *l, const double *x, double *y) {
  for (int col = 0; col < ncol; ++col) {
    const double *dd = d + (size_t)col * n1;
    const double *uu = u + (size_t)col * (n1 - 1);
    const double *ll = l + (size_t)col * (n1 - 1);
    const double *xx = x + (size_t)col * n1;
    double *yy = y + (size_t)col * n1;
    if (n1 > 1) {
      yy[0] = dd[0] * xx[0] + uu[0] * xx[1];
      for (int i = 1; i < n1 - 1; ++i) yy[i] = ll[i - 1] * xx[i - 1] + dd[i] * xx[i] + uu[i] * xx[i + 1];
      yy[n1 - 1] = ll[n1 - 2] * xx[n1 - 2] + dd[n1 - 1] * xx[n1 - 1];
    } else {
      yy[0] = dd[0] * xx[0];
    }
  }
}
