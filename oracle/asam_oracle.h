/*
 * Shared definitions of the CPU oracle (TEST INFRASTRUCTURE ONLY): the block
 * geometry handed in by the tests and the index maps of the Fortran layout
 * (see asam_oracle.c for the conventions).
 */
#ifndef ASAM_ORACLE_H
#define ASAM_ORACLE_H
#include <stddef.h>

#define EPS 1.0e-30 /* CG/Kind_Mod_gf.f90 Eps */
#define HALF 0.5

typedef struct {
  int nx, ny, nz;
  int per_x, per_y, per_z; /* 1 = periodic side pair, 0 = closed walls */
  const double *volc, *fu, *fv, *fw;
  /* halo rule of the outer walls per component and side (W,E,S,N,B,T):
   * 0 none, 1 ZeroGrad, 2 ZeroValue, 3 MeanValue, 4 Function,
   * 5 InFlowOutFlow, 6 Extrapolation; bc[6*ic + side].  NULL = ZeroGrad
   * everywhere, the default BCMetVec (MODULE/BoundaryCond_Mod.f90:240-247). */
  const int *bc;
  /* diffusion coefficients (DH horizontal, DV vertical; padded cell fields,
   * the reference's DiffKoeff) or NULL: no diffusion.  jac_diff: add the
   * diffusion Jacobian (JacDiffusion) to the stage matrix. */
  const double *dh, *dv;
  int jac_diff;
  /* data of the open-boundary halo rules (kinds 3-6 of bc): MeanProfile
   * (ncomp*nz, level iz at [ic*nz + iz-1]), the Function values at the halo
   * cells (ncomp padded fields), the ambient state VecAmb (ncomp padded
   * fields), the face velocities whose sign InFlowOutFlow tests and the
   * density component; NULL where the kinds in use need none. */
  const double *bc_mean, *bc_fval, *bc_amb, *bc_uf, *bc_vf;
  int bc_rho;
} ora_geom;

#define NXP(g) ((g)->nx + 2)
#define NYP(g) ((g)->ny + 2)
#define NZP(g) ((g)->nz + 2)
#define NPAD(g) ((size_t)NXP(g) * NYP(g) * NZP(g))
#define PIDX(g, i, j, k) ((size_t)(i) + (size_t)NXP(g) * ((size_t)(j) + (size_t)NYP(g) * (size_t)(k)))
#define FUI(g, i, j, k) ((size_t)((i) + 1) + (size_t)((g)->nx + 3) * ((size_t)((j)-1) + (size_t)(g)->ny * (size_t)((k)-1)))
#define FVI(g, i, j, k) ((size_t)((i)-1) + (size_t)(g)->nx * ((size_t)((j) + 1) + (size_t)((g)->ny + 3) * (size_t)((k)-1)))
#define FWI(g, i, j, k) ((size_t)((i)-1) + (size_t)(g)->nx * ((size_t)((j)-1) + (size_t)(g)->ny * (size_t)((k) + 1)))
#define UFI(g, i, j, k) ((size_t)(i) + (size_t)((g)->nx + 1) * ((size_t)((j)-1) + (size_t)(g)->ny * (size_t)((k)-1)))
#define VFI(g, i, j, k) ((size_t)((i)-1) + (size_t)(g)->nx * ((size_t)(j) + (size_t)((g)->ny + 1) * (size_t)((k)-1)))
#define WFI(g, i, j, k) ((size_t)((i)-1) + (size_t)(g)->nx * ((size_t)((j)-1) + (size_t)(g)->ny * (size_t)(k)))

/* entry points shared between the oracle's translation units */
void ora_exchange_cell(const ora_geom *g, int ncomp, double *c);
void ora_bound_cond(const ora_geom *g, int ncomp, int comp0, double *c);
void ora_exchange_flux(const ora_geom *g, int ncomp, double *f);
void ora_advection(const ora_geom *g, const double *c, const double *rho, const double *uf, const double *vf,
                   const double *wf, double *f);
void ora_diffusion(const ora_geom *g, int ncomp, int rho_pos, const double *c, double *f);
void ora_jac(const ora_geom *g, const double *rho, const double *uf, const double *vf, const double *wf,
             double beta0, double dt, double *val);
void ora_bicgstab(const ora_geom *g, int ncomp, const double *val, double *x, const double *b, int *maxiter,
                  double *tol, int iterg);
int ora_ros_coeffs(int method, double *beta0_out, double alpha[16], double beta[16], double gamma1[5]);

#endif
