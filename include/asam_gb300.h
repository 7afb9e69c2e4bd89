/*
 * asam_gb300 -- C-ABI of the GB300 (sm_103a) implementation of ASAM's implicit
 * Rosenbrock transport stage.
 *
 * Every entry point takes plain pointers and sizes.  Field pointers may point
 * to host memory (staged through the context's device buffers) or to device
 * memory (used in place); the library tells them apart itself.  Layouts are
 * the Fortran layouts of ASAM (ix fastest):
 *   cell field   (nx+2)*(ny+2)*(nz+2) doubles, c(ix0:ix1+1,iy0:iy1+1,iz0:iz1+1)
 *   state        ncomp such fields back to back (component ic at ic*npad)
 *   FU (nx+3)*ny*nz, FV nx*(ny+3)*nz, FW nx*ny*(nz+3)   (WeiFU/WeiFV/WeiFW)
 *   uF (nx+1)*ny*nz, vF nx*(ny+1)*nz, wF nx*ny*(nz+1)   (VelocityFace_T)
 *   VolC (nx+2)*(ny+2)*(nz+2)
 *   DIA matrix 7*npad doubles, Val(m,7) column-major
 * All calls return an asam_status; asam_last_error() describes the last
 * failure.  A context is not thread-safe; its work runs on one CUDA stream.
 */
#ifndef ASAM_GB300_H
#define ASAM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  ASAM_OK = 0,
  ASAM_NOT_CONVERGED = 1, /* Krylov iteration limit hit (reference: MaxIter=2*Iter) */
  ASAM_BREAKDOWN = 2,     /* rho == 0 in BiCGStab */
  ASAM_NAN_DETECTED = 3,
  ASAM_BAD_ARG = 4,
  ASAM_CUDA_ERROR = 5,
  ASAM_NO_DEVICE = 6,
  ASAM_IO_ERROR = 7,   /* a restart or geometry file cannot be opened, is short, or does not fit */
  ASAM_UNSUPPORTED = 8 /* a file form this library does not read (Globe/Cyl grids, Struct_Bound above 6) */
} asam_status;

typedef enum {
  ASAM_PREC_FP64 = 0,        /* plain FP64, reference operation order (drop-in) */
  ASAM_PREC_FP32_REFINED = 1 /* FP32 inner BiCGStab + preconditioner inside FP64 refinement */
} asam_precision;

/* Rosenbrock methods of ADVECT/Int_Mod.f90:96-234 (InitRos3MetC). */
typedef enum {
  ASAM_ROS3AMF = 0,
  ASAM_ROSRK32 = 1,
  ASAM_ROSEUL = 2,
  ASAM_ROS3P = 3,
  ASAM_ROS3PW = 4,
  ASAM_ROSRK3 = 5,
  ASAM_ROSTVD = 6,
  ASAM_ROSRK4 = 7
} asam_method;

typedef struct {
  int nx, ny, nz;                          /* interior cells of the block */
  int periodic_x, periodic_y, periodic_z;  /* 1: side pair is periodic ('iw'/'ie' self-neighbour); 0: closed wall */
  int ncomp;                               /* cell components of VecMet (Vector4Cell_T%Vec) */
  int rho_pos;                             /* 0-based index of the density component (RhoPos-1) */
  int method;                              /* asam_method (Control_Mod Method) */
  int bicgstab_maxiter;                    /* BiCGStabMaxIter (Control_Mod.f90:581, default 30) */
  double bicgstab_tol;                     /* BiCGStabTol (Control_Mod.f90:580, default 1e-6) */
  int gs_iter;                             /* IterG (CG/MatSpDiag_Mod.f90:14, default 5) */
  int precision;                           /* asam_precision */
  int inner_precond;                       /* refined mode's FP32 inner preconditioner:
                                              0 = the Gauss-Seidel sweeps of the FP64 path,
                                              1, 2, 3 = line solves (Thomas along z, x, y: the
                                              tridiagonal part of the stage matrix on that axis) */
  int inner_gs_iter;                       /* refined mode: IterG of the FP32 inner Gauss-Seidel
                                              (1+inner_gs_iter sweeps; the FP64 path keeps gs_iter) */
  int gs_schedule;                         /* refined mode, schedule of the FP32 inner sweeps (same
                                              results either way): 0 = one persistent launch, CTAs
                                              take tiles in wavefront order and wait for their
                                              neighbours (bounded waits); 1 = one launch per tile level */
  int gs_group;                            /* refined mode: components per CTA of the FP32 inner
                                              Gauss-Seidel (1..16; 0 = library default) */
} asam_config;

typedef struct asam_ctx asam_ctx;

/* Create a context for one block: uploads the cut-cell geometry (face areas
 * and volumes of MODULE/Domain_Mod.f90:447-460, read by
 * INIT/ReadWeights_Mod.f90:408) and allocates the stage work space
 * (replaces InitRos3MetC's allocations, ADVECT/Int_Mod.f90:235-257, and
 * Allocate_Jac, CHEMIE/Chemie_Mod.f90:294-345). */
int asam_create(const asam_config *cfg, const double *volc, const double *fu, const double *fv, const double *fw,
                asam_ctx **out);
int asam_destroy(asam_ctx *ctx);

/* No reference counterpart: how the Krylov iterations are launched (results
 * are identical in every mode; graphs are never used on the legacy default
 * stream, which cannot be captured):
 *   0 every kernel launched individually, the host takes the exit decisions;
 *   1 (default) the BiCGStab half-iterations are captured as CUDA graphs and
 *     replayed, the host takes the exit decisions;
 *   2 the whole Rosenbrock step is one CUDA graph in which each BiCGStab
 *     loop is a graph WHILE node driven by a condition kernel (bounded by
 *     MaxIter), so a step is one launch and one host read; in a refined
 *     context the FP64 refinement is an outer WHILE node (bounded by 8
 *     passes) around the FP32 BiCGStab's loop.  Transport steps
 *     (asam_ros_step); the dynamical step keeps mode 1. */
int asam_set_graphs(asam_ctx *ctx, int on);

/* Run the context's work on this CUDA stream (cudaStream_t); NULL = the legacy
 * default stream.  Until this is called the context uses a stream of its own. */
int asam_set_stream(asam_ctx *ctx, void *stream);
/* Device pointer of the context's resident state buffer (ncomp*npad doubles). */
int asam_state_device_ptr(asam_ctx *ctx, double **dptr);
/* Block until the context's stream is idle. */
int asam_synchronize(asam_ctx *ctx);

/* Face velocities uF, vF, wF (VelocityFace_T, MODULE/VelocityFace_Mod.f90:211-213). */
int asam_set_velocity(asam_ctx *ctx, const double *uf, const double *vf, const double *wf);

/* Periodic halo fill of ncomp fields: ExchangeCell
 * (MODULE/Vector4CellPar_Mod.f90:752, RandCopyCell_VecCell :611-659). */
int asam_exchange_cell(asam_ctx *ctx, int ncomp, double *c);

/* Halo rule of the outer walls (sides that are not periodic), applied to the
 * state at the start of every Rosenbrock stage like BoundaryCondition and
 * BoundaryVelocity (ADVECT/Int_Mod.f90:283-287; BoundaryCompute
 * ADVECT/BoundaryCondition_Mod.f90:70-346 and BoundaryVelocityCellCompute
 * :424-970 for the kinds below).  kinds[6*ic + side], sides W,E,S,N,B,T.
 * The default of a new context is ZeroGrad everywhere, the reference's
 * default BCMetVec (MODULE/BoundaryCond_Mod.f90:240-247).  A closed box with
 * free-slip walls (BCVel='FreeSlip') has ZeroValue for the momentum
 * components normal to a wall (:292-294 and the other sides).
 * The open-boundary kinds of BoundaryCompute (transport stage only; their
 * data from asam_set_boundary_data):
 *   MEAN_VALUE      halo = 2*MeanProfile(ic,iz) - interior (bottom and top:
 *                   the profile's first and last level)
 *   FUNCTION        halo = 2*F - interior, F the value of the case's start
 *                   function at the halo cell (times RhoFun for all but the
 *                   number concentrations), as the caller evaluates it
 *   INFLOW_OUTFLOW  W/E/S/N: where the face velocity points into the block
 *                   (or is zero) halo = Rho(halo)*VecAmb(halo), else the
 *                   interior value; the bottom and top keep their halos
 *   EXTRAPOLATION   B/T: halo = 2*c(iz0+1) - c(iz0+2); the lateral sides keep
 *                   their halos
 * Whatever the kinds, a face velocity pointing into the block through an
 * outer wall carries the halo's value in (the first-order inflow of
 * AdvectionComputeP, ADVECT/Advection_Mod.f90:975-1044). */
enum {
  ASAM_BC_NONE = 0,
  ASAM_BC_ZERO_GRAD = 1,
  ASAM_BC_ZERO_VALUE = 2,
  ASAM_BC_MEAN_VALUE = 3,
  ASAM_BC_FUNCTION = 4,
  ASAM_BC_INFLOW_OUTFLOW = 5,
  ASAM_BC_EXTRAPOLATION = 6
};
int asam_set_boundary(asam_ctx *ctx, const int *kinds);
/* Data of the open-boundary kinds, copied into the context (host or device
 * pointers; NULL drops an array, refused while a kind uses it): mean_profile
 * ncomp*nz with level iz of component ic at [ic*nz + iz-1] (MeanProfile,
 * ADVECT/Diagnostic_Mod.f90:275-314); function_values ncomp padded fields
 * whose halo cells hold F; ambient ncomp padded fields of VecAmb.  The
 * values stay until the next call: a time-dependent F is evaluated by the
 * caller, once per step (the reference evaluates it at each stage's time). */
int asam_set_boundary_data(asam_ctx *ctx, const double *mean_profile, const double *function_values,
                           const double *ambient);
/* Apply the halo rule to a state (ncomp padded fields) once. */
int asam_boundary_condition(asam_ctx *ctx, double *c);

/* Diffusion of every component (the FcnMet diffusion terms,
 * ADVECT/Function_Mod.f90:1106-1239, DiffusionCompute
 * ADVECT/Diffusion_Mod.f90:11-275, with CrossDiff off and Prandtl number 1):
 * dh, dv the density-weighted horizontal and vertical coefficients (padded
 * cell fields, the DiffKoeff of the TkeDis/TkeOme models; dv NULL = dh);
 * jac != 0 also adds JacDiffusionCompute (:1504-1708) to the stage matrix.
 * dh NULL switches diffusion off.  The face coefficients are computed once
 * here; call again when the coefficients change.  The adjoint entry points
 * refuse a context with diffusion. */
int asam_set_diffusion(asam_ctx *ctx, const double *dh, const double *dv, int jac);

/* Advection right-hand side of all components: the FcnMet advection terms
 * (ADVECT/Function_Mod.f90:1032-1099, 1312-1345): AdvectionComputeP
 * (ADVECT/Advection_Mod.f90:737-1054), ExchangeFlux, AdvectionScale.
 * c: state with current halos; f: output. */
int asam_fcn(asam_ctx *ctx, const double *c, double *f);

/* Face-flux divergence, DivCompute (ADVECT/Advection_Mod.f90:2901-2916):
 * rhs(interior) -= sum F*u.  One field. */
int asam_div(asam_ctx *ctx, double *rhs);

/* Transport Jacobian into the context's DIA matrix: JacAdvectionCompute
 * (ADVECT/Advection_Mod.f90:2220-2872) + JacScaleCompute
 * (ADVECT/Function_Mod.f90:1782-1939), A = I - beta0*dt*J.  c: state (the
 * density component is used). */
int asam_jac(asam_ctx *ctx, const double *c, double dt);
/* Copy the context's DIA matrix out (7*npad doubles) / in. */
int asam_get_jac(asam_ctx *ctx, double *val);
int asam_set_jac(asam_ctx *ctx, const double *val);

/* Stage operator y = A x: MatVecMet_Vec4CellSp
 * (MODULE/SpMatrix4CellPar_Mod.f90:70-84). */
int asam_matvec(asam_ctx *ctx, const double *x, double *y);

/* Transport preconditioner px = P^-1 x: PSolve_Vec4CellSp
 * (MODULE/SpMatrix4CellPar_Mod.f90:86-102; GaussSeidel_SpDiag,
 * CG/MatSpDiag_Mod.f90:191-235). */
int asam_psolve(asam_ctx *ctx, const double *x, double *px);
/* No reference counterpart: the refined mode's FP32 inner preconditioner
 * (x rounded to FP32, 1+inner_gs_iter Gauss-Seidel sweeps in the configured
 * schedule or the column line solve, halo handling as PSolve, result widened
 * to FP64), for tests and measurement.  Refined precision only. */
int asam_inner_psolve(asam_ctx *ctx, const double *x, double *px);
/* No reference counterpart, diagnostic: the polls of one dependency wait of
 * the persistent Gauss-Seidel schedule before its CTA gives up (0: the
 * default 2^21, each poll followed by a short sleep).  A wait that gives up
 * sets an error flag; every CTA then leaves, and the call returns
 * ASAM_CUDA_ERROR ("a dependency wait gave up") with the context still
 * usable.  A limit of a few polls makes the waits run out, which is how the
 * give-up path is tested. */
int asam_set_wait_limit(asam_ctx *ctx, int polls);

/* BiCGStabMetSp: BiCGStabMet_Vec4CellSp (MODULE/SpMatrix4CellPar_Mod.f90:245-348).
 * x in/out (initial guess), b right-hand side.  maxiter/tol in/out with the
 * reference's conventions: on return *maxiter = -Iter (converged at the half
 * step), Iter (converged), 2*Iter (limit hit); *tol = final residual norm. */
int asam_bicgstab(asam_ctx *ctx, double *x, const double *b, int *maxiter, double *tol);

/* One Rosenbrock step with fixed dt (Ros3MetC with ErrControl=.FALSE.,
 * ADVECT/Int_Mod.f90:1059-1122, stages StageRos :263-374, transport part with
 * prescribed steady face velocities).  c: state in/out.  iters/resid: per
 * stage BiCGStab iteration count / residual (may be NULL, else >= nStage). */
int asam_ros_step(asam_ctx *ctx, double *c, double dt, int *iters, double *resid);

/* ---- tangent-linear / adjoint pair of the transport stage ------------------
 * For one passive component `comp` of the state (not the density), with the
 * density and the face velocities held fixed.  The flux operator is piecewise
 * linear in the component (Koren limiter branches); the tangent-linear model
 * freezes the branches of the state it is linearised around.  These have no
 * counterpart in the reference, which has no adjoint. */
/* df = F'(c) dc for the FcnMet advection terms of component comp (single padded fields). */
int asam_fcn_tlm(asam_ctx *ctx, const double *c, int comp, const double *dc, double *df);
/* lc = F'(c)^T lf, the exact transpose of asam_fcn_tlm. */
int asam_fcn_adj(asam_ctx *ctx, const double *c, int comp, const double *lf, double *lc);
/* y = A^T x for the context's DIA matrix (one padded field): a gather from the
 * column-oriented storage of SpAVec_SpDiag (CG/MatSpDiag_Mod.f90:87-108). */
int asam_matvec_adj(asam_ctx *ctx, const double *x, double *y);
/* Solve A_per^T x = b for the periodic interior system transposed (adjoint of
 * the stage solve), BiCGStab with a diagonal preconditioner.  maxiter/tol in:
 * limit and relative tolerance; maxiter out: iterations used. */
int asam_bicgstab_adj(asam_ctx *ctx, double *x, const double *b, int *maxiter, double *tol);
/* Tangent-linear / adjoint of one Rosenbrock step (asam_ros_step) of component
 * comp around state c; du/lam are interior perturbations (padded fields, halos
 * ignored).  tol: relative tolerance of the stage solves. */
int asam_ros_step_tlm(asam_ctx *ctx, const double *c, int comp, const double *du, double *du_out, double dt,
                      double tol);
int asam_ros_step_adj(asam_ctx *ctx, const double *c, int comp, const double *lam, double *lam_out, double dt,
                      double tol);
/* Gradient of J = sum over the box of (c_comp/Rho)^2 * VolC after nsteps steps
 * with respect to the initial component field (interior of a padded field).
 * box = {i0,i1,j0,j1,k0,k1}, 1-based interior indices, inclusive.  The forward
 * states are checkpointed every ckpt_every steps; the reverse sweep recomputes
 * each segment once from its checkpoint, recording the stage states of its
 * steps: memory (nsteps/ckpt_every + ckpt_every*nStage + nStage + 3) states;
 * cost one forward sweep plus, per step, one forward recomputation and one
 * adjoint step. */
int asam_tracer_gradient(asam_ctx *ctx, const double *c0, int comp, int nsteps, double dt, int ckpt_every,
                         const int *box, double tol, double *J, double *grad);
/* The same objective's gradient with respect to the initial component field
 * (grad_c), the initial density (grad_rho; padded fields) and the steady face
 * mass fluxes (grad_uf/vf/wf, the extents of asam_set_velocity), with the
 * density evolving with the wind: the reverse sweep runs the coupled
 * density-component adjoint (the component's flux depends on the density
 * through the mixing ratio, the stage matrix on the density and the wind).
 * Faces with zero velocity are not differentiable (the upwind side switches
 * there) and get 0.  Cost per step: one forward recomputation (segments are
 * recorded with the stage increments of Rho and the component) and the
 * coupled adjoint step. */
int asam_tracer_wind_gradient(asam_ctx *ctx, const double *c0, int comp, int nsteps, double dt, int ckpt_every,
                              const int *box, double tol, double *J, double *grad_c, double *grad_rho,
                              double *grad_uf, double *grad_vf, double *grad_wf);

/* Global mass of one component: TotalScalar (ADVECT/Diagnostic_Mod.f90:13-31). */
int asam_total_scalar(asam_ctx *ctx, const double *c, int comp, double *out);

/* Batched vertical-column tridiagonal solve, Solve_1D (Thomas,
 * MULTI/TriDiagT_Mod.f90:135-155), over ncol independent columns of length n1:
 * d[col*n1+i], u[col*(n1-1)+i], l[col*(n1-1)+i]; b overwritten by the solution.
 * Host or device arrays; synchronous.  The inputs go through a device
 * workspace that the library keeps per device, grown to the largest call (a
 * call allocates only when it is larger than every earlier one); calls are
 * serialised. */
int asam_tri_solve(int ncol, int n1, const double *d, const double *u, const double *l, double *b);
/* Same solve without any allocation (no counterpart in the reference).  For
 * callers that cannot let a library allocate device memory: a host model
 * that owns all device memory through its own pool, or one that overlaps this
 * solve with other streams (cudaMalloc/cudaFree synchronise the device).  d,
 * u, l and b must be device pointers of the current device (or managed
 * memory); the work runs on `stream` (NULL = legacy default stream) and is not
 * waited for.  The elimination factors go to a fixed 32 MiB array inside the
 * library, so ncol*n1 may not exceed 4194304 (ASAM_BAD_ARG otherwise).  Every
 * call looks the array's device address up on the current device (so a reset
 * device is handled); make the first call on a device before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race. */
int asam_tri_solve_noalloc(int ncol, int n1, const double *d, const double *u, const double *l, double *b,
                           void *stream);
/* y = T x for the same column batch, MatVecT_1D (MULTI/TriDiagT_Mod.f90:113-133). */
int asam_tri_matvec(int ncol, int n1, const double *d, const double *u, const double *l, const double *x, double *y);

/* ---- Pressure projection (sound solve) of one block --------------------------
 * ProjectVelFace (ADVECT/IntSub_Mod.f90:25-71) with MultiTriT, GradFull and
 * MethSound='FGMRES': Rhs (MATRIX/Rhs_Mod.f90:110-187), FGMRES(StepGMRES)
 * (SOLU/Iter_Mod.f90:121-199) on MatVec1 = MatVecFull (MATRIX/MatVec_Mod.f90:184)
 * preconditioned by PSolve1 (MATRIX/PreCond_Mod.f90:1555), whose pressure
 * block is the semi-coarsening multigrid Solve_3D (MULTI/TriDiagT_Mod.f90:1073)
 * on the tridiagonal Laplacian hierarchy of LaplTFullCompute
 * (MULTI/JacAccGrav_Mod.f90:1056), then UpdateVelocity (Rhs_Mod.f90:589).
 * Scope: blocks whose sides are closed outer boundaries or periodic (the
 * block is its own neighbour across the side pair), default orders (z,x,y)
 * and coarsening factors 2.  A periodic side carries the boundary face
 * unknowns u_w ... w_t of PressureVelocity (MODULE/VecPrVel_Mod.f90:10-18)
 * with MatVecFull's face equations, Exchange after every operator
 * application, DOT2, and PSolve1's Schur step SchurPreFull on the Dirichlet
 * hierarchy of SetFactorD (MATRIX/PreCond_Mod.f90:20-844,
 * MULTI/Reverse_Mod.f90:95-213).  The multigrid relaxes planes and x-lines of
 * one parity concurrently (zebra order of the reference's plane/line
 * Gauss-Seidel; each relaxation is the reference's arithmetic).
 * Interior cell fields below are nx*ny*nz doubles, x fastest (p(1,ix0+1:ix1,..)).
 * A PressureVelocity vector is such a pressure field followed by the face
 * unknowns of the periodic sides in the reference's order u_w, u_e (ny*nz
 * each, y fastest), v_s, v_n (nx*nz, x fastest), w_b, w_t (nx*ny, x fastest):
 * nx*ny*nz + asam_proj_face_count() doubles (just the pressure for a closed
 * block).
 */
typedef struct {
  int ref_level;   /* RefLevel of the block (grid input; 4 for generated blocks) */
  int gauss_iter2; /* GaussIter2 (Control_Mod.f90:55, default 1) */
  int gauss_iter3; /* GaussIter3 (default 1) */
  int mult_iter2;  /* MultIter2 (default 1) */
  int mult_iter3;  /* MultIter3 (default 1) */
  int step_gmres;  /* StepGMRES (Control_Mod.f90:66, default 10) */
  int max_restart; /* QMRMaxIter (Control_Mod.f90:583, default 10) */
  double tol;      /* QMRTol (Control_Mod.f90:582, default 1e-6) */
  double fac_anela;/* FacAnela (MODULE/Physics_Mod.f90:117, 1 = compressible) */
  double prefac2;  /* PreFac2 of SchurPreFull (Control_Mod.f90:59); 0 = the default 0.5 */
} asam_proj_config;

/* Set up the projection of a context: dx[nx], dy[ny], dz[nz] cell widths and
 * metr = MetrXY[ny], MetrXZ[nz], MetrYX[nx], MetrYZ[nz], MetrZX[nx], MetrZY[ny]
 * back to back (NULL: all 1, Cartesian).  Allocates the hierarchy. */
int asam_proj_setup(asam_ctx *ctx, const asam_proj_config *cfg, const double *dx, const double *dy, const double *dz,
                    const double *metr);
/* Sound weights of WeightDiagCompute (MULTI/JacAccGrav_Mod.f90:4152-4391):
 * DTU/DUU with uF extents, DTV/DUV vF, DTW/DUW wF; DUT and DTT interior. */
int asam_proj_weights(asam_ctx *ctx, const double *dtu, const double *dtv, const double *dtw, const double *duu,
                      const double *duv, const double *duw, const double *dut, const double *dtt);
/* The sound weights computed on the device instead, for ThetaKind='Density'
 * (WeightDiagCompute, MULTI/JacAccGrav_Mod.f90:4259-4282, with
 * CellToFaceRhoWeight :3254-3702 on closed walls and periodic x/y sides): state holds rho theta
 * (th_pos), the density (rho_pos) and optionally vapour, cloud and rain water
 * (rv_pos, rc_pos, rr_pos; -1 = absent); tabs is the padded absolute
 * temperature (TAbsCell).  The reference points its vapour at the cloud-water
 * component (JacAccGrav_Mod.f90:313); pass rv_pos = rc_pos to reproduce that. */
int asam_proj_weights_density(asam_ctx *ctx, const double *state, int th_pos, int rho_pos, int rv_pos, int rc_pos,
                              int rr_pos, const double *tabs);
/* Copy one weight array to out (which: 0 DTU, 1 DTV, 2 DTW, 3 DUU, 4 DUV,
 * 5 DUW, 6 DUT, 7 DTT); returns its length, -1 on error.  Diagnostic. */
long asam_proj_get_weights(asam_ctx *ctx, int which, double *out);
/* LaplTFullCompute with the Neumann factors of SetFactorN
 * (MULTI/JacAccGrav_Mod.f90:1056-1310, MULTI/Reverse_Mod.f90:215-292) for
 * beta0 and dtP = dt (ADVECT/Int_Mod.f90:293-295); with periodic sides also
 * the Dirichlet hierarchy of SetFactorD (MULTI/JacAccGrav_Mod.f90:453-469). */
int asam_lapl_compute(asam_ctx *ctx, double beta0, double dtp);
/* Export one assembled array of 3D level level3 and plane level level2
 * (>= level3) in the reversed order (z fastest, then x, then y):
 * which 0 diagonal, 1/2 z couplings u/l, 3/4 x couplings, 5/6 y couplings
 * (level2 == level3 only); entries past the last row/line/plane are 0.
 * Returns the count (out may be NULL), -1 on error.  Diagnostic. */
long asam_lapl_get(asam_ctx *ctx, int level3, int level2, int which, double *out);
/* y = A x, MatVecP_Tri (MULTI/JacAccGrav_Mod.f90:531-545). */
int asam_lapl_matvec(asam_ctx *ctx, const double *x, double *y);
/* x = one Solve_3D from x=0 (VCycleCG, MULTI/JacAccGrav_Mod.f90:4466-4517). */
int asam_lapl_vcycle(asam_ctx *ctx, const double *b, double *x);
/* SolveSound / FGMRES (SOLU/Iter_Mod.f90:9-199): x in/out (start value) and
 * b are PressureVelocity vectors; *maxiter in: restarts (QMRMaxIter), out:
 * inner steps taken; *tol in: relative tolerance, out: final residual
 * estimate / initial residual.  ASAM_NOT_CONVERGED when the tolerance was not
 * reached. */
int asam_solve_sound(asam_ctx *ctx, double *x, const double *b, int *maxiter, double *tol);
/* Number of boundary face unknowns in a PressureVelocity vector of this
 * context (2*ny*nz per periodic x pair, 2*nx*nz per y pair, 2*nx*ny per z
 * pair; 0 for a closed block), -1 without asam_proj_setup. */
long asam_proj_face_count(asam_ctx *ctx);
/* b = MatVec1(x) = MatVecFull (MATRIX/MatVec_Mod.f90:184-258) on
 * PressureVelocity vectors, without the Exchange that FGMRES applies after it. */
int asam_proj_matvec1(asam_ctx *ctx, const double *x, double *b);
/* b = PSolve1(x) (MATRIX/PreCond_Mod.f90:1555-1571) on PressureVelocity vectors:
 * the context's FGMRES preconditioner, i.e. the periodic-Laplacian one
 * instead when asam_proj_set_preconditioner (or the refined default) selects
 * it. */
int asam_proj_psolve1(asam_ctx *ctx, const double *x, double *b);
/* asam_lapl_get and asam_lapl_vcycle on the Dirichlet hierarchy LaplDirichlet
 * (SetFactorD, MULTI/JacAccGrav_Mod.f90:453-469) of a block with periodic
 * sides (-1 / ASAM_BAD_ARG for a closed block, which has none). */
long asam_lapl_get_dirichlet(asam_ctx *ctx, int level3, int level2, int which, double *out);
int asam_lapl_vcycle_dirichlet(asam_ctx *ctx, const double *b, double *x);
/* ProjectVelFace for one stage (ADVECT/IntSub_Mod.f90:25-71): uf/vf/wf the
 * face-velocity increments (updated), incr the cell increments of all
 * components (ncomp*npad, updated: th_pos, rho_pos and the listed scalars
 * via DivScalar), state the old state (needed when nscalar > 0); th_pos /
 * rho_pos 0-based or -1; pressure (nullable) receives x*DUT; steps and
 * resid (nullable) the FGMRES inner steps and relative residual. */
int asam_project_vel_face(asam_ctx *ctx, double *uf, double *vf, double *wf, double *incr, const double *state,
                          int th_pos, int rho_pos, const int *scalars, int nscalar, double *pressure, int *steps,
                          double *resid);
/* Precision of the multigrid V-cycle that preconditions FGMRES (PSolve1):
 * 0 FP64 (the reference's arithmetic, bit-exact), 1 FP32 (a rounded copy of
 * the hierarchy; FGMRES is flexible, so the FP64 Arnoldi relation and its
 * residual test are unchanged and the tolerance is met as before), -1 (the
 * default) FP32 when the context runs ASAM_PREC_FP32_REFINED, else FP64.
 * No reference counterpart.  asam_lapl_vcycle follows the same choice. */
int asam_proj_set_precision(asam_ctx *ctx, int prec);
/* FGMRES preconditioner of a block with periodic x/y sides: 0 PSolve1 (the
 * reference's, three V-cycles per step), 1 the periodic Laplacian (the face
 * unknowns eliminated exactly, the Schur complement on the pressure solved by
 * one V-cycle of a hierarchy whose relaxations couple across the periodic
 * sides), -1 (the default) 1 when the context runs ASAM_PREC_FP32_REFINED,
 * else 0.  FGMRES is flexible, so the tolerance is met either way.  Takes
 * effect at the next asam_lapl_compute.  No reference counterpart. */
int asam_proj_set_preconditioner(asam_ctx *ctx, int kind);
/* Smoothing schedule of the periodic-Laplacian preconditioner's V-cycle:
 * GaussIter2 and GaussIter3 of its hierarchy (the sweeps of a level grow by
 * them from level to level; Control_Mod.f90:55 for the reference's own).
 * Default 0, 0: one sweep on every level.  No reference counterpart; the
 * reference's hierarchies keep asam_proj_config's values. */
int asam_proj_set_pre_schedule(asam_ctx *ctx, int gauss_iter2, int gauss_iter3);
/* Number of multigrid V-cycles run by this context's projection (diagnostic). */
long long asam_proj_vcycles(asam_ctx *ctx);

/* ---------------------------------------------------------------------------
 * Dynamical-core stage of a closed block: the momentum branch (uPosL>0) of
 * StageRos (ADVECT/Int_Mod.f90:263-374) around the transport solve and the
 * pressure projection.  Needs asam_proj_setup first.  The state holds the
 * six LR momentum components (Rho times the face velocity left/right of the
 * cell) besides Rho, rho theta and the moisture/tracer components; the face
 * velocities VelF are the context's (asam_set_velocity), advanced by
 * asam_ros_step_dyn.  Component positions are 0-based, -1 = absent (the
 * reference's zero component).
 * ------------------------------------------------------------------------- */
typedef struct {
  int th_pos;       /* ThPos: rho theta */
  int rv_pos;       /* RhoVPos */
  int rc_pos;       /* RhoCPos */
  int rr_pos;       /* RhoRPos */
  int ri_pos;       /* RhoIPos */
  int mom_pos[6];   /* uPosL, uPosR, vPosL, vPosR, wPosL, wPosR */
  int pgradient;    /* PGradient (MODULE/Physics_Mod.f90:107) */
  int buoyancy;     /* Buoyancy (:129) */
  int free_slip;    /* FreeSlip (:189, default 1): ShiftVel1 at the boundary cells, else ShiftNoSlip */
  int wall_no_slip; /* BCVel of the six walls: 0 'FreeSlip', 1 'NoSlip' (MODULE/BoundaryCond_Mod.f90:292-299) */
  double grav;      /* Grav (9.81) */
} asam_dyn_config;
/* Configure the stage: bound_cells = BoundCell list, (ix,iy,iz) triples of
 * interior cells (1-based) that hold a piece of the terrain surface;
 * scalars = the components that ProjectVelFace corrects with DivScalar
 * (MATRIX/Rhs_Mod.f90:883-889: 1..uPosL-1 without ThPos and RhoPos).
 * Sets the walls' halo rule of the momentum components from wall_no_slip
 * (the BCVel -> BCMetVec derivation, MODULE/BoundaryCond_Mod.f90:279-390). */
int asam_dyn_setup(asam_ctx *ctx, const asam_dyn_config *cfg, const int *bound_cells, int nbound,
                   const int *scalars, int nscalar);
/* VelocityFaceToCellLR (ADVECT/VelocityCellFace_Mod.f90:72-95, 541-654): the
 * momentum components of c (ncomp*npad, in/out) from face values uf/vf/wf,
 * with the boundary-cell shift, then ExchangeCell. */
int asam_face_to_cell(asam_ctx *ctx, const double *uf, const double *vf, const double *wf, double *c);
/* VelocityCellToFaceLR (:27-52, 1369-1894): face values from the momentum
 * components of c; outer walls take the adjacent cell value where the normal
 * component's halo rule is ZeroGrad, 0 otherwise. */
int asam_cell_to_face(asam_ctx *ctx, const double *c, double *uf, double *vf, double *wf);
/* AbsTCompute ThetaKind='Density' and PreCompute (ADVECT/Diagnostic_Mod.f90:
 * 593-615, 710-865) over the padded box: tabs and pre (npad each, nullable). */
int asam_thermo(asam_ctx *ctx, const double *c, double *tabs, double *pre);
/* FcnMet of the dynamical stage (ADVECT/Function_Mod.f90:989-1506): the
 * advection of every component with the context's face velocities, the
 * pressure gradient PGradComputeCFull (ADVECT/PressureGrad_Mod.f90:245-276)
 * from pre, AdvectionScale and the buoyancy AuftriebDryComputeLRFull
 * (ADVECT/Buoyancy_Mod.f90:43-63). */
int asam_fcn_dyn(asam_ctx *ctx, const double *c, const double *pre, double *f);
/* One Rosenbrock step of the dynamical core (Ros3MetC + StageRos,
 * ADVECT/Int_Mod.f90:1059-1122, 263-374): c (in/out), the context's VelF
 * advanced.  Per stage: iters/resid the BiCGStab MaxIter/Tol outputs,
 * psteps/presid the FGMRES inner steps and relative residual (nullable). */
int asam_ros_step_dyn(asam_ctx *ctx, double *c, double dt, int *iters, double *resid, int *psteps,
                      double *presid);
/* Read the context's face velocities VelF. */
int asam_get_velocity(asam_ctx *ctx, double *uf, double *vf, double *wf);

/* DOT(VecMet,VecMet): the interior dot product of the state with itself over
 * all components (Dot_VecCell, MODULE/Vector4CellPar_Mod.f90:84-102), which the
 * reference's driver checks for NaN after every step
 * (ADVECT/MainProg.f90:975-980); returns ASAM_NAN_DETECTED when it is NaN.
 * asam_ros_step and the solves return ASAM_NAN_DETECTED as soon as a
 * residual norm is NaN. */
int asam_state_dot(asam_ctx *ctx, const double *c, double *out);

/* Batched ensemble (no single reference routine: ASAM advances the blocks of
 * one process in turn, DO ibLoc=1,nbLoc, inside Ros3MetC; here the blocks are
 * independent domains).  A batch groups existing contexts, each with its own
 * geometry, wind, configuration and CUDA stream; asam_batch_ros_step advances
 * every member by nsteps Rosenbrock steps of its own dt, members running
 * concurrently on the GPU, driven by up to nthreads host threads (0: one per
 * member, at most 64), largest members first.  states[m] is member m's state
 * (device or host pointer, as asam_ros_step).  iters/resid (optional, NULL
 * allowed): nmember*nsteps*4 entries, as asam_ros_step per step; status
 * (optional): nmember entries.  Returns the first failure's status if any
 * member failed (asam_last_error names it), else NOT_CONVERGED/BREAKDOWN if
 * any member reported it, else OK.  A context may belong to several batches
 * but must not be used elsewhere while a batch call runs. */
/* No reference counterpart: picks the block's solver settings (inner_precond,
 * inner_gs_iter, gs_schedule, gs_group of the refined mode, and whether the
 * BiCGStab half-iterations are replayed from CUDA graphs) by timing complete
 * solves of its first Rosenbrock stage at state c (host or device) and step
 * dt, one setting at a time; keeps the fastest in the context and returns it
 * in choice[5] (that order) with its solve time in *best_ms (may be NULL).
 * The settings change speed only: every candidate solves to the configured
 * tolerance.  An FP64 context only chooses the graph capture. */
int asam_autotune(asam_ctx *ctx, const double *c, double dt, int *choice, double *best_ms);

typedef struct asam_batch asam_batch;
int asam_batch_create(int nmember, asam_ctx *const *members, int nthreads, asam_batch **out);
int asam_batch_destroy(asam_batch *batch);
int asam_batch_ros_step(asam_batch *batch, double *const *states, const double *dt, int nsteps, int *iters,
                        double *resid, int *status);
/* One-graph mode (on = 1; 0 returns to the host threads): every member must
 * have its own stream (FP64 or refined).  asam_batch_ros_step then records
 * the whole call -- nsteps device-driven steps of every member, the BiCGStab
 * loops as graph WHILE/IF nodes with their exit decisions on the device --
 * into one CUDA graph with one branch per member, launches it once and reads
 * every member's per-stage outputs once.  The graph is kept while the device
 * states, step sizes, step count and tolerances stay the same.  Results are
 * bitwise those of the members run alone.  No reference counterpart. */
int asam_batch_set_graph(asam_batch *batch, int on);

/* Rosenbrock coefficients of InitRos3MetC (ADVECT/Int_Mod.f90:78-261):
 * alpha/beta 4x4 row-major, gamma1[5].  Returns nStage (0 = unknown method). */
int asam_ros_coeffs(int method, double *beta0, double *alpha, double *beta, double *gamma1);

/* No reference counterpart, diagnostic: clock cycles per FMA of a dependent
 * FP64 chain run by the first `lanes` threads of each of `warps` warps of one
 * block (one SM), the slowest warp's.  Shows that the FP64 unit's cost is per
 * warp instruction (independent of the active lanes) and shared by the SM's
 * warps. */
int asam_probe_fp64_chain(int warps, int lanes, int iters, double *cycles_per_op);
/* Diagnostic: scalar FP64 FMA throughput of the current device in GFLOP/s
 * (no reference counterpart; used for the FP64 roofline of the benchmark). */
int asam_probe_fp64_fma(int iters, double *gflops);

/* Diagnostic: count operand pairs (n pseudo-random pairs, exponents within
 * +-span binades) where the library's FMA-corrected quotient from a
 * precomputed reciprocal differs from the IEEE quotient (no reference
 * counterpart; guards the bit-exact FP64 path). */
int asam_probe_div(long long n, long long seed, int span, long long *mismatches);

/* Batched block-tridiagonal column solve of the density/buoyancy-coupled
 * line preconditioners (MultiTriTB, MultiTriTR): Solve_1D of
 * MULTI/TriDiagTB_Mod.f90:143-163, which MULTI/TriDiagTR_Mod.f90:155-175
 * repeats statement for statement,
 * a Thomas elimination with 2x2 blocks (Div_2, Div_22, Mult_2, Mult_22 of
 * CG/Matrix_Mod.f90), over ncol independent columns of n1 levels.
 * d[(col*n1+i)*4 + r+2c] = A%d(r+1,c+1,i+1); u, l[(col*(n1-1)+i)*4 + r+2c];
 * b[(col*n1+i)*2 + r] overwritten by the solution.  Host or device pointers. */
int asam_tri_tb_solve(int ncol, int n1, const double *d, const double *u, const double *l, double *b);

/* Assembly of the same columns: Allocate_1D and Compute_1D of
 * MULTI/TriDiagTB_Mod.f90:32-93 (variant 0) or of MULTI/TriDiagTR_Mod.f90:32-105
 * (variant 1, the density-weight terms DUR in the second block column too),
 * in the reference's statement order.  Per column, faces f, fg, dtu, duu
 * [col*(n1+1) + i] (F, FG, DTU, DUU of faces 1..n1+1), cells vol, dut, dur
 * [col*n1 + i] (dur only for variant 1); d, u, l as for asam_tri_tb_solve,
 * overwritten.  Host or device pointers. */
typedef struct {
  double beta0_dtp; /* beta0*dtp */
  double fac1_l;    /* Fac1_L, the weight of the first face (boundary condition of the line) */
  double fac1_r;    /* Fac1_R, the weight of the last face */
  double grav_comp; /* GravComp */
  double fac_anela; /* FacAnela */
  double fac2_l;    /* Fac2_L, the weight of the first face between lines (asam_tri_tb_compute_2d) */
  double fac2_r;    /* Fac2_R, the weight of the last one */
  double fac3_l;    /* Fac3_L, the weight of the first face between planes (asam_tri_tb_compute_3d) */
  double fac3_r;    /* Fac3_R, the weight of the last one */
} asam_tri_tb_coefs;
int asam_tri_tb_compute(int variant, int ncol, int n1, const asam_tri_tb_coefs *coefs, const double *f,
                        const double *fg, const double *vol, const double *dtu, const double *duu, const double *dut,
                        const double *dur, double *d, double *u, double *l);

/* Assembly of the plane systems: Allocate_2D and Compute_2D of
 * MULTI/TriDiagTB_Mod.f90:221-343 (variant 0) or MULTI/TriDiagTR_Mod.f90:230-387
 * (variant 1) on nplane planes of n2 lines of n1 levels.  Per plane p:
 * z faces f1, f1g, dtu1, duu1 [(p*n2 + j)*(n1+1) + i]; the faces between
 * lines f2, f2g, dtu2, duu2 [(p*(n2+1) + j)*n1 + i] (F2, F2G, DTU2, DUU2 of
 * faces 1..n2+1); cells vol, dut, dur [(p*n2 + j)*n1 + i].  Out: the lines'
 * blocks d [(p*n2 + j)*n1 + i][4] and couplings u1, l1
 * [(p*n2 + j)*(n1-1) + i][4] (as asam_tri_tb_compute per line), and the
 * couplings between lines j and j+1, u2, l2 [(p*(n2-1) + j)*n1 + i][4]
 * (TriDiagTB's are a vector, the first block column; entries 2 and 3 are
 * 0).  Bit for bit the reference's line-by-line sweep, all elements at once.
 * Host or device pointers. */
int asam_tri_tb_compute_2d(int variant, int nplane, int n2, int n1, const asam_tri_tb_coefs *coefs,
                           const double *f1, const double *f1g, const double *dtu1, const double *duu1,
                           const double *f2, const double *f2g, const double *dtu2, const double *duu2,
                           const double *vol, const double *dut, const double *dur, double *d, double *u1,
                           double *l1, double *u2, double *l2);

/* Assembly of a 3D level: Compute_3D of MULTI/TriDiagTB_Mod.f90:663-780
 * (variant 0) or MULTI/TriDiagTR_Mod.f90:707-864 (variant 1) on n3 planes of
 * n2 lines of n1 levels coupled through the faces between planes f3, f3g,
 * dtu3, duu3 [(k*n2 + j)*n1 + i] (faces 1..n3+1); the plane arrays as for
 * asam_tri_tb_compute_2d with p = k.  couple selects the reference's branch:
 * 1, the level stores the couplings between planes u3, l3
 * [(k*n2 + j)*n1 + i][4] (k < n3-1; TriDiagTB's the first block column) and
 * its interior and last faces leave DUU3 out, as the reference does there;
 * 0, no couplings (u3, l3 unused) and every face term has DUU3 (the coarse
 * levels).  The first face has DUU3 in both. */
int asam_tri_tb_compute_3d(int variant, int couple, int n3, int n2, int n1, const asam_tri_tb_coefs *coefs,
                           const double *f1, const double *f1g, const double *dtu1, const double *duu1,
                           const double *f2, const double *f2g, const double *dtu2, const double *duu2,
                           const double *f3, const double *f3g, const double *dtu3, const double *duu3,
                           const double *vol, const double *dut, const double *dur, double *d, double *u1,
                           double *l1, double *u2, double *l2, double *u3, double *l3);

/* y = A x on one level of n3 planes of n2 lines of n1 levels: MatVecTB_2D/3D
 * (MULTI/TriDiagTB_Mod.f90:345-372, 782-816; variant 0: the couplings between
 * lines and planes are vectors that multiply the neighbour's first
 * component) or MatVecTR_2D/3D (MULTI/TriDiagTR_Mod.f90:389-416, 866-900;
 * variant 1: 2x2 blocks), with the layouts of asam_tri_tb_compute_3d (n3 = 1:
 * a plane, u3/l3 unused; n2 = n3 = 1: a line); x, y [(k*n2 + j)*n1 + i][2]. */
int asam_tri_tb_matvec_3d(int variant, int n3, int n2, int n1, const double *d, const double *u1, const double *l1,
                          const double *u2, const double *l2, const double *u3, const double *l3, const double *x,
                          double *y);

/* GaussSeidel_2D of TriDiagTB (variant 0, MULTI/TriDiagTB_Mod.f90:374-418) or
 * TriDiagTR (variant 1, TriDiagTR_Mod.f90:418-462) on nplane planes assembled
 * by asam_tri_tb_compute_2d: gauss_iter symmetric line sweeps (lines 1..n2-1
 * forward, n2..2 backward, each line's right-hand side minus its couplings,
 * then Solve_1D), then line 1 once more, as the reference; planes in
 * parallel, each plane's sweep in the reference's order.  b, x
 * [(p*n2 + j)*n1 + i][2]; x in: the initial guess, out: the result;
 * gauss_iter >= 1 when n2 > 1. */
int asam_tri_tb_gauss_seidel_2d(int variant, int nplane, int n2, int n1, const double *d, const double *u1,
                                const double *l1, const double *u2, const double *l2, const double *b, double *x,
                                int gauss_iter);
/* RestrictTB_2D / ProlongateTB_2D (TriDiagTB_Mod.f90:495-560, the same in
 * TriDiagTR): fine planes n2 x n1, coarse (n2+1)/2 x (n1+1)/2; restriction
 * sums 2x2 fine entries (an odd last line or level alone) in the reference's
 * order, prolongation copies each coarse entry to its fine cells. */
int asam_tri_tb_restrict_2d(int nplane, int n2, int n1, const double *res, double *resc);
int asam_tri_tb_prolong_2d(int nplane, int n2, int n1, const double *xc, double *x);
/* Solve_2D of TriDiagTB (variant 0, MULTI/TriDiagTB_Mod.f90:419-494) or
 * TriDiagTR (variant 1, TriDiagTR_Mod.f90:463-538): mult_iter (MultIter2)
 * V-cycles of Multigrid_2D on nplane independent planes over a hierarchy of
 * nlev levels the caller assembled with asam_tri_tb_compute_2d, finest
 * first: level l has n2s[l] lines of n1s[l] levels, n2s[l+1] =
 * (n2s[l]+1)/2 and n1s[l+1] = (n1s[l]+1)/2, its blocks at d[l], u1[l],
 * l1[l], u2[l], l2[l].  Down: GaussSeidel_2D with GaussIter = 1, then raised
 * by gauss_iter2 per level, the residual b - A x restricted to the coarser
 * level's right-hand side with a zero guess; up: GaussSeidel_2D again (the
 * coarsest twice with the same count), the prolonged coarse guess added to
 * the finer one.  b, x on the finest level as asam_tri_tb_gauss_seidel_2d;
 * x in: the initial guess, out: the result.  nlev <= 32. */
int asam_tri_tb_multigrid_2d(int variant, int nplane, int nlev, const int *n2s, const int *n1s,
                             const double *const *d, const double *const *u1, const double *const *l1,
                             const double *const *u2, const double *const *l2, const double *b, double *x,
                             int gauss_iter2, int mult_iter);
/* Solve_3D of TriDiagTB (variant 0, MULTI/TriDiagTB_Mod.f90:818-952) or
 * TriDiagTR (variant 1, TriDiagTR_Mod.f90:902-1041): mult_iter3 (MultIter3)
 * V-cycles of Multigrid_3D over nlev3 levels, finest first.  Level L has
 * n3s[L] planes of n2s[L] lines of n1s[L] levels (each size halved, rounding
 * up, on the next level), its couplings between planes u3[L], l3[L] as
 * asam_tri_tb_compute_3d writes them (unused when n3s[L] is 1) and its
 * planes' hierarchy of nlev2s[L] plane levels, all planes of plane level m
 * at d[o+m], u1[o+m], l1[o+m], u2[o+m], l2[o+m] with o the sum of
 * nlev2s[0..L-1] (the layout of asam_tri_tb_multigrid_2d's levels; plane
 * level 0 is the level's own planes).  Down: GaussSeidel_3D with GaussIter 1,
 * raised by gauss_iter3 per level -- plane sweeps forward and backward, each
 * plane solved by Solve_2D (gauss_iter2, mult_iter2) from the current guess,
 * then planes 1 and n3 once more -- the residual restricted by RestrictTB_3D,
 * a zero coarse guess; up: GaussSeidel_3D again, the prolonged guess added.
 * b, x [((k*n2 + j)*n1 + i)*2 + r] on the finest level; x in: the initial
 * guess, out: the result.  nlev3 and every nlev2s[L] <= 32. */
int asam_tri_tb_multigrid_3d(int variant, int nlev3, const int *n3s, const int *n2s, const int *n1s, const int *nlev2s,
                             const double *const *u3, const double *const *l3, const double *const *d,
                             const double *const *u1, const double *const *l1, const double *const *u2,
                             const double *const *l2, const double *b, double *x, int gauss_iter2, int mult_iter2,
                             int gauss_iter3, int mult_iter3);

/* The TriDiagTB / TriDiagTR preconditioner of the projection, resident on the
 * device: LaplTBCompute (variant 0) or LaplTRCompute (variant 1,
 * MULTI/JacAccGrav_Mod.f90:1312-1667) builds ref_level levels (RefLevel),
 * level L3 of ceil(n3/2^L3) planes with the plane levels L2 = L3 ..
 * ref_level-1 of ceil(n2/2^L2) x ceil(n1/2^L2), every one from the finest
 * fields coarsened by FaceCoarse, CFaceCoarse, VolCoarse and CVolCoarse
 * (:685-891; shift 0 on level 0 too) and assembled by Compute_3D (with the
 * couplings between planes on the level itself, without them on its plane
 * levels).  Inputs in the reversed index order (n1 the column direction,
 * as ReverseWeight / Reverse leave them): faces[0..3] = F1, F1G, DTU1, DUU1
 * [(k*n2 + j)*(n1+1) + i], faces[4..7] = F2, F2G, DTU2, DUU2
 * [(k*(n2+1) + j)*n1 + i], faces[8..11] = F3, F3G, DTU3, DUU3
 * [(k*n2 + j)*n1 + i] (k to n3), vol = VolG, dut = DUTG, dur = DURG
 * (variant 1 only) [(k*n2 + j)*n1 + i]; coefs as asam_tri_tb_compute_3d.
 * 1 <= ref_level <= 24. */
typedef struct asam_tri_tb_hier asam_tri_tb_hier;
int asam_tri_tb_hier_create(int variant, int ref_level, int n3, int n2, int n1, const asam_tri_tb_coefs *coefs,
                            const double *const *faces, const double *vol, const double *dut, const double *dur,
                            asam_tri_tb_hier **out);
/* one assembled array of the hierarchy (tests): which 0..6 = d, u1, l1, u2,
 * l2, u3, l3 of plane level level2 of level level3 (u3, l3 only for
 * level2 == level3), in the layouts of asam_tri_tb_compute_3d */
int asam_tri_tb_hier_get(const asam_tri_tb_hier *h, int level3, int level2, int which, double *dst);
/* mult_iter3 V-cycles of Multigrid_3D over the hierarchy (asam_tri_tb_multigrid_3d);
 * VCycleCG (JacAccGrav_Mod.f90:4502-4515) runs one from x = 0. */
int asam_tri_tb_hier_vcycle(asam_tri_tb_hier *h, const double *b, double *x, int gauss_iter2, int mult_iter2,
                            int gauss_iter3, int mult_iter3);
/* on != 0: the smoothers of later V-cycles in zebra order, the GPU's parallel
 * order -- per Gauss-Seidel iteration the lines (planes) of parity 0 with
 * the forward right-hand side, parity 1 forward, parity 1 backward, parity 0
 * backward, all lines (planes) of one parity at once, then the reference's
 * closing solves; every relaxation is the reference's arithmetic, only the
 * order of the lines and planes differs.  0 (the default): the reference's
 * sequential order. */
int asam_tri_tb_hier_set_zebra(asam_tri_tb_hier *h, int on);
void asam_tri_tb_hier_destroy(asam_tri_tb_hier *h);

/* y = A x for the same blocks: MatVecTB_1D (MULTI/TriDiagTB_Mod.f90:121-141),
 * the same as MatVecTR_1D (MULTI/TriDiagTR_Mod.f90:133-153). */
int asam_tri_tb_matvec(int ncol, int n1, const double *d, const double *u, const double *l, const double *x,
                       double *y);

/* ---- Restart files (INIT/Restart_Mod.f90:14-82) --------------------------
 * The file of one rank as WriteRestart writes it with gfortran: unformatted
 * sequential records (4-byte length markers, records above the maximum
 * subrecord length split into subrecords), REAL 8 bytes, INTEGER 4 bytes:
 * Time, GMVStep, OutputTime, then per block one record per component
 * (Vec(ib)%Vec(ic)%c, the padded cell array with its nFrac extent) and one
 * record holding uF, vF, wF.  Every array may live in device or host memory;
 * device arrays are staged through pinned buffers. */
typedef struct {
  double time;        /* Time */
  int gmv_step;       /* GetGMVStep() / SetGMVStep */
  double output_time; /* GetOutputTime() / SetOutputTime */
} asam_restart_header;

typedef struct {
  int nx, ny, nz; /* interior cells of the block (ix1-ix0, iy1-iy0, iz1-iz0) */
  int ncomp;      /* UBOUND(Vec(ibLoc)%Vec,1) */
  int nfrac;      /* 4th extent of each component's c array; 0 or 1 without size classes */
  double *c;      /* ncomp arrays of (nx+2)(ny+2)(nz+2)*nfrac values back to back */
  double *uf;     /* uF(ix0:ix1,iy0+1:iy1,iz0+1:iz1) */
  double *vf;     /* vF(ix0+1:ix1,iy0:iy1,iz0+1:iz1) */
  double *wf;     /* wF(ix0+1:ix1,iy0+1:iy1,iz0:iz1) */
} asam_restart_block;

/* WriteRestart (Restart_Mod.f90:14-43) without its RestartTime test: writes
 * the file unconditionally; the caller schedules.  Waits for all device work
 * before reading device arrays. */
int asam_restart_write(const char *path, const asam_restart_header *hdr, int nblock,
                       const asam_restart_block *blocks);

/* ReadRestart (Restart_Mod.f90:45-81): fills hdr and the blocks' arrays;
 * ASAM_IO_ERROR when a record's length differs from the block's array. */
int asam_restart_read(const char *path, asam_restart_header *hdr, int nblock, const asam_restart_block *blocks);

/* The reference's restart file name for a grid file and rank:
 * 'RESTART/'//TRIM(FileName(1:INDEX(FileName,'.grid')))//ADJUSTL(rank)
 * (Restart_Mod.f90:24-27).  cap = size of buf in bytes. */
int asam_restart_file_name(const char *grid_file, int rank, char *buf, int cap);

/* gfortran's -fmax-subrecord-length for files this library writes (default
 * and maximum 2147483639 bytes); the reader accepts any split. */
int asam_restart_set_max_subrecord(long long bytes);

/* ---- Cut-cell geometry files (.Weight2) ----------------------------------
 * ReadWeights (INIT/ReadWeights_Mod.f90:568-1330) and WriteWeightBlk
 * (GRID/OutputWeightBlk_Mod.f90:501-670) for Cartesian grids: Fortran
 * list-directed text holding per block the origin, the cell widths, the face
 * areas and cell volumes that differ from the reader's Cartesian defaults,
 * the cut-face midpoints and the boundary cells with their surface data.
 * Host arrays only (ASAM_BAD_ARG for device memory).  Layouts of the weights
 * as in the block's fields: FU (nx+3)*ny*nz, FV nx*(ny+3)*nz, FW
 * nx*ny*(nz+3), VolC (nx+2)*(ny+2)*(nz+2), ix fastest. */
typedef struct {
  int nx, ny, nz;        /* interior cells */
  double origin[3];      /* x0 y0 z0 */
  double *dx, *dy, *dz;  /* nx, ny, nz cell widths */
  double *fu, *fv, *fw;  /* face areas (WeiFU/WeiFV/WeiFW) */
  double *volc;          /* cell volumes */
  int nmid[3];           /* cut-face midpoints of the YZ, ZX and XY faces */
  int *mid_ijk[3];       /* 3*nmid[d]: ix iy iz */
  double *mid_xs[3];     /* 3*nmid[d]: xS yS zS */
  int nbound;            /* NrB_Cells */
  int struct_bound;      /* 0-6: what follows the six surface values of a boundary cell */
  int nsoil;             /* soil layers per boundary cell in soil_type */
  int *bound_ijk;        /* 3*nbound: ix iy iz (1-based) */
  double *bound_xs;      /* 3*nbound: xS yS zS */
  double *bound_surf;    /* 6*nbound: zRauh alb ee xFLS yFLS zFLS */
  int *land_class;       /* nbound: LandClass */
  int *soil_type;        /* nbound*nsoil: SoilType(1:nsoil) */
  double *normal;        /* 3*nbound: n1 n2 n3 (reader output) */
  double *fl, *dl;       /* nbound each: FL, dL (reader output) */
} asam_weight2_block;

typedef struct {
  int periodic[3];    /* 1: the side pair is periodic (the halo volumes' defaults depend on it) */
  int nr_soil_layers; /* Domain%nrsoillayers (#NrSoilLayers, default 7; at most 57) */
  int land_class_def; /* LandClassDef (default 5) */
  int real_island;    /* RealIsland: a boundary cell of full volume becomes sea (class 9) */
  int expect[3];      /* the caller's nx ny nz ('Error WeightFile' when the file differs); 0 = any */
} asam_weight2_options;

typedef struct asam_weight2_file asam_weight2_file;

/* ReadWeights for block ib (1-based): parses the file into *out and fills
 * info's sizes (nx ny nz, origin, nmid, nbound, struct_bound, nsoil; its
 * pointers are zeroed).  ASAM_IO_ERROR for a file that is short, malformed
 * or does not fit (an index outside the block, 'Error WeightFile'),
 * ASAM_UNSUPPORTED for Globe/Cyl grids and Struct_Bound above 6. */
int asam_weight2_open(const char *path, int ib, const asam_weight2_options *opt, asam_weight2_file **out,
                      asam_weight2_block *info);

/* Copies the block read by asam_weight2_open into dst's arrays, sized from
 * its info; a NULL pointer skips that array.  Also the normal, area and wall
 * distance of each boundary cell (ReadWeights_Mod.f90:1283-1319). */
int asam_weight2_fetch(const asam_weight2_file *f, const asam_weight2_block *dst);

void asam_weight2_close(asam_weight2_file *f);

/* WriteWeightBlk for nblock blocks: lists the weights that differ from the
 * reader's defaults for the given periodicity, each as the shortest decimal
 * that reads back to the same double; the blocks' normal/fl/dl are unused. */
int asam_weight2_write(const char *path, int nblock, const asam_weight2_block *blocks, const int periodic[3]);

/* Sizes of the padded cell field for a configuration. */
long long asam_npad(const asam_config *cfg);

/* Number of CUDA kernels this library has launched since it was loaded
 * (diagnostic; no reference counterpart). */
long long asam_launch_count(void);

/* Text of the last error (thread-local). */
const char *asam_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* ASAM_GB300_H */
