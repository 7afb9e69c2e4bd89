"""GB300-native implicit Rosenbrock transport stage of ASAM (All Scale Atmospheric Model).

Python host mirror of the reference's Fortran seams for this path, on top of
the C-ABI in ``include/asam_gb300.h``.  Method names follow the reference:

=====================  =======================================================
``Fcn``                FcnMet advection terms (ADVECT/Function_Mod.f90:989)
``DivCompute``         ADVECT/Advection_Mod.f90:2901
``Jac``                JacMeteo -> JacAdvectionCompute + JacScaleCompute
                       (ADVECT/Function_Mod.f90:1508, 1782)
``MatVecMet``          MODULE/SpMatrix4CellPar_Mod.f90:70
``PSolve``             MODULE/SpMatrix4CellPar_Mod.f90:86
``BiCGStabMetSp``      MODULE/SpMatrix4CellPar_Mod.f90:245 (MaxIter/Tol in-out)
``Ros3MetC``           ADVECT/Int_Mod.f90:1059 (fixed dt)
``TotalScalar``        ADVECT/Diagnostic_Mod.f90:13
``ExchangeCell``       MODULE/Vector4CellPar_Mod.f90:752
``BoundaryCondition``  ADVECT/BoundaryCondition_Mod.f90:1143 (outer-wall halos)
``JacAccGrav``         pressure-Laplacian hierarchy, LaplTFullCompute
                       (MULTI/JacAccGrav_Mod.f90:1056)
``MatVecP``            MULTI/JacAccGrav_Mod.f90:531 (MatVecP_Tri)
``VCycleCG``           MULTI/JacAccGrav_Mod.f90:4466 (one Solve_3D)
``SolveSound``         SOLU/Iter_Mod.f90:9 (FGMRES, MatVec1, PSolve1)
``ProjectVelFace``     ADVECT/IntSub_Mod.f90:25
``VelocityFaceToCellLR``  ADVECT/VelocityCellFace_Mod.f90:72
``VelocityCellToFaceLR``  ADVECT/VelocityCellFace_Mod.f90:27
``AbsTPreCompute``     AbsTCompute + PreCompute (ADVECT/Diagnostic_Mod.f90:593, 710)
``FcnMet``             FcnMet with PGradComputeC and buoyancy (ADVECT/Function_Mod.f90:989)
``Ros3MetC_dyn``       Ros3MetC + StageRos with prognostic momentum (ADVECT/Int_Mod.f90:263)
``Solve_1D``           MULTI/TriDiagT_Mod.f90:135 (batched over columns)
``MatVecT_1D``         MULTI/TriDiagT_Mod.f90:113 (batched over columns)
=====================  =======================================================

Fields are numpy arrays in the Fortran layout (ix fastest): a state is
``(ncomp, nz+2, ny+2, nx+2)`` float64, C-contiguous.  All compute runs in the
CUDA library; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import (ASAM_BREAKDOWN, ASAM_CUDA_ERROR, ASAM_NOT_CONVERGED, ASAM_OK, AsamConfig, AsamDynConfig, AsamError, AsamProjConfig,
                   check, ptr)

METHODS = {"Ros3AMF": 0, "RosRK32": 1, "RosEul": 2, "Ros3P": 3, "Ros3Pw": 4, "RosRK3": 5, "RosTVD": 6,
           "RosRK4": 7}
PRECISIONS = {"fp64": 0, "fp32_refined": 1}
INNER_PRECONDS = {"gauss_seidel": 0, "line": 1, "xline": 2, "yline": 3}
GS_SCHEDULES = {"persistent": 0, "levels": 1}

__all__ = ["TransportBlock", "Solve_1D", "MatVecT_1D", "ros_coeffs", "METHODS", "PRECISIONS", "AsamError"]


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def ros_coeffs(method: str | int):
    """InitRos3MetC coefficient tables (ADVECT/Int_Mod.f90:78-261): (nStage, beta0, alpha, beta, gamma1)."""
    lib = _lib.load()
    m = METHODS[method] if isinstance(method, str) else int(method)
    b0 = C.c_double()
    al = np.zeros(16)
    be = np.zeros(16)
    gm = np.zeros(5)
    n = lib.asam_ros_coeffs(m, C.byref(b0), al.ctypes.data_as(_lib._D), be.ctypes.data_as(_lib._D),
                            gm.ctypes.data_as(_lib._D))
    if n <= 0:
        raise ValueError(f"unknown Rosenbrock method {method!r}")
    return n, b0.value, al.reshape(4, 4), be.reshape(4, 4), gm


class TransportBlock:
    """One ASAM block (``Floor(ib)``) resident on the GPU: geometry, face velocities,
    the 7-diagonal stage matrix and the Krylov work space."""

    def __init__(self, geo, ncomp: int, rho_pos: int = 0, method: str = "RosRK3", bicgstab_tol: float = 1e-6,
                 bicgstab_maxiter: int = 30, gs_iter: int = 5, precision: str = "fp64",
                 inner_precond: str = "gauss_seidel", inner_gs_iter: int = 1, gs_schedule: str = "persistent",
                 gs_group: int = 0):
        self.lib = _lib.load()
        g = geo.grid
        self.grid = g
        self.ncomp = ncomp
        self.cfg = AsamConfig(g.nx, g.ny, g.nz, int(g.periodic_x), int(g.periodic_y), int(g.periodic_z), ncomp,
                              rho_pos, METHODS[method], bicgstab_maxiter, bicgstab_tol, gs_iter,
                              PRECISIONS[precision], INNER_PRECONDS[inner_precond], inner_gs_iter,
                              GS_SCHEDULES[gs_schedule], gs_group)
        self._geo = [_f64(geo.volc), _f64(geo.fu), _f64(geo.fv), _f64(geo.fw)]
        h = C.c_void_p()
        check(self.lib.asam_create(C.byref(self.cfg), *(ptr(a) for a in self._geo), C.byref(h)), "asam_create")
        self.h = h
        self.nstage = ros_coeffs(method)[0]

    # -- lifetime -------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.asam_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def state_shape(self):
        g = self.grid
        return (self.ncomp, g.nz + 2, g.ny + 2, g.nx + 2)

    def _state(self, c) -> np.ndarray:
        a = _f64(c)
        if a.size != self.ncomp * self.grid.npad:
            raise ValueError(f"state must have {self.ncomp}*npad elements")
        return a

    def set_graphs(self, mode):
        """0/False: launch every kernel; 1/True (default): replay the BiCGStab
        half-iterations from CUDA graphs; 2: steps as one device-driven graph
        (WHILE nodes for the Krylov loops; refined contexts: the FP64
        refinement as an outer WHILE node).  The results are the same."""
        check(self.lib.asam_set_graphs(self.h, int(mode)), "asam_set_graphs")

    def set_stream(self, stream_handle: int | None):
        """cudaStream_t as an integer; 0/None selects the legacy default stream."""
        check(self.lib.asam_set_stream(self.h, stream_handle or None), "asam_set_stream")

    def state_device_ptr(self) -> int:
        p = C.c_void_p()
        check(self.lib.asam_state_device_ptr(self.h, C.byref(p)), "asam_state_device_ptr")
        return p.value

    def synchronize(self):
        check(self.lib.asam_synchronize(self.h), "asam_synchronize")

    # -- reference seams ------------------------------------------------------------
    def set_velocity(self, uf, vf, wf):
        self._vel = [_f64(uf), _f64(vf), _f64(wf)]
        check(self.lib.asam_set_velocity(self.h, *(ptr(a) for a in self._vel)), "asam_set_velocity")

    def ExchangeCell(self, c: np.ndarray, ncomp: int | None = None) -> np.ndarray:
        a = _f64(c).copy()
        n = ncomp if ncomp is not None else a.size // self.grid.npad
        check(self.lib.asam_exchange_cell(self.h, n, ptr(a)), "asam_exchange_cell")
        return a

    def set_boundary(self, kinds):
        """Halo rule of the outer walls, applied to the state at the start of
        every stage (BoundaryCondition / BoundaryVelocity, ADVECT/Int_Mod.f90:
        283-287): (ncomp, 6) ints, sides W,E,S,N,B,T, 0 none, 1 ZeroGrad,
        2 ZeroValue, and the open-boundary kinds of BoundaryCompute
        (ADVECT/BoundaryCondition_Mod.f90:70-346) 3 MeanValue, 4 Function,
        5 InFlowOutFlow (lateral sides), 6 Extrapolation (bottom and top),
        whose data come from set_boundary_data first.  A new block has
        ZeroGrad everywhere."""
        k = np.ascontiguousarray(kinds, dtype=np.int32).reshape(-1)
        if k.size != 6 * self.ncomp:
            raise ValueError("kinds must have 6 entries per component")
        check(self.lib.asam_set_boundary(self.h, k.ctypes.data_as(C.POINTER(C.c_int))), "asam_set_boundary")

    def set_boundary_data(self, mean_profile=None, function_values=None, ambient=None):
        """Data of the open-boundary kinds: MeanProfile (ncomp, nz), the
        Function values F at the halo cells and the ambient state VecAmb
        (ncomp padded fields each); None drops an array."""
        g = self.grid
        arrs = []
        for a, n in ((mean_profile, self.ncomp * g.nz), (function_values, self.ncomp * g.npad),
                     (ambient, self.ncomp * g.npad)):
            if a is None:
                arrs.append(None)
                continue
            a = _f64(a).reshape(-1)
            if a.size != n:
                raise ValueError(f"boundary data of {a.size} values, expected {n}")
            arrs.append(a)
        check(self.lib.asam_set_boundary_data(self.h, *[None if a is None else ptr(a) for a in arrs]),
              "asam_set_boundary_data")

    def set_diffusion(self, dh, dv=None, jac: bool = True):
        """Diffusion of every component with coefficients DH, DV (padded cell
        fields; DV defaults to DH), or None to switch it off; jac adds the
        diffusion Jacobian to the stage matrix."""
        if dh is None:
            self._diff = None
            check(self.lib.asam_set_diffusion(self.h, None, None, 0), "asam_set_diffusion")
            return
        self._diff = (_f64(dh), None if dv is None else _f64(dv))
        check(self.lib.asam_set_diffusion(self.h, ptr(self._diff[0]), None if dv is None else ptr(self._diff[1]),
                                          int(bool(jac))), "asam_set_diffusion")

    def BoundaryCondition(self, c: np.ndarray) -> np.ndarray:
        a = self._state(c).copy()
        check(self.lib.asam_boundary_condition(self.h, ptr(a)), "asam_boundary_condition")
        return a

    def Fcn(self, c: np.ndarray) -> np.ndarray:
        a = self._state(c)
        f = np.empty_like(a)
        check(self.lib.asam_fcn(self.h, ptr(a), ptr(f)), "asam_fcn")
        return f

    def DivCompute(self, rhs: np.ndarray) -> np.ndarray:
        a = _f64(rhs).copy()
        check(self.lib.asam_div(self.h, ptr(a)), "asam_div")
        return a

    def Jac(self, c: np.ndarray, dt: float):
        a = self._state(c)
        check(self.lib.asam_jac(self.h, ptr(a), float(dt)), "asam_jac")

    def jac_matrix(self) -> np.ndarray:
        val = np.empty((7, self.grid.npad))
        check(self.lib.asam_get_jac(self.h, ptr(val)), "asam_get_jac")
        return val

    def set_jac_matrix(self, val: np.ndarray):
        v = _f64(val)
        check(self.lib.asam_set_jac(self.h, ptr(v)), "asam_set_jac")

    def MatVecMet(self, x: np.ndarray) -> np.ndarray:
        a = self._state(x)
        y = np.empty_like(a)
        check(self.lib.asam_matvec(self.h, ptr(a), ptr(y)), "asam_matvec")
        return y

    def PSolve(self, x: np.ndarray) -> np.ndarray:
        a = self._state(x)
        y = np.empty_like(a)
        check(self.lib.asam_psolve(self.h, ptr(a), ptr(y)), "asam_psolve")
        return y

    def autotune(self, c, dt: float) -> dict:
        """Pick this block's solver settings (asam_autotune): the refined mode's
        inner solver and, for either precision, the CUDA-graph replay of the
        Krylov iterations.  c: host state array or device pointer (int)."""
        choice = (C.c_int * 5)()
        ms = C.c_double()
        p = C.c_void_p(c) if isinstance(c, int) else ptr(self._state(c))
        check(self.lib.asam_autotune(self.h, p, float(dt), choice, C.byref(ms)), "asam_autotune")
        names = {v: k for k, v in INNER_PRECONDS.items()}
        scheds = {v: k for k, v in GS_SCHEDULES.items()}
        return {"inner_precond": names[choice[0]], "inner_gs_iter": choice[1], "gs_schedule": scheds[choice[2]],
                "gs_group": choice[3], "graphs": bool(choice[4]), "stage_solve_ms": ms.value}

    def inner_psolve(self, x: np.ndarray) -> np.ndarray:
        """The refined mode's FP32 inner preconditioner applied to x (no reference
        counterpart; for tests and measurement)."""
        a = self._state(x)
        y = np.empty_like(a)
        check(self.lib.asam_inner_psolve(self.h, ptr(a), ptr(y)), "asam_inner_psolve")
        return y

    def set_wait_limit(self, polls: int):
        """Polls of one dependency wait of the persistent Gauss-Seidel schedule
        before its CTA gives up (0: the default); a wait that runs out makes
        the call raise AsamError (ASAM_CUDA_ERROR) and leaves the context
        usable.  Diagnostic, no reference counterpart."""
        check(self.lib.asam_set_wait_limit(self.h, int(polls)), "asam_set_wait_limit")

    def BiCGStabMetSp(self, x: np.ndarray, b: np.ndarray, MaxIter: int, Tol: float):
        """Solve A x = b in place of x; returns (MaxIter, Tol) with the reference's
        sentinels (negative: converged at the half step; 2*Iter: limit hit)."""
        if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous):
            raise TypeError("x must be a C-contiguous float64 array (updated in place)")
        bb = self._state(b)
        it = C.c_int(int(MaxIter))
        tol = C.c_double(float(Tol))
        st = self.lib.asam_bicgstab(self.h, ptr(x), ptr(bb), C.byref(it), C.byref(tol))
        check(st, "asam_bicgstab", allow=(ASAM_OK, ASAM_NOT_CONVERGED, ASAM_BREAKDOWN))
        return it.value, tol.value

    def Ros3MetC(self, c: np.ndarray, dt: float):
        """One fixed-dt Rosenbrock step of state c (updated in place).  Returns the
        per-stage BiCGStab (MaxIter, Tol) outputs."""
        if not (isinstance(c, np.ndarray) and c.dtype == np.float64 and c.flags.c_contiguous):
            raise TypeError("c must be a C-contiguous float64 array (updated in place)")
        iters = (C.c_int * 4)()
        resid = (C.c_double * 4)()
        st = self.lib.asam_ros_step(self.h, ptr(c), float(dt), iters, resid)
        check(st, "asam_ros_step", allow=(ASAM_OK, ASAM_NOT_CONVERGED, ASAM_BREAKDOWN))
        return [iters[i] for i in range(self.nstage)], [resid[i] for i in range(self.nstage)]

    def ros_step_device(self, dptr: int, dt: float):
        """Rosenbrock step on a device-resident state (no host copies)."""
        iters = (C.c_int * 4)()
        resid = (C.c_double * 4)()
        st = self.lib.asam_ros_step(self.h, C.c_void_p(dptr), float(dt), iters, resid)
        check(st, "asam_ros_step", allow=(ASAM_OK, ASAM_NOT_CONVERGED, ASAM_BREAKDOWN))
        return [iters[i] for i in range(self.nstage)], [resid[i] for i in range(self.nstage)]

    def state_dot(self, c) -> float:
        """DOT(VecMet,VecMet) over all components (the driver's NaN check);
        raises AsamError (ASAM_NAN_DETECTED) when it is NaN."""
        a = self._state(c)
        out = C.c_double()
        check(self.lib.asam_state_dot(self.h, ptr(a), C.byref(out)), "asam_state_dot")
        return out.value

    def TotalScalar(self, c: np.ndarray, comp: int = 0) -> float:
        a = self._state(c)
        out = C.c_double()
        check(self.lib.asam_total_scalar(self.h, ptr(a), int(comp), C.byref(out)), "asam_total_scalar")
        return out.value

    # ---- pressure projection (closed or periodic sides) ----------------------
    def proj_setup(self, dx, dy, dz, metr=None, ref_level: int = 4, gauss_iter2: int = 1, gauss_iter3: int = 1,
                   mult_iter2: int = 1, mult_iter3: int = 1, step_gmres: int = 10, max_restart: int = 10,
                   tol: float = 1e-6, fac_anela: float = 1.0, prefac2: float = 0.5):
        """Projection set-up: cell widths dx[nx], dy[ny], dz[nz]; metr the six
        metric arrays MetrXY, MetrXZ, MetrYX, MetrYZ, MetrZX, MetrZY back to
        back (None: Cartesian).  Defaults are Control_Mod's.  A block with
        periodic sides carries boundary face unknowns: its PressureVelocity
        vectors (SolveSound, MatVec1, PSolve1) are flat arrays of
        ``proj_nvec`` values, the pressure followed by u_w, u_e, v_s, v_n,
        w_b, w_t of the periodic sides."""
        g = self.grid
        self._pdx, self._pdy, self._pdz = _f64(dx), _f64(dy), _f64(dz)
        if self._pdx.size != g.nx or self._pdy.size != g.ny or self._pdz.size != g.nz:
            raise ValueError("dx, dy, dz must have nx, ny, nz entries")
        self._pmetr = None if metr is None else _f64(metr)
        if self._pmetr is not None and self._pmetr.size != 2 * (g.nx + g.ny + g.nz):
            raise ValueError("metr must hold 2*(nx+ny+nz) values")
        self.pcfg = AsamProjConfig(ref_level, gauss_iter2, gauss_iter3, mult_iter2, mult_iter3, step_gmres, max_restart,
                                   tol, fac_anela, prefac2)
        check(self.lib.asam_proj_setup(self.h, C.byref(self.pcfg), ptr(self._pdx), ptr(self._pdy), ptr(self._pdz),
                                       None if self._pmetr is None else ptr(self._pmetr)), "asam_proj_setup")
        self.proj_nface = int(self.lib.asam_proj_face_count(self.h))
        self.proj_nvec = g.nx * g.ny * g.nz + self.proj_nface

    def _pv(self, like=None) -> np.ndarray:
        """An empty PressureVelocity vector ((nz, ny, nx) for a closed block)."""
        g = self.grid
        return np.empty((g.nz, g.ny, g.nx)) if self.proj_nface == 0 else np.empty(self.proj_nvec)

    def MatVec1(self, x) -> np.ndarray:
        """MatVecFull on a PressureVelocity vector (no Exchange)."""
        a = _f64(x)
        y = self._pv()
        check(self.lib.asam_proj_matvec1(self.h, ptr(a), ptr(y)), "asam_proj_matvec1")
        return y

    def PSolve1(self, x) -> np.ndarray:
        """PSolve1 (PressurePre, Schur step, PressurePre) on a PressureVelocity
        vector -- the context's FGMRES preconditioner, so the periodic-Laplacian
        one when proj_set_preconditioner (or the refined default) selects it."""
        a = _f64(x)
        y = self._pv()
        check(self.lib.asam_proj_psolve1(self.h, ptr(a), ptr(y)), "asam_proj_psolve1")
        return y

    def lapl_array_dirichlet(self, level3: int, level2: int, which: int) -> np.ndarray:
        """One array of the Dirichlet hierarchy (periodic blocks)."""
        n = self.lib.asam_lapl_get_dirichlet(self.h, level3, level2, which, None)
        if n < 0:
            raise ValueError("no such level/array (or no Dirichlet hierarchy)")
        out = np.empty(n)
        if self.lib.asam_lapl_get_dirichlet(self.h, level3, level2, which, ptr(out)) != n:
            raise AsamError(4, "asam_lapl_get_dirichlet")
        return out

    def VCycleCG_dirichlet(self, b) -> np.ndarray:
        a = _f64(b)
        x = np.empty_like(a)
        check(self.lib.asam_lapl_vcycle_dirichlet(self.h, ptr(a), ptr(x)), "asam_lapl_vcycle_dirichlet")
        return x

    def proj_set_precision(self, prec):
        """Precision of the FGMRES preconditioner's V-cycle: "fp64" (the
        reference's arithmetic), "fp32" (rounded copy of the hierarchy), or
        None (follow the block's precision)."""
        code = {None: -1, "fp64": 0, "fp32": 1}[prec]
        check(self.lib.asam_proj_set_precision(self.h, code), "asam_proj_set_precision")

    def proj_set_preconditioner(self, kind):
        """FGMRES preconditioner of a block with periodic x/y sides: "psolve1"
        (the reference's PSolve1), "periodic" (one V-cycle on the periodic
        Laplacian, face unknowns eliminated), or None (periodic for refined
        contexts, else PSolve1).  Takes effect at the next JacAccGrav."""
        code = {None: -1, "psolve1": 0, "periodic": 1}[kind]
        check(self.lib.asam_proj_set_preconditioner(self.h, code), "asam_proj_set_preconditioner")

    def proj_set_pre_schedule(self, gauss_iter2: int = 0, gauss_iter3: int = 0):
        """Sweep growth per level (GaussIter2, GaussIter3) of the periodic
        preconditioner's V-cycle; 0, 0 (the default) smooths every level once."""
        check(self.lib.asam_proj_set_pre_schedule(self.h, int(gauss_iter2), int(gauss_iter3)),
              "asam_proj_set_pre_schedule")

    def proj_weights(self, dtu, dtv, dtw, duu, duv, duw, dut, dtt):
        """Sound weights (WeightDiagCompute): face arrays with uF/vF/wF extents,
        DUT and DTT interior (nz, ny, nx)."""
        arrs = [_f64(a) for a in (dtu, dtv, dtw, duu, duv, duw, dut, dtt)]
        check(self.lib.asam_proj_weights(self.h, *[ptr(a) for a in arrs]), "asam_proj_weights")

    def WeightDiagCompute(self, state, tabs, th_pos: int, rho_pos: int, rv_pos: int = -1, rc_pos: int = -1,
                          rr_pos: int = -1):
        """Sound weights of ThetaKind='Density' from the state and the absolute
        temperature (padded), computed on the device."""
        st = self._state(state)
        t = _f64(tabs)
        check(self.lib.asam_proj_weights_density(self.h, ptr(st), th_pos, rho_pos, rv_pos, rc_pos, rr_pos, ptr(t)),
              "asam_proj_weights_density")

    def proj_weight(self, which: int) -> np.ndarray:
        n = self.lib.asam_proj_get_weights(self.h, which, None)
        if n < 0:
            raise ValueError("no weights")
        out = np.empty(n)
        self.lib.asam_proj_get_weights(self.h, which, ptr(out))
        return out

    def JacAccGrav(self, beta0: float, dtp: float):
        """Assemble the tridiagonal pressure-Laplacian hierarchy (LaplTFullCompute)."""
        check(self.lib.asam_lapl_compute(self.h, float(beta0), float(dtp)), "asam_lapl_compute")

    def lapl_array(self, level3: int, level2: int, which: int) -> np.ndarray:
        """One assembled array in the reversed order (see asam_lapl_get)."""
        n = self.lib.asam_lapl_get(self.h, level3, level2, which, None)
        if n < 0:
            raise ValueError("no such level/array")
        out = np.empty(n)
        if self.lib.asam_lapl_get(self.h, level3, level2, which, ptr(out)) != n:
            raise AsamError(4, "asam_lapl_get")
        return out

    def MatVecP(self, x) -> np.ndarray:
        a = _f64(x)
        y = np.empty_like(a)
        check(self.lib.asam_lapl_matvec(self.h, ptr(a), ptr(y)), "asam_lapl_matvec")
        return y

    def VCycleCG(self, b) -> np.ndarray:
        a = _f64(b)
        x = np.empty_like(a)
        check(self.lib.asam_lapl_vcycle(self.h, ptr(a), ptr(x)), "asam_lapl_vcycle")
        return x

    def SolveSound(self, x: np.ndarray, b, MaxIter: int | None = None, Tol: float | None = None):
        """FGMRES on PressureVelocity vectors (the pressure of a closed block),
        x updated in place; returns (inner steps, relative residual estimate)."""
        if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous):
            raise TypeError("x must be a C-contiguous float64 array (updated in place)")
        bb = _f64(b)
        it = C.c_int(int(self.pcfg.max_restart if MaxIter is None else MaxIter))
        tol = C.c_double(float(self.pcfg.tol if Tol is None else Tol))
        st = self.lib.asam_solve_sound(self.h, ptr(x), ptr(bb), C.byref(it), C.byref(tol))
        check(st, "asam_solve_sound", allow=(ASAM_OK, ASAM_NOT_CONVERGED))
        return it.value, tol.value

    def ProjectVelFace(self, uf: np.ndarray, vf: np.ndarray, wf: np.ndarray, incr: np.ndarray, state=None,
                       th_pos: int = -1, rho_pos: int = -1, scalars=()):
        """Project the face-velocity increments uf/vf/wf (updated in place) and
        update the cell increments incr (in place).  Returns (pressure,
        inner steps, relative residual)."""
        for a in (uf, vf, wf, incr):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise TypeError("uf, vf, wf, incr must be C-contiguous float64 arrays (updated in place)")
        st_arr = None if state is None else self._state(state)
        sc = (C.c_int * max(1, len(scalars)))(*scalars)
        g = self.grid
        p = np.empty((g.nz, g.ny, g.nx))
        steps = C.c_int()
        res = C.c_double()
        st = self.lib.asam_project_vel_face(self.h, ptr(uf), ptr(vf), ptr(wf), ptr(incr),
                                            None if st_arr is None else ptr(st_arr), int(th_pos), int(rho_pos), sc,
                                            len(scalars), ptr(p), C.byref(steps), C.byref(res))
        check(st, "asam_project_vel_face", allow=(ASAM_OK, ASAM_NOT_CONVERGED))
        return p, steps.value, res.value

    # -- dynamical-core stage (momentum branch of StageRos) -------------------------
    def dyn_setup(self, th_pos: int, mom_pos, rv_pos: int = -1, rc_pos: int = -1, rr_pos: int = -1,
                  ri_pos: int = -1, pgradient: bool = True, buoyancy: bool = True, free_slip: bool = True,
                  wall_no_slip: bool = False, grav: float = 9.81, bound_cells=None, scalars=()):
        """asam_dyn_setup: component positions (0-based, -1 absent), the
        physics switches, the BoundCell list ((n,3) 1-based interior cells)
        and the DivScalar components of ProjectVelFace.  Needs proj_setup."""
        self.dcfg = AsamDynConfig(int(th_pos), int(rv_pos), int(rc_pos), int(rr_pos), int(ri_pos),
                                  (C.c_int * 6)(*[int(q) for q in mom_pos]), int(bool(pgradient)),
                                  int(bool(buoyancy)), int(bool(free_slip)), int(bool(wall_no_slip)), float(grav))
        bc = np.zeros((0, 3), dtype=np.int32) if bound_cells is None else np.ascontiguousarray(bound_cells,
                                                                                              dtype=np.int32)
        self._bound = bc.reshape(-1, 3)
        sc = (C.c_int * max(1, len(scalars)))(*scalars)
        check(self.lib.asam_dyn_setup(self.h, C.byref(self.dcfg), self._bound.ctypes.data_as(_lib._I),
                                      len(self._bound), sc, len(scalars)), "asam_dyn_setup")

    def VelocityFaceToCellLR(self, uf, vf, wf, c) -> np.ndarray:
        a = self._state(c).copy()
        u, v, w = _f64(uf), _f64(vf), _f64(wf)
        check(self.lib.asam_face_to_cell(self.h, ptr(u), ptr(v), ptr(w), ptr(a)), "asam_face_to_cell")
        return a

    def VelocityCellToFaceLR(self, c):
        a = self._state(c)
        g = self.grid
        u = np.empty((g.nz, g.ny, g.nx + 1))
        v = np.empty((g.nz, g.ny + 1, g.nx))
        w = np.empty((g.nz + 1, g.ny, g.nx))
        check(self.lib.asam_cell_to_face(self.h, ptr(a), ptr(u), ptr(v), ptr(w)), "asam_cell_to_face")
        return u, v, w

    def AbsTPreCompute(self, c):
        """AbsTCompute ('Density') and PreCompute: (TAbsCell, PreCell), padded."""
        a = self._state(c)
        t = np.empty(self.grid.pshape)
        p = np.empty(self.grid.pshape)
        check(self.lib.asam_thermo(self.h, ptr(a), ptr(t), ptr(p)), "asam_thermo")
        return t, p

    def FcnMet(self, c, pre) -> np.ndarray:
        """FcnMet of the dynamical stage: advection, pressure gradient, scale, buoyancy."""
        a = self._state(c)
        pp = _f64(pre)
        f = np.empty_like(a)
        check(self.lib.asam_fcn_dyn(self.h, ptr(a), ptr(pp), ptr(f)), "asam_fcn_dyn")
        return f

    def Ros3MetC_dyn(self, c: np.ndarray, dt: float):
        """One Rosenbrock step of the dynamical core: c (in place) and the
        block's face velocities advance.  Returns (BiCGStab (iters, resid),
        FGMRES (steps, relative residual)) per stage."""
        if not (isinstance(c, np.ndarray) and c.dtype == np.float64 and c.flags.c_contiguous):
            raise TypeError("c must be a C-contiguous float64 array (updated in place)")
        it = (C.c_int * 4)()
        rs = (C.c_double * 4)()
        ps = (C.c_int * 4)()
        pr = (C.c_double * 4)()
        st = self.lib.asam_ros_step_dyn(self.h, ptr(c), float(dt), it, rs, ps, pr)
        check(st, "asam_ros_step_dyn", allow=(ASAM_OK, ASAM_NOT_CONVERGED, ASAM_BREAKDOWN))
        n = self.nstage
        return (list(it[:n]), list(rs[:n])), (list(ps[:n]), list(pr[:n]))

    def get_velocity(self):
        g = self.grid
        u = np.empty((g.nz, g.ny, g.nx + 1))
        v = np.empty((g.nz, g.ny + 1, g.nx))
        w = np.empty((g.nz + 1, g.ny, g.nx))
        check(self.lib.asam_get_velocity(self.h, ptr(u), ptr(v), ptr(w)), "asam_get_velocity")
        return u, v, w


class Batch:
    """Independent blocks advanced together on one GPU (asam_batch_*): each member
    keeps its own geometry, wind, configuration and stream; the members' steps
    run concurrently."""

    def __init__(self, blocks, nthreads: int = 0):
        self.lib = _lib.load()
        self.blocks = list(blocks)
        arr = (C.c_void_p * len(self.blocks))(*[b.h.value for b in self.blocks])
        h = C.c_void_p()
        check(self.lib.asam_batch_create(len(self.blocks), arr, int(nthreads), C.byref(h)), "asam_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.asam_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_graph(self, on: bool = True):
        """One-graph mode (members with their own streams): a call records
        the whole run -- nsteps device-driven steps of every member -- as one
        CUDA graph with one branch per member (kept while the states, step
        sizes and step count stay the same) and launches it once."""
        check(self.lib.asam_batch_set_graph(self.h, int(bool(on))), "asam_batch_set_graph")

    def ros_step(self, states, dt, nsteps: int = 1):
        """Advance every member nsteps steps.  states: per member a C-contiguous
        float64 host array (updated in place) or a device pointer (int); dt: one
        value or one per member.  Returns (iters[m][step][stage], status[m])."""
        n = len(self.blocks)
        if len(states) != n:
            raise ValueError(f"expected {n} states")
        ptrs = []
        for b, c in zip(self.blocks, states):
            if isinstance(c, int):
                ptrs.append(c)
            else:
                if not (isinstance(c, np.ndarray) and c.dtype == np.float64 and c.flags.c_contiguous):
                    raise TypeError("states must be C-contiguous float64 arrays (updated in place) or device pointers")
                b._state(c)
                ptrs.append(c.ctypes.data)
        parr = (C.c_void_p * n)(*ptrs)
        dts = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (n,)))
        iters = np.zeros((n, nsteps, 4), dtype=np.int32)
        resid = np.zeros((n, nsteps, 4), dtype=np.float64)
        status = np.zeros(n, dtype=np.int32)
        rc = self.lib.asam_batch_ros_step(self.h, parr, dts.ctypes.data_as(_lib._D), int(nsteps),
                                          iters.ctypes.data_as(_lib._I), resid.ctypes.data_as(_lib._D),
                                          status.ctypes.data_as(_lib._I))
        check(rc, "asam_batch_ros_step", allow=(ASAM_OK, ASAM_NOT_CONVERGED, ASAM_BREAKDOWN))
        its = [[list(iters[m, s, :b.nstage]) for s in range(nsteps)] for m, b in enumerate(self.blocks)]
        return its, status


def Solve_1D(d: np.ndarray, u: np.ndarray, l: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Thomas solve of a batch of columns: d,b (ncol,n1); u,l (ncol,n1-1)."""
    lib = _lib.load()
    d, u, l, x = _f64(d), _f64(u), _f64(l), _f64(b).copy()
    ncol, n1 = d.shape
    check(lib.asam_tri_solve(ncol, n1, ptr(d), ptr(u), ptr(l), ptr(x)), "asam_tri_solve")
    return x


def Solve_TB_1D(d: np.ndarray, u: np.ndarray, l: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Block Thomas solve of TriDiagTB (2x2 blocks) on a batch of columns:
    d (ncol,n1,4), u,l (ncol,n1-1,4) with blocks column-major, b (ncol,n1,2)."""
    lib = _lib.load()
    d, u, l, x = _f64(d), _f64(u), _f64(l), _f64(b).copy()
    ncol, n1 = d.shape[:2]
    check(lib.asam_tri_tb_solve(ncol, n1, ptr(d), ptr(u), ptr(l), ptr(x)), "asam_tri_tb_solve")
    return x


def Compute_TB_1D(f, fg, vol, dtu, duu, dut, dur=None, beta0_dtp: float = 1.0, fac1_l: float = 0.0,
                  fac1_r: float = 0.0, grav_comp: float = 0.0, fac_anela: float = 0.0):
    """Allocate_1D + Compute_1D of TriDiagTB (dur None) or TriDiagTR (dur
    given) on a batch of columns: faces f, fg, dtu, duu (ncol, n1+1), cells
    vol, dut, dur (ncol, n1).  Returns d (ncol,n1,4), u, l (ncol,n1-1,4)."""
    lib = _lib.load()
    faces = [_f64(a) for a in (f, fg, dtu, duu)]
    cells = [_f64(a) for a in (vol, dut)] + ([_f64(dur)] if dur is not None else [])
    ncol, n1 = cells[0].shape
    if any(a.shape != (ncol, n1 + 1) for a in faces) or any(a.shape != (ncol, n1) for a in cells):
        raise ValueError("faces (ncol, n1+1), cells (ncol, n1)")
    d = np.empty((ncol, n1, 4))
    u = np.empty((ncol, max(n1 - 1, 0), 4))
    l = np.empty_like(u)
    co = _lib.AsamTriTbCoefs(beta0_dtp, fac1_l, fac1_r, grav_comp, fac_anela)
    check(lib.asam_tri_tb_compute(int(dur is not None), ncol, n1, C.byref(co), *[ptr(a) for a in faces[:2]],
                                  ptr(cells[0]), ptr(faces[2]), ptr(faces[3]), ptr(cells[1]),
                                  ptr(cells[2]) if dur is not None else None, ptr(d),
                                  ptr(u) if u.size else None, ptr(l) if l.size else None), "asam_tri_tb_compute")
    return d, u, l


def Compute_TB_2D(z_faces, x_faces, vol, dut, dur=None, beta0_dtp: float = 1.0, fac1_l: float = 0.0,
                  fac1_r: float = 0.0, grav_comp: float = 0.0, fac_anela: float = 0.0, fac2_l: float = 0.0,
                  fac2_r: float = 0.0):
    """Allocate_2D + Compute_2D of TriDiagTB (dur None) or TriDiagTR on a batch
    of planes: z_faces = (F1, F1G, DTU1, DUU1) (nplane, n2, n1+1), x_faces =
    (F2, F2G, DTU2, DUU2) (nplane, n2+1, n1), cells vol, dut, dur (nplane, n2,
    n1).  Returns d, u1, l1 (the lines) and u2, l2 (between lines)."""
    lib = _lib.load()
    zf = [_f64(a) for a in z_faces]
    xf = [_f64(a) for a in x_faces]
    cells = [_f64(a) for a in (vol, dut)] + ([_f64(dur)] if dur is not None else [])
    nplane, n2, n1 = cells[0].shape
    if (any(a.shape != (nplane, n2, n1 + 1) for a in zf) or any(a.shape != (nplane, n2 + 1, n1) for a in xf)
            or any(a.shape != (nplane, n2, n1) for a in cells)):
        raise ValueError("z faces (nplane, n2, n1+1), x faces (nplane, n2+1, n1), cells (nplane, n2, n1)")
    d = np.empty((nplane, n2, n1, 4))
    u1 = np.empty((nplane, n2, max(n1 - 1, 0), 4))
    l1 = np.empty_like(u1)
    u2 = np.empty((nplane, max(n2 - 1, 0), n1, 4))
    l2 = np.empty_like(u2)
    co = _lib.AsamTriTbCoefs(beta0_dtp, fac1_l, fac1_r, grav_comp, fac_anela, fac2_l, fac2_r)
    opt = lambda a: ptr(a) if a.size else None  # noqa: E731
    check(lib.asam_tri_tb_compute_2d(int(dur is not None), nplane, n2, n1, C.byref(co), *[ptr(a) for a in zf],
                                     *[ptr(a) for a in xf], ptr(cells[0]), ptr(cells[1]),
                                     ptr(cells[2]) if dur is not None else None, ptr(d), opt(u1), opt(l1), opt(u2),
                                     opt(l2)), "asam_tri_tb_compute_2d")
    return d, u1, l1, u2, l2


def Compute_TB_3D(z_faces, x_faces, y_faces, vol, dut, dur=None, couple: bool = True, **coefs):
    """Compute_3D of TriDiagTB (dur None) or TriDiagTR of one level: z_faces
    (n3, n2, n1+1), x_faces (n3, n2+1, n1), y_faces = (F3, F3G, DTU3, DUU3)
    (n3+1, n2, n1), cells (n3, n2, n1); coefs the fields of
    asam_tri_tb_coefs.  couple: the reference's branch with the couplings
    between planes stored.  Returns d, u1, l1, u2, l2, u3, l3."""
    lib = _lib.load()
    zf, xf, yf = ([_f64(a) for a in f] for f in (z_faces, x_faces, y_faces))
    cells = [_f64(a) for a in (vol, dut)] + ([_f64(dur)] if dur is not None else [])
    n3, n2, n1 = cells[0].shape
    if (any(a.shape != (n3, n2, n1 + 1) for a in zf) or any(a.shape != (n3, n2 + 1, n1) for a in xf)
            or any(a.shape != (n3 + 1, n2, n1) for a in yf) or any(a.shape != (n3, n2, n1) for a in cells)):
        raise ValueError("z (n3,n2,n1+1), x (n3,n2+1,n1), y faces (n3+1,n2,n1), cells (n3,n2,n1)")
    d = np.empty((n3, n2, n1, 4))
    u1 = np.empty((n3, n2, max(n1 - 1, 0), 4))
    l1 = np.empty_like(u1)
    u2 = np.empty((n3, max(n2 - 1, 0), n1, 4))
    l2 = np.empty_like(u2)
    u3 = np.zeros((max(n3 - 1, 0), n2, n1, 4))
    l3 = np.zeros_like(u3)
    co = _lib.AsamTriTbCoefs(**{k: float(v) for k, v in coefs.items()})
    opt = lambda a: ptr(a) if a.size else None  # noqa: E731
    check(lib.asam_tri_tb_compute_3d(int(dur is not None), int(bool(couple)), n3, n2, n1, C.byref(co),
                                     *[ptr(a) for a in zf], *[ptr(a) for a in xf], *[ptr(a) for a in yf],
                                     ptr(cells[0]), ptr(cells[1]), ptr(cells[2]) if dur is not None else None, ptr(d),
                                     opt(u1), opt(l1), opt(u2), opt(l2), opt(u3), opt(l3)), "asam_tri_tb_compute_3d")
    return d, u1, l1, u2, l2, u3, l3


def MatVecTB_3D(blocks, x, tr: bool = False) -> np.ndarray:
    """MatVecTB_2D/3D (MatVecTR_2D/3D with tr) of a level assembled by
    Compute_TB_3D: blocks = (d, u1, l1, u2, l2, u3, l3), x (n3, n2, n1, 2)."""
    lib = _lib.load()
    d = _f64(blocks[0])
    n3, n2, n1 = d.shape[:3]
    rest = [_f64(a) for a in blocks[1:]]
    xx = _f64(x)
    y = np.empty_like(xx)
    check(lib.asam_tri_tb_matvec_3d(int(bool(tr)), n3, n2, n1, ptr(d), *[ptr(a) if a.size else None for a in rest],
                                    ptr(xx), ptr(y)), "asam_tri_tb_matvec_3d")
    return y


def GaussSeidelTB_2D(blocks, b, x0, gauss_iter: int, tr: bool = False) -> np.ndarray:
    """GaussSeidel_2D of TriDiagTB (TriDiagTR with tr) on planes assembled by
    Compute_TB_2D: blocks = (d, u1, l1, u2, l2); b, x0 (nplane, n2, n1, 2)."""
    lib = _lib.load()
    d = _f64(blocks[0])
    nplane, n2, n1 = d.shape[:3]
    rest = [_f64(a) for a in blocks[1:5]]
    bb, x = _f64(b), _f64(x0).copy()
    check(lib.asam_tri_tb_gauss_seidel_2d(int(bool(tr)), nplane, n2, n1, ptr(d),
                                          *[ptr(a) if a.size else None for a in rest], ptr(bb), ptr(x),
                                          int(gauss_iter)), "asam_tri_tb_gauss_seidel_2d")
    return x


def RestrictTB_2D(res) -> np.ndarray:
    lib = _lib.load()
    r = _f64(res)
    nplane, n2, n1 = r.shape[:3]
    out = np.empty((nplane, (n2 + 1) // 2, (n1 + 1) // 2, 2))
    check(lib.asam_tri_tb_restrict_2d(nplane, n2, n1, ptr(r), ptr(out)), "asam_tri_tb_restrict_2d")
    return out


def ProlongateTB_2D(xc, n2: int, n1: int) -> np.ndarray:
    lib = _lib.load()
    c = _f64(xc)
    out = np.empty((c.shape[0], n2, n1, 2))
    check(lib.asam_tri_tb_prolong_2d(c.shape[0], n2, n1, ptr(c), ptr(out)), "asam_tri_tb_prolong_2d")
    return out


def SolveTB_2D(levels, b, x0, gauss_iter2: int = 1, mult_iter: int = 1, tr: bool = False) -> np.ndarray:
    """Solve_2D of TriDiagTB (TriDiagTR with tr): mult_iter V-cycles of
    Multigrid_2D over the plane hierarchy levels = [(d, u1, l1, u2, l2), ...]
    finest first, each as Compute_TB_2D returns it, level l+1 of ((n2+1)/2,
    (n1+1)/2); b, x0 (nplane, n2, n1, 2) on the finest level."""
    lib = _lib.load()
    keep = [[_f64(a) for a in lv[:5]] for lv in levels]
    nlev = len(keep)
    n2s = (C.c_int * nlev)(*[k[0].shape[1] for k in keep])
    n1s = (C.c_int * nlev)(*[k[0].shape[2] for k in keep])
    arrs = [(C.c_void_p * nlev)(*[k[j].ctypes.data if k[j].size else None for k in keep]) for j in range(5)]
    bb, x = _f64(b), _f64(x0).copy()
    check(lib.asam_tri_tb_multigrid_2d(int(bool(tr)), keep[0][0].shape[0], nlev, n2s, n1s, *arrs, ptr(bb), ptr(x),
                                       int(gauss_iter2), int(mult_iter)), "asam_tri_tb_multigrid_2d")
    return x


def SolveTB_3D(levels, b, x0, gauss_iter2: int = 1, mult_iter2: int = 1, gauss_iter3: int = 1, mult_iter3: int = 1,
               tr: bool = False) -> np.ndarray:
    """Solve_3D of TriDiagTB (TriDiagTR with tr): mult_iter3 V-cycles of
    Multigrid_3D over levels = [(plane_levels, u3, l3), ...] finest first --
    plane_levels the hierarchy of the level's planes as SolveTB_2D takes it,
    u3, l3 (n3-1, n2, n1, 4) as Compute_TB_3D returns them; each plane solved
    by Solve_2D (gauss_iter2, mult_iter2); b, x0 (n3, n2, n1, 2)."""
    lib = _lib.load()
    lv = [([[_f64(a) for a in p[:5]] for p in planes], _f64(u3), _f64(l3)) for planes, u3, l3 in levels]
    for planes, _, _ in lv:  # the C-ABI derives the plane levels' sizes by halving
        n3, n2, n1 = planes[0][0].shape[:3]
        for p in planes:
            if p[0].shape[:3] != (n3, n2, n1):
                raise ValueError(f"SolveTB_3D: plane level of shape {p[0].shape[:3]}, expected {(n3, n2, n1)}")
            n2, n1 = (n2 + 1) // 2, (n1 + 1) // 2
    flat = [k for planes, _, _ in lv for k in planes]
    nl = len(lv)
    ints = lambda v: (C.c_int * len(v))(*v)  # noqa: E731
    ptrs = lambda arrs: (C.c_void_p * len(arrs))(*[a.ctypes.data if a.size else None for a in arrs])  # noqa: E731
    bb, x = _f64(b), _f64(x0).copy()
    check(lib.asam_tri_tb_multigrid_3d(int(bool(tr)), nl, ints([p[0][0].shape[0] for p, _, _ in lv]),
                                       ints([p[0][0].shape[1] for p, _, _ in lv]),
                                       ints([p[0][0].shape[2] for p, _, _ in lv]), ints([len(p) for p, _, _ in lv]),
                                       ptrs([u for _, u, _ in lv]), ptrs([l for _, _, l in lv]),
                                       *[ptrs([k[j] for k in flat]) for j in range(5)], ptr(bb), ptr(x),
                                       int(gauss_iter2), int(mult_iter2), int(gauss_iter3), int(mult_iter3)),
          "asam_tri_tb_multigrid_3d")
    return x


class TriTBHierarchy:
    """The TriDiagTB (TriDiagTR with dur) preconditioner resident on the
    device: LaplTBCompute / LaplTRCompute (MULTI/JacAccGrav_Mod.f90:1312-1667)
    of ref_level levels from the finest fields -- z_faces (F1, F1G, DTU1,
    DUU1) (n3, n2, n1+1), x_faces (n3, n2+1, n1), y_faces (n3+1, n2, n1),
    vol, dut, dur (n3, n2, n1) in the reversed index order -- and its
    V-cycles (VCycleCG, :4502-4515)."""

    def __init__(self, z_faces, x_faces, y_faces, vol, dut, dur=None, ref_level: int = 1, **coefs):
        self.lib = _lib.load()
        fs = [_f64(a) for a in list(z_faces) + list(x_faces) + list(y_faces)]
        cells = [_f64(a) for a in (vol, dut) + ((dur,) if dur is not None else ())]
        n3, n2, n1 = cells[0].shape
        if (any(a.shape != (n3, n2, n1 + 1) for a in fs[:4]) or any(a.shape != (n3, n2 + 1, n1) for a in fs[4:8])
                or any(a.shape != (n3 + 1, n2, n1) for a in fs[8:]) or any(a.shape != (n3, n2, n1) for a in cells)):
            raise ValueError("z (n3,n2,n1+1), x (n3,n2+1,n1), y faces (n3+1,n2,n1), cells (n3,n2,n1)")
        self.tr = dur is not None
        self.ref_level = int(ref_level)
        self.shape = (n3, n2, n1)
        co = _lib.AsamTriTbCoefs(**{k: float(v) for k, v in coefs.items()})
        h = C.c_void_p()
        check(self.lib.asam_tri_tb_hier_create(int(self.tr), self.ref_level, n3, n2, n1, C.byref(co),
                                               (C.c_void_p * 12)(*[a.ctypes.data for a in fs]), ptr(cells[0]),
                                               ptr(cells[1]), ptr(cells[2]) if self.tr else None, C.byref(h)),
              "asam_tri_tb_hier_create")
        self.h = h

    def level(self, level3: int, level2: int):
        """(d, u1, l1, u2, l2) of plane level level2 of level level3, with u3,
        l3 appended when level2 == level3."""
        n3 = -(-self.shape[0] // 2 ** level3)
        n2, n1 = (-(-n // 2 ** level2) for n in self.shape[1:])
        shapes = [(n3, n2, n1, 4), (n3, n2, n1 - 1, 4), (n3, n2, n1 - 1, 4), (n3, n2 - 1, n1, 4), (n3, n2 - 1, n1, 4)]
        if level2 == level3:
            shapes += [(n3 - 1, n2, n1, 4)] * 2
        out = []
        for w, shp in enumerate(shapes):
            a = np.empty(shp)
            check(self.lib.asam_tri_tb_hier_get(self.h, int(level3), int(level2), w, ptr(a) if a.size else
                                                C.cast(C.pointer(C.c_double(0.0)), C.c_void_p)),
                  "asam_tri_tb_hier_get")
            out.append(a)
        return tuple(out)

    def set_zebra(self, on: bool = True) -> None:
        """Zebra order of the smoothers (lines and planes of one parity at
        once, the GPU's parallel order) for later V-cycles; off: the
        reference's sequential order."""
        check(self.lib.asam_tri_tb_hier_set_zebra(self.h, int(bool(on))), "asam_tri_tb_hier_set_zebra")

    def vcycle(self, b, x0=None, gauss_iter2: int = 1, mult_iter2: int = 1, gauss_iter3: int = 1,
               mult_iter3: int = 1) -> np.ndarray:
        bb = _f64(b)
        x = np.zeros_like(bb) if x0 is None else _f64(x0).copy()
        if bb.shape != self.shape + (2,) or x.shape != bb.shape:
            raise ValueError(f"b, x0 of shape {self.shape + (2,)}")
        check(self.lib.asam_tri_tb_hier_vcycle(self.h, ptr(bb), ptr(x), int(gauss_iter2), int(mult_iter2),
                                               int(gauss_iter3), int(mult_iter3)), "asam_tri_tb_hier_vcycle")
        return x

    def close(self):
        if self.h:
            self.lib.asam_tri_tb_hier_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def MatVecTB_1D(d: np.ndarray, u: np.ndarray, l: np.ndarray, x: np.ndarray) -> np.ndarray:
    lib = _lib.load()
    d, u, l, xx = _f64(d), _f64(u), _f64(l), _f64(x)
    ncol, n1 = d.shape[:2]
    y = np.empty_like(xx)
    check(lib.asam_tri_tb_matvec(ncol, n1, ptr(d), ptr(u), ptr(l), ptr(xx), ptr(y)), "asam_tri_tb_matvec")
    return y


def MatVecT_1D(d: np.ndarray, u: np.ndarray, l: np.ndarray, x: np.ndarray) -> np.ndarray:
    lib = _lib.load()
    d, u, l, xx = _f64(d), _f64(u), _f64(l), _f64(x)
    ncol, n1 = d.shape
    y = np.empty_like(xx)
    check(lib.asam_tri_matvec(ncol, n1, ptr(d), ptr(u), ptr(l), ptr(xx), ptr(y)), "asam_tri_matvec")
    return y
