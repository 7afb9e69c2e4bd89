"""CPU oracle of the ASAM transport stage -- TEST INFRASTRUCTURE ONLY.

ctypes binding of ``oracle/asam_oracle.c``, a loop-for-loop C restatement of
the reference Fortran (see that file's header for the routines and
conventions).  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may use it, and only as the checker.  Parity with the
Fortran binary itself is unpinned (no Fortran compiler is available); the
restatement is checked against analytic known answers and an independent
Python restatement in ``tests/``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "libasam_oracle.so"


class OraGeom(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("per_x", C.c_int), ("per_y", C.c_int),
                ("per_z", C.c_int), ("volc", C.c_void_p), ("fu", C.c_void_p), ("fv", C.c_void_p),
                ("fw", C.c_void_p), ("bc", C.c_void_p), ("dh", C.c_void_p), ("dv", C.c_void_p),
                ("jac_diff", C.c_int), ("bc_mean", C.c_void_p), ("bc_fval", C.c_void_p), ("bc_amb", C.c_void_p),
                ("bc_uf", C.c_void_p), ("bc_vf", C.c_void_p), ("bc_rho", C.c_int)]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            import sys
            sys.path.insert(0, str(_HERE.parent))
            from asam_gb300.build import build_oracle
            build_oracle()
        lib = C.CDLL(str(LIB_PATH))
        G = C.POINTER(OraGeom)
        V, I, D = C.c_void_p, C.c_int, C.c_double
        sig = {
            "ora_exchange_cell": (None, [G, I, V]),
            "ora_exchange_flux": (None, [G, I, V]),
            "ora_bound_cond": (None, [G, I, I, V]),
            "ora_diffusion": (None, [G, I, I, V, V]),
            "ora_fcn": (None, [G, I, I, V, V, V, V, V]),
            "ora_div": (None, [G, V, V, V, V]),
            "ora_jac": (None, [G, V, V, V, V, D, D, V]),
            "ora_spmv": (None, [G, V, V, V]),
            "ora_gauss_seidel": (None, [G, V, V, V, I]),
            "ora_psolve": (None, [G, I, V, V, V, I]),
            "ora_matvec": (None, [G, I, V, V, V]),
            "ora_dot": (D, [G, I, V, V]),
            "ora_bicgstab": (None, [G, I, V, V, V, C.POINTER(C.c_int), C.POINTER(C.c_double), I]),
            "ora_bicgstab_halfsteps": (None, [G, I, V, V, V, I, I]),
            "ora_ros_coeffs": (I, [I, C.POINTER(C.c_double), V, V, V]),
            "ora_ros_step": (I, [G, I, I, V, V, V, V, D, I, D, I, I, V, V]),
            "ora_total_scalar": (D, [G, V]),
            "ora_tri_solve": (None, [I, I, V, V, V, V]),
            "ora_tri_tb_solve": (None, [I, I, V, V, V, V, V]),
            "ora_tri_tb_matvec": (None, [I, I, V, V, V, V, V]),
            "ora_tri_tb_compute": (None, [I, I, I] + [V] * 11),
            "ora_tri_tb_compute_2d": (None, [I, I, I, I] + [V] * 17),
            "ora_tri_tb_compute_3d": (None, [I, I, I, I, I] + [V] * 23),
            "ora_tri_tb_matvec_3d": (None, [I, I, I, I] + [V] * 9),
            "ora_tri_tb_gauss_seidel_2d": (None, [I, I, I, I] + [V] * 7 + [I]),
            "ora_tri_tb_restrict_2d": (None, [I, I, I, V, V]),
            "ora_tri_tb_prolong_2d": (None, [I, I, I, V, V]),
            "ora_tri_tb_multigrid_2d": (None, [I, I, I, V, V] + [V] * 7 + [I, I]),
            "ora_tri_tb_gauss_seidel_3d": (None, [I, I, I, V, V] + [V] * 9 + [I, I, I]),
            "ora_tri_tb_restrict_3d": (None, [I, I, I, V, V]),
            "ora_tri_tb_prolong_3d": (None, [I, I, I, V, V]),
            "ora_tri_tb_multigrid_3d": (None, [I, I, V, V, V, V] + [V] * 9 + [I, I, I, I]),
            "ora_tri_tb_lapl_level": (None, [I, I, I, I, V, V, V, V, V, I, I] + [V] * 7),
            "ora_tri_tb_set_zebra": (None, [I]),
            "ora_tri_matvec": (None, [I, I, V, V, V, V, V]),
        }
        sig.update({
            "ora_proj_create": (V, [C.POINTER(C.c_int), C.POINTER(C.c_double)] + [V] * 16),
            "ora_proj_destroy": (None, [V]),
            "ora_proj_set_zebra": (None, [V, I]),
            "ora_lapl_compute": (None, [V, D, D]),
            "ora_lapl_get": (C.c_long, [V, I, I, I, V]),
            "ora_lapl_get_dirichlet": (C.c_long, [V, I, I, I, V]),
            "ora_lapl_matvec": (None, [V, V, V]),
            "ora_lapl_vcycle": (None, [V, V, V]),
            "ora_psolve1": (None, [V, V, V]),
            "ora_proj_nvec": (C.c_long, [V]),
            "ora_lapl_vcycle_dirichlet": (I, [V, V, V]),
            "ora_proj_exchange": (None, [V, V]),
            "ora_proj_dot2": (D, [V, V, V]),
            "ora_matvec1": (None, [V, V, V]),
            "ora_fgmres": (I, [V, V, V, I, D, I, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "ora_proj_rhs": (None, [V, V, V, V, V, V]),
            "ora_proj_update": (None, [V, V, V, V, V, V, V, I, V, V, V]),
            "ora_weights_density": (None, [V] * 15),
            "ora_proj_set_weights": (None, [V] * 9),
        })
        sig.update({
            "ora_face_to_cell": (None, [G, I, V, V, V, V, V, I, I, V]),
            "ora_cell_to_face": (None, [G, V, V, V, V, V]),
            "ora_thermo": (None, [G, V, V, V, V, V, V, V, V]),
            "ora_fcn_dyn": (None, [G, I, I, V, I, I, D, V, V, V, V, V, V, V, V, V, V, V]),
            "ora_ros_step_dyn": (I, [G, V, V, V, V, V, V, V, V, V, V, V, V, V, I, V, I, D, V, V, V, V]),
        })
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _p(a: np.ndarray) -> int:
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


class Oracle:
    """Oracle bound to one geometry (keeps the arrays alive)."""

    def __init__(self, geo, bc=None):
        self.lib = load()
        g = geo.grid
        self.grid = g
        self._keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (geo.volc, geo.fu, geo.fv, geo.fw)]
        self.g = OraGeom(g.nx, g.ny, g.nz, int(g.periodic_x), int(g.periodic_y), int(g.periodic_z),
                         *(a.ctypes.data for a in self._keep), None, None, None, 0)
        self.gp = C.byref(self.g)
        self.npad = g.npad
        self.set_boundary(bc)

    def set_boundary(self, kinds):
        """Halo rule of the outer walls, (ncomp, 6) ints W,E,S,N,B,T (0 none,
        1 ZeroGrad, 2 ZeroValue, 3 MeanValue, 4 Function, 5 InFlowOutFlow,
        6 Extrapolation); None = ZeroGrad everywhere."""
        if kinds is None:
            self._bc = None
            self.g.bc = None
        else:
            self._bc = np.ascontiguousarray(kinds, dtype=np.int32).reshape(-1)
            self.g.bc = self._bc.ctypes.data

    def set_boundary_data(self, mean=None, fval=None, amb=None, vel=None, rho_pos=0):
        """Data of the open-boundary halo rules: MeanProfile (ncomp, nz), the
        Function values and the ambient state (ncomp padded fields), the face
        velocities (uF, vF, wF) whose sign InFlowOutFlow tests when bound_cond
        is called alone (a step uses its own), the density component."""
        keep = {}
        for name, a in (("bc_mean", mean), ("bc_fval", fval), ("bc_amb", amb)):
            if a is None:
                setattr(self.g, name, None)
            else:
                keep[name] = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                setattr(self.g, name, keep[name].ctypes.data)
        if vel is None:
            self.g.bc_uf = self.g.bc_vf = None
        else:
            keep["uf"], keep["vf"] = (np.ascontiguousarray(v, dtype=np.float64).reshape(-1) for v in vel[:2])
            self.g.bc_uf, self.g.bc_vf = keep["uf"].ctypes.data, keep["vf"].ctypes.data
        self.g.bc_rho = int(rho_pos)
        self._bc_data = keep

    def set_diffusion(self, dh, dv=None, jac=True):
        """Diffusion coefficients DH, DV (padded cell fields; DV defaults to
        DH) or None: no diffusion; jac adds the diffusion Jacobian."""
        if dh is None:
            self._diff = None
            self.g.dh = self.g.dv = None
            self.g.jac_diff = 0
            return
        dh = np.ascontiguousarray(dh, dtype=np.float64)
        dv = dh if dv is None else np.ascontiguousarray(dv, dtype=np.float64)
        self._diff = (dh, dv)
        self.g.dh, self.g.dv = dh.ctypes.data, dv.ctypes.data
        self.g.jac_diff = int(bool(jac))

    def exchange_cell(self, c):
        a = np.ascontiguousarray(c, dtype=np.float64).copy()
        self.lib.ora_exchange_cell(self.gp, a.size // self.npad, _p(a))
        return a

    def diffusion(self, c, rho_pos=0):
        """The diffusion terms of FcnMet alone (unscaled, masked), every component."""
        a = np.ascontiguousarray(c, dtype=np.float64)
        f = np.zeros_like(a)
        self.lib.ora_diffusion(self.gp, a.size // self.npad, int(rho_pos), _p(a), _p(f))
        return f

    def bound_cond(self, c, comp0=0):
        a = np.ascontiguousarray(c, dtype=np.float64).copy()
        self.lib.ora_bound_cond(self.gp, a.size // self.npad, int(comp0), _p(a))
        return a

    def fcn(self, c, vel, rho_pos=0):
        a = np.ascontiguousarray(c, dtype=np.float64)
        f = np.empty_like(a)
        uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
        self.lib.ora_fcn(self.gp, a.size // self.npad, rho_pos, _p(a), _p(uf), _p(vf), _p(wf), _p(f))
        return f

    def div(self, rhs, vel):
        a = np.ascontiguousarray(rhs, dtype=np.float64).copy()
        uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
        self.lib.ora_div(self.gp, _p(uf), _p(vf), _p(wf), _p(a))
        return a

    def jac(self, rho, vel, beta0, dt):
        r = np.ascontiguousarray(rho, dtype=np.float64)
        uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
        val = np.empty((7, self.npad))
        self.lib.ora_jac(self.gp, _p(r), _p(uf), _p(vf), _p(wf), float(beta0), float(dt), _p(val))
        return val

    def spmv(self, val, x):
        v = np.ascontiguousarray(val, dtype=np.float64)
        xx = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.npad)
        self.lib.ora_spmv(self.gp, _p(v), _p(xx), _p(y))
        return y

    def gauss_seidel(self, val, b, iterg=5):
        v = np.ascontiguousarray(val, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty(self.npad)
        self.lib.ora_gauss_seidel(self.gp, _p(v), _p(bb), _p(x), iterg)
        return x

    def psolve(self, val, x, iterg=5):
        v = np.ascontiguousarray(val, dtype=np.float64)
        xx = np.ascontiguousarray(x, dtype=np.float64)
        px = np.empty_like(xx)
        self.lib.ora_psolve(self.gp, xx.size // self.npad, _p(v), _p(xx), _p(px), iterg)
        return px

    def matvec(self, val, x):
        v = np.ascontiguousarray(val, dtype=np.float64)
        xx = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(xx)
        self.lib.ora_matvec(self.gp, xx.size // self.npad, _p(v), _p(xx), _p(y))
        return y

    def dot(self, x, y):
        xx = np.ascontiguousarray(x, dtype=np.float64)
        yy = np.ascontiguousarray(y, dtype=np.float64)
        return self.lib.ora_dot(self.gp, xx.size // self.npad, _p(xx), _p(yy))

    def bicgstab(self, val, x, b, maxiter, tol, iterg=5):
        """x updated in place; returns (MaxIter, Tol) with the reference's sentinels."""
        v = np.ascontiguousarray(val, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        it = C.c_int(maxiter)
        tl = C.c_double(tol)
        self.lib.ora_bicgstab(self.gp, x.size // self.npad, _p(v), _p(x), _p(bb), C.byref(it), C.byref(tl), iterg)
        return it.value, tl.value

    def bicgstab_halfsteps(self, val, x, b, nhalf, iterg=5):
        """x updated in place by exactly nhalf BiCGStab half-steps (a run whose
        exit lands there: MaxIter -k leaves after 2k-1, +k after 2k)."""
        v = np.ascontiguousarray(val, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        self.lib.ora_bicgstab_halfsteps(self.gp, x.size // self.npad, _p(v), _p(x), _p(bb), int(nhalf), iterg)

    def ros_step(self, c, vel, dt, method=5, tol=1e-6, maxiter=30, iterg=5, rho_pos=0):
        """c updated in place; returns (iters, resid) per stage."""
        uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
        iters = np.zeros(4, dtype=np.int32)
        resid = np.zeros(4)
        n = self.lib.ora_ros_step(self.gp, c.size // self.npad, rho_pos, _p(c), _p(uf), _p(vf), _p(wf), float(dt),
                                  int(method), float(tol), int(maxiter), int(iterg), iters.ctypes.data,
                                  resid.ctypes.data)
        return list(iters[:n]), list(resid[:n])

    # -- dynamical-core stage (oracle/asam_dyn.c) ------------------------------
    def face_to_cell(self, pos, vel, c, bound=None, free_slip=True):
        a = np.ascontiguousarray(c, dtype=np.float64).copy()
        uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
        pp = np.ascontiguousarray(pos, dtype=np.int32)
        bd = np.zeros((0, 3), np.int32) if bound is None else np.ascontiguousarray(bound, dtype=np.int32)
        self.lib.ora_face_to_cell(self.gp, a.size // self.npad, pp.ctypes.data, _p(uf), _p(vf), _p(wf),
                                  bd.ctypes.data, len(bd.reshape(-1, 3)), int(bool(free_slip)), _p(a))
        return a

    def cell_to_face(self, pos, c):
        g = self.grid
        a = np.ascontiguousarray(c, dtype=np.float64)
        pp = np.ascontiguousarray(pos, dtype=np.int32)
        u = np.empty((g.nz, g.ny, g.nx + 1))
        v = np.empty((g.nz, g.ny + 1, g.nx))
        w = np.empty((g.nz + 1, g.ny, g.nx))
        self.lib.ora_cell_to_face(self.gp, pp.ctypes.data, _p(a), _p(u), _p(v), _p(w))
        return u, v, w

    def thermo(self, c, rho_pos, th_pos, rv_pos=-1, rc_pos=-1, rr_pos=-1, ri_pos=-1):
        a = np.ascontiguousarray(c, dtype=np.float64)
        n = self.npad
        comp = lambda q: None if q < 0 else a.ctypes.data + 8 * n * q
        t = np.empty(self.grid.pshape)
        p = np.empty(self.grid.pshape)
        self.lib.ora_thermo(self.gp, comp(rho_pos), comp(th_pos), comp(rv_pos), comp(rc_pos), comp(rr_pos),
                            comp(ri_pos), _p(t), _p(p))
        return t, p

    def fcn_dyn(self, c, vel, pre, pos, dx, dy, dz, mxy=None, myx=None, rho_pos=0, pgrad=True, buoy=True,
                grav=9.81):
        g = self.grid
        a = np.ascontiguousarray(c, dtype=np.float64)
        f = np.empty_like(a)
        uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
        pr = np.ascontiguousarray(pre, dtype=np.float64)
        pp = np.ascontiguousarray(pos, dtype=np.int32)
        mxy = np.ones(g.ny) if mxy is None else np.ascontiguousarray(mxy, dtype=np.float64)
        myx = np.ones(g.nx) if myx is None else np.ascontiguousarray(myx, dtype=np.float64)
        dx, dy, dz = (np.ascontiguousarray(q, dtype=np.float64) for q in (dx, dy, dz))
        self.lib.ora_fcn_dyn(self.gp, a.size // self.npad, int(rho_pos), pp.ctypes.data, int(bool(pgrad)),
                             int(bool(buoy)), float(grav), _p(a), _p(uf), _p(vf), _p(wf), _p(pr), _p(dx), _p(dy),
                             _p(dz), _p(mxy), _p(myx), _p(f))
        return f

    def ros_step_dyn(self, proj, c, vel, dt, *, rho_pos, th_pos, pos, dx, dy, dz, rv_pos=-1, rc_pos=-1, rr_pos=-1,
                     ri_pos=-1, pgrad=True, buoy=True, free_slip=True, method=5, bicg_tol=1e-6, bicg_maxiter=30,
                     iterg=5, proj_maxiter=10, proj_step=10, proj_tol=1e-6, grav=9.81, bound=None, scalars=(),
                     mxy=None, myx=None):
        """One step of the dynamical core; c and vel (uf, vf, wf arrays) updated
        in place.  proj: an OracleProj of this block.  Returns per stage
        (iters, resid, fgmres steps, fgmres relative residual)."""
        g = self.grid
        uf, vf, wf = vel
        for a in (c, uf, vf, wf):
            assert a.dtype == np.float64 and a.flags.c_contiguous
        ip = np.array([c.size // self.npad, rho_pos, th_pos, rv_pos, rc_pos, rr_pos, ri_pos, *pos, int(bool(pgrad)),
                       int(bool(buoy)), int(bool(free_slip)), method, bicg_maxiter, iterg, proj_maxiter, proj_step],
                      dtype=np.int32)
        dp = np.array([grav, bicg_tol, proj_tol])
        mxy = np.ones(g.ny) if mxy is None else np.ascontiguousarray(mxy, dtype=np.float64)
        myx = np.ones(g.nx) if myx is None else np.ascontiguousarray(myx, dtype=np.float64)
        dx, dy, dz = (np.ascontiguousarray(q, dtype=np.float64) for q in (dx, dy, dz))
        bd = np.zeros((0, 3), np.int32) if bound is None else np.ascontiguousarray(bound, dtype=np.int32)
        sc = np.ascontiguousarray(list(scalars) or [0], dtype=np.int32)
        it = np.zeros(4, np.int32)
        rs = np.zeros(4)
        ps = np.zeros(4, np.int32)
        pr = np.zeros(4)
        n = self.lib.ora_ros_step_dyn(self.gp, proj.h, ip.ctypes.data, dp.ctypes.data, _p(c), _p(uf), _p(vf), _p(wf),
                                      _p(dx), _p(dy), _p(dz), _p(mxy), _p(myx), bd.ctypes.data,
                                      len(bd.reshape(-1, 3)), sc.ctypes.data, len(scalars), float(dt),
                                      it.ctypes.data, rs.ctypes.data, ps.ctypes.data, pr.ctypes.data)
        return list(it[:n]), list(rs[:n]), list(ps[:n]), list(pr[:n])

    def total_scalar(self, c):
        a = np.ascontiguousarray(c, dtype=np.float64)
        return self.lib.ora_total_scalar(self.gp, _p(a))


def ros_coeffs(method: int):
    lib = load()
    b0 = C.c_double()
    al, be, gm = np.zeros(16), np.zeros(16), np.zeros(5)
    n = lib.ora_ros_coeffs(int(method), C.byref(b0), al.ctypes.data, be.ctypes.data, gm.ctypes.data)
    return n, b0.value, al.reshape(4, 4), be.reshape(4, 4), gm


def tri_solve(d, u, l, b):
    lib = load()
    d, u, l = (np.ascontiguousarray(a, dtype=np.float64) for a in (d, u, l))
    x = np.ascontiguousarray(b, dtype=np.float64).copy()
    ncol, n1 = d.shape
    lib.ora_tri_solve(ncol, n1, _p(d), _p(u), _p(l), _p(x))
    return x


def tri_matvec(d, u, l, x):
    lib = load()
    d, u, l, xx = (np.ascontiguousarray(a, dtype=np.float64) for a in (d, u, l, x))
    ncol, n1 = d.shape
    y = np.empty_like(xx)
    lib.ora_tri_matvec(ncol, n1, _p(d), _p(u), _p(l), _p(xx), _p(y))
    return y


def tri_tb_solve(d, u, l, b):
    """Solve_1D of MULTI/TriDiagTB_Mod.f90:143-163 on columns: d (ncol, n1, 4),
    u/l (ncol, n1-1, 4) with 2x2 blocks column-major, b (ncol, n1, 2)."""
    lib = load()
    d, u, l = (np.ascontiguousarray(a, dtype=np.float64) for a in (d, u, l))
    x = np.ascontiguousarray(b, dtype=np.float64).copy()
    ncol, n1 = d.shape[:2]
    w = np.empty(max(n1 - 1, 1) * 4)
    lib.ora_tri_tb_solve(ncol, n1, _p(d), _p(u), _p(l), _p(x), _p(w))
    return x


def tri_tb_matvec(d, u, l, x):
    """MatVecTB_1D of MULTI/TriDiagTB_Mod.f90:121-141 on columns."""
    lib = load()
    d, u, l, xx = (np.ascontiguousarray(a, dtype=np.float64) for a in (d, u, l, x))
    ncol, n1 = d.shape[:2]
    y = np.empty_like(xx)
    lib.ora_tri_tb_matvec(ncol, n1, _p(d), _p(u), _p(l), _p(xx), _p(y))
    return y


def tri_tb_compute(f, fg, vol, dtu, duu, dut, dur=None, beta0_dtp=1.0, fac1_l=0.0, fac1_r=0.0, grav_comp=0.0,
                   fac_anela=0.0):
    """Allocate_1D + Compute_1D of TriDiagTB (dur None, MULTI/TriDiagTB_Mod.f90:32-93)
    or TriDiagTR (MULTI/TriDiagTR_Mod.f90:32-105) on columns: faces (ncol, n1+1),
    cells (ncol, n1).  Returns d (ncol, n1, 4), u, l (ncol, n1-1, 4)."""
    lib = load()
    faces = [np.ascontiguousarray(a, dtype=np.float64) for a in (f, fg, dtu, duu)]
    vol, dut = (np.ascontiguousarray(a, dtype=np.float64) for a in (vol, dut))
    tr = dur is not None
    durr = np.ascontiguousarray(dur, dtype=np.float64) if tr else vol
    ncol, n1 = vol.shape
    s = np.array([beta0_dtp, fac1_l, fac1_r, grav_comp, fac_anela])
    d = np.empty((ncol, n1, 4))
    u = np.empty((ncol, max(n1 - 1, 1), 4))
    l = np.empty_like(u)
    lib.ora_tri_tb_compute(int(tr), ncol, n1, _p(s), _p(faces[0]), _p(faces[1]), _p(vol), _p(faces[2]),
                           _p(faces[3]), _p(dut), _p(durr), _p(d), _p(u), _p(l))
    return d, u[:, :n1 - 1], l[:, :n1 - 1]


def tri_tb_compute_2d(z_faces, x_faces, vol, dut, dur=None, beta0_dtp=1.0, fac1_l=0.0, fac1_r=0.0, grav_comp=0.0,
                      fac_anela=0.0, fac2_l=0.0, fac2_r=0.0):
    """Allocate_2D + Compute_2D of TriDiagTB (dur None, MULTI/TriDiagTB_Mod.f90:260-343)
    or TriDiagTR (MULTI/TriDiagTR_Mod.f90:273-387) on planes: z_faces = (F1, F1G,
    DTU1, DUU1) each (nplane, n2, n1+1), x_faces = (F2, F2G, DTU2, DUU2) each
    (nplane, n2+1, n1), cells (nplane, n2, n1).  Returns d (nplane, n2, n1, 4),
    u1, l1 (nplane, n2, n1-1, 4), u2, l2 (nplane, n2-1, n1, 4)."""
    lib = load()
    zf = [np.ascontiguousarray(a, dtype=np.float64) for a in z_faces]
    xf = [np.ascontiguousarray(a, dtype=np.float64) for a in x_faces]
    vol, dut = (np.ascontiguousarray(a, dtype=np.float64) for a in (vol, dut))
    tr = dur is not None
    durr = np.ascontiguousarray(dur, dtype=np.float64) if tr else vol
    nplane, n2, n1 = vol.shape
    s = np.array([beta0_dtp, fac1_l, fac1_r, grav_comp, fac_anela, fac2_l, fac2_r])
    d = np.empty((nplane, n2, n1, 4))
    u1 = np.empty((nplane, n2, max(n1 - 1, 1), 4))
    l1 = np.empty_like(u1)
    u2 = np.empty((nplane, max(n2 - 1, 1), n1, 4))
    l2 = np.empty_like(u2)
    lib.ora_tri_tb_compute_2d(int(tr), nplane, n2, n1, _p(s), *[_p(a) for a in zf], *[_p(a) for a in xf], _p(vol),
                              _p(dut), _p(durr), _p(d), _p(u1), _p(l1), _p(u2), _p(l2))
    return d, u1[:, :, :n1 - 1], l1[:, :, :n1 - 1], u2[:, :n2 - 1], l2[:, :n2 - 1]


def tri_tb_compute_3d(z_faces, x_faces, y_faces, vol, dut, dur=None, couple=True, beta0_dtp=1.0, fac1_l=0.0,
                      fac1_r=0.0, grav_comp=0.0, fac_anela=0.0, fac2_l=0.0, fac2_r=0.0, fac3_l=0.0, fac3_r=0.0):
    """Compute_3D of TriDiagTB (dur None, MULTI/TriDiagTB_Mod.f90:663-780) or
    TriDiagTR (MULTI/TriDiagTR_Mod.f90:707-864) of one level: z_faces (n3, n2,
    n1+1), x_faces (n3, n2+1, n1), y_faces = (F3, F3G, DTU3, DUU3) (n3+1, n2,
    n1), cells (n3, n2, n1).  Returns d, u1, l1, u2, l2, u3, l3 (u3, l3 of
    shape (n3-1, n2, n1, 4), zero when couple is False)."""
    lib = load()
    zf = [np.ascontiguousarray(a, dtype=np.float64) for a in z_faces]
    xf = [np.ascontiguousarray(a, dtype=np.float64) for a in x_faces]
    yf = [np.ascontiguousarray(a, dtype=np.float64) for a in y_faces]
    vol, dut = (np.ascontiguousarray(a, dtype=np.float64) for a in (vol, dut))
    tr = dur is not None
    durr = np.ascontiguousarray(dur, dtype=np.float64) if tr else vol
    n3, n2, n1 = vol.shape
    s = np.array([beta0_dtp, fac1_l, fac1_r, grav_comp, fac_anela, fac2_l, fac2_r, fac3_l, fac3_r])
    d = np.empty((n3, n2, n1, 4))
    u1 = np.empty((n3, n2, max(n1 - 1, 1), 4))
    l1 = np.empty_like(u1)
    u2 = np.empty((n3, max(n2 - 1, 1), n1, 4))
    l2 = np.empty_like(u2)
    u3 = np.zeros((max(n3 - 1, 1), n2, n1, 4))
    l3 = np.zeros_like(u3)
    lib.ora_tri_tb_compute_3d(int(tr), int(bool(couple)), n3, n2, n1, _p(s), *[_p(a) for a in zf],
                              *[_p(a) for a in xf], *[_p(a) for a in yf], _p(vol), _p(dut), _p(durr), _p(d), _p(u1),
                              _p(l1), _p(u2), _p(l2), _p(u3), _p(l3))
    return (d, u1[:, :, :n1 - 1], l1[:, :, :n1 - 1], u2[:, :n2 - 1], l2[:, :n2 - 1], u3[:n3 - 1], l3[:n3 - 1])


def tri_tb_matvec_3d(blocks, x, tr=False):
    """MatVecTB_2D/3D (or MatVecTR with tr) of a level assembled by
    tri_tb_compute_3d: blocks = (d, u1, l1, u2, l2, u3, l3), x (n3, n2, n1, 2)."""
    lib = load()
    d = np.ascontiguousarray(blocks[0], dtype=np.float64)
    n3, n2, n1 = d.shape[:3]
    rest = [np.ascontiguousarray(a, dtype=np.float64) if a.size else np.zeros(4) for a in blocks[1:]]
    xx = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(xx)
    lib.ora_tri_tb_matvec_3d(int(tr), n3, n2, n1, _p(d), *[_p(a) for a in rest], _p(xx), _p(y))
    return y


def _tb_plane_blocks(blocks):
    d, u1, l1, u2, l2 = (np.ascontiguousarray(a, dtype=np.float64) for a in blocks[:5])
    return d, *[a if a.size else np.zeros(4) for a in (u1, l1, u2, l2)]


def tri_tb_gauss_seidel_2d(blocks, b, x0, iters, tr=False):
    """GaussSeidel_2D (MULTI/TriDiagTB_Mod.f90:374-418; TriDiagTR with tr) of
    planes assembled by tri_tb_compute_2d: blocks = (d, u1, l1, u2, l2),
    b and the initial guess x0 (nplane, n2, n1, 2)."""
    lib = load()
    d, u1, l1, u2, l2 = _tb_plane_blocks(blocks)
    nplane, n2, n1 = d.shape[:3]
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    lib.ora_tri_tb_gauss_seidel_2d(int(tr), nplane, n2, n1, _p(d), _p(u1), _p(l1), _p(u2), _p(l2), _p(bb), _p(x),
                                   int(iters))
    return x


def tri_tb_restrict_2d(res):
    """RestrictTB_2D of planes res (nplane, n2, n1, 2) -> ((n2+1)/2, (n1+1)/2)."""
    lib = load()
    r = np.ascontiguousarray(res, dtype=np.float64)
    nplane, n2, n1 = r.shape[:3]
    out = np.empty((nplane, (n2 + 1) // 2, (n1 + 1) // 2, 2))
    lib.ora_tri_tb_restrict_2d(nplane, n2, n1, _p(r), _p(out))
    return out


def tri_tb_prolong_2d(xc, n2, n1):
    """ProlongateTB_2D of coarse planes xc onto fine planes n2 x n1."""
    lib = load()
    c = np.ascontiguousarray(xc, dtype=np.float64)
    out = np.empty((c.shape[0], n2, n1, 2))
    lib.ora_tri_tb_prolong_2d(c.shape[0], n2, n1, _p(c), _p(out))
    return out


def tri_tb_multigrid_2d(levels, b, x0, gauss_iter2=1, mult_iter=1, tr=False):
    """Solve_2D of TriDiagTB (MULTI/TriDiagTB_Mod.f90:419-494; TriDiagTR with
    tr): mult_iter V-cycles of Multigrid_2D over the plane hierarchy levels =
    [(d, u1, l1, u2, l2), ...] finest first (each as tri_tb_compute_2d returns
    it, level l+1 of ((n2+1)/2, (n1+1)/2)), b and the guess x0 (nplane, n2,
    n1, 2) on the finest level."""
    lib = load()
    keep = [_tb_plane_blocks(lv) for lv in levels]
    nlev = len(keep)
    n2s = (C.c_int * nlev)(*[k[0].shape[1] for k in keep])
    n1s = (C.c_int * nlev)(*[k[0].shape[2] for k in keep])
    arrs = [(C.c_void_p * nlev)(*[k[j].ctypes.data for k in keep]) for j in range(5)]
    nplane = keep[0][0].shape[0]
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    lib.ora_tri_tb_multigrid_2d(int(tr), nplane, nlev, C.cast(n2s, C.c_void_p), C.cast(n1s, C.c_void_p),
                                *[C.cast(a, C.c_void_p) for a in arrs], _p(bb), _p(x), int(gauss_iter2),
                                int(mult_iter))
    return x


def _ptrs(arrs):
    return C.cast((C.c_void_p * len(arrs))(*[a.ctypes.data if a is not None and a.size else None for a in arrs]),
                  C.c_void_p)


def _ints(vals):
    return C.cast((C.c_int * len(vals))(*vals), C.c_void_p)


def _level3(level):
    """(plane_levels, u3, l3) with contiguous float64 arrays: plane_levels =
    [(d, u1, l1, u2, l2), ...] of all the level's planes, finest first."""
    planes, u3, l3 = level
    keep = [_tb_plane_blocks(lv) for lv in planes]
    return keep, np.ascontiguousarray(u3, dtype=np.float64), np.ascontiguousarray(l3, dtype=np.float64)


def tri_tb_gauss_seidel_3d(level, b, x0, iters, gauss_iter2=1, mult_iter2=1, tr=False):
    """GaussSeidel_3D (MULTI/TriDiagTB_Mod.f90:818-874; TriDiagTR with tr) of
    one level: level = (plane_levels, u3, l3) -- plane_levels the hierarchy of
    its n3 planes as tri_tb_multigrid_2d takes it, u3, l3 (n3-1, n2, n1, 4);
    b, x0 (n3, n2, n1, 2); each plane solved by Solve_2D."""
    lib = load()
    keep, u3, l3 = _level3(level)
    n3, n2, n1 = keep[0][0].shape[:3]
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    lib.ora_tri_tb_gauss_seidel_3d(int(tr), n3, len(keep), _ints([k[0].shape[1] for k in keep]),
                                   _ints([k[0].shape[2] for k in keep]), *[_ptrs([k[j] for k in keep]) for j in range(5)],
                                   _p(u3) if u3.size else None, _p(l3) if l3.size else None, _p(bb), _p(x),
                                   int(iters), int(gauss_iter2), int(mult_iter2))
    return x


def tri_tb_restrict_3d(res):
    """RestrictTB_3D of a level res (n3, n2, n1, 2) -> halved sizes."""
    lib = load()
    r = np.ascontiguousarray(res, dtype=np.float64)
    n3, n2, n1 = r.shape[:3]
    out = np.empty(((n3 + 1) // 2, (n2 + 1) // 2, (n1 + 1) // 2, 2))
    lib.ora_tri_tb_restrict_3d(n3, n2, n1, _p(r), _p(out))
    return out


def tri_tb_prolong_3d(xc, n3, n2, n1):
    """ProlongateTB_3D of a coarse level onto n3 x n2 x n1."""
    lib = load()
    c = np.ascontiguousarray(xc, dtype=np.float64)
    out = np.empty((n3, n2, n1, 2))
    lib.ora_tri_tb_prolong_3d(n3, n2, n1, _p(c), _p(out))
    return out


def tri_tb_multigrid_3d(levels, b, x0, gauss_iter2=1, mult_iter2=1, gauss_iter3=1, mult_iter3=1, tr=False):
    """Solve_3D (MULTI/TriDiagTB_Mod.f90:876-952; TriDiagTR with tr):
    mult_iter3 V-cycles of Multigrid_3D over levels = [(plane_levels, u3,
    l3), ...] finest first, each level's sizes halved (rounding up) from the
    last; b, x0 (n3, n2, n1, 2) on the finest level."""
    lib = load()
    lv = [_level3(L) for L in levels]
    flat = [k for keep, _, _ in lv for k in keep]
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    lib.ora_tri_tb_multigrid_3d(int(tr), len(lv), _ints([k[0][0].shape[0] for k, _, _ in lv]),
                                _ints([k[0][0].shape[1] for k, _, _ in lv]), _ints([k[0][0].shape[2] for k, _, _ in lv]),
                                _ints([len(k) for k, _, _ in lv]), _ptrs([u for _, u, _ in lv]),
                                _ptrs([l for _, _, l in lv]), *[_ptrs([k[j] for k in flat]) for j in range(5)], _p(bb),
                                _p(x), int(gauss_iter2), int(mult_iter2), int(gauss_iter3), int(mult_iter3))
    return x


def tri_tb_set_zebra(on):
    """The zebra order of the TriDiagTB/TR smoothers in the oracle (the GPU's
    parallel order) for all later calls; off: the reference's order."""
    load().ora_tri_tb_set_zebra(int(bool(on)))


def tri_tb_lapl_level(z_faces, x_faces, y_faces, vol, dut, dur, level3, level2, coefs):
    """One level of LaplTBCompute (dur None; LaplTRCompute with dur,
    MULTI/JacAccGrav_Mod.f90:1312-1667): the finest faces z (F1, F1G, DTU1,
    DUU1) (n3, n2, n1+1), x (n3, n2+1, n1), y (n3+1, n2, n1) and cells
    coarsened with the shifts 2^level2-1 (directions 1, 2) and 2^level3-1
    (direction 3), then Compute_3D, with the couplings between planes when
    level2 == level3.  Returns d, u1, l1, u2, l2, u3, l3 as tri_tb_compute_3d."""
    lib = load()
    fs = [np.ascontiguousarray(a, dtype=np.float64) for a in list(z_faces) + list(x_faces) + list(y_faces)]
    vol, dut = (np.ascontiguousarray(a, dtype=np.float64) for a in (vol, dut))
    tr = dur is not None
    durr = np.ascontiguousarray(dur, dtype=np.float64) if tr else None
    n3, n2, n1 = vol.shape
    c3 = -(-n3 // 2 ** level3)
    c2, c1 = -(-n2 // 2 ** level2), -(-n1 // 2 ** level2)
    keys = ("beta0_dtp", "fac1_l", "fac1_r", "grav_comp", "fac_anela", "fac2_l", "fac2_r", "fac3_l", "fac3_r")
    sv = np.array([float(coefs.get(k, 1.0 if k == "beta0_dtp" else 0.0)) for k in keys])
    d = np.empty((c3, c2, c1, 4))
    u1 = np.empty((c3, c2, max(c1 - 1, 1), 4))
    l1 = np.empty_like(u1)
    u2 = np.empty((c3, max(c2 - 1, 1), c1, 4))
    l2 = np.empty_like(u2)
    u3 = np.zeros((max(c3 - 1, 1), c2, c1, 4))
    l3 = np.zeros_like(u3)
    lib.ora_tri_tb_lapl_level(int(tr), n3, n2, n1, _p(sv), _ptrs(fs), _p(vol), _p(dut),
                              _p(durr) if tr else None, int(level3), int(level2), _p(d), _p(u1), _p(l1), _p(u2),
                              _p(l2), _p(u3), _p(l3))
    return (d, u1[:, :, :c1 - 1], l1[:, :, :c1 - 1], u2[:, :c2 - 1], l2[:, :c2 - 1], u3[:c3 - 1], l3[:c3 - 1])


def tri_tb_lapl_compute(z_faces, x_faces, y_faces, vol, dut, dur=None, ref_level=1, **coefs):
    """LaplTBCompute / LaplTRCompute (MULTI/JacAccGrav_Mod.f90:1312-1667): the
    hierarchy of ref_level levels, level L3 with the plane levels L2 = L3 ..
    ref_level-1, each built from the finest fields (tri_tb_lapl_level), as
    tri_tb_multigrid_3d takes it: [(plane_levels, u3, l3), ...]."""
    levels = []
    for L3 in range(ref_level):
        planes, u3, l3 = [], None, None
        for L2 in range(L3, ref_level):
            blk = tri_tb_lapl_level(z_faces, x_faces, y_faces, vol, dut, dur, L3, L2, coefs)
            planes.append(blk[:5])
            if L2 == L3:
                u3, l3 = blk[5], blk[6]
        levels.append((planes, u3, l3))
    return levels


class OracleProj:
    """Oracle of the pressure projection of one block (oracle/asam_proj.c)
    whose sides are closed walls or periodic (the grid's periodic_x/y/z).

    Arrays use the same Fortran layouts as the library: faces with uF/vF/wF
    extents, interior cell fields (nz, ny, nx), padded state fields.  A block
    with periodic sides carries boundary face unknowns: its PressureVelocity
    vectors (rhs, fgmres, psolve1, matvec1, update) are flat arrays of
    ``nvec`` values, the pressure (x fastest) followed by u_w, u_e, v_s, v_n,
    w_b, w_t of the periodic sides; a closed block keeps (nz, ny, nx)."""

    def __init__(self, geo, dx, dy, dz, weights, metr=None, ref_level=4, gauss_iter2=1, gauss_iter3=1, mult_iter2=1,
                 mult_iter3=1, zebra=1, fac_anela=1.0, prefac2=0.5):
        self.lib = load()
        g = geo.grid
        self.grid = g
        n = 2 * (g.nx + g.ny + g.nz)
        metr = np.ones(n) if metr is None else metr
        self._keep = [np.ascontiguousarray(a, dtype=np.float64) for a in
                      (geo.fu, geo.fv, geo.fw, geo.volc, *weights, dx, dy, dz, metr)]
        per = (int(bool(g.periodic_x)), int(bool(g.periodic_y)), int(bool(g.periodic_z)))
        ip = (C.c_int * 12)(g.nx, g.ny, g.nz, ref_level, gauss_iter2, gauss_iter3, mult_iter2, mult_iter3, zebra,
                            *per)
        dp = (C.c_double * 2)(fac_anela, prefac2)
        self.h = self.lib.ora_proj_create(ip, dp, *[_p(a) for a in self._keep])
        self.nvec = int(self.lib.ora_proj_nvec(self.h))
        self.nface = self.nvec - g.nx * g.ny * g.nz

    def _pv(self):
        return self._cell() if self.nface == 0 else np.zeros(self.nvec)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ora_proj_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_zebra(self, on: bool):
        self.lib.ora_proj_set_zebra(self.h, int(on))

    def lapl_compute(self, beta0, dtp):
        self.lib.ora_lapl_compute(self.h, beta0, dtp)

    def lapl_get(self, level3, level2, which, dirichlet=False):
        f = self.lib.ora_lapl_get_dirichlet if dirichlet else self.lib.ora_lapl_get
        n = f(self.h, level3, level2, which, None)
        if n < 0:
            raise ValueError("no such level")
        out = np.empty(n)
        f(self.h, level3, level2, which, _p(out))
        return out

    def _cell(self):
        g = self.grid
        return np.empty((g.nz, g.ny, g.nx))

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = self._cell()
        self.lib.ora_lapl_matvec(self.h, _p(x), _p(y))
        return y

    def vcycle(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = self._cell()
        self.lib.ora_lapl_vcycle(self.h, _p(b), _p(x))
        return x

    def vcycle_dirichlet(self, b):
        """One Solve_3D on LaplDirichlet (periodic blocks)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = self._cell()
        if self.lib.ora_lapl_vcycle_dirichlet(self.h, _p(b), _p(x)) != 0:
            raise ValueError("no Dirichlet hierarchy: the block has no periodic side")
        return x

    def psolve1(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        b = self._pv()
        self.lib.ora_psolve1(self.h, _p(x), _p(b))
        return b

    def matvec1(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        b = self._pv()
        self.lib.ora_matvec1(self.h, _p(x), _p(b))
        return b

    def exchange(self, v):
        """Exchange of the face unknowns in place (u_w = u_w + u_e; u_e = u_w ...)."""
        self.lib.ora_proj_exchange(self.h, _p(v))

    def dot2(self, x, y):
        return float(self.lib.ora_proj_dot2(self.h, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y))))

    def fgmres(self, x, b, maxiter=10, tol=1e-6, step=10):
        """x updated in place; returns (inner steps, rho, rho0)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        rho, rho0 = C.c_double(), C.c_double()
        steps = self.lib.ora_fgmres(self.h, _p(x), _p(b), maxiter, tol, step, C.byref(rho), C.byref(rho0))
        return steps, rho.value, rho0.value

    def rhs(self, u, v, w, incr_th=None):
        b = self._pv()
        self.lib.ora_proj_rhs(self.h, _p(u), _p(v), _p(w), None if incr_th is None else _p(incr_th), _p(b))
        return b

    def update(self, x, u, v, w, incr_th=None, incr_rho=None, incr_c=(), c=(), rho=None):
        """UpdateVelocity in place (x becomes x*DUT)."""
        nc = len(incr_c)
        pi = (C.c_void_p * max(1, nc))(*[_p(a) for a in incr_c])
        pc = (C.c_void_p * max(1, nc))(*[_p(a) for a in c])
        self.lib.ora_proj_update(self.h, _p(x), _p(u), _p(v), _p(w), None if incr_th is None else _p(incr_th),
                                 None if incr_rho is None else _p(incr_rho), nc, pi, pc,
                                 None if rho is None else _p(rho))

    def weights_density(self, rth, rho, rv, rc, rr, t):
        """Density-kind sound weights (padded inputs; None for absent water);
        returns [DTU, DTV, DTW, DUU, DUV, DUW, DUT, DTT] and installs them."""
        g = self.grid
        nx, ny, nz = g.nx, g.ny, g.nz
        out = [np.empty((nz, ny, nx + 1)), np.empty((nz, ny + 1, nx)), np.empty((nz + 1, ny, nx)),
               np.empty((nz, ny, nx + 1)), np.empty((nz, ny + 1, nx)), np.empty((nz + 1, ny, nx)),
               np.empty((nz, ny, nx)), np.empty((nz, ny, nx))]
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (rth, rho, rv, rc, rr, t)]
        ptrs = [None if a is None else _p(a) for a in keep]
        self.lib.ora_weights_density(self.h, *ptrs, *[_p(a) for a in out])
        self.lib.ora_proj_set_weights(self.h, *[_p(a) for a in out])
        return out
