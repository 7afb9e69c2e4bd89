"""Tangent-linear and adjoint pair of the transport stage (GPU, through the C-ABI).

Checks: tangent-linear flux and step against central finite differences of the
forward operators; dot-product tests <L x, y> = <x, L^T y> for the flux, the
stage operator, the stage solve and the whole step; the checkpointed
gradient of J = sum_box (tracer mixing ratio)^2 V against central finite
differences and the tangent-linear chain.
"""
import ctypes as C

import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

NAME = "hill_24x20x16"


@pytest.fixture(scope="module")
def env(built_lib):
    import asam_gb300
    from asam_gb300 import _lib

    return asam_gb300, _lib.load()


def _smooth_tracer(geo, c):
    """Replace the last component by Rho times a smooth O(1) mixing ratio, so that
    cell-to-cell differences are far larger than the finite-difference steps and
    the Koren limiter does not switch branch inside them."""
    g = geo.grid
    x = (np.arange(g.nx + 2) - 0.5) * g.dx
    y = (np.arange(g.ny + 2) - 0.5) * g.dy
    zc = 0.5 * (g.zP[:-1] + g.zP[1:])
    z = np.concatenate([[zc[0] - g.dz[0]], zc, [zc[-1] + g.dz[-1]]])
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    q = 1.0 + 0.3 * np.sin(2 * np.pi * X / (g.nx * g.dx) + 0.3) * np.cos(2 * np.pi * Y / (g.ny * g.dy)) \
        + 0.2 * Z / g.zP[-1]
    out = c.copy()
    out[-1] = c[0] * q
    return out


def _setup(env, name=NAME, method="RosRK3", tol=1e-13):
    asam, lib = env
    geo, vel, st = cases.get(name)
    blk = asam.TransportBlock(geo, ncomp=st.c.shape[0], method=method, bicgstab_tol=tol, bicgstab_maxiter=200)
    blk.set_velocity(*vel)
    c = blk.ExchangeCell(_smooth_tracer(geo, st.c))
    return blk, geo, vel, c


def _interior(geo, x):
    g = geo.grid
    return x.reshape(g.pshape)[1:-1, 1:-1, 1:-1]


def _idot(geo, x, y):
    return float(np.sum(_interior(geo, x) * _interior(geo, y)))


def _rand_interior(geo, rng):
    x = np.zeros(geo.grid.pshape)
    x[1:-1, 1:-1, 1:-1] = rng.standard_normal(x[1:-1, 1:-1, 1:-1].shape)
    return x.reshape(-1)


def test_flux_tlm_matches_central_differences(env):
    blk, geo, vel, c = _setup(env)
    lib = blk.lib
    comp = c.shape[0] - 1
    rng = np.random.default_rng(11)
    dc = rng.standard_normal(c[comp].shape).reshape(-1) * np.abs(c[comp]).max()
    df = np.empty_like(dc)
    assert lib.asam_fcn_tlm(blk.h, c.ctypes.data, comp, dc.ctypes.data, df.ctypes.data) == 0
    eps = 1e-8
    cp, cm = c.copy(), c.copy()
    cp[comp] += eps * dc.reshape(c[comp].shape)
    cm[comp] -= eps * dc.reshape(c[comp].shape)
    fd = (blk.Fcn(cp)[comp] - blk.Fcn(cm)[comp]).reshape(-1) / (2 * eps)
    err = np.abs(fd - df)
    scale = np.abs(df).max()
    # piecewise linear: agreement except where a limiter branch flips inside +-eps
    assert np.quantile(err, 0.999) <= 1e-6 * scale
    blk.close()


def test_flux_adjoint_dot_product(env):
    blk, geo, vel, c = _setup(env)
    lib = blk.lib
    comp = c.shape[0] - 1
    rng = np.random.default_rng(5)
    n = geo.grid.npad
    x = rng.standard_normal(n)
    y = rng.standard_normal(n)
    fx = np.empty(n)
    aty = np.empty(n)
    assert lib.asam_fcn_tlm(blk.h, c.ctypes.data, comp, x.ctypes.data, fx.ctypes.data) == 0
    assert lib.asam_fcn_adj(blk.h, c.ctypes.data, comp, y.ctypes.data, aty.ctypes.data) == 0
    lhs, rhs = float(fx @ y), float(x @ aty)
    assert abs(lhs - rhs) <= 1e-13 * max(abs(lhs), np.abs(fx).sum() * np.abs(y).max())
    blk.close()


def test_stage_operator_transpose(env):
    blk, geo, vel, c = _setup(env)
    lib = blk.lib
    blk.Jac(c, 4.0)
    n = geo.grid.npad
    rng = np.random.default_rng(6)
    val = blk.jac_matrix()
    x = rng.standard_normal(n)
    y = rng.standard_normal(n)
    aty = np.empty(n)
    assert lib.asam_matvec_adj(blk.h, x.ctypes.data, aty.ctypes.data) == 0  # A^T x
    import tests.pyref as pyref

    A = pyref.dia_scipy(val, geo.grid)
    assert np.allclose(aty, A.T @ x, rtol=1e-13, atol=1e-13 * np.abs(aty).max())
    blk.close()


def test_stage_solve_adjoint_dot_product(env):
    blk, geo, vel, c = _setup(env)
    lib = blk.lib
    blk.Jac(c, 6.0)
    comp = c.shape[0] - 1
    rng = np.random.default_rng(7)
    b = _rand_interior(geo, rng)
    y = _rand_interior(geo, rng)
    B = np.zeros_like(c)
    B[comp] = b.reshape(c[comp].shape)
    X = np.zeros_like(c)
    # both solves to 1e-15 (the limit may end them one iteration short of it:
    # status 1 is accepted), so the dot-product identity holds to 1e-12
    it, tol = blk.BiCGStabMetSp(X, B, 400, 1e-15)
    x = np.ascontiguousarray(X[comp]).reshape(-1)
    z = np.zeros_like(y)
    mi = C.c_int(800)
    tl = C.c_double(1e-15)
    st = lib.asam_bicgstab_adj(blk.h, z.ctypes.data, y.ctypes.data, C.byref(mi), C.byref(tl))
    assert st in (0, 1)
    lhs, rhs = _idot(geo, x, y), _idot(geo, b, z)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs), (lhs, rhs, it, mi.value)
    blk.close()


def test_step_tlm_and_adjoint(env):
    blk, geo, vel, c = _setup(env)
    lib = blk.lib
    comp = c.shape[0] - 1
    dt = 4.0
    tol = 1e-14
    rng = np.random.default_rng(8)
    du = _rand_interior(geo, rng) * np.abs(c[comp]).max() * 1e-2
    out = np.empty_like(du)
    assert lib.asam_ros_step_tlm(blk.h, c.ctypes.data, comp, du.ctypes.data, out.ctypes.data, dt, tol) == 0
    # central differences of the forward step
    eps = 1e-6
    cp, cm = c.copy(), c.copy()
    cp[comp] += eps * du.reshape(c[comp].shape)
    cm[comp] -= eps * du.reshape(c[comp].shape)
    blk.Ros3MetC(cp, dt)
    blk.Ros3MetC(cm, dt)
    fd = (cp[comp] - cm[comp]).reshape(-1) / (2 * eps)
    e = _interior(geo, fd - out)
    assert np.quantile(np.abs(e), 0.999) <= 1e-6 * np.abs(_interior(geo, out)).max()
    # dot-product test of the step adjoint
    lam = _rand_interior(geo, rng)
    lout = np.empty_like(lam)
    assert lib.asam_ros_step_adj(blk.h, c.ctypes.data, comp, lam.ctypes.data, lout.ctypes.data, dt, tol) == 0
    lhs, rhs = _idot(geo, out, lam), _idot(geo, du, lout)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1e-300)
    blk.close()


def test_checkpointed_gradient(env):
    blk, geo, vel, c = _setup(env)
    lib = blk.lib
    comp = c.shape[0] - 1
    g = geo.grid
    nsteps, dt, ck = 5, 3.0, 2
    box = (C.c_int * 6)(3, 10, 4, 12, 2, 8)
    J = C.c_double()
    grad = np.empty(g.npad)
    tol = 1e-14
    assert lib.asam_tracer_gradient(blk.h, c.ctypes.data, comp, nsteps, dt, ck, box, tol, C.byref(J),
                                    grad.ctypes.data) == 0

    def objective(state):
        s = state.copy()
        for _ in range(nsteps):
            blk.Ros3MetC(s, dt)
        s = blk.ExchangeCell(s)
        q = s[comp] / (s[0] + 1e-30)
        V = geo.volc
        sl = (slice(box[4], box[5] + 1), slice(box[2], box[3] + 1), slice(box[0], box[1] + 1))
        return float(np.sum(q[sl] ** 2 * V[sl]))

    assert abs(objective(c) - J.value) <= 1e-10 * abs(J.value)
    # forward trajectory for the tangent-linear chain
    states = [c.copy()]
    for _ in range(nsteps):
        s = states[-1].copy()
        blk.Ros3MetC(s, dt)
        states.append(s)
    final = blk.ExchangeCell(states[-1])
    sl = (slice(box[4], box[5] + 1), slice(box[2], box[3] + 1), slice(box[0], box[1] + 1))
    dJdc = np.zeros(g.pshape)
    dJdc[sl] = 2.0 * final[comp][sl] / (final[0][sl] + 1e-30) ** 2 * geo.volc[sl]
    rng = np.random.default_rng(9)
    fd_rel = []
    for direction in range(32):  # 32 seeded directions
        d = _rand_interior(geo, rng) * np.abs(c[comp]).max()
        ad = _idot(geo, grad, d)
        # exact: the tangent-linear chain of the same steps (dot-product identity)
        dd = d.copy()
        for s in range(nsteps):
            out = np.empty_like(dd)
            assert lib.asam_ros_step_tlm(blk.h, states[s].ctypes.data, comp, dd.ctypes.data, out.ctypes.data, dt,
                                         tol) == 0
            dd = out
        tl = _idot(geo, dJdc.reshape(-1), dd)
        assert abs(tl - ad) <= 1e-10 * abs(ad), (direction, tl, ad)
        # central finite differences (eps = 1e-6); the limiter's kinks inside the
        # perturbation limit the agreement
        eps = 1e-6
        cp, cm = c.copy(), c.copy()
        cp[comp] += eps * d.reshape(c[comp].shape)
        cm[comp] -= eps * d.reshape(c[comp].shape)
        fd = (objective(cp) - objective(cm)) / (2 * eps)
        fd_rel.append(abs(fd - ad) / abs(ad))
    # the Koren limiter's kinks inside the +-eps perturbation bound the finite
    # differences of some directions: every direction within 1e-3, the median
    # within 1e-5 (the exact check above is the tangent-linear chain)
    fd_rel = np.array(fd_rel)
    assert fd_rel.max() <= 1e-3, fd_rel
    assert np.median(fd_rel) <= 1e-5, fd_rel
    blk.close()


def test_wind_and_density_gradient(env):
    """Coupled density-component adjoint: gradient of the same objective with
    respect to the initial tracer, the initial density and the face mass fluxes.
    The tracer part equals the density-fixed gradient (density does not depend
    on the tracer); the density and wind parts match central finite
    differences (faces with zero velocity left unperturbed)."""
    blk, geo, vel, c = _setup(env)
    lib = blk.lib
    comp = c.shape[0] - 1
    g = geo.grid
    nsteps, dt, ck = 3, 3.0, 2
    box = (C.c_int * 6)(3, 10, 4, 12, 2, 8)
    tol = 1e-14
    J = C.c_double()
    gc, gr = np.empty(g.npad), np.empty(g.npad)
    uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
    gu, gv, gw = np.empty(uf.size), np.empty(vf.size), np.empty(wf.size)
    assert lib.asam_tracer_wind_gradient(blk.h, c.ctypes.data, comp, nsteps, dt, ck, box, tol, C.byref(J),
                                         gc.ctypes.data, gr.ctypes.data, gu.ctypes.data, gv.ctypes.data,
                                         gw.ctypes.data) == 0
    J0 = C.c_double()
    g0 = np.empty(g.npad)
    assert lib.asam_tracer_gradient(blk.h, c.ctypes.data, comp, nsteps, dt, ck, box, tol, C.byref(J0),
                                    g0.ctypes.data) == 0
    assert abs(J.value - J0.value) <= 1e-12 * abs(J0.value)
    assert np.abs(_interior(geo, gc - g0)).max() <= 1e-8 * np.abs(_interior(geo, g0)).max()
    sl = (slice(box[4], box[5] + 1), slice(box[2], box[3] + 1), slice(box[0], box[1] + 1))

    def objective(state, u, v, w):
        blk.set_velocity(u, v, w)
        s = state.copy()
        for _ in range(nsteps):
            blk.Ros3MetC(s, dt)
        s = blk.ExchangeCell(s)
        q = s[comp] / (s[0] + 1e-30)
        return float(np.sum(q[sl] ** 2 * geo.volc[sl]))

    rng = np.random.default_rng(21)
    eps = 1e-5  # the solves' 1e-13 tolerance limits the finite differences
    # density: perturb the interior density (every mixing ratio changes with it)
    for _ in range(2):
        d = _rand_interior(geo, rng).reshape(g.pshape) * 1e-3 * c[0]
        cp, cm = c.copy(), c.copy()
        cp[0] += eps * d
        cm[0] -= eps * d
        fd = (objective(cp, uf, vf, wf) - objective(cm, uf, vf, wf)) / (2 * eps)
        ad = float(np.sum(_interior(geo, gr) * _interior(geo, d.reshape(-1))))
        assert abs(fd - ad) <= 1e-4 * max(abs(ad), 1e-30) + 1e-12 * abs(J.value), (fd, ad)
    # wind: relative perturbations of the active faces (no sign change)
    for _ in range(2):
        du = rng.standard_normal(uf.shape) * 1e-2 * uf
        dw = rng.standard_normal(wf.shape) * 1e-2 * wf
        fd = (objective(c, uf + eps * du, vf, wf + eps * dw) - objective(c, uf - eps * du, vf, wf - eps * dw)) / (
            2 * eps)
        ad = float(np.sum(gu * du.reshape(-1)) + np.sum(gw * dw.reshape(-1)))
        assert abs(fd - ad) <= 1e-4 * abs(ad), (fd, ad)
    blk.set_velocity(uf, vf, wf)
    blk.close()
