"""GPU parity on the benchmark configurations themselves (not only on small
cases), through the C-ABI against the oracle:

* configuration 1: the 64x64x64 dry warm bubble (periodic in x/y, rigid bottom
  and lid, dx=dy=dz=100 m, u=10 m/s, theta' 2 K bubble + U(+-0.01 K) noise),
  full Rosenbrock steps with prognostic momentum and the projection
  (boundary face unknowns of the periodic sides), dt = 1 s, BiCGStab and
  FGMRES at 1e-10: 1e-12 relative per prognostic field and in the face
  velocities after every one of 3 steps, iteration counts equal or within one
  (the six LR momentum components and the three face velocities are the
  components of one vector each and are measured against its largest
  component, cases.state_relerr);
* configuration 2 at its full size 256x256x128 (cut-cell hill with roughness,
  snapping, the small-cell merge, stretched levels): 2 transport steps
  (prescribed winds, dt = 2 s, BiCGStab 1e-10) at 1e-12 per field;
* configuration 2's generator on a 48x48x128 periodic window, and the same
  window of the headline workload (configuration 3's seed): 2 full Rosenbrock
  steps of the dynamical core at 1e-12 each;
* configuration 5 at its full size (128x128x64 cut-cell hill, h = 800 m,
  half-width 4 km, a passive tracer, RosRK3 dt = 2 s, 40 steps, checkpoints
  every 8, J = volume integral of the tracer mixing ratio squared over a
  16x16x8 box at the final time): the gradient with respect to the initial
  tracer and the wind against central differences (eps = 1e-6) along 32
  seeded directions, and the dot-product tests of the stage-solve and step
  adjoints.
The step counts are what the single-threaded oracle finishes in a few minutes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle
from asam_gb300 import METHODS, TransportBlock
from asam_gb300 import geometry as G
from tests import cases

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-12


def _kinds(ncomp, mom):
    k = np.ones((ncomp, 6), np.int32)
    for q, p in enumerate(mom):
        for sd in range(6):
            k[p, sd] = 2 if q // 2 == sd // 2 else 1
    return k


def _dyn_parity(work, dt, nsteps):
    geo, vel, st, pos, (dx, dy, dz), bc = work
    nc = st.c.shape[0]
    o = oracle.Oracle(geo, bc=_kinds(nc, pos["mom"]))
    pr = oracle.OracleProj(geo, dx, dy, dz, G.projection_inputs(geo)[0], zebra=1)
    sc = [pos[k] for k in ("qv", "tracer") if k in pos]
    cr, cg = st.c.copy(), st.c.copy()
    ur = [a.copy() for a in vel]
    with TransportBlock(geo, ncomp=nc, rho_pos=0, bicgstab_tol=1e-10) as blk:
        blk.set_velocity(*vel)
        blk.proj_setup(dx, dy, dz, tol=1e-10, max_restart=20)
        blk.dyn_setup(pos["th"], pos["mom"], rv_pos=pos.get("qv", -1), bound_cells=bc, scalars=sc)
        for step in range(nsteps):
            it_r, _, ps_r, _ = o.ros_step_dyn(pr, cr, ur, dt, rho_pos=0, th_pos=pos["th"], pos=pos["mom"], dx=dx,
                                              dy=dy, dz=dz, rv_pos=pos.get("qv", -1), bound=bc, scalars=sc,
                                              bicg_tol=1e-10, proj_tol=1e-10, proj_maxiter=20)
            (it_g, _), (ps_g, _) = blk.Ros3MetC_dyn(cg, dt)
            for a, b in zip(it_g, it_r):
                assert abs(abs(a) - abs(b)) <= 1, (step, it_g, it_r)
            for a, b in zip(ps_g, ps_r):
                assert abs(a - b) <= 1, (step, ps_g, ps_r)
            errs = cases.state_relerr(cg, cr, mom=pos["mom"])
            assert max(errs) <= STEP_TOL, (step, errs, cases.field_relerr(cg, cr))
            vmax = max(float(np.max(np.abs(b))) for b in ur)
            for a, b in zip(blk.get_velocity(), ur):
                assert float(np.max(np.abs(a - b))) <= STEP_TOL * vmax, step


def test_config1_bubble_64_full_step(built_lib):
    _dyn_parity(G.bubble_dyn_case(64, 64, 64), 1.0, 3)


def test_config2_256_transport_steps(built_lib):
    geo, vel, st = G.hill_case(256, 256, 128, seed=2)
    o = oracle.Oracle(geo)
    cr, cg = st.c.copy(), st.c.copy()
    with TransportBlock(geo, ncomp=st.c.shape[0], method="RosRK3", bicgstab_tol=1e-10) as blk:
        blk.set_velocity(*vel)
        for step in range(2):
            it_r, _ = o.ros_step(cr, vel, 2.0, method=METHODS["RosRK3"], tol=1e-10)
            it_g, _ = blk.Ros3MetC(cg, 2.0)
            for a, b in zip(it_g, it_r):
                assert abs(abs(a) - abs(b)) <= 1, (step, it_g, it_r)
            errs = cases.field_relerr(cg, cr)
            assert max(errs) <= STEP_TOL, (step, errs)


def test_config2_window_full_step(built_lib):
    _dyn_parity(G.hill_dyn_case(48, 48, 128, seed=2), 2.0, 2)


def test_config3_window_full_step(built_lib):
    """The headline workload's generator and seed (the mixed-precision
    configuration, 512x512x128, seed 3) on a 48x48x128 periodic window: 2 full
    FP64 dynamical steps at 1e-12 against the oracle."""
    _dyn_parity(G.hill_dyn_case(48, 48, 128, seed=3), 2.0, 2)


ADJ_TOL = 1e-14  # Krylov tolerance of every forward and adjoint solve below


def _config5():
    """The adjoint configuration's workload and target box (the bench's)."""
    geo, vel, st = G.hill_case(128, 128, 64, seed=5, height=800.0, halfwidth=4000.0, moist=False, momentum=False,
                               tracer=True)
    g = geo.grid
    i0 = max(1, int(0.3 * g.nx) + 1)
    j0 = max(1, g.ny // 2 - 7)
    k0 = max(1, g.nz // 8)
    box = (i0, min(g.nx, i0 + 15), j0, min(g.ny, j0 + 15), k0, min(g.nz, k0 + 7))
    return geo, vel, st, box


def _interior(geo, x):
    return x.reshape(geo.grid.pshape)[1:-1, 1:-1, 1:-1]


def _idot(geo, x, y):
    return float(np.sum(_interior(geo, x) * _interior(geo, y)))


def _rand_interior(geo, rng):
    x = np.zeros(geo.grid.pshape)
    x[1:-1, 1:-1, 1:-1] = rng.standard_normal(x[1:-1, 1:-1, 1:-1].shape)
    return x.reshape(-1)


def test_config5_adjoint_full_size(built_lib):
    geo, vel, st, box = _config5()
    g = geo.grid
    nc = st.c.shape[0]
    comp = nc - 1
    nsteps, dt, ck = 40, 2.0, 8
    sl = (slice(box[4], box[5] + 1), slice(box[2], box[3] + 1), slice(box[0], box[1] + 1))
    uf, vf, wf = (np.ascontiguousarray(v, dtype=np.float64) for v in vel)
    with TransportBlock(geo, ncomp=nc, method="RosRK3", bicgstab_tol=ADJ_TOL, bicgstab_maxiter=400) as blk:
        lib = blk.lib
        blk.set_velocity(uf, vf, wf)
        c = np.ascontiguousarray(st.c, dtype=np.float64).copy()
        J = C.c_double()
        gc, gr = np.empty(g.npad), np.empty(g.npad)
        gu, gv, gw = np.empty(uf.size), np.empty(vf.size), np.empty(wf.size)
        cbox = (C.c_int * 6)(*box)
        assert lib.asam_tracer_wind_gradient(blk.h, c.ctypes.data, comp, nsteps, dt, ck, cbox, ADJ_TOL, C.byref(J),
                                             gc.ctypes.data, gr.ctypes.data, gu.ctypes.data, gv.ctypes.data,
                                             gw.ctypes.data) == 0

        def objective(state, u, v, w):
            blk.set_velocity(u, v, w)
            s = state.copy()
            for _ in range(nsteps):
                blk.Ros3MetC(s, dt)
            s = blk.ExchangeCell(s)
            q = s[comp] / (s[0] + 1e-30)
            return float(np.sum(q[sl] ** 2 * geo.volc[sl]))

        j0 = objective(c, uf, vf, wf)
        assert abs(j0 - J.value) <= 1e-10 * abs(J.value), (j0, J.value)
        rng = np.random.default_rng(55)
        eps = 1e-6
        cmax = float(np.abs(c[comp]).max())
        rel_c, rel_w = [], []
        for q in range(32):  # 16 directions in the initial tracer, 16 in the wind
            cp, cm = c.copy(), c.copy()
            up, um = [uf, vf, wf], [uf, vf, wf]
            if q % 2 == 0:
                dc = (_rand_interior(geo, rng) * cmax).reshape(c[comp].shape)
                cp[comp] += eps * dc
                cm[comp] -= eps * dc
                ad = _idot(geo, gc, dc.reshape(-1))
            else:  # relative perturbations: a face at rest stays at rest
                dw = [rng.standard_normal(f.shape) * 1e-2 * f for f in (uf, vf, wf)]
                up = [f + eps * e for f, e in zip((uf, vf, wf), dw)]
                um = [f - eps * e for f, e in zip((uf, vf, wf), dw)]
                ad = sum(float(np.sum(gq * e.reshape(-1))) for gq, e in zip((gu, gv, gw), dw))
            fd = (objective(cp, *up) - objective(cm, *um)) / (2 * eps)
            (rel_c if q % 2 == 0 else rel_w).append(abs(fd - ad) / abs(ad))
        blk.set_velocity(uf, vf, wf)
        rel_c, rel_w = np.array(rel_c), np.array(rel_w)
        print("config5 fd rel: tracer max %.3e median %.3e, wind max %.3e median %.3e"
              % (rel_c.max(), np.median(rel_c), rel_w.max(), np.median(rel_w)))
        # exact: the tracer gradient against the tangent-linear chain of the
        # same 40 steps (dot-product identity over the trajectory)
        states = [c.copy()]
        for _ in range(nsteps):
            s1 = states[-1].copy()
            blk.Ros3MetC(s1, dt)
            states.append(s1)
        final = blk.ExchangeCell(states[-1])
        dJdc = np.zeros(g.pshape)
        dJdc[sl] = 2.0 * final[comp][sl] / (final[0][sl] + 1e-30) ** 2 * geo.volc[sl]
        tlm_rel = []
        for _ in range(4):
            d = _rand_interior(geo, rng) * cmax
            dd = d.copy()
            for st_ in states[:-1]:
                out = np.empty_like(dd)
                assert lib.asam_ros_step_tlm(blk.h, st_.ctypes.data, comp, dd.ctypes.data, out.ctypes.data, dt,
                                             ADJ_TOL) == 0
                dd = out
            tl = _idot(geo, dJdc.reshape(-1), dd)
            ad = _idot(geo, gc, d)
            tlm_rel.append(abs(tl - ad) / abs(ad))
        print("config5 tangent-linear chain rel: max %.3e" % max(tlm_rel))
        # dot-product test of one step's adjoint at the initial state
        du = _rand_interior(geo, rng) * cmax * 1e-2
        out = np.empty_like(du)
        assert lib.asam_ros_step_tlm(blk.h, c.ctypes.data, comp, du.ctypes.data, out.ctypes.data, dt, ADJ_TOL) == 0
        lam = _rand_interior(geo, rng)
        lout = np.empty_like(lam)
        assert lib.asam_ros_step_adj(blk.h, c.ctypes.data, comp, lam.ctypes.data, lout.ctypes.data, dt, ADJ_TOL) == 0
        lhs, rhs = _idot(geo, out, lam), _idot(geo, du, lout)
        step_dot = abs(lhs - rhs) / abs(lhs)
        # dot-product test of the stage solve's adjoint (the step's first stage matrix)
        blk.Jac(c, dt)
        b = _rand_interior(geo, rng)
        y = _rand_interior(geo, rng)
        B = np.zeros_like(c)
        B[comp] = b.reshape(c[comp].shape)
        X = np.zeros_like(c)
        it_f, _ = blk.BiCGStabMetSp(X, B, 400, 1e-15)
        x = np.ascontiguousarray(X[comp]).reshape(-1)
        z = np.zeros_like(y)
        mi, tl = C.c_int(800), C.c_double(1e-15)
        assert lib.asam_bicgstab_adj(blk.h, z.ctypes.data, y.ctypes.data, C.byref(mi), C.byref(tl)) in (0, 1)
        xy, bz = _idot(geo, x, y), _idot(geo, b, z)
        solve_dot = abs(xy - bz) / abs(xy)
        print("config5 dot: step %.3e (%r %r) solve %.3e (%r %r, forward %d, adjoint %d iterations)"
              % (step_dot, lhs, rhs, solve_dot, xy, bz, it_f, mi.value))
        assert step_dot <= 1e-12, step_dot
        assert solve_dot <= 1e-12, solve_dot
        assert max(tlm_rel) <= 1e-10, tlm_rel
        # central differences: the Koren limiter's kinks inside +-eps limit
        # their agreement with the exact derivative
        assert rel_c.max() <= 2e-3 and np.median(rel_c) <= 1e-4, rel_c
        assert rel_w.max() <= 2e-3 and np.median(rel_w) <= 1e-4, rel_w


def test_config2_256_transport_50_steps(built_lib):
    """Configuration 2's full run on the GPU (256x256x128, 50 transport steps,
    dt = 2 s, BiCGStab 1e-10), beyond what the oracle finishes in a test: every
    solve converges, every field stays finite, and the total mass of Rho and of
    the tracer (TotalScalar) is conserved to round-off over the whole run."""
    geo, vel, st = G.hill_case(256, 256, 128, seed=2)
    c = st.c.copy()
    with TransportBlock(geo, ncomp=c.shape[0], method="RosRK3", bicgstab_tol=1e-10, bicgstab_maxiter=30) as blk:
        blk.set_velocity(*vel)
        comps = [0, c.shape[0] - 1]
        m0 = [blk.TotalScalar(c, q) for q in comps]
        for step in range(50):
            its, res = blk.Ros3MetC(c, 2.0)
            # MaxIter sentinels: -Iter (half step) or Iter <= 30 converged; 2*Iter = 60 not
            assert all(abs(i) <= 30 for i in its), (step, its, res)
        m1 = [blk.TotalScalar(c, q) for q in comps]
    assert np.isfinite(c).all()
    for a, b in zip(m0, m1):
        assert abs(b - a) <= 1e-12 * abs(a), (a, b)
