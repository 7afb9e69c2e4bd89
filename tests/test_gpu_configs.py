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
* configuration 2's generator on a 48x48x128 periodic window: 2 full
  Rosenbrock steps of the dynamical core at 1e-12.
The step counts are what the single-threaded oracle finishes in a few minutes.
"""
from __future__ import annotations

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
