"""GPU parity of the diffusion terms with the oracle (DiffusionCompute,
JacDiffusionCompute, ADVECT/Diffusion_Mod.f90:11-275, 1504-1708).

Bit-exact: the flux right-hand side with diffusion (every case: periodic
sides, closed walls, one column, one-cell-wide slab) and the stage matrix with
the diffusion Jacobian.  The Rosenbrock step with diffusion: 1e-12 per field
(FP64), 1e-10 (refined); the dynamical step of a closed block: 1e-12 per
field after each step (the momentum components as one vector) and in the
face velocities.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

import oracle
from asam_gb300 import TransportBlock
from asam_gb300 import geometry as G
from tests import cases

pytestmark = pytest.mark.gpu

ALL = list(cases.CASES)


def _setup(name, **kw):
    geo, vel, st = cases.get(name)
    # a consistent cut-cell geometry has the faces of zero-volume cells closed;
    # with an open face the diffusion Jacobian row of such a cell carries
    # entries of order 1/Eps (as in the reference) and the stage solve loses
    # its meaning there
    geo = G.close_dead_faces(copy.deepcopy(geo))
    o = oracle.Oracle(geo)
    c = o.bound_cond(o.exchange_cell(st.c))
    dh, dv = G.diffusion_coefficients(geo, c[0], seed=3)
    o.set_diffusion(dh, dv)
    blk = TransportBlock(geo, ncomp=st.c.shape[0], rho_pos=0, **kw)
    blk.set_velocity(*vel)
    blk.set_diffusion(dh, dv)
    return geo, vel, st, o, c, blk


@pytest.mark.parametrize("name", ALL)
def test_fcn_and_jac_with_diffusion_bitwise(built_lib, name):
    geo, vel, st, o, c, blk = _setup(name)
    with blk:
        got = blk.Fcn(c)
        blk.Jac(c, 2.0)
        val = blk.jac_matrix()
    ref = o.fcn(c, vel)
    diff = np.argwhere(got != ref)
    assert diff.size == 0, f"{len(diff)} mismatches, first {diff[:3].tolist()}"
    np.testing.assert_array_equal(val, o.jac(c[0], vel, 1.0, 2.0))


@pytest.mark.parametrize("name", ["hill_24x20x16", "flat_walls_9x6x5", "bubble_12x10x8"])
@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_ros_step_with_diffusion(built_lib, name, precision):
    import asam_gb300 as asam

    kw = {"precision": precision, "inner_precond": "xline"} if precision == "fp32_refined" else {}
    geo, vel, st, o, c, blk = _setup(name, method="RosRK3", bicgstab_tol=1e-10, **kw)
    cr, cg = st.c.copy(), st.c.copy()
    tol = 1e-12 if precision == "fp64" else 1e-10
    with blk:
        for _ in range(2):
            it_r, _ = o.ros_step(cr, vel, 2.0, method=asam.METHODS["RosRK3"], tol=1e-10)
            it_g, _ = blk.Ros3MetC(cg, 2.0)
            if precision == "fp64":
                for a, b in zip(it_g, it_r):
                    assert abs(abs(a) - abs(b)) <= 1
            assert max(cases.field_relerr(cg, cr)) <= tol


def test_diffusion_off_again_and_adjoint_refused(built_lib):
    from asam_gb300._lib import ptr

    geo, vel, st, o, c, blk = _setup("hill_24x20x16")
    with blk:
        dc = np.zeros(geo.grid.pshape)
        out = np.zeros(geo.grid.pshape)
        cc = np.ascontiguousarray(c)
        assert blk.lib.asam_fcn_tlm(blk.h, ptr(cc), 8, ptr(dc), ptr(out)) == 4  # ASAM_BAD_ARG
        blk.set_diffusion(None)
        o.set_diffusion(None)
        np.testing.assert_array_equal(blk.Fcn(c), o.fcn(c, vel))
        assert blk.lib.asam_fcn_tlm(blk.h, ptr(cc), 8, ptr(dc), ptr(out)) == 0


def test_dyn_step_with_diffusion(built_lib):
    geo, vel, st, pos, (dx, dy, dz), bc = G.dyn_case(13, 9, 10, seed=7, moist=True, tracer=True)
    nc = st.c.shape[0]
    kinds = np.ones((nc, 6), np.int32)
    for q, p in enumerate(pos["mom"]):
        for sd in range(6):
            kinds[p, sd] = 2 if q // 2 == sd // 2 else 1
    o = oracle.Oracle(geo, bc=kinds)
    dh, dv = G.diffusion_coefficients(geo, st.c[0], seed=4)
    o.set_diffusion(dh, dv)
    pr = oracle.OracleProj(geo, dx, dy, dz, G.projection_inputs(geo)[0], zebra=1)
    sc = [pos["qv"], pos["tracer"]]
    cr, cg = st.c.copy(), st.c.copy()
    ur = [a.copy() for a in vel]
    with TransportBlock(geo, ncomp=nc, rho_pos=0, bicgstab_tol=1e-10) as blk:
        blk.set_velocity(*vel)
        blk.set_diffusion(dh, dv)
        blk.proj_setup(dx, dy, dz, tol=1e-10, max_restart=20)
        blk.dyn_setup(pos["th"], pos["mom"], rv_pos=pos["qv"], bound_cells=bc, scalars=sc)
        for step in range(2):
            o.ros_step_dyn(pr, cr, ur, 2.0, rho_pos=0, th_pos=pos["th"], pos=pos["mom"], dx=dx, dy=dy, dz=dz,
                           rv_pos=pos["qv"], bound=bc, scalars=sc, bicg_tol=1e-10, proj_tol=1e-10, proj_maxiter=20)
            blk.Ros3MetC_dyn(cg, 2.0)
            errs = cases.state_relerr(cg, cr, mom=pos["mom"])
            assert max(errs) <= 1e-12, (step, errs)
            vmax = max(float(np.max(np.abs(b))) for b in ur)
            for a, b in zip(blk.get_velocity(), ur):
                assert float(np.max(np.abs(a - b))) <= 1e-12 * vmax, step
