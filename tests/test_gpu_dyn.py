"""GPU parity of the dynamical-core stage and of the outer-wall halo rule
against the oracle (oracle/asam_dyn.c, oracle/asam_oracle.c).

Bit-exact: the wall halos (BoundaryCondition), VelocityFaceToCellLR with the
boundary-cell shift, VelocityCellToFaceLR, and FcnMet with the pressure
gradient and the buoyancy (same pressure input).  AbsTCompute evaluates pow(),
whose last bits differ between CUDA and the C library: temperature and
pressure agree to 4e-15 relative.  The whole Rosenbrock step of the
dynamical core runs two Krylov solves per stage whose dot products are
reduced in a different order: with both solves at tolerance 1e-10 the
states and velocities agree to 1e-12 relative per field after every step,
BiCGStab iteration counts within one.  Blocks periodic in x and y carry the
projection's boundary face unknowns.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from asam_gb300 import AsamError, TransportBlock
from asam_gb300 import geometry as G
from tests import cases

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-12     # FP64 dynamical step against the oracle, per field, after each step
REFINED_TOL = 1e-10  # the FP32-refined step against the FP64 oracle


def _kinds(ncomp, mom, no_slip=False):
    k = np.ones((ncomp, 6), np.int32)
    for q, p in enumerate(mom):
        for sd in range(6):
            k[p, sd] = 2 if (no_slip or q // 2 == sd // 2) else 1
    return k


DYN = {
    "dyn_hill_13x9x10": lambda: G.dyn_case(13, 9, 10, seed=7, moist=True, tracer=True),
    "dyn_hill_24x20x16": lambda: G.dyn_case(24, 20, 16, seed=5),
    "dyn_flat_10x8x7": lambda: G.dyn_case(10, 8, 7, hill=False),
    "dyn_per_hill_12x10x8": lambda: G.dyn_case(12, 10, 8, seed=9, moist=True, tracer=True, periodic=True),
    "dyn_per_flat_10x8x7": lambda: G.dyn_case(10, 8, 7, hill=False, periodic=True),
    "bubble_16x16x16": lambda: G.bubble_dyn_case(16, 16, 16),
}
_cache = {}


def _case(name):
    if name not in _cache:
        _cache[name] = DYN[name]()
    return _cache[name]


def _block(name, free_slip=True, no_slip=False, proj_tol=1e-6, proj_restarts=10, **kw):
    geo, vel, st, pos, (dx, dy, dz), bc = _case(name)
    blk = TransportBlock(geo, ncomp=st.c.shape[0], rho_pos=0, **kw)
    blk.set_velocity(*vel)
    blk.proj_setup(dx, dy, dz, tol=proj_tol, max_restart=proj_restarts)
    sc = [pos[k] for k in ("qv", "tracer") if k in pos]
    blk.dyn_setup(pos["th"], pos["mom"], rv_pos=pos.get("qv", -1), free_slip=free_slip, wall_no_slip=no_slip,
                  bound_cells=bc, scalars=sc)
    return blk


def test_bound_cond_bitwise(built_lib):
    geo, vel, st = cases.get("flat_walls_9x6x5")
    rng = np.random.default_rng(2)
    nc = st.c.shape[0]
    kinds = rng.integers(0, 3, size=(nc, 6)).astype(np.int32)
    c = rng.standard_normal(st.c.shape)
    with TransportBlock(geo, ncomp=nc, rho_pos=0) as blk:
        np.testing.assert_array_equal(blk.BoundaryCondition(c), oracle.Oracle(geo).bound_cond(c))  # default ZeroGrad
        blk.set_boundary(kinds)
        np.testing.assert_array_equal(blk.BoundaryCondition(c), oracle.Oracle(geo, bc=kinds).bound_cond(c))
        with pytest.raises(AsamError):
            blk.set_boundary(np.full((nc, 6), 3, np.int32))


@pytest.mark.parametrize("name", ["flat_walls_9x6x5", "hill_24x20x16"])
def test_ros_step_wall_rules(built_lib, name):
    """Transport step with mixed wall rules on the closed sides."""
    import asam_gb300 as asam

    geo, vel, st = cases.get(name)
    nc = st.c.shape[0]
    kinds = np.ones((nc, 6), np.int32)
    kinds[1::2] = 2  # ZeroValue for every other component
    kinds[nc - 1, 4] = 0  # leave one halo alone
    o = oracle.Oracle(geo, bc=kinds)
    cr, cg = st.c.copy(), st.c.copy()
    with TransportBlock(geo, ncomp=nc, rho_pos=0, method="RosRK3", bicgstab_tol=1e-10) as blk:
        blk.set_velocity(*vel)
        blk.set_boundary(kinds)
        for _ in range(2):
            it_r, _ = o.ros_step(cr, vel, 2.0, method=asam.METHODS["RosRK3"], tol=1e-10)
            it_g, _ = blk.Ros3MetC(cg, 2.0)
            for a, b in zip(it_g, it_r):
                assert abs(abs(a) - abs(b)) <= 1
            assert max(cases.field_relerr(cg, cr)) <= 1e-12


@pytest.mark.parametrize("name", list(DYN))
@pytest.mark.parametrize("free_slip", [True, False])
def test_face_cell_bitwise(built_lib, name, free_slip):
    geo, vel, st, pos, _, bc = _case(name)
    nc = st.c.shape[0]
    o = oracle.Oracle(geo, bc=_kinds(nc, pos["mom"]))
    rng = np.random.default_rng(4)
    c0 = rng.standard_normal(st.c.shape)
    ref = o.face_to_cell(pos["mom"], vel, c0, bc, free_slip=free_slip)
    with _block(name, free_slip=free_slip) as blk:
        got = blk.VelocityFaceToCellLR(*vel, c0)
        np.testing.assert_array_equal(got, ref)
        for a, b in zip(blk.VelocityCellToFaceLR(c0), o.cell_to_face(pos["mom"], c0)):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("name", list(DYN))
def test_thermo_and_fcn(built_lib, name):
    geo, vel, st, pos, (dx, dy, dz), bc = _case(name)
    o = oracle.Oracle(geo)
    c = st.c
    tr, pr = o.thermo(c, 0, pos["th"], rv_pos=pos.get("qv", -1))
    fr = o.fcn_dyn(c, vel, pr, pos["mom"], dx, dy, dz)
    with _block(name) as blk:
        tg, pg = blk.AbsTPreCompute(c)
        np.testing.assert_allclose(tg, tr, rtol=4e-15, atol=0)
        np.testing.assert_allclose(pg, pr, rtol=4e-15, atol=0)
        fg = blk.FcnMet(c, pr)
    diff = np.argwhere(fg != fr)
    assert diff.size == 0, f"{len(diff)} mismatches, first {diff[:3].tolist()}"


@pytest.mark.parametrize("name", ["dyn_hill_13x9x10", "dyn_hill_24x20x16", "dyn_flat_10x8x7", "dyn_per_hill_12x10x8",
                                  "dyn_per_flat_10x8x7", "bubble_16x16x16"])
def test_ros_step_dyn_matches_oracle(built_lib, name):
    geo, vel, st, pos, (dx, dy, dz), bc = _case(name)
    nc = st.c.shape[0]
    o = oracle.Oracle(geo, bc=_kinds(nc, pos["mom"]))
    W = G.projection_inputs(geo)[0]
    pr = oracle.OracleProj(geo, dx, dy, dz, W, zebra=1)
    sc = [pos[k] for k in ("qv", "tracer") if k in pos]
    cr, cg = st.c.copy(), st.c.copy()
    ur = [a.copy() for a in vel]
    V = geo.volc[1:-1, 1:-1, 1:-1]
    m0 = float(np.sum(cg[0][1:-1, 1:-1, 1:-1] * V))
    # the projection solved to 1e-10: one FGMRES step more or less moves the
    # solution far below the tolerance of the comparison
    with _block(name, bicgstab_tol=1e-10, proj_tol=1e-10, proj_restarts=20) as blk:
        for step in range(2):
            it_r, _, ps_r, pres_r = o.ros_step_dyn(pr, cr, ur, 2.0, rho_pos=0, th_pos=pos["th"], pos=pos["mom"],
                                                   dx=dx, dy=dy, dz=dz, rv_pos=pos.get("qv", -1), bound=bc,
                                                   scalars=sc, bicg_tol=1e-10, proj_tol=1e-10, proj_maxiter=20)
            (it_g, _), (ps_g, pres_g) = blk.Ros3MetC_dyn(cg, 2.0)
            for a, b in zip(it_g, it_r):
                assert abs(abs(a) - abs(b)) <= 1, (step, it_g, it_r)
            assert all(r <= 1e-10 for r in pres_g), pres_g
            errs = cases.field_relerr(cg, cr)
            assert max(errs) <= STEP_TOL, (step, errs)
            for a, b in zip(blk.get_velocity(), ur):
                assert cases.relerr(a, b) <= STEP_TOL
    m1 = float(np.sum(cg[0][1:-1, 1:-1, 1:-1] * V))
    assert abs(m1 - m0) <= 1e-13 * m0


@pytest.mark.parametrize("name", ["dyn_hill_13x9x10", "dyn_per_hill_12x10x8", "dyn_per_flat_10x8x7"])
def test_ros_step_dyn_refined(built_lib, name):
    """The dynamical step with the FP32-refined transport solve and the FP32
    multigrid (on periodic blocks: the periodic-Laplacian preconditioner)
    stays within the step tolerance of the FP64 oracle.  Both projections are
    solved to 1e-12, so the two preconditioners' iterates agree far below it."""
    geo, vel, st, pos, (dx, dy, dz), bc = _case(name)
    nc = st.c.shape[0]
    o = oracle.Oracle(geo, bc=_kinds(nc, pos["mom"]))
    pr = oracle.OracleProj(geo, dx, dy, dz, G.projection_inputs(geo)[0], zebra=1)
    sc = [pos[k] for k in ("qv", "tracer") if k in pos]
    cr, cg = st.c.copy(), st.c.copy()
    ur = [a.copy() for a in vel]
    with _block(name, bicgstab_tol=1e-10, proj_tol=1e-12, proj_restarts=40, precision="fp32_refined",
                inner_precond="xline") as blk:
        for step in range(2):
            o.ros_step_dyn(pr, cr, ur, 2.0, rho_pos=0, th_pos=pos["th"], pos=pos["mom"], dx=dx, dy=dy, dz=dz,
                           rv_pos=pos.get("qv", -1), bound=bc, scalars=sc, bicg_tol=1e-10, proj_tol=1e-12,
                           proj_maxiter=40)
            blk.Ros3MetC_dyn(cg, 2.0)
            assert max(cases.field_relerr(cg, cr)) <= REFINED_TOL, step
            for a, b in zip(blk.get_velocity(), ur):
                assert cases.relerr(a, b) <= REFINED_TOL


def test_dyn_bad_calls(built_lib):
    geo, vel, st, pos, (dx, dy, dz), bc = _case("dyn_flat_10x8x7")
    with TransportBlock(geo, ncomp=st.c.shape[0], rho_pos=0) as blk:
        with pytest.raises(AsamError):
            blk.dyn_setup(pos["th"], pos["mom"])  # no projection yet
        blk.proj_setup(dx, dy, dz)
        with pytest.raises(AsamError):
            blk.dyn_setup(pos["th"], [1, 1, 3, 4, 5, 6])  # duplicate position
        with pytest.raises(AsamError):
            blk.dyn_setup(pos["th"], pos["mom"], bound_cells=[[0, 1, 1]])  # outside the interior
        with pytest.raises(AsamError):
            blk.Ros3MetC_dyn(st.c.copy(), 1.0)  # not set up
