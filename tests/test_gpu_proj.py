"""GPU parity of the pressure projection against the oracle (oracle/asam_proj.c).

Bit-exact: every array of the assembled Laplacian hierarchy (all 3D levels and
their plane levels), the operator MatVecP_Tri and one multigrid V-cycle in the
zebra ordering.  Within the Krylov tolerance (the dot products are reduced in
a different order): FGMRES and the whole ProjectVelFace.  The reference's
lexicographic ordering (oracle) and the GPU's zebra ordering agree to the
Krylov tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from asam_gb300 import AsamError, TransportBlock
from asam_gb300 import geometry as G
from tests import cases

pytestmark = pytest.mark.gpu

BETA0, DTP = 0.435866521508459, 2.0
PROJ = ["proj_hill_24x20x16", "proj_hill_odd_13x7x9", "proj_flat_16x12x10", "proj_column_1x1x12", "proj_slab_9x1x6"]
REF_LEVEL = 4


def _pair(name, zebra=1, ref_level=REF_LEVEL, **proj):
    geo = cases.get(name)
    W, dx, dy, dz, vel = cases.proj_inputs(geo)
    blk = TransportBlock(geo, ncomp=3, rho_pos=0)
    blk.proj_setup(dx, dy, dz, ref_level=ref_level, **proj)
    blk.proj_weights(*W)
    blk.JacAccGrav(BETA0, DTP)
    o = oracle.OracleProj(geo, dx, dy, dz, W, zebra=zebra, ref_level=ref_level)
    o.lapl_compute(BETA0, DTP)
    return geo, W, vel, blk, o


@pytest.mark.parametrize("name", PROJ)
def test_hierarchy_bitwise(name):
    geo, W, vel, blk, o = _pair(name)
    with blk:
        for L3 in range(REF_LEVEL):
            for L2 in range(L3, REF_LEVEL):
                for which in range(7 if L2 == L3 else 5):
                    np.testing.assert_array_equal(blk.lapl_array(L3, L2, which), o.lapl_get(L3, L2, which),
                                                  err_msg=f"level {L3}/{L2} array {which}")


@pytest.mark.parametrize("name", PROJ)
def test_matvec_and_vcycle_bitwise(name):
    geo, W, vel, blk, o = _pair(name)
    g = geo.grid
    rng = np.random.default_rng(11)
    with blk:
        for _ in range(2):
            x = rng.standard_normal((g.nz, g.ny, g.nx))
            np.testing.assert_array_equal(blk.MatVecP(x), o.matvec(x))
            b = rng.standard_normal((g.nz, g.ny, g.nx))
            np.testing.assert_array_equal(blk.VCycleCG(b), o.vcycle(b))


@pytest.mark.parametrize("name", PROJ)
def test_solve_sound_matches_oracle(name):
    geo, W, (u, v, w), blk, o = _pair(name)
    with blk:
        b = o.rhs(u, v, w)
        x_ref = np.zeros_like(b)
        steps_ref, rho, rho0 = o.fgmres(x_ref, b, maxiter=10, tol=1e-6, step=10)
        x = np.zeros_like(b)
        steps, rel = blk.SolveSound(x, b, MaxIter=10, Tol=1e-6)
        assert abs(steps - steps_ref) <= 1
        assert rel <= 1e-6
        if steps != steps_ref:  # compare against the oracle run with the GPU's step count
            x_ref = _oracle_steps(o, b, steps)
        scale = max(np.max(np.abs(x_ref)), 1e-300)
        # same Krylov subspace: the iterates differ by the rounding of the dots
        assert np.max(np.abs(x - x_ref)) <= 1e-9 * scale


def _oracle_steps(o, b, steps, step=10):
    """The oracle's FGMRES with exactly `steps` inner steps (restart cycles of
    `step`): tolerance 0 for the full cycles, then a last cycle of the rest."""
    x = np.zeros_like(b)
    full, rest = divmod(steps, step)
    if full:
        o.fgmres(x, b, maxiter=full, tol=0.0, step=step)
    if rest:
        o.fgmres(x, b, maxiter=1, tol=0.0, step=rest)
    return x


def _state(geo, ncomp, seed):
    g = geo.grid
    rng = np.random.default_rng(seed)
    st = np.empty((ncomp,) + g.pshape)
    st[0] = 1.0 + 0.1 * rng.random(g.pshape)
    st[1] = st[0] * (300.0 + rng.random(g.pshape))
    st[2] = st[0] * rng.random(g.pshape)
    return st


@pytest.mark.parametrize("name", ["proj_hill_24x20x16", "proj_hill_odd_13x7x9", "proj_flat_16x12x10", "proj_slab_9x1x6"])
def test_project_vel_face_matches_oracle(name):
    geo, W, (u, v, w), blk, o = _pair(name)
    g = geo.grid
    rng = np.random.default_rng(13)
    state = _state(geo, 3, 17)
    incr = rng.standard_normal((3,) + g.pshape)
    with blk:
        u1, v1, w1, incr1 = u.copy(), v.copy(), w.copy(), incr.copy()
        p, steps, rel = blk.ProjectVelFace(u1, v1, w1, incr1, state, th_pos=1, rho_pos=0, scalars=[2])
        u2, v2, w2, incr2 = u.copy(), v.copy(), w.copy(), incr.copy()
        b = o.rhs(u2, v2, w2, incr_th=incr2[1])
        x = np.zeros_like(b)
        o.fgmres(x, b, maxiter=10, tol=1e-6, step=10)
        o.update(x, u2, v2, w2, incr_th=incr2[1], incr_rho=incr2[0], incr_c=[incr2[2]], c=[state[2]], rho=state[0])
        assert rel <= 1e-6
        for got, ref in ((u1, u2), (v1, v2), (w1, w2), (incr1, incr2), (p, x)):
            scale = max(np.max(np.abs(ref)), 1e-300)
            assert np.max(np.abs(got - ref)) <= 1e-8 * scale


@pytest.mark.parametrize("name", ["proj_hill_24x20x16", "proj_flat_16x12x10"])
def test_zebra_vs_reference_ordering(name):
    geo, W, (u, v, w), blk, o = _pair(name, zebra=0)
    with blk:
        b = o.rhs(u, v, w)
        x_ref = np.zeros_like(b)
        o.fgmres(x_ref, b, maxiter=20, tol=1e-12, step=10)
        x = np.zeros_like(b)
        blk.SolveSound(x, b, MaxIter=20, Tol=1e-12)
        live = geo.volc[1:-1, 1:-1, 1:-1] > 0
        assert np.max(np.abs(x - x_ref)[live]) <= 1e-9 * np.max(np.abs(x_ref)[live])


def test_larger_block_converges():
    geo = cases._hill_closed(96, 80, 48, seed=9)
    W, dx, dy, dz, (u, v, w) = cases.proj_inputs(geo, seed=21)
    g = geo.grid
    with TransportBlock(geo, ncomp=3, rho_pos=0) as blk:
        blk.proj_setup(dx, dy, dz)
        blk.proj_weights(*W)
        blk.JacAccGrav(BETA0, DTP)
        rng = np.random.default_rng(3)
        b = rng.standard_normal((g.nz, g.ny, g.nx))
        x = blk.VCycleCG(b)
        assert np.linalg.norm(b - blk.MatVecP(x)) / np.linalg.norm(b) < 0.05
        x = np.zeros_like(b)
        steps, rel = blk.SolveSound(x, b)
        assert rel <= 1e-6 and steps <= 60
        true = np.linalg.norm(b + blk.MatVecP(x)) / np.linalg.norm(b)  # MatVec1 = -A
        assert true <= 2e-6


def test_bad_calls_raise():
    geo = cases.get("proj_flat_16x12x10")
    W, dx, dy, dz, _ = cases.proj_inputs(geo)
    with TransportBlock(geo, ncomp=3, rho_pos=0) as blk:
        with pytest.raises(AsamError):
            blk.JacAccGrav(BETA0, DTP)  # no set-up
        blk.proj_setup(dx, dy, dz)
        with pytest.raises(AsamError):
            blk.JacAccGrav(BETA0, DTP)  # no weights
        with pytest.raises(AsamError):
            blk.proj_setup(dx, dy, dz, ref_level=0)
    per = cases.get("bubble_12x10x8")[0]
    with TransportBlock(per, ncomp=3, rho_pos=0) as blk:
        g = per.grid
        blk.proj_setup(np.full(g.nx, g.dx), np.full(g.ny, g.dy), g.dz)  # periodic x/y: face unknowns
        assert blk.proj_nface == 2 * g.ny * g.nz + 2 * g.nx * g.nz
        with pytest.raises(ValueError):
            blk.lapl_array_dirichlet(0, 0, 0)  # not assembled yet
        with pytest.raises(AsamError):
            blk.proj_set_pre_schedule(-1, 0)
        with pytest.raises(KeyError):
            blk.proj_set_preconditioner("jacobi")
        blk.proj_set_pre_schedule(1, 1)  # the reference's growth, accepted
        with pytest.raises(AsamError):
            blk.proj_setup(np.full(g.nx, g.dx), np.full(g.ny, g.dy), g.dz, prefac2=-1.0)
    # the dynamical core refuses a block periodic in z (the buoyancy's
    # neighbour terms across a vertical periodic side are not built)
    grid = G.Grid(6, 5, 4, 100.0, 100.0, G.uniform_levels(4, 100.0), True, True, True)
    zper = G.cut_cell_geometry(grid, None, snap=0.0, merge=0.0)
    with TransportBlock(zper, ncomp=8, rho_pos=0) as blk:
        blk.proj_setup(np.full(6, 100.0), np.full(5, 100.0), np.full(4, 100.0))
        with pytest.raises(AsamError):
            blk.dyn_setup(7, [1, 2, 3, 4, 5, 6])


@pytest.mark.parametrize("name", ["proj_hill_24x20x16", "proj_hill_odd_13x7x9"])
def test_density_weights_and_hierarchy_bitwise(name):
    geo = cases.get(name)
    g = geo.grid
    W, dx, dy, dz, _ = cases.proj_inputs(geo)
    rng = np.random.default_rng(31)
    rho = 1.0 + 0.1 * rng.random(g.pshape)
    rth = rho * (300.0 + 5.0 * rng.random(g.pshape))
    rv = 0.01 * rho * rng.random(g.pshape)
    rc = 0.001 * rho * rng.random(g.pshape)
    t = 290.0 + 10.0 * rng.random(g.pshape)
    state = np.ascontiguousarray(np.stack([rho, rth, rv, rc]))
    o = oracle.OracleProj(geo, dx, dy, dz, W, zebra=1)
    ref = o.weights_density(rth, rho, rv, rc, None, t)
    o.lapl_compute(BETA0, DTP)
    with TransportBlock(geo, ncomp=4, rho_pos=0) as blk:
        blk.proj_setup(dx, dy, dz)
        blk.WeightDiagCompute(state, t, th_pos=1, rho_pos=0, rv_pos=2, rc_pos=3)
        for which in range(8):
            np.testing.assert_array_equal(blk.proj_weight(which), ref[which].ravel(), err_msg=f"weight {which}")
        blk.JacAccGrav(BETA0, DTP)
        for L3 in range(REF_LEVEL):
            for L2 in range(L3, REF_LEVEL):
                for which in range(7 if L2 == L3 else 5):
                    np.testing.assert_array_equal(blk.lapl_array(L3, L2, which), o.lapl_get(L3, L2, which))


@pytest.mark.parametrize("name", ["proj_hill_24x20x16", "proj_hill_odd_13x7x9", "proj_column_1x1x12"])
def test_fp32_multigrid_preconditioner(name):
    """The FP32 copy of the hierarchy: one V-cycle agrees with the FP64 one to
    FP32 accuracy, and FGMRES preconditioned by it reaches the same tolerance
    (the FP64 Arnoldi relation is unchanged) and the oracle's solution."""
    geo, W, (u, v, w), blk, o = _pair(name)
    g = geo.grid
    rng = np.random.default_rng(17)
    live = geo.volc[1:-1, 1:-1, 1:-1] > 0
    with blk:
        # cells without volume have a zero right-hand side in the projection
        b = rng.standard_normal((g.nz, g.ny, g.nx)) * live
        x64 = blk.VCycleCG(b)
        blk.proj_set_precision("fp32")
        x32 = blk.VCycleCG(b)
        assert np.all(np.isfinite(x32))
        assert np.max(np.abs(x32 - x64)[live]) <= 1e-5 * np.max(np.abs(x64)[live])
        rhs = o.rhs(u, v, w)
        xr = np.zeros_like(rhs)
        o.fgmres(xr, rhs, maxiter=20, tol=1e-10, step=10)
        x = np.zeros_like(rhs)
        steps, rel = blk.SolveSound(x, rhs, MaxIter=20, Tol=1e-10)
        assert rel <= 1e-10
        assert np.max(np.abs(x - xr)) <= 1e-8 * max(np.max(np.abs(xr)), 1e-300)
        blk.proj_set_precision("fp64")
        np.testing.assert_array_equal(blk.VCycleCG(b), x64)


# ---------------------------------------------------------------------------
# Blocks with periodic sides: boundary face unknowns, LaplDirichlet, SchurPreFull
# ---------------------------------------------------------------------------
PROJ_PER = list(cases.PROJ_PERIODIC)


@pytest.mark.parametrize("name", PROJ_PER)
def test_periodic_hierarchies_bitwise(name):
    """LaplNeumann and LaplDirichlet (SetFactorD) of a periodic block, every
    array of every level, bit for bit."""
    geo, W, vel, blk, o = _pair(name)
    with blk:
        assert blk.proj_nface == o.nface > 0
        for L3 in range(REF_LEVEL):
            for L2 in range(L3, REF_LEVEL):
                for which in range(7 if L2 == L3 else 5):
                    np.testing.assert_array_equal(blk.lapl_array(L3, L2, which), o.lapl_get(L3, L2, which),
                                                  err_msg=f"N level {L3}/{L2} array {which}")
                    np.testing.assert_array_equal(blk.lapl_array_dirichlet(L3, L2, which),
                                                  o.lapl_get(L3, L2, which, dirichlet=True),
                                                  err_msg=f"D level {L3}/{L2} array {which}")


@pytest.mark.parametrize("name", PROJ_PER)
def test_periodic_operators_bitwise(name):
    """MatVecFull with the face equations, the Dirichlet V-cycle and the whole
    PSolve1 (PressurePre, b2pBx1Full, Exchange, SchurPreFull, Exchange,
    b1pBTx2Full, PressurePre) equal the oracle bit for bit."""
    geo, W, vel, blk, o = _pair(name)
    g = geo.grid
    rng = np.random.default_rng(12)
    with blk:
        for _ in range(2):
            x = rng.standard_normal(o.nvec)
            np.testing.assert_array_equal(blk.MatVec1(x), o.matvec1(x))
            np.testing.assert_array_equal(blk.PSolve1(x), o.psolve1(x))
            b = rng.standard_normal((g.nz, g.ny, g.nx))
            np.testing.assert_array_equal(blk.VCycleCG_dirichlet(b), o.vcycle_dirichlet(b))
            np.testing.assert_array_equal(blk.VCycleCG(b), o.vcycle(b))


@pytest.mark.parametrize("name", PROJ_PER)
def test_periodic_solve_sound_matches_oracle(name):
    """FGMRES on the PressureVelocity system: inner steps equal or within one
    at tolerance 1e-10, and the same number of steps gives the same iterate
    up to the rounding of the dot products."""
    geo, W, (u, v, w), blk, o = _pair(name)
    with blk:
        b = o.rhs(u, v, w)
        x_ref = np.zeros_like(b)
        steps_ref, rho, rho0 = o.fgmres(x_ref, b, maxiter=20, tol=1e-10, step=10)
        x = np.zeros_like(b)
        steps, rel = blk.SolveSound(x, b, MaxIter=20, Tol=1e-10)
        assert abs(steps - steps_ref) <= 1, (steps, steps_ref)
        assert rel <= 1e-10
        if steps != steps_ref:
            x_ref = _oracle_steps(o, b, steps)
        assert np.max(np.abs(x - x_ref)) <= 1e-9 * np.max(np.abs(x_ref))
        nc = geo.grid.nx * geo.grid.ny * geo.grid.nz
        m = (o.nvec - nc) // 2  # both copies of each shared face hold one value
        if geo.grid.periodic_x:
            k = geo.grid.ny * geo.grid.nz
            np.testing.assert_array_equal(x[nc:nc + k], x[nc + k:nc + 2 * k])
        assert m > 0


@pytest.mark.parametrize("name", PROJ_PER)
def test_periodic_project_vel_face_matches_oracle(name):
    """ProjectVelFace of a periodic block: the boundary faces take the face
    unknowns (UpdateVelocity), both copies of a shared face stay equal."""
    geo, W, (u, v, w), blk, o = _pair(name, tol=1e-10, max_restart=20)
    g = geo.grid
    rng = np.random.default_rng(13)
    state = _state(geo, 3, 17)
    incr = rng.standard_normal((3,) + g.pshape)
    with blk:
        u1, v1, w1, incr1 = u.copy(), v.copy(), w.copy(), incr.copy()
        p, steps, rel = blk.ProjectVelFace(u1, v1, w1, incr1, state, th_pos=1, rho_pos=0, scalars=[2])
        u2, v2, w2, incr2 = u.copy(), v.copy(), w.copy(), incr.copy()
        b = o.rhs(u2, v2, w2, incr_th=incr2[1])
        x = np.zeros_like(b)
        steps_ref, _, _ = o.fgmres(x, b, maxiter=20, tol=1e-10, step=10)
        assert abs(steps - steps_ref) <= 1 and rel <= 1e-10
        o.update(x, u2, v2, w2, incr_th=incr2[1], incr_rho=incr2[0], incr_c=[incr2[2]], c=[state[2]], rho=state[0])
        for got, ref in ((u1, u2), (v1, v2), (w1, w2), (incr1, incr2), (p.ravel(), x[:g.nx * g.ny * g.nz])):
            scale = max(np.max(np.abs(ref)), 1e-300)
            assert np.max(np.abs(got - ref)) <= 1e-8 * scale
        if g.periodic_x:
            np.testing.assert_array_equal(u1[:, :, 0], u1[:, :, -1])
        if g.periodic_y:
            np.testing.assert_array_equal(v1[:, 0, :], v1[:, -1, :])


@pytest.mark.parametrize("name", PROJ_PER)
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_periodic_laplacian_preconditioner(name, prec):
    """The refined mode's preconditioner of a periodic block (no reference
    counterpart): the face unknowns are eliminated exactly, so the face rows
    of Exchange(MatVec1(pre(v))) reproduce v's face rows; the pressure rows
    keep the residual of one V-cycle on the periodic Laplacian, which
    contracts; FGMRES with it reaches the oracle's solution."""
    geo, W, (u, v, w), blk, o = _pair(name)
    g = geo.grid
    nc = g.nx * g.ny * g.nz
    rng = np.random.default_rng(21)
    with blk:
        blk.proj_set_precision(prec)
        blk.proj_set_preconditioner("periodic")
        blk.JacAccGrav(BETA0, DTP)
        for _ in range(2):
            # a vector of the operator's range after Exchange, as FGMRES's
            # Krylov vectors are (zero on the rows of closed faces)
            x = o.matvec1(rng.standard_normal(o.nvec))
            o.exchange(x)
            z = blk.PSolve1(x)
            r = o.matvec1(z)
            o.exchange(r)
            face_tol = 1e-12 if prec == "fp64" else 1e-6
            np.testing.assert_allclose(r[nc:], x[nc:], rtol=0, atol=face_tol * np.max(np.abs(x[nc:])))
            assert np.linalg.norm(r[:nc] - x[:nc]) <= 0.5 * np.linalg.norm(x[:nc])
        b = o.rhs(u, v, w)
        x_ref = np.zeros_like(b)
        o.fgmres(x_ref, b, maxiter=40, tol=1e-12, step=10)
        x = np.zeros_like(b)
        steps, rel = blk.SolveSound(x, b, MaxIter=40, Tol=1e-12)
        assert rel <= 1e-12, (steps, rel)
        assert np.max(np.abs(x - x_ref)) <= 1e-9 * np.max(np.abs(x_ref))
        blk.proj_set_preconditioner("psolve1")
        blk.JacAccGrav(BETA0, DTP)
        if prec == "fp64":  # back to PSolve1: the Dirichlet hierarchy is assembled again
            np.testing.assert_array_equal(blk.PSolve1(x), o.psolve1(x))
