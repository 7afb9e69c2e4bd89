"""CPU checks of the projection oracle (oracle/asam_proj.c) -- no GPU needed.

* the level-0 pressure Laplacian of the oracle equals an independent numpy
  restatement of LaplTFullCompute/ComputeFull_1D/2D/3D
  (MULTI/JacAccGrav_Mod.f90:1056-1310, MULTI/TriDiagT_Mod.f90:62-90, 330-403,
  790-883) bit for bit;
* known answer: every face term of a row enters the diagonal with the
  opposite sign of its coupling and carries the DUT of the column it
  multiplies, so A (1/DUT) = (1e-40 + FacAnela*Vol)/DUT;
* a single column is solved exactly by one V-cycle (Thomas, Solve_1D);
* the V-cycle contracts the residual, and FGMRES reaches its tolerance with
  both the reference's lexicographic smoother and the zebra ordering, whose
  solutions agree to the Krylov tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from tests import cases, pyref

BETA0, DTP = 0.435866521508459, 2.0
PROJ = ["proj_hill_24x20x16", "proj_hill_odd_13x7x9", "proj_flat_16x12x10", "proj_column_1x1x12", "proj_slab_9x1x6"]


def _make(name, zebra=1, **kw):
    geo = cases.get(name)
    W, dx, dy, dz, vel = cases.proj_inputs(geo)
    o = oracle.OracleProj(geo, dx, dy, dz, W, zebra=zebra, **kw)
    o.lapl_compute(BETA0, DTP)
    return geo, W, dx, dy, dz, vel, o


def _level0_numpy(geo, W, dx, dy, dz):
    return pyref.lapl_level0(geo, W, dx, dy, dz, BETA0, DTP)


@pytest.mark.parametrize("name", PROJ)
def test_level0_assembly_matches_numpy(name):
    geo, W, dx, dy, dz, _, o = _make(name)
    ref = _level0_numpy(geo, W, dx, dy, dz)
    for which in range(7):
        got = o.lapl_get(0, 0, which)
        np.testing.assert_array_equal(got, ref[which], err_msg=f"array {which}")


@pytest.mark.parametrize("name", ["proj_hill_24x20x16", "proj_flat_16x12x10"])
def test_row_sums_known_answer(name):
    geo, W, *_, o = _make(name)
    dut = W[6]
    vol = geo.volc[1:-1, 1:-1, 1:-1]
    eps = 1.0e-30
    dutc = (dut * vol) / (vol + eps)  # the level-0 DUT (CVolCoarse with shift 0)
    live = vol > 0
    x = np.where(live, 1.0 / np.where(live, dutc, 1.0), 0.0)
    y = o.matvec(x)
    expect = (1.0e-40 + vol) * x
    scale = np.max(np.abs(o.matvec(np.ones_like(x))))
    assert np.max(np.abs(y - expect)[live]) <= 1e-11 * scale


def test_column_is_solved_exactly():
    geo, W, *_, o = _make("proj_column_1x1x12")
    b = np.random.default_rng(5).standard_normal((geo.grid.nz, 1, 1))
    x = o.vcycle(b)
    r = b - o.matvec(x)
    assert np.max(np.abs(r)) <= 1e-13 * np.max(np.abs(b))


@pytest.mark.parametrize("name", PROJ)
@pytest.mark.parametrize("zebra", [0, 1])
def test_vcycle_contracts_and_fgmres_converges(name, zebra):
    geo, W, dx, dy, dz, (u, v, w), o = _make(name, zebra=zebra)
    g = geo.grid
    b = np.random.default_rng(7).standard_normal((g.nz, g.ny, g.nx))
    x = o.vcycle(b)
    red = np.linalg.norm(b - o.matvec(x)) / np.linalg.norm(b)
    assert red < 0.05
    rhs = o.rhs(u, v, w)
    xs = np.zeros_like(rhs)
    steps, rho, rho0 = o.fgmres(xs, rhs, maxiter=10, tol=1e-6)
    assert rho <= 1e-6 * rho0
    true = np.linalg.norm(rhs - o.matvec1(xs)) / np.linalg.norm(rhs)
    assert true <= 2e-6


@pytest.mark.parametrize("name", ["proj_hill_24x20x16", "proj_hill_odd_13x7x9", "proj_flat_16x12x10"])
def test_orderings_agree_to_krylov_tolerance(name):
    sols = []
    for zebra in (0, 1):
        geo, W, dx, dy, dz, (u, v, w), o = _make(name, zebra=zebra)
        rhs = o.rhs(u, v, w)
        xs = np.zeros_like(rhs)
        o.fgmres(xs, rhs, maxiter=20, tol=1e-12)
        sols.append(xs)
    live = cases.get(name).volc[1:-1, 1:-1, 1:-1] > 0
    assert np.max(np.abs(sols[0] - sols[1])[live]) <= 1e-9 * np.max(np.abs(sols[0])[live])


def _moist_state(geo, seed=31):
    g = geo.grid
    rng = np.random.default_rng(seed)
    rho = 1.0 + 0.1 * rng.random(g.pshape)
    rth = rho * (300.0 + 5.0 * rng.random(g.pshape))
    rv = 0.01 * rho * rng.random(g.pshape)
    rc = 0.001 * rho * rng.random(g.pshape)
    t = 290.0 + 10.0 * rng.random(g.pshape)
    return rth, rho, rv, rc, t


@pytest.mark.parametrize("name", ["proj_hill_odd_13x7x9", "proj_flat_16x12x10"])
def test_density_weights_formula(name):
    """WeightDiagCompute 'Density' (JacAccGrav_Mod.f90:4259-4282) and the
    interior/wall faces of CellToFaceRhoWeight, restated in numpy."""
    geo, W, dx, dy, dz, _, o = _make(name)
    g = geo.grid
    rth, rho, rv, rc, t = _moist_state(geo)
    dtu, dtv, dtw, duu, duv, duw, dut, dtt = o.weights_density(rth, rho, rv, rc, None, t)
    eps = 1.0e-30
    Rd, Rv, Cpd, Cpv, Cpl = 1004.0 - 717.0, 461.0, 1004.0, 1885.0, 4186.0
    I = (slice(1, -1),) * 3
    rvl, rll = rv[I], rc[I] + 0.0
    rd = rho[I] - rvl - rll + eps
    kap = (Rd + Rv * rvl / rd) / (Cpd + Cpv * rvl / rd + Cpl * rll / rd)
    np.testing.assert_array_equal(dut, t[I] / (rth[I] + eps) * (rd * Rd + rvl * Rv) / (1.0 - kap))
    np.testing.assert_array_equal(dtt, np.ones_like(dtt))
    th = rth / (rho + eps)
    V = geo.volc
    vt = V * rth / (rho + eps)
    ex = (vt[1:-1, 1:-1, 1:-2] + vt[1:-1, 1:-1, 2:-1]) / (V[1:-1, 1:-1, 1:-2] + V[1:-1, 1:-1, 2:-1] + eps)
    np.testing.assert_array_equal(dtu[:, :, 1:-1], ex)
    np.testing.assert_array_equal(dtu[:, :, 0], th[1:-1, 1:-1, 1])
    np.testing.assert_array_equal(dtu[:, :, -1], th[1:-1, 1:-1, -2])
    ez = (vt[1:-2, 1:-1, 1:-1] + vt[2:-1, 1:-1, 1:-1]) / (V[1:-2, 1:-1, 1:-1] + V[2:-1, 1:-1, 1:-1] + eps)
    np.testing.assert_array_equal(dtw[1:-1], ez)
    fu = geo.fu[:, :, 1:g.nx + 2]
    np.testing.assert_array_equal(duu, fu / (fu + eps))
