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


# ---------------------------------------------------------------------------
# Blocks with periodic sides: boundary face unknowns, LaplDirichlet, the full
# PSolve1 (SchurPreFull) and Exchange
# ---------------------------------------------------------------------------
PROJ_PER = list(cases.PROJ_PERIODIC)


def _facs(geo):
    g = geo.grid
    return (2.0 if g.periodic_z else 0.0, 2.0 if g.periodic_x else 0.0, 2.0 if g.periodic_y else 0.0)


@pytest.mark.parametrize("name", PROJ_PER)
def test_dirichlet_level0_matches_numpy(name):
    """LaplDirichlet (SetFactorD: Fac=2 on the periodic sides) against the
    numpy restatement with those factors, bit for bit; LaplNeumann unchanged."""
    geo, W, dx, dy, dz, _, o = _make(name)
    refd = pyref.lapl_level0(geo, W, dx, dy, dz, BETA0, DTP, facs=_facs(geo))
    refn = _level0_numpy(geo, W, dx, dy, dz)
    for which in range(7):
        np.testing.assert_array_equal(o.lapl_get(0, 0, which, dirichlet=True), refd[which], err_msg=f"D {which}")
        np.testing.assert_array_equal(o.lapl_get(0, 0, which), refn[which], err_msg=f"N {which}")


def _periodic_laplacian(geo, W, dx, dy, dz):
    """The pressure operator of a periodic block with the shared boundary face
    treated as an interior face (the interior-face terms of ComputeFull_1D/2D/3D
    across the wrap), as a scipy matrix on the natural (x fastest) cell order:
    eliminating the face unknowns of the PressureVelocity system gives it."""
    import scipy.sparse as sp

    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    eps = 1.0e-30
    d, uz, lz, ux, lx, u3, l3 = (a.reshape(ny, nx, nz) for a in pyref.lapl_level0(geo, W, dx, dy, dz, BETA0, DTP))
    idx = lambda i, j, k: i + nx * (j + ny * k)  # noqa: E731 (0-based)
    rows, cols, vals = [], [], []

    def add(r, c, v):
        rows.append(r)
        cols.append(c)
        vals.append(v)

    for j in range(ny):
        for i in range(nx):
            for k in range(nz):
                p = idx(i, j, k)
                add(p, p, d[j, i, k])
                if k < nz - 1:
                    add(p, idx(i, j, k + 1), uz[j, i, k])
                    add(idx(i, j, k + 1), p, lz[j, i, k])
                if i < nx - 1:
                    add(p, idx(i + 1, j, k), ux[j, i, k])
                    add(idx(i + 1, j, k), p, lx[j, i, k])
                if j < ny - 1:
                    add(p, idx(i, j + 1, k), u3[j, i, k])
                    add(idx(i, j + 1, k), p, l3[j, i, k])
    dtu, dtv, dtw, duu, duv, duw, dut, _ = W
    bd2 = (BETA0 * DTP) ** 2
    vol = geo.volc[1:-1, 1:-1, 1:-1]
    D = (dut * vol) / (vol + eps)
    if g.periodic_x:
        F = geo.fu[:, :, 1]
        T = (dtu[:, :, 0] * F) / (F + eps)
        U = (duu[:, :, 0] * F) / (F + eps)
        for k in range(nz):
            for j in range(ny):
                den = dx[0] + dx[-1]
                a, b = idx(0, j, k), idx(nx - 1, j, k)
                add(a, a, bd2 * 2.0 * F[k, j] * T[k, j] * U[k, j] * D[k, j, 0] / den)
                add(a, b, -(bd2 * 2.0 * F[k, j] * T[k, j] * U[k, j] * D[k, j, nx - 1] / den))
                add(b, b, bd2 * 2.0 * F[k, j] * T[k, j] * U[k, j] * D[k, j, nx - 1] / den)
                add(b, a, -(bd2 * 2.0 * F[k, j] * T[k, j] * U[k, j] * D[k, j, 0] / den))
    if g.periodic_y:
        F = geo.fv[:, 1, :]
        T = (dtv[:, 0, :] * F) / (F + eps)
        for k in range(nz):
            for i in range(nx):
                den = dy[0] + dy[-1]
                a, b = idx(i, 0, k), idx(i, ny - 1, k)
                # the y couplings of the 3D level carry no DUU3 (ComputeFull_3D)
                add(a, a, bd2 * 2.0 * F[k, i] * T[k, i] * D[k, 0, i] / den)
                add(a, b, -(bd2 * 2.0 * F[k, i] * T[k, i] * D[k, ny - 1, i] / den))
                add(b, b, bd2 * 2.0 * F[k, i] * T[k, i] * D[k, ny - 1, i] / den)
                add(b, a, -(bd2 * 2.0 * F[k, i] * T[k, i] * D[k, 0, i] / den))
    n = nx * ny * nz
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


@pytest.mark.parametrize("name", PROJ_PER)
def test_periodic_projection_known_answer(name):
    """Known answer: FGMRES on the PressureVelocity system (face unknowns,
    Exchange, DOT2, the full PSolve1) converges to the solution of the
    periodic pressure Laplacian in which the shared boundary face is an
    interior face; the face unknown equals the interior-face velocity formula
    and both copies of a shared face are identical."""
    import scipy.sparse.linalg as spla

    geo, W, dx, dy, dz, (u, v, w), o = _make(name)
    g = geo.grid
    nc = g.nx * g.ny * g.nz
    rhs = o.rhs(u, v, w)
    assert rhs.size == o.nvec and o.nface > 0 and np.all(rhs[nc:] == 0.0)
    x = np.zeros_like(rhs)
    steps, rho, rho0 = o.fgmres(x, rhs, maxiter=40, tol=1e-13)
    assert rho <= 1e-13 * rho0
    # the operator of the PressureVelocity system is -L_per after eliminating the faces
    L = _periodic_laplacian(geo, W, dx, dy, dz)
    vol = geo.volc[1:-1, 1:-1, 1:-1].ravel()
    live = vol > 0
    p_ref = np.zeros(nc)
    A = L[live][:, live]
    p_ref[live] = spla.spsolve(A.tocsc(), -rhs[:nc][live])
    err = np.max(np.abs(x[:nc] - p_ref)[live]) / np.max(np.abs(p_ref[live]))
    assert err <= 1e-8, err
    # both copies of a shared face hold the same unknown
    off = nc
    for per, m in ((g.periodic_x, g.ny * g.nz), (g.periodic_y, g.nx * g.nz), (g.periodic_z, g.nx * g.ny)):
        if per:
            np.testing.assert_array_equal(x[off:off + m], x[off + m:off + 2 * m])
            off += 2 * m


@pytest.mark.parametrize("name", PROJ_PER)
def test_periodic_preconditioner_and_orderings(name):
    """PSolve1 with the Schur step approximates the inverse (a few FGMRES
    steps per decade), and the reference's lexicographic smoother and the
    zebra ordering give the same solution to the Krylov tolerance."""
    sols = []
    for zebra in (0, 1):
        geo, W, dx, dy, dz, (u, v, w), o = _make(name, zebra=zebra)
        rhs = o.rhs(u, v, w)
        x = np.zeros_like(rhs)
        steps, rho, rho0 = o.fgmres(x, rhs, maxiter=10, tol=1e-6)
        assert rho <= 1e-6 * rho0 and steps <= 30
        true = np.sqrt(o.dot2(*(2 * [_resid(o, rhs, x)])) / o.dot2(rhs, rhs))
        assert true <= 2e-6
        xs = np.zeros_like(rhs)
        o.fgmres(xs, rhs, maxiter=40, tol=1e-12)
        sols.append(xs)
    nc = geo.grid.nx * geo.grid.ny * geo.grid.nz
    live = geo.volc[1:-1, 1:-1, 1:-1].ravel() > 0
    assert np.max(np.abs(sols[0][:nc] - sols[1][:nc])[live]) <= 1e-9 * np.max(np.abs(sols[0][:nc])[live])


def _resid(o, b, x):
    r = b - o.matvec1(x)
    o.exchange(r)
    return r


@pytest.mark.parametrize("name", ["proj_per_hill_16x12x10", "proj_per_x_hill_13x7x9"])
def test_density_weights_periodic_faces(name):
    """CellToFaceRhoWeight on a periodic side ('iw'/'ie'/'is'/'in', equal
    refinement, MULTI/JacAccGrav_Mod.f90:3313-3321, 3360-3368, 3407-3415,
    3454-3462): theta of the inner cell and of the halo image, each divided
    first and then weighted by its volume."""
    geo, W, dx, dy, dz, _, o = _make(name)
    g = geo.grid
    rth, rho, rv, rc, t = _moist_state(geo)
    dtu, dtv, dtw, *_ = o.weights_density(rth, rho, rv, rc, None, t)
    eps = 1.0e-30
    th = rth / (rho + eps)
    V = geo.volc
    I = slice(1, -1)
    west = (th[I, I, 1] * V[I, I, 1] + th[I, I, 0] * V[I, I, 0]) / (V[I, I, 1] + V[I, I, 0] + eps)
    east = (th[I, I, -1] * V[I, I, -1] + th[I, I, -2] * V[I, I, -2]) / (V[I, I, -1] + V[I, I, -2] + eps)
    np.testing.assert_array_equal(dtu[:, :, 0], west)
    np.testing.assert_array_equal(dtu[:, :, -1], east)
    if g.periodic_y:
        south = (th[I, 1, I] * V[I, 1, I] + th[I, 0, I] * V[I, 0, I]) / (V[I, 1, I] + V[I, 0, I] + eps)
        np.testing.assert_array_equal(dtv[:, 0, :], south)
    else:
        np.testing.assert_array_equal(dtv[:, 0, :], th[I, 1, I])
    np.testing.assert_array_equal(dtw[0], th[1, I, I])
