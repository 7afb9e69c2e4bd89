"""Pins of the CPU oracle (CPU only, no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by
(1) an independent numpy restatement in gather form (tests/pyref.py) that
must agree bit for bit, (2) analytic known answers (constant mixing ratio,
mass conservation, upwind linearisation, triangular/tridiagonal algebra,
converged Krylov solution of the periodic system) and (3) the committed
golden fixtures of tests/golden/.
"""
import numpy as np
import pytest

from tests import cases, pyref

SMALL = ["bubble_12x10x8", "hill_24x20x16", "hill_odd_13x7x9_reverse", "flat_walls_9x6x5", "column_1x1x12",
         "slab_1x9x6"]


@pytest.fixture(scope="module")
def oracle_mod(built_oracle):
    import oracle

    return oracle


@pytest.mark.parametrize("name", SMALL)
def test_fcn_matches_independent_restatement(oracle_mod, name):
    geo, vel, st = cases.get(name)
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    got = o.fcn(c, vel)
    ref = pyref.fcn(geo, c, vel)
    assert np.array_equal(got, ref), cases.relerr(got, ref)


@pytest.mark.parametrize("name", SMALL)
def test_fcn_constant_mixing_ratio(oracle_mod, name):
    """A tracer with constant mixing ratio q advects exactly like q*Rho."""
    geo, vel, st = cases.get(name)
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    q = 0.37
    cc = np.stack([c[0], q * c[0]])
    f = o.fcn(np.ascontiguousarray(cc), vel)
    scale = np.abs(f[0]).max() + 1e-300
    assert np.abs(f[1] - q * f[0]).max() <= 1e-13 * max(scale, 1e-12)


@pytest.mark.parametrize("name", SMALL)
def test_fcn_conserves_mass(oracle_mod, name):
    """sum(f*V) over the interior vanishes: every face flux leaves one cell and enters another."""
    geo, vel, st = cases.get(name)
    g = geo.grid
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    f = o.fcn(c, vel)
    V = geo.volc[1:-1, 1:-1, 1:-1]
    uf, vf, wf = vel
    flux_scale = (np.abs(uf).max() * geo.fu.max() + np.abs(vf).max() * geo.fv.max() + np.abs(wf).max()
                  * geo.fw.max()) * np.abs(c / (c[0] + 1e-30)).reshape(c.shape[0], -1).max(1)
    for ic in range(c.shape[0]):
        tot = (f[ic, 1:-1, 1:-1, 1:-1] * V).sum()
        assert abs(tot) <= 1e-12 * flux_scale[ic] * g.nx * g.ny * g.nz + 1e-300


@pytest.mark.parametrize("name", SMALL)
def test_jacobian_is_upwind_linearisation(oracle_mod, name):
    """With beta0*dt = 1 the DIA matrix is I - J; J*c must equal the first-order upwind RHS."""
    geo, vel, st = cases.get(name)
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    rho = c[0]
    val = o.jac(rho, vel, 1.0, 1.0)
    A = pyref.dia_scipy(val, geo.grid)
    n = geo.grid.npad
    for ic in (0, c.shape[0] - 1):
        x = c[ic].reshape(-1)
        Jx = x - A @ x
        ref = pyref.upwind_rhs(geo, c[ic], vel, rho).reshape(-1)
        interior = np.zeros(geo.grid.pshape, dtype=bool)
        interior[1:-1, 1:-1, 1:-1] = True
        m = interior.reshape(-1)
        scale = np.abs(ref[m]).max() + np.abs(x[m]).max() * 1e-3
        assert np.abs(Jx[m] - ref[m]).max() <= 1e-10 * scale, (ic, np.abs(Jx[m] - ref[m]).max(), scale)
        assert n == x.size


@pytest.mark.parametrize("name", SMALL)
def test_spmv_matches_scipy(oracle_mod, name):
    geo, vel, st = cases.get(name)
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    val = o.jac(c[0], vel, 0.79, 7.0)
    x = np.ascontiguousarray(c[1 % c.shape[0]].reshape(-1))
    got = o.spmv(val, x)
    ref = pyref.dia_scipy(val, geo.grid) @ x
    assert np.allclose(got, ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())


@pytest.mark.parametrize("name", SMALL)
def test_gauss_seidel_matches_triangular_solves(oracle_mod, name):
    geo, vel, st = cases.get(name)
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    val = o.jac(c[0], vel, 1.0, 30.0)
    b = np.ascontiguousarray(c[-1].reshape(-1))
    got = o.gauss_seidel(val, b, 5)
    ref = pyref.gauss_seidel(val, geo.grid, b, 5)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_gauss_seidel_diagonal_is_exact(oracle_mod):
    geo, vel, st = cases.get("bubble_12x10x8")
    o = oracle_mod.Oracle(geo)
    n = geo.grid.npad
    val = np.zeros((7, n))
    rng = np.random.default_rng(0)
    val[3] = 1.0 + rng.random(n)
    b = rng.standard_normal(n)
    assert np.array_equal(o.gauss_seidel(val, b, 5), b / val[3])


@pytest.mark.parametrize("name", ["hill_24x20x16", "flat_walls_9x6x5", "hill_odd_13x7x9_reverse"])
def test_bicgstab_solves_periodic_system(oracle_mod, name):
    """The converged BiCGStab solution equals the direct solution of the interior system
    with periodic images substituted for the halo columns."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    geo, vel, st = cases.get(name)
    g = geo.grid
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    val = o.jac(c[0], vel, 1.0, 40.0)
    b = 40.0 * o.fcn(c, vel)
    x = np.zeros_like(b)
    it, tol = o.bicgstab(val, x, b, 60, 1e-13)
    assert it < 0 or it <= 60
    # interior periodic operator
    A = pyref.dia_scipy(val, g)
    P = np.arange(g.npad).reshape(g.pshape)
    idx = P.copy()
    if g.periodic_x:
        idx[:, :, 0] = P[:, :, g.nx]
        idx[:, :, g.nx + 1] = P[:, :, 1]
    if g.periodic_y:
        idx[:, 0, :] = P[:, g.ny, :]
        idx[:, g.ny + 1, :] = P[:, 1, :]
    interior = P[1:-1, 1:-1, 1:-1].reshape(-1)
    cols = idx.reshape(-1)
    A = A.tocoo()
    keep_row = np.isin(A.row, interior)
    pos = -np.ones(g.npad, dtype=np.int64)
    pos[interior] = np.arange(interior.size)
    rows = pos[A.row[keep_row]]
    ccol = pos[cols[A.col[keep_row]]]
    ok = ccol >= 0
    Aint = sp.csr_matrix((A.data[keep_row][ok], (rows[ok], ccol[ok])), shape=(interior.size, interior.size))
    for ic in range(b.shape[0]):
        bi = b[ic].reshape(-1)[interior]
        if not np.any(bi):
            continue
        xd = spl.spsolve(Aint.tocsc(), bi)
        xi = x[ic].reshape(-1)[interior]
        assert np.abs(xi - xd).max() <= 1e-9 * np.abs(xd).max(), ic


@pytest.mark.parametrize("name", SMALL)
def test_ros_step_conserves_mass_and_mixing_ratio(oracle_mod, name):
    geo, vel, st = cases.get(name)
    o = oracle_mod.Oracle(geo)
    q = 0.25
    c = np.ascontiguousarray(np.stack([st.c[0], q * st.c[0], st.c[-1]]))
    m0 = [o.total_scalar(np.ascontiguousarray(c[i])) for i in range(3)]
    o.ros_step(c, vel, 3.0, method=5, tol=1e-12)
    m1 = [o.total_scalar(np.ascontiguousarray(c[i])) for i in range(3)]
    for a, b in zip(m0, m1):
        assert abs(a - b) <= 1e-12 * abs(a) + 1e-300
    V = geo.volc[1:-1, 1:-1, 1:-1]
    live = V > 0
    ratio = c[1, 1:-1, 1:-1, 1:-1][live] / c[0, 1:-1, 1:-1, 1:-1][live]
    assert np.abs(ratio - q).max() <= 1e-11


@pytest.mark.parametrize("ncol,n1", [(1, 1), (5, 2), (9, 17), (40, 64)])
def test_thomas_matches_dense(oracle_mod, ncol, n1):
    rng = np.random.default_rng(n1)
    d = 4.0 + rng.random((ncol, n1))
    u = rng.standard_normal((ncol, max(n1 - 1, 0)))
    l = rng.standard_normal((ncol, max(n1 - 1, 0)))
    b = rng.standard_normal((ncol, n1))
    x = oracle_mod.tri_solve(d, u, l, b)
    y = oracle_mod.tri_matvec(d, u, l, x)
    for q in range(ncol):
        T = np.diag(d[q]) + np.diag(u[q], 1) + np.diag(l[q], -1)
        assert np.allclose(T @ x[q], b[q], rtol=1e-12, atol=1e-12)
        assert np.allclose(T @ x[q], y[q], rtol=1e-13, atol=1e-13)


def test_ros_coefficients(oracle_mod):
    # Ros3Pw and RosRK3 tables of ADVECT/Int_Mod.f90:148-205 (alpha, beta scaled by beta0)
    n, b0, al, be, gm = oracle_mod.ros_coeffs(4)
    assert n == 3 and b0 == 7.88675134594812865529e-01
    assert al[0, 0] == 2.0 * b0 and be[1, 0] == -2.53589838486224561365e+00 * b0
    n, b0, al, be, gm = oracle_mod.ros_coeffs(5)
    assert n == 3 and b0 == 1.0 and al[0, 0] == 1.0 / 3.0 and al[2, 2] == 1.0
    assert list(gm[:4]) == [0.0, 1.0 / 3.0, 0.5, 1.0]
    n, b0, *_ = oracle_mod.ros_coeffs(0)
    assert n == 2 and b0 == float(np.float32(0.5) + np.sqrt(np.float32(3.0)) / np.float32(6.0))


def test_bicgstab_halfsteps_reproduces_exits():
    """The oracle's fixed half-step count reproduces the tolerance-driven exits
    bit for bit (the comparison of runs whose counts differ by one)."""
    import oracle
    from tests import cases as CS

    geo, vel, st = CS.get("hill_24x20x16")
    o = oracle.Oracle(geo)
    c = o.exchange_cell(st.c)
    val = o.jac(c[0], vel, 0.435866521508459, 20.0)
    b = np.random.default_rng(3).standard_normal(st.c.shape)
    for tol in (1e-4, 1e-8, 1e-12):
        x1 = np.zeros_like(b)
        it, _ = o.bicgstab(val, x1, b, 30, tol)
        half = 2 * (-it) - 1 if it < 0 else (it if it > 30 else 2 * it)
        x2 = np.zeros_like(b)
        o.bicgstab_halfsteps(val, x2, b, half)
        assert np.array_equal(x1, x2), (tol, it)
