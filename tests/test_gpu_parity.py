"""Parity of the CUDA library (through the C-ABI) with the CPU oracle.

Bit-exact where the kernel restates the reference's operation order
(flux RHS, Jacobian, stage operator, preconditioner, Thomas); the Krylov
solves and the Rosenbrock step differ only by the summation order of the dot
products and are held to 1e-12 relative per field (the drop-in tolerance),
with BiCGStab iteration counts equal or within one.
"""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12  # relative, per prognostic field
REFINED_TOL = 1e-10  # FP32-refined vs FP64 oracle

ALL = list(cases.CASES)


@pytest.fixture(scope="module")
def env(built_lib):
    import asam_gb300
    import oracle

    return asam_gb300, oracle


def _block(env, name, **kw):
    asam, _ = env
    geo, vel, st = cases.get(name)
    blk = asam.TransportBlock(geo, ncomp=st.c.shape[0], rho_pos=st.rho_pos, **kw)
    blk.set_velocity(*vel)
    return blk


@pytest.mark.parametrize("name", ALL)
def test_exchange_cell_bitwise(env, name):
    _, oracle = env
    geo, vel, st = cases.get(name)
    with _block(env, name) as blk:
        got = blk.ExchangeCell(st.c)
    ref = oracle.Oracle(geo).exchange_cell(st.c)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("name", ALL)
def test_fcn_bitwise(env, name):
    _, oracle = env
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    c = o.exchange_cell(st.c)
    ref = o.fcn(c, vel, st.rho_pos)
    with _block(env, name) as blk:
        got = blk.Fcn(c)
    assert np.isfinite(got).all()
    diff = np.argwhere(got != ref)
    assert diff.size == 0, f"{len(diff)} mismatches, first {diff[:3].tolist()} max rel {cases.relerr(got, ref):.3e}"


@pytest.mark.parametrize("name", ALL)
def test_div_bitwise(env, name):
    _, oracle = env
    geo, vel, st = cases.get(name)
    rhs = np.ascontiguousarray(st.c[0])
    ref = oracle.Oracle(geo).div(rhs, vel)
    with _block(env, name) as blk:
        got = blk.DivCompute(rhs)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("name", ALL)
def test_jac_bitwise(env, name):
    asam, oracle = env
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    c = o.exchange_cell(st.c)
    n, beta0, *_ = asam.ros_coeffs("Ros3Pw")
    ref = o.jac(c[st.rho_pos], vel, beta0, 2.0)
    with _block(env, name, method="Ros3Pw") as blk:
        blk.Jac(c, 2.0)
        got = blk.jac_matrix()
    for d in range(7):
        assert np.array_equal(got[d], ref[d]), f"diagonal {d}: max rel {cases.relerr(got[d], ref[d]):.3e}"


def _system(env, name, dt=2.0):
    asam, oracle = env
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    c = o.exchange_cell(st.c)
    n, beta0, *_ = asam.ros_coeffs("RosRK3")
    val = o.jac(c[st.rho_pos], vel, beta0, dt)
    b = dt * o.fcn(c, vel, st.rho_pos)
    return o, c, val, b


@pytest.mark.parametrize("name", ALL)
def test_matvec_bitwise(env, name):
    o, c, val, b = _system(env, name)
    ref = o.matvec(val, c)
    with _block(env, name) as blk:
        blk.set_jac_matrix(val)
        got = blk.MatVecMet(c)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("name", ALL)
def test_psolve_bitwise(env, name):
    o, c, val, b = _system(env, name)
    ref = o.psolve(val, b)
    with _block(env, name) as blk:
        blk.set_jac_matrix(val)
        got = blk.PSolve(b)
    diff = np.argwhere(got != ref)
    assert diff.size == 0, f"{len(diff)} mismatches, first {diff[:3].tolist()} max rel {cases.relerr(got, ref):.3e}"


@pytest.mark.parametrize("name", ALL)
@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_bicgstab(env, name, tol):
    o, c, val, b = _system(env, name, dt=20.0)
    xr = np.zeros_like(b)
    it_r, tol_r = o.bicgstab(val, xr, b, 30, tol)
    with _block(env, name) as blk:
        blk.set_jac_matrix(val)
        xg = np.zeros_like(b)
        it_g, tol_g = blk.BiCGStabMetSp(xg, b, 30, tol)
    assert abs(abs(it_g) - abs(it_r)) <= 1, (it_g, it_r)
    if it_g != it_r:  # compare against the oracle run with the GPU's count of half-steps
        # MaxIter -k: left after half-step 2k-1; k: after 2k; 2*MaxIter: not converged
        half = 2 * (-it_g) - 1 if it_g < 0 else (it_g if it_g > 30 else 2 * it_g)
        xr = np.zeros_like(b)
        o.bicgstab_halfsteps(val, xr, b, half)
    errs = cases.field_relerr(xg, xr)
    assert max(errs) <= FP64_TOL, errs


@pytest.mark.parametrize("name", ALL)
def test_ros_step_fp64(env, name):
    asam, oracle = env
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    cr = st.c.copy()
    cg = st.c.copy()
    with _block(env, name, method="RosRK3", bicgstab_tol=1e-10) as blk:
        for step in range(3):
            it_r, _ = o.ros_step(cr, vel, 2.0, method=asam.METHODS["RosRK3"], tol=1e-10)
            it_g, _ = blk.Ros3MetC(cg, 2.0)
            for a, b in zip(it_g, it_r):
                assert abs(abs(a) - abs(b)) <= 1, (step, it_g, it_r)
            errs = cases.field_relerr(cg, cr)
            assert max(errs) <= FP64_TOL, (step, errs)


@pytest.mark.parametrize("method", ["Ros3AMF", "RosRK32", "RosEul", "Ros3P", "Ros3Pw", "RosTVD", "RosRK4"])
def test_ros_methods(env, method):
    asam, oracle = env
    name = "hill_24x20x16"
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    cr, cg = st.c.copy(), st.c.copy()
    o.ros_step(cr, vel, 5.0, method=asam.METHODS[method], tol=1e-10)
    with _block(env, name, method=method, bicgstab_tol=1e-10) as blk:
        blk.Ros3MetC(cg, 5.0)
    assert max(cases.field_relerr(cg, cr)) <= FP64_TOL


def test_ros_coeffs_match_oracle(env):
    asam, oracle = env
    for m, mid in asam.METHODS.items():
        a = asam.ros_coeffs(m)
        b = oracle.ros_coeffs(mid)
        assert a[0] == b[0] and a[1] == b[1]
        assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4])


@pytest.mark.parametrize("iterg", [0, 1, 3])
@pytest.mark.parametrize("name", ALL)
def test_inner_psolve_fp32(env, name, iterg):
    """FP32 inner Gauss-Seidel: the persistent and the level-by-level schedule
    give the same bits (same arithmetic, only the order of the tiles differs),
    repeated calls reproduce them, and the result is the FP64 oracle's to FP32
    accuracy."""
    o, c, val, b = _system(env, name)
    ref = o.psolve(val, b, iterg=iterg)
    got = {}
    for sched in ("persistent", "levels"):
        with _block(env, name, precision="fp32_refined", inner_gs_iter=iterg, gs_schedule=sched) as blk:
            blk.set_jac_matrix(val)
            got[sched] = blk.inner_psolve(b)
            for _ in range(2):
                assert np.array_equal(blk.inner_psolve(b), got[sched])
    assert np.array_equal(got["persistent"], got["levels"])
    errs = cases.field_relerr(got["persistent"], ref)
    assert max(errs) <= 2e-5, errs


def test_persistent_gs_wait_gives_up(env):
    """The persistent schedule's bounded dependency waits: with a limit of one
    poll the waits run out (a tile's dependencies are computed by CTAs that
    started at the same time), every CTA leaves, the call returns
    ASAM_CUDA_ERROR with the schedule's message instead of hanging or
    trapping, and the same context afterwards reproduces its earlier result
    bit for bit (the completion counters need no repair)."""
    asam, _ = env
    name = "hill_24x20x16"
    _, _, val, b = _system(env, name)
    with _block(env, name, precision="fp32_refined", inner_gs_iter=3, gs_schedule="persistent") as blk:
        blk.set_jac_matrix(val)
        want = blk.inner_psolve(b)
        blk.set_wait_limit(1)
        with pytest.raises(asam.AsamError) as e:
            for _ in range(5):
                blk.inner_psolve(b)
        assert e.value.status == asam.ASAM_CUDA_ERROR
        assert "gave up" in str(e.value)
        blk.set_wait_limit(0)
        for _ in range(2):
            assert np.array_equal(blk.inner_psolve(b), want)


@pytest.mark.parametrize("precond,axis", [("line", 2), ("xline", 0), ("yline", 1)])
@pytest.mark.parametrize("name", ALL)
def test_inner_line_psolve_fp32(env, name, precond, axis):
    """FP32 line preconditioners against scipy's solve of the tridiagonal part of
    the stage matrix along the axis, with PSolve's halo handling."""
    import tests.pyref as pyref

    o, c, val, b = _system(env, name)
    geo = cases.get(name)[0]
    g = geo.grid
    bx = o.exchange_cell(b)
    x = pyref.line_solve(val, g, bx, axis).reshape(b.shape)
    x[:, [0, -1], :, :] = 0
    x[:, :, [0, -1], :] = 0
    x[:, :, :, [0, -1]] = 0
    ref = o.exchange_cell(x)
    with _block(env, name, precision="fp32_refined", inner_precond=precond) as blk:
        blk.set_jac_matrix(val)
        got = blk.inner_psolve(b)
    errs = cases.field_relerr(got, ref)
    assert max(errs) <= 2e-5, errs


@pytest.mark.parametrize("precision,inner", [("fp64", "gauss_seidel"), ("fp32_refined", "xline"),
                                             ("fp32_refined", "gauss_seidel")])
@pytest.mark.parametrize("name", ["hill_24x20x16", "flat_walls_9x6x5"])
def test_graph_captured_iterations_identical(env, name, precision, inner):
    """BiCGStab half-iterations replayed from CUDA graphs, and whole steps run
    as one graph whose Krylov loops are WHILE nodes (refined: the FP64
    refinement as an outer WHILE around the FP32 BiCGStab's loop; with the
    persistent Gauss-Seidel inner preconditioner too), give the bits and the
    iteration counts of the individually launched kernels, over several steps."""
    geo, vel, st = cases.get(name)
    out = {}
    for mode in (1, 0, 2):  # 2: the whole step as one graph with WHILE/IF nodes
        c = st.c.copy()
        with _block(env, name, method="RosRK3", bicgstab_tol=1e-12, precision=precision,
                    inner_precond=inner) as blk:
            blk.set_graphs(mode)
            its = [blk.Ros3MetC(c, 3.0)[0] for _ in range(4)]
        out[mode] = (c, its)
    for mode in (1, 2):
        assert np.array_equal(out[mode][0], out[0][0]), mode
        assert out[mode][1] == out[0][1], (mode, out[mode][1], out[0][1])


@pytest.mark.parametrize("name", ["hill_24x20x16", "hill_odd_13x7x9_reverse"])
def test_refined_step_schedules_identical(env, name):
    geo, vel, st = cases.get(name)
    out = {}
    for sched in ("persistent", "levels"):
        c = st.c.copy()
        with _block(env, name, method="RosRK3", bicgstab_tol=1e-12, precision="fp32_refined",
                    gs_schedule=sched) as blk:
            its = [blk.Ros3MetC(c, 4.0)[0] for _ in range(2)]
        out[sched] = (c, its)
    assert np.array_equal(out["persistent"][0], out["levels"][0])
    assert out["persistent"][1] == out["levels"][1]


@pytest.mark.parametrize("name", ["hill_24x20x16", "bubble_12x10x8"])
def test_autotuned_refined_step(env, name):
    """The autotuner only picks among settings that solve to the tolerance: the
    tuned refined step still matches the FP64 oracle."""
    asam, oracle = env
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    cr, cg = st.c.copy(), st.c.copy()
    with _block(env, name, method="RosRK3", bicgstab_tol=1e-12, precision="fp32_refined") as blk:
        choice = blk.autotune(st.c, 4.0)
        assert choice["inner_precond"] in asam.INNER_PRECONDS and 0 <= choice["inner_gs_iter"] <= 3
        assert 1 <= choice["gs_group"] <= st.c.shape[0] and choice["stage_solve_ms"] > 0
        for _ in range(2):
            o.ros_step(cr, vel, 4.0, method=asam.METHODS["RosRK3"], tol=1e-12)
            blk.Ros3MetC(cg, 4.0)
    errs = cases.field_relerr(cg, cr)
    assert max(errs) <= REFINED_TOL, (choice, errs)


@pytest.mark.parametrize("inner", ["line", "xline", "yline", "gauss_seidel"])
@pytest.mark.parametrize("name", ["hill_24x20x16", "hill_odd_13x7x9_reverse", "flat_walls_9x6x5"])
def test_ros_step_refined(env, name, inner):
    asam, oracle = env
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    cr, cg = st.c.copy(), st.c.copy()
    with _block(env, name, method="RosRK3", bicgstab_tol=1e-12, precision="fp32_refined",
                inner_precond=inner) as blk:
        for _ in range(2):
            o.ros_step(cr, vel, 4.0, method=asam.METHODS["RosRK3"], tol=1e-12)
            blk.Ros3MetC(cg, 4.0)
    errs = cases.field_relerr(cg, cr)
    assert max(errs) <= REFINED_TOL, errs


@pytest.mark.parametrize("name", ALL)
def test_total_scalar(env, name):
    _, oracle = env
    geo, vel, st = cases.get(name)
    ref = oracle.Oracle(geo).total_scalar(np.ascontiguousarray(st.c[0]))
    with _block(env, name) as blk:
        got = blk.TotalScalar(st.c, 0)
    assert abs(got - ref) <= 1e-13 * abs(ref)


@pytest.mark.parametrize("ncol,n1", [(1, 1), (7, 2), (31, 9), (32, 8), (33, 64), (65, 17), (100, 1), (5, 130),
                                     (1000, 128)])
def test_thomas_bitwise(env, ncol, n1):
    asam, oracle = env
    rng = np.random.default_rng(ncol * 1000 + n1)
    d = 4.0 + rng.random((ncol, n1))
    u = rng.standard_normal((ncol, max(n1 - 1, 0)))
    l = rng.standard_normal((ncol, max(n1 - 1, 0)))
    b = rng.standard_normal((ncol, n1))
    ref = oracle.tri_solve(d, u, l, b)
    got = asam.Solve_1D(d, u, l, b)
    assert np.array_equal(got, ref)
    assert np.array_equal(asam.MatVecT_1D(d, u, l, b), oracle.tri_matvec(d, u, l, b))


@pytest.mark.parametrize("span", [4, 30, 120])
def test_corrected_division_matches_ieee(env, span):
    """The FMA-corrected quotient from a precomputed reciprocal (used for the
    divisions by VolC+Eps, Rho+Eps and the Gauss-Seidel diagonal) equals the
    IEEE quotient on 2e7 random operand pairs."""
    import ctypes as C

    from asam_gb300 import _lib

    lib = _lib.load()
    bad = C.c_longlong(-1)
    _lib.check(lib.asam_probe_div(20_000_000, 1000 + span, span, C.byref(bad)), "asam_probe_div")
    assert bad.value == 0


@pytest.mark.parametrize("precision", ["fp64", "fp32_refined"])
def test_nan_detected(env, precision):
    """A NaN in the state stops the step with ASAM_NAN_DETECTED (the reference's
    driver stops on ISNAN(DOT(VecMet,VecMet))); the context stays usable."""
    asam, _ = env
    from asam_gb300 import _lib

    name = "hill_24x20x16"
    geo, vel, st = cases.get(name)
    with _block(env, name, method="RosRK3", bicgstab_tol=1e-10, precision=precision) as blk:
        bad = st.c.copy()
        bad[-1, 5, 6, 7] = np.nan
        with pytest.raises(_lib.AsamError) as err:
            blk.state_dot(bad)
        assert err.value.status == 3
        with pytest.raises(_lib.AsamError) as err:
            blk.Ros3MetC(bad, 2.0)
        assert err.value.status == 3
        good = st.c.copy()
        blk.Ros3MetC(good, 2.0)
        assert np.isfinite(good).all()
        assert blk.state_dot(good) > 0
