"""Open boundaries of the transport stage on the GPU, through the C-ABI,
against the oracle: the halo rules MeanValue, Function, InFlowOutFlow and
Extrapolation of BoundaryCompute (ADVECT/BoundaryCondition_Mod.f90:70-346)
bit for bit, the flux right-hand side with the first-order inflow through
the outer walls (ADVECT/Advection_Mod.f90:975-1044) and random halos bit for
bit, Rosenbrock steps of a channel with flow through every wall at 1e-12
(FP64) and 1e-10 (refined), the device-driven step graph bitwise equal to
the stream path, and the refusals (a kind without its data, the dynamical
core, the adjoint)."""
import numpy as np
import pytest

from tests import cases

pytestmark = pytest.mark.gpu

CHANNEL = "channel_open_10x7x6"
FP64_TOL = 1e-12
REFINED_TOL = 1e-10


@pytest.fixture(scope="module")
def env(built_lib):
    import asam_gb300
    import oracle

    return asam_gb300, oracle


def _data(geo, nc, seed):
    rng = np.random.default_rng(seed)
    g = geo.grid
    return (rng.standard_normal((nc, g.nz)), rng.standard_normal((nc,) + g.pshape),
            1.0 + rng.random((nc,) + g.pshape))


def _block(env, geo, vel, st, **kw):
    asam, _ = env
    blk = asam.TransportBlock(geo, ncomp=st.c.shape[0], rho_pos=st.rho_pos, **kw)
    blk.set_velocity(*vel)
    return blk


@pytest.mark.parametrize("name", [CHANNEL, "bubble_12x10x8"])
def test_bound_cond_open_kinds_bitwise(env, name):
    """Every kind on every side (random), the density on InFlowOutFlow too."""
    _, oracle = env
    geo, vel, st = cases.get(name)
    nc = st.c.shape[0]
    mean, fval, amb = _data(geo, nc, 8)
    rng = np.random.default_rng(9)
    with _block(env, geo, vel, st) as blk:
        blk.set_boundary_data(mean, fval, amb)
        for trial in range(3):
            kinds = rng.integers(0, 7, size=(nc, 6)).astype(np.int32)
            kinds[st.rho_pos, :4] = 5
            o = oracle.Oracle(geo, bc=kinds)
            o.set_boundary_data(mean, fval, amb, vel, rho_pos=st.rho_pos)
            c = rng.standard_normal(st.c.shape) + 2.0
            blk.set_boundary(kinds)
            got = blk.BoundaryCondition(c)
            ref = o.bound_cond(c)
            np.testing.assert_array_equal(got, ref)


def test_fcn_open_channel_random_halos_bitwise(env):
    """The inflow reads the halo values as they are: random halos."""
    _, oracle = env
    geo, vel, st = cases.get(CHANNEL)
    rng = np.random.default_rng(5)
    c = st.c.copy()
    halo = np.ones(c.shape[1:], dtype=bool)
    halo[1:-1, 1:-1, 1:-1] = False
    for ic in range(c.shape[0]):
        c[ic][halo] = (np.abs(c[ic][~halo]).max() + 1e-3) * (0.5 + rng.random(int(halo.sum())))
    ref = oracle.Oracle(geo).fcn(c, vel, st.rho_pos)
    with _block(env, geo, vel, st) as blk:
        got = blk.Fcn(c)
    diff = np.argwhere(got != ref)
    assert diff.size == 0, f"{len(diff)} mismatches, first {diff[:3].tolist()}"


def _channel_kinds(nc):
    kinds = np.ones((nc, 6), np.int32)
    kinds[:, 0] = kinds[:, 1] = 5  # InFlowOutFlow west/east
    kinds[:, 2] = 3                # MeanValue south
    kinds[:, 3] = 4                # Function north
    kinds[:, 4] = 6                # Extrapolation on the ground
    kinds[:, 5] = 2                # ZeroValue on the lid
    return kinds


def _channel_data(geo, st):
    nc = st.c.shape[0]
    c = st.c
    mean = np.stack([c[ic][1:-1, 1:-1, 1:-1].mean(axis=(1, 2)) for ic in range(nc)])
    fval = 0.9 * c.copy()
    # the ambient state as the halo's density times VecAmb: a density factor
    # and each component's mean interior mixing ratio
    inner = np.s_[1:-1, 1:-1, 1:-1]
    amb = np.empty_like(c)
    for ic in range(nc):
        amb[ic] = 1.02 if ic == st.rho_pos else float((c[ic][inner] / c[st.rho_pos][inner]).mean())
    return mean, fval, amb


@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("fp32_refined", REFINED_TOL)])
def test_ros_step_open_channel(env, precision, tol):
    """Three RosRK3 steps of the channel with a different open rule on every
    side against the oracle."""
    asam, oracle = env
    geo, vel, st = cases.get(CHANNEL)
    nc = st.c.shape[0]
    kinds = _channel_kinds(nc)
    mean, fval, amb = _channel_data(geo, st)
    o = oracle.Oracle(geo, bc=kinds)
    o.set_boundary_data(mean, fval, amb, vel, rho_pos=st.rho_pos)
    cr, cg = st.c.copy(), st.c.copy()
    with _block(env, geo, vel, st, method="RosRK3", bicgstab_tol=1e-10, precision=precision) as blk:
        blk.set_boundary_data(mean, fval, amb)
        blk.set_boundary(kinds)
        for step in range(3):
            it_r, _ = o.ros_step(cr, vel, 2.0, method=asam.METHODS["RosRK3"], tol=1e-10)
            it_g, _ = blk.Ros3MetC(cg, 2.0)
            if precision == "fp64":
                for a, b in zip(it_g, it_r):
                    assert abs(abs(a) - abs(b)) <= 1, (step, it_g, it_r)
            errs = cases.field_relerr(cg, cr)
            assert max(errs) <= tol, (step, errs)
    # mass crossed the open walls
    V = geo.volc[1:-1, 1:-1, 1:-1]
    m0, m1 = ((a[st.rho_pos][1:-1, 1:-1, 1:-1] * V).sum() for a in (st.c, cr))
    assert abs(m1 - m0) > 1e-6 * m0


def test_step_graph_open_channel_identical(env):
    """The whole step as one device-driven graph gives the stream path's bits
    with the open rules (their data are read through the captured pointers;
    new data after the capture are seen by the next step)."""
    geo, vel, st = cases.get(CHANNEL)
    nc = st.c.shape[0]
    kinds = _channel_kinds(nc)
    mean, fval, amb = _channel_data(geo, st)
    out = {}
    for mode in (0, 2):
        c = st.c.copy()
        with _block(env, geo, vel, st, method="RosRK3", bicgstab_tol=1e-12) as blk:
            blk.set_graphs(mode)
            blk.set_boundary_data(mean, fval, amb)
            blk.set_boundary(kinds)
            its = [blk.Ros3MetC(c, 2.0)[0] for _ in range(2)]
            blk.set_boundary_data(mean * 1.01, fval, amb)
            its += [blk.Ros3MetC(c, 2.0)[0] for _ in range(2)]
        out[mode] = (c, its)
    assert np.array_equal(out[2][0], out[0][0])
    assert out[2][1] == out[0][1]


def test_open_boundary_refusals(env):
    asam, _ = env
    from asam_gb300._lib import AsamError

    geo, vel, st = cases.get(CHANNEL)
    nc = st.c.shape[0]
    mean, fval, amb = _data(geo, nc, 1)
    with _block(env, geo, vel, st) as blk:
        kinds = np.ones((nc, 6), np.int32)
        for k in (3, 4, 5):  # each kind needs its array first
            kinds[1, 0] = k
            with pytest.raises(AsamError):
                blk.set_boundary(kinds)
        kinds[1, 0] = 6  # Extrapolation needs none
        blk.set_boundary(kinds)
        blk.set_boundary_data(mean, None, None)
        kinds[1, 0] = 3
        blk.set_boundary(kinds)
        with pytest.raises(AsamError):
            blk.set_boundary_data(None, None, None)  # MeanValue in use
        with pytest.raises(ValueError):
            blk.set_boundary_data(mean[:, :-1])
        # the adjoint is built for the closed-wall rules only
        c = np.ascontiguousarray(st.c)
        dc = np.zeros_like(c[1])
        df = np.zeros_like(c[1])
        assert blk.lib.asam_fcn_tlm(blk.h, c.ctypes.data, 1, dc.ctypes.data, df.ctypes.data) == asam._lib.ASAM_BAD_ARG
    # the dynamical core refuses the open rules (its BoundaryVelocity and
    # projection are built for closed and periodic sides), in either order
    from asam_gb300 import geometry as G

    geo, vel, st, pos, (dx, dy, dz), bc = G.dyn_case(10, 8, 7, hill=False)
    nc = st.c.shape[0]
    kinds = np.ones((nc, 6), np.int32)
    kinds[pos["th"], 4] = 6
    for order in ("boundary_first", "dyn_first"):
        with asam.TransportBlock(geo, ncomp=nc, rho_pos=0) as blk:
            blk.set_velocity(*vel)
            blk.proj_setup(dx, dy, dz)
            if order == "boundary_first":
                blk.set_boundary(kinds)
                with pytest.raises(AsamError):
                    blk.dyn_setup(pos["th"], pos["mom"])
            else:
                blk.dyn_setup(pos["th"], pos["mom"])
                with pytest.raises(AsamError):
                    blk.set_boundary(kinds)
