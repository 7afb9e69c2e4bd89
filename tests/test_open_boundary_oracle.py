"""Pins of the oracle's open boundaries (CPU only, no GPU): the halo rules
MeanValue, Function, InFlowOutFlow and Extrapolation of BoundaryCompute
(ADVECT/BoundaryCondition_Mod.f90:70-346), the first-order inflow through
the faces of the outer walls (ADVECT/Advection_Mod.f90:975-1044) and the
outflow term the Jacobian keeps on those walls (:2390-2410 and its twins),
against the independent numpy restatement of tests/pyref.py, a constant
mixing ratio and the upwind linearisation."""
import numpy as np
import pytest

from tests import cases, pyref

CHANNEL = "channel_open_10x7x6"


@pytest.fixture(scope="module")
def oracle_mod(built_oracle):
    import oracle

    return oracle


def _random_halos(c, seed):
    """The state with every halo cell replaced by positive random values
    (the interior unchanged): inflow then carries values unrelated to the
    interior."""
    rng = np.random.default_rng(seed)
    out = c.copy()
    halo = np.ones(c.shape[1:], dtype=bool)
    halo[1:-1, 1:-1, 1:-1] = False
    for ic in range(c.shape[0]):
        scale = np.abs(c[ic][~halo]).max() + 1e-3
        out[ic][halo] = scale * (0.5 + rng.random(int(halo.sum())))
    return out


def _data(geo, nc, seed):
    rng = np.random.default_rng(seed)
    g = geo.grid
    mean = rng.standard_normal((nc, g.nz))
    fval = rng.standard_normal((nc,) + g.pshape)
    amb = 1.0 + rng.random((nc,) + g.pshape)
    return mean, fval, amb


@pytest.mark.parametrize("periodic_x", [False, True])
def test_bound_cond_open_kinds_match_numpy(oracle_mod, periodic_x):
    """Every kind 0-6 on every side, the density first and last in the
    component order (InFlowOutFlow reads the density halo as updated so far);
    a periodic side keeps its halos."""
    geo, vel, st = cases.get(CHANNEL)
    if periodic_x:
        geo, vel, st = cases.get("bubble_12x10x8")
    nc = st.c.shape[0]
    rng = np.random.default_rng(7)
    mean, fval, amb = _data(geo, nc, 8)
    g = geo.grid
    for rho_pos in (0, nc - 1):
        kinds = rng.integers(0, 7, size=(nc, 6)).astype(np.int32)
        kinds[rho_pos, :4] = 5  # the density itself on InFlowOutFlow
        o = oracle_mod.Oracle(geo, bc=kinds)
        o.set_boundary_data(mean, fval, amb, vel, rho_pos=rho_pos)
        c = rng.standard_normal(st.c.shape) + 2.0
        got = o.bound_cond(c)
        ref = pyref.bound_cond(c, kinds, (g.periodic_x, g.periodic_y, g.periodic_z), mean=mean, fval=fval, amb=amb,
                               vel=vel, rho_pos=rho_pos)
        np.testing.assert_array_equal(got, ref)
        assert not np.array_equal(got, c)


def test_inflow_outflow_picks_the_ambient_on_inflow(oracle_mod):
    """InFlowOutFlow on the west wall: halo = Rho(halo)*VecAmb where uF >= 0
    (all of the channel's west faces), the interior value on the east wall
    where the flow leaves."""
    geo, vel, st = cases.get(CHANNEL)
    nc = st.c.shape[0]
    kinds = np.zeros((nc, 6), np.int32)
    kinds[:, 0] = kinds[:, 1] = 5
    mean, fval, amb = _data(geo, nc, 3)
    o = oracle_mod.Oracle(geo, bc=kinds)
    o.set_boundary_data(None, None, amb, vel, rho_pos=0)
    c = np.random.default_rng(4).random(st.c.shape) + 1.0
    got = o.bound_cond(c)
    assert (vel[0][:, :, 0] >= 0).all() and (vel[0][:, :, -1] > 0).all()
    rho_h = c[0][1:-1, 1:-1, 0] * amb[0][1:-1, 1:-1, 0]
    np.testing.assert_array_equal(got[0][1:-1, 1:-1, 0], rho_h)
    for ic in range(1, nc):
        np.testing.assert_array_equal(got[ic][1:-1, 1:-1, 0], rho_h * amb[ic][1:-1, 1:-1, 0])
        np.testing.assert_array_equal(got[ic][1:-1, 1:-1, -1], c[ic][1:-1, 1:-1, -2])


def test_fcn_open_channel_matches_restatement(oracle_mod):
    """Flux right-hand side with flow through every outer wall: the inflow
    from the halos and the zeroed wall halos, bit for bit."""
    geo, vel, st = cases.get(CHANNEL)
    o = oracle_mod.Oracle(geo)
    c = _random_halos(st.c, 5)
    got = o.fcn(c, vel)
    ref = pyref.fcn(geo, c, vel)
    assert np.array_equal(got, ref), cases.relerr(got, ref)
    # the inflow matters: other mixing ratios in the west halo change the
    # west column's right-hand side
    c2 = c.copy()
    c2[1:, 1:-1, 1:-1, 0] *= 2.0
    assert not np.array_equal(o.fcn(c2, vel)[1:, 1:-1, 1:-1, 1], got[1:, 1:-1, 1:-1, 1])


def test_fcn_open_channel_constant_mixing_ratio(oracle_mod):
    """A tracer q*Rho (halos included) advects exactly like q*Rho through
    open walls too."""
    geo, vel, st = cases.get(CHANNEL)
    o = oracle_mod.Oracle(geo)
    c = _random_halos(st.c, 6)
    q = 0.37
    cc = np.ascontiguousarray(np.stack([c[0], q * c[0]]))
    f = o.fcn(cc, vel)
    scale = np.abs(f[0]).max()
    assert np.abs(f[1] - q * f[0]).max() <= 1e-13 * scale


def test_jacobian_keeps_the_wall_outflow(oracle_mod):
    """With beta0*dt = 1 the DIA matrix is I - J and J*c is the first-order
    upwind right-hand side, the outflow through the outer walls included."""
    geo, vel, st = cases.get(CHANNEL)
    o = oracle_mod.Oracle(geo)
    c = o.exchange_cell(st.c)
    rho = c[0]
    val = o.jac(rho, vel, 1.0, 1.0)
    A = pyref.dia_scipy(val, geo.grid)
    interior = np.zeros(geo.grid.pshape, dtype=bool)
    interior[1:-1, 1:-1, 1:-1] = True
    m = interior.reshape(-1)
    for ic in (0, c.shape[0] - 1):
        x = np.where(interior, c[ic], 0.0).reshape(-1)  # the halos carry no state dependence
        Jx = x - A @ x
        ref = pyref.upwind_rhs(geo, np.where(interior, c[ic], 0.0), vel, rho).reshape(-1)
        scale = np.abs(ref[m]).max()
        assert np.abs(Jx[m] - ref[m]).max() <= 1e-12 * scale
    # the wall terms are there: the east column's diagonal carries the outflow
    closed = o.jac(rho, (vel[0] * np.where(np.arange(vel[0].shape[2]) == vel[0].shape[2] - 1, 0.0, 1.0),
                         vel[1], vel[2]), 1.0, 1.0)
    assert not np.array_equal(closed[3], val[3])


def test_ros_step_open_channel_mixing_ratio(oracle_mod):
    """A step of the open channel with InFlowOutFlow on the lateral walls,
    MeanValue on the lid and Extrapolation on the ground: the mass change of
    a constant-mixing-ratio tracer is q times the density's."""
    import asam_gb300 as asam

    geo, vel, st = cases.get(CHANNEL)
    nc = st.c.shape[0]
    kinds = np.ones((nc, 6), np.int32)
    kinds[:, :4] = 5
    kinds[:, 4] = 6
    kinds[:, 5] = 3
    g = geo.grid
    q = 0.25
    c = st.c.copy()
    c[nc - 1] = q * c[0]
    mean = np.stack([c[ic][1:-1, 1:-1, 1:-1].mean(axis=(1, 2)) for ic in range(nc)])
    amb = np.ones((nc,) + g.pshape)
    amb[nc - 1] = q
    o = oracle_mod.Oracle(geo, bc=kinds)
    o.set_boundary_data(mean, None, amb, vel, rho_pos=0)
    c0 = c.copy()
    o.ros_step(c, vel, 1.0, method=asam.METHODS["RosRK3"], tol=1e-12)
    V = geo.volc[1:-1, 1:-1, 1:-1]
    dm = [((c[ic] - c0[ic])[1:-1, 1:-1, 1:-1] * V).sum() for ic in (0, nc - 1)]
    assert abs(dm[0]) > 0
    assert abs(dm[1] - q * dm[0]) <= 1e-9 * abs(q * dm[0])
