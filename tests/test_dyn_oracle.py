"""CPU checks of the dynamical-core oracle (oracle/asam_dyn.c) and of the
outer-wall halo rule -- no GPU needed.

* BoundaryCompute's ZeroGrad/ZeroValue halos equal a numpy restatement;
* the BoundCell list of the generator holds exactly the surface cells;
* VelocityFaceToCellLR then VelocityCellToFaceLR is the identity on the
  interior faces of a flat box (to rounding) and zero on the walls of the
  normal components; the boundary-cell shift follows ShiftVel1 / ShiftNoSlip;
* AbsTCompute/PreCompute and the pressure-gradient and buoyancy sources of
  FcnMet equal numpy restatements; without them FcnMet is the transport Fcn;
* a few Rosenbrock steps of the dynamical core conserve the total mass to
  rounding and keep the FGMRES residual below its tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from asam_gb300 import geometry as G
from tests import pyref


def _kinds(ncomp, mom, no_slip=False):
    k = np.ones((ncomp, 6), np.int32)
    for q, p in enumerate(mom):
        for sd in range(6):
            k[p, sd] = 2 if (no_slip or q // 2 == sd // 2) else 1
    return k


@pytest.fixture(scope="module")
def hill():
    return G.dyn_case(13, 9, 10, seed=7, moist=True, tracer=True)


@pytest.fixture(scope="module")
def flat():
    return G.dyn_case(10, 8, 7, hill=False)


def test_bound_cond_matches_numpy(hill):
    geo, vel, st, pos, _, _ = hill
    nc = st.c.shape[0]
    rng = np.random.default_rng(1)
    kinds = rng.integers(0, 3, size=(nc, 6)).astype(np.int32)
    o = oracle.Oracle(geo, bc=kinds)
    c = rng.standard_normal(st.c.shape)
    np.testing.assert_array_equal(o.bound_cond(c), pyref.bound_cond(c, kinds))
    o.set_boundary(None)  # default: ZeroGrad everywhere
    np.testing.assert_array_equal(o.bound_cond(c), pyref.bound_cond(c, np.ones((nc, 6), np.int32)))


def test_boundary_cells(hill, flat):
    geo, *_, bc = hill
    g = geo.grid
    assert len(bc) > 0
    vol = geo.volc[1:-1, 1:-1, 1:-1]
    assert np.all(vol[bc[:, 2] - 1, bc[:, 1] - 1, bc[:, 0] - 1] > 0)
    # every cut cell whose floor is closed holds surface
    fw = geo.fw[1:g.nz + 1]
    full = g.dx * g.dy * np.asarray(g.dz)[:, None, None]
    cut = (vol > 0) & (vol < full) & (fw == 0)
    k, j, i = np.nonzero(cut)
    listed = {tuple(r) for r in bc.tolist()}
    assert all((ii + 1, jj + 1, kk + 1) in listed for kk, jj, ii in zip(k, j, i))
    assert len(flat[-1]) == 0


def test_face_cell_round_trip_flat(flat):
    geo, vel, st, pos, _, bc = flat
    o = oracle.Oracle(geo, bc=_kinds(st.c.shape[0], pos["mom"]))
    c = o.face_to_cell(pos["mom"], vel, np.zeros_like(st.c), bc)
    u, v, w = o.cell_to_face(pos["mom"], c)
    for got, ref in zip((u, v, w), vel):
        assert np.max(np.abs(got - ref)) <= 1e-15 * np.max(np.abs(ref))
    assert not u[:, :, 0].any() and not u[:, :, -1].any()
    assert not w[0].any() and not w[-1].any()


@pytest.mark.parametrize("free_slip", [True, False])
def test_boundary_shift_formula(hill, free_slip):
    geo, vel, st, pos, _, bc = hill
    o = oracle.Oracle(geo)
    c = o.face_to_cell(pos["mom"], vel, np.zeros_like(st.c), bc, free_slip=free_slip)
    uf = vel[0]
    eps = 1e-30
    for ix, iy, iz in bc[:25]:
        FL, FR = geo.fu[iz - 1, iy - 1, ix], geo.fu[iz - 1, iy - 1, ix + 1]
        l, r = uf[iz - 1, iy - 1, ix - 1], uf[iz - 1, iy - 1, ix]
        if free_slip:
            cl, cr = (l, (FR * r + (FL - FR) * l) / (FL + eps)) if FL > FR else ((FL * l + (FR - FL) * r) / (FR + eps), r)
        else:
            m = max(FR, FL)
            with np.errstate(invalid="ignore", divide="ignore"):
                cl, cr = FL * l / m, FR * r / m
        np.testing.assert_array_equal([c[pos["mom"][0], iz, iy, ix], c[pos["mom"][1], iz, iy, ix]], [cl, cr])


def test_thermo_matches_numpy(hill):
    geo, vel, st, pos, _, _ = hill
    o = oracle.Oracle(geo)
    c = st.c
    t, p = o.thermo(c, 0, pos["th"], rv_pos=pos["qv"])
    tr, pr = pyref.thermo(c[0], c[pos["th"]], rv=c[pos["qv"]])
    # both evaluate pow(); numpy's and the C library's may differ in the last bits
    np.testing.assert_allclose(t, tr, rtol=1e-15, atol=0)
    # the closed walls copy the pressure of the adjacent cell (PreCompute :816-862)
    I = (slice(1, -1), slice(1, -1), slice(1, -1))
    np.testing.assert_allclose(p[I], pr[I], rtol=1e-15, atol=0)
    np.testing.assert_array_equal(p[1:-1, 1:-1, 0], p[1:-1, 1:-1, 1])
    np.testing.assert_array_equal(p[0, 1:-1, 1:-1], p[1, 1:-1, 1:-1])
    # a dry isothermal-ish check: p = rho Rd T
    assert np.all(np.abs(pr[I] / (c[0][I] * pyref.RD * tr[I]) - 1.0) < 0.02)


def test_fcn_dyn_sources(hill):
    geo, vel, st, pos, (dx, dy, dz), _ = hill
    o = oracle.Oracle(geo)
    c = st.c
    _, p = o.thermo(c, 0, pos["th"], rv_pos=pos["qv"])
    f0 = o.fcn(c, vel)
    f_off = o.fcn_dyn(c, vel, p, pos["mom"], dx, dy, dz, pgrad=False, buoy=False)
    np.testing.assert_array_equal(f_off, f0)
    f = o.fcn_dyn(c, vel, p, pos["mom"], dx, dy, dz)
    pg, bu = pyref.momentum_sources(geo, p, c[0], dx, dy, dz)
    I = (slice(1, -1), slice(1, -1), slice(1, -1))
    V = geo.volc[I]
    for q, comp in enumerate(pos["mom"]):
        # (a + pg)/(V+Eps) (+ bu) against a/(V+Eps): compare the sources
        src = pg[q] / (V + 1e-30) + (bu[q - 4] if q >= 4 else 0.0)
        d = f[comp][I] - f0[comp][I]
        scale = np.max(np.abs(src)) + np.max(np.abs(f0[comp][I]))
        assert np.max(np.abs(d - src)) <= 1e-13 * scale, q
    others = [i for i in range(c.shape[0]) if i not in pos["mom"]]
    np.testing.assert_array_equal(f[others], f0[others])


def test_ros_step_dyn_conserves_mass(hill):
    geo, vel, st, pos, (dx, dy, dz), bc = hill
    nc = st.c.shape[0]
    o = oracle.Oracle(geo, bc=_kinds(nc, pos["mom"]))
    W = G.projection_inputs(geo)[0]
    pr = oracle.OracleProj(geo, dx, dy, dz, W, zebra=1)
    c = st.c.copy()
    u, v, w = (a.copy() for a in vel)
    V = geo.volc[1:-1, 1:-1, 1:-1]
    m0 = float(np.sum(c[0][1:-1, 1:-1, 1:-1] * V))
    for _ in range(2):
        it, rs, ps, prr = o.ros_step_dyn(pr, c, (u, v, w), 2.0, rho_pos=0, th_pos=pos["th"], pos=pos["mom"], dx=dx,
                                         dy=dy, dz=dz, rv_pos=pos["qv"], bound=bc,
                                         scalars=[pos["qv"], pos["tracer"]], bicg_tol=1e-10, proj_tol=1e-10,
                                         proj_maxiter=20)
        assert all(r <= 1e-10 for r in prr)
    assert np.all(np.isfinite(c))
    m1 = float(np.sum(c[0][1:-1, 1:-1, 1:-1] * V))
    assert abs(m1 - m0) <= 1e-13 * m0
    # walls stay closed
    assert not u[:, :, 0].any() and not u[:, :, -1].any() and not w[0].any() and not w[-1].any()


@pytest.fixture(scope="module")
def per_hill():
    return G.dyn_case(12, 10, 8, seed=9, moist=True, tracer=True, periodic=True)


def test_fcn_dyn_sources_periodic(per_hill):
    """The pressure gradient of a periodic block also acts across the shared
    boundary face (PGradComputeCFull's neighbour loop)."""
    geo, vel, st, pos, (dx, dy, dz), _ = per_hill
    o = oracle.Oracle(geo)
    c = o.exchange_cell(st.c)
    _, p = o.thermo(c, 0, pos["th"], rv_pos=pos["qv"])
    f0 = o.fcn(c, vel)
    f = o.fcn_dyn(c, vel, p, pos["mom"], dx, dy, dz)
    pg, bu = pyref.momentum_sources(geo, p, c[0], dx, dy, dz)
    assert np.any(pg[0][:, :, 0]) and np.any(pg[3][:, -1, :])
    I = (slice(1, -1), slice(1, -1), slice(1, -1))
    V = geo.volc[I]
    for q, comp in enumerate(pos["mom"]):
        src = pg[q] / (V + 1e-30) + (bu[q - 4] if q >= 4 else 0.0)
        d = f[comp][I] - f0[comp][I]
        scale = np.max(np.abs(src)) + np.max(np.abs(f0[comp][I]))
        assert np.max(np.abs(d - src)) <= 1e-13 * scale, q


def test_ros_step_dyn_periodic_conserves_mass(per_hill):
    """Two steps of the dynamical core of a periodic block (boundary face
    unknowns in the projection): mass conserved to rounding, the FGMRES
    tolerance reached, both copies of a periodic face keep equal velocities."""
    geo, vel, st, pos, (dx, dy, dz), bc = per_hill
    nc = st.c.shape[0]
    o = oracle.Oracle(geo, bc=_kinds(nc, pos["mom"]))
    W = G.projection_inputs(geo)[0]
    pr = oracle.OracleProj(geo, dx, dy, dz, W, zebra=1)
    assert pr.nface > 0
    c = st.c.copy()
    u, v, w = (a.copy() for a in vel)
    V = geo.volc[1:-1, 1:-1, 1:-1]
    m0 = float(np.sum(c[0][1:-1, 1:-1, 1:-1] * V))
    for _ in range(2):
        it, rs, ps, prr = o.ros_step_dyn(pr, c, (u, v, w), 2.0, rho_pos=0, th_pos=pos["th"], pos=pos["mom"], dx=dx,
                                         dy=dy, dz=dz, rv_pos=pos["qv"], bound=bc,
                                         scalars=[pos["qv"], pos["tracer"]], bicg_tol=1e-10, proj_tol=1e-10,
                                         proj_maxiter=40)
        assert all(r <= 1e-10 for r in prr)
    assert np.all(np.isfinite(c))
    m1 = float(np.sum(c[0][1:-1, 1:-1, 1:-1] * V))
    assert abs(m1 - m0) <= 1e-13 * m0
    np.testing.assert_array_equal(u[:, :, 0], u[:, :, -1])
    np.testing.assert_array_equal(v[:, 0, :], v[:, -1, :])
    assert not w[0].any() and not w[-1].any()
