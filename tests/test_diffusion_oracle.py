"""CPU checks of the diffusion terms of the oracle (DiffusionCompute and
JacDiffusionCompute, ADVECT/Diffusion_Mod.f90:11-275, 1504-1708):

* the oracle's diffusion equals an independent numpy restatement in gather
  form bit for bit (periodic sides with their half fluxes, closed walls,
  one-column and one-cell-wide domains);
* known answers: a constant mixing ratio does not diffuse, the diffusion of a
  component conserves its total (walls with ZeroGrad halos carry no flux);
* the diffusion part of the stage matrix is the linearisation of the
  diffusion operator on every cell with volume away from the boundary rows.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

import oracle
from asam_gb300 import geometry as G
from tests import cases, pyref

ALL = list(cases.CASES)


def _setup(name, seed=3, close=False):
    geo, vel, st = cases.get(name)
    if close:
        geo = G.close_dead_faces(copy.deepcopy(geo))
    o = oracle.Oracle(geo)
    c = o.bound_cond(o.exchange_cell(st.c))
    dh, dv = G.diffusion_coefficients(geo, c[0], seed=seed)
    o.set_diffusion(dh, dv)
    return geo, vel, st, o, c, dh, dv


@pytest.mark.parametrize("name", ALL)
def test_diffusion_matches_numpy(name):
    geo, vel, st, o, c, dh, dv = _setup(name)
    got = o.diffusion(c)
    for q in range(c.shape[0]):
        np.testing.assert_array_equal(got[q], pyref.diffusion(geo, c[q], c[0], dh, dv), err_msg=f"component {q}")


@pytest.mark.parametrize("name", ["hill_24x20x16", "flat_walls_9x6x5", "bubble_12x10x8"])
def test_diffusion_known_answers(name):
    """On the cut-cell hill the faces of zero-volume cells are closed first:
    otherwise the zero-volume mask drops what diffuses into such a cell, as the
    reference does."""
    geo, vel, st, o, c, dh, dv = _setup(name, close=True)
    g = geo.grid
    # constant mixing ratio: no diffusion (up to the rounding of c/(Rho+Eps))
    cc = np.stack([c[0], 0.37 * c[0]])
    f = o.diffusion(cc)
    ref = np.abs(o.diffusion(np.stack([c[0], c[-1]]))[1]).max()
    assert np.abs(f[1]).max() <= 1e-12 * ref
    # conservation of the component's total
    f = o.diffusion(c)
    I = (slice(1, -1),) * 3
    for q in range(c.shape[0]):
        tot = f[q][I].sum()
        if g.periodic_x or g.periodic_y or g.periodic_z:
            # the half fluxes deposited in periodic halos belong to the opposite interior cells
            tot = tot + f[q].sum() - f[q][I].sum()
        assert abs(tot) <= 1e-11 * np.abs(f[q][I]).sum(), q


@pytest.mark.parametrize("name", ["hill_24x20x16", "flat_walls_9x6x5"])
def test_diffusion_jacobian_linearises_operator(name):
    geo, vel, st, o, c, dh, dv = _setup(name)
    g = geo.grid
    zero = tuple(np.zeros_like(v) for v in vel)  # diffusion alone
    beta0, dt = 1.0, 2.0
    val_d = o.jac(c[0], zero, beta0, dt)
    o.set_diffusion(None)
    val_0 = o.jac(c[0], zero, beta0, dt)
    jd = (val_0 - val_d) / (beta0 * dt)  # the diffusion entries of J (off-diagonals and diagonal)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(g.pshape)
    x = o.bound_cond(o.exchange_cell(x[None]))[0]
    o.set_diffusion(dh, dv)
    # J dc from the column-oriented DIA storage, as the stage operator applies
    # it, for the component perturbation dc = x (Rho+Eps), i.e. dphi = x
    rho = c[0]
    dc = x * (rho + 1e-30)
    jx = o.spmv(np.ascontiguousarray(jd), dc).reshape(g.pshape)
    fx = o.diffusion(np.stack([rho, dc]))[1] / (geo.volc + 1e-30)
    I = (slice(2, -2),) * 3  # away from the boundary rows
    live = geo.volc[I] > 0  # the Jacobian has no zero-volume mask: rows of cells without volume differ
    scale = np.abs(fx[I]).max()
    assert np.abs(jx[I] - fx[I])[live].max() <= 1e-10 * scale
