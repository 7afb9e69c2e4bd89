"""Small seeded cases shared by the tests (sizes the oracle finishes in seconds)."""
from __future__ import annotations

import functools

import numpy as np

from asam_gb300 import geometry as G


def _flat(nx, ny, nz, u0=10.0, v0=0.0, per_x=True, per_y=True, seed=1):
    grid = G.Grid(nx, ny, nz, 100.0, 100.0, G.uniform_levels(nz, 100.0), per_x, per_y, False)
    geo = G.cut_cell_geometry(grid, None, snap=0.0, merge=0.0)
    vel = G.face_velocity(geo, u0, v0)
    if not per_x:
        vel[0][:, :, 0] = 0.0
        vel[0][:, :, -1] = 0.0
    if not per_y:
        vel[1][:, 0, :] = 0.0
        vel[1][:, -1, :] = 0.0
    st = G.initial_state(geo, *vel, theta0=300.0, bubble_amp=2.0, bubble_radius=400.0, bubble_z=500.0, noise=0.01,
                         seed=seed)
    return geo, vel, st


def _hill(nx, ny, nz, u0=10.0, v0=0.0, seed=2, height=600.0, halfwidth=800.0):
    grid = G.Grid(nx, ny, nz, 200.0, 200.0, G.stretched_levels(nz, 50.0, 400.0))
    h = G.gaussian_hill_terrain(grid, height, halfwidth, 50.0, 600.0, seed=seed)
    geo = G.cut_cell_geometry(grid, h, snap=0.01, merge=0.1)
    vel = G.face_velocity(geo, u0, v0)
    st = G.initial_state(geo, *vel, theta0=300.0, n_bv=0.01, moist=True, tracer=True, seed=seed + 7)
    return geo, vel, st


def _channel(nx, ny, nz, u0=6.0, v0=1.5, seed=11):
    """Flat block with outer walls on all sides and flow through them: inflow
    on the west, outflow on the east, and face velocities of both signs on
    the south/north walls, the ground and the lid (the open boundaries of
    AdvectionComputeP and the InFlowOutFlow rule)."""
    grid = G.Grid(nx, ny, nz, 100.0, 100.0, G.uniform_levels(nz, 100.0), False, False, False)
    geo = G.cut_cell_geometry(grid, None, snap=0.0, merge=0.0)
    uf, vf, wf = (a.copy() for a in G.face_velocity(geo, u0, v0))
    rng = np.random.default_rng(seed)
    uf *= 1.0 + 0.2 * rng.standard_normal(uf.shape)
    vf[:, 0, :] = 2.0 * rng.standard_normal((nz, nx))
    vf[:, -1, :] = 2.0 * rng.standard_normal((nz, nx))
    wf[0] = 0.5 * rng.standard_normal((ny, nx))
    wf[-1] = 0.5 * rng.standard_normal((ny, nx))
    vel = (uf, vf, wf)
    st = G.initial_state(geo, *vel, theta0=300.0, bubble_amp=2.0, bubble_radius=300.0, bubble_z=300.0, noise=0.01,
                         seed=seed)
    return geo, vel, st


def _hill_closed(nx, ny, nz, seed=4, height=600.0, halfwidth=800.0):
    return G.closed_hill_case(nx, ny, nz, seed=seed, height=height, halfwidth=halfwidth)


def _flat_closed(nx, ny, nz):
    grid = G.Grid(nx, ny, nz, 100.0, 100.0, G.uniform_levels(nz, 100.0), False, False, False)
    return G.cut_cell_geometry(grid, None, snap=0.0, merge=0.0)


def proj_inputs(geo, seed=3, amp=1.0):
    return G.projection_inputs(geo, seed=seed, amp=amp)


def _hill_periodic(nx, ny, nz, seed=4, per_y=True, height=600.0, halfwidth=800.0):
    """Cut-cell hill periodic in x (and y), rigid bottom and lid, the faces of
    zero-volume cells closed: a block with boundary face unknowns."""
    grid = G.Grid(nx, ny, nz, 200.0, 200.0, G.stretched_levels(nz, 50.0, 400.0), True, per_y, False)
    h = G.gaussian_hill_terrain(grid, height, halfwidth, 50.0, 600.0, seed=seed)
    return G.close_dead_faces(G.cut_cell_geometry(grid, h, snap=0.01, merge=0.1))


def _flat_periodic(nx, ny, nz):
    grid = G.Grid(nx, ny, nz, 100.0, 100.0, G.uniform_levels(nz, 100.0), True, True, False)
    return G.cut_cell_geometry(grid, None, snap=0.0, merge=0.0)


PROJ_PERIODIC = {
    "proj_per_hill_16x12x10": lambda: _hill_periodic(16, 12, 10),
    "proj_per_x_hill_13x7x9": lambda: _hill_periodic(13, 7, 9, seed=6, per_y=False),
    "proj_per_flat_12x10x8": lambda: _flat_periodic(12, 10, 8),
    "proj_per_slab_9x1x6": lambda: _flat_periodic(9, 1, 6),
}


PROJ_CASES = {
    "proj_hill_24x20x16": lambda: _hill_closed(24, 20, 16),
    "proj_hill_odd_13x7x9": lambda: _hill_closed(13, 7, 9, seed=6),
    "proj_flat_16x12x10": lambda: _flat_closed(16, 12, 10),
    "proj_column_1x1x12": lambda: _flat_closed(1, 1, 12),
    "proj_slab_9x1x6": lambda: _flat_closed(9, 1, 6),
    **PROJ_PERIODIC,
}


CASES = {
    "channel_open_10x7x6": lambda: _channel(10, 7, 6),
    "bubble_12x10x8": lambda: _flat(12, 10, 8),
    "hill_24x20x16": lambda: _hill(24, 20, 16),
    "hill_odd_13x7x9_reverse": lambda: _hill(13, 7, 9, u0=-7.0, v0=4.0, seed=5),
    "flat_walls_9x6x5": lambda: _flat(9, 6, 5, u0=3.0, v0=-2.0, per_x=False, per_y=False),
    "column_1x1x12": lambda: _flat(1, 1, 12, u0=2.0, v0=1.0),
    "slab_1x9x6": lambda: _hill(1, 9, 6, u0=5.0, v0=-3.0, seed=9),
}


@functools.lru_cache(maxsize=None)
def get(name: str):
    return CASES[name]() if name in CASES else PROJ_CASES[name]()


def relerr(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / max |b| (field-normwise), with a floor for all-zero fields."""
    den = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / den


def field_relerr(a: np.ndarray, b: np.ndarray) -> list[float]:
    return [relerr(a[i], b[i]) for i in range(a.shape[0])]


def state_relerr(a: np.ndarray, b: np.ndarray, mom=()) -> list[float]:
    """Per-field max |a-b| relative to the field's largest magnitude, except
    that the six LR momentum components (indices `mom`) are the Cartesian
    components of one vector field and are measured against the largest
    magnitude among them: a component that is nearly zero everywhere (the
    cross-wind v of a flow along x) would otherwise turn rounding-level
    differences of the Krylov solves into large relative numbers."""
    mom = list(mom)
    vscale = max((float(np.max(np.abs(b[q]))) for q in mom), default=0.0)
    out = []
    for i in range(a.shape[0]):
        den = vscale if i in mom else float(np.max(np.abs(b[i])))
        out.append(float(np.max(np.abs(a[i] - b[i]))) / max(den, 1e-300))
    return out
