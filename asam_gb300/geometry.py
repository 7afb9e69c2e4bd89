"""Seeded synthetic cut-cell geometry, face velocities and initial states.

ASAM reads face areas and cell volumes from the ``.Weight2`` file written by
its GRID preprocessor (INIT/ReadWeights_Mod.f90:408-1712, cut faces
:671-675/:763-767/:873-877, cut volumes :1148-1152).  No such decks exist for
the workloads here, so this module builds the same arrays from a terrain
height field, in the native Fortran extents of MODULE/Domain_Mod.f90:447-460:

* terrain: one height per column (Gaussian hill + Gaussian-correlated
  roughness), periodic in x and y;
* vertex snapping: a column height within ``snap * dz`` of a level is moved
  onto the level, as GRID/Grid_Mod.f90:17-36 classifies vertices within
  ``distx_coeff`` (default 0.01, GRID/Control_Mod.f90:8) of the surface;
* shaved cells: volume fraction ``clip((z_top - h)/dz, 0, 1)``, lateral face
  open above the higher of the two adjacent columns, horizontal face open
  where the column's terrain lies below it;
* small-cell merge (a rule of this package; the reference has none): a cut
  cell with volume fraction below ``merge`` gives its volume and its lateral
  face areas to the cell above, and its faces are closed.

Halo cells: x/y halos hold the periodic image, z halos (rigid bottom and lid)
have zero volume.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

G = 9.81
CP = 1004.0
RD = 287.0
KAPPA = RD / CP
P0 = 1.0e5


@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: np.ndarray  # (nz,) level thicknesses
    periodic_x: bool = True
    periodic_y: bool = True
    periodic_z: bool = False

    @property
    def zP(self) -> np.ndarray:
        return np.concatenate([[0.0], np.cumsum(self.dz)])

    @property
    def npad(self) -> int:
        return (self.nx + 2) * (self.ny + 2) * (self.nz + 2)

    @property
    def pshape(self) -> tuple[int, int, int]:
        """numpy shape (k, j, i) of a padded cell field (C order = Fortran ix fastest)."""
        return (self.nz + 2, self.ny + 2, self.nx + 2)


@dataclass
class Geometry:
    grid: Grid
    volc: np.ndarray  # (nz+2, ny+2, nx+2)
    fu: np.ndarray  # (nz, ny, nx+3)
    fv: np.ndarray  # (nz, ny+3, nx)
    fw: np.ndarray  # (nz+3, ny, nx)
    h: np.ndarray | None = None  # (ny, nx) terrain heights after snapping
    merged: int = 0
    info: dict = field(default_factory=dict)


def stretched_levels(nz: int, dz_bottom: float, dz_top: float) -> np.ndarray:
    """Geometric level thicknesses from dz_bottom at the surface to dz_top at the lid."""
    if nz == 1:
        return np.array([dz_bottom])
    ratio = (dz_top / dz_bottom) ** (1.0 / (nz - 1))
    return dz_bottom * ratio ** np.arange(nz)


def uniform_levels(nz: int, dz: float) -> np.ndarray:
    return np.full(nz, float(dz))


def gaussian_hill_terrain(grid: Grid, height: float, halfwidth: float, rough_sigma: float = 0.0,
                          rough_corr: float = 2000.0, seed: int = 0, xc: float | None = None,
                          yc: float | None = None) -> np.ndarray:
    """Column heights h[j, i] (interior): hill with h = height/2 at distance halfwidth,
    plus a periodic Gaussian random field of std rough_sigma and correlation length rough_corr."""
    nx, ny = grid.nx, grid.ny
    Lx, Ly = nx * grid.dx, ny * grid.dy
    xc = Lx / 2 if xc is None else xc
    yc = Ly / 2 if yc is None else yc
    x = (np.arange(nx) + 0.5) * grid.dx
    y = (np.arange(ny) + 0.5) * grid.dy
    X, Y = np.meshgrid(x, y)
    r2 = (X - xc) ** 2 + (Y - yc) ** 2
    h = height * np.exp(-np.log(2.0) * r2 / (halfwidth ** 2)) if height > 0 else np.zeros_like(X)
    if rough_sigma > 0:
        rng = np.random.default_rng(seed)
        noise = rng.standard_normal((ny, nx))
        kx = np.fft.fftfreq(nx, d=grid.dx) * 2 * np.pi
        ky = np.fft.fftfreq(ny, d=grid.dy) * 2 * np.pi
        KX, KY = np.meshgrid(kx, ky)
        filt = np.exp(-0.25 * (KX ** 2 + KY ** 2) * rough_corr ** 2)
        field_ = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
        std = field_.std()
        if std > 0:
            field_ *= rough_sigma / std
        h = h + field_
    return np.maximum(h, 0.0)


def snap_terrain(h: np.ndarray, zP: np.ndarray, dz: np.ndarray, snap: float) -> np.ndarray:
    """Move heights lying within snap*dz of a level onto that level."""
    if snap <= 0:
        return h.copy()
    hs = h.copy()
    idx = np.clip(np.searchsorted(zP, h), 1, len(zP) - 1)
    for cand in (idx - 1, idx):
        cand = np.clip(cand, 0, len(zP) - 1)
        lev = zP[cand]
        thick = dz[np.clip(cand, 0, len(dz) - 1)]
        close = np.abs(h - lev) < snap * thick
        hs = np.where(close, lev, hs)
    return hs


def cut_cell_geometry(grid: Grid, h: np.ndarray | None = None, snap: float = 0.01, merge: float = 0.1) -> Geometry:
    """Face areas and volumes (native Fortran extents) for terrain h[j,i] (None = flat)."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    dx, dy, dz = grid.dx, grid.dy, np.asarray(grid.dz, dtype=np.float64)
    zP = grid.zP
    if h is None:
        h = np.zeros((ny, nx))
    h = snap_terrain(np.asarray(h, dtype=np.float64), zP, dz, snap)
    # heights on columns -2..nx+1 (x) and -2..ny+1 (y), periodic wrap
    hp = np.pad(h, ((2, 2), (2, 2)), mode="wrap")  # hp[j+2, i+2] = h of interior column (i,j) 0-based

    # volume fraction of interior cells vf[k, j, i]
    ztop = zP[1:][:, None, None]
    vfrac = np.clip((ztop - h[None, :, :]) / dz[:, None, None], 0.0, 1.0)
    # x faces: native FU(ix0-1:ix1+1): face index f=-1..nx+1 between padded cells f and f+1,
    # i.e. between interior columns f-1 and f (0-based); heights hp[:, f+1] and hp[:, f+2]
    fi = np.arange(-1, nx + 2)
    hl = hp[2:ny + 2, fi + 1]
    hr = hp[2:ny + 2, fi + 2]
    hmax_x = np.maximum(hl, hr)  # (ny, nx+3)
    zlo = zP[:-1][:, None, None]
    zhi = zP[1:][:, None, None]
    fu_open = np.clip(zhi - np.maximum(zlo, hmax_x[None]), 0.0, dz[:, None, None])
    fu = fu_open * dy  # (nz, ny, nx+3)
    fj = np.arange(-1, ny + 2)
    hs_ = hp[fj + 1, 2:nx + 2]
    hn_ = hp[fj + 2, 2:nx + 2]
    hmax_y = np.maximum(hs_, hn_)  # (ny+3, nx)
    fv_open = np.clip(zhi - np.maximum(zlo, hmax_y[None]), 0.0, dz[:, None, None])
    fv = fv_open * dx  # (nz, ny+3, nx)
    # z faces: native FW(iz0-1:iz1+1): face kf=-1..nz+1 at height zP[kf] (clamped)
    kf = np.arange(-1, nz + 2)
    zf = zP[np.clip(kf, 0, nz)]
    fw = np.where(h[None, :, :] <= zf[:, None, None], dx * dy, 0.0)
    fw = np.broadcast_to(fw, (nz + 3, ny, nx)).copy()

    vol_full = dx * dy * dz[:, None, None]
    vol = vfrac * vol_full
    merged = 0
    if merge > 0:
        small = (vfrac > 0.0) & (vfrac < merge)
        ks, js, is_ = np.nonzero(small)
        def twins(native: int, n: int, periodic: bool) -> list[int]:
            # native index f+1 of face f; faces f and f+-n are one face when periodic
            out = [native]
            if periodic:
                out += [t for t in (native - n, native + n) if 0 <= t <= n + 2]
            return out

        for k, j, i in zip(ks, js, is_):
            if k + 1 >= nz:
                continue
            merged += 1
            vol[k + 1, j, i] += vol[k, j, i]
            vol[k, j, i] = 0.0
            # lateral faces of the merged cell move up one level (clipped to the full face)
            for base in (i + 1, i + 2):
                for fidx in twins(base, nx, grid.periodic_x):
                    fu[k + 1, j, fidx] = min(fu[k + 1, j, fidx] + fu[k, j, fidx], dy * dz[k + 1])
                    fu[k, j, fidx] = 0.0
            for base in (j + 1, j + 2):
                for fidx in twins(base, ny, grid.periodic_y):
                    fv[k + 1, fidx, i] = min(fv[k + 1, fidx, i] + fv[k, fidx, i], dx * dz[k + 1])
                    fv[k, fidx, i] = 0.0
            # horizontal face between the merged cell and the cell above (native index k+2)
            fw[k + 2, j, i] = 0.0

    volc = np.zeros(grid.pshape)
    volc[1:nz + 1, 1:ny + 1, 1:nx + 1] = vol
    _fill_halo_xy(volc, grid)
    geo = Geometry(grid=grid, volc=volc, fu=np.ascontiguousarray(fu), fv=np.ascontiguousarray(fv),
                   fw=np.ascontiguousarray(fw), h=h, merged=merged)
    full = dx * dy * dz[:, None, None]
    frac = vol / full
    geo.info = {
        "cut_cells": int(np.count_nonzero((frac > 0) & (frac < 1))),
        "dead_cells": int(np.count_nonzero(frac == 0)),
        "merged": merged,
        "min_live_fraction": float(frac[frac > 0].min()) if np.any(frac > 0) else 0.0,
    }
    return geo


def _fill_halo_xy(a: np.ndarray, grid: Grid) -> None:
    """Periodic halo images in x and y of a padded (k, j, i) field (all k)."""
    nx, ny = grid.nx, grid.ny
    if grid.periodic_x:
        a[:, :, 0] = a[:, :, nx]
        a[:, :, nx + 1] = a[:, :, 1]
    if grid.periodic_y:
        a[:, 0, :] = a[:, ny, :]
        a[:, ny + 1, :] = a[:, 1, :]


def close_dead_faces(geo: Geometry) -> Geometry:
    """Close every face of an interior cell with zero volume (in place).

    Snapping the terrain onto a level can leave the face that lies on the
    ground surface open (h == zf) above a cell of zero volume.  The transport
    never carries flux through it, but the pressure projection would couple
    the live cell above to a cell with no volume; a consistent cut-cell
    geometry has all faces of a zero-volume cell closed.
    """
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    dead = geo.volc[1:nz + 1, 1:ny + 1, 1:nx + 1] <= 0.0
    k, j, i = np.nonzero(dead)
    # native index f+1 of face f (west face of interior cell i+1 has FU index i);
    # on a periodic axis faces f and f+-n are one face, stored twice
    for base in (i + 1, i + 2):
        for shift in ((-nx, 0, nx) if g.periodic_x else (0,)):
            t = base + shift
            ok = (t >= 0) & (t <= nx + 2)
            geo.fu[k[ok], j[ok], t[ok]] = 0.0
    for base in (j + 1, j + 2):
        for shift in ((-ny, 0, ny) if g.periodic_y else (0,)):
            t = base + shift
            ok = (t >= 0) & (t <= ny + 2)
            geo.fv[k[ok], t[ok], i[ok]] = 0.0
    geo.fw[k + 1, j, i] = 0.0
    geo.fw[k + 2, j, i] = 0.0
    geo.info["dead_cells_closed"] = int(dead.sum())
    return geo


def closed_hill_case(nx: int, ny: int, nz: int, seed: int = 4, height: float = 600.0, halfwidth: float = 800.0,
                     dx: float = 200.0) -> Geometry:
    """Cut-cell Gaussian hill with roughness in a closed box (walls on all six
    sides), stretched levels 50 -> 400 m, snapping and merging; the faces of
    zero-volume cells closed.  The block of the pressure projection."""
    grid = Grid(nx, ny, nz, dx, dx, stretched_levels(nz, 50.0, 400.0), False, False, False)
    h = gaussian_hill_terrain(grid, height, halfwidth, 50.0, 600.0, seed=seed)
    return close_dead_faces(cut_cell_geometry(grid, h, snap=0.01, merge=0.1))


def projection_inputs(geo: Geometry, seed: int = 3, amp: float = 1.0):
    """Seeded inputs of the pressure projection of a block: the sound
    weights of WeightDiagCompute (DTU ~ potential temperature at the faces
    ~300 K, DUT ~ dp/d(rho theta) ~400, DUU = F/(F+Eps), DTT = 1), the cell
    widths, and a face-velocity increment of amplitude amp that vanishes on the
    walls (a periodic side's two copies of one face get equal values).  Returns (weights, dx, dy, dz, (u, v, w)); weights in the order
    DTU, DTV, DTW, DUU, DUV, DUW, DUT, DTT with uF/vF/wF extents and interior
    cell shapes (nz, ny, nx)."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    rng = np.random.default_rng(seed)
    fu = geo.fu[:, :, 1:nx + 2]
    fv = geo.fv[:, 1:ny + 2, :]
    fw = geo.fw[1:nz + 2]
    eps = 1.0e-30
    duu, duv, duw = fu / (fu + eps), fv / (fv + eps), fw / (fw + eps)
    dtu = 300.0 + 5.0 * rng.standard_normal(fu.shape)
    dtv = 300.0 + 5.0 * rng.standard_normal(fv.shape)
    dtw = 300.0 + 5.0 * rng.standard_normal(fw.shape)
    dut = 400.0 + 10.0 * rng.standard_normal((nz, ny, nx))
    dtt = np.ones((nz, ny, nx))
    dx = np.full(nx, g.dx)
    dy = np.full(ny, g.dy)
    dz = np.asarray(g.dz, dtype=np.float64).copy()
    u = amp * rng.standard_normal(fu.shape) * (fu > 0)
    v = amp * rng.standard_normal(fv.shape) * (fv > 0)
    w = amp * rng.standard_normal(fw.shape) * (fw > 0)
    # a periodic side is one face stored twice (first and last): same
    # velocity and weights on both; a closed side has no normal flow
    if g.periodic_x:
        u[:, :, nx] = u[:, :, 0]
        dtu[:, :, nx] = dtu[:, :, 0]
    else:
        u[:, :, 0] = u[:, :, nx] = 0.0
    if g.periodic_y:
        v[:, ny, :] = v[:, 0, :]
        dtv[:, ny, :] = dtv[:, 0, :]
    else:
        v[:, 0, :] = v[:, ny, :] = 0.0
    if g.periodic_z:
        w[nz] = w[0]
        dtw[nz] = dtw[0]
    else:
        w[0] = w[nz] = 0.0
    weights = [np.ascontiguousarray(a) for a in (dtu, dtv, dtw, duu, duv, duw, dut, dtt)]
    return weights, dx, dy, dz, tuple(np.ascontiguousarray(a) for a in (u, v, w))


def boundary_cells(geo: Geometry) -> np.ndarray:
    """BoundCell list of a cut-cell geometry: the live interior cells that hold
    a piece of the terrain surface, i.e. whose opposite face areas differ along
    some axis (the surface closes the difference).  (n, 3) int32 of 1-based
    (ix, iy, iz), x fastest."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    vol = geo.volc[1:nz + 1, 1:ny + 1, 1:nx + 1]
    dif = ((geo.fu[:, :, 1:nx + 1] != geo.fu[:, :, 2:nx + 2]) | (geo.fv[:, 1:ny + 1, :] != geo.fv[:, 2:ny + 2, :]) |
           (geo.fw[1:nz + 1] != geo.fw[2:nz + 2]))
    k, j, i = np.nonzero((vol > 0) & dif)
    return np.ascontiguousarray(np.stack([i + 1, j + 1, k + 1], axis=1).astype(np.int32).reshape(-1, 3))


def closed_face_velocity(geo: Geometry, amp: float, seed: int = 0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Seeded smooth face velocities of a block: amplitude amp, zero on the
    walls and on closed faces, equal on the two copies of a periodic side's
    face.  uF (nz, ny, nx+1), vF (nz, ny+1, nx), wF (nz+1, ny, nx)."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    rng = np.random.default_rng(seed)

    def smooth(shape):
        a = rng.standard_normal(shape)
        for ax in range(3):
            a = (a + np.roll(a, 1, axis=ax) + np.roll(a, -1, axis=ax)) / 3.0
        return a / max(float(np.std(a)), 1e-300)

    fu = geo.fu[:, :, 1:nx + 2]
    fv = geo.fv[:, 1:ny + 2, :]
    fw = geo.fw[1:nz + 2]
    u = amp * smooth(fu.shape) * (fu > 0)
    v = amp * smooth(fv.shape) * (fv > 0)
    w = 0.3 * amp * smooth(fw.shape) * (fw > 0)
    # a periodic side stores one face twice (equal values), a wall has no normal flow
    if g.periodic_x:
        u[:, :, nx] = u[:, :, 0]
    else:
        u[:, :, 0] = u[:, :, nx] = 0.0
    if g.periodic_y:
        v[:, ny, :] = v[:, 0, :]
    else:
        v[:, 0, :] = v[:, ny, :] = 0.0
    w[0] = w[nz] = 0.0
    return tuple(np.ascontiguousarray(a) for a in (u, v, w))


def dyn_case(nx: int, ny: int, nz: int, seed: int = 5, hill: bool = True, moist: bool = False,
             tracer: bool = False, amp: float = 1.0, bubble: float = 2.0, periodic: bool = False):
    """Block for the dynamical core: a cut-cell hill (or flat ground) in a box
    with six walls (periodic=True: periodic in x and y, rigid bottom and lid),
    a stratified (N=0.01) state with a warm bubble, seeded face velocities of
    amplitude amp that vanish on the walls.
    Returns (geo, (uF, vF, wF), state, positions, (dx, dy, dz), boundary cells);
    positions maps rho, mom (uL,uR,vL,vR,wL,wR), th, qv, tracer to components."""
    if hill:
        if periodic:
            grid = Grid(nx, ny, nz, 200.0, 200.0, stretched_levels(nz, 50.0, 400.0), True, True, False)
            h = gaussian_hill_terrain(grid, 600.0, 800.0, 50.0, 600.0, seed=seed)
            geo = close_dead_faces(cut_cell_geometry(grid, h, snap=0.01, merge=0.1))
        else:
            geo = closed_hill_case(nx, ny, nz, seed=seed)
    else:
        grid = Grid(nx, ny, nz, 200.0, 200.0, stretched_levels(nz, 50.0, 400.0), periodic, periodic, False)
        geo = cut_cell_geometry(grid, None, snap=0.0, merge=0.0)
    g = geo.grid
    vel = closed_face_velocity(geo, amp, seed=seed + 1)
    st = initial_state(geo, *vel, theta0=300.0, n_bv=0.01, bubble_amp=bubble, bubble_radius=600.0,
                       bubble_z=min(1000.0, 0.3 * float(g.zP[-1])), moist=moist, tracer=tracer, momentum=True,
                       seed=seed + 2)
    pos = {"rho": 0, "mom": [1, 2, 3, 4, 5, 6], "th": 7}
    if moist:
        pos["qv"] = 8
    if tracer:
        pos["tracer"] = 8 + int(moist)
    widths = (np.full(g.nx, g.dx), np.full(g.ny, g.dy), np.asarray(g.dz, dtype=np.float64).copy())
    return geo, vel, st, pos, widths, boundary_cells(geo)


def diffusion_coefficients(geo: Geometry, rho: np.ndarray, kh: float = 50.0, kv: float = 5.0, seed: int = 0,
                           spread: float = 0.2) -> tuple[np.ndarray, np.ndarray]:
    """Seeded density-weighted eddy diffusivities (padded cell fields, m^2/s
    times Rho): horizontal kh and vertical kv decaying with height, with a
    seeded relative spread; the halos follow the state's density."""
    g = geo.grid
    rng = np.random.default_rng(seed)
    zc = np.concatenate([[0.0], 0.5 * (g.zP[:-1] + g.zP[1:]), [g.zP[-1]]])
    prof = np.exp(-zc / max(float(g.zP[-1]) * 0.5, 1.0))[:, None, None]
    noise = 1.0 + spread * rng.uniform(-1.0, 1.0, size=g.pshape)
    dh = np.ascontiguousarray(rho * kh * prof * noise)
    dv = np.ascontiguousarray(rho * kv * prof * noise)
    return dh, dv


def face_velocity(geo: Geometry, u0: float, v0: float = 0.0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Prescribed steady face velocities with zero discrete divergence in flux form.

    Every x-face column carries the same volume flux u0*dy*Ztop (so the flow
    speeds up over the hill), every y-face column v0*dx*Ztop; the vertical
    face fluxes follow by integrating the continuity equation up each column
    from the rigid bottom (the lid flux vanishes up to rounding and is set to 0).
    Returns uF (nz, ny, nx+1), vF (nz, ny+1, nx), wF (nz+1, ny, nx).
    """
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    ztop = g.zP[-1]
    fu = geo.fu[:, :, 1:nx + 2]  # faces 0..nx
    fv = geo.fv[:, 1:ny + 2, :]
    su = fu.sum(axis=0)
    sv = fv.sum(axis=0)
    with np.errstate(divide="ignore", invalid="ignore"):
        ucol = np.where(su > 0, u0 * g.dy * ztop / su, 0.0)
        vcol = np.where(sv > 0, v0 * g.dx * ztop / sv, 0.0)
    uf = np.where(fu > 0, ucol[None], 0.0)
    vf = np.where(fv > 0, vcol[None], 0.0)
    fx = uf * fu
    fy = vf * fv
    hdiv = (fx[:, :, 1:] - fx[:, :, :-1]) + (fy[:, 1:, :] - fy[:, :-1, :])  # (nz, ny, nx)
    flux_w = np.zeros((nz + 1, ny, nx))
    flux_w[1:] = -np.cumsum(hdiv, axis=0)
    flux_w[0] = 0.0
    flux_w[nz] = 0.0
    fw = geo.fw[1:nz + 2]  # faces 0..nz
    with np.errstate(divide="ignore", invalid="ignore"):
        wf = np.where(fw > 0, flux_w / fw, 0.0)
    return np.ascontiguousarray(uf), np.ascontiguousarray(vf), np.ascontiguousarray(wf)


def _pad_state(field_: np.ndarray, grid: Grid) -> np.ndarray:
    """Interior (nz,ny,nx) -> padded field: periodic x/y images, z halos copy the adjacent level."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    out = np.zeros(grid.pshape)
    out[1:nz + 1, 1:ny + 1, 1:nx + 1] = field_
    out[0] = out[1]
    out[nz + 1] = out[nz]
    _fill_halo_xy(out, grid)
    return out


def hydrostatic_profile(z: np.ndarray, theta0: float, n_bv: float) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Exner-pressure hydrostatic state of theta(z) = theta0*exp(N^2 z/g) (neutral if N=0).
    Returns (rho, theta, exner)."""
    if n_bv > 0:
        theta = theta0 * np.exp(n_bv ** 2 * z / G)
        exner = 1.0 - G ** 2 / (CP * theta0 * n_bv ** 2) * (1.0 - np.exp(-n_bv ** 2 * z / G))
    else:
        theta = np.full_like(z, theta0)
        exner = 1.0 - G * z / (CP * theta0)
    p = P0 * exner ** (1.0 / KAPPA)
    T = theta * exner
    rho = p / (RD * T)
    return rho, theta, exner


@dataclass
class State:
    names: list[str]
    c: np.ndarray  # (ncomp, nz+2, ny+2, nx+2)
    rho_pos: int = 0


def initial_state(geo: Geometry, uf: np.ndarray, vf: np.ndarray, wf: np.ndarray, *, theta0: float = 300.0,
                  n_bv: float = 0.0, bubble_amp: float = 0.0, bubble_radius: float = 1000.0,
                  bubble_z: float = 1000.0, noise: float = 0.0, moist: bool = False, tracer: bool = False,
                  momentum: bool = True, seed: int = 0) -> State:
    """Cell components of the transport stage: Rho, the six LR momentum
    components (Rho times the face velocity left/right of the cell), Rho*theta,
    and optionally Rho*qv and Rho*tracer."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    rng = np.random.default_rng(seed)
    zc = 0.5 * (g.zP[:-1] + g.zP[1:])
    xc = (np.arange(nx) + 0.5) * g.dx
    yc = (np.arange(ny) + 0.5) * g.dy
    rho1, th1, ex1 = hydrostatic_profile(zc, theta0, n_bv)
    rho = np.broadcast_to(rho1[:, None, None], (nz, ny, nx)).copy()
    theta = np.broadcast_to(th1[:, None, None], (nz, ny, nx)).copy()
    Z, Y, X = np.meshgrid(zc, yc, xc, indexing="ij")
    if bubble_amp != 0.0:
        r2 = (X - nx * g.dx / 2) ** 2 + (Y - ny * g.dy / 2) ** 2 + (Z - bubble_z) ** 2
        theta = theta + bubble_amp * np.exp(-r2 / bubble_radius ** 2)
    if noise > 0:
        theta = theta + rng.uniform(-noise, noise, size=theta.shape)
    names, comps = ["Rho"], [rho]
    if momentum:
        names += ["uL", "uR", "vL", "vR", "wL", "wR"]
        comps += [rho * uf[:, :, :-1], rho * uf[:, :, 1:], rho * vf[:, :-1, :], rho * vf[:, 1:, :],
                  rho * wf[:-1], rho * wf[1:]]
    names.append("RhoTheta")
    comps.append(rho * theta)
    if moist:
        T = theta * ex1[:, None, None]
        rh = np.clip(np.exp(rng.normal(np.log(0.7), 0.15, size=theta.shape)), 0.5, 0.9)
        es = 611.2 * np.exp(17.67 * (T - 273.15) / (T - 29.65))
        p = rho * RD * T
        qv = rh * 0.622 * es / p
        names.append("RhoQv")
        comps.append(rho * qv)
    if tracer:
        cx, cy, cz = nx * g.dx * 0.3, ny * g.dy * 0.5, min(2000.0, g.zP[-1] * 0.3)
        sig = max(2000.0, 4 * g.dx)
        blob = np.exp(-((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) / (2 * sig ** 2))
        blob = blob * (1.0 + 0.01 * rng.standard_normal(blob.shape))
        names.append("RhoTracer")
        comps.append(rho * blob)
    c = np.stack([_pad_state(f, g) for f in comps])
    return State(names=names, c=np.ascontiguousarray(c), rho_pos=0)


# ---------------------------------------------------------------------------
# Named workloads (seeded stand-ins for the benchmark configurations)
# ---------------------------------------------------------------------------
def bubble_case(nx: int = 64, ny: int = 64, nz: int = 64, seed: int = 1):
    """Dry warm bubble on a flat grid: dx=dy=dz=100 m, u=10 m/s, theta0=300 K neutral,
    2 K Gaussian bubble of radius 1 km at 1 km height, U(+-0.01 K) noise."""
    grid = Grid(nx, ny, nz, 100.0, 100.0, uniform_levels(nz, 100.0))
    geo = cut_cell_geometry(grid, None, snap=0.0, merge=0.0)
    uf, vf, wf = face_velocity(geo, 10.0, 0.0)
    st = initial_state(geo, uf, vf, wf, theta0=300.0, n_bv=0.0, bubble_amp=2.0, bubble_radius=1000.0,
                       bubble_z=1000.0, noise=0.01, seed=seed)
    return geo, (uf, vf, wf), st


def bubble_dyn_case(nx: int = 64, ny: int = 64, nz: int = 64, seed: int = 1):
    """The warm bubble with prognostic momentum for the dynamical core:
    bubble_case's grid (periodic x/y, rigid bottom and lid, no orography,
    dx=dy=dz=100 m), state and u=10 m/s face velocities.  Returns (geo,
    (uF, vF, wF), state, positions, (dx, dy, dz), boundary cells) like
    dyn_case; a flat grid has no boundary cells."""
    geo, vel, st = bubble_case(nx, ny, nz, seed=seed)
    g = geo.grid
    pos = {"rho": 0, "mom": [1, 2, 3, 4, 5, 6], "th": 7}
    widths = (np.full(g.nx, g.dx), np.full(g.ny, g.dy), np.asarray(g.dz, dtype=np.float64).copy())
    return geo, vel, st, pos, widths, boundary_cells(geo)


def hill_dyn_case(nx: int = 512, ny: int = 512, nz: int = 128, seed: int = 3, dx: float = 200.0,
                  height: float = 1000.0, halfwidth: float = 5000.0, u0: float = 10.0, n_bv: float = 0.01):
    """The cut-cell hill of hill_case for the dynamical core: periodic in x and
    y, rigid bottom and lid, dx=dy=200 m, dz 50->400 m, Gaussian hill with
    correlated roughness, snapping and the small-cell merge, the faces of
    zero-volume cells closed (the pressure system needs them closed);
    stratified (N), moist, one tracer, u=10 m/s.  Returns (geo, (uF, vF, wF),
    state, positions, (dx, dy, dz), boundary cells) like dyn_case."""
    grid = Grid(nx, ny, nz, dx, dx, stretched_levels(nz, 50.0, 400.0))
    h = gaussian_hill_terrain(grid, height, halfwidth, 50.0, 2000.0, seed=seed)
    geo = close_dead_faces(cut_cell_geometry(grid, h, snap=0.01, merge=0.1))
    uf, vf, wf = face_velocity(geo, u0, 0.0)
    st = initial_state(geo, uf, vf, wf, theta0=300.0, n_bv=n_bv, moist=True, tracer=True, momentum=True, noise=0.0,
                       seed=seed + 100)
    g = geo.grid
    pos = {"rho": 0, "mom": [1, 2, 3, 4, 5, 6], "th": 7, "qv": 8, "tracer": 9}
    widths = (np.full(g.nx, g.dx), np.full(g.ny, g.dy), np.asarray(g.dz, dtype=np.float64).copy())
    return geo, (uf, vf, wf), st, pos, widths, boundary_cells(geo)


def hill_case(nx: int = 256, ny: int = 256, nz: int = 128, seed: int = 2, dx: float = 200.0,
              dz_bottom: float = 50.0, dz_top: float = 400.0, height: float = 1000.0, halfwidth: float = 5000.0,
              rough_sigma: float = 50.0, rough_corr: float = 2000.0, u0: float = 10.0, n_bv: float = 0.01,
              moist: bool = True, tracer: bool = True, momentum: bool = True):
    """Cut-cell Gaussian hill with correlated roughness, stretched levels, snapping and
    the small-cell merge; stratified (N), moist (qv from clipped lognormal RH) with a tracer blob."""
    grid = Grid(nx, ny, nz, dx, dx, stretched_levels(nz, dz_bottom, dz_top))
    h = gaussian_hill_terrain(grid, height, halfwidth, rough_sigma, rough_corr, seed=seed)
    geo = cut_cell_geometry(grid, h, snap=0.01, merge=0.1)
    uf, vf, wf = face_velocity(geo, u0, 0.0)
    st = initial_state(geo, uf, vf, wf, theta0=300.0, n_bv=n_bv, moist=moist, tracer=tracer, momentum=momentum,
                       noise=0.0, seed=seed + 100)
    return geo, (uf, vf, wf), st
