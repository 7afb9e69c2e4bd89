"""Cut-cell geometry files (``<case>.Weight2``) of the GRID preprocessor.

Python side of the library's compiled reader and writer (``asam_weight2_*``
in ``include/asam_gb300.h``): ``read_weight2`` is ReadWeights
(INIT/ReadWeights_Mod.f90:568-1330) and ``write_weight2`` is WriteWeightBlk
(GRID/OutputWeightBlk_Mod.f90:501-670) for Cartesian grids, the geometry data
contract of the transport and dynamical stages: per block the origin, the
cell widths, the face areas FU/FV/FW, the cell volumes VolC, the cut-face
midpoints and the boundary-cell list with its surface data, soil types and
land classes.

The file is Fortran list-directed text that lists only the weights that
differ from the reader's Cartesian defaults (full faces, dx*dy*dz volumes,
halo volumes from the periodic partner's or the block's own edge cells);
values are written as the shortest decimal that reads back to the same
double, so a written and re-read block is bit-identical.

Index mapping of a single block with ix0 = iy0 = iz0 = 0 onto the library's
arrays: ``FU(ix,iy,iz)`` = ``fu[iz-1, iy-1, ix+1]``, ``FV(ix,iy,iz)`` =
``fv[iz-1, iy+1, ix-1]``, ``FW(ix,iy,iz)`` = ``fw[iz+1, iy-1, ix-1]``,
``VolC(ix,iy,iz)`` = ``volc[iz, iy, ix]``.

Globe and Cyl grids (spherical and cylindrical face and volume formulas) and
multi-block neighbour halos are not read: the reader refuses them.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .geometry import Geometry, Grid, boundary_cells

# roughness length per land class 0..9 (the zrough table of SOIL/SoilData_Mod.f90:104)
ZROUGH = (0.05, 1.0, 0.15, 1.0, 1.0, 1.0, 0.2, 0.5, 0.03, 0.01)
LAND_CLASS_DEF = 5       # LandClassDef default (MODULE/Physics_Mod.f90:560)
NR_SOIL_LAYERS = 7       # Domain%nrsoillayers default (INIT/Grid_Mod.f90:676)
LAND_CLASS_SEA = 9


@dataclass
class BoundCells:
    """Floor(ib)%BoundCell (ReadWeights_Mod.f90:1190-1320): 1-based indices,
    surface midpoint, surface data and the normal derived from the face
    areas (the Hinneburg rule: a pair of closed opposite faces counts as a
    full area difference)."""
    ijk: np.ndarray  # (n, 3) int32, ix iy iz
    xs: np.ndarray  # (n, 3) xS yS zS
    surf: np.ndarray  # (n, 6) zRauh alb ee xFLS yFLS zFLS
    struct_bound: int = 3
    land_class: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int32))  # LandClass
    soil_type: np.ndarray = field(default_factory=lambda: np.zeros((0, 0), dtype=np.int32))  # SoilType(1:nrsoil)
    normal: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))  # n1 n2 n3
    fl: np.ndarray = field(default_factory=lambda: np.zeros(0))  # FL
    dl: np.ndarray = field(default_factory=lambda: np.zeros(0))  # dL


@dataclass
class WeightBlock:
    geo: Geometry
    origin: tuple[float, float, float]
    dx: np.ndarray  # (nx,)
    dy: np.ndarray  # (ny,)
    dz: np.ndarray  # (nz,)
    mid_faces: tuple  # per axis (n, 3) int32 ijk and (n, 3) midpoints
    bound: BoundCells


# ---------------------------------------------------------------- writer
def surface_data(geo: Geometry, zrauh=0.1, albedo=0.08, emissivity=0.8):
    """Boundary cells of a generated geometry with the GRID writer's surface
    constants (OutputWeightBlk_Mod.f90:518-521): midpoint at the cell centre
    in x, y and at the terrain height (else the cell centre) in z; the cut
    surface's midpoint the same point."""
    g = geo.grid
    ijk = boundary_cells(geo)
    zP = np.concatenate([[0.0], np.cumsum(g.dz)])
    xc = (ijk[:, 0] - 0.5) * g.dx
    yc = (ijk[:, 1] - 0.5) * g.dy
    if geo.h is not None:
        zc = np.clip(geo.h[ijk[:, 1] - 1, ijk[:, 0] - 1], zP[ijk[:, 2] - 1], zP[ijk[:, 2]])
    else:
        zc = 0.5 * (zP[ijk[:, 2] - 1] + zP[ijk[:, 2]])
    xs = np.stack([xc, yc, zc], axis=1)
    surf = np.column_stack([np.full(len(ijk), zrauh), np.full(len(ijk), albedo), np.full(len(ijk), emissivity), xs])
    return BoundCells(ijk=ijk, xs=xs, surf=surf)


def _raise(status: int, where: str) -> None:
    if status == _lib.ASAM_OK:
        return
    msg = f"{where}: " + _lib.load().asam_last_error().decode(errors="replace")
    if status == _lib.ASAM_UNSUPPORTED:
        raise NotImplementedError(msg)
    if status in (_lib.ASAM_IO_ERROR, _lib.ASAM_BAD_ARG):
        raise ValueError(msg)
    raise _lib.AsamError(status, where)


def _f64(a, shape=None, what=""):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != tuple(shape):
        raise ValueError(f"Weight2: {what} has shape {a.shape}, expected {tuple(shape)}")
    return a


def _i32(a, shape=None, what=""):
    a = np.ascontiguousarray(a, dtype=np.int32)
    if shape is not None and a.shape != tuple(shape):
        raise ValueError(f"Weight2: {what} has shape {a.shape}, expected {tuple(shape)}")
    return a


def _addr(a: np.ndarray):
    return a.ctypes.data if a.size else None


def _describe(b, keep: list) -> _lib.AsamWeight2Block:
    """asam_weight2_block of a Geometry, a (Geometry, origin, BoundCells|None)
    tuple or a WeightBlock; the arrays it points to are appended to keep."""
    mids = None
    if isinstance(b, WeightBlock):
        geo, origin, bound, mids = b.geo, b.origin, b.bound, b.mid_faces
        dx, dy, dz = b.dx, b.dy, b.dz
    else:
        geo, origin, bound = (b, (0.0, 0.0, 0.0), None) if isinstance(b, Geometry) else b
        g = geo.grid
        dx, dy, dz = np.full(g.nx, g.dx), np.full(g.ny, g.dy), g.dz
    bound = bound if bound is not None else surface_data(geo)
    nx, ny, nz = len(dx), len(dy), len(dz)
    d = _lib.AsamWeight2Block()
    d.nx, d.ny, d.nz = nx, ny, nz
    d.origin[:] = [float(v) for v in origin]
    arrs = {"dx": _f64(dx, (nx,), "dx"), "dy": _f64(dy, (ny,), "dy"), "dz": _f64(dz, (nz,), "dz"),
            "fu": _f64(geo.fu, (nz, ny, nx + 3), "fu"), "fv": _f64(geo.fv, (nz, ny + 3, nx), "fv"),
            "fw": _f64(geo.fw, (nz + 3, ny, nx), "fw"), "volc": _f64(geo.volc, (nz + 2, ny + 2, nx + 2), "volc")}
    n = len(bound.ijk)
    sb = int(bound.struct_bound)
    nsoil = bound.soil_type.shape[1] if sb in (4, 6) and bound.soil_type.ndim == 2 else 0
    arrs.update(bound_ijk=_i32(bound.ijk, (n, 3), "bound ijk"), bound_xs=_f64(bound.xs, (n, 3), "bound xs"),
                bound_surf=_f64(bound.surf, (n, 6), "bound surf"))
    if sb in (5, 6):
        arrs["land_class"] = _i32(bound.land_class, (n,), "land_class")
    if nsoil:
        arrs["soil_type"] = _i32(bound.soil_type, (n, nsoil), "soil_type")
    for k, a in arrs.items():
        setattr(d, k, _addr(a))
    keep += arrs.values()
    d.nbound, d.struct_bound, d.nsoil = n, sb, nsoil
    for a in range(3):
        if mids is not None and len(mids[a][0]):
            mi = _i32(mids[a][0], (len(mids[a][0]), 3), "midpoint ijk")
            mx = _f64(mids[a][1], (len(mi), 3), "midpoints")
            d.nmid[a], d.mid_ijk[a], d.mid_xs[a] = len(mi), _addr(mi), _addr(mx)
            keep += [mi, mx]
    return d


def write_weight2(path, blocks, grid_type: str = "Cart", periodic=(True, True, False)) -> None:
    """WriteWeightBlk.  blocks: Geometry objects, (Geometry, origin,
    BoundCells|None) tuples (None: the boundary cells of the geometry with
    the GRID writer's surface constants) or WeightBlocks as read."""
    if grid_type != "Cart":
        raise NotImplementedError("Weight2 writer: Cartesian grids only")
    keep: list = []
    descs = (_lib.AsamWeight2Block * len(blocks))(*[_describe(b, keep) for b in blocks])
    per = (C.c_int * 3)(*[int(bool(v)) for v in periodic])
    _raise(_lib.load().asam_weight2_write(os.fsencode(str(path)), len(blocks), descs, per), "asam_weight2_write")


def read_weight2(path, ib: int = 1, periodic=(True, True, False), expect=None,
                 nr_soil_layers: int = NR_SOIL_LAYERS, land_class_def: int = LAND_CLASS_DEF,
                 real_island: bool = False) -> WeightBlock:
    """ReadWeights for block ib (1-based) of a Cartesian file.  expect =
    (nx, ny, nz) checks the extents like the reference's 'Error WeightFile'
    stops.  nr_soil_layers (the grid deck's #NrSoilLayers), land_class_def
    (LandClassDef) and real_island (RealIsland) are the model inputs the
    boundary cells' land and soil classes depend on."""
    lib = _lib.load()
    opt = _lib.AsamWeight2Options()
    opt.periodic[:] = [int(bool(v)) for v in periodic]
    opt.nr_soil_layers, opt.land_class_def, opt.real_island = nr_soil_layers, land_class_def, int(real_island)
    opt.expect[:] = [int(v) for v in expect] if expect is not None else [0, 0, 0]
    info = _lib.AsamWeight2Block()
    h = C.c_void_p()
    _raise(lib.asam_weight2_open(os.fsencode(str(path)), ib, C.byref(opt), C.byref(h), C.byref(info)),
           "asam_weight2_open")
    try:
        nx, ny, nz, n, ns = info.nx, info.ny, info.nz, info.nbound, info.nsoil
        a = dict(dx=np.empty(nx), dy=np.empty(ny), dz=np.empty(nz), fu=np.empty((nz, ny, nx + 3)),
                 fv=np.empty((nz, ny + 3, nx)), fw=np.empty((nz + 3, ny, nx)), volc=np.empty((nz + 2, ny + 2, nx + 2)),
                 bound_ijk=np.empty((n, 3), np.int32), bound_xs=np.empty((n, 3)), bound_surf=np.empty((n, 6)),
                 land_class=np.empty(n, np.int32), soil_type=np.empty((n, ns), np.int32), normal=np.empty((n, 3)),
                 fl=np.empty(n), dl=np.empty(n))
        dst = _lib.AsamWeight2Block()
        for k, v in a.items():
            setattr(dst, k, _addr(v))
        mids = []
        for d in range(3):
            mi, mx = np.empty((info.nmid[d], 3), np.int32), np.empty((info.nmid[d], 3))
            dst.mid_ijk[d], dst.mid_xs[d] = _addr(mi), _addr(mx)
            mids.append((mi, mx))
        _raise(lib.asam_weight2_fetch(h, C.byref(dst)), "asam_weight2_fetch")
    finally:
        lib.asam_weight2_close(h)
    dx, dy, dz = a["dx"], a["dy"], a["dz"]
    if not (np.all(dx == dx[0]) and np.all(dy == dy[0])):
        raise NotImplementedError("Weight2 reader: the library's grids have uniform dx and dy")
    geo = Geometry(grid=Grid(nx=nx, ny=ny, nz=nz, dx=float(dx[0]), dy=float(dy[0]), dz=dz.copy(),
                             periodic_x=bool(periodic[0]), periodic_y=bool(periodic[1]),
                             periodic_z=bool(periodic[2])),
                   volc=a["volc"], fu=a["fu"], fv=a["fv"], fw=a["fw"])
    bound = BoundCells(ijk=a["bound_ijk"], xs=a["bound_xs"], surf=a["bound_surf"], struct_bound=info.struct_bound,
                       land_class=a["land_class"], soil_type=a["soil_type"], normal=a["normal"], fl=a["fl"],
                       dl=a["dl"])
    return WeightBlock(geo=geo, origin=tuple(info.origin), dx=dx, dy=dy, dz=dz, mid_faces=tuple(mids), bound=bound)
