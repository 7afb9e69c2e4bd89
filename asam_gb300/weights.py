"""Cut-cell geometry files (``<case>.Weight2``) of the GRID preprocessor.

Writer of ``WriteWeightBlk`` (GRID/OutputWeightBlk_Mod.f90:501-670) and reader
of ``ReadWeights`` (INIT/ReadWeights_Mod.f90:568-1330) for Cartesian grids,
the geometry data contract of the transport and dynamical stages: per block
the origin, the cell widths, the face areas FU/FV/FW, the cell volumes VolC,
the cut-face midpoints and the boundary-cell list with its surface data.

The file is Fortran list-directed text.  Per block, after the grid type and
the block count:

  ``#.... Block ib ....``; ``x0 y0 z0``; ``nx`` and nx widths dx; ny, dy; nz, dz;
  ``NrW_FacesYZ`` then that many ``ix iy iz`` / ``FU`` pairs (FU over
  ix0-1:ix1+1), ``NrMP_FacesYZ`` then ``ix iy iz`` / ``xS yS zS`` pairs;
  the same for FV (ZX) and FW (XY); ``NrW_Cells`` then ``ix iy iz`` / ``VolC``;
  ``NrB_Cells  Struct_Bound`` then per boundary cell ``ix iy iz`` / ``xS yS zS``
  / ``zRauh alb ee xFLS yFLS zFLS`` (Struct_Bound 0-3), followed on the same
  READ by the soil types of every soil layer (4), the land class (5), or the
  land class and the soil types (6).

Every weight not listed keeps the reader's Cartesian default
(ReadWeights_Mod.f90:633-640, 893-940): full faces dy*dz, dx*dz, dx*dy over
the whole face range; VolC = 1, interior cells dx*dy*dz, the halo layer
beside a face of the block dxLoc*dy*dz with dxLoc the width of the periodic
partner's last cell (periodic side) or of the block's own first cell (outer
wall).  The writer lists exactly the weights that differ from that default,
so a written and re-read geometry is bit-identical (values are written as
the shortest decimal that reads back to the same double).

Index mapping of a single block with ix0 = iy0 = iz0 = 0 onto the library's
arrays: ``FU(ix,iy,iz)`` = ``fu[iz-1, iy-1, ix+1]``, ``FV(ix,iy,iz)`` =
``fv[iz-1, iy+1, ix-1]``, ``FW(ix,iy,iz)`` = ``fw[iz+1, iy-1, ix-1]``,
``VolC(ix,iy,iz)`` = ``volc[iz, iy, ix]``.

Globe and Cyl grids (spherical and cylindrical face and volume formulas) and
multi-block neighbour halos are not read: the reader refuses them.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

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


def _fmt(v: float) -> str:
    r = repr(float(v))
    return r.upper() if ("e" in r or "E" in r) else r


# ---------------------------------------------------------------- defaults
def default_weights(dx, dy, dz, periodic=(True, True, False)):
    """The reader's Cartesian weights before the file's lists are applied:
    fu (nz, ny, nx+3), fv (nz, ny+3, nx), fw (nz+3, ny, nx), volc (nz+2, ny+2, nx+2)."""
    dx, dy, dz = (np.asarray(a, dtype=np.float64) for a in (dx, dy, dz))
    nx, ny, nz = dx.size, dy.size, dz.size
    fu = np.broadcast_to((dz[:, None] * dy[None, :])[:, :, None], (nz, ny, nx + 3)).copy()
    fv = np.broadcast_to((dz[:, None] * dx[None, :])[:, None, :], (nz, ny + 3, nx)).copy()
    fw = np.broadcast_to((dy[:, None] * dx[None, :])[None, :, :], (nz + 3, ny, nx)).copy()
    volc = np.ones((nz + 2, ny + 2, nx + 2))
    volc[1:-1, 1:-1, 1:-1] = dx[None, None, :] * dy[None, :, None] * dz[:, None, None]
    px, py, pz = periodic
    # ReadWeights_Mod.f90:905-1000: dxLoc*dy*dz beside each face of the block
    dxw, dxe = (dx[-1], dx[0]) if px else (dx[0], dx[-1])
    dyS, dyN = (dy[-1], dy[0]) if py else (dy[0], dy[-1])
    dzb, dzt = (dz[-1], dz[0]) if pz else (dz[0], dz[-1])
    volc[1:-1, 1:-1, 0] = dxw * dy[None, :] * dz[:, None]
    volc[1:-1, 1:-1, -1] = dxe * dy[None, :] * dz[:, None]
    volc[1:-1, 0, 1:-1] = dyS * dx[None, :] * dz[:, None]
    volc[1:-1, -1, 1:-1] = dyN * dx[None, :] * dz[:, None]
    volc[0, 1:-1, 1:-1] = dzb * dx[None, :] * dy[:, None]
    volc[-1, 1:-1, 1:-1] = dzt * dx[None, :] * dy[:, None]
    return fu, fv, fw, volc


# index tables: array axis (k, j, i) -> Fortran (ix, iy, iz) offsets
_OFF = {"fu": (-1, 1, 1), "fv": (1, -1, 1), "fw": (1, 1, -1), "volc": (0, 0, 0)}


def _entries(name, arr, ref):
    k, j, i = np.nonzero(arr != ref)
    ox, oy, oz = _OFF[name]
    return np.stack([i + ox, j + oy, k + oz], axis=1), arr[k, j, i]


def _place(name, arr, ijk, vals):
    ox, oy, oz = _OFF[name]
    i, j, k = ijk[:, 0] - ox, ijk[:, 1] - oy, ijk[:, 2] - oz
    if (i < 0).any() or (j < 0).any() or (k < 0).any() or (k >= arr.shape[0]).any() or \
            (j >= arr.shape[1]).any() or (i >= arr.shape[2]).any():
        raise ValueError(f"Weight2: {name} index outside the block")
    arr[k, j, i] = vals


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


def _pairs(ijk: np.ndarray, vals: np.ndarray) -> list[str]:
    """Lines ``ix iy iz`` / ``value`` for every entry (the shortest decimal
    that reads back to the same double)."""
    return [f" {x} {y} {z}\n {v!r}" for x, y, z, v in
            zip(ijk[:, 0].tolist(), ijk[:, 1].tolist(), ijk[:, 2].tolist(), vals.tolist())]


def write_weight2(path, blocks, grid_type: str = "Cart", periodic=(True, True, False)) -> None:
    """blocks: list of Geometry, or of (Geometry, origin, BoundCells|None)."""
    if grid_type != "Cart":
        raise NotImplementedError("Weight2 writer: Cartesian grids only")
    out = [f" {grid_type}", f" {len(blocks)}  ! Number of blocks"]
    for ib, b in enumerate(blocks, start=1):
        geo, origin, bound = (b, (0.0, 0.0, 0.0), None) if isinstance(b, Geometry) else b
        g = geo.grid
        bound = bound if bound is not None else surface_data(geo)
        dx, dy, dz = np.full(g.nx, g.dx), np.full(g.ny, g.dy), np.asarray(g.dz, dtype=np.float64)
        out.append(f" #.... Block {ib} .....................................................")
        out.append(" " + " ".join(_fmt(v) for v in origin))
        for n, d in ((g.nx, dx), (g.ny, dy), (g.nz, dz)):
            out.append(f" {n}")
            out += [" " + _fmt(v) for v in d]
        ref = default_weights(dx, dy, dz, periodic)
        for name, arr, r, tag in (("fu", geo.fu, ref[0], "YZ"), ("fv", geo.fv, ref[1], "ZX"),
                                  ("fw", geo.fw, ref[2], "XY")):
            ijk, vals = _entries(name, arr, r)
            out.append(f" {len(vals)}   NrW_Faces{tag}")
            out += _pairs(ijk, vals)
            out.append(f" 0   NrMP_Faces{tag}")
        ijk, vals = _entries("volc", geo.volc, ref[3])
        out.append(f" {len(vals)}    NrW_Cells")
        out += _pairs(ijk, vals)
        sb = bound.struct_bound
        nsoil = bound.soil_type.shape[1] if sb in (4, 6) else 0
        out.append(f"{len(bound.ijk):12d}      NrB_Cells{sb:6d}   Struct_Bound{nsoil:6d}  Nr_SoilLayers")
        for q, (t, xs, s) in enumerate(zip(bound.ijk.tolist(), bound.xs.tolist(), bound.surf.tolist())):
            out.append(" {} {} {}".format(*t))
            out.append(" " + " ".join(_fmt(v) for v in xs))
            extra = []
            if sb in (5, 6):
                extra.append(str(int(bound.land_class[q])))
            if sb in (4, 6):
                extra += [str(int(v)) for v in bound.soil_type[q]]
            out.append(" " + " ".join([_fmt(v) for v in s] + extra))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


# ---------------------------------------------------------------- reader
class _ListReader:
    """Fortran list-directed READ: each READ starts on a new record (line),
    takes values across lines as needed and drops the rest of its last line;
    ``r*c`` repeats, ``D`` exponents, commas and a ``/`` terminator."""

    def __init__(self, lines):
        self.lines = lines
        self.pos = 0

    def line(self) -> str:
        if self.pos >= len(self.lines):
            raise ValueError("Weight2: unexpected end of file")
        s = self.lines[self.pos]
        self.pos += 1
        return s

    def values(self, n: int) -> list[str]:
        vals: list[str] = []
        while len(vals) < n:
            for tok in self.line().replace(",", " ").split():
                if tok.startswith("/"):
                    break
                if "*" in tok and tok.split("*", 1)[0].isdigit():
                    r, c = tok.split("*", 1)
                    vals += [c] * int(r)
                else:
                    vals.append(tok)
            else:
                continue
            break
        if len(vals) < n:
            raise ValueError("Weight2: list-directed read terminated early")
        return vals[:n]

    def records(self, n: int, nint: int, nreal: int):
        """n pairs of READs, ``nint`` integers on one line and ``nreal`` reals on
        the next: (n, nint) int64 and (n, nreal) float64.  Bulk-parsed when the
        2n lines hold exactly those values (the writers' layout), else read
        READ by READ."""
        lines = self.lines[self.pos:self.pos + 2 * n]
        if len(lines) == 2 * n and n > 0:
            chunk = " ".join(lines)
            if "*" not in chunk and "/" not in chunk and "," not in chunk and len(lines[0].split()) == nint:
                tok = chunk.replace("D", "E").replace("d", "e").split()
                if len(tok) == n * (nint + nreal):
                    try:
                        a = np.array(tok, dtype=np.float64).reshape(n, nint + nreal)
                    except ValueError:
                        a = None
                    if a is not None and np.all(a[:, :nint] == np.round(a[:, :nint])):
                        self.pos += 2 * n
                        return a[:, :nint].astype(np.int64), np.ascontiguousarray(a[:, nint:])
        ijk = np.zeros((n, nint), dtype=np.int64)
        vals = np.zeros((n, nreal))
        for i in range(n):
            ijk[i] = self.ints(nint)
            vals[i] = self.reals(nreal)
        return ijk, vals

    def ints(self, n: int) -> list[int]:
        return [int(v) for v in self.values(n)]

    def reals(self, n: int) -> list[float]:
        return [float(v.replace("D", "E").replace("d", "e")) for v in self.values(n)]


def read_weight2(path, ib: int = 1, periodic=(True, True, False), expect=None,
                 nr_soil_layers: int = NR_SOIL_LAYERS, land_class_def: int = LAND_CLASS_DEF,
                 real_island: bool = False) -> WeightBlock:
    """ReadWeights for block ib (1-based) of a Cartesian file.  expect =
    (nx, ny, nz) checks the extents like the reference's 'Error WeightFile'
    stops.  nr_soil_layers (the grid deck's #NrSoilLayers), land_class_def
    (LandClassDef) and real_island (RealIsland) are the model inputs the
    boundary cells' land and soil classes depend on."""
    with open(path) as f:
        rd = _ListReader(f.read().splitlines())
    grid_type = rd.values(1)[0].strip("'\"")
    if grid_type != "Cart":
        raise NotImplementedError(f"Weight2 reader: grid type {grid_type!r} (Cartesian grids only)")
    nb = rd.ints(1)[0]
    if not 1 <= ib <= nb:
        raise ValueError(f"Weight2: block {ib} of {nb}")
    while True:
        s = rd.line()
        at = s.find("#.... Block")
        if at >= 0 and int(s[at + len("#.... Block"):].split()[0]) == ib:
            break
    origin = tuple(rd.reals(3))
    d = []
    for axis in "xyz":
        n = rd.ints(1)[0]
        if expect is not None and n != expect["xyz".index(axis)]:
            raise ValueError(f"Error WeightFile (n{axis})")
        d.append(np.array([rd.reals(1)[0] for _ in range(n)]))
    dx, dy, dz = d
    fu, fv, fw, volc = default_weights(dx, dy, dz, periodic)
    mids = []
    for name, arr in (("fu", fu), ("fv", fv), ("fw", fw)):
        ijk, vals = rd.records(rd.ints(1)[0], 3, 1)
        _place(name, arr, ijk, vals[:, 0])
        mi, mx = rd.records(rd.ints(1)[0], 3, 3)
        mids.append((mi.astype(np.int32), mx))
    ijk, vals = rd.records(rd.ints(1)[0], 3, 1)
    _place("volc", volc, ijk, vals[:, 0])
    head = rd.values(3)
    nbc, sb = int(head[0]), int(head[2])
    if sb not in range(7):
        raise NotImplementedError(f"Weight2 reader: Struct_Bound {sb}")
    bi, bx, bs = np.zeros((nbc, 3), dtype=np.int32), np.zeros((nbc, 3)), np.zeros((nbc, 6))
    land = np.full(nbc, land_class_def, dtype=np.int32)
    soil = np.zeros((nbc, nr_soil_layers), dtype=np.int32)
    # ReadWeights_Mod.f90:1236-1279: what follows the six surface values, and
    # the roughness and land class each Struct_Bound implies
    ntail = {4: nr_soil_layers, 5: 1, 6: 1 + nr_soil_layers}.get(sb, 0)
    for i in range(nbc):
        bi[i] = rd.ints(3)
        bx[i] = rd.reals(3)
        v = rd.values(6 + ntail)
        bs[i] = [float(t.replace("D", "E").replace("d", "e")) for t in v[:6]]
        tail = [int(t) for t in v[6:]]
        if sb == 4:
            soil[i] = tail
            bs[i, 0] = 0.05
        elif sb == 5:
            land[i] = LAND_CLASS_SEA  # only the sea class is read
            bs[i, 0] = ZROUGH[land[i]]
        elif sb == 6:
            land[i] = tail[0]
            soil[i] = tail[1:]
            bs[i, 0] = ZROUGH[land[i]]
        else:
            soil[i, -1] = 5
    nx, ny, nz = dx.size, dy.size, dz.size
    if real_island:  # a boundary cell with a full volume is an island in the sea
        vol = volc[bi[:, 2], bi[:, 1], bi[:, 0]]
        full = vol >= dx[bi[:, 0] - 1] * dy[bi[:, 1] - 1] * dz[bi[:, 2] - 1] * 0.9999
        land[full] = LAND_CLASS_SEA
    if not (np.all(dx == dx[0]) and np.all(dy == dy[0])):
        raise NotImplementedError("Weight2 reader: the library's grids have uniform dx and dy")
    geo = Geometry(grid=Grid(nx=nx, ny=ny, nz=nz, dx=float(dx[0]), dy=float(dy[0]), dz=dz.copy(),
                             periodic_x=periodic[0], periodic_y=periodic[1], periodic_z=periodic[2]),
                   volc=volc, fu=fu, fv=fv, fw=fw)
    bound = BoundCells(ijk=bi, xs=bx, surf=bs, struct_bound=sb, land_class=land, soil_type=soil)
    bound.normal, bound.fl, bound.dl = _normals(geo, dx, dy, dz, bi)
    return WeightBlock(geo=geo, origin=origin, dx=dx, dy=dy, dz=dz, mid_faces=tuple(mids), bound=bound)


def _normals(geo, dx, dy, dz, ijk):
    """Surface normal, area and wall distance of each boundary cell
    (ReadWeights_Mod.f90:1283-1319)."""
    i, j, k = ijk[:, 0].astype(np.int64), ijk[:, 1].astype(np.int64), ijk[:, 2].astype(np.int64)
    fuR, fuL = geo.fu[k - 1, j - 1, i + 1], geo.fu[k - 1, j - 1, i]
    fvR, fvL = geo.fv[k - 1, j + 1, i - 1], geo.fv[k - 1, j, i - 1]
    fwR, fwL = geo.fw[k + 1, j - 1, i - 1], geo.fw[k, j - 1, i - 1]
    ddx, ddy, ddz = dx[i - 1], dy[j - 1], dz[k - 1]
    n1 = np.where((fuR == 0) & (fuL == 0), ddy * ddz * 2.0, fuR - fuL)
    n2 = np.where((fvR == 0) & (fvL == 0), ddx * ddz * 2.0, fvR - fvL)
    n3 = np.where((fwR == 0) & (fwL == 0), ddx * ddy * 2.0, fwR - fwL)
    fl = np.sqrt(n1 * n1 + n2 * n2 + n3 * n3)
    pos = fl > 0
    with np.errstate(invalid="ignore", divide="ignore"):
        n = np.where(pos[:, None], np.stack([n1, n2, n3], axis=1) / fl[:, None], [0.0, 0.0, 1.0])
    fl = np.where(pos, fl, 1e-10)
    dl = 0.5 * np.sqrt((n[:, 0] * ddx) ** 2 + (n[:, 1] * ddy) ** 2 + (n[:, 2] * ddz) ** 2)
    return n, fl, dl
