"""Cut-cell geometry files (``<case>.Weight2``): a pure-Python restatement of
ReadWeights (INIT/ReadWeights_Mod.f90:568-1330) and WriteWeightBlk
(GRID/OutputWeightBlk_Mod.f90:501-670) for Cartesian grids.

Test infrastructure only: the tests use it to check the library's compiled
reader and writer; nothing in the product imports it.

Parity pinned only by hand-written files: the reference ships no
``.Weight2`` deck and this image has no Fortran compiler to run its GRID
preprocessor.  The tests hold a file in the writer's layout with every
value known by hand (defaults, listed weights, midpoints, boundary cells
and the normals the reader derives from them).

The file is Fortran list-directed text.  Per block, after the grid type and
the block count (ReadWeights_Mod.f90:571-1280):

  ``#.... Block ib ....``; ``x0 y0 z0``; ``nx`` and nx widths dx; ny, dy; nz, dz;
  ``NrW_FacesYZ`` then that many ``ix iy iz`` / ``FU`` pairs (FU over
  ix0-1:ix1+1), ``NrMP_FacesYZ`` then ``ix iy iz`` / ``xS yS zS`` pairs;
  the same for FV (ZX) and FW (XY); ``NrW_Cells`` then ``ix iy iz`` / ``VolC``;
  ``NrB_Cells  Struct_Bound`` then per boundary cell ``ix iy iz`` / ``xS yS zS``
  / ``zRauh alb ee xFLS yFLS zFLS`` (Struct_Bound 0-3), followed on the same
  READ by the soil types of every soil layer (4), the land class (5), or the
  land class and the soil types (6).

Every weight not listed keeps the reader's Cartesian default
(ReadWeights_Mod.f90:633-640, 893-1000): full faces dy*dz, dx*dz, dx*dy over
the whole face range; VolC = 1, interior cells dx*dy*dz, the halo layer
beside a face of the block dxLoc*dy*dz with dxLoc the width of the periodic
partner's last cell (periodic side) or of the block's own first cell (outer
wall).

Index mapping of a single block with ix0 = iy0 = iz0 = 0 onto numpy arrays
(ix fastest): ``FU(ix,iy,iz)`` = ``fu[iz-1, iy-1, ix+1]``, ``FV(ix,iy,iz)`` =
``fv[iz-1, iy+1, ix-1]``, ``FW(ix,iy,iz)`` = ``fw[iz+1, iy-1, ix-1]``,
``VolC(ix,iy,iz)`` = ``volc[iz, iy, ix]``.

A block is a dict: origin, dx, dy, dz, fu, fv, fw, volc, mids (three
(ijk, xs) pairs), and bound = dict(ijk, xs, surf, struct_bound, land, soil)
plus, from the reader, normal, fl and dl.
"""
from __future__ import annotations

import numpy as np

# roughness length per land class 0..9 (the zrough table of SOIL/SoilData_Mod.f90:104)
ZROUGH = (0.05, 1.0, 0.15, 1.0, 1.0, 1.0, 0.2, 0.5, 0.03, 0.01)
LAND_CLASS_SEA = 9


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
    # dx(jx)*dy(jy)*dzLoc: the product of the widths first (ReadWeights_Mod.f90:962-987)
    volc[0, 1:-1, 1:-1] = dx[None, :] * dy[:, None] * dzb
    volc[-1, 1:-1, 1:-1] = dx[None, :] * dy[:, None] * dzt
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


def _fmt(v: float) -> str:
    r = repr(float(v))
    return r.upper() if ("e" in r or "E" in r) else r


def _pairs(ijk: np.ndarray, vals: np.ndarray) -> list[str]:
    return [f" {x} {y} {z}\n {v!r}" for x, y, z, v in
            zip(ijk[:, 0].tolist(), ijk[:, 1].tolist(), ijk[:, 2].tolist(), vals.tolist())]


def write(path, blocks, periodic=(True, True, False)) -> None:
    """WriteWeightBlk for a list of block dicts: the weights that differ from
    the reader's defaults, each as Python's shortest round-trip decimal."""
    out = [" Cart", f" {len(blocks)}  ! Number of blocks"]
    for ib, b in enumerate(blocks, start=1):
        dx, dy, dz = (np.asarray(b[k], dtype=np.float64) for k in ("dx", "dy", "dz"))
        out.append(f" #.... Block {ib} .....................................................")
        out.append(" " + " ".join(_fmt(v) for v in b["origin"]))
        for d in (dx, dy, dz):
            out.append(f" {d.size}")
            out += [" " + _fmt(v) for v in d]
        ref = default_weights(dx, dy, dz, periodic)
        mids = b.get("mids") or [(np.zeros((0, 3), np.int64), np.zeros((0, 3)))] * 3
        for a, (name, tag) in enumerate((("fu", "YZ"), ("fv", "ZX"), ("fw", "XY"))):
            ijk, vals = _entries(name, b[name], ref[a])
            out.append(f" {len(vals)}   NrW_Faces{tag}")
            out += _pairs(ijk, vals)
            mi, mx = mids[a]
            out.append(f" {len(mi)}   NrMP_Faces{tag}")
            for t, x in zip(np.asarray(mi).tolist(), np.asarray(mx).tolist()):
                out.append(" {} {} {}".format(*t))
                out.append(" " + " ".join(_fmt(v) for v in x))
        ijk, vals = _entries("volc", b["volc"], ref[3])
        out.append(f" {len(vals)}    NrW_Cells")
        out += _pairs(ijk, vals)
        bd = b["bound"]
        sb = bd["struct_bound"]
        soil = np.asarray(bd.get("soil", np.zeros((len(bd["ijk"]), 0), np.int32)))
        nsoil = soil.shape[1] if sb in (4, 6) else 0
        out.append(f"{len(bd['ijk']):12d}      NrB_Cells{sb:6d}   Struct_Bound{nsoil:6d}  Nr_SoilLayers")
        for q, (t, xs, s) in enumerate(zip(np.asarray(bd["ijk"]).tolist(), np.asarray(bd["xs"]).tolist(),
                                           np.asarray(bd["surf"]).tolist())):
            out.append(" {} {} {}".format(*t))
            out.append(" " + " ".join(_fmt(v) for v in xs))
            extra = []
            if sb in (5, 6):
                extra.append(str(int(bd["land"][q])))
            if sb in (4, 6):
                extra += [str(int(v)) for v in soil[q]]
            out.append(" " + " ".join([_fmt(v) for v in s] + extra))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


class ListReader:
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

    def ints(self, n: int) -> list[int]:
        return [int(v) for v in self.values(n)]

    def reals(self, n: int) -> list[float]:
        return [float(v.replace("D", "E").replace("d", "e")) for v in self.values(n)]

    def records(self, n: int, nint: int, nreal: int):
        ijk = np.zeros((n, nint), dtype=np.int64)
        vals = np.zeros((n, nreal))
        for i in range(n):
            ijk[i] = self.ints(nint)
            vals[i] = self.reals(nreal)
        return ijk, vals


def read(path, ib: int = 1, periodic=(True, True, False), expect=None, nr_soil_layers: int = 7,
         land_class_def: int = 5, real_island: bool = False) -> dict:
    """ReadWeights for block ib (1-based) of a Cartesian file."""
    with open(path) as f:
        rd = ListReader(f.read().splitlines())
    grid_type = rd.values(1)[0].strip("'\"")
    if grid_type != "Cart":
        raise NotImplementedError(f"Weight2 reader: grid type {grid_type!r}")
    nb = rd.ints(1)[0]
    if not 1 <= ib <= nb:
        raise ValueError(f"Weight2: block {ib} of {nb}")
    while True:  # ReadWeights_Mod.f90:581-585
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
        mids.append(rd.records(rd.ints(1)[0], 3, 3))
    ijk, vals = rd.records(rd.ints(1)[0], 3, 1)
    _place("volc", volc, ijk, vals[:, 0])
    head = rd.values(3)  # NumBoundCell, Str_Read, nr_structbound (ReadWeights_Mod.f90:1217)
    nbc, sb = int(head[0]), int(head[2])
    if sb not in range(7):
        raise NotImplementedError(f"Weight2 reader: Struct_Bound {sb}")
    bi, bx, bs = np.zeros((nbc, 3), dtype=np.int64), np.zeros((nbc, 3)), np.zeros((nbc, 6))
    land = np.full(nbc, land_class_def, dtype=np.int64)
    soil = np.zeros((nbc, nr_soil_layers), dtype=np.int64)
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
        elif nr_soil_layers > 0:
            soil[i, -1] = 5
    if real_island:  # a boundary cell with a full volume is an island in the sea
        vol = volc[bi[:, 2], bi[:, 1], bi[:, 0]]
        full = vol >= dx[bi[:, 0] - 1] * dy[bi[:, 1] - 1] * dz[bi[:, 2] - 1] * 0.9999
        land[full] = LAND_CLASS_SEA
    normal, fl, dl = normals(fu, fv, fw, dx, dy, dz, bi)
    return dict(origin=origin, dx=dx, dy=dy, dz=dz, fu=fu, fv=fv, fw=fw, volc=volc, mids=mids,
                bound=dict(ijk=bi, xs=bx, surf=bs, struct_bound=sb, land=land, soil=soil, normal=normal, fl=fl,
                           dl=dl))


def normals(fu, fv, fw, dx, dy, dz, ijk):
    """Surface normal, area and wall distance of each boundary cell
    (ReadWeights_Mod.f90:1283-1319): the area differences of opposite faces,
    a pair of closed opposite faces counting as twice the full face."""
    i, j, k = ijk[:, 0].astype(np.int64), ijk[:, 1].astype(np.int64), ijk[:, 2].astype(np.int64)
    fuR, fuL = fu[k - 1, j - 1, i + 1], fu[k - 1, j - 1, i]
    fvR, fvL = fv[k - 1, j + 1, i - 1], fv[k - 1, j, i - 1]
    fwR, fwL = fw[k + 1, j - 1, i - 1], fw[k, j - 1, i - 1]
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
