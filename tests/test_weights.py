"""Cut-cell geometry files (.Weight2): the library's compiled reader and
writer (asam_weight2_*) on a hand-written file in the layout WriteWeightBlk
writes (GRID/OutputWeightBlk_Mod.f90:501-670) read to known arrays, against
the oracle's restatement of ReadWeights (INIT/ReadWeights_Mod.f90:568-1330)
on the same files, generated geometries written and re-read bit for bit in
both directions between the library and the oracle, block selection, the
boundary-cell normals (ReadWeights_Mod.f90:1283-1319), soil and land classes
and the refusals.  Host arrays only: no GPU involved."""
import copy

import numpy as np
import pytest

from asam_gb300 import geometry as G
from asam_gb300 import weights as W
from oracle import weight2 as ORA
from tests import cases

pytestmark = pytest.mark.usefixtures("built_lib")


def _same_as_oracle(b, o):
    """A WeightBlock read by the library equals the oracle's read, bit for bit."""
    for k in ("fu", "fv", "fw", "volc"):
        assert np.array_equal(getattr(b.geo, k), o[k]), k
    for k in ("dx", "dy", "dz"):
        assert np.array_equal(getattr(b, k), o[k]), k
    assert b.origin == o["origin"]
    for (mi, mx), (oi, ox) in zip(b.mid_faces, o["mids"]):
        assert np.array_equal(mi, oi) and np.array_equal(mx, ox)
    bc, ob = b.bound, o["bound"]
    assert bc.struct_bound == ob["struct_bound"]
    for a, k in (("ijk", "ijk"), ("xs", "xs"), ("surf", "surf"), ("land_class", "land"), ("soil_type", "soil"),
                 ("normal", "normal"), ("fl", "fl"), ("dl", "dl")):
        assert np.array_equal(getattr(bc, a), ob[k]), a

KNOWN = """ Cart
           1   ! Number of blocks
 #.... Block           1 .....................................................
   0.0000000000000000        0.0000000000000000        0.0000000000000000
           2
   100.00000000000000
   100.00000000000000
           1
   50.000000000000000
           2
   10.000000000000000
   20.000000000000000
           2   NrW_FacesYZ
           0           1           1
   0.0000000000000000
           1           1           1
   2.5D+02
           1   NrMP_FacesYZ
           1           1           1
   100.0  25.0  5.0
           1   NrW_FacesZX
           2          -1           2
   1.0E3
           0   NrMP_FacesZX
           1   NrW_FacesXY
           1           1           0
   0.0000000000000000
           0   NrMP_FacesXY
           2    NrW_Cells
           1           1           1
   2.0D4
           2           1           2
   1.25E5
           1      NrB_Cells     3   Struct_Bound     0  Nr_SoilLayers
           1           1           1
   50.0 25.0 2.0
  0.1000000D+00  0.8000000D-01  0.8000000D+00  0.5000000D+02  0.2500000D+02  0.2000000D+01
"""


def test_known_file(tmp_path):
    p = tmp_path / "known.Weight2"
    p.write_text(KNOWN)
    b = W.read_weight2(str(p), expect=(2, 1, 2))
    _same_as_oracle(b, ORA.read(str(p), expect=(2, 1, 2)))
    g = b.geo
    assert (g.grid.nx, g.grid.ny, g.grid.nz) == (2, 1, 2)
    assert g.grid.dx == 100.0 and g.grid.dy == 50.0 and np.array_equal(g.grid.dz, [10.0, 20.0])
    fu, fv, fw, vol = ORA.default_weights([100.0, 100.0], [50.0], [10.0, 20.0])
    fu[0, 0, 1] = 0.0  # FU(0,1,1)
    fu[0, 0, 2] = 250.0  # FU(1,1,1)
    fv[1, 0, 1] = 1000.0  # FV(2,-1,2)
    fw[1, 0, 0] = 0.0  # FW(1,1,0)
    vol[1, 1, 1] = 2.0e4  # VolC(1,1,1)
    vol[2, 1, 2] = 1.25e5  # VolC(2,1,2)
    for got, exp in ((g.fu, fu), (g.fv, fv), (g.fw, fw), (g.volc, vol)):
        assert np.array_equal(got, exp)
    # the untouched defaults: full faces, interior volumes, periodic halos
    assert g.fu[1, 0, 4] == 50.0 * 20.0 and g.fw[3, 0, 1] == 100.0 * 50.0
    assert g.volc[1, 1, 2] == 100.0 * 50.0 * 10.0 and g.volc[1, 1, 0] == 100.0 * 50.0 * 10.0
    assert g.volc[0, 1, 1] == 100.0 * 50.0 * 10.0 and g.volc[0, 0, 0] == 1.0
    mi, mx = b.mid_faces[0]
    assert mi.tolist() == [[1, 1, 1]] and mx.tolist() == [[100.0, 25.0, 5.0]]
    bc = b.bound
    assert bc.ijk.tolist() == [[1, 1, 1]] and bc.xs.tolist() == [[50.0, 25.0, 2.0]]
    assert np.allclose(bc.surf, [[0.1, 0.08, 0.8, 50.0, 25.0, 2.0]])
    # normal of cell (1,1,1): FU(1)-FU(0) = 250 - 0, FV(1,1)-FV(1,0) = 0,
    # FW(1,1,1)-FW(1,1,0) = 5000 - 0
    n = np.array([250.0, 0.0, 5000.0])
    fl = np.sqrt((n * n).sum())
    assert np.allclose(bc.normal[0], n / fl, rtol=0, atol=1e-15) and bc.fl[0] == fl
    with pytest.raises(ValueError, match="nx"):
        W.read_weight2(str(p), expect=(3, 1, 2))


@pytest.mark.parametrize("name", ["hill_24x20x16", "bubble_12x10x8", "hill_odd_13x7x9_reverse"])
def test_round_trip_generated(tmp_path, name):
    geo, _, _ = cases.get(name)
    p = tmp_path / "case.Weight2"
    W.write_weight2(str(p), [geo])
    b = W.read_weight2(str(p), expect=(geo.grid.nx, geo.grid.ny, geo.grid.nz))
    for a in ("fu", "fv", "fw", "volc"):
        assert np.array_equal(getattr(b.geo, a), getattr(geo, a)), a
    assert np.array_equal(b.geo.grid.dz, geo.grid.dz)
    assert (b.geo.grid.dx, b.geo.grid.dy) == (geo.grid.dx, geo.grid.dy)
    assert np.array_equal(b.bound.ijk, G.boundary_cells(geo))
    assert b.bound.surf.shape == (len(b.bound.ijk), 6)
    norm = np.linalg.norm(b.bound.normal, axis=1)
    assert np.allclose(norm, 1.0)
    # the file lists only what differs from the reader's defaults
    text = p.read_text()
    assert text.startswith(" Cart\n")
    # the oracle reads the library's file to the same block, and the library
    # reads the oracle's file of the same geometry to the same block
    _same_as_oracle(b, ORA.read(str(p)))
    q = tmp_path / "oracle.Weight2"
    g = geo.grid
    bd = W.surface_data(geo)
    ORA.write(str(q), [dict(origin=(0.0, 0.0, 0.0), dx=np.full(g.nx, g.dx), dy=np.full(g.ny, g.dy), dz=g.dz,
                            fu=geo.fu, fv=geo.fv, fw=geo.fw, volc=geo.volc,
                            bound=dict(ijk=bd.ijk, xs=bd.xs, surf=bd.surf, struct_bound=3))])
    _same_as_oracle(W.read_weight2(str(q)), ORA.read(str(q)))
    _same_as_oracle(W.read_weight2(str(q)), ORA.read(str(p)))


def test_two_blocks_and_closed_faces(tmp_path):
    g0, _, _ = cases.get("hill_24x20x16")
    g1 = G.close_dead_faces(copy.deepcopy(g0))
    p = tmp_path / "two.Weight2"
    W.write_weight2(str(p), [g0, (g1, (2400.0, 0.0, 0.0), None)])
    b1 = W.read_weight2(str(p), ib=2)
    assert b1.origin == (2400.0, 0.0, 0.0)
    for a in ("fu", "fv", "fw", "volc"):
        assert np.array_equal(getattr(b1.geo, a), getattr(g1, a))
    b0 = W.read_weight2(str(p), ib=1)
    assert np.array_equal(b0.geo.fw, g0.fw)
    with pytest.raises(ValueError):
        W.read_weight2(str(p), ib=3)


def test_walls_change_the_halo_defaults(tmp_path):
    geo, _, _ = cases.get("hill_24x20x16")
    p = tmp_path / "w.Weight2"
    W.write_weight2(str(p), [geo], periodic=(False, False, False))
    b = W.read_weight2(str(p), periodic=(False, False, False))
    assert np.array_equal(b.geo.volc, geo.volc)
    fu, fv, fw, vol = ORA.default_weights(np.full(3, 2.0), np.full(2, 3.0), np.array([1.0, 4.0]), (False, False, False))
    assert vol[1, 1, 0] == 2.0 * 3.0 * 1.0 and vol[2, 1, 1] == 2.0 * 3.0 * 4.0 and vol[3, 1, 1] == 2.0 * 3.0 * 4.0


def test_oracle_list_directed_reader():
    rd = ORA.ListReader(["1, 2 3*4.5D0 rest", "7 8", "9 / 10", "11"])
    assert rd.values(2) == ["1", "2"]  # the rest of the line is dropped
    assert rd.ints(2) == [7, 8]
    with pytest.raises(ValueError):
        rd.values(2)  # '/' ends the read
    rd = ORA.ListReader(["2*1.5d+01 x"])
    assert rd.reals(2) == [15.0, 15.0]


# KNOWN in other list-directed forms: a quoted grid type, commas, repeat
# counts, trailing text, READs spread over several lines, D/d exponents, a
# leading '+', CR-LF line ends
KNOWN_FORMS = """ 'Cart'
 1, blocks
 #.... Block 1 ....
 3*0.0
 2 nx
 1.0D2, ignored
 +100
 1
 5.0d1
 2
 10.0
 2.0E+01
 2   NrW_FacesYZ
 0,
 1 1
 0.0
 1,1,1
 2.5D+02
 1
 1
 1 1
 1.0D2, 2.5E1
 5.0
 1
 2 -1 2 3
 1000.
 0
 1   NrW_FacesXY
 1 1 0
 2*0.0
 0
 2    NrW_Cells
 1 1 1
 20000
 2 1 2
 1.25E5
 1 'NrB_Cells' 3 Struct_Bound
 1 1 1
 50.0,25.0,2.0
 0.1 0.08 0.8
 50.0 25.0 2.0
""".replace("\n", "\r\n")


def test_list_directed_forms(tmp_path):
    """The library and the oracle read the same block from KNOWN and from the
    same content written in other list-directed forms."""
    p, q = tmp_path / "known.Weight2", tmp_path / "forms.Weight2"
    p.write_text(KNOWN)
    q.write_bytes(KNOWN_FORMS.encode())
    ref = W.read_weight2(str(p))
    _same_as_oracle(W.read_weight2(str(q)), ORA.read(str(p)))
    _same_as_oracle(W.read_weight2(str(q)), ORA.read(str(q)))
    for k in ("fu", "fv", "fw", "volc"):
        assert np.array_equal(getattr(W.read_weight2(str(q)).geo, k), getattr(ref.geo, k))


def test_write_keeps_midpoints_and_classes(tmp_path):
    """A block as read (cut-face midpoints, Struct_Bound 6 classes) written by
    the library reads back to the same block."""
    p = tmp_path / "k.Weight2"
    p.write_text(KNOWN.replace("3   Struct_Bound", "6   Struct_Bound").replace(_SURF, _SURF.rstrip("\n") + " 7 1 1 2\n"))
    b = W.read_weight2(str(p), nr_soil_layers=3)
    assert len(b.mid_faces[0][0]) == 1 and b.bound.land_class.tolist() == [7]
    q = tmp_path / "w.Weight2"
    W.write_weight2(str(q), [b])
    c = W.read_weight2(str(q), nr_soil_layers=3)
    _same_as_oracle(c, ORA.read(str(p), nr_soil_layers=3))
    _same_as_oracle(c, ORA.read(str(q), nr_soil_layers=3))


def test_bad_calls(tmp_path):
    """Null arguments and missing arrays are refused with ASAM_BAD_ARG, a
    missing file with ASAM_IO_ERROR; nothing is written for a refused call."""
    import ctypes as C

    from asam_gb300 import _lib

    lib = _lib.load()
    opt = _lib.AsamWeight2Options()
    opt.nr_soil_layers, opt.land_class_def = 7, 5
    info, h = _lib.AsamWeight2Block(), C.c_void_p()
    assert lib.asam_weight2_open(None, 1, C.byref(opt), C.byref(h), C.byref(info)) == _lib.ASAM_BAD_ARG
    assert lib.asam_weight2_open(str(tmp_path / "none").encode(), 1, C.byref(opt), C.byref(h),
                                 C.byref(info)) == _lib.ASAM_IO_ERROR
    opt.land_class_def = 10
    assert lib.asam_weight2_open(b"x", 1, C.byref(opt), C.byref(h), C.byref(info)) == _lib.ASAM_BAD_ARG
    assert lib.asam_weight2_fetch(None, C.byref(info)) == _lib.ASAM_BAD_ARG
    blk = _lib.AsamWeight2Block()
    blk.nx = blk.ny = blk.nz = 2
    per = (C.c_int * 3)(1, 1, 0)
    out = tmp_path / "refused.Weight2"
    assert lib.asam_weight2_write(str(out).encode(), 1, C.byref(blk), per) == _lib.ASAM_BAD_ARG
    assert not out.exists()
    geo = cases.get("hill_24x20x16")[0]
    bd = W.surface_data(geo)
    assert len(bd.ijk) > 0
    bd.struct_bound = 6  # land classes missing
    with pytest.raises(ValueError):
        W.write_weight2(str(out), [(geo, (0.0, 0.0, 0.0), bd)])


@pytest.mark.parametrize("reader", ["library", "oracle"])
def test_refusals(tmp_path, reader):
    read = W.read_weight2 if reader == "library" else ORA.read
    p = tmp_path / "g.Weight2"
    p.write_text(" Globe\n 1\n")
    with pytest.raises(NotImplementedError):
        read(str(p))
    p.write_text(KNOWN.replace("3   Struct_Bound", "7   Struct_Bound"))
    with pytest.raises(NotImplementedError):
        read(str(p))
    p.write_text(KNOWN.replace("           2          -1           2", "           2          -3           2"))
    with pytest.raises(ValueError):
        read(str(p))
    p.write_text(KNOWN[:400])
    with pytest.raises(ValueError):
        read(str(p))
    p.write_text(KNOWN.replace("   1.0E3", "   1.0E3x"))
    with pytest.raises(ValueError):
        read(str(p))
    p.write_text(KNOWN.replace("           0           1           1\n", "           0           1 /\n"))
    with pytest.raises(ValueError):
        read(str(p))


_SURF = "  0.1000000D+00  0.8000000D-01  0.8000000D+00  0.5000000D+02  0.2500000D+02  0.2000000D+01\n"


@pytest.mark.parametrize("sb,tail,land,soil,zrauh", [
    (3, "", [W.LAND_CLASS_DEF], [0, 0, 5], 0.1),                        # roughness as read, last layer 5
    (4, " 3 4\n 6\n", [W.LAND_CLASS_DEF], [3, 4, 6], 0.05),            # soil types over two lines
    (5, " 2\n", [W.LAND_CLASS_SEA], [0, 0, 0], W.ZROUGH[9]),            # any class read becomes sea
    (6, " 7 1 1 2\n", [7], [1, 1, 2], W.ZROUGH[7]),                     # land class, then the soil types
])
def test_soil_and_land_classes(tmp_path, sb, tail, land, soil, zrauh):
    """Struct_Bound 3-6 (ReadWeights_Mod.f90:1236-1279) with three soil
    layers: the soil types and the land class follow the six surface values
    on the same list-directed READ; 4 sets the roughness to 0.05, 5 and 6
    take it from the land class's roughness length."""
    text = KNOWN.replace("3   Struct_Bound", f"{sb}   Struct_Bound")
    if tail:
        text = text.replace(_SURF, _SURF.rstrip("\n") + tail)
    p = tmp_path / "k.Weight2"
    p.write_text(text)
    b = W.read_weight2(str(p), nr_soil_layers=3)
    _same_as_oracle(b, ORA.read(str(p), nr_soil_layers=3))
    bc = b.bound
    assert bc.struct_bound == sb
    assert bc.land_class.tolist() == land and bc.soil_type.tolist() == [soil]
    assert bc.surf[0, 0] == zrauh and bc.surf[0, 1] == 0.08


def test_real_island(tmp_path):
    """With RealIsland a boundary cell of full volume becomes sea (class 9);
    the known file's cell (1,1,1) has VolC 2e4 < dx*dy*dz = 5e4, so a full
    volume is written for it first."""
    p = tmp_path / "k.Weight2"
    p.write_text(KNOWN)
    assert W.read_weight2(str(p), real_island=True).bound.land_class.tolist() == [W.LAND_CLASS_DEF]
    p.write_text(KNOWN.replace("   2.0D4", "   5.0D4"))
    assert W.read_weight2(str(p), real_island=True).bound.land_class.tolist() == [W.LAND_CLASS_SEA]
    assert ORA.read(str(p), real_island=True)["bound"]["land"].tolist() == [W.LAND_CLASS_SEA]
    assert W.read_weight2(str(p)).bound.land_class.tolist() == [W.LAND_CLASS_DEF]


@pytest.mark.parametrize("sb", [4, 6])
def test_soil_classes_round_trip(tmp_path, sb):
    """The writer's soil and land columns read back as written."""
    geo = G.close_dead_faces(copy.deepcopy(cases.get("hill_24x20x16")[0]))
    bound = W.surface_data(geo)
    n = len(bound.ijk)
    assert n > 100
    rng = np.random.default_rng(5)
    bound.struct_bound = sb
    bound.land_class = rng.integers(0, 10, n).astype(np.int32)
    bound.soil_type = rng.integers(1, 9, (n, 4)).astype(np.int32)
    p = tmp_path / "s.Weight2"
    W.write_weight2(str(p), [(geo, (0.0, 0.0, 0.0), bound)])
    b = W.read_weight2(str(p), nr_soil_layers=4)
    _same_as_oracle(b, ORA.read(str(p), nr_soil_layers=4))
    got = b.bound
    assert np.array_equal(got.soil_type, bound.soil_type)
    if sb == 6:
        assert np.array_equal(got.land_class, bound.land_class)
        assert np.array_equal(got.surf[:, 0], np.asarray(W.ZROUGH)[bound.land_class])
    else:
        assert (got.land_class == W.LAND_CLASS_DEF).all() and (got.surf[:, 0] == 0.05).all()
    assert np.array_equal(got.surf[:, 1:], bound.surf[:, 1:])


def test_large_lists_parallel_paths(tmp_path):
    """A deck whose weight lists are long enough for the threaded reader and
    writer (more than 65536 pairs in one list): written and re-read bit for
    bit, equal to the oracle's reading; a pair spread over two lines in the
    middle of a long list (the threaded reader's layout assumption broken)
    and a malformed value there are read exactly as the one-READ-at-a-time
    reader reads them."""
    geo = G.close_dead_faces(G.hill_case(96, 96, 24, seed=4)[0])
    p = tmp_path / "big.Weight2"
    W.write_weight2(str(p), [geo])
    text = p.read_text()
    nfu = int(text.split("NrW_FacesYZ")[0].split()[-1])
    assert nfu > 65536
    b = W.read_weight2(str(p))
    for k in ("fu", "fv", "fw", "volc"):
        assert np.array_equal(getattr(b.geo, k), getattr(geo, k)), k
    lines = text.split("\n")
    head = next(i for i, s in enumerate(lines) if "NrW_FacesYZ" in s)
    mid = head + 1 + 2 * (nfu // 2)  # an 'ix iy iz' line in the middle of the FU list
    ix, iy, iz = lines[mid].split()
    split = lines[:mid] + [f" {ix}", f" {iy} {iz}"] + lines[mid + 1:]
    q = tmp_path / "split.Weight2"
    q.write_text("\n".join(split))
    bq = W.read_weight2(str(q))
    assert np.array_equal(bq.geo.fu, geo.fu)
    bad = lines[:mid + 1] + [" 1.0x"] + lines[mid + 2:]
    q.write_text("\n".join(bad))
    with pytest.raises(ValueError, match="bad weight"):
        W.read_weight2(str(q))


def test_halo_volume_product_order(tmp_path):
    """The reader's default halo volumes multiply in its own order
    (ReadWeights_Mod.f90:905-987): dxLoc*dy*dz on the lateral sides and
    dx*dy*dzLoc on the bottom and top -- widths chosen so that the other
    order rounds differently.  A file listing no weights reads to exactly
    those products, in the library and in the oracle."""
    dx, dy, dz = 0.1, 0.7, 1.7
    assert (dx * dy) * dz != (dz * dx) * dy
    text = " Cart\n 1\n #.... Block 1 ....\n 0.0 0.0 0.0\n 2\n 0.1\n 0.1\n 1\n 0.7\n 2\n 1.7\n 1.7\n" \
           " 0 NrW_FacesYZ\n 0 NrMP_FacesYZ\n 0 NrW_FacesZX\n 0 NrMP_FacesZX\n 0 NrW_FacesXY\n 0 NrMP_FacesXY\n" \
           " 0 NrW_Cells\n 0 NrB_Cells 3 Struct_Bound\n"
    p = tmp_path / "o.Weight2"
    p.write_text(text)
    for periodic in ((True, True, False), (False, False, False)):
        b = W.read_weight2(str(p), periodic=periodic)
        o = ORA.read(str(p), periodic=periodic)
        assert np.array_equal(b.geo.volc, o["volc"])
        v = b.geo.volc
        assert v[0, 1, 1] == (dx * dy) * dz and v[-1, 1, 1] == (dx * dy) * dz
        assert v[1, 1, 0] == (dx * dy) * dz and v[1, 0, 1] == (dy * dx) * dz
        assert v[1, 1, 1] == (dx * dy) * dz
