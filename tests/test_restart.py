"""Restart files (INIT/Restart_Mod.f90:14-82) on host arrays: the oracle's
record format against a hand-assembled known answer, the library's reader and
writer against the oracle byte for byte, gfortran subrecord splits, the
reference's file name and RestartTime scheduling, and the refusals.  Host
arrays only: the library copies them with the C library, no GPU involved."""
import struct

import numpy as np
import pytest

from oracle import restart as ORA


def _block(nx, ny, nz, ncomp, nfrac=1, seed=0):
    r = np.random.default_rng(seed)
    npad = (nx + 2) * (ny + 2) * (nz + 2) * nfrac
    return (r.standard_normal((ncomp, npad)), r.standard_normal((nx + 1) * ny * nz),
            r.standard_normal(nx * (ny + 1) * nz), r.standard_normal(nx * ny * (nz + 1)))


def _desc(dims, b):
    from asam_gb300 import restart as R

    return R.block(*dims, *b)


def test_oracle_known_answer_layout():
    # 1x1x1 block, one component: 27 padded cells, 2 + 2 + 2 face values
    c = np.arange(27.0).reshape(1, 27)
    uf, vf, wf = np.array([1.5, 2.5]), np.array([3.5, 4.5]), np.array([5.5, 6.5])
    data = ORA.encode(12.5, 7, 30.0, [(c, uf, vf, wf)])
    exp = (struct.pack("<idi", 8, 12.5, 8) + struct.pack("<iii", 4, 7, 4) + struct.pack("<idi", 8, 30.0, 8)
           + struct.pack("<i", 216) + struct.pack("<27d", *range(27)) + struct.pack("<i", 216)
           + struct.pack("<i", 48) + struct.pack("<6d", 1.5, 2.5, 3.5, 4.5, 5.5, 6.5) + struct.pack("<i", 48))
    assert data == exp


def test_oracle_subrecord_split_known_answer():
    payload = bytes(range(10))
    enc = ORA.encode_record(payload, max_sub=4)
    exp = (struct.pack("<i", -4) + payload[:4] + struct.pack("<i", 4)
           + struct.pack("<i", -4) + payload[4:8] + struct.pack("<i", -4)
           + struct.pack("<i", 2) + payload[8:] + struct.pack("<i", -2))
    assert enc == exp
    assert ORA.decode_records(enc) == [payload]


NAMES = [("Hill.grid", 0, "RESTART/Hill.0"), ("Bubble.grid", 17, "RESTART/Bubble.17"),
         ("case/run.grid.bak", 3, "RESTART/case/run.3"), ("Block", 2, "RESTART/2")]


@pytest.mark.parametrize("name,rank,exp", NAMES)
def test_oracle_file_name(name, rank, exp):
    assert ORA.file_name(name, rank) == exp


def case_file_name(tmp_path, name, rank, exp):
    from asam_gb300 import restart as R

    assert ORA.file_name(name, rank) == exp
    assert R.restart_file_name(name, rank) == exp


WRITES = [((4, 3, 5), 3, 1), ((1, 1, 1), 1, 1), ((6, 2, 3), 2, 2), ((5, 4, 3), 0, 1)]


def case_library_write_matches_oracle(tmp_path, dims, ncomp, nfrac):
    from asam_gb300 import restart as R

    b = _block(*dims, ncomp, nfrac, seed=1)
    path = tmp_path / "r.0"
    R.write_restart(str(path), [_desc(dims, b)], 42.25, 3, 60.0)
    assert path.read_bytes() == ORA.encode(42.25, 3, 60.0, [b])


def case_library_read_of_oracle_file_two_blocks(tmp_path):
    from asam_gb300 import restart as R

    d0, d1 = (4, 3, 2), (2, 5, 3)
    b0, b1 = _block(*d0, 2, seed=2), _block(*d1, 2, seed=3)
    path = tmp_path / "r.1"
    path.write_bytes(ORA.encode(-1.0, 11, 2.0, [b0, b1]))
    z0 = tuple(np.zeros_like(a) for a in b0)
    z1 = tuple(np.zeros_like(a) for a in b1)
    t, g, o = R.read_restart(str(path), [_desc(d0, z0), _desc(d1, z1)])
    assert (t, g, o) == (-1.0, 11, 2.0)
    for got, exp in zip(z0 + z1, b0 + b1):
        assert np.array_equal(got, exp)


def case_subrecords_both_ways(tmp_path, max_sub):
    from asam_gb300 import restart as R

    dims = (7, 5, 4)
    b = _block(*dims, 2, seed=4)
    path = tmp_path / "r.2"
    try:
        R.set_max_subrecord(max_sub)
        R.write_restart(str(path), [_desc(dims, b)], 1.0, 0, 0.0)
    finally:
        R.set_max_subrecord(ORA.GFORTRAN_MAX_SUBRECORD)
    assert path.read_bytes() == ORA.encode(1.0, 0, 0.0, [b], max_sub=max_sub)
    # the reader takes any split, including one it did not write
    path.write_bytes(ORA.encode(2.0, 1, 0.0, [b], max_sub=max_sub + 5))
    z = tuple(np.zeros_like(a) for a in b)
    R.read_restart(str(path), [_desc(dims, z)])
    for got, exp in zip(z, b):
        assert np.array_equal(got, exp)


def case_refusals(tmp_path):
    from asam_gb300 import _lib
    from asam_gb300 import restart as R

    dims = (3, 3, 3)
    b = _block(*dims, 2, seed=5)
    path = tmp_path / "r.3"
    path.write_bytes(ORA.encode(0.0, 0, 0.0, [b]))
    # block of other extents: the first component record does not fit
    other = _block(3, 3, 4, 2)
    with pytest.raises(_lib.AsamError) as e:
        R.read_restart(str(path), [_desc((3, 3, 4), other)])
    assert e.value.status == 7
    # one component more than the file holds
    more = _block(*dims, 3)
    with pytest.raises(_lib.AsamError) as e:
        R.read_restart(str(path), [_desc(dims, more)])
    assert e.value.status == 7
    # truncated file
    path.write_bytes(ORA.encode(0.0, 0, 0.0, [b])[:-20])
    with pytest.raises(_lib.AsamError) as e:
        R.read_restart(str(path), [_desc(dims, tuple(np.zeros_like(a) for a in b))])
    assert e.value.status == 7
    # corrupt trailing marker
    data = bytearray(ORA.encode(0.0, 0, 0.0, [b]))
    data[12] ^= 1
    path.write_bytes(bytes(data))
    with pytest.raises(_lib.AsamError) as e:
        R.read_restart(str(path), [_desc(dims, tuple(np.zeros_like(a) for a in b))])
    assert e.value.status == 7
    # missing file and missing directory
    with pytest.raises(_lib.AsamError) as e:
        R.read_restart(str(tmp_path / "none"), [_desc(dims, b)])
    assert e.value.status == 7
    with pytest.raises(_lib.AsamError) as e:
        R.write_restart(str(tmp_path / "no" / "dir"), [_desc(dims, b)], 0.0)
    assert e.value.status == 7
    lib = _lib.load()
    assert lib.asam_restart_set_max_subrecord(0) == 4
    assert lib.asam_restart_set_max_subrecord(2147483640) == 4
    assert lib.asam_restart_write(None, None, 0, None) == 4


def case_restart_schedule(tmp_path):
    from asam_gb300 import restart as R

    dims = (3, 2, 2)
    b = _block(*dims, 2, seed=6)
    (tmp_path / "RESTART").mkdir()
    w = R.Restart([dims], restart_time_incr=10.0, directory=str(tmp_path))
    assert w.ReadRestart([b[0]], [b[1:]], 5.0, "Hill.grid") == 5.0  # no restart: first write after t=15
    assert w.RestartTime == 15.0
    assert not w.WriteRestart([b[0]], [b[1:]], 15.0, "Hill.grid")
    w.GMVStep, w.OutputTime = 4, 20.0
    assert w.WriteRestart([b[0]], [b[1:]], 15.5, "Hill.grid")
    assert w.RestartTime == 25.0
    f = tmp_path / "RESTART" / "Hill.0"
    assert f.read_bytes() == ORA.encode(15.5, 4, 20.0, [b])
    r = R.Restart([dims], restart_time_incr=10.0, restart=True, directory=str(tmp_path))
    z = tuple(np.zeros_like(a) for a in b)
    assert r.ReadRestart([z[0]], [z[1:]], 0.0, "Hill.grid") == 15.5
    assert (r.GMVStep, r.OutputTime, r.RestartTime) == (4, 20.0, 0.0)
    for got, exp in zip(z, b):
        assert np.array_equal(got, exp)


LIBRARY_CASES = ([(case_file_name, n) for n in NAMES] + [(case_library_write_matches_oracle, w) for w in WRITES]
                 + [(case_library_read_of_oracle_file_two_blocks, ()), (case_refusals, ()),
                    (case_restart_schedule, ())] + [(case_subrecords_both_ways, (m,)) for m in (8, 1000, 4096 + 3)])


@pytest.mark.parametrize("fn,args", LIBRARY_CASES, ids=[f"{k:02d}_{fn.__name__}" for k, (fn, _) in
                                                          enumerate(LIBRARY_CASES)])
def test_library_restart_io(built_lib, tmp_path, fn, args):
    """The library's reader and writer on host arrays, in the test process."""
    fn(tmp_path, *args)


def test_descriptor_keeps_temporaries_alive(built_lib, tmp_path):
    """A descriptor built from temporary arrays stays valid: the reader fills
    arrays that only the descriptor references, and the process keeps working
    on the heap afterwards (run in a child so a heap corruption cannot take
    the test runner down)."""
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    code = f"""
import sys, gc
sys.path.insert(0, {str(root)!r})
import numpy as np
from asam_gb300 import restart as R
from oracle import restart as ORA
dims = (5, 4, 3)
r = np.random.default_rng(9)
b = (r.standard_normal((2, 7 * 6 * 5)), r.standard_normal(6 * 4 * 3), r.standard_normal(5 * 5 * 3),
     r.standard_normal(5 * 4 * 4))
path = {str(tmp_path / "r.0")!r}
open(path, "wb").write(ORA.encode(3.0, 1, 0.0, [b]))
for it in range(50):
    desc = R.block(*dims, *(np.zeros_like(a) for a in b))
    gc.collect()
    assert R.read_restart(path, [desc]) == (3.0, 1, 0.0)
    for got, exp in zip(desc._keep, b):
        assert np.array_equal(got, exp)
    R.write_restart(path + ".w", [R.block(*dims, *(a.copy() for a in b))], 3.0, 1, 0.0)
    junk = [np.ones(1000 + k) * k for k in range(200)]
    assert sum(float(j.sum()) for j in junk) > 0
print("ok")
"""
    res = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and res.stdout.strip().endswith("ok"), res.stdout[-4000:] + res.stderr[-4000:]
