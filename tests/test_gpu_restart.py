"""Restart files from and into device memory (INIT/Restart_Mod.f90:14-82):
the file written from a device-resident state is the oracle's byte for byte,
reading it back restores every array bitwise, a run resumed from the file
continues bitwise like the uninterrupted run, and arrays larger than the
staging chunk cross subrecord splits in both directions."""
from __future__ import annotations

import numpy as np
import pytest

from asam_gb300 import TransportBlock
from asam_gb300 import restart as R
from oracle import restart as ORA
from tests import cases

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).ravel()).cuda()


@pytest.mark.parametrize("name", ["hill_24x20x16", "bubble_12x10x8"])
def test_resume_from_restart_is_bitwise(built_lib, tmp_path, name):
    torch = pytest.importorskip("torch")
    geo, vel, st = cases.get(name)
    nx, ny, nz = geo.grid.nx, geo.grid.ny, geo.grid.nz
    ncomp = st.c.shape[0]
    velh = tuple(np.ascontiguousarray(v, dtype=np.float64).ravel() for v in vel)
    veld = tuple(_dev(torch, v) for v in velh)
    blk = TransportBlock(geo, ncomp=ncomp, rho_pos=0)
    blk.set_velocity(*vel)
    c = _dev(torch, st.c).reshape(ncomp, -1)
    for _ in range(2):
        blk.ros_step_device(c.data_ptr(), 2.0)
    path = tmp_path / "RESTART_hill.0"
    R.write_restart(str(path), [R.block(nx, ny, nz, c, *veld)], 4.0, 2, 10.0)
    host = (c.cpu().numpy(),) + velh
    assert path.read_bytes() == ORA.encode(4.0, 2, 10.0, [host])
    # uninterrupted run
    for _ in range(2):
        blk.ros_step_device(c.data_ptr(), 2.0)
    torch.cuda.synchronize()
    blk.close()
    # resumed run: fresh block, state and velocity from the file
    c2 = torch.zeros_like(c)
    vel2 = tuple(torch.zeros_like(v) for v in veld)
    t, g, o = R.read_restart(str(path), [R.block(nx, ny, nz, c2, *vel2)])
    assert (t, g, o) == (4.0, 2, 10.0)
    for a, b in zip(vel2, veld):
        assert torch.equal(a, b)
    blk2 = TransportBlock(geo, ncomp=ncomp, rho_pos=0)
    blk2.set_velocity(*(v.cpu().numpy() for v in vel2))
    for _ in range(2):
        blk2.ros_step_device(c2.data_ptr(), 2.0)
    torch.cuda.synchronize()
    blk2.close()
    assert torch.equal(c2, c)


@pytest.mark.parametrize("max_sub", [None, 50_000_003])
def test_large_arrays_through_the_staging_chunks(built_lib, tmp_path, max_sub):
    # one component of 172*172*162 padded cells is 38 MB, above the 32 MB
    # staging chunk; an odd subrecord length splits records mid-value
    torch = pytest.importorskip("torch")
    nx, ny, nz = 170, 170, 160
    g = torch.Generator(device="cuda").manual_seed(7)
    npad = (nx + 2) * (ny + 2) * (nz + 2)
    c = torch.randn(2, npad, dtype=torch.float64, device="cuda", generator=g)
    uf = torch.randn((nx + 1) * ny * nz, dtype=torch.float64, device="cuda", generator=g)
    vf = torch.randn(nx * (ny + 1) * nz, dtype=torch.float64, device="cuda", generator=g)
    wf = torch.randn(nx * ny * (nz + 1), dtype=torch.float64, device="cuda", generator=g)
    host_vf = vf.cpu().numpy()  # one array from host memory, the rest from the device
    path = tmp_path / "big.0"
    try:
        if max_sub:
            R.set_max_subrecord(max_sub)
        R.write_restart(str(path), [R.block(nx, ny, nz, c, uf, host_vf, wf)], 1.5, 9, 3.0)
    finally:
        R.set_max_subrecord(ORA.GFORTRAN_MAX_SUBRECORD)
    ref = ORA.encode(1.5, 9, 3.0, [(c.cpu().numpy(), uf.cpu().numpy(), host_vf, wf.cpu().numpy())],
                     max_sub=max_sub or ORA.GFORTRAN_MAX_SUBRECORD)
    data = path.read_bytes()
    assert len(data) == len(ref) and data == ref
    c2, uf2, wf2 = torch.empty_like(c), torch.empty_like(uf), torch.empty_like(wf)
    vf2 = np.empty_like(host_vf)
    assert R.read_restart(str(path), [R.block(nx, ny, nz, c2, uf2, vf2, wf2)]) == (1.5, 9, 3.0)
    torch.cuda.synchronize()
    assert torch.equal(c2, c) and torch.equal(uf2, uf) and torch.equal(wf2, wf)
    assert np.array_equal(vf2, host_vf)


def test_weight2_refuses_device_arrays(built_lib, tmp_path):
    """The .Weight2 routines take host arrays: a device array in a block to
    write or to fill is refused with ASAM_BAD_ARG before any file is made
    or any array is touched."""
    import ctypes as C

    torch = pytest.importorskip("torch")
    from asam_gb300 import _lib
    from asam_gb300 import weights as W

    geo = cases.get("hill_24x20x16")[0]
    p = tmp_path / "h.Weight2"
    W.write_weight2(str(p), [geo])
    lib = _lib.load()
    opt = _lib.AsamWeight2Options()
    opt.periodic[:] = [1, 1, 0]
    opt.nr_soil_layers, opt.land_class_def = 7, 5
    info, h = _lib.AsamWeight2Block(), C.c_void_p()
    assert lib.asam_weight2_open(str(p).encode(), 1, C.byref(opt), C.byref(h), C.byref(info)) == _lib.ASAM_OK
    try:
        nx, ny, nz = info.nx, info.ny, info.nz
        fu = torch.zeros((nz, ny, nx + 3), dtype=torch.float64, device="cuda")
        dst = _lib.AsamWeight2Block()
        dst.fu = fu.data_ptr()
        assert lib.asam_weight2_fetch(h, C.byref(dst)) == _lib.ASAM_BAD_ARG
        torch.cuda.synchronize()
        assert not fu.any().item()
    finally:
        lib.asam_weight2_close(h)
    b = W.read_weight2(str(p))
    keep = []
    desc = W._describe(b, keep)
    dz = torch.from_numpy(b.dz).cuda()
    desc.dz = dz.data_ptr()
    q = tmp_path / "refused.Weight2"
    per = (C.c_int * 3)(1, 1, 0)
    assert lib.asam_weight2_write(str(q).encode(), 1, C.byref(desc), per) == _lib.ASAM_BAD_ARG
    assert not q.exists()
