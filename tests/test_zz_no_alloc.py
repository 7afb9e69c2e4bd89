"""The column Thomas solve that allocates nothing (asam_tri_solve_noalloc).

It exists for callers that cannot let the library allocate device memory (a
host model that owns all device memory through its own pool, or one that
overlaps the solve with other streams, where cudaMalloc/cudaFree would
synchronise the device).  Checked through the C-ABI against the allocating
entry point asam_tri_solve, bit for bit (the Thomas tests' tolerance), on two
calls in a row so that the second call runs on the scratch array the first
one left behind.  Device memory for the inputs comes from torch (plumbing
only).  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(ncol, n1, seed):
    rng = np.random.default_rng(seed)
    d = 4.0 + rng.random((ncol, n1))
    u = rng.standard_normal((ncol, n1 - 1))
    l = rng.standard_normal((ncol, n1 - 1))
    b = rng.standard_normal((ncol, n1))
    return d, u, l, b


def test_tri_solve_noalloc_matches_allocating_entry_point(built_lib):
    torch = pytest.importorskip("torch")
    import asam_gb300
    from asam_gb300 import _lib

    lib = _lib.load()
    for ncol, n1, seed in ((4096, 130, 1), (1000, 64, 2)):  # second call reuses the first call's scratch
        d, u, l, b = _inputs(ncol, n1, seed)
        ref = asam_gb300.Solve_1D(d, u, l, b)
        dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (d, u, l, b)]
        rc = lib.asam_tri_solve_noalloc(ncol, n1, *(C.c_void_p(t.data_ptr()) for t in dev), None)
        assert rc == 0, lib.asam_last_error()
        torch.cuda.synchronize()
        got = dev[3].cpu().numpy()
        assert np.array_equal(got, ref)


def test_tri_solve_noalloc_rejects_oversize_and_host_pointers(built_lib):
    torch = pytest.importorskip("torch")
    from asam_gb300 import _lib

    lib = _lib.load()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(x.data_ptr())
    assert lib.asam_tri_solve_noalloc(1 << 20, 5, p, p, p, p, None) == 4
    assert b"exceeds" in lib.asam_last_error()
    h = np.zeros(8)
    assert lib.asam_tri_solve_noalloc(2, 4, h.ctypes.data, h.ctypes.data, h.ctypes.data, h.ctypes.data, None) == 4
