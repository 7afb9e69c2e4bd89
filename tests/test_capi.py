"""The C-ABI library builds, loads and exports every symbol include/asam_gb300.h declares
(no compute calls: this runs without a GPU)."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "asam_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(asam_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["asam_create", "asam_fcn", "asam_jac", "asam_matvec", "asam_psolve", "asam_bicgstab",
              "asam_ros_step", "asam_total_scalar", "asam_tri_solve"]:
        assert s in syms


def test_library_exports_all_symbols(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\sT\s(asam_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_library_loads_with_ctypes(built_lib):
    from asam_gb300 import _lib

    lib = _lib.load()
    for name, _, _ in _lib.SIGNATURES:
        assert hasattr(lib, name)
    assert {n for n, _, _ in _lib.SIGNATURES} == set(declared_symbols())


def test_ros_coeffs_host_only(built_lib):
    # pure host function of the library: InitRos3MetC tables
    import asam_gb300

    n, beta0, al, be, gm = asam_gb300.ros_coeffs("RosRK3")
    assert n == 3 and beta0 == 1.0
    n, beta0, al, be, gm = asam_gb300.ros_coeffs("Ros3Pw")
    assert n == 3 and abs(beta0 - 0.7886751345948129) < 1e-15


def test_npad(built_lib):
    from asam_gb300 import _lib

    lib = _lib.load()
    cfg = _lib.AsamConfig(10, 20, 30, 1, 1, 0, 3, 0, 5, 30, 1e-6, 5, 0, 1, 1, 0, 0)
    assert lib.asam_npad(cfg) == 12 * 22 * 32
