"""Build recipe of the CUDA library (sm_103a) and of the CPU oracle.

The library is a set of translation units compiled in parallel by nvcc and
linked into ``asam_gb300/libasam_gb300.so``:

* ``k64.cu``  FP64 kernels with ``-fmad=false`` (reference rounding, no FMA)
* ``k32.cu``  FP32 kernels of the refined mode
* ``capi.cu`` context, drivers and the ``extern "C"`` entry points
* ``tri_noalloc.cu`` the column solve that allocates nothing
* ``adjoint.cu`` tangent-linear and adjoint of the transport stage
* ``proj.cu`` pressure projection: Laplacian hierarchy, multigrid, FGMRES
* ``dyn.cu`` dynamical-core stage: momentum sources, face/cell velocities,
  thermodynamics and the stage driver around the transport solve and the
  projection
* ``restart.cu`` and ``weight2.cu`` restart and cut-cell geometry files (host)

The oracle (``oracle/asam_oracle.c`` for the transport stage,
``oracle/asam_proj.c`` for the pressure projection, ``oracle/asam_dyn.c`` for
the dynamical-core stage) is a test-only checker
compiled by gcc into ``oracle/_build/libasam_oracle.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libasam_gb300.so"
ORACLE_SRC = [ROOT / "oracle" / "asam_oracle.c", ROOT / "oracle" / "asam_proj.c", ROOT / "oracle" / "asam_dyn.c",
              ROOT / "oracle" / "asam_tritb.c"]
ORACLE_DEPS = ORACLE_SRC + [ROOT / "oracle" / "asam_oracle.h"]
ORACLE_LIB = ROOT / "oracle" / "_build" / "libasam_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "k64.cu": ["-fmad=false"],
    "k32.cu": [],
    "k64fma.cu": [],
    "capi.cu": [],
    "tri_noalloc.cu": ["-fmad=false"],
    "adjoint.cu": ["-fmad=false"],
    "batch.cu": [],
    "tune.cu": [],
    "step_graph.cu": ["-fmad=false"],
    "proj.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "dyn.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "restart.cu": [],
    "tritb.cu": ["-fmad=false"],
    "weight2.cu": ["-Xcompiler", "-ffp-contract=off"],
}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build asam_gb300")
    return cand


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [
        INCLUDE / "asam_gb300.h"
    ]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile the CUDA library if a source is newer than the .so."""
    if not force and not _stale(LIB, _sources()):
        return LIB
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    common = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}",
              "-Xptxas", "-v" if verbose else "-O3"]

    def compile_unit(name: str) -> Path:
        obj = BUILD / (name.replace(".cu", ".o"))
        cmd = common + UNITS[name] + ["-c", str(CSRC / name), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{res.stderr}")
        if verbose:
            sys.stderr.write(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) with gcc."""
    if not force and not _stale(ORACLE_LIB, ORACLE_DEPS):
        return ORACLE_LIB
    ORACLE_LIB.parent.mkdir(exist_ok=True)
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           *map(str, ORACLE_SRC), "-o", str(tmp), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"gcc failed for the oracle:\n{res.stderr}")
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_oracle(force="--force" in sys.argv))
