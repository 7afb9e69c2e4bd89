"""Restart I/O of Restart_Mod (INIT/Restart_Mod.f90:14-82) over the C-ABI.

``Restart`` mirrors the module: ``RestartTime`` scheduling, ``WriteRestart``
(writes when Time > RestartTime, then advances RestartTime by
RestartTimeIncr) and ``ReadRestart`` (reads when Restart is set, else
schedules the first write).  ``Vec`` is a list with one ``(ncomp, npad)``
float64 array per block (CUDA tensor, CPU tensor or numpy array, the
library's padded cell layout); ``Vel`` a list of ``(uF, vF, wF)`` in the face
layouts.  The file is the gfortran unformatted file the reference writes, so
a Fortran run can resume from a GPU run and the other way round.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _lib


def _ptr(a) -> int:
    if hasattr(a, "data_ptr"):  # torch tensor
        if str(a.dtype) != "torch.float64" or not a.is_contiguous():
            raise ValueError("restart arrays must be contiguous float64")
        return a.data_ptr()
    if a.dtype.str != "<f8" or not a.flags["C_CONTIGUOUS"]:
        raise ValueError("restart arrays must be contiguous float64")
    return a.ctypes.data


def _numel(a) -> int:
    return a.numel() if hasattr(a, "numel") and callable(a.numel) else a.size


def block(nx: int, ny: int, nz: int, c, uf, vf, wf) -> _lib.AsamRestartBlock:
    """Descriptor of one block: c is (ncomp, npad*nFrac).

    The descriptor holds raw addresses, so it keeps references to the four
    arrays (``_keep``): a descriptor built from temporaries stays valid for
    as long as the descriptor itself lives."""
    npad = (nx + 2) * (ny + 2) * (nz + 2)
    ncomp = c.shape[0]
    per = _numel(c) // max(ncomp, 1)
    if per % npad:
        raise ValueError("component arrays are not a multiple of the padded block")
    for a, n in ((uf, (nx + 1) * ny * nz), (vf, nx * (ny + 1) * nz), (wf, nx * ny * (nz + 1))):
        if _numel(a) != n:
            raise ValueError("face velocity of the wrong size")
    desc = _lib.AsamRestartBlock(nx, ny, nz, ncomp, per // npad, _ptr(c), _ptr(uf), _ptr(vf), _ptr(wf))
    desc._keep = (c, uf, vf, wf)
    return desc


def _array(blocks):
    """ctypes array of the descriptors; the copies carry no references, so the
    caller keeps ``blocks`` (and with it the arrays) alive across the call."""
    blocks = list(blocks)
    for b in blocks:
        if not hasattr(b, "_keep"):
            raise TypeError("restart blocks must come from asam_gb300.restart.block()")
    return blocks, (_lib.AsamRestartBlock * len(blocks))(*blocks)


def write_restart(path: str, blocks, time: float, gmv_step: int = 0, output_time: float = 0.0) -> None:
    lib = _lib.load()
    blocks, arr = _array(blocks)
    hdr = _lib.AsamRestartHeader(time, gmv_step, output_time)
    _lib.check(lib.asam_restart_write(os.fsencode(path), C.byref(hdr), len(blocks), arr), "asam_restart_write")


def read_restart(path: str, blocks) -> tuple[float, int, float]:
    lib = _lib.load()
    blocks, arr = _array(blocks)
    hdr = _lib.AsamRestartHeader()
    _lib.check(lib.asam_restart_read(os.fsencode(path), C.byref(hdr), len(blocks), arr), "asam_restart_read")
    return hdr.time, hdr.gmv_step, hdr.output_time


def restart_file_name(grid_file: str, rank: int) -> str:
    lib = _lib.load()
    buf = C.create_string_buffer(len(grid_file) + 32)
    _lib.check(lib.asam_restart_file_name(grid_file.encode(), rank, buf, len(buf)), "asam_restart_file_name")
    return buf.value.decode()


def set_max_subrecord(nbytes: int) -> None:
    """gfortran's -fmax-subrecord-length for the files written here."""
    _lib.check(_lib.load().asam_restart_set_max_subrecord(nbytes), "asam_restart_set_max_subrecord")


class Restart:
    """Module state of Restart_Mod: RestartTime, RestartTimeIncr, Restart
    (MODULE/Control_Mod.f90:18-20, default increment 1e20)."""

    def __init__(self, dims, restart_time_incr: float = 1.0e20, restart: bool = False, rank: int = 0,
                 directory: str = "."):
        self.dims = list(dims)  # (nx, ny, nz) per local block
        self.RestartTimeIncr = restart_time_incr
        self.Restart = restart
        self.RestartTime = 0.0
        self.rank = rank
        self.directory = directory
        self.GMVStep = 0
        self.OutputTime = 0.0

    def _path(self, FileName: str) -> str:
        return os.path.join(self.directory, restart_file_name(FileName, self.rank))

    def _blocks(self, Vec, Vel):
        return [block(*d, c, *v) for d, c, v in zip(self.dims, Vec, Vel)]

    def WriteRestart(self, Vec, Vel, Time: float, FileName: str) -> bool:
        """Restart_Mod.f90:14-43.  Returns whether a file was written."""
        if not Time > self.RestartTime:
            return False
        write_restart(self._path(FileName), self._blocks(Vec, Vel), Time, self.GMVStep, self.OutputTime)
        self.RestartTime = self.RestartTime + self.RestartTimeIncr
        return True

    def ReadRestart(self, Vec, Vel, Time: float, FileName: str) -> float:
        """Restart_Mod.f90:45-81.  Returns Time (read from the file when
        Restart is set).  After a read RestartTime keeps its initial value,
        as in the reference, so the next WriteRestart writes."""
        if self.Restart:
            Time, self.GMVStep, self.OutputTime = read_restart(self._path(FileName), self._blocks(Vec, Vel))
        else:
            self.RestartTime = Time + self.RestartTimeIncr
        return Time
