"""Restart files: a numpy restatement of WriteRestart / ReadRestart
(INIT/Restart_Mod.f90:14-82) for the tests.

Test infrastructure only: the tests use it to check the library's restart
reader and writer; nothing in the product imports it.

Parity unpinned: the reference ships no restart file and this image has no
Fortran compiler to make one.  The record layout restated here is gfortran's
documented format for unformatted sequential files (the reference builds
with mpif90 over gfortran, default kinds: INTEGER 4 bytes, REAL(8)):
each record is one or more subrecords ``[marker][bytes][marker]``, 4-byte
little-endian markers holding the subrecord's byte count, at most 2147483639
bytes per subrecord; the leading marker is negative when another subrecord
follows, the trailing one when another preceded.

Records of one rank's file (Restart_Mod.f90:28-39): Time (REAL 8), GMVStep
(INTEGER 4), OutputTime (REAL 8); then per block one record per component
``Vec(ib)%Vec(ic)%c`` (the padded cell array, column-major, with its nFrac
extent) and one record with ``uF, vF, wF`` back to back.
"""
from __future__ import annotations

import struct

import numpy as np

GFORTRAN_MAX_SUBRECORD = 2147483639


def file_name(grid_file: str, rank: int) -> str:
    """'RESTART/'//TRIM(FileName(1:INDEX(FileName,'.grid')))//ADJUSTL(iName)
    (Restart_Mod.f90:24-27); Fortran drops the trailing blanks of FILE=."""
    at = grid_file.find(".grid")
    stem = grid_file[:at + 1].rstrip(" ") if at >= 0 else ""
    return f"RESTART/{stem}{rank}"


def encode_record(payload: bytes, max_sub: int = GFORTRAN_MAX_SUBRECORD) -> bytes:
    n = max(1, -(-len(payload) // max_sub))
    out = []
    for k in range(n):
        part = payload[k * max_sub:(k + 1) * max_sub]
        lead = -len(part) if k + 1 < n else len(part)
        tail = -len(part) if k > 0 else len(part)
        out += [struct.pack("<i", lead), part, struct.pack("<i", tail)]
    return b"".join(out)


def decode_records(data: bytes) -> list[bytes]:
    """Split a file into its logical records, checking every marker."""
    recs, pos = [], 0
    while pos < len(data):
        parts, first = [], True
        while True:
            (lead,) = struct.unpack_from("<i", data, pos)
            n = abs(lead)
            part = data[pos + 4:pos + 4 + n]
            if len(part) != n:
                raise ValueError("file ends inside a record")
            (tail,) = struct.unpack_from("<i", data, pos + 4 + n)
            if abs(tail) != n or (tail < 0) != (not first):
                raise ValueError("corrupt record marker")
            parts.append(part)
            pos += 8 + n
            first = False
            if lead >= 0:
                break
        recs.append(b"".join(parts))
    return recs


def block_records(c: np.ndarray, uf: np.ndarray, vf: np.ndarray, wf: np.ndarray) -> list[bytes]:
    """c: (ncomp, ...) float64, one row per component in the padded layout."""
    c = np.ascontiguousarray(c, dtype="<f8")
    recs = [c[ic].tobytes() for ic in range(c.shape[0])]
    recs.append(b"".join(np.ascontiguousarray(a, dtype="<f8").tobytes() for a in (uf, vf, wf)))
    return recs


def encode(time: float, gmv_step: int, output_time: float, blocks, max_sub: int = GFORTRAN_MAX_SUBRECORD) -> bytes:
    """The bytes of one rank's restart file; blocks = [(c, uf, vf, wf), ...]."""
    recs = [struct.pack("<d", time), struct.pack("<i", gmv_step), struct.pack("<d", output_time)]
    for b in blocks:
        recs += block_records(*b)
    return b"".join(encode_record(r, max_sub) for r in recs)


def decode(data: bytes, shapes):
    """Inverse of encode; shapes = [(nx, ny, nz, ncomp, nfrac), ...].  Returns
    (time, gmv_step, output_time, [(c, uf, vf, wf), ...])."""
    recs = decode_records(data)
    if len(recs) < 3:
        raise ValueError("restart file without header")
    (time,) = struct.unpack("<d", recs[0])
    (gmv,) = struct.unpack("<i", recs[1])
    (out_t,) = struct.unpack("<d", recs[2])
    k, blocks = 3, []
    for nx, ny, nz, ncomp, nfrac in shapes:
        npad = (nx + 2) * (ny + 2) * (nz + 2) * max(nfrac, 1)
        c = np.empty((ncomp, npad))
        for ic in range(ncomp):
            c[ic] = np.frombuffer(recs[k], dtype="<f8", count=npad)
            if len(recs[k]) != 8 * npad:
                raise ValueError("component record of the wrong length")
            k += 1
        nu, nv, nw = (nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)
        v = np.frombuffer(recs[k], dtype="<f8")
        if v.size != nu + nv + nw:
            raise ValueError("velocity record of the wrong length")
        blocks.append((c, v[:nu].copy(), v[nu:nu + nv].copy(), v[nu + nv:].copy()))
        k += 1
    return time, gmv, out_t, blocks
