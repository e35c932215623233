"""NIfTI-1 (.nii / .nii.gz) and raw displacement (.dat) files of the deeds boundary.

Mirrors the reference's reader (src/imageIOgzType.h:7-105): a 352-byte header,
dims as int16 at byte 40 (dim[0..4]), datatype/bitpix as int16 at byte 70, data
from byte 352, i fastest.  Supported datatypes 2 (uint8), 4 (int16), 8 (int32),
16 (float32), 64 (float64), 512 (uint16).  Writers emit a correct 352-byte
header (the reference writes 10 bytes from an 8-byte dims buffer,
src/imageIOgzType.h:194-198; that overflow is not reproduced).

``*_displacements.dat`` is raw little-endian float32 ``[u | v | w]`` on the last
control grid (src/deedsBCV0.cpp:341-349); its grid step is inferred from the
file size exactly as applyBCV does (src/applyBCV.cpp:161-164).
"""
from __future__ import annotations

import gzip
import struct

import numpy as np

_DT = {2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64, 512: np.uint16}
_DT_INV = {np.dtype(v): k for k, v in _DT.items()}


def _open(path, mode):
    return gzip.open(path, mode) if str(path).endswith("gz") else open(path, mode)


def read(path):
    """Return (volume as (m, n, o[, p]) Fortran array in its stored dtype, header bytes)."""
    with _open(path, "rb") as f:
        raw = f.read()
    if len(raw) < 352:
        raise ValueError(f"{path}: truncated NIfTI header ({len(raw)} bytes)")
    hdr = raw[:352]
    dims = struct.unpack_from("<8h", hdr, 40)
    dtype_code, bitpix = struct.unpack_from("<2h", hdr, 70)
    if dtype_code not in _DT:
        raise ValueError(f"{path}: datatype {dtype_code} not supported")
    m, n, o, p = (max(int(d), 1) for d in dims[1:5])
    dt = np.dtype(_DT[dtype_code])
    count = m * n * o * p
    offs = int(struct.unpack_from("<f", hdr, 108)[0]) or 352
    data = np.frombuffer(raw, dtype=dt.newbyteorder("<"), count=count, offset=offs) if len(raw) >= offs + count * dt.itemsize else None
    if data is None:
        raise ValueError(f"{path}: truncated data (need {count * dt.itemsize} bytes)")
    shape = (m, n, o) if p == 1 else (m, n, o, p)
    return np.asarray(data, dtype=dt).reshape(shape, order="F"), hdr


def make_header(shape, dtype, template=None):
    hdr = bytearray(template if template is not None else b"\x00" * 352)
    if len(hdr) < 352:
        hdr.extend(b"\x00" * (352 - len(hdr)))
    hdr = hdr[:352]
    struct.pack_into("<i", hdr, 0, 348)
    m, n, o = shape[:3]
    p = shape[3] if len(shape) > 3 else 1
    ndim = 4 if p > 1 else (3 if o > 1 else 2)
    struct.pack_into("<8h", hdr, 40, ndim, m, n, o, p, 1, 1, 1)
    code = _DT_INV[np.dtype(dtype)]
    struct.pack_into("<2h", hdr, 70, code, np.dtype(dtype).itemsize * 8)
    if template is None:
        struct.pack_into("<8f", hdr, 76, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0)
    struct.pack_into("<f", hdr, 108, 352.0)
    if template is None:
        hdr[344:348] = b"n+1\x00"
    return bytes(hdr)


def write(path, vol, header=None, dtype=None):
    vol = np.asarray(vol)
    if dtype is not None:
        vol = vol.astype(dtype)
    hdr = make_header(vol.shape, vol.dtype, header)
    with _open(path, "wb") as f:
        f.write(hdr)
        f.write(np.asarray(vol, dtype=vol.dtype.newbyteorder("<")).tobytes(order="F"))


def write_dat(path, flow):
    np.asarray(flow, dtype="<f4").tofile(path)


def read_dat(path):
    return np.fromfile(path, dtype="<f4")


def grid_step_from_dat(n_floats, m, n, o):
    """applyBCV's inference: round((sz/(len/3))^(1/3)) (src/applyBCV.cpp:163-164)."""
    sz3 = n_floats // 3
    ratio = float(np.float32(m * n * o) / np.float32(sz3))  # float division, as in the reference
    return int(np.floor(ratio ** 0.3333333 + 0.5))  # double pow, round half away from zero
