"""Parallel gzip IO of the NIfTI volumes (host code of the library, no device).

Files written in parallel chunks are ordinary multi-member gzip (any gzip reader
returns the original bytes); the library's reader inflates its own files in
parallel and any other gzip file through zlib; the size query and the
too-small-buffer contract of deeds_gz_read.
"""
import ctypes as C
import gzip

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L():
    from deedsbcv_gb300 import _lib
    return _lib.load()


def _write(L, path, head, data, threads=0):
    st = L.deeds_gz_write(str(path).encode(), head.ctypes.data_as(C.c_void_p), head.nbytes,
                          data.ctypes.data_as(C.c_void_p), data.nbytes, -1, threads)
    assert st == 0, L.deeds_gz_last_error()


def _read(L, path, cap=None, threads=0):
    total = C.c_size_t(0)
    assert L.deeds_gz_read(str(path).encode(), None, 0, C.byref(total), threads) == 0
    n = total.value if cap is None else cap
    out = np.zeros(max(n, 1), np.uint8)
    st = L.deeds_gz_read(str(path).encode(), out.ctypes.data_as(C.c_void_p), n, C.byref(total), threads)
    return st, out[:n], total.value


@pytest.mark.parametrize("nbytes", [0, 1000, (4 << 20) - 352, 10_000_003])
def test_parallel_gzip_round_trip(L, tmp_path, nbytes):
    rng = np.random.default_rng(nbytes)
    head = rng.integers(0, 256, 352, dtype=np.uint8)
    # half noise, half runs: members compress differently
    data = rng.integers(0, 256, nbytes, dtype=np.uint8)
    data[: nbytes // 2] = (np.arange(nbytes // 2) // 977 % 7).astype(np.uint8)
    p = tmp_path / "v.nii.gz"
    _write(L, p, head, data)
    ref = np.concatenate([head, data])
    with gzip.open(p, "rb") as f:  # a standard reader: concatenated members
        assert f.read() == ref.tobytes()
    for threads in (0, 1, 3):
        st, out, total = _read(L, p, threads=threads)
        assert st == 0 and total == ref.size and out.tobytes() == ref.tobytes()


def test_reader_accepts_single_member_and_plain_files(L, tmp_path):
    data = np.random.default_rng(1).integers(0, 256, 3_000_001, dtype=np.uint8).tobytes()
    p = tmp_path / "single.gz"
    with gzip.open(p, "wb") as f:
        f.write(data)
    st, out, total = _read(L, p)
    assert st == 0 and out.tobytes() == data
    q = tmp_path / "plain.nii"
    q.write_bytes(data[:12345])
    st, out, total = _read(L, q)
    assert st == 0 and out.tobytes() == data[:12345]


def test_too_small_buffer_reports_size(L, tmp_path):
    head = np.zeros(352, np.uint8)
    data = np.arange(9_000_000, dtype=np.uint8)
    p = tmp_path / "v.nii.gz"
    _write(L, p, head, data)
    st, _, total = _read(L, p, cap=1000)
    assert st != 0 and total == 352 + data.size
    g = tmp_path / "single.gz"
    with gzip.open(g, "wb") as f:
        f.write(data.tobytes())
    st, _, total = _read(L, g, cap=1000)
    assert st != 0 and total == data.size
