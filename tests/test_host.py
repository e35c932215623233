"""CPU-side checks of the product: the C ABI library loads and exports every
declared symbol, its host-side MST code matches the reference, and the
command-line / file-format boundary behaves like the reference's."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import pyoracle as orc
from deedsbcv_gb300 import _lib, nifti, phantom

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "deedsbcv_gb300", "_build")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from deedsbcv_gb300 import build
        build.build()
    return _lib.load()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "deeds_gpu.h")).read()
    return sorted(set(re.findall(r"\b(deeds_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    declared = header_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_lib.EXPORTS)


def test_create_without_gpu_reports_error(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = lib.deeds_create(C.byref(h), 0)
    assert st == 2  # DEEDS_ERR_CUDA, no crash, no exit()
    assert lib.deeds_last_error(None)
    assert lib.deeds_version().startswith(b"deeds")


@pytest.mark.parametrize("gs", [4, 5, 6, 8])
def test_host_prims_matches_reference(lib, golden, gs):
    p = golden("prims")
    m, n, o = (int(x) for x in p["dims"])
    sad = orc.edge_sad(p["image"], m, n, o, gs)
    mean = np.zeros(1, np.float32)
    sd = np.zeros(1, np.float32)
    im = np.ascontiguousarray(p["image"], np.float32)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert lib.deeds_image_stats(ptr(im), im.size, ptr(mean), ptr(sd)) == 0
    assert (float(mean[0]), float(sd[0])) == orc.image_stats(im)
    m1, n1, o1 = m // gs, n // gs, o // gs
    ordered = np.zeros(m1 * n1 * o1, np.int32)
    parents = np.zeros_like(ordered)
    edgemst = np.zeros(m1 * n1 * o1, np.float32)
    assert lib.deeds_prims_from_sad(ptr(sad), C.c_float(sd[0]), m1, n1, o1, gs, ptr(ordered), ptr(parents),
                                    ptr(edgemst)) == 0
    assert np.array_equal(ordered, p[f"ordered_{gs}"])
    assert np.array_equal(parents, p[f"parents_{gs}"])
    assert edgemst.tobytes() == p[f"edgemst_{gs}"].tobytes()


def test_nifti_roundtrip(tmp_path):
    vol = np.asfortranarray(np.random.default_rng(0).normal(size=(7, 5, 6)).astype(np.float32))
    for name in ("a.nii.gz", "a.nii"):
        nifti.write(tmp_path / name, vol)
        back, hdr = nifti.read(tmp_path / name)
        assert back.shape == vol.shape and np.array_equal(back, vol)
        assert len(hdr) == 352
    seg = np.asfortranarray(np.arange(7 * 5 * 6, dtype=np.int16).reshape(7, 5, 6, order="F"))
    nifti.write(tmp_path / "s.nii.gz", seg)
    back, _ = nifti.read(tmp_path / "s.nii.gz")
    assert back.dtype == np.int16 and np.array_equal(back, seg)


def test_truncated_nifti_raises(tmp_path):
    p = tmp_path / "t.nii.gz"
    nifti.write(p, np.zeros((4, 4, 4), np.float32))
    import gzip
    raw = gzip.open(p).read()[:400]
    with gzip.open(p, "wb") as f:
        f.write(raw)
    with pytest.raises(ValueError):
        nifti.read(p)


@pytest.mark.parametrize("g", [4, 5, 6, 8])
def test_grid_step_inferred_from_dat_size(g):
    m, n, o = 192, 160, 256
    sz1 = (m // g) * (n // g) * (o // g)
    assert nifti.grid_step_from_dat(3 * sz1, m, n, o) == g


def _cli(*args):
    exe = os.path.join(BUILD, "deedsBCV")
    if not os.path.exists(exe):
        pytest.skip("CLI not built")
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=60)


@pytest.fixture()
def pair_files(tmp_path):
    pair = phantom.make_pair((24, 20, 28), seed=1, n_organs=4, max_disp=2.0)
    f, m = tmp_path / "f.nii.gz", tmp_path / "m.nii.gz"
    nifti.write(f, pair["fixed"])
    nifti.write(m, pair["moving"])
    return str(f), str(m), str(tmp_path / "out")


@pytest.mark.parametrize("flags,expect", [
    ([], "levels=5 G=8x7x6x5x4 L=8x7x6x5x4 Q=5x4x3x2x1 alpha=1.6"),
    (["-G", "6x5x4", "-L", "5x4x3", "-Q", "3x2x1", "-a", "2"], "levels=3 G=6x5x4 L=5x4x3 Q=3x2x1 alpha=2"),
    # -l is overridden once any of -G/-L/-Q is given (src/parseArguments.h:122-124)
    (["-l", "3", "-L", "6x5"], "levels=5 G=8x7x6x5x4 L=6x5x6x5x4 Q=5x4x3x2x1"),
    # levels beyond 5 take the built-in defaults (src/parseArguments.h:42-44)
    (["-l", "6"], "levels=6 G=8x7x6x5x4x3 L=8x7x6x5x4x3 Q=5x4x3x2x1x1"),
])
def test_cli_parses_like_reference(pair_files, flags, expect):
    f, m, out = pair_files
    r = _cli("-F", f, "-M", m, "-O", out, *flags)
    assert expect in r.stdout, r.stdout + r.stderr


def test_cli_rejects_non_gz(tmp_path, pair_files):
    f, m, out = pair_files
    r = _cli("-F", f.replace(".nii.gz", ".nii"), "-M", m, "-O", out)
    assert "images must have nii.gz format" in r.stdout


def test_cli_mismatch_warning(pair_files):
    f, m, out = pair_files
    r = _cli("-F", f, "-M", m, "-O", out, "-G", "6x5x4", "-L", "5x4")
    assert "#grid=3, #search=2" in r.stdout


def _linear_cli(*args):
    exe = os.path.join(BUILD, "linearBCV")
    if not os.path.exists(exe):
        pytest.skip("CLI not built")
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=60)


@pytest.mark.parametrize("flags,expect", [
    ([], "levels=4 G=7x6x5x4 L=5x4x3x2 Q=4x3x2x1 affine"),  # src/linearBCV.cpp:86-89
    (["-G", "6x5", "-L", "4x3", "-Q", "3x2"], "levels=2 G=6x5 L=4x3 Q=3x2 affine"),
    (["-R", "1"], "levels=4 G=7x6x5x4 L=5x4x3x2 Q=4x3x2x1 rigid"),
])
def test_linear_cli_parses_like_reference(pair_files, flags, expect):
    f, m, out = pair_files
    r = _linear_cli("-F", f, "-M", m, "-O", out, *flags)
    assert "Starting linear reg. of f.nii.gz and m.nii.gz" in r.stdout
    assert expect in r.stdout, r.stdout
    if "-R" in flags:
        assert "Searching only for rigid (6 parameter) transform" in r.stdout


def test_linear_cli_usage_and_non_gz(tmp_path, pair_files):
    r = _linear_cli("-h", "x", "y")
    assert r.returncode == 1 and "./linearBCV -F fixed.nii.gz -M moving.nii.gz -O output" in r.stdout
    f, m, out = pair_files
    plain = tmp_path / "f.nii"
    plain.write_bytes(b"\0" * 400)
    r = _linear_cli("-F", str(plain), "-M", m, "-O", out)
    assert "images must have nii.gz format" in r.stdout and r.returncode != 0


def _stats_case(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "ct_integers":  # many exact ties when the running sum's grid step exceeds 1
        return rng.choice(np.array([-1000.0, -1000.0, 0.0, 40.0, 1200.0], np.float32), n) + \
            rng.integers(-50, 50, n).astype(np.float32)
    if kind == "uniform":
        return rng.uniform(-1024, 3000, n).astype(np.float32)
    if kind == "crossing_zero":  # the sum wanders around zero through many binades
        return rng.normal(0, 100, n).astype(np.float32)
    if kind == "negative":
        return -rng.uniform(0, 4000, n).astype(np.float32)
    if kind == "offset":
        return (1e6 + rng.uniform(0, 1, n)).astype(np.float32)
    if kind == "huge":
        return (rng.uniform(0.5, 1, n) * 1e30).astype(np.float32)
    if kind == "tiny":
        return (rng.uniform(-1, 1, n) * 1e-30).astype(np.float32)
    if kind == "constant":
        return np.full(n, 37.25, np.float32)
    if kind == "steps":  # long runs of one value, then a jump
        return np.repeat(rng.uniform(-500, 500, n // 4096 + 1), 4096)[:n].astype(np.float32)
    x = rng.uniform(0, 100, n).astype(np.float32)  # nan / inf
    x[n // 3] = np.nan if kind == "nan" else np.inf
    return x


@pytest.mark.parametrize("kind", ["ct_integers", "uniform", "crossing_zero", "negative", "offset", "huge", "tiny",
                                  "constant", "steps", "nan", "inf"])
@pytest.mark.parametrize("n", [(1 << 20) + 12345, 3 * 1000 * 1000])
def test_image_stats_parallel_chunks_match_sequential_reference(lib, kind, n):
    """The library evaluates the reference's sequential float sums in parallel
    chunks (exact by a grid-translation argument); every case must give the
    sequential oracle's mean and standard deviation to the bit."""
    im = np.ascontiguousarray(_stats_case(kind, n, 5), np.float32)
    mean = np.zeros(1, np.float32)
    sd = np.zeros(1, np.float32)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert lib.deeds_image_stats(ptr(im), im.size, ptr(mean), ptr(sd)) == 0
    rm, rs = orc.image_stats(im)
    got = np.array([mean[0], sd[0]], np.float32)
    ref = np.array([rm, rs], np.float32)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)) or \
        (np.isnan(got).tolist() == np.isnan(ref).tolist() and np.array_equal(got[~np.isnan(got)], ref[~np.isnan(ref)])), \
        (kind, got, ref)


@pytest.mark.parametrize("dims,levels", [((48, 40, 64), 4), ((13, 11, 17), 6), ((24, 20, 32), 2)])
def test_host_prims_tie_heavy_matches_oracle(lib, dims, levels):
    """Block SADs drawn from a few values make most edge weights bit-equal, so
    the tree is decided by the heap's element moves alone: the library's heap
    (vertex-major weights, aligned storage, prefetching) must pop in exactly the
    order of the oracle's std::push_heap / std::pop_heap restatement."""
    m1, n1, o1 = dims
    sz = m1 * n1 * o1
    rng = np.random.default_rng(sz + levels)
    sad = (rng.integers(0, levels, 6 * sz) * np.float32(64.0)).astype(np.float32)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    got = [np.zeros(sz, np.int32), np.zeros(sz, np.int32), np.zeros(sz, np.float32)]
    ref = [np.zeros(sz, np.int32), np.zeros(sz, np.int32), np.zeros(sz, np.float32)]
    assert lib.deeds_prims_from_sad(ptr(sad), C.c_float(37.5), m1, n1, o1, 4, *(ptr(a) for a in got)) == 0
    orc.lib().orc_prims_from_sad(ptr(sad), C.c_float(37.5), m1, n1, o1, 4, *(ptr(a) for a in ref))
    for a, b in zip(got, ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def _symmetric_sad(m1, n1, o1, draw):
    """Per-node SADs to the 6 neighbours (nb order -x,+x,-y,+y,-z,+z) with one value
    per undirected edge, as block SADs of an image have; 0 off the grid."""
    sz = m1 * n1 * o1
    sad = np.zeros(6 * sz, np.float32)
    v = np.arange(sz)
    i, j, k = v % m1, (v // m1) % n1, v // (m1 * n1)
    for ax, (ok, step) in enumerate(((j + 1 < n1, m1), (i + 1 < m1, 1), (k + 1 < o1, m1 * n1))):
        src = v[ok]
        vals = draw(src.size).astype(np.float32)
        sad[(2 * ax + 1) * sz + src] = vals
        sad[(2 * ax) * sz + src + step] = vals
    return sad


def _prims_both(lib, sad, sd, dims, g):
    m1, n1, o1 = dims
    sz = m1 * n1 * o1
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    got = [np.zeros(sz, np.int32), np.zeros(sz, np.int32), np.zeros(sz, np.float32)]
    ref = [np.zeros(sz, np.int32), np.zeros(sz, np.int32), np.zeros(sz, np.float32)]
    assert lib.deeds_prims_from_sad(ptr(sad), C.c_float(sd), m1, n1, o1, g, *(ptr(a) for a in got)) == 0
    orc.lib().orc_prims_from_sad(ptr(sad), C.c_float(sd), m1, n1, o1, g, *(ptr(a) for a in ref))
    return got, ref


def _counts(lib):
    a = (C.c_longlong * 4)()
    lib.deeds_mst_path_counts(a)
    return list(a)


@pytest.mark.parametrize("dims", [(24, 20, 32), (13, 11, 17), (1, 9, 7), (5, 1, 6)])
def test_unique_mst_without_prim_walk(lib, dims):
    """Continuous edge weights: the minimum spanning tree is unique, so the
    library builds it by Kruskal's grouping alone (no heap walk); it must be
    Prim's tree node for node."""
    rng = np.random.default_rng(sum(dims))
    sad = _symmetric_sad(*dims, lambda k: rng.uniform(0, 5000, k))
    before = _counts(lib)
    got, ref = _prims_both(lib, sad, 137.0, dims, 4)
    after = _counts(lib)
    for a, b in zip(got, ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert after[0] - before[0] == 1 and after[2] == before[2], (before, after)


@pytest.mark.parametrize("dims,levels", [((24, 20, 32), 40), ((48, 40, 64), 400), ((13, 11, 17), 3),
                                         ((100, 90, 8), 50), ((300, 250, 1), 20)])
def test_ambiguous_ties_decided_by_partial_prim_walk(lib, dims, levels):
    """Symmetric SADs from a few values: many equal weights on cycles, so Prim's
    heap decides ties.  The library walks Prim's heap only until every ambiguous
    group has its picks and takes the rest from Kruskal's forced edges; the tree
    must still equal the full walk's.  Trees of 2^16 nodes and more have their
    weights evaluated in slab blocks by helper threads while the walk starts
    (one slab per block where a slab holds more than 8192 nodes, one block for a
    single slab)."""
    rng = np.random.default_rng(levels)
    sad = _symmetric_sad(*dims, lambda k: rng.integers(0, levels, k) * 64.0)
    before = _counts(lib)
    got, ref = _prims_both(lib, sad, 37.5, dims, 4)
    after = _counts(lib)
    for a, b in zip(got, ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert after[1] - before[1] == 1


def test_mst_paths_on_phantom_levels(lib):
    """Block SADs of a CT-like phantom at every default grid: trees identical to
    the oracle's full Prim walk, whichever construction each level takes."""
    shape = (96, 80, 128)
    pair = phantom.make_pair(shape, seed=11)
    for name in ("fixed", "moving"):
        im = np.ascontiguousarray(pair[name].ravel(order="F") + np.float32(1024), np.float32)
        _, sd = orc.image_stats(im)
        for g in (8, 7, 6, 5, 4):
            sad = orc.edge_sad(im, *shape, g)
            dims = tuple(s // g for s in shape)
            got, ref = _prims_both(lib, sad, sd, dims, g)
            for a, b in zip(got, ref):
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (name, g)


def test_nan_weights_take_the_full_walk(lib):
    """A zero standard deviation makes zero SADs NaN weights: the order is then the
    heap's alone, so the library walks it fully, as the reference."""
    dims = (9, 7, 5)
    rng = np.random.default_rng(3)
    sad = _symmetric_sad(*dims, lambda k: rng.integers(0, 3, k) * 8.0)
    got, ref = _prims_both(lib, sad, 0.0, dims, 2)
    for a, b in zip(got, ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
