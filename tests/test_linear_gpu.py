"""linearBCV on the GPU against the reference (golden vectors) and the oracle.

Bit-exact: the affine-only warp, the cost smoothing passes, estimateAffine2
(matrix and number of points), the whole registration (matrix file text and the
warped label map of the reference binary, affine and rigid), the linearBCV
command line on NIfTI files, and a 96x80x128 pair against the oracle.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest
import torch

import pyoracle as orc

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def api():
    from deedsbcv_gb300 import api as A
    return A


def matrix_text(X):
    return "".join("%g  %g  %g  %g\n" % tuple(float(X[i + 4 * j]) for j in range(4)) for i in range(4))


def _cuda(a, dtype=np.float32):
    return torch.from_numpy(np.ascontiguousarray(a, dtype)).cuda()


def test_lin_warp_bit_exact(api, golden):
    g = golden("linear")
    m, n, o = (int(x) for x in g["warp_dims"])
    out = api.warpAffineLinear(_cuda(g["warp_image"]), g["warp_X"], m, n, o).cpu().numpy()
    assert np.array_equal(out.view(np.uint32), g["warp_out"].view(np.uint32))
    # odd sizes, a large shift (many voxels outside) against the oracle
    rng = np.random.default_rng(3)
    m, n, o = 37, 29, 41
    im = rng.normal(0, 300, m * n * o).astype(np.float32)
    X = np.array([0.93, 0.08, -0.05, 6.3, -0.07, 1.05, 0.02, -7.9, 0.04, -0.06, 1.02, 3.1, 0, 0, 0, 1], np.float32)
    out = api.warpAffineLinear(_cuda(im), X, m, n, o).cpu().numpy()
    assert np.array_equal(out.view(np.uint32), orc.lin_warp(im, X, m, n, o).view(np.uint32))


@pytest.mark.parametrize("shape", [(9, 6, 9, 1331), (5, 4, 6, 125), (1, 3, 2, 27), (7, 1, 1, 8), (12, 10, 12, 343)])
def test_lin_smooth_bit_exact(api, shape):
    m1, n1, o1, len3 = shape
    rng = np.random.default_rng(m1 * 100 + len3)
    cost = (rng.integers(0, 4000, m1 * n1 * o1 * len3) * np.float32(0.0123)).astype(np.float32)
    t = _cuda(cost)
    api.smoothCosts(t, m1, n1, o1, len3)
    ref = orc.lin_smooth(cost, m1, n1, o1, len3)
    assert np.array_equal(t.cpu().numpy().view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("kind", ["midpoints", "tiny", "nan", "mixed_sign"])
def test_lin_smooth_both_evaluations_bit_exact(api, kind):
    """The smoothing step runs in float-float when that provably rounds like the
    reference's double expression, else in double: even integers near 2^24 give
    sums on float midpoints (the double path decides), tiny values fall below the
    float-float range, NaN propagates, mixed signs cancel."""
    m1, n1, o1, len3 = 9, 7, 8, 125
    rng = np.random.default_rng(7)
    size = m1 * n1 * o1 * len3
    if kind == "midpoints":
        cost = (16777216.0 + 2.0 * rng.integers(0, 8, size)).astype(np.float32)
    elif kind == "tiny":
        cost = (rng.uniform(0, 1, size) * 1e-30).astype(np.float32)
    elif kind == "nan":
        cost = rng.uniform(0, 100, size).astype(np.float32)
        cost[rng.integers(0, size, 20)] = np.nan
    else:
        cost = rng.normal(0, 1000, size).astype(np.float32)
    t = _cuda(cost)
    api.smoothCosts(t, m1, n1, o1, len3)
    ref = orc.lin_smooth(cost, m1, n1, o1, len3)
    got = t.cpu().numpy()
    both_nan = np.isnan(got) & np.isnan(ref)
    assert np.all(both_nan | (got.view(np.uint32) == ref.view(np.uint32)))


@pytest.mark.parametrize("key", ["5_3_2", "4_2_1"])
@pytest.mark.parametrize("rigid", [0, 1])
def test_estimate_affine_bit_exact(api, golden, key, rigid):
    g = golden("linear")
    m, n, o = (int(x) for x in g["est_dims"])
    gs, hw, q = (int(x) for x in key.split("_"))
    a1 = g[f"est_alpha1_{key}"]
    c1 = _cuda(g[f"est_counts1_{key}"].astype(np.float32) * a1)
    c2 = _cuda(g[f"est_counts2_{key}"].astype(np.float32) * a1)
    f = _cuda(g["est_fixed"].astype(np.float32) + np.float32(1024))
    mv = _cuda(g["est_moving"].astype(np.float32) + np.float32(1024))
    X, used = api.estimateAffine2(g["est_Xprev"], f, mv, c1, c2, m, n, o, gs, q, hw, rigid)
    assert used == int(g[f"est_used_{key}_{rigid}"])
    assert np.array_equal(X.view(np.uint32), g[f"est_X_{key}_{rigid}"].view(np.uint32))
    if rigid == 0:
        assert hashlib.sha256(c1.cpu().numpy().tobytes()).digest() == g[f"est_smooth1_sha256_{key}"].tobytes()
        assert hashlib.sha256(c2.cpu().numpy().tobytes()).digest() == g[f"est_smooth2_sha256_{key}"].tobytes()


@pytest.mark.parametrize("rigid", [0, 1])
def test_linear_register_matches_reference_binary(api, golden, rigid):
    g = golden("linear")
    dims = tuple(int(x) for x in g["e2e_dims"])
    f = g["e2e_fixed"].astype(np.float32)
    mv = g["e2e_moving"].astype(np.float32)
    X = api.linear_register(f, mv, dims, api.linear_params(rigid=rigid))
    assert matrix_text(X) == bytes(g[f"e2e_matrix_txt_{rigid}"]).decode()
    seg = api.affine_warp_segmentation(g["e2e_moving_labels"], dims, X)
    assert np.array_equal(seg, g[f"e2e_seg_{rigid}"])
    # device-pointer entry gives the same bits
    Xd = api.linear_register(_cuda(f), _cuda(mv), dims, api.linear_params(rigid=rigid))
    assert np.array_equal(Xd.view(np.uint32), X.view(np.uint32))


def test_linear_cli_matches_reference_binary(golden, tmp_path):
    from deedsbcv_gb300 import nifti
    g = golden("linear")
    m, n, o = (int(x) for x in g["e2e_dims"])
    shp = lambda a: np.asarray(a).reshape((m, n, o), order="F")  # noqa: E731
    nifti.write(str(tmp_path / "f.nii.gz"), shp(g["e2e_fixed"]).astype(np.int16))
    nifti.write(str(tmp_path / "m.nii.gz"), shp(g["e2e_moving"]).astype(np.int16))
    nifti.write(str(tmp_path / "s.nii.gz"), shp(g["e2e_moving_labels"]).astype(np.int16))
    exe = os.path.join(ROOT, "deedsbcv_gb300", "_build", "linearBCV")
    for rigid in (0, 1):
        stem = str(tmp_path / f"out{rigid}")
        args = [exe, "-F", str(tmp_path / "f.nii.gz"), "-M", str(tmp_path / "m.nii.gz"), "-O", stem,
                "-S", str(tmp_path / "s.nii.gz")] + (["-R", "1"] if rigid else [])
        r = subprocess.run(args, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "# points used:" in r.stdout
        with open(stem + "_matrix.txt") as fh:
            assert fh.read() == bytes(g[f"e2e_matrix_txt_{rigid}"]).decode()
        seg, _ = nifti.read(stem + "_deformed_seg.nii.gz")
        assert np.array_equal(seg.ravel(order="F").astype(np.int16), g[f"e2e_seg_{rigid}"])


@pytest.mark.parametrize("rigid", [0, 1])
def test_linear_register_matches_oracle_96x80x128(api, rigid):
    from deedsbcv_gb300 import phantom
    dims = (96, 80, 128)
    pr = phantom.make_pair(dims, seed=11, max_disp=2.0, affine=(6.0, 0.06, 5.0))
    f = pr["fixed"].ravel(order="F").astype(np.float32)
    mv = pr["moving"].ravel(order="F").astype(np.float32)
    X = api.linear_register(f, mv, dims, api.linear_params(rigid=rigid))
    ref = orc.linear_register(f + np.float32(1024), mv + np.float32(1024), *dims, rigid=rigid)
    assert np.array_equal(X.view(np.uint32), ref.view(np.uint32))


def test_linear_invalid_arguments_raise(api):
    from deedsbcv_gb300._lib import DeedsError
    f = np.zeros(20 * 20 * 20, np.float32)
    with pytest.raises(DeedsError):  # grid 7 leaves fewer than 5 control points per axis
        api.linear_register(f, f, (20, 20, 20))
    with pytest.raises(DeedsError):  # an all-background pair has no usable control points
        api.linear_register(np.full(48 ** 3, -1000, np.float32), np.full(48 ** 3, -1000, np.float32), (48, 48, 48),
                            api.linear_params(grid=(6,), radius=(2,), quant=(2,)))
