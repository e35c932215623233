"""Pin the linearBCV restatement (oracle/deeds_oracle.cpp) to the reference.

Golden vectors come from the unmodified reference (tests/golden/make_golden.py):
its affine-only warp, QR inverse, affineRobust and estimateAffine2 through the
stage harness oracle/ref_linear.cpp, and the linearBCV binary end to end (matrix
file text and the warped label map) for an affine and a rigid fit.
"""
import hashlib

import numpy as np
import pytest

import pyoracle as orc

IDENT = np.eye(4, dtype=np.float32).ravel()


def matrix_text(X):
    """The matrix file as src/linearBCV.cpp:286-293 writes it (ostream default
    float format, 6 significant digits)."""
    return "".join("%g  %g  %g  %g\n" % tuple(float(X[i + 4 * j]) for j in range(4)) for i in range(4))


def test_linear_warp_and_qr_inverse_bit_exact(golden):
    g = golden("linear")
    m, n, o = (int(x) for x in g["warp_dims"])
    out = orc.lin_warp(g["warp_image"], g["warp_X"], m, n, o)
    assert np.array_equal(out.view(np.uint32), g["warp_out"].view(np.uint32))
    assert (out == 0).any() and (out != 0).any()  # both branches of the bounds test are exercised
    Xi = orc.qrsolve(g["warp_X"], IDENT, 4, 4)
    assert np.array_equal(Xi.view(np.uint32), g["qrinv"].view(np.uint32))


@pytest.mark.parametrize("rigid", [0, 1])
def test_affine_robust_bit_exact(golden, rigid):
    g = golden("linear")
    npts = g["robust_p1"].size // 4
    RT = orc.affine_robust(g["robust_p1"], g["robust_p2"], npts, rigid)
    assert np.array_equal(RT.view(np.uint32), g[f"robust_{rigid}"].view(np.uint32))


@pytest.mark.parametrize("key", ["5_3_2", "4_2_1"])
@pytest.mark.parametrize("rigid", [0, 1])
def test_estimate_affine_bit_exact(golden, key, rigid):
    g = golden("linear")
    m, n, o = (int(x) for x in g["est_dims"])
    gs, hw, q = (int(x) for x in key.split("_"))
    a1 = g[f"est_alpha1_{key}"]
    c1 = g[f"est_counts1_{key}"].astype(np.float32) * a1
    c2 = g[f"est_counts2_{key}"].astype(np.float32) * a1
    f = g["est_fixed"].astype(np.float32) + np.float32(1024)
    mv = g["est_moving"].astype(np.float32) + np.float32(1024)
    X, s1, s2, used = orc.estimate_affine(g["est_Xprev"], f, mv, c1, c2, m, n, o, gs, q, hw, rigid)
    assert used == int(g[f"est_used_{key}_{rigid}"])
    assert np.array_equal(X.view(np.uint32), g[f"est_X_{key}_{rigid}"].view(np.uint32))
    if rigid == 0:
        assert hashlib.sha256(s1.tobytes()).digest() == g[f"est_smooth1_sha256_{key}"].tobytes()
        assert hashlib.sha256(s2.tobytes()).digest() == g[f"est_smooth2_sha256_{key}"].tobytes()


@pytest.mark.parametrize("rigid", [0, 1])
def test_linear_register_matches_reference_binary(golden, rigid):
    g = golden("linear")
    m, n, o = (int(x) for x in g["e2e_dims"])
    f = g["e2e_fixed"].astype(np.float32) + np.float32(1024)
    mv = g["e2e_moving"].astype(np.float32) + np.float32(1024)
    X = orc.linear_register(f, mv, m, n, o, rigid=rigid)
    assert matrix_text(X) == bytes(g[f"e2e_matrix_txt_{rigid}"]).decode()
    zero = np.zeros(m * n * o, np.float32)
    seg = orc.warp_affine_s(g["e2e_moving_labels"].astype(np.int16), X, zero, zero, zero, m, n, o)
    assert np.array_equal(seg, g[f"e2e_seg_{rigid}"])
    # the fit recovers the phantom's misalignment: X is close to the inverse of the true map
    A = g["e2e_true_affine"].reshape(4, 4).astype(np.float64)
    Xm = np.array([[X[i * 4 + j] for j in range(4)] for i in range(3)] + [[0, 0, 0, 1]], np.float64)
    centre = np.array([m / 2, n / 2, o / 2, 1.0])
    assert np.abs((A @ Xm) @ centre - centre)[:3].max() < 1.5


@pytest.mark.parametrize("rigid", [0, 1])
def test_library_host_fit_bit_exact(golden, rigid):
    """The library's own least-trimmed-squares fit (host code, no device calls)
    against the reference's affineRobust."""
    from deedsbcv_gb300 import api
    g = golden("linear")
    npts = g["robust_p1"].size // 4
    RT = api.affineRobust(g["robust_p1"], g["robust_p2"], npts, rigid)
    assert np.array_equal(RT.view(np.uint32), g[f"robust_{rigid}"].view(np.uint32))


@pytest.mark.parametrize("npts,rigid", [(40001, 0), (40001, 1), (9, 0), (9, 1)])
def test_library_host_fit_matches_oracle_large(npts, rigid):
    """The library's fit (fused Gram-Schmidt passes, radix median) against the
    oracle's plain restatement on seeded point sets with 20% outliers."""
    from deedsbcv_gb300 import api
    rng = np.random.default_rng(npts + rigid)
    p1 = np.ones((4, npts), np.float32)
    p1[:3] = rng.uniform(0, 200, (3, npts))
    p2 = p1.copy()
    p2[:3] += rng.normal(0, 1, (3, npts)).astype(np.float32)
    out = rng.choice(npts, npts // 5, replace=False)
    p2[:3, out] += rng.uniform(-20, 20, (3, out.size)).astype(np.float32)
    RT = api.affineRobust(p1.ravel(), p2.ravel(), npts, rigid)
    ref = orc.affine_robust(p1.ravel(), p2.ravel(), npts, rigid)
    assert np.array_equal(RT.view(np.uint32), ref.view(np.uint32))
