"""Warps and field upsampling against the oracle, bit for bit, on inputs chosen to
exercise both evaluations of the trilinear blend.

The GPU kernels evaluate each blend in float-float and keep the result only when
it provably rounds like the reference's double expression; otherwise they
evaluate the double expression.  The inputs here: CT-like values with
fractional displacements (the float-float path almost everywhere), values near
2^24 with dyadic displacements (blends that land exactly on midpoints between
floats, so the double path must decide), tiny values (below the float-float
path's range) and NaNs.  Every output must equal the oracle's (src/dataCostD.h,
src/transformations.h, src/affineLTS1.h restated in oracle/).
"""
import numpy as np
import pytest

import pyoracle as orc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DIMS = (40, 32, 48)
GRID = (10, 8, 12)


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from deedsbcv_gb300 import api as _api
    _api.context(0)
    return _api


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def same(a, b):
    """Equal bits, or NaN in both (the NaN payload may differ between CPU and GPU)."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    nan = np.isnan(a) & np.isnan(b)
    return a.shape == b.shape and bool(np.all(nan | (a.view(np.uint32) == b.view(np.uint32))))


def _case(kind, seed):
    rng = np.random.default_rng(seed)
    m, n, o = DIMS
    sz = m * n * o
    g = GRID[0] * GRID[1] * GRID[2]
    if kind == "ct":
        im = rng.uniform(-1024, 3000, sz).astype(np.float32)
        grid = [rng.uniform(-4, 4, g).astype(np.float32) for _ in range(3)]
    elif kind == "midpoints":
        # even integers above 2^24 are spaced 2 apart: blends with dyadic weights hit
        # the odd integers between them, exactly on a midpoint
        im = (16777216.0 + 2.0 * rng.integers(0, 64, sz)).astype(np.float32)
        grid = [(rng.integers(-8, 9, g) * 0.25).astype(np.float32) for _ in range(3)]
    elif kind == "tiny":
        im = (rng.uniform(-1, 1, sz) * 1e-33).astype(np.float32)
        grid = [rng.uniform(-3, 3, g).astype(np.float32) for _ in range(3)]
    else:  # nan
        im = rng.uniform(0, 100, sz).astype(np.float32)
        im[rng.integers(0, sz, 50)] = np.nan
        grid = [rng.uniform(-3, 3, g).astype(np.float32) for _ in range(3)]
    return im, grid


@pytest.mark.parametrize("kind", ["ct", "midpoints", "tiny", "nan"])
def test_upsample_and_warps_bit_exact(api, kind):
    m, n, o = DIMS
    m2, n2, o2 = GRID
    im, grid = _case(kind, 11)
    up = api.upsampleDeformationsCL(cu(grid[0]), cu(grid[1]), cu(grid[2]), m2, n2, o2, m, n, o)
    ref_up = orc.upsample(grid[0], grid[1], grid[2], m, n, o, m2, n2, o2)
    for a, b in zip(up, ref_up):
        assert same(host(a), b)
    X = np.eye(4, dtype=np.float32).ravel()
    X[[0, 5, 10]] = [1.02, 0.97, 1.01]
    X[[3, 7, 11]] = [0.75, -1.5, 0.25]
    assert same(host(api.warpAffine(cu(im), X, *up, m, n, o)), orc.warp_affine(im, X, *ref_up, m, n, o))
    assert same(host(api.warpImageCL(cu(im), *up, m, n, o)), orc.warp_image(im, *ref_up, m, n, o))
    assert same(host(api.warpAffineLinear(cu(im), X, m, n, o)), orc.lin_warp(im, X, m, n, o))


def _blend_double(im, u, v, w, dims):
    """warpImageCL's blend in float64, in the reference's types and order (the
    oracle's value before its final rounding to float)."""
    m, n, o = dims
    f32 = np.float32
    im3 = im.reshape(o, n, m)  # [k, j, i]
    k, j, i = np.meshgrid(np.arange(o), np.arange(n), np.arange(m), indexing="ij")
    U, V, W = (a.reshape(o, n, m) for a in (u, v, w))
    x, y, z = np.floor(U), np.floor(V), np.floor(W)
    dx, dy, dz = (U - x).astype(f32), (V - y).astype(f32), (W - z).astype(f32)
    x, y, z = x.astype(np.int64) + j, y.astype(np.int64) + i, z.astype(np.int64) + k
    cl = lambda a, hi: np.clip(a, 0, hi - 1)  # noqa: E731
    y0, y1, x0, x1, z0, z1 = cl(y, m), cl(y + 1, m), cl(x, n), cl(x + 1, n), cl(z, o), cl(z + 1, o)
    c = lambda yy, xx, zz: im3[zz, xx, yy].astype(np.float64)  # noqa: E731
    ddx, ddy, ddz = dx.astype(np.float64), dy.astype(np.float64), dz.astype(np.float64)
    a_, b_, c_ = 1.0 - ddx, 1.0 - ddy, 1.0 - ddz
    ab, ady, dxb = a_ * b_, a_ * ddy, ddx * b_
    dxdy = (dx * dy).astype(f32)
    acc = ab * c_ * c(y0, x0, z0)
    acc = acc + ady * c_ * c(y1, x0, z0)
    acc = acc + dxb * c_ * c(y0, x1, z0)
    acc = acc + ab * ddz * c(y0, x0, z1)
    acc = acc + dxdy.astype(np.float64) * c_ * c(y1, x1, z0)
    acc = acc + ady * ddz * c(y1, x0, z1)
    acc = acc + dxb * ddz * c(y0, x1, z1)
    acc = acc + ((dxdy * dz).astype(f32) * im3[z1, x1, y1]).astype(f32).astype(np.float64)
    return acc.ravel()


def test_midpoint_inputs_reach_the_double_path():
    """Some warp blends of the midpoint inputs lie exactly halfway between two
    floats: no float-float value can decide those, so the comparison in
    test_upsample_and_warps_bit_exact covers the double path too."""
    m, n, o = DIMS
    m2, n2, o2 = GRID
    im, grid = _case("midpoints", 11)
    u, v, w = orc.upsample(grid[0], grid[1], grid[2], m, n, o, m2, n2, o2)
    acc = _blend_double(im, u, v, w, DIMS)
    f = acc.astype(np.float32)
    assert np.array_equal(f, orc.warp_image(im, u, v, w, m, n, o))  # the replication is the oracle's
    nxt = np.nextafter(f, np.where(acc > f, np.float32(np.inf), np.float32(-np.inf)).astype(np.float32))
    tie = (acc != f) & ((acc - f.astype(np.float64)) == (nxt.astype(np.float64) - acc))
    assert tie.sum() >= 20, tie.sum()
