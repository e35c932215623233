"""Parity at the benchmark workloads' full sizes: the GPU registration through the
C ABI against the oracle (oracle/deeds_oracle.cpp, itself pinned bit for bit to the
reference's binaries by tests/test_oracle_golden.py) on the same seeded inputs.

The workloads are the synthetic stand-ins for the reference's datasets:
  * 192x160x256 CT-like pair, 13 organs, 10-voxel B-spline deformation (seed 2,
    the benchmark's pair), default 5 levels;
  * 192x192x208 cross-contrast pair (per-organ intensity remap, inverted
    background, 0.7-1.3 bias field, Rician noise, 12-voxel deformation);
  * the two largest pairs of the 16-pair uneven batch (dims drawn from
    128x112x144 .. 224x192x288), registered through the batched entry point
    together with the smallest pair.

Contract (end to end, where stage inputs differ after the first level):
argmin displacements identical on >= 99.9 % of control points and warped-label
Dice within 0.1 points (0.001) of the oracle's.
"""
import numpy as np
import pytest

import pyoracle as orc

torch = pytest.importorskip("torch")
pytestmark = [pytest.mark.gpu, pytest.mark.slow]

ARGMIN_AGREE = 0.999
DICE_TOL = 0.001


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from deedsbcv_gb300 import api as _api
    _api.context(0)
    return _api


def _against_oracle(api, pair, flow):
    from deedsbcv_gb300 import phantom
    shape = pair["fixed"].shape
    f = pair["fixed"].ravel(order="F") + np.float32(1024)
    mv = pair["moving"].ravel(order="F") + np.float32(1024)
    rflow, ux, vx, wx, _ = orc.register(f, mv, *shape, want_full=True)
    agree = float(np.mean(flow == rflow))
    labels = pair["moving_labels"].astype(np.int16)
    seg_gpu = api.apply_flow(flow, labels, dims=shape)
    seg_ref = orc.warp_affine_s(labels, np.eye(4, dtype=np.float32).ravel(), ux, vx, wx, *shape)
    lab = pair["fixed_labels"].ravel(order="F")
    d_gpu, d_ref = phantom.dice(lab, seg_gpu), phantom.dice(lab, seg_ref)
    assert agree >= ARGMIN_AGREE, (shape, agree)
    assert abs(d_gpu - d_ref) <= DICE_TOL, (shape, d_gpu, d_ref)
    assert d_gpu > phantom.dice(lab, pair["moving_labels"].ravel(order="F")), shape  # registration helped
    return agree


def test_benchmark_pair_192x160x256_vs_oracle(api):
    from deedsbcv_gb300 import phantom
    pair = phantom.make_pair((192, 160, 256), seed=2, n_organs=13, max_disp=10.0)
    flow, _ = api.register(pair["fixed"], pair["moving"], want_warped=False)
    _against_oracle(api, pair, flow)


def test_cross_contrast_192x192x208_vs_oracle(api):
    from deedsbcv_gb300 import phantom
    pair = phantom.make_pair((192, 192, 208), seed=3, max_disp=12.0, contrast="cross")
    flow, _ = api.register(pair["fixed"], pair["moving"], want_warped=False)
    _against_oracle(api, pair, flow)


def test_largest_uneven_batch_pairs_vs_oracle(api):
    from deedsbcv_gb300 import phantom
    work = sorted(phantom.batch_workload(), key=lambda t: -int(np.prod(t[0])))
    chosen = [work[0], work[1], work[-1]]  # the two largest and the smallest: uneven in one batch
    pairs = [phantom.make_pair(shape, seed=s, max_disp=10.0) for shape, s in chosen]
    out = api.register_batch([(p["fixed"], p["moving"]) for p in pairs], params=api.default_params())
    for p, (flow, _) in zip(pairs[:2], out[:2]):
        _against_oracle(api, p, flow)
