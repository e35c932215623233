"""Image statistics of primsGraph on the device (src/primsMST.h:101-110).

The registration computes the mean and standard deviation that scale its MST
edge weights on the GPU (exact parallel-chunk evaluation of the reference's
sequential float chains).  Every case must equal the sequential oracle to the
bit: the adversarial inputs of the host version's test (CT-like integers with
exact ties, sums through zero, negative sums, large offsets, huge and tiny
magnitudes, constants, long runs, NaN, Inf) and the full-size CT phantom.
"""
import numpy as np
import pytest

import pyoracle as orc
from test_host import _stats_case

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from deedsbcv_gb300 import api as _api
    _api.context(0)
    return _api


def _same(got, ref):
    got = np.asarray(got, np.float32)
    ref = np.asarray(ref, np.float32)
    if np.array_equal(got.view(np.uint32), ref.view(np.uint32)):
        return True
    # NaN payloads may differ; NaN positions and every other bit may not
    return np.isnan(got).tolist() == np.isnan(ref).tolist() and np.array_equal(got[~np.isnan(got)],
                                                                                ref[~np.isnan(ref)])


@pytest.mark.parametrize("kind", ["ct_integers", "uniform", "crossing_zero", "negative", "offset", "huge", "tiny",
                                  "constant", "steps", "nan", "inf"])
@pytest.mark.parametrize("n", [(1 << 20) + 12345, 3 * 1000 * 1000, 4095, 1])
def test_device_image_stats_match_sequential_reference(api, kind, n):
    im = np.ascontiguousarray(_stats_case(kind, n, 5), np.float32)
    got = api.image_stats_device(torch.from_numpy(im).cuda())
    assert _same(got, orc.image_stats(im)), (kind, n, got, orc.image_stats(im))


def test_device_image_stats_full_size_phantom(api):
    from deedsbcv_gb300 import phantom

    pair = phantom.make_pair((192, 160, 256), seed=2)
    for name in ("fixed", "moving"):
        im = np.ascontiguousarray(pair[name].ravel(order="F") + np.float32(1024), np.float32)
        got = api.image_stats_device(torch.from_numpy(im).cuda())
        assert _same(got, orc.image_stats(im)), name
