"""Multi-atlas label fusion (no reference counterpart: the reference's README
names joint label fusion as future work, README.md:8, README.md:201).

The GPU vote must equal the float32 restatement in oracle/fusion_ref.py bit for
bit (same operation order; built with --fmad=false), for majority and weighted
voting, patch radii 0-2, one and many atlases; the end-to-end multi-atlas call
(deeds registrations of every atlas to the target, label warps, fusion) must
fuse exactly what it warped, and fusion must not be worse than the mean single
atlas on a phantom whose atlases are deformed copies of the target anatomy.
"""
import numpy as np
import pytest

import fusion_ref

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from deedsbcv_gb300 import api as _api
    _api.context(0)
    return _api


def _flat_cuda(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).ravel(order="F"))).to(dtype).cuda()


def _case(shape, n_atlas, n_labels, seed):
    rng = np.random.default_rng(seed)
    target = np.asfortranarray(rng.normal(0, 100, shape).astype(np.float32))
    images = [np.asfortranarray((target + rng.normal(0, 30 + 20 * a, shape)).astype(np.float32))
              for a in range(n_atlas)]
    labels = [np.asfortranarray(rng.integers(0, n_labels, shape).astype(np.int16)) for _ in range(n_atlas)]
    return target, images, labels


@pytest.mark.parametrize("shape,n_atlas,radius,power", [((23, 17, 29), 5, 2, 2), ((23, 17, 29), 5, 1, 1),
                                                          ((16, 16, 16), 7, 0, 2), ((31, 9, 12), 4, 2, 0),
                                                          ((12, 10, 8), 1, 1, 2), ((9, 8, 7), 64, 1, 3)])
def test_fusion_matches_oracle(api, shape, n_atlas, radius, power):
    target, images, labels = _case(shape, n_atlas, 5, sum(shape) + n_atlas)
    m, n, o = shape
    got = api.fuse_labels_device(_flat_cuda(target, torch.float32), [_flat_cuda(a, torch.float32) for a in images],
                                 [_flat_cuda(a, torch.int16) for a in labels], m, n, o, radius=radius, eps=1.0,
                                 power=power).cpu().numpy()
    ref = fusion_ref.fuse_labels(target, images, labels, radius=radius, eps=1.0, power=power)
    assert np.array_equal(got, ref.ravel(order="F"))


def test_fusion_rejects_bad_arguments(api):
    target, images, labels = _case((8, 8, 8), 2, 3, 1)
    t = _flat_cuda(target, torch.float32)
    ims = [_flat_cuda(a, torch.float32) for a in images]
    labs = [_flat_cuda(a, torch.int16) for a in labels]
    with pytest.raises(RuntimeError):
        api.fuse_labels_device(t, ims * 33, labs * 33, 8, 8, 8)  # 66 atlases, above the maximum of 64
    with pytest.raises(RuntimeError):
        api.fuse_labels_device(t, ims, labs, 8, 8, 8, radius=-1)


def test_multi_atlas_end_to_end(api):
    from deedsbcv_gb300 import phantom

    shape = (64, 56, 72)
    case = phantom.make_atlases(shape, n_atlases=4, seed=5, max_disp=5.0)
    params = api.default_params(grid=[6, 5, 4], radius=[5, 4, 3], quant=[3, 2, 1])
    fused, wl, wi = api.multi_atlas(case["target"], case["atlas_images"], case["atlas_labels"], params=params,
                                    radius=2, eps=1.0, power=2)
    ref = fusion_ref.fuse_labels(case["target"], wi, wl, radius=2, eps=1.0, power=2)
    assert np.array_equal(fused, ref)
    truth = case["target_labels"]
    single = [phantom.dice(truth, w) for w in wl]
    before = [phantom.dice(truth, a) for a in case["atlas_labels"]]
    fused_dice = phantom.dice(truth, fused)
    assert min(single) > np.mean(before)          # the registrations help
    assert fused_dice >= np.mean(single) - 1e-3   # fusion is not worse than the mean atlas
