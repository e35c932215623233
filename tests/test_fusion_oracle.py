"""CPU checks of the label-fusion oracle (oracle/fusion_ref.py) against direct
per-voxel restatements of the rule: majority voting with ties to the smaller
label, and weighted voting with explicit patch sums."""
import itertools

import numpy as np

import fusion_ref


def test_majority_vote_is_the_mode_with_smallest_label_on_ties():
    rng = np.random.default_rng(0)
    shape = (5, 4, 3)
    labels = [np.asfortranarray(rng.integers(0, 3, shape).astype(np.int16)) for _ in range(4)]
    images = [np.zeros(shape, np.float32)] * 4
    got = fusion_ref.fuse_labels(np.zeros(shape, np.float32), images, labels, radius=1, power=0)
    for idx in itertools.product(*(range(s) for s in shape)):
        votes = [int(l[idx]) for l in labels]
        counts = {v: votes.count(v) for v in votes}
        top = max(counts.values())
        assert got[idx] == min(v for v, c in counts.items() if c == top)


def test_weighted_vote_uses_clamped_patch_ssd():
    rng = np.random.default_rng(1)
    shape = (4, 5, 3)
    target = rng.normal(0, 10, shape).astype(np.float32)
    images = [(target + rng.normal(0, s, shape)).astype(np.float32) for s in (1.0, 5.0, 20.0)]
    labels = [np.asfortranarray(rng.integers(0, 2, shape).astype(np.int16)) for _ in range(3)]
    r, eps = 1, np.float32(1.0)
    got = fusion_ref.fuse_labels(target, images, labels, radius=r, eps=1.0, power=2)
    for idx in itertools.product(*(range(s) for s in shape)):
        score = {}
        for a in range(3):
            d = 0.0
            for off in itertools.product(range(-r, r + 1), repeat=3):
                p = tuple(min(max(idx[k] + off[k], 0), shape[k] - 1) for k in range(3))
                d += float(target[p] - images[a][p]) ** 2
            w = (1.0 / (d + float(eps))) ** 2
            score[int(labels[a][idx])] = score.get(int(labels[a][idx]), 0.0) + w
        top = max(score.values())
        # the float32 sums agree with the float64 ones to ~1e-6 relative; labels
        # whose scores are that close are accepted either way
        close = [lab for lab, s in score.items() if abs(s - top) <= 1e-5 * top]
        assert int(got[idx]) in close
