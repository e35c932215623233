"""Pin the float64 soft-min definition (oracle/softmin_ref.py) to the reference.

The soft form has no counterpart in the reference, but two of its parts reduce to
reference outputs: quantising the continuous MIND-SSC level with the reference's
thresholds must give the reference binary's descriptor codes (golden vectors),
and as tau -> 0 the soft marginals must select the hard min-sum labels of
regularisationCL (the oracle, itself pinned bit-exact to the reference).
"""
import numpy as np
import pytest
import torch

import pyoracle as orc
import softmin_ref as sref


def _vol(flat, m, n, o):
    # flat index i + j*m + k*m*n  ->  tensor (o, n, m)
    return torch.from_numpy(np.asarray(flat, np.float64).reshape(o, n, m))


def quantise(s):
    """Reference code of continuous levels s (12, o, n, m): 5-bit thermometer per channel."""
    lvl = sum((s > c + 1.5).to(torch.int64) for c in range(5))
    therm = torch.tensor([0, 1, 3, 7, 15, 31], dtype=torch.int64)[lvl]
    code = torch.zeros(s.shape[1:], dtype=torch.int64)
    for l in range(12):
        code |= therm[l] << (5 * l)
    return code.reshape(-1).numpy().view(np.uint64)


@pytest.mark.parametrize("qs", [1, 2, 3])
def test_soft_descriptor_quantises_to_reference_codes(golden, qs):
    g = golden("mind")
    m, n, o = (int(x) for x in g["dims"])
    for key, img in ((f"codes_q{qs}", g["fixed"]), (f"mcodes_q{qs}", g["moving"])):
        s = sref.soft_mind(_vol(img, m, n, o), qs)
        codes = quantise(s)
        ref = g[key]
        # per-channel agreement; float64 exp vs the reference's float32 log thresholds
        # may differ exactly at a threshold
        a = codes[:, None] >> (5 * np.arange(12, dtype=np.uint64))[None, :] & np.uint64(31)
        b = ref[:, None] >> (5 * np.arange(12, dtype=np.uint64))[None, :] & np.uint64(31)
        assert (a == b).mean() > 0.999, (key, (a == b).mean())


def test_soft_tree_low_temperature_selects_hard_labels(golden):
    r = golden("reg")
    p = golden("prims")
    m, n, o = (int(x) for x in r["dims"])
    gs, hw, q = 4, 2, 1
    key = "4_2_1"
    m1, n1, o1 = m // gs, n // gs, o // gs
    sz1 = m1 * n1 * o1
    cost = r[f"counts_{key}"].astype(np.float32) * r[f"alpha1_{key}"]
    zero = np.zeros(sz1, np.float32)
    ordered, parents, edgemst = p["ordered_4"], p["parents_4"], p["edgemst_4"]
    _, u1, v1, w1 = orc.regularisation(cost, zero, zero, zero, m1, n1, o1, hw, q, ordered, parents, edgemst)
    E = sref.soft_tree(torch.from_numpy(cost.astype(np.float64)).view(sz1, -1), ordered, parents, edgemst, hw, q,
                       tau=1e-3).numpy()
    hard = np.stack([u1, v1, w1])
    agree = (np.abs(E - hard).max(axis=0) < 0.05).mean()
    assert agree > 0.99, agree


def test_soft_reference_gradient_matches_central_differences():
    torch.manual_seed(0)
    o, n, m, g, hw, q, qs = 8, 8, 8, 4, 1, 1, 1
    fixed = torch.randn(o, n, m, dtype=torch.float64)
    moving = torch.randn(o, n, m, dtype=torch.float64)
    sz1 = (m // g) * (n // g) * (o // g)
    ordered = np.arange(sz1, dtype=np.int32)
    parents = np.array([0, 0, 0, 1, 2, 3, 4, 5][:sz1], np.int32)
    edgemst = np.linspace(0.3, 1.0, sz1).astype(np.float32)
    tree = (ordered, parents, edgemst)
    gt = torch.randn(3, sz1, dtype=torch.float64)

    def loss(f, mv, a):
        d = sref.soft_register(f, mv, a, tree, g, hw, q, 0.5, 0.01, qs)
        return ((d - gt) ** 2).mean()

    f = fixed.clone().requires_grad_()
    a = torch.tensor(1.6, dtype=torch.float64, requires_grad=True)
    loss(f, moving, a).backward()
    h = 1e-3
    for idx in [(1, 2, 3), (4, 4, 4), (7, 0, 5)]:
        fp, fm = fixed.clone(), fixed.clone()
        fp[idx] += h
        fm[idx] -= h
        fd = (loss(fp, moving, a.detach()) - loss(fm, moving, a.detach())).item() / (2 * h)
        assert abs(fd - f.grad[idx].item()) <= 1e-6 + 1e-4 * abs(fd)
    fd = (loss(fixed, moving, a.detach() + h) - loss(fixed, moving, a.detach() - h)).item() / (2 * h)
    assert abs(fd - a.grad.item()) <= 1e-7 + 1e-4 * abs(fd)
