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


def test_soft_tree_prior_offsets_match_reference_bp(golden):
    """With a prior field the pairwise term is |lab(child) - lab(parent) - off|^2,
    off = (prior[parent] - prior[child]) / q (src/regularisation.h:205-208): at tau =
    1e-3, prior + expected displacement equals the reference binary's BP output."""
    r = golden("reg")
    p = golden("prims")
    m, n, o = (int(x) for x in r["dims"])
    for key in ("4_2_1", "5_3_2", "8_2_3"):
        gs, hw, q = (int(x) for x in key.split("_"))
        sz1 = (m // gs) * (n // gs) * (o // gs)
        cost = torch.from_numpy(r[f"counts_{key}"].astype(np.float32) * r[f"alpha1_{key}"]).double().view(sz1, -1)
        prior = torch.from_numpy(np.stack([r[f"u0_{key}"], r[f"v0_{key}"], r[f"w0_{key}"]])).double()
        E = sref.soft_tree(cost, p[f"ordered_{gs}"], p[f"parents_{gs}"], p[f"edgemst_{gs}"], hw, q, 1e-3, prior=prior)
        hard = np.stack([r[f"u1_{key}"], r[f"v1_{key}"], r[f"w1_{key}"]])
        agree = (np.abs((E + prior).numpy() - hard).max(axis=0) < 0.05 * q).mean()
        assert agree > 0.98, (key, agree)


def test_soft_upsample_matches_reference_upsample(golden):
    """The float64 upsampling of the multi-level soft form uses the reference's
    coordinates (src/transformations.h:245-279): against the reference binary's
    output for a 5x4x6 -> 24x20x28 grid (non-integer ratios)."""
    t = golden("transforms")
    m, n, o = (int(x) for x in t["dims"])
    m2, n2, o2 = (int(x) for x in t["grid_dims"])
    grid = torch.from_numpy(t["grid"].astype(np.float64)).view(3, o2, n2, m2)
    up = sref.upsample(grid, (m2, n2, o2), (m, n, o)).reshape(3, -1).numpy()
    assert np.abs(up - t["up"]).max() <= 1e-5 * np.abs(t["up"]).max()


def test_soft_warp_matches_reference_warp(golden):
    """The float64 warp is warpAffine with the identity (src/dataCostD.h:267-295):
    against the oracle's restatement (pinned bit-exact to the reference binary) and
    the reference binary's warpImageCL output on the same field."""
    t = golden("transforms")
    m, n, o = (int(x) for x in t["dims"])
    f = t["field"]
    eye = np.eye(4, dtype=np.float32).ravel()
    ref = orc.warp_affine(t["image"], eye, f[0], f[1], f[2], m, n, o)
    full = torch.from_numpy(f.astype(np.float64)).view(3, o, n, m)
    mine = sref.warp(_vol(t["image"], m, n, o), full).reshape(-1).numpy()
    scale = np.abs(t["image"]).max()
    assert np.abs(mine - ref).max() <= 1e-5 * scale
    assert np.abs(mine - t["warp_image"]).max() <= 1e-5 * scale


def test_soft_register_levels_gradient_matches_central_differences():
    """Autograd of the float64 multi-level composition (upsampled prior, warped
    moving image, prior offsets in the pairwise term) against central differences."""
    torch.manual_seed(1)
    m = n = o = 12
    levels = [(4, 1, 1, 1), (3, 1, 1, 1)]
    fixed = torch.randn(o, n, m, dtype=torch.float64)
    moving = torch.randn(o, n, m, dtype=torch.float64)
    trees = [orc.prims_graph(fixed.reshape(-1).numpy().astype(np.float32), m, n, o, g) for g, *_ in levels]
    gt = torch.randn(3, o // 3, n // 3, m // 3, dtype=torch.float64)

    def loss(f, mv, a):
        d = sref.soft_register_levels(f, mv, a, trees, levels, 0.5, 0.01)
        return ((d - gt) ** 2).mean()

    f = fixed.clone().requires_grad_()
    mv = moving.clone().requires_grad_()
    a = torch.tensor(1.6, dtype=torch.float64, requires_grad=True)
    loss(f, mv, a).backward()
    h = 1e-3
    for idx in [(1, 2, 3), (6, 5, 4), (11, 0, 7)]:
        for base, grad, which in ((fixed, f.grad, 0), (moving, mv.grad, 1)):
            p_, m_ = base.clone(), base.clone()
            p_[idx] += h
            m_[idx] -= h
            args_p = (p_, moving) if which == 0 else (fixed, p_)
            args_m = (m_, moving) if which == 0 else (fixed, m_)
            fd = (loss(*args_p, a.detach()) - loss(*args_m, a.detach())).item() / (2 * h)
            assert abs(fd - grad[idx].item()) <= 1e-6 + 1e-3 * abs(fd), (idx, which, fd, grad[idx].item())
    fd = (loss(fixed, moving, a.detach() + h) - loss(fixed, moving, a.detach() - h)).item() / (2 * h)
    assert abs(fd - a.grad.item()) <= 1e-7 + 1e-3 * abs(fd)
