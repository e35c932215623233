"""Soft-min form on the GPU against the float64 definition (oracle/softmin_ref.py).

Forward stages within float32 tolerances of the float64 oracle; the hand-written
adjoint against the oracle's autograd gradient and against FP64 central finite
differences (step 1e-3) on 64 random voxels; alpha's gradient likewise; tau -> 0
against the hard belief propagation of the same cost volume.
"""
import numpy as np
import pytest
import torch

import softmin_ref as sref

pytestmark = pytest.mark.gpu

DIMS = (20, 16, 24)  # m, n, o


@pytest.fixture(scope="module")
def api():
    from deedsbcv_gb300 import api as A
    return A


def _pair(seed, dims=DIMS):
    from deedsbcv_gb300 import phantom
    m, n, o = dims
    pr = phantom.make_pair((m, n, o), seed=seed, max_disp=3.0, spacing=8)
    f = np.asarray(pr["fixed"], np.float32).ravel(order="F")
    mv = np.asarray(pr["moving"], np.float32).ravel(order="F")
    return f, mv


def _t64(flat, dims):
    m, n, o = dims
    return torch.from_numpy(np.asarray(flat, np.float64).reshape(o, n, m))


def _case(api, seed=3, hw=2, q=1, g=4, dims=DIMS):
    m, n, o = dims
    f, mv = _pair(seed, dims)
    fd = torch.from_numpy(f).cuda()
    md = torch.from_numpy(mv).cuda()
    tree = api.soft_tree(fd, m, n, o, g)
    return f, mv, fd, md, tree


def test_soft_descriptor_matches_float64(api):
    m, n, o = DIMS
    f, _ = _pair(1)
    for qs in (1, 2, 3):
        s = api.soft_descriptor(torch.from_numpy(f).cuda(), m, n, o, qs).cpu().numpy()
        ref = sref.soft_mind(_t64(f, DIMS), qs).reshape(12, -1).numpy()
        assert np.abs(s - ref).max() < 2e-4, (qs, np.abs(s - ref).max())


@pytest.mark.parametrize("g,hw,q", [(4, 2, 1), (4, 3, 1), (4, 4, 1), (5, 1, 2), (3, 3, 1),
                                    (5, 2, 2), (5, 3, 2), (6, 2, 3), (6, 3, 3), (6, 2, 2), (6, 3, 2)])
def test_soft_cost_matches_float64(api, g, hw, q):
    # (4, *, 1): column kernels; (5|6, 2|3, 2|3): row kernels; the rest generic halo kernels
    m, n, o = DIMS
    f, mv = _pair(2)
    qs = 1
    sF = api.soft_descriptor(torch.from_numpy(f).cuda(), m, n, o, qs)
    sM = api.soft_descriptor(torch.from_numpy(mv).cuda(), m, n, o, qs)
    P = api.soft_params(grid=g, radius=hw, quant=q, alpha=1.6, eps=0.01)
    cost = api.soft_cost(sF.reshape(-1), sM.reshape(-1), m, n, o, P).cpu().numpy()
    rF = sref.soft_mind(_t64(f, DIMS), qs)
    rM = sref.soft_mind(_t64(mv, DIMS), qs)
    ref = sref.soft_cost(rF, rM, g, hw, q, torch.tensor(1.6, dtype=torch.float64), 0.01).numpy()
    assert np.abs(cost - ref).max() <= 1e-4 * np.abs(ref).max()


def _ref_disp(f, mv, tree, alpha, g, hw, q, tau, eps=0.01, qs=1, grad=False):
    F = _t64(f, DIMS).requires_grad_(grad)
    M = _t64(mv, DIMS).requires_grad_(grad)
    a = torch.tensor(float(alpha), dtype=torch.float64, requires_grad=grad)
    d = sref.soft_register(F, M, a, tree, g, hw, q, tau, eps, qs)
    return d, F, M, a


@pytest.mark.parametrize("tau", [0.1, 0.5, 2.0])
def test_soft_forward_matches_float64(api, tau):
    m, n, o = DIMS
    g, hw, q = 4, 2, 1
    f, mv, fd, md, tree = _case(api, hw=hw)
    d = api.soft_level(fd, md, 1.6, (m, n, o), grid=g, radius=hw, quant=q, tau=tau, tree=tree).detach().cpu()
    ref, *_ = _ref_disp(f, mv, tree, 1.6, g, hw, q, tau)
    assert torch.allclose(d.double(), ref, atol=2e-3), (d.double() - ref).abs().max()


def _grads(api, tau, hw=2, seed=3, g=4, q=1):
    m, n, o = DIMS
    f, mv, fd, md, tree = _case(api, seed=seed, hw=hw, g=g)
    sz1 = (m // g) * (n // g) * (o // g)
    gt = torch.from_numpy(np.random.default_rng(seed).normal(0, 1, (3, sz1))).double()
    F = fd.clone().requires_grad_()
    M = md.clone().requires_grad_()
    a = torch.tensor(1.6, requires_grad=True)
    d = api.soft_level(F, M, a, (m, n, o), grid=g, radius=hw, quant=q, tau=tau, tree=tree)
    loss = ((d - gt.float().cuda()) ** 2).mean()
    loss.backward()
    return f, mv, tree, gt, F.grad.cpu().double(), M.grad.cpu().double(), a.grad.double().item()


@pytest.mark.parametrize("tau,g,hw,q", [(0.1, 4, 2, 1), (0.5, 4, 2, 1), (2.0, 4, 2, 1), (0.5, 4, 3, 1), (0.5, 3, 2, 1),
                                        (0.5, 5, 1, 2), (0.5, 5, 3, 2), (0.1, 6, 3, 3), (0.5, 6, 2, 2)])
def test_soft_adjoint_matches_float64_autograd(api, tau, g, hw, q):
    # (4, *, 1): column kernels; (3, 2, 1) and (5, 1, 2): generic halo kernels; (5, 3, 2), (6, 3, 3)
    # and (6, 2, 2): row kernels with the moving side gathered
    f, mv, tree, gt, gF, gM, ga = _grads(api, tau, hw, g=g, q=q)
    qs = int(0.5 * q + 1.0)
    F = _t64(f, DIMS).requires_grad_()
    M = _t64(mv, DIMS).requires_grad_()
    a = torch.tensor(1.6, dtype=torch.float64, requires_grad=True)
    cost = sref.soft_cost(sref.soft_mind(F, qs), sref.soft_mind(M, qs), g, hw, q, a, 0.01)
    cost.retain_grad()
    d = sref.soft_tree(cost, *tree, hw, q, tau)
    ((d - gt) ** 2).mean().backward()
    for mine, ref in ((gF, F.grad.reshape(-1)), (gM, M.grad.reshape(-1))):
        err = (mine - ref).norm() / ref.norm()
        assert err < 2e-3, err.item()
    # dL/dalpha = -sum_c sum_l cbar (C - mean_l C) / alpha sums terms of both signs
    # (cancellation up to ~30x here), so float32 rounding is bounded relative to the
    # size of those terms rather than to the (small) sum
    C = cost.detach()
    terms = (cost.grad * (C - C.mean(dim=1, keepdim=True))).abs().sum().item() / 1.6
    tol = max(2e-3 * abs(a.grad.item()), 2e-4 * terms)
    assert abs(ga - a.grad.item()) <= tol, (ga, a.grad.item(), terms)


def test_soft_adjoint_matches_central_differences(api):
    """FP64 central differences (step 1e-3) of the float64 definition at 64 random
    voxels (32 fixed, 32 moving) and at alpha, against the GPU adjoint."""
    m, n, o = DIMS
    g, hw, q, tau = 4, 2, 1, 0.5
    f, mv, tree, gt, gF, gM, ga = _grads(api, tau, hw, seed=5)
    rng = np.random.default_rng(7)
    h = 1e-3
    F0, M0 = _t64(f, DIMS), _t64(mv, DIMS)
    a0 = torch.tensor(1.6, dtype=torch.float64)

    def loss(Fv, Mv, av):
        d = sref.soft_register(Fv, Mv, av, tree, g, hw, q, tau, 0.01, 1)
        return ((d - gt) ** 2).mean().item()

    scale = max(gF.abs().max().item(), gM.abs().max().item())
    # voxels near the node-covered region where gradients are non-zero
    for which, base, gmine in (("fixed", F0, gF), ("moving", M0, gM)):
        idx = rng.choice(m * n * o, 32, replace=False)
        for p in idx:
            k, j, i = p // (m * n), (p // m) % n, p % m
            up, dn = base.clone(), base.clone()
            up[k, j, i] += h
            dn[k, j, i] -= h
            if which == "fixed":
                fd = (loss(up, M0, a0) - loss(dn, M0, a0)) / (2 * h)
            else:
                fd = (loss(F0, up, a0) - loss(F0, dn, a0)) / (2 * h)
            assert abs(fd - gmine[p].item()) <= 2e-3 * scale + 1e-2 * abs(fd), (which, p, fd, gmine[p].item())
    fd = (loss(F0, M0, a0 + h) - loss(F0, M0, a0 - h)) / (2 * h)
    assert abs(fd - ga) <= 2e-3 * abs(fd) + 1e-8, (fd, ga)


def test_soft_low_temperature_approaches_hard_argmin(api):
    m, n, o = DIMS
    g, hw, q = 4, 2, 1
    f, mv, fd, md, tree = _case(api, hw=hw)
    sF = api.soft_descriptor(fd, m, n, o, 1).reshape(-1)
    sM = api.soft_descriptor(md, m, n, o, 1).reshape(-1)
    P = api.soft_params(grid=g, radius=hw, quant=q)
    cost = api.soft_cost(sF, sM, m, n, o, P).reshape(-1).contiguous()
    m1, n1, o1 = m // g, n // g, o // g
    z = torch.zeros(m1 * n1 * o1, device="cuda")
    u1, v1, w1 = api.regularisationCL(cost.clone(), z, z, z, m1, n1, o1, hw, q, *tree)
    hard = torch.stack([u1, v1, w1]).cpu()
    d = api.soft_level(fd, md, 1.6, (m, n, o), grid=g, radius=hw, quant=q, tau=0.002, tree=tree).detach().cpu()
    agree = ((d - hard).abs().amax(0) < 0.05).float().mean().item()
    assert agree > 0.97, agree


def test_soft_invalid_arguments_raise(api):
    m, n, o = DIMS
    f, mv, fd, md, tree = _case(api)
    with pytest.raises(api.DeedsError):
        api.soft_level(fd, md, 1.6, (m, n, o), tau=0.0, tree=tree)
    with pytest.raises(api.DeedsError):
        api.soft_level(fd, md, 1.6, (m, n, o), radius=6, tree=tree)
    bad = (tree[0], np.full_like(tree[1], 10 ** 6), tree[2])
    with pytest.raises(api.DeedsError):
        api.soft_level(fd, md, 1.6, (m, n, o), tree=bad)
    # a child listed before its parent (the sweeps' order requires parents first)
    rev = (np.ascontiguousarray(tree[0][::-1]), tree[1], tree[2])
    with pytest.raises(api.DeedsError):
        api.soft_level(fd, md, 1.6, (m, n, o), tree=rev)
