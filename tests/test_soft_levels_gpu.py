"""Multi-level soft-min registration on the GPU against the float64 definition.

The pieces the level loop adds to a single soft level, each against
oracle/softmin_ref.py in float64 (forward values and the hand-written adjoints
against autograd): field upsampling, warping of the moving image by the
upsampled prior, the prior's offsets in the pairwise term, and the whole
composition over three levels with gradients for both images and alpha at the
temperatures 0.1, 0.5 and 2.0.
"""
import numpy as np
import pytest
import torch

import softmin_ref as sref

pytestmark = pytest.mark.gpu

DIMS = (20, 16, 24)  # m, n, o
LEVELS = [(6, 2, 2, 1), (4, 2, 1, 1), (3, 2, 1, 1)]  # (grid, radius, quant, mind radius)


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


def _rel(a, b):
    return ((a - b).norm() / b.norm()).item()


@pytest.mark.parametrize("src,dst", [((5, 4, 6), (20, 16, 24)), ((4, 3, 4), (5, 4, 6)), ((5, 4, 6), (24, 20, 28))])
def test_soft_upsample_and_adjoint_match_float64(api, src, dst):
    rng = np.random.default_rng(0)
    (mA, nA, oA), (m, n, o) = src, dst
    field = rng.normal(0, 2, (3, mA * nA * oA)).astype(np.float32)
    ctx = api.context(0)
    out = api.SoftUpsample.apply(torch.from_numpy(field).cuda(), src, dst, ctx)
    F = torch.from_numpy(field.astype(np.float64)).view(3, oA, nA, mA).requires_grad_()
    ref = sref.upsample(F, src, dst)
    assert _rel(out.cpu().double(), ref.reshape(3, -1)) < 1e-6
    gout = rng.normal(0, 1, (3, m * n * o))
    ref.backward(torch.from_numpy(gout).view(3, o, n, m))
    fin = torch.from_numpy(field).cuda().requires_grad_()
    api.SoftUpsample.apply(fin, src, dst, ctx).backward(torch.from_numpy(gout).float().cuda())
    assert _rel(fin.grad.cpu().double(), F.grad.reshape(3, -1)) < 1e-5


def test_soft_warp_and_adjoint_match_float64(api):
    rng = np.random.default_rng(1)
    m, n, o = DIMS
    gd = (5, 4, 6)
    f, mv = _pair(4)
    grid = rng.normal(0, 1.5, (3, gd[0] * gd[1] * gd[2])).astype(np.float32)
    ctx = api.context(0)
    M = torch.from_numpy(mv).cuda().requires_grad_()
    G = torch.from_numpy(grid).cuda().requires_grad_()
    out = api.SoftWarp.apply(M, G, DIMS, gd, ctx)
    M64 = _t64(mv, DIMS).requires_grad_()
    G64 = torch.from_numpy(grid.astype(np.float64)).view(3, gd[2], gd[1], gd[0]).requires_grad_()
    ref = sref.warp(M64, sref.upsample(G64, gd, DIMS))
    assert (out.detach().cpu().double() - ref.reshape(-1)).abs().max().item() <= 1e-5 * np.abs(mv).max()
    gout = rng.normal(0, 1, m * n * o)
    ref.reshape(-1).backward(torch.from_numpy(gout))
    out.backward(torch.from_numpy(gout).float().cuda())
    assert _rel(M.grad.cpu().double(), M64.grad.reshape(-1)) < 1e-5
    # the position derivative jumps where a sample crosses a voxel boundary; float32
    # and float64 coordinates can fall either side of one for a few voxels
    assert _rel(G.grad.cpu().double(), G64.grad.reshape(3, -1)) < 2e-3


@pytest.mark.parametrize("tau", [0.1, 0.5, 2.0])
def test_soft_level_with_prior_matches_float64(api, tau):
    """The prior's offsets in the pairwise term (forward and dL/dprior)."""
    m, n, o = DIMS
    g, hw, q = 4, 2, 1
    m1, n1, o1 = m // g, n // g, o // g
    f, mv = _pair(5)
    fd, md = torch.from_numpy(f).cuda(), torch.from_numpy(mv).cuda()
    tree = api.soft_tree(fd, m, n, o, g)
    rng = np.random.default_rng(2)
    prior = rng.normal(0, 1.0, (3, m1 * n1 * o1)).astype(np.float32)
    gt = rng.normal(0, 1, (3, m1 * n1 * o1))
    P = torch.from_numpy(prior).cuda().requires_grad_()
    a = torch.tensor(1.6, requires_grad=True)
    params = api.soft_params(g, hw, q, 1.6, tau, 0.01, 1)
    d = api.SoftDeedsLevel.apply(fd, md, a, P, DIMS, params, tree, api.context(0))
    ((d - torch.from_numpy(gt).float().cuda()) ** 2).mean().backward()
    P64 = torch.from_numpy(prior.astype(np.float64)).requires_grad_()
    cost = sref.soft_cost(sref.soft_mind(_t64(f, DIMS), 1), sref.soft_mind(_t64(mv, DIMS), 1), g, hw, q,
                          torch.tensor(1.6, dtype=torch.float64), 0.01)
    ref = sref.soft_tree(cost, *tree, hw, q, tau, prior=P64)
    assert (d.detach().cpu().double() - ref).abs().max().item() < 2e-3
    ((ref - torch.from_numpy(gt)) ** 2).mean().backward()
    assert _rel(P.grad.cpu().double(), P64.grad) < 2e-3


def _oracle_levels(f, mv, trees, tau, gt, perturb=None):
    F64, M64 = _t64(f, DIMS).requires_grad_(), _t64(mv, DIMS).requires_grad_()
    a64 = torch.tensor(1.6, dtype=torch.float64, requires_grad=True)
    ref = sref.soft_register_levels(F64, M64, a64, trees, LEVELS, tau, 0.01, perturb).reshape(3, -1)
    ((ref - gt) ** 2).mean().backward()
    return ref.detach(), F64.grad.reshape(-1), M64.grad.reshape(-1), a64.grad.item()


@pytest.mark.parametrize("tau", [0.1, 0.5, 2.0])
def test_soft_register_levels_matches_float64(api, tau):
    m, n, o = DIMS
    f, mv = _pair(6)
    fd, md = torch.from_numpy(f).cuda(), torch.from_numpy(mv).cuda()
    trees = [api.soft_tree(fd, m, n, o, g) for g, *_ in LEVELS]
    gl = LEVELS[-1][0]
    gt = torch.from_numpy(np.random.default_rng(6).normal(0, 1, (3, (m // gl) * (n // gl) * (o // gl))))
    F, M = fd.clone().requires_grad_(), md.clone().requires_grad_()
    a = torch.tensor(1.6, requires_grad=True)
    d = api.soft_register_levels(F, M, a, DIMS, LEVELS, tau=tau, trees=trees)
    ((d - gt.float().cuda()) ** 2).mean().backward()
    gF, gM, ga = F.grad.cpu().double(), M.grad.cpu().double(), a.grad.item()
    ref, rF, rM, ra = _oracle_levels(f, mv, trees, tau, gt)
    err = (d.detach().cpu().double() - ref).abs().max().item()
    # three levels compound float32 rounding through the warps: 5e-3 voxels
    assert err < 5e-3, err
    # How far forward changes of the observed size move the float64 gradients: at
    # tau = 0.1 the expected displacements sit near whole labels, so many warp
    # samples lie next to a voxel boundary where the trilinear position derivative
    # jumps, and 1e-5 voxels of forward change move dL/dalpha by several percent.
    # The float32 gradients are held to three times that spread (and to 5e-3 where
    # the problem is well conditioned).
    spread = [0.0, 0.0, 0.0]
    for seed in (1, 2):
        gen = torch.Generator().manual_seed(seed)
        pert = lambda li, E: E + err * torch.randn(E.shape, generator=gen, dtype=E.dtype)  # noqa: E731
        _, pF, pM, pa = _oracle_levels(f, mv, trees, tau, gt, pert)
        for k, v in enumerate((_rel(pF, rF), _rel(pM, rM), abs(pa - ra) / abs(ra))):
            spread[k] = max(spread[k], v)
    assert _rel(gF, rF) < max(5e-3, 3 * spread[0]), (_rel(gF, rF), spread)
    assert _rel(gM, rM) < max(5e-3, 3 * spread[1]), (_rel(gM, rM), spread)
    assert abs(ga - ra) <= max(5e-3, 3 * spread[2]) * abs(ra) + 1e-5, (ga, ra, spread)


def test_soft_warp_invalid_arguments_raise(api):
    ctx = api.context(0)
    x = torch.zeros(3 * 8, device="cuda")
    with pytest.raises(Exception):
        api.SoftWarp.apply(torch.zeros(8, device="cuda"), x, (2, 2, 2), (0, 2, 2), ctx)
    with pytest.raises(Exception):
        api.SoftUpsample.apply(x, (2, 2, 2), (4, 4, 0), ctx)


def test_soft_kept_state_matches_recompute(api):
    """The backward over the kept forward state gives the recomputing backward's
    gradients, and a second backward through a retained graph (whose slot the
    first backward released) recomputes to the same values."""
    m, n, o = DIMS
    f, mv = _pair(7)
    fd, md = torch.from_numpy(f).cuda(), torch.from_numpy(mv).cuda()
    trees = [api.soft_tree(fd, m, n, o, g) for g, *_ in LEVELS]
    gl = LEVELS[-1][0]
    gt = torch.from_numpy(np.random.default_rng(7).normal(0, 1, (3, (m // gl) * (n // gl) * (o // gl)))).float().cuda()

    def run(keep):
        F, M = fd.clone().requires_grad_(), md.clone().requires_grad_()
        a = torch.tensor(1.6, requires_grad=True)
        d = api.soft_register_levels(F, M, a, DIMS, LEVELS, tau=0.5, trees=trees, keep_state=keep)
        loss = ((d - gt) ** 2).mean()
        out = []
        for retain in (True, False):
            loss.backward(retain_graph=retain)
            out.append((F.grad.clone(), M.grad.clone(), a.grad.clone()))
            F.grad, M.grad, a.grad = None, None, None
        return d.detach(), out

    d0, r = run(False)
    d1, k = run(True)
    # Same kernels on the same inputs, but the cost kernels and the adjoints sum
    # with float atomics, whose order varies between runs: across three levels
    # the fields differ by ~1e-5 voxels.  A backward over the wrong or a stale
    # state differs at order one.  Between the two forwards, a finer level's
    # trilinear warp samples the coarser field, whose derivative in position
    # jumps at voxel faces: the few nodes whose sample sits on a face carry a
    # different gradient, so the two runs agree to 1e-2 and a backward repeated
    # over one forward's graph to 1e-3.
    assert (d0 - d1).abs().max().item() <= 1e-4
    for got, tol in ((k[0], 1e-2), (k[1], 1e-2), (r[1], 1e-3)):
        for x, y in zip(got, r[0]):
            assert _rel(x.cpu().double(), y.cpu().double()) < tol


def test_soft_kept_slot_checks(api):
    """deeds_soft_backward_kept_dev refuses a slot that holds no state or was
    filled for other parameters; released slots are reused; trim frees them."""
    import ctypes as C
    m, n, o = DIMS
    g, hw, q = 4, 2, 1
    sz1 = (m // g) * (n // g) * (o // g)
    f, mv = _pair(8)
    fd, md = torch.from_numpy(f).cuda(), torch.from_numpy(mv).cuda()
    ctx = api.Context(0)
    tree = api._tree_arrays(api.soft_tree(fd, m, n, o, g, ctx))
    params = api.soft_params(g, hw, q, 1.6, 0.5, 0.01, 1)
    out = torch.empty(3 * sz1, device="cuda")
    gd = torch.randn(3 * sz1, device="cuda")
    gf = torch.empty_like(fd)
    L = ctx._L

    def keep():
        slot = C.c_int(-1)
        api._soft_call(ctx, L.deeds_soft_forward_keep_dev, fd, md, DIMS, params, tree, None, api._ptr(out),
                       C.byref(slot))
        return slot.value

    def back(slot, p, prior=None):
        return L.deeds_soft_backward_kept_dev(ctx.handle, slot, api._ptr(fd), api._ptr(md), m, n, o, C.byref(p),
                                              api._ptr(prior), api._ptr(gd), api._ptr(gf), None, None, None,
                                              api._stream())

    s0 = keep()
    s1 = keep()
    assert (s0, s1) == (0, 1)
    ctx.check(back(s0, params))
    g_first = gf.clone()
    ctx.check(back(s0, params))  # the state survives a backward
    assert _rel(gf.cpu().double(), g_first.cpu().double()) < 1e-5
    other = api.soft_params(g, hw, q, 1.7, 0.5, 0.01, 1)
    with pytest.raises(api.DeedsError):
        ctx.check(back(s0, other))
    prior = torch.zeros(3 * sz1, device="cuda")
    with pytest.raises(api.DeedsError):
        ctx.check(back(s0, params, prior))
    with pytest.raises(api.DeedsError):
        ctx.check(back(5, params))
    ctx.check(L.deeds_soft_release(ctx.handle, s0))
    with pytest.raises(api.DeedsError):
        ctx.check(L.deeds_soft_release(ctx.handle, s0))
    with pytest.raises(api.DeedsError):
        ctx.check(back(s0, params))
    assert keep() == s0  # the first free slot is reused
    for s in (s0, s1):
        ctx.check(L.deeds_soft_release(ctx.handle, s))
    ctx.check(L.deeds_soft_trim(ctx.handle))
    assert keep() == 0
    ctx.close()


def _batch_case(api, seeds, levels):
    m, n, o = DIMS
    pairs = [_pair(s) for s in seeds]
    F = torch.stack([torch.from_numpy(f) for f, _ in pairs]).cuda()
    M = torch.stack([torch.from_numpy(mv) for _, mv in pairs]).cuda()
    trees = [[api.soft_tree(F[i], m, n, o, g) for g, *_ in levels] for i in range(len(seeds))]
    gl = levels[-1][0]
    gt = torch.from_numpy(np.random.default_rng(9).normal(0, 1, (len(seeds), 3, (m // gl) * (n // gl) * (o // gl))))
    return F, M, trees, gt.float().cuda()


@pytest.mark.parametrize("keep", [True, False])
def test_soft_batch_matches_single_pairs(api, keep):
    """Pairs run concurrently on lanes give each pair's own soft_register_levels
    field and gradients; a second backward through the retained graph agrees."""
    F, M, trees, gt = _batch_case(api, (11, 12, 13), LEVELS)
    Fb, Mb = F.clone().requires_grad_(), M.clone().requires_grad_()
    ab = torch.tensor(1.6, requires_grad=True)
    d = api.soft_register_levels_batch(Fb, Mb, ab, DIMS, LEVELS, tau=0.5, trees=trees, keep_state=keep)
    loss = ((d - gt) ** 2).mean(dim=(1, 2)).sum()
    loss.backward(retain_graph=True)
    first = (Fb.grad.clone(), Mb.grad.clone(), ab.grad.clone())
    Fb.grad, Mb.grad, ab.grad = None, None, None
    loss.backward()
    for x, y in zip((Fb.grad, Mb.grad, ab.grad), first):
        assert _rel(x.cpu().double(), y.cpu().double()) < 1e-3
    ga_total = 0.0
    for i in range(F.shape[0]):
        Fi, Mi = F[i].clone().requires_grad_(), M[i].clone().requires_grad_()
        ai = torch.tensor(1.6, requires_grad=True)
        di = api.soft_register_levels(Fi, Mi, ai, DIMS, LEVELS, tau=0.5, trees=trees[i])
        ((di - gt[i]) ** 2).mean().backward()
        # float atomics in the cost kernels and adjoints: ~1e-5 voxels across levels
        assert (d[i].detach() - di.detach()).abs().max().item() <= 1e-4
        # The two runs are separate forwards whose coarser fields differ by ~1e-5
        # voxels; the next level's trilinear warp has a derivative in position that
        # jumps at voxel faces, so the few nodes whose sample sits on a face carry a
        # different gradient (3.6e-3 relative seen on 1 of ~5 runs): 1e-2 here.
        assert _rel(first[0][i].cpu().double(), Fi.grad.cpu().double()) < 1e-2
        assert _rel(first[1][i].cpu().double(), Mi.grad.cpu().double()) < 1e-2
        ga_total += ai.grad.item()
    assert abs(first[2].item() - ga_total) <= 1e-3 * abs(ga_total) + 1e-5


def test_soft_batch_more_pairs_than_lanes(api):
    """Ten pairs run as a wave of eight lanes and a wave of two."""
    lv = LEVELS[-1:]
    F, M, trees, gt = _batch_case(api, tuple(range(20, 30)), lv)
    Fb = F.clone().requires_grad_()
    d = api.soft_register_levels_batch(Fb, M, 1.6, DIMS, lv, tau=0.5, trees=trees)
    ((d - gt) ** 2).mean(dim=(1, 2)).sum().backward()
    for i in (0, 7, 8, 9):
        Fi = F[i].clone().requires_grad_()
        di = api.soft_register_levels(Fi, M[i], 1.6, DIMS, lv, tau=0.5, trees=trees[i])
        ((di - gt[i]) ** 2).mean().backward()
        assert (d[i].detach() - di.detach()).abs().max().item() <= 1e-4
        assert _rel(Fb.grad[i].cpu().double(), Fi.grad.cpu().double()) < 1e-3


def test_soft_batch_error_names_pair_and_frees_slots(api):
    """A bad tree in pair 2 fails the batch with the pair named; the slots that
    the failed call took are free again, so the next batch reuses slot 0."""
    import ctypes as C
    lv = LEVELS[-1:]
    F, M, trees, _ = _batch_case(api, (31, 32, 33), lv)
    ctx = api.Context(0)
    bad = [list(t) for t in trees]
    o_, p_, e_ = api._tree_arrays(bad[2][0])
    o_ = o_.copy()
    o_[1] = o_[0]  # a node repeated in the order
    bad[2][0] = (o_, p_, e_)
    Fb = F.clone().requires_grad_()
    with pytest.raises(api.DeedsError, match="pair 2"):
        api.soft_register_levels_batch(Fb, M, 1.6, DIMS, lv, tau=0.5, trees=bad, ctx=ctx)
    g, hw, q, qs = lv[0]
    params = api.soft_params(g, hw, q, 1.6, 0.5, 0.01, qs)
    sz1 = (DIMS[0] // g) * (DIMS[1] // g) * (DIMS[2] // g)
    out = torch.empty(3, 3, sz1, device="cuda")
    slots = (C.c_int * 3)()
    ta = [api._tree_arrays(t[0]) for t in trees]
    ctx.check(ctx._L.deeds_soft_forward_batch_dev(
        ctx.handle, 3, api._ptrs(F), api._ptrs(M), *DIMS, C.byref(params), api._ptrs([t[0] for t in ta]),
        api._ptrs([t[1] for t in ta]), api._ptrs([t[2] for t in ta]), None, api._ptrs(out), slots, api._stream()))
    assert list(slots) == [0, 0, 0]  # each pair's lane had its slot 0 free again
    ctx.check(ctx._L.deeds_soft_release_batch(ctx.handle, 3, slots))
    with pytest.raises(api.DeedsError):
        ctx.check(ctx._L.deeds_soft_release_batch(ctx.handle, 3, slots))
    ctx.close()
