"""ORACLE (test infrastructure only): float64 PyTorch definition of the
differentiable soft-min deeds layer, used as the double-precision reference for
the GPU forward and its hand-written adjoint.

The soft form has no counterpart in the reference; it relaxes one deeds level
(src/deedsBCV0.cpp:238-306) so that it is differentiable in both images and in
the regularisation weight alpha:

* descriptor: MIND-SSC as in src/MINDSSCbox.h:127-224 up to the normalised
  distances mind1 = (d - min d)/max(mean(d - min d), 1e-6); instead of the
  5-threshold quantisation the continuous level s = 6 exp(-mind1) is kept
  (the reference counts thresholds -log((c+1.5)/6) > mind1, i.e. levels of
  6 exp(-mind1));
* cost: cost[node][label] = alpha1 * sum over the node's samples and the 12
  channels of phi(sF - sM(p + d(label))), phi(x) = sqrt(x^2 + eps^2) - eps, with
  the reference's sampling, clamp-to-edge and alpha1 = 0.5 (g/(alpha q))/maxsamp
  (src/dataCostD.h:141-200);
* tree: the MST of the hard path (ordered, parents, edgemst; constants);
* messages: the reference's upward recursion (src/regularisation.h:190-238)
  with min replaced by the soft-min -tau log sum exp(-x/tau):
      B_c = cost_c + sum_children (M_k - min M_k)
      M_c(l_p) = softmin_l (edgemst_c B_c(l) + |lab(l) - lab(l_p)|^2);
* marginals, root to leaves: log p_root = log softmax(-B_root / tau);
      log p_c(l) = -edgemst_c B_c(l) / tau + logsumexp_lp(log p_p(lp) + M_c(lp)/tau - |lab(l)-lab(lp)|^2/tau)
  (the soft counterpart of the reference's argmin backtrack, :282-293);
* output: the expected displacement E_c = sum_l p_c(l) d(l), d = (label - hw) q.

Volumes are tensors of shape (o, n, m) (C order), so flat index = i + j*m + k*m*n.
"""
from __future__ import annotations

import numpy as np
import torch

DX = (1, 1, -1, 0, 1, 0)
DY = (1, -1, 0, -1, 0, 1)
DZ = (0, 0, 1, 1, 1, 1)
SX = (-1, 0, -1, 0, 0, 1, 0, 0, 0, -1, 0, 0)
SY = (0, -1, 0, 1, 0, 0, 0, 1, 0, 0, 0, -1)
SZ = (0, 0, 0, 0, -1, 0, -1, 0, -1, 0, -1, 0)


def _shift_or_self(vol, dz, dy, dx):
    """vol[k+dz, j+dx?..] with out-of-volume positions replaced by the voxel itself."""
    o, n, m = vol.shape
    out = vol.clone()
    ks = slice(max(0, -dz), min(o, o - dz))
    js = slice(max(0, -dx), min(n, n - dx))
    is_ = slice(max(0, -dy), min(m, m - dy))
    src_k = slice(ks.start + dz, ks.stop + dz)
    src_j = slice(js.start + dx, js.stop + dx)
    src_i = slice(is_.start + dy, is_.stop + dy)
    out[ks, js, is_] = vol[src_k, src_j, src_i]
    return out


def _box1(x, r, dim):
    """Windowed sum over [max(0,i-r), min(L-1,i+r)] along dim (the reference's box sum)."""
    L = x.shape[dim]
    P = torch.cumsum(x, dim=dim)
    idx_hi = torch.clamp(torch.arange(L) + r, max=L - 1)
    idx_lo = torch.arange(L) - r - 1
    hi = torch.index_select(P, dim, idx_hi)
    lo = torch.index_select(P, dim, torch.clamp(idx_lo, min=0))
    mask = (idx_lo >= 0).to(x.dtype)
    shape = [1] * x.dim()
    shape[dim] = L
    return hi - lo * mask.view(shape)


def box3(x, r):
    # axis order i (last), j, k as the reference
    return _box1(_box1(_box1(x, r, 2), r, 1), r, 0)


def soft_mind(vol, qs):
    """(12, o, n, m) continuous MIND-SSC levels 6*exp(-mind1)."""
    d = []
    for l in range(6):
        sh = _shift_or_self(vol, DZ[l] * qs, DY[l] * qs, DX[l] * qs)
        d.append(box3((sh - vol) ** 2, qs))
    v = []
    for l in range(12):
        v.append(_shift_or_self(d[l // 2], SZ[l] * qs, SY[l] * qs, SX[l] * qs))
    v = torch.stack(v)
    mn = v.min(dim=0, keepdim=True).values
    vv = v - mn
    noise = torch.clamp(vv.sum(dim=0, keepdim=True) / 12.0, min=1e-6)
    return 6.0 * torch.exp(-vv / noise)


def sampling(g):
    s = 2 if g > 4 else 1
    maxsamp = float(np.ceil(g / s) * np.ceil(g / s) * g)
    return s, maxsamp


def soft_cost(sF, sM, g, hw, q, alpha, eps):
    """cost (sz1, len3) of two (12, o, n, m) descriptor volumes; alpha is a 0-d tensor."""
    _, o, n, m = sF.shape
    m1, n1, o1 = m // g, n // g, o // g
    s, maxsamp = sampling(g)
    alpha1 = 0.5 * (g / (alpha * q)) / maxsamp
    length = 2 * hw + 1
    ii = torch.arange(0, g, 1)
    jj = torch.arange(0, g, s)
    kk = torch.arange(0, g, s)
    # sample coordinates per node: (nodes, samples)
    ny, nx, nz = torch.meshgrid(torch.arange(m1), torch.arange(n1), torch.arange(o1), indexing="ij")
    ny, nx, nz = ny.reshape(-1), nx.reshape(-1), nz.reshape(-1)  # node index = y + x*m1 + z*m1*n1 order below
    order = (ny + nx * m1 + nz * m1 * n1).argsort()
    ny, nx, nz = ny[order], nx[order], nz[order]
    si, sj, sk = torch.meshgrid(ii, jj, kk, indexing="ij")
    si, sj, sk = si.reshape(-1), sj.reshape(-1), sk.reshape(-1)
    py = ny[:, None] * g + si[None, :]
    px = nx[:, None] * g + sj[None, :]
    pz = nz[:, None] * g + sk[None, :]
    fvals = sF[:, pz, px, py]  # (12, nodes, samples)
    costs = []
    for lz in range(length):
        for lx in range(length):
            for ly in range(length):
                qy = torch.clamp(py + (ly - hw) * q, 0, m - 1)
                qx = torch.clamp(px + (lx - hw) * q, 0, n - 1)
                qz = torch.clamp(pz + (lz - hw) * q, 0, o - 1)
                diff = fvals - sM[:, qz, qx, qy]
                phi = torch.sqrt(diff * diff + eps * eps) - eps
                costs.append(phi.sum(dim=(0, 2)))
    # labels ordered ly fastest: the loops above produce lz, lx, ly nesting -> index ly + lx*len + lz*len^2
    return alpha1 * torch.stack(costs, dim=1)


def label_grid(hw):
    length = 2 * hw + 1
    lab = torch.arange(length ** 3)
    ly = lab % length
    lx = (lab // length) % length
    lz = lab // (length * length)
    return torch.stack([lx, ly, lz], dim=1).to(torch.float64)  # (len3, 3): x, y, z label coords


def edge_offsets(prior, parents, root, q):
    """(sz1, 3) label-unit offsets (x, y, z) of each node's edge to its parent from a
    prior grid field (3, sz1) [u, v, w]: (prior[parent] - prior[node]) / q, as the
    reference's regularisationCL (src/regularisation.h:205-208); zero at the root."""
    par = torch.as_tensor(np.asarray(parents, np.int64)).clone()
    par[int(root)] = int(root)
    off = (prior[:, par] - prior) / q  # (3, sz1)
    return off.T


def soft_tree(cost, ordered, parents, edgemst, hw, q, tau, prior=None):
    """Expected displacement (3, sz1) as [u(x), v(y), w(z)] from the soft recursion,
    relative to the prior field (3, sz1) when one is given: the pairwise term of an
    edge is |lab(l_child) - lab(l_parent) - off|^2 with off the prior's difference
    parent - child in label units."""
    sz1, len3 = cost.shape
    lab = label_grid(hw)
    Q = ((lab[:, None, :] - lab[None, :, :]) ** 2).sum(-1)  # (l, lp)
    offs = None
    if prior is not None:
        offs = edge_offsets(prior, parents, int(ordered[0]), q)  # (sz1, 3)

    def Qc(c):
        if offs is None:
            return Q
        d = lab[None, :, :] - lab[:, None, :] + offs[c][None, None, :]  # (l, lp, 3): lp - l + off
        return (d ** 2).sum(-1)
    children = [[] for _ in range(sz1)]
    for t in range(1, sz1):
        c = int(ordered[t])
        children[int(parents[c])].append(c)
    B = [None] * sz1
    M = [None] * sz1
    for t in range(sz1 - 1, -1, -1):
        c = int(ordered[t])
        b = cost[c]
        for k in children[c]:
            b = b + (M[k] - M[k].min().detach())
        B[c] = b
        if t > 0:
            e = float(edgemst[c])
            M[c] = -tau * torch.logsumexp(-(e * b[:, None] + Qc(c)) / tau, dim=0)  # over l, for each lp
    logp = [None] * sz1
    root = int(ordered[0])
    logp[root] = torch.log_softmax(-B[root] / tau, dim=0)
    for t in range(1, sz1):
        c = int(ordered[t])
        p = int(parents[c])
        e = float(edgemst[c])
        r = logp[p] + M[c] / tau
        G = torch.logsumexp(r[None, :] - Qc(c) / tau, dim=1)  # over lp, for each l
        logp[c] = -e * B[c] / tau + G
    P = torch.stack([torch.exp(lp) for lp in logp])  # (sz1, len3)
    disp = (lab - hw) * q  # (len3, 3) x, y, z
    return (P @ disp).T  # (3, sz1): u, v, w


def soft_register(fixed, moving, alpha, tree, g, hw, q, tau, eps, qs):
    """Full soft level in float64: fixed/moving (o, n, m) tensors, alpha 0-d tensor."""
    ordered, parents, edgemst = tree
    sF = soft_mind(fixed, qs)
    sM = soft_mind(moving, qs)
    cost = soft_cost(sF, sM, g, hw, q, alpha, eps)
    return soft_tree(cost, ordered, parents, edgemst, hw, q, tau)


def upsample(field, src_dims, dst_dims):
    """Trilinear upsampling of a (3, o2, n2, m2) field to (3, o, n, m) with the
    reference's coordinates (src/transformations.h:245-279): node (i, j, k) reads the
    source at (i / (m/m2), j / (n/n2), k / (o/o2)), corners clamped to the grid."""
    m2, n2, o2 = src_dims
    m, n, o = dst_dims
    dt = field.dtype
    y = torch.arange(m, dtype=dt) / (m / m2)
    x = torch.arange(n, dtype=dt) / (n / n2)
    z = torch.arange(o, dtype=dt) / (o / o2)
    return _trilinear(field, z[:, None, None], x[None, :, None], y[None, None, :])


def _trilinear(vol, zc, xc, yc):
    """Trilinear interpolation of vol (..., o, n, m) at coordinates zc, xc, yc
    (broadcastable, voxel units), clamp-to-edge corners; differentiable in vol
    and in the coordinates (piecewise)."""
    o, n, m = vol.shape[-3:]
    z0f, x0f, y0f = torch.floor(zc), torch.floor(xc), torch.floor(yc)
    dz, dx, dy = zc - z0f, xc - x0f, yc - y0f
    z0, x0, y0 = z0f.long(), x0f.long(), y0f.long()
    zc0, zc1 = z0.clamp(0, o - 1), (z0 + 1).clamp(0, o - 1)
    xc0, xc1 = x0.clamp(0, n - 1), (x0 + 1).clamp(0, n - 1)
    yc0, yc1 = y0.clamp(0, m - 1), (y0 + 1).clamp(0, m - 1)
    shape = torch.broadcast_shapes(zc.shape, xc.shape, yc.shape)
    zc0, zc1, xc0, xc1, yc0, yc1 = (t.expand(shape) for t in (zc0, zc1, xc0, xc1, yc0, yc1))
    dz, dx, dy = (t.expand(shape) for t in (dz, dx, dy))

    def at(zz, xx, yy):
        return vol[..., zz, xx, yy]

    return (at(zc0, xc0, yc0) * (1 - dz) * (1 - dx) * (1 - dy) + at(zc0, xc0, yc1) * (1 - dz) * (1 - dx) * dy
            + at(zc0, xc1, yc0) * (1 - dz) * dx * (1 - dy) + at(zc0, xc1, yc1) * (1 - dz) * dx * dy
            + at(zc1, xc0, yc0) * dz * (1 - dx) * (1 - dy) + at(zc1, xc0, yc1) * dz * (1 - dx) * dy
            + at(zc1, xc1, yc0) * dz * dx * (1 - dy) + at(zc1, xc1, yc1) * dz * dx * dy)


def warp(moving, full):
    """moving (o, n, m) sampled at p + field, field (3, o, n, m) [u(x), v(y), w(z)]
    (warpAffine with the identity, src/dataCostD.h:267-295, in float arithmetic)."""
    o, n, m = moving.shape
    dt = moving.dtype
    zz = torch.arange(o, dtype=dt)[:, None, None] + full[2]
    xx = torch.arange(n, dtype=dt)[None, :, None] + full[0]
    yy = torch.arange(m, dtype=dt)[None, None, :] + full[1]
    return _trilinear(moving, zz, xx, yy)


def soft_register_levels(fixed, moving, alpha, trees, levels, tau, eps, perturb=None):
    """Multi-level soft registration in float64 (the deeds level loop,
    src/deedsBCV0.cpp:222-306, forward direction only): per level the prior grid
    field is the previous level's result upsampled to this grid, the moving image is
    warped by the prior upsampled to full resolution, and the soft level returns the
    displacement relative to the prior.  levels: [(g, hw, q, qs)], trees: per level
    (ordered, parents, edgemst).  perturb (tests only): callable (level, E) -> E
    applied to each level's expected displacement, to measure how far rounding-size
    changes of the forward move the gradients.  Returns the last grid field
    (3, o1, n1, m1)."""
    o, n, m = fixed.shape
    prev = None
    prev_dims = None
    for li, ((g, hw, q, qs), tree) in enumerate(zip(levels, trees)):
        m1, n1, o1 = m // g, n // g, o // g
        if prev is None:
            U = torch.zeros(3, o1, n1, m1, dtype=fixed.dtype)
            warped = moving
        else:
            U = upsample(prev, prev_dims, (m1, n1, o1))
            warped = warp(moving, upsample(U, (m1, n1, o1), (m, n, o)))
        sF = soft_mind(fixed, qs)
        sM = soft_mind(warped, qs)
        cost = soft_cost(sF, sM, g, hw, q, alpha, eps)
        # node order y fastest = the (o1, n1, m1) C order of U
        E = soft_tree(cost, tree[0], tree[1], tree[2], hw, q, tau, prior=U.reshape(3, -1))
        if perturb is not None:
            E = perturb(li, E)
        prev = U + E.reshape(3, o1, n1, m1)
        prev_dims = (m1, n1, o1)
    return prev
