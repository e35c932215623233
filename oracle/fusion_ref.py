"""Oracle for multi-atlas label fusion (test infrastructure only: tests/ and
bench.py's checks import it; the library never does).

The reference has no label fusion: its README names joint label fusion of
several registered atlases as future work (README.md:8, README.md:201).  This
restates the library's documented rule in float32 numpy with the same order of
operations, so that the GPU result is reproduced bit for bit:

  D_i(x)  = window sums over (2r+1)^3 of (T - A_i)^2, clamp-to-edge, separable
            (axis i, then j, then k; each window summed in offset order -r..r
            starting from 0);
  w_i(x)  = (1 / (D_i(x) + eps))^p  (p multiplications of the reciprocal);
  label   = argmax over the atlases' labels L of sum_i w_i [L_i == L] (the sum
            in atlas order; ties to the smaller label).

Volumes are Fortran-ordered (m, n, o) arrays (i fastest), as the library's.
"""
import numpy as np


def window_sum(vol, axis, r):
    """Clamp-to-edge window sum of radius r along one axis, in offset order."""
    ext = vol.shape[axis]
    base = np.arange(ext)
    out = np.zeros_like(vol, dtype=np.float32)
    for d in range(-r, r + 1):
        out = (out + np.take(vol, np.clip(base + d, 0, ext - 1), axis=axis)).astype(np.float32)
    return out


def patch_ssd(target, image, r):
    df = (np.asarray(target, np.float32) - np.asarray(image, np.float32)).astype(np.float32)
    sq = (df * df).astype(np.float32)
    return window_sum(window_sum(window_sum(sq, 0, r), 1, r), 2, r)


def fuse_labels(target, images, labels, radius=2, eps=1.0, power=2):
    eps = np.float32(eps)
    n = len(images)
    w, lab = [], []
    for a in range(n):
        inv = (np.float32(1.0) / (patch_ssd(target, images[a], radius) + eps)).astype(np.float32)
        x = np.ones_like(inv, dtype=np.float32)
        for _ in range(power):
            x = (x * inv).astype(np.float32)
        w.append(x)
        lab.append(np.asarray(labels[a]).astype(np.int32))
    best = lab[0].copy()
    best_s = np.full(best.shape, -1.0, np.float32)
    for a in range(n):
        s = np.zeros(best.shape, np.float32)
        for b in range(n):
            s = np.where(lab[b] == lab[a], (s + w[b]).astype(np.float32), s)
        take = (s > best_s) | ((s == best_s) & (lab[a] < best))
        best = np.where(take, lab[a], best)
        best_s = np.where(take, s, best_s)
    return best.astype(np.int16)
