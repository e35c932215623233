"""Seeded synthetic CT-like image pairs for registration tests and benchmarks.

No public dataset is available offline, so every workload in this package runs
on volumes from this generator.  A pair is built from one label map:

* fixed: a -1000 HU background, an ellipsoidal body at 0 HU, and ``n_organs``
  random ellipsoid organs with intensities drawn from [-100, 300] HU, plus
  Gaussian noise (sigma 20);
* moving: the same anatomy resampled through a smooth random displacement field
  (cubic B-spline on a control grid of spacing 16 voxels, scaled to a given
  maximum displacement), with its own noise draw.
* ``affine=(max_degrees, max_scale, max_shift)`` composes a seeded affine map
  (rotations about the three axes, per-axis scaling and a translation about the
  volume centre) with the displacement field: moving(p) = anatomy(A p + disp(p));
  the 4x4 map is returned in the deeds matrix layout (X[0..3] gives y, X[4..7] x,
  X[8..11] z, src/linearBCV.cpp:289-296).
* ``contrast="cross"`` re-maps the moving anatomy's intensities per organ into
  [0, 1000] with an inverted background, multiplies a smooth bias field in
  [0.7, 1.3] and adds Rician noise (sigma 15).

Arrays are Fortran-ordered views of (m, n, o) volumes so that the flat index is
``i + j*m + k*m*n`` (i fastest), the layout of the deeds volumes.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def _bspline_basis(size, spacing, n_ctrl):
    """(size, n_ctrl) uniform cubic B-spline weights: voxel v sits at control
    coordinate v/spacing + 1 (one control point of margin on each side)."""
    t = np.arange(size, dtype=np.float64) / spacing + 1.0
    f = np.floor(t).astype(int)
    u = t - f
    w = np.stack([(1 - u) ** 3, 3 * u ** 3 - 6 * u ** 2 + 4, -3 * u ** 3 + 3 * u ** 2 + 3 * u + 1, u ** 3], 1) / 6.0
    B = np.zeros((size, n_ctrl))
    for r in range(4):
        B[np.arange(size), np.clip(f - 1 + r, 0, n_ctrl - 1)] += w[:, r]
    return B


def _bspline_field(shape, spacing, max_disp, rng):
    """Smooth displacement field (3, m, n, o) from random control-point offsets
    on a grid of the given spacing, interpolated with cubic B-splines."""
    ctrl = tuple(int(np.ceil(s / spacing)) + 3 for s in shape)
    coarse = rng.uniform(-1.0, 1.0, size=(3,) + ctrl)
    B = [_bspline_basis(shape[a], spacing, ctrl[a]) for a in range(3)]
    out = np.empty((3,) + tuple(shape), dtype=np.float32)
    for d in range(3):
        t = np.tensordot(B[0], coarse[d], axes=(1, 0))             # (m, c1, c2)
        t = np.tensordot(t, B[1], axes=(1, 1))                     # (m, c2, n)
        t = np.tensordot(t, B[2], axes=(1, 1))                     # (m, n, o)
        out[d] = t
    peak = float(np.abs(out).max())
    if peak > 0:
        out *= np.float32(max_disp / peak)
    return out


def _organ_labels(shape, n_organs, rng):
    m, n, o = shape
    dims = np.array([m, n, o], dtype=np.float32)
    c = dims / 2
    body_r = dims * 0.45
    ax = [np.arange(s, dtype=np.float32) for s in shape]
    body = (((ax[0] - c[0]) / body_r[0]) ** 2)[:, None, None] + (((ax[1] - c[1]) / body_r[1]) ** 2)[None, :, None] \
        + (((ax[2] - c[2]) / body_r[2]) ** 2)[None, None, :] <= 1.0
    labels = np.zeros(shape, dtype=np.uint8)
    for lab in range(1, n_organs + 1):
        centre = c + rng.uniform(-0.45, 0.45, 3).astype(np.float32) * body_r
        radii = rng.uniform(0.08, 0.22, 3).astype(np.float32) * dims
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        q = q.astype(np.float32)
        # the rotated ellipsoid lies inside the sphere of its largest radius
        rmax = float(radii.max())
        lo = [max(int(np.floor(centre[a] - rmax)), 0) for a in range(3)]
        hi = [min(int(np.ceil(centre[a] + rmax)) + 1, shape[a]) for a in range(3)]
        if any(h <= l for l, h in zip(lo, hi)):
            continue
        dy = (ax[0][lo[0]:hi[0]] - centre[0])[:, None, None]
        dx = (ax[1][lo[1]:hi[1]] - centre[1])[None, :, None]
        dz = (ax[2][lo[2]:hi[2]] - centre[2])[None, None, :]
        r2 = np.zeros((hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]), dtype=np.float32)
        for a in range(3):
            proj = q[0, a] * dy + q[1, a] * dx + q[2, a] * dz
            r2 += (proj / radii[a]) ** 2
        sub = labels[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        sub[(r2 <= 1.0) & body[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]] = lab
    return body, labels


def _render(body, labels, organ_hu, background, body_hu):
    img = np.full(labels.shape, background, dtype=np.float32)
    img[body] = body_hu
    for lab, hu in enumerate(organ_hu, start=1):
        img[labels == lab] = hu
    return img


def _affine(shape, max_degrees, max_scale, max_shift, rng):
    """4x4 float64 map of (y, x, z, 1) about the volume centre."""
    ang = np.deg2rad(rng.uniform(-max_degrees, max_degrees, 3))
    ca, sa = np.cos(ang), np.sin(ang)
    rx = np.array([[1, 0, 0], [0, ca[0], -sa[0]], [0, sa[0], ca[0]]])
    ry = np.array([[ca[1], 0, sa[1]], [0, 1, 0], [-sa[1], 0, ca[1]]])
    rz = np.array([[ca[2], -sa[2], 0], [sa[2], ca[2], 0], [0, 0, 1]])
    lin = rz @ ry @ rx @ np.diag(1.0 + rng.uniform(-max_scale, max_scale, 3))
    c = (np.array(shape, np.float64) - 1) / 2
    t = c - lin @ c + rng.uniform(-max_shift, max_shift, 3)
    A = np.eye(4)
    A[:3, :3] = lin
    A[:3, 3] = t
    return A


def make_pair(shape, seed=0, n_organs=None, max_disp=6.0, spacing=16, contrast="same", affine=None):
    """Return dict(fixed, moving, fixed_labels, moving_labels, disp[, affine]) for one pair.

    ``disp`` (3, m, n, o) float32 maps fixed to moving: moving(p) = anatomy(p + disp(p))
    with components ordered (y, x, z) = (dim 1, dim 2, dim 3).  With ``affine``
    the map is moving(p) = anatomy(A p + disp(p)) and ``affine`` in the result
    holds A as 16 float32 values in the deeds matrix layout.
    """
    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    if n_organs is None:
        n_organs = int(rng.integers(6, 13))
    body, labels = _organ_labels(shape, n_organs, rng)
    organ_hu = rng.uniform(-100.0, 300.0, n_organs).astype(np.float32)
    fixed = _render(body, labels, organ_hu, -1000.0, 0.0)
    disp = _bspline_field(shape, spacing, max_disp, rng)
    grid = np.meshgrid(*[np.arange(s, dtype=np.float32) for s in shape], indexing="ij")
    A = None
    if affine is not None:
        A = _affine(shape, *affine, rng)
        pos = [sum(A[d, e] * grid[e] for e in range(3)) + A[d, 3] for d in range(3)]
        coords = [(pos[d] + disp[d]).astype(np.float32) for d in range(3)]
    else:
        coords = [grid[d] + disp[d] for d in range(3)]
    mov_labels = ndimage.map_coordinates(labels, coords, order=0, mode="nearest").astype(np.uint8)
    mov_body = ndimage.map_coordinates(body.astype(np.uint8), coords, order=0, mode="nearest").astype(bool)
    if contrast == "same":
        moving = ndimage.map_coordinates(fixed, coords, order=1, mode="nearest").astype(np.float32)
        moving += rng.normal(0.0, 20.0, shape).astype(np.float32)
    elif contrast == "cross":
        remap = rng.uniform(0.0, 1000.0, n_organs).astype(np.float32)
        anat = _render(mov_body, mov_labels, remap, 1000.0, 300.0)
        bias = _bspline_field(shape, 48, 1.0, rng)[0]
        bias = 1.0 + 0.3 * bias / max(float(np.abs(bias).max()), 1e-6)
        anat = anat * bias
        re = anat + rng.normal(0.0, 15.0, shape).astype(np.float32)
        im = rng.normal(0.0, 15.0, shape).astype(np.float32)
        moving = np.sqrt(re * re + im * im).astype(np.float32)
    else:
        raise ValueError(f"unknown contrast {contrast!r}")
    fixed = fixed + rng.normal(0.0, 20.0, shape).astype(np.float32)
    out = {
        "fixed": np.asfortranarray(fixed.astype(np.float32)),
        "moving": np.asfortranarray(moving.astype(np.float32)),
        "fixed_labels": np.asfortranarray(labels),
        "moving_labels": np.asfortranarray(mov_labels),
        "disp": disp,
    }
    if A is not None:
        out["affine"] = A[:3, :].ravel().astype(np.float32).tolist() + [0.0, 0.0, 0.0, 1.0]
        out["affine"] = np.array(out["affine"], np.float32)
    return out


def make_atlases(shape, n_atlases=4, seed=0, n_organs=None, max_disp=6.0, spacing=16):
    """A multi-atlas segmentation case: one anatomy seen n_atlases + 1 times.

    The target is the anatomy rendered with noise; atlas k is the same anatomy
    deformed by its own seeded B-spline field (moving(p) = anatomy(p + disp_k(p)))
    with its own noise, and its labels deformed alike.  Returns dict(target,
    target_labels, atlas_images, atlas_labels) of Fortran-ordered volumes."""
    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    if n_organs is None:
        n_organs = int(rng.integers(6, 13))
    body, labels = _organ_labels(shape, n_organs, rng)
    organ_hu = rng.uniform(-100.0, 300.0, n_organs).astype(np.float32)
    clean = _render(body, labels, organ_hu, -1000.0, 0.0)
    grid = np.meshgrid(*[np.arange(s, dtype=np.float32) for s in shape], indexing="ij")
    images, labs = [], []
    for k in range(n_atlases):
        r = np.random.default_rng((seed, k + 1))
        disp = _bspline_field(shape, spacing, max_disp, r)
        coords = [grid[d] + disp[d] for d in range(3)]
        im = ndimage.map_coordinates(clean, coords, order=1, mode="nearest").astype(np.float32)
        im += r.normal(0.0, 20.0, shape).astype(np.float32)
        images.append(np.asfortranarray(im))
        labs.append(np.asfortranarray(ndimage.map_coordinates(labels, coords, order=0, mode="nearest").astype(np.uint8)))
    target = clean + rng.normal(0.0, 20.0, shape).astype(np.float32)
    return {"target": np.asfortranarray(target.astype(np.float32)), "target_labels": np.asfortranarray(labels),
            "atlas_images": images, "atlas_labels": labs}


def batch_workload(n=16, seed=100):
    """The uneven-size batch: n (shape, seed) pairs with dims drawn uniformly from
    128x112x144 up to 224x192x288; pair i is make_pair(shape, seed + 1 + i,
    max_disp=10.0)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        shape = (int(rng.integers(128, 225)), int(rng.integers(112, 193)), int(rng.integers(144, 289)))
        out.append((shape, seed + 1 + i))
    return out


def dice(a, b):
    """Mean Dice over the labels present in ``a`` except 0 (diceMulti's formula)."""
    a = np.asarray(a).ravel(order="F")
    b = np.asarray(b).ravel(order="F")
    scores = []
    for lab in np.unique(a):
        if lab == 0:
            continue
        pa, pb = a == lab, b == lab
        scores.append(2.0 * np.count_nonzero(pa & pb) / (np.count_nonzero(pa) + np.count_nonzero(pb)))
    return float(np.mean(scores)) if scores else 1.0
