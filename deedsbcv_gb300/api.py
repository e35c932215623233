"""Python mirror of the deeds hot-path functions over libdeeds_gpu's C ABI.

Function names and argument meaning follow the reference (mattiaspaul/deedsBCV)
so that code and tests read like it: ``descriptor`` (src/MINDSSCbox.h:127),
``dataCostCL`` (src/dataCostD.h:108), ``primsGraph`` (src/primsMST.h:52),
``regularisationCL`` (src/regularisation.h:115), ``upsampleDeformationsCL``
(src/transformations.h:245), ``warpAffine`` / ``warpImageCL`` / ``warpAffineS``
(src/dataCostD.h:213-315), ``consistentMappingCL`` (src/transformations.h:189),
``jacobian`` (src/transformations.h:84) and ``register`` (deedsBCV's main).
Instead of the reference's process globals, dimensions are explicit.

Stage functions take flat CUDA tensors whose element order is
``i + j*m + k*m*n`` (i fastest) and run on torch's current CUDA stream.  64-bit
descriptor codes are carried in int64 tensors (same bits as uint64).  Errors raise
``DeedsError``; nothing falls back to a CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import DeedsError, DeedsLinearParams, DeedsParams, DeedsSoftParams  # noqa: F401

try:  # torch is plumbing for device memory and streams only
    import torch
except ImportError:  # pragma: no cover
    torch = None


class Context:
    """One libdeeds_gpu context (device scratch + streams) on one CUDA device."""

    def __init__(self, device=0):
        self._L = _lib.load()
        self.handle = C.c_void_p()
        st = self._L.deeds_create(C.byref(self.handle), int(device))
        _lib.check(st, None)
        self.device = int(device)

    def close(self):
        if self.handle:
            self._L.deeds_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        _lib.check(st, self.handle)

    def set_profiling(self, on=True):
        self.check(self._L.deeds_set_profiling(self.handle, int(bool(on))))

    def reset_stage_times(self):
        self.check(self._L.deeds_reset_stage_times(self.handle))

    def stage_times(self):
        """{stage: (milliseconds, kernel launches)} accumulated since the last reset."""
        ms = (C.c_float * len(_lib.STAGES))()
        ln = (C.c_longlong * len(_lib.STAGES))()
        self.check(self._L.deeds_stage_times(self.handle, ms, ln))
        return {name: (float(ms[i]), int(ln[i])) for i, name in enumerate(_lib.STAGES)}

    def popc_rate(self):
        """Measured popc64 operations per second of this GPU (probe kernel)."""
        r = C.c_double()
        self.check(self._L.deeds_measure_popc_rate(self.handle, C.byref(r)))
        return r.value


_contexts = {}


def context(device=0) -> Context:
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


def kernel_launches():
    """Kernels launched by libdeeds_gpu in this process so far."""
    return int(_lib.load().deeds_kernel_launches())


def default_params(levels=None, grid=None, radius=None, quant=None, alpha=None, verbose=False):
    p = DeedsParams()
    _lib.load().deeds_default_params(C.byref(p))
    if grid is not None:
        n = len(grid)
        if radius is None or quant is None or len(radius) != n or len(quant) != n:
            raise ValueError("grid, radius and quant need the same number of levels")
        p.levels = n
        for i in range(n):
            p.grid[i], p.radius[i], p.quant[i] = int(grid[i]), int(radius[i]), int(quant[i])
    if levels is not None:
        p.levels = int(levels)
    if alpha is not None:
        p.alpha = float(alpha)
    p.verbose = int(bool(verbose))
    return p


def _dev(t, dtype, n, name):
    if torch is None or not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name}: expected a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name}: expected {dtype}, got {t.dtype}")
    if not t.is_contiguous() or t.numel() < n:
        raise ValueError(f"{name}: expected a contiguous tensor with >= {n} elements")
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _affine(X):
    if X is None:
        X = np.eye(4, dtype=np.float32).ravel()
    X = np.ascontiguousarray(np.asarray(X, dtype=np.float32).ravel())
    if X.size != 16:
        raise ValueError("X must have 16 elements")
    return X


def descriptor(im, m, n, o, qs, ctx=None):
    """MIND-SSC codes (int64 CUDA tensor, uint64 bits) of a float32 CUDA volume."""
    ctx = ctx or context(im.device.index or 0)
    sz = m * n * o
    out = torch.empty(sz, dtype=torch.int64, device=im.device)
    ctx.check(ctx._L.deeds_mind_ssc_dev(ctx.handle, _dev(im, torch.float32, sz, "im"), m, n, o, int(qs),
                                         C.c_void_p(out.data_ptr()), _stream()))
    return out


def dataCostCL(F, M, m, n, o, g, hw, q, alpha, ctx=None):
    """Hamming cost volume (float32 CUDA tensor, sz1*len3) of two code volumes."""
    ctx = ctx or context(F.device.index or 0)
    sz = m * n * o
    sz1 = (m // g) * (n // g) * (o // g)
    out = torch.empty(sz1 * (2 * hw + 1) ** 3, dtype=torch.float32, device=F.device)
    ctx.check(ctx._L.deeds_data_cost_dev(ctx.handle, _dev(F, torch.int64, sz, "F"), _dev(M, torch.int64, sz, "M"),
                                          m, n, o, int(g), int(hw), int(q), float(alpha),
                                          C.c_void_p(out.data_ptr()), _stream()))
    return out


def mst_edges(im, m, n, o, g, ctx=None):
    """Per-node block SADs to the 6 neighbours (CUDA tensor 6*sz1)."""
    ctx = ctx or context(im.device.index or 0)
    sz1 = (m // g) * (n // g) * (o // g)
    out = torch.empty(6 * sz1, dtype=torch.float32, device=im.device)
    ctx.check(ctx._L.deeds_mst_edges_dev(ctx.handle, _dev(im, torch.float32, m * n * o, "im"), m, n, o, int(g),
                                          C.c_void_p(out.data_ptr()), _stream()))
    return out


def image_stats(im_host):
    im = np.ascontiguousarray(np.asarray(im_host, dtype=np.float32).ravel(order="F"))
    mean = np.zeros(1, np.float32)
    sd = np.zeros(1, np.float32)
    _lib.check(_lib.load().deeds_image_stats(im.ctypes.data_as(C.c_void_p), im.size, mean.ctypes.data_as(C.c_void_p),
                                             sd.ctypes.data_as(C.c_void_p)))
    return float(mean[0]), float(sd[0])


def fuse_labels_device(target, images, labels, m, n, o, radius=2, eps=1.0, power=2, ctx=None):
    """Multi-atlas label fusion of atlases already warped onto ``target``
    (flat m*n*o float32 CUDA tensors, i fastest; ``labels`` int16 CUDA tensors): per voxel the label with
    the largest sum of weights (1 / (patch SSD + eps))^power, the patch being the
    (2 radius + 1)^3 window (clamp-to-edge); power 0 is majority voting.
    Returns the fused labels (int16 CUDA tensor)."""
    ctx = ctx or context(target.device.index or 0)
    n_atlas = len(images)
    if n_atlas != len(labels):
        raise ValueError("images and labels differ in count")
    sz = m * n * o
    ims = (C.c_void_p * n_atlas)(*[_dev(a, torch.float32, sz, "image").value for a in images])
    labs = (C.c_void_p * n_atlas)(*[_dev(a, torch.int16, sz, "labels").value for a in labels])
    out = torch.empty(sz, dtype=torch.int16, device=target.device)
    ctx.check(ctx._L.deeds_fuse_labels_dev(ctx.handle, _dev(target, torch.float32, sz, "target"), ims, labs, n_atlas,
                                            m, n, o, int(radius), C.c_float(eps), int(power),
                                            C.c_void_p(out.data_ptr()), _stream()))
    return out


def multi_atlas(target, atlas_images, atlas_labels, params=None, lanes=3, radius=2, eps=1.0, power=2, ctx=None):
    """Multi-atlas segmentation of ``target`` (numpy (m, n, o) volumes): every
    atlas image is registered to the target with deeds (batched), its labels are
    warped with the resulting field, and the warped labels are fused on the GPU
    (see fuse_labels_device).  Returns (fused labels, warped atlas labels, warped
    atlas images) as Fortran-ordered numpy arrays (int16, int16 (n, m, n, o),
    float32 (n, m, n, o))."""
    ctx = ctx or context(0)
    params = params or default_params()
    tgt = np.asfortranarray(np.asarray(target, np.float32))
    m, n, o = tgt.shape
    sz = m * n * o
    n_atlas = len(atlas_images)
    ims = [np.ascontiguousarray(np.asarray(a, np.float32).ravel(order="F")) for a in atlas_images]
    labs = [np.ascontiguousarray(np.asarray(a).astype(np.int16).ravel(order="F")) for a in atlas_labels]
    t_flat = np.ascontiguousarray(tgt.ravel(order="F"))
    fused = np.zeros(sz, np.int16)
    wl = np.zeros(n_atlas * sz, np.int16)
    wi = np.zeros(n_atlas * sz, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    ims_p = (C.c_void_p * n_atlas)(*[a.ctypes.data for a in ims])
    labs_p = (C.c_void_p * n_atlas)(*[a.ctypes.data for a in labs])
    ctx.check(ctx._L.deeds_multi_atlas(ctx.handle, p(t_flat), ims_p, labs_p, n_atlas, m, n, o, C.byref(params),
                                        int(lanes), int(radius), C.c_float(eps), int(power), p(fused), p(wl), p(wi)))
    shp = lambda a: a.reshape((m, n, o), order="F")  # noqa: E731
    return (shp(fused), [shp(wl[k * sz:(k + 1) * sz]) for k in range(n_atlas)],
            [shp(wi[k * sz:(k + 1) * sz]) for k in range(n_atlas)])


def image_stats_device(im, ctx=None):
    """The reference's mean and standard deviation of a float32 CUDA tensor,
    computed on the device (bit-identical to ``image_stats``)."""
    ctx = ctx or context(im.device.index or 0)
    out = torch.empty(2, dtype=torch.float32, device=im.device)
    ctx.check(ctx._L.deeds_image_stats_dev(ctx.handle, _dev(im, torch.float32, im.numel(), "im"), im.numel(),
                                            C.c_void_p(out.data_ptr()), _stream()))
    mean, sd = out.cpu().tolist()
    return mean, sd


def primsGraph(im, m, n, o, g, ctx=None):
    """MST of the control grid: (ordered, parents, edgemst) as numpy arrays.

    Edge SADs run on the GPU; the statistics and Prim's heap walk on the host.
    ``im`` is a float32 CUDA tensor (flat, i fastest)."""
    sad = mst_edges(im, m, n, o, g, ctx).cpu().numpy()
    _, sd = image_stats(im.cpu().numpy())
    m1, n1, o1 = m // g, n // g, o // g
    sz1 = m1 * n1 * o1
    ordered = np.zeros(sz1, np.int32)
    parents = np.zeros(sz1, np.int32)
    edgemst = np.zeros(sz1, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    _lib.check(_lib.load().deeds_prims_from_sad(p(sad), C.c_float(sd), m1, n1, o1, int(g), p(ordered), p(parents),
                                                p(edgemst)))
    return ordered, parents, edgemst


def regularisationCL(cost, u0, v0, w0, m1, n1, o1, hw, q, ordered, parents, edgemst, want_allinds=False, ctx=None):
    """Tree BP.  ``cost`` (CUDA) is overwritten with the upward-pass state.
    Returns (u1, v1, w1[, allinds]) as CUDA tensors."""
    ctx = ctx or context(cost.device.index or 0)
    sz1 = m1 * n1 * o1
    len3 = (2 * hw + 1) ** 3
    dev = cost.device
    u1 = torch.empty(sz1, dtype=torch.float32, device=dev)
    v1 = torch.empty_like(u1)
    w1 = torch.empty_like(u1)
    ai = torch.empty(sz1 * len3, dtype=torch.int16, device=dev) if want_allinds else None
    ordered = np.ascontiguousarray(ordered, np.int32)
    parents = np.ascontiguousarray(parents, np.int32)
    edgemst = np.ascontiguousarray(edgemst, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    ctx.check(ctx._L.deeds_tree_bp_dev(
        ctx.handle, _dev(cost, torch.float32, sz1 * len3, "cost"), _dev(u0, torch.float32, sz1, "u0"),
        _dev(v0, torch.float32, sz1, "v0"), _dev(w0, torch.float32, sz1, "w0"), m1, n1, o1, int(hw), int(q),
        p(ordered), p(parents), p(edgemst), C.c_void_p(u1.data_ptr()), C.c_void_p(v1.data_ptr()),
        C.c_void_p(w1.data_ptr()), C.c_void_p(ai.data_ptr()) if ai is not None else None, _stream()))
    return (u1, v1, w1, ai) if want_allinds else (u1, v1, w1)


def upsampleDeformationsCL(u0, v0, w0, m2, n2, o2, m, n, o):
    s2 = m2 * n2 * o2
    dev = u0.device
    u = torch.empty(m * n * o, dtype=torch.float32, device=dev)
    v = torch.empty_like(u)
    w = torch.empty_like(u)
    _lib.check(_lib.load().deeds_upsample_dev(
        _dev(u0, torch.float32, s2, "u0"), _dev(v0, torch.float32, s2, "v0"), _dev(w0, torch.float32, s2, "w0"),
        m2, n2, o2, C.c_void_p(u.data_ptr()), C.c_void_p(v.data_ptr()), C.c_void_p(w.data_ptr()), m, n, o,
        _stream()))
    return u, v, w


def warpAffine(im, X, u, v, w, m, n, o):
    sz = m * n * o
    X = _affine(X)
    out = torch.empty(sz, dtype=torch.float32, device=im.device)
    fu = _dev(u, torch.float32, sz, "u") if u is not None else None
    fv = _dev(v, torch.float32, sz, "v") if v is not None else None
    fw = _dev(w, torch.float32, sz, "w") if w is not None else None
    _lib.check(_lib.load().deeds_warp_affine_dev(_dev(im, torch.float32, sz, "im"), X.ctypes.data_as(C.c_void_p),
                                                 fu, fv, fw, m, n, o, C.c_void_p(out.data_ptr()), _stream()))
    return out


def warpImageCL(im, u, v, w, m, n, o):
    sz = m * n * o
    out = torch.empty(sz, dtype=torch.float32, device=im.device)
    _lib.check(_lib.load().deeds_warp_image_dev(_dev(im, torch.float32, sz, "im"), _dev(u, torch.float32, sz, "u"),
                                                _dev(v, torch.float32, sz, "v"), _dev(w, torch.float32, sz, "w"),
                                                m, n, o, C.c_void_p(out.data_ptr()), _stream()))
    return out


def warpAffineS(seg, X, u, v, w, m, n, o):
    sz = m * n * o
    X = _affine(X)
    out = torch.empty(sz, dtype=torch.int16, device=seg.device)
    _lib.check(_lib.load().deeds_warp_seg_dev(_dev(seg, torch.int16, sz, "seg"), X.ctypes.data_as(C.c_void_p),
                                              _dev(u, torch.float32, sz, "u"), _dev(v, torch.float32, sz, "v"),
                                              _dev(w, torch.float32, sz, "w"), m, n, o,
                                              C.c_void_p(out.data_ptr()), _stream()))
    return out


def consistentMappingCL(u, v, w, u2, v2, w2, m, n, o, g, ctx=None):
    """In place on six CUDA tensors."""
    ctx = ctx or context(u.device.index or 0)
    sz = m * n * o
    ptrs = [_dev(t, torch.float32, sz, nm) for t, nm in zip((u, v, w, u2, v2, w2), ("u", "v", "w", "u2", "v2", "w2"))]
    ctx.check(ctx._L.deeds_consistent_dev(ctx.handle, *ptrs, m, n, o, int(g), _stream()))


def jacobian(u, v, w, m, n, o, g, ctx=None):
    ctx = ctx or context(u.device.index or 0)
    sz = m * n * o
    js = C.c_float()
    neg = C.c_float()
    ctx.check(ctx._L.deeds_jacobian_dev(ctx.handle, _dev(u, torch.float32, sz, "u"), _dev(v, torch.float32, sz, "v"),
                                         _dev(w, torch.float32, sz, "w"), m, n, o, int(g), C.byref(js), C.byref(neg),
                                         _stream()))
    return js.value, neg.value


def _host(a, dtype, name):
    a = np.asarray(a)
    if a.ndim == 3:
        a = a.ravel(order="F")
    return np.ascontiguousarray(a, dtype=dtype)


def register(fixed, moving, dims=None, X=None, params=None, want_warped=True, ctx=None):
    """Full deeds registration of host volumes (raw intensities, e.g. HU).

    Returns (flow, warped): flow is the *_displacements.dat payload (3*sz1
    float32, [u|v|w] on the last grid), warped the moving image resampled by the
    final field (or None)."""
    if dims is None:
        dims = np.asarray(fixed).shape
    m, n, o = (int(d) for d in dims)
    ctx = ctx or context(0)
    params = params or default_params()
    f = _host(fixed, np.float32, "fixed")
    mv = _host(moving, np.float32, "moving")
    Xa = _affine(X)
    g = params.grid[params.levels - 1]
    flow = np.zeros(3 * (m // g) * (n // g) * (o // g), np.float32)
    warped = np.zeros(m * n * o, np.float32) if want_warped else None
    p = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None  # noqa: E731
    ctx.check(ctx._L.deeds_register(ctx.handle, p(f), p(mv), m, n, o, p(Xa), C.byref(params), p(flow), p(warped)))
    return flow, warped


def register_batch(pairs, params=None, lanes=0, want_warped=False, ctx=None):
    """Register a list of (fixed, moving[, X]) host volume pairs, possibly of
    different sizes, with several pairs in flight (deeds_register_batch).
    Returns a list of (flow, warped-or-None)."""
    ctx = ctx or context(0)
    params = params or default_params()
    n = len(pairs)
    arr = (_lib.DeedsPair * max(n, 1))()
    keep = []
    outs = []
    g = params.grid[params.levels - 1]
    for i, pr in enumerate(pairs):
        fixed, moving = pr[0], pr[1]
        X = pr[2] if len(pr) > 2 else None
        m, nn, o = (int(d) for d in np.asarray(fixed).shape)
        f = _host(fixed, np.float32, "fixed")
        mv = _host(moving, np.float32, "moving")
        Xa = _affine(X)
        flow = np.zeros(3 * (m // g) * (nn // g) * (o // g), np.float32)
        warped = np.zeros(m * nn * o, np.float32) if want_warped else None
        keep += [f, mv, Xa]
        outs.append((flow, warped))
        p = lambda a: a.ctypes.data_as(C.c_void_p).value if a is not None else None  # noqa: E731
        arr[i] = _lib.DeedsPair(p(f), p(mv), m, nn, o, p(Xa), p(flow), p(warped))
    ctx.check(ctx._L.deeds_register_batch(ctx.handle, arr, n, C.byref(params), int(lanes)))
    return outs


def register_device(fixed, moving, m, n, o, X=None, params=None, flow_out=None, warped_out=None, ctx=None):
    """Full registration of device-resident volumes (float32 CUDA tensors)."""
    ctx = ctx or context(fixed.device.index or 0)
    params = params or default_params()
    sz = m * n * o
    g = params.grid[params.levels - 1]
    sz1 = (m // g) * (n // g) * (o // g)
    if flow_out is None:
        flow_out = torch.empty(3 * sz1, dtype=torch.float32, device=fixed.device)
    Xa = _affine(X)
    ctx.check(ctx._L.deeds_register_dev(ctx.handle, _dev(fixed, torch.float32, sz, "fixed"),
                                         _dev(moving, torch.float32, sz, "moving"), m, n, o,
                                         Xa.ctypes.data_as(C.c_void_p), C.byref(params),
                                         _dev(flow_out, torch.float32, 3 * sz1, "flow_out"),
                                         _dev(warped_out, torch.float32, sz, "warped_out") if warped_out is not None
                                         else None, _stream()))
    return flow_out


def warp_segmentation(seg, ctx=None):
    """Warp an int16 label volume by the context's last registration (the -S output)."""
    ctx = ctx or context(0)
    s = _host(seg, np.int16, "seg")
    out = np.zeros_like(s)
    ctx.check(ctx._L.deeds_warp_segmentation(ctx.handle, s.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)))
    return out


def apply_flow(flow, volume, dims=None, X=None, grid_step=0, ctx=None):
    """applyBCV (int16 labels, nearest) / applyBCVfloat (float, trilinear)."""
    ctx = ctx or context(0)
    if dims is None:
        dims = np.asarray(volume).shape
    m, n, o = (int(d) for d in dims)
    fl = np.ascontiguousarray(np.asarray(flow, np.float32).ravel())
    vol = np.asarray(volume)
    if vol.dtype == np.int16 or np.issubdtype(vol.dtype, np.integer):
        v = _host(vol, np.int16, "volume")
        dtype = 0
    else:
        v = _host(vol, np.float32, "volume")
        dtype = 1
    out = np.zeros_like(v)
    Xa = _affine(X)
    ctx.check(ctx._L.deeds_apply_flow(ctx.handle, fl.ctypes.data_as(C.c_void_p), fl.size, int(grid_step),
                                       Xa.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p), dtype, m, n, o,
                                       out.ctypes.data_as(C.c_void_p)))
    return out


# ---------------------------------------------------------------------------
# Soft-min form (no counterpart in the reference): one deeds level relaxed so that
# it is differentiable in both images and alpha.  See include/deeds_gpu.h.

def soft_params(grid=4, radius=3, quant=1, alpha=1.6, tau=0.5, eps=0.01, mind_radius=0):
    p = DeedsSoftParams()
    _lib.load().deeds_soft_default_params(C.byref(p))
    p.grid, p.radius, p.quant, p.mind_radius = int(grid), int(radius), int(quant), int(mind_radius)
    p.alpha, p.tau, p.eps = float(alpha), float(tau), float(eps)
    return p


def soft_descriptor(im, m, n, o, qs, ctx=None):
    """Continuous MIND-SSC levels 6*exp(-mind1): float32 CUDA tensor (12, m*n*o)."""
    ctx = ctx or context(im.device.index or 0)
    sz = m * n * o
    out = torch.empty(12 * sz, dtype=torch.float32, device=im.device)
    ctx.check(ctx._L.deeds_soft_descriptor_dev(ctx.handle, _dev(im, torch.float32, sz, "im"), m, n, o, int(qs),
                                                C.c_void_p(out.data_ptr()), _stream()))
    return out.view(12, sz)


def soft_cost(sF, sM, m, n, o, params, ctx=None):
    """Soft cost volume (sz1, len3) of two soft descriptors."""
    ctx = ctx or context(sF.device.index or 0)
    sz = m * n * o
    g, hw = params.grid, params.radius
    sz1 = (m // g) * (n // g) * (o // g)
    len3 = (2 * hw + 1) ** 3
    out = torch.empty(sz1 * len3, dtype=torch.float32, device=sF.device)
    ctx.check(ctx._L.deeds_soft_cost_dev(ctx.handle, _dev(sF, torch.float32, 12 * sz, "sF"),
                                          _dev(sM, torch.float32, 12 * sz, "sM"), m, n, o, C.byref(params),
                                          C.c_void_p(out.data_ptr()), _stream()))
    return out.view(sz1, len3)


def _tree_arrays(tree):
    ordered, parents, edgemst = tree
    return (np.ascontiguousarray(ordered, np.int32), np.ascontiguousarray(parents, np.int32),
            np.ascontiguousarray(edgemst, np.float32))


def _soft_call(ctx, fn, fixed, moving, dims, params, tree, *rest):
    m, n, o = dims
    sz = m * n * o
    ordered, parents, edgemst = tree
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    ctx.check(fn(ctx.handle, _dev(fixed, torch.float32, sz, "fixed"), _dev(moving, torch.float32, sz, "moving"),
                 m, n, o, C.byref(params), p(ordered), p(parents), p(edgemst), *rest, _stream()))


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class _KeptSoftState:
    """A library slot that holds one soft level's forward state; released when
    the backward has used it or when the autograd node goes away."""

    def __init__(self, dctx, slot):
        self.dctx, self.slot = dctx, slot

    def release(self):
        if self.slot is not None and self.dctx.handle:
            self.dctx._L.deeds_soft_release(self.dctx.handle, self.slot)
        self.slot = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class SoftDeedsLevel(torch.autograd.Function if torch is not None else object):
    """Expected displacement (3, sz1) [u, v, w] of one soft-min deeds level.

    forward(fixed, moving, alpha, prior, dims, params, tree, ctx, keep): fixed/moving
    are flat float32 CUDA tensors (i fastest), alpha a 0-d tensor (its value
    replaces params.alpha), prior None or the current grid field (3, sz1) that the
    pairwise term is taken relative to (src/regularisation.h:205-208), tree =
    (ordered, parents, edgemst) host arrays of the fixed image's MST at params.grid.
    With keep (and a gradient wanted) the library keeps the level's descriptors,
    cost volume, messages and marginals on the device and the backward runs only
    the adjoint kernels; without it the backward recomputes the forward state."""

    @staticmethod
    def forward(fctx, fixed, moving, alpha, prior, dims, params, tree, dctx, keep=True):
        params = soft_params(params.grid, params.radius, params.quant, float(alpha.detach()), params.tau, params.eps,
                             params.mind_radius)
        tree = _tree_arrays(tree)
        m, n, o = dims
        g = params.grid
        sz1 = (m // g) * (n // g) * (o // g)
        out = torch.empty(3 * sz1, dtype=torch.float32, device=fixed.device)
        fixed_c, moving_c = fixed.detach().contiguous(), moving.detach().contiguous()
        prior_c = None
        if prior is not None:
            prior_c = prior.detach().contiguous()
            _dev(prior_c, torch.float32, 3 * sz1, "prior")
        fctx.kept = None
        if keep and any(fctx.needs_input_grad[:4]):
            slot = C.c_int(-1)
            _soft_call(dctx, dctx._L.deeds_soft_forward_keep_dev, fixed_c, moving_c, dims, params, tree,
                       _ptr(prior_c), _ptr(out), C.byref(slot))
            fctx.kept = _KeptSoftState(dctx, slot.value)
        else:
            _soft_call(dctx, dctx._L.deeds_soft_forward_dev, fixed_c, moving_c, dims, params, tree, _ptr(prior_c),
                       _ptr(out))
        fctx.save_for_backward(fixed_c, moving_c, prior_c)
        fctx.soft = (dims, params, tree, dctx)
        fctx.alpha_like = (alpha.dtype, alpha.device) if isinstance(alpha, torch.Tensor) else (torch.float32, "cpu")
        return out.view(3, sz1)

    @staticmethod
    def backward(fctx, gdisp):
        fixed, moving, prior = fctx.saved_tensors
        dims, params, tree, dctx = fctx.soft
        gdisp = gdisp.detach().contiguous().to(torch.float32)
        need_f, need_m, need_a, need_p = fctx.needs_input_grad[:4]
        gf = torch.empty_like(fixed) if need_f else None
        gm = torch.empty_like(moving) if need_m else None
        gp = torch.empty_like(prior) if (need_p and prior is not None) else None
        ga = C.c_float(0.0)
        grads = (_ptr(gdisp), _ptr(gf), _ptr(gm), _ptr(gp), C.byref(ga) if need_a else None)
        kept = fctx.kept
        if kept is not None and kept.slot is not None:
            m, n, o = dims
            sz = m * n * o
            dctx.check(dctx._L.deeds_soft_backward_kept_dev(
                dctx.handle, kept.slot, _dev(fixed, torch.float32, sz, "fixed"),
                _dev(moving, torch.float32, sz, "moving"), m, n, o, C.byref(params), _ptr(prior), *grads, _stream()))
            kept.release()  # a second backward (retain_graph) recomputes
        else:
            _soft_call(dctx, dctx._L.deeds_soft_backward_dev, fixed, moving, dims, params, tree, _ptr(prior), *grads)
        adt, adev = fctx.alpha_like
        galpha = torch.tensor(ga.value, dtype=adt, device=adev) if need_a else None
        return gf, gm, galpha, gp, None, None, None, None, None


class SoftUpsample(torch.autograd.Function if torch is not None else object):
    """Trilinear upsampling of a grid field (3, mA*nA*oA) to (3, m*n*o) with the
    coordinates of upsampleDeformationsCL (src/transformations.h:245-279)."""

    @staticmethod
    def forward(fctx, field, src_dims, dst_dims, dctx):
        mA, nA, oA = src_dims
        m, n, o = dst_dims
        f = _dev(field.detach().contiguous(), torch.float32, 3 * mA * nA * oA, "field")
        out = torch.empty(3 * m * n * o, dtype=torch.float32, device=field.device)
        dctx.check(dctx._L.deeds_soft_upsample_dev(dctx.handle, f, mA, nA, oA, _ptr(out), m, n, o, _stream()))
        fctx.dims = (tuple(src_dims), tuple(dst_dims), dctx)
        return out.view(3, m * n * o)

    @staticmethod
    def backward(fctx, gout):
        (mA, nA, oA), (m, n, o), dctx = fctx.dims
        gout = gout.detach().contiguous().to(torch.float32)
        gin = torch.empty(3 * mA * nA * oA, dtype=torch.float32, device=gout.device)
        dctx.check(dctx._L.deeds_soft_upsample_backward_dev(dctx.handle, _ptr(gout), m, n, o, _ptr(gin), mA, nA, oA,
                                                             _stream()))
        return gin.view(3, mA * nA * oA), None, None, None


class SoftWarp(torch.autograd.Function if torch is not None else object):
    """The moving image (flat, m*n*o) sampled at p + field(p), field = the grid
    field (3, mA*nA*oA) upsampled to full resolution on the fly (warpAffine with the
    identity, src/dataCostD.h:267-295); differentiable in the image and the grid."""

    @staticmethod
    def forward(fctx, moving, grid, dims, grid_dims, dctx):
        m, n, o = dims
        mA, nA, oA = grid_dims
        mov = moving.detach().contiguous()
        gr = grid.detach().contiguous()
        out = torch.empty(m * n * o, dtype=torch.float32, device=moving.device)
        dctx.check(dctx._L.deeds_soft_warp_dev(dctx.handle, _dev(mov, torch.float32, m * n * o, "moving"), m, n, o,
                                               _dev(gr, torch.float32, 3 * mA * nA * oA, "grid"), mA, nA, oA,
                                               _ptr(out), _stream()))
        fctx.save_for_backward(mov, gr)
        fctx.dims = (tuple(dims), tuple(grid_dims), dctx)
        return out

    @staticmethod
    def backward(fctx, gout):
        mov, gr = fctx.saved_tensors
        (m, n, o), (mA, nA, oA), dctx = fctx.dims
        need_m, need_g = fctx.needs_input_grad[:2]
        gout = gout.detach().contiguous().to(torch.float32)
        gm = torch.empty_like(mov) if need_m else None
        gg = torch.empty_like(gr) if need_g else None
        dctx.check(dctx._L.deeds_soft_warp_backward_dev(dctx.handle, _ptr(mov), m, n, o, _ptr(gr), mA, nA, oA,
                                                         _ptr(gout), _ptr(gm), _ptr(gg), _stream()))
        return gm, gg, None, None, None


def soft_tree(fixed, m, n, o, g, ctx=None):
    """The hard path's MST of the fixed image at grid g (constant for the soft level)."""
    return primsGraph(fixed.detach().contiguous(), m, n, o, g, ctx)


def soft_level(fixed, moving, alpha, dims, grid=4, radius=3, quant=1, tau=0.5, eps=0.01, mind_radius=0, tree=None,
               ctx=None, keep_state=True):
    """Differentiable soft-min deeds level: expected displacement (3, sz1) [u, v, w].

    Gradients flow to ``fixed`` and ``moving`` (through the continuous MIND-SSC
    descriptor) and to ``alpha`` (a float or 0-d tensor).  keep_state=False trades
    the resident forward state for a recomputation in the backward."""
    m, n, o = dims
    ctx = ctx or context(fixed.device.index or 0)
    if tree is None:
        tree = soft_tree(fixed, m, n, o, grid, ctx)
    if not isinstance(alpha, torch.Tensor):
        alpha = torch.tensor(float(alpha), dtype=torch.float32)
    params = soft_params(grid, radius, quant, float(alpha.detach()), tau, eps, mind_radius)
    return SoftDeedsLevel.apply(fixed, moving, alpha, None, tuple(dims), params, tree, ctx, keep_state)


def soft_register_levels(fixed, moving, alpha, dims, levels, tau=0.5, eps=0.01, trees=None, ctx=None,
                         keep_state=True):
    """Differentiable multi-level soft-min registration (the level loop of
    src/deedsBCV0.cpp:222-306, forward direction).

    levels: [(grid, radius, quant, mind_radius)], coarse to fine.  At each level the
    prior grid field U is the previous level's field upsampled to this grid
    (zero at the first level), the moving image is warped by U at full resolution,
    and the soft level's expected displacement E is taken relative to U; the level
    returns U + E.  Returns the last grid field (3, sz1) [u, v, w].  trees: the
    fixed image's MST per level (computed when None); keep_state as in soft_level."""
    m, n, o = dims
    ctx = ctx or context(fixed.device.index or 0)
    if not isinstance(alpha, torch.Tensor):
        alpha = torch.tensor(float(alpha), dtype=torch.float32)
    prev, prev_dims = None, None
    for li, (g, hw, q, qs) in enumerate(levels):
        gdims = (m // g, n // g, o // g)
        tree = trees[li] if trees is not None else soft_tree(fixed, m, n, o, g, ctx)
        params = soft_params(g, hw, q, float(alpha.detach()), tau, eps, qs)
        if prev is None:
            E = SoftDeedsLevel.apply(fixed, moving, alpha, None, tuple(dims), params, tree, ctx, keep_state)
            prev = E
        else:
            U = SoftUpsample.apply(prev, prev_dims, gdims, ctx)
            warped = SoftWarp.apply(moving, U, tuple(dims), gdims, ctx)
            E = SoftDeedsLevel.apply(fixed, warped, alpha, U, tuple(dims), params, tree, ctx, keep_state)
            prev = U + E
        prev_dims = gdims
    return prev


def _ptrs(ts):
    """ctypes array of the data pointers of a sequence of tensors / numpy arrays."""
    vals = [t.data_ptr() if isinstance(t, torch.Tensor) else t.ctypes.data for t in ts]
    return (C.c_void_p * len(vals))(*vals)


class _KeptSoftBatch:
    """The library slots holding a batch's forward states (one per pair, in the
    pairs' lanes); released after the backward or with the autograd node."""

    def __init__(self, dctx, slots):
        self.dctx, self.slots = dctx, slots

    def release(self):
        if self.slots is not None and self.dctx.handle:
            self.dctx._L.deeds_soft_release_batch(self.dctx.handle, len(self.slots), self.slots)
        self.slots = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


class SoftDeedsLevelBatch(torch.autograd.Function if torch is not None else object):
    """SoftDeedsLevel for P pairs of one size at once: fixed/moving (P, m*n*o),
    prior None or (P, 3, sz1), trees a list of P MSTs; returns (P, 3, sz1).  The
    library runs the pairs concurrently on lane streams (the tree sweeps of one
    pair are latency-bound and leave SMs to the others).  keep as in
    SoftDeedsLevel."""

    @staticmethod
    def forward(fctx, fixed, moving, alpha, prior, dims, params, trees, dctx, keep=True):
        params = soft_params(params.grid, params.radius, params.quant, float(alpha.detach()), params.tau, params.eps,
                             params.mind_radius)
        m, n, o = dims
        sz = m * n * o
        g = params.grid
        sz1 = (m // g) * (n // g) * (o // g)
        npairs = fixed.shape[0]
        trees = [_tree_arrays(t) for t in trees]
        if len(trees) != npairs or moving.shape[0] != npairs:
            raise ValueError("fixed, moving and trees need one entry per pair")
        fixed_c, moving_c = fixed.detach().contiguous(), moving.detach().contiguous()
        _dev(fixed_c, torch.float32, npairs * sz, "fixed")
        _dev(moving_c, torch.float32, npairs * sz, "moving")
        if fixed_c.numel() != npairs * sz or moving_c.numel() != npairs * sz:
            raise ValueError(f"fixed/moving: expected ({npairs}, {sz})")
        prior_c = None
        if prior is not None:
            prior_c = prior.detach().contiguous()
            _dev(prior_c, torch.float32, npairs * 3 * sz1, "prior")
        out = torch.empty(npairs, 3, sz1, dtype=torch.float32, device=fixed.device)
        slots = None
        if keep and any(fctx.needs_input_grad[:4]):
            slots = (C.c_int * npairs)()
        dctx.check(dctx._L.deeds_soft_forward_batch_dev(
            dctx.handle, npairs, _ptrs(fixed_c.view(npairs, sz)), _ptrs(moving_c.view(npairs, sz)), m, n, o,
            C.byref(params), _ptrs([t[0] for t in trees]), _ptrs([t[1] for t in trees]), _ptrs([t[2] for t in trees]),
            _ptrs(prior_c.view(npairs, -1)) if prior_c is not None else None, _ptrs(out), slots, _stream()))
        fctx.kept = _KeptSoftBatch(dctx, slots) if slots is not None else None
        fctx.save_for_backward(fixed_c, moving_c, prior_c)
        fctx.soft = (dims, params, trees, dctx)
        fctx.alpha_like = (alpha.dtype, alpha.device)
        return out

    @staticmethod
    def backward(fctx, gdisp):
        fixed, moving, prior = fctx.saved_tensors
        dims, params, trees, dctx = fctx.soft
        m, n, o = dims
        npairs = len(trees)
        gdisp = gdisp.detach().contiguous().to(torch.float32)
        need_f, need_m, need_a, need_p = fctx.needs_input_grad[:4]
        fv, mv = fixed.view(npairs, -1), moving.view(npairs, -1)
        gf = torch.empty_like(fixed) if need_f else None
        gm = torch.empty_like(moving) if need_m else None
        gp = torch.empty_like(prior) if (need_p and prior is not None) else None
        ga = (C.c_float * npairs)() if need_a else None
        kept = fctx.kept
        slots = kept.slots if kept is not None else None
        rows = lambda t: _ptrs(t.view(npairs, -1)) if t is not None else None  # noqa: E731
        dctx.check(dctx._L.deeds_soft_backward_batch_dev(
            dctx.handle, npairs, slots, _ptrs(fv), _ptrs(mv), m, n, o, C.byref(params), _ptrs([t[0] for t in trees]),
            _ptrs([t[1] for t in trees]), _ptrs([t[2] for t in trees]), rows(prior), rows(gdisp), rows(gf), rows(gm),
            rows(gp), ga, _stream()))
        if slots is not None:
            kept.release()  # a second backward (retain_graph) recomputes
        adt, adev = fctx.alpha_like
        galpha = torch.tensor(float(sum(ga)), dtype=adt, device=adev) if need_a else None
        return gf, gm, galpha, gp, None, None, None, None, None


def soft_register_levels_batch(fixed, moving, alpha, dims, levels, tau=0.5, eps=0.01, trees=None, ctx=None,
                               keep_state=True):
    """soft_register_levels for P pairs of one size at once, the pairs of each
    level running concurrently (SoftDeedsLevelBatch).  fixed/moving: (P, m*n*o)
    tensors or lists of P flat tensors; trees: per pair, the list of its
    per-level MSTs (computed when None).  Returns the last grid fields
    (P, 3, sz1); pair i's field and gradients are those of soft_register_levels
    on pair i."""
    m, n, o = dims
    if isinstance(fixed, (list, tuple)):
        fixed = torch.stack([f.reshape(-1) for f in fixed])
    if isinstance(moving, (list, tuple)):
        moving = torch.stack([mv.reshape(-1) for mv in moving])
    npairs = fixed.shape[0]
    ctx = ctx or context(fixed.device.index or 0)
    if not isinstance(alpha, torch.Tensor):
        alpha = torch.tensor(float(alpha), dtype=torch.float32)
    if trees is None:
        trees = [[soft_tree(fixed[i], m, n, o, lv[0], ctx) for lv in levels] for i in range(npairs)]
    prev, prev_dims = None, None
    for li, (g, hw, q, qs) in enumerate(levels):
        gdims = (m // g, n // g, o // g)
        params = soft_params(g, hw, q, float(alpha.detach()), tau, eps, qs)
        level_trees = [trees[i][li] for i in range(npairs)]
        if prev is None:
            prev = SoftDeedsLevelBatch.apply(fixed, moving, alpha, None, tuple(dims), params, level_trees, ctx,
                                             keep_state)
        else:
            U = torch.stack([SoftUpsample.apply(prev[i], prev_dims, gdims, ctx) for i in range(npairs)])
            warped = torch.stack([SoftWarp.apply(moving[i], U[i], tuple(dims), gdims, ctx) for i in range(npairs)])
            E = SoftDeedsLevelBatch.apply(fixed, warped, alpha, U, tuple(dims), params, level_trees, ctx, keep_state)
            prev = U + E
        prev_dims = gdims
    return prev


# ---------------------------------------------------------------------------
# linearBCV (src/linearBCV.cpp): affine / rigid pre-registration.

def linear_params(grid=(7, 6, 5, 4), radius=(5, 4, 3, 2), quant=(4, 3, 2, 1), rigid=False, verbose=False):
    p = DeedsLinearParams()
    _lib.load().deeds_linear_default_params(C.byref(p))
    if not (len(grid) == len(radius) == len(quant)):
        raise ValueError("grid, radius and quant need the same number of levels")
    p.levels = len(grid)
    for i in range(len(grid)):
        p.grid[i], p.radius[i], p.quant[i] = int(grid[i]), int(radius[i]), int(quant[i])
    p.rigid = int(bool(rigid))
    p.verbose = int(bool(verbose))
    return p


def linear_register(fixed, moving, dims, params=None, ctx=None):
    """The linearBCV matrix (16 float32, deeds layout) of two volumes in HU.

    fixed/moving: float32 arrays (flat, i fastest, or (m, n, o) Fortran-ordered)
    on the host, or flat float32 CUDA tensors; +1024 is applied inside."""
    m, n, o = dims
    params = params or linear_params()
    X = np.zeros(16, np.float32)
    if torch is not None and isinstance(fixed, torch.Tensor) and fixed.is_cuda:
        ctx = ctx or context(fixed.device.index or 0)
        sz = m * n * o
        ctx.check(ctx._L.deeds_linear_register_dev(ctx.handle, _dev(fixed, torch.float32, sz, "fixed"),
                                                   _dev(moving, torch.float32, sz, "moving"), m, n, o,
                                                   C.byref(params), X.ctypes.data_as(C.c_void_p), _stream()))
        return X
    ctx = ctx or context(0)
    f = np.ascontiguousarray(np.asarray(fixed, np.float32).ravel(order="F"))
    mv = np.ascontiguousarray(np.asarray(moving, np.float32).ravel(order="F"))
    ctx.check(ctx._L.deeds_linear_register(ctx.handle, f.ctypes.data_as(C.c_void_p), mv.ctypes.data_as(C.c_void_p),
                                           m, n, o, C.byref(params), X.ctypes.data_as(C.c_void_p)))
    return X


def warpAffineLinear(im, X, m, n, o):
    """warpAffine of src/affineLTS1.h:39-68 (affine only, zero outside) on a CUDA tensor."""
    sz = m * n * o
    X = _affine(X)
    out = torch.empty(sz, dtype=torch.float32, device=im.device)
    _lib.check(_lib.load().deeds_lin_warp_dev(_dev(im, torch.float32, sz, "im"), X.ctypes.data_as(C.c_void_p),
                                              m, n, o, C.c_void_p(out.data_ptr()), _stream()))
    return out


def smoothCosts(cost, m1, n1, o1, len3):
    """The in-place smoothing passes of estimateAffine2 on one cost volume (CUDA tensor)."""
    _lib.check(_lib.load().deeds_lin_smooth_dev(_dev(cost, torch.float32, m1 * n1 * o1 * len3, "cost"), m1, n1, o1,
                                                int(len3), _stream()))
    return cost


def estimateAffine2(Xprev, fixed, moving, cost, cost2, m, n, o, g, q, hw, rigid=False, ctx=None):
    """estimateAffine2 on CUDA tensors (+1024-shifted images; the cost volumes are
    smoothed in place): (X, points used)."""
    ctx = ctx or context(fixed.device.index or 0)
    sz = m * n * o
    len3 = (2 * hw + 1) ** 3
    sz1 = (m // g) * (n // g) * (o // g)
    Xp = _affine(Xprev)
    X = np.zeros(16, np.float32)
    used = C.c_int(0)
    ctx.check(ctx._L.deeds_estimate_affine_dev(
        ctx.handle, _dev(fixed, torch.float32, sz, "fixed"), _dev(moving, torch.float32, sz, "moving"),
        _dev(cost, torch.float32, sz1 * len3, "cost"), _dev(cost2, torch.float32, sz1 * len3, "cost2"), m, n, o,
        int(g), int(hw), int(q), int(bool(rigid)), Xp.ctypes.data_as(C.c_void_p), X.ctypes.data_as(C.c_void_p),
        C.byref(used), _stream()))
    return X, used.value


def affineRobust(pts1, pts2, length, rigid=False):
    """affineRobust (src/QRsolve.h:258-296) on host point sets (column layout)."""
    p1 = np.ascontiguousarray(pts1, np.float32)
    p2 = np.ascontiguousarray(pts2, np.float32)
    RT = np.zeros(16, np.float32)
    _lib.check(_lib.load().deeds_affine_robust(p1.ctypes.data_as(C.c_void_p), p2.ctypes.data_as(C.c_void_p),
                                               int(length), int(bool(rigid)), RT.ctypes.data_as(C.c_void_p)), None)
    return RT


def affine_warp_segmentation(seg, dims, X, ctx=None):
    """The -S output of linearBCV: int16 labels warped by X alone (host arrays)."""
    m, n, o = dims
    ctx = ctx or context(0)
    sg = np.ascontiguousarray(np.asarray(seg, np.int16).ravel(order="F"))
    out = np.zeros_like(sg)
    Xa = _affine(X)
    ctx.check(ctx._L.deeds_affine_warp_segmentation(ctx.handle, sg.ctypes.data_as(C.c_void_p), m, n, o,
                                                    Xa.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)))
    return out
