"""ORACLE (test infrastructure only): ctypes binding of oracle/deeds_oracle.cpp.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, as the checker.  Volumes are numpy arrays whose flat order is
``i + j*m + k*m*n`` (pass Fortran-ordered (m, n, o) arrays or flat vectors).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build(quiet=True):
    """Compile the oracle library (and nothing else) with make."""
    out = subprocess.run(["make", "-C", HERE, "all"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


P = C.c_void_p
I = C.c_int
F = C.c_float


def _declare(L):
    L.orc_mind_step.argtypes = [I]; L.orc_mind_step.restype = I
    L.orc_mind_thresholds.argtypes = [P]
    L.orc_descriptor.argtypes = [P, P, I, I, I, I]
    L.orc_datacost_alpha1.argtypes = [I, F, F]; L.orc_datacost_alpha1.restype = F
    L.orc_data_cost.argtypes = [P, P, P, I, I, I, I, I, I, F]
    L.orc_image_stats.argtypes = [P, C.c_size_t, P, P]
    L.orc_edge_sad.argtypes = [P, P, I, I, I, I]
    L.orc_prims_from_sad.argtypes = [P, F, I, I, I, I, P, P, P]
    L.orc_prims_graph.argtypes = [P, I, I, I, I, P, P, P]
    L.orc_message_dt.argtypes = [P, P, I, F, F, F]
    L.orc_regularisation.argtypes = [P, P, P, P, P, P, P, I, I, I, I, F, P, P, P, P]
    L.orc_interp3.argtypes = [P, P, P, P, P, I, I, I, I, I, I, I]
    L.orc_upsample.argtypes = [P, P, P, P, P, P, I, I, I, I, I, I]
    L.orc_warp_affine.argtypes = [P, P, P, P, P, P, I, I, I]
    L.orc_warp_image.argtypes = [P, P, P, P, P, I, I, I]
    L.orc_warp_affine_s.argtypes = [P, P, P, P, P, P, I, I, I]
    L.orc_consistent_mapping.argtypes = [P, P, P, P, P, P, I, I, I, I]
    L.orc_jacobian.argtypes = [P, P, P, I, I, I, I, P]; L.orc_jacobian.restype = F
    L.orc_register.argtypes = [P, P, I, I, I, P, I, P, P, P, F, P, P, P, P, P, I]
    L.orc_register.restype = I
    L.orc_lin_warp.argtypes = [P, P, P, I, I, I]
    L.orc_qrsolve.argtypes = [P, P, P, I, I]
    L.orc_affine_robust.argtypes = [P, P, P, I, I]
    L.orc_lin_smooth.argtypes = [P, I, I, I, I]
    L.orc_estimate_affine.argtypes = [P, P, P, P, P, P, I, I, I, I, F, I, I]
    L.orc_estimate_affine.restype = I
    L.orc_linear_register.argtypes = [P, P, I, I, I, I, P, P, P, I, P]


def _flat(a, dtype):
    a = np.asarray(a)
    if a.ndim > 1:
        a = a.ravel(order="F")
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def mind_step(q):
    return lib().orc_mind_step(int(q))


def mind_thresholds():
    t = np.zeros(5, np.float32)
    lib().orc_mind_thresholds(_p(t))
    return t


def descriptor(im, m, n, o, qs):
    im = _flat(im, np.float32)
    out = np.zeros(m * n * o, np.uint64)
    lib().orc_descriptor(_p(out), _p(im), m, n, o, qs)
    return out


def datacost_alpha1(g, q, alpha):
    return lib().orc_datacost_alpha1(g, float(q), float(alpha))


def data_cost(F_, M_, m, n, o, g, hw, q, alpha):
    F_ = _flat(F_, np.uint64); M_ = _flat(M_, np.uint64)
    len3 = (2 * hw + 1) ** 3
    sz1 = (m // g) * (n // g) * (o // g)
    out = np.zeros(sz1 * len3, np.float32)
    lib().orc_data_cost(_p(F_), _p(M_), _p(out), m, n, o, g, hw, int(q), float(alpha))
    return out


def image_stats(im):
    im = _flat(im, np.float32)
    mean = np.zeros(1, np.float32); sd = np.zeros(1, np.float32)
    lib().orc_image_stats(_p(im), im.size, _p(mean), _p(sd))
    return float(mean[0]), float(sd[0])


def edge_sad(im, m, n, o, g):
    im = _flat(im, np.float32)
    sz1 = (m // g) * (n // g) * (o // g)
    out = np.zeros(6 * sz1, np.float32)
    lib().orc_edge_sad(_p(im), _p(out), m, n, o, g)
    return out


def prims_graph(im, m, n, o, g):
    im = _flat(im, np.float32)
    sz1 = (m // g) * (n // g) * (o // g)
    ordered = np.zeros(sz1, np.int32); parents = np.zeros(sz1, np.int32); edgemst = np.zeros(sz1, np.float32)
    lib().orc_prims_graph(_p(im), m, n, o, g, _p(ordered), _p(parents), _p(edgemst))
    return ordered, parents, edgemst


def regularisation(cost, u0, v0, w0, m1, n1, o1, hw, q, ordered, parents, edgemst, want_allinds=False):
    """Returns (cost_after_upward_pass, u1, v1, w1[, allinds])."""
    cost = _flat(cost, np.float32).copy()
    u0 = _flat(u0, np.float32); v0 = _flat(v0, np.float32); w0 = _flat(w0, np.float32)
    ordered = _flat(ordered, np.int32); parents = _flat(parents, np.int32); edgemst = _flat(edgemst, np.float32)
    sz1 = m1 * n1 * o1
    u1 = np.zeros(sz1, np.float32); v1 = np.zeros(sz1, np.float32); w1 = np.zeros(sz1, np.float32)
    ai = np.zeros(cost.size, np.int16) if want_allinds else None
    lib().orc_regularisation(_p(cost), _p(u0), _p(v0), _p(w0), _p(u1), _p(v1), _p(w1), m1, n1, o1, hw,
                             float(q), _p(ordered), _p(parents), _p(edgemst), _p(ai) if ai is not None else None)
    if want_allinds:
        return cost, u1, v1, w1, ai
    return cost, u1, v1, w1


def message_dt(row, len_, offx, offy, offz):
    row = _flat(row, np.float32).copy()
    arg = np.zeros(row.size, np.int16)
    lib().orc_message_dt(_p(row), _p(arg), len_, float(offx), float(offy), float(offz))
    return row, arg


def upsample(u0, v0, w0, m, n, o, m2, n2, o2):
    u0 = _flat(u0, np.float32); v0 = _flat(v0, np.float32); w0 = _flat(w0, np.float32)
    s = m * n * o
    u = np.zeros(s, np.float32); v = np.zeros(s, np.float32); w = np.zeros(s, np.float32)
    lib().orc_upsample(_p(u), _p(v), _p(w), _p(u0), _p(v0), _p(w0), m, n, o, m2, n2, o2)
    return u, v, w


def interp3(inp, x1, y1, z1, m, n, o, m2, n2, o2, relative):
    inp = _flat(inp, np.float32)
    x1 = _flat(x1, np.float32); y1 = _flat(y1, np.float32); z1 = _flat(z1, np.float32)
    out = np.zeros(m * n * o, np.float32)
    lib().orc_interp3(_p(out), _p(inp), _p(x1), _p(y1), _p(z1), m, n, o, m2, n2, o2, int(relative))
    return out


def warp_affine(inp, X, u, v, w, m, n, o):
    inp = _flat(inp, np.float32); X = _flat(X, np.float32)
    u = _flat(u, np.float32); v = _flat(v, np.float32); w = _flat(w, np.float32)
    out = np.zeros(m * n * o, np.float32)
    lib().orc_warp_affine(_p(out), _p(inp), _p(X), _p(u), _p(v), _p(w), m, n, o)
    return out


def warp_image(inp, u, v, w, m, n, o):
    inp = _flat(inp, np.float32)
    u = _flat(u, np.float32); v = _flat(v, np.float32); w = _flat(w, np.float32)
    out = np.zeros(m * n * o, np.float32)
    lib().orc_warp_image(_p(out), _p(inp), _p(u), _p(v), _p(w), m, n, o)
    return out


def warp_affine_s(inp, X, u, v, w, m, n, o):
    inp = _flat(inp, np.int16); X = _flat(X, np.float32)
    u = _flat(u, np.float32); v = _flat(v, np.float32); w = _flat(w, np.float32)
    out = np.zeros(m * n * o, np.int16)
    lib().orc_warp_affine_s(_p(out), _p(inp), _p(X), _p(u), _p(v), _p(w), m, n, o)
    return out


def consistent_mapping(u, v, w, u2, v2, w2, m, n, o, g):
    f = [_flat(a, np.float32).copy() for a in (u, v, w, u2, v2, w2)]
    lib().orc_consistent_mapping(*[_p(a) for a in f], m, n, o, g)
    return f


def jacobian(u, v, w, m, n, o, g):
    u = _flat(u, np.float32); v = _flat(v, np.float32); w = _flat(w, np.float32)
    neg = np.zeros(1, np.float32)
    s = lib().orc_jacobian(_p(u), _p(v), _p(w), m, n, o, g, _p(neg))
    return float(s), float(neg[0])


def register(fixed, moving, m, n, o, X=None, G=(8, 7, 6, 5, 4), L=(8, 7, 6, 5, 4), Q=(5, 4, 3, 2, 1),
             alpha=1.6, want_full=False, verbose=False):
    """Full deeds registration on +1024-shifted images.  Returns flow (3*sz1,)
    and, with want_full, (flow, ux, vx, wx, warped)."""
    fixed = _flat(fixed, np.float32); moving = _flat(moving, np.float32)
    if X is None:
        X = np.eye(4, dtype=np.float32).ravel()
    X = _flat(X, np.float32)
    lv = len(G)
    Ga = np.asarray(G, np.int32); La = np.asarray(L, np.int32); Qa = np.asarray(Q, np.int32)
    g = G[-1]
    sz1 = (m // g) * (n // g) * (o // g)
    flow = np.zeros(3 * sz1, np.float32)
    s = m * n * o
    if want_full:
        ux = np.zeros(s, np.float32); vx = np.zeros(s, np.float32); wx = np.zeros(s, np.float32)
        warped = np.zeros(s, np.float32)
        lib().orc_register(_p(fixed), _p(moving), m, n, o, _p(X), lv, _p(Ga), _p(La), _p(Qa), float(alpha),
                           _p(flow), _p(ux), _p(vx), _p(wx), _p(warped), int(verbose))
        return flow, ux, vx, wx, warped
    lib().orc_register(_p(fixed), _p(moving), m, n, o, _p(X), lv, _p(Ga), _p(La), _p(Qa), float(alpha),
                       _p(flow), None, None, None, None, int(verbose))
    return flow


# ---- linearBCV (src/linearBCV.cpp, src/affineLTS1.h, src/QRsolve.h)

LINEAR_DEFAULTS = dict(G=(7, 6, 5, 4), L=(5, 4, 3, 2), Q=(4, 3, 2, 1))  # src/linearBCV.cpp:86-89


def lin_warp(inp, X, m, n, o):
    """warpAffine of src/affineLTS1.h:39-68 (affine only, zero outside)."""
    inp = _flat(inp, np.float32); X = _flat(X, np.float32)
    out = np.zeros(m * n * o, np.float32)
    lib().orc_lin_warp(_p(out), _p(inp), _p(X), m, n, o)
    return out


def qrsolve(A, b, length, nrhs):
    A = _flat(A, np.float32); b = _flat(b, np.float32)
    X = np.zeros(4 * nrhs, np.float32)
    lib().orc_qrsolve(_p(X), _p(A), _p(b), int(length), int(nrhs))
    return X


def affine_robust(p1, p2, length, rigid=False):
    p1 = _flat(p1, np.float32); p2 = _flat(p2, np.float32)
    RT = np.zeros(16, np.float32)
    lib().orc_affine_robust(_p(RT), _p(p1), _p(p2), int(length), int(bool(rigid)))
    return RT


def lin_smooth(cost, m1, n1, o1, len3):
    cost = _flat(cost, np.float32).copy()
    lib().orc_lin_smooth(_p(cost), m1, n1, o1, len3)
    return cost


def estimate_affine(Xprev, fixed, moving, cost, cost2, m, n, o, g, q, hw, rigid=False):
    """estimateAffine2: returns (X, smoothed cost, smoothed cost2, points used)."""
    Xprev = _flat(Xprev, np.float32); fixed = _flat(fixed, np.float32); moving = _flat(moving, np.float32)
    c1 = _flat(cost, np.float32).copy(); c2 = _flat(cost2, np.float32).copy()
    X = np.zeros(16, np.float32)
    used = lib().orc_estimate_affine(_p(X), _p(Xprev), _p(fixed), _p(moving), _p(c1), _p(c2), m, n, o, g, float(q),
                                     hw, int(bool(rigid)))
    return X, c1, c2, used


def linear_register(fixed, moving, m, n, o, G=LINEAR_DEFAULTS["G"], L=LINEAR_DEFAULTS["L"], Q=LINEAR_DEFAULTS["Q"],
                    rigid=False):
    """The linearBCV level loop on +1024-shifted images: the 16-float matrix."""
    fixed = _flat(fixed, np.float32); moving = _flat(moving, np.float32)
    Ga = np.asarray(G, np.int32); La = np.asarray(L, np.int32); Qa = np.asarray(Q, np.int32)
    X = np.zeros(16, np.float32)
    lib().orc_linear_register(_p(fixed), _p(moving), m, n, o, len(G), _p(Ga), _p(La), _p(Qa), int(bool(rigid)),
                              _p(X))
    return X
