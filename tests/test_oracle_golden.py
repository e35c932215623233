"""Pin the oracle (oracle/deeds_oracle.cpp) to the reference's own outputs.

The golden vectors in tests/golden/ were produced by the unmodified reference
(tests/golden/make_golden.py).  Every stage must match bit for bit.
"""
import hashlib

import numpy as np
import pytest

import pyoracle as orc


def test_mind_thresholds_are_glibc_logf():
    t = orc.mind_thresholds()
    expect = -np.log((np.arange(5, dtype=np.float32) + np.float32(1.5)) / np.float32(6)).astype(np.float32)
    # float32 log, possibly 1 ulp apart from numpy's; the oracle value is what
    # the codes below depend on, so only sanity-check here
    assert np.allclose(t, expect, rtol=1e-6)
    assert [orc.mind_step(q) for q in (5, 4, 3, 2, 1)] == [3, 3, 2, 2, 1]


@pytest.mark.parametrize("qs", [1, 2, 3])
def test_descriptor_bit_exact(golden, qs):
    g = golden("mind")
    m, n, o = (int(x) for x in g["dims"])
    assert np.array_equal(orc.descriptor(g["fixed"], m, n, o, qs), g[f"codes_q{qs}"])
    assert np.array_equal(orc.descriptor(g["moving"], m, n, o, qs), g[f"mcodes_q{qs}"])


def test_data_cost_bit_exact(golden):
    g = golden("datacost")
    m, n, o = (int(x) for x in g["dims"])
    for (gs, hw, q) in g["cases"]:
        cost = orc.data_cost(g["F"], g["M"], m, n, o, int(gs), int(hw), int(q), float(g["alpha"]))
        ref = g[f"cost_{gs}_{hw}_{q}"]
        assert cost.shape == ref.shape
        assert np.array_equal(cost.view(np.uint32), ref.view(np.uint32)), (gs, hw, q)


@pytest.mark.parametrize("gs", [4, 5, 6, 8])
def test_prims_graph_identical(golden, gs):
    g = golden("prims")
    m, n, o = (int(x) for x in g["dims"])
    ordered, parents, edgemst = orc.prims_graph(g["image"], m, n, o, gs)
    assert np.array_equal(ordered, g[f"ordered_{gs}"])
    assert np.array_equal(parents, g[f"parents_{gs}"])
    assert np.array_equal(edgemst.view(np.uint32), g[f"edgemst_{gs}"].view(np.uint32))


@pytest.mark.parametrize("key", ["4_2_1", "5_3_2", "8_2_3"])
def test_regularisation_bit_exact(golden, key):
    r = golden("reg")
    p = golden("prims")
    m, n, o = (int(x) for x in r["dims"])
    gs, hw, q = (int(x) for x in key.split("_"))
    m1, n1, o1 = m // gs, n // gs, o // gs
    cost = r[f"counts_{key}"].astype(np.float32) * r[f"alpha1_{key}"]
    post, u1, v1, w1 = orc.regularisation(cost, r[f"u0_{key}"], r[f"v0_{key}"], r[f"w0_{key}"], m1, n1, o1, hw, q,
                                          p[f"ordered_{gs}"], p[f"parents_{gs}"], p[f"edgemst_{gs}"])
    assert hashlib.sha256(post.tobytes()).digest() == r[f"post_sha256_{key}"].tobytes()
    assert np.array_equal(post.reshape(m1 * n1 * o1, -1)[p[f"ordered_{gs}"][0]], r[f"post_root_{key}"])
    for name, arr in (("u1", u1), ("v1", v1), ("w1", w1)):
        assert np.array_equal(arr.view(np.uint32), r[f"{name}_{key}"].view(np.uint32)), name


def test_transforms_bit_exact(golden):
    t = golden("transforms")
    m, n, o = (int(x) for x in t["dims"])
    m2, n2, o2 = (int(x) for x in t["grid_dims"])
    up = orc.upsample(*t["grid"], m, n, o, m2, n2, o2)
    for i in range(3):
        assert np.array_equal(up[i].view(np.uint32), t["up"][i].view(np.uint32))
    f = t["field"]
    wa = orc.warp_affine(t["image"], t["X"], f[0], f[1], f[2], m, n, o)
    assert np.array_equal(wa.view(np.uint32), t["warp_affine"].view(np.uint32))
    wi = orc.warp_image(t["image"], f[0], f[1], f[2], m, n, o)
    assert np.array_equal(wi.view(np.uint32), t["warp_image"].view(np.uint32))
    ws = orc.warp_affine_s(t["seg"], t["X"], f[0], f[1], f[2], m, n, o)
    assert np.array_equal(ws, t["warp_seg"])
    cm, cn, co, cg = (int(x) for x in t["cons_dims"])
    out = orc.consistent_mapping(*t["cons_in"], cm, cn, co, cg)
    for i in range(6):
        assert np.array_equal(out[i].view(np.uint32), t["cons_out"][i].view(np.uint32)), i
    js, _ = orc.jacobian(*t["cons_in"][:3], cm, cn, co, cg)
    assert np.float32(js) == t["jac_std"]


def test_register_end_to_end_matches_reference_binary(golden):
    e = golden("e2e")
    m, n, o = (int(x) for x in e["dims"])
    fixed = e["fixed"].astype(np.float32).ravel(order="F") + np.float32(1024)
    moving = e["moving"].astype(np.float32).ravel(order="F") + np.float32(1024)
    flow, ux, vx, wx, warped = orc.register(fixed, moving, m, n, o, G=tuple(e["G"]), L=tuple(e["L"]),
                                            Q=tuple(e["Q"]), want_full=True)
    assert np.array_equal(flow.view(np.uint32), e["flow"].view(np.uint32))
    assert np.array_equal((warped - np.float32(1024)).view(np.uint32), e["warped"].view(np.uint32))
    seg = orc.warp_affine_s(e["moving_labels"].astype(np.int16), np.eye(4, dtype=np.float32).ravel(), ux, vx, wx, m, n, o)
    assert np.array_equal(seg, e["warped_seg"])


def _apply_inputs(e):
    """The applyBCV / applyBCVfloat inputs of apply.npz: the e2e flow, the float
    image 0.37 x moving + 11.125 and the moving labels."""
    m, n, o = (int(x) for x in e["dims"])
    img = (e["moving"].astype(np.float32) * np.float32(0.37) + np.float32(11.125)).astype(np.float32)
    return (m, n, o), e["flow"], img.ravel(order="F"), e["moving_labels"].astype(np.int16).ravel(order="F")


def test_apply_float_and_affine_match_reference_binaries(golden):
    """applyBCVfloat (trilinear, with and without an affine matrix) and applyBCV with
    a matrix (src/applyBCV.cpp:161-198): the grid step inferred from the .dat size,
    upsampling, then the warp; the reference binaries wrote apply.npz."""
    e, a = golden("e2e"), golden("apply")
    (m, n, o), flow, img, lab = _apply_inputs(e)
    sz1 = flow.size // 3
    g = int(round((m * n * o / sz1) ** (1.0 / 3.0)))
    ux, vx, wx = orc.upsample(flow[:sz1], flow[sz1:2 * sz1], flow[2 * sz1:], m, n, o, m // g, n // g, o // g)
    eye = np.eye(4, dtype=np.float32).ravel()
    w = orc.warp_affine(img, eye, ux, vx, wx, m, n, o)
    assert np.array_equal(w.view(np.uint32), a["warped_float"].view(np.uint32))
    w = orc.warp_affine(img, a["X"], ux, vx, wx, m, n, o)
    assert np.array_equal(w.view(np.uint32), a["warped_float_affine"].view(np.uint32))
    s = orc.warp_affine_s(lab, a["X"], ux, vx, wx, m, n, o)
    assert np.array_equal(s, a["warped_seg_affine"])
