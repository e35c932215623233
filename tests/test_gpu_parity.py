"""GPU parity: every stage of the CUDA path against the reference's golden
vectors and the oracle, through the C ABI (deedsbcv_gb300.api -> libdeeds_gpu.so).

Tolerances (the contract for this path):
  * MIND-SSC codes, Hamming cost volumes, MST, warps, upsampling, consistent
    mapping: bit-exact;
  * BP messages (post-sweep cost rows): within 1e-4 relative;
  * argmin displacements: >= 99.9 % of control points identical;
  * warped-label Dice: within 0.1 points (0.001) of the oracle's.
"""
import hashlib
import os

import numpy as np
import pytest

import pyoracle as orc

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BP_RTOL = 1e-4
ARGMIN_AGREE = 0.999
DICE_TOL = 0.001


@pytest.fixture(scope="module")
def api():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from deedsbcv_gb300 import api as _api
    _api.context(0)
    return _api


def cu(a, dtype=None):
    a = np.asarray(a)
    if a.ndim > 1:
        a = a.ravel(order="F")
    if a.dtype == np.uint64:
        a = a.view(np.int64)
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def host(t, dtype=None):
    a = t.detach().cpu().numpy()
    if dtype is not None:
        a = a.view(dtype)
    return a


def same_bits(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


@pytest.mark.parametrize("qs", [1, 2, 3])
def test_mind_golden(api, golden, qs):
    g = golden("mind")
    m, n, o = (int(x) for x in g["dims"])
    for key, img in (("codes", g["fixed"]), ("mcodes", g["moving"])):
        codes = host(api.descriptor(cu(img), m, n, o, qs), np.uint64)
        assert same_bits(codes, g[f"{key}_q{qs}"]), (key, qs, int(np.count_nonzero(codes != g[f"{key}_q{qs}"])))


@pytest.mark.parametrize("shape,top", [((100, 37, 29), 3), ((64, 33, 17), 1), ((20, 70, 11), 7), ((161, 12, 9), 2)])
def test_mind_integer_images_vs_oracle(api, shape, top):
    """Small-integer images: the distances are integers, so many SSC quotients are
    equal or near-equal across voxels and some fall close to a threshold (where the
    quantiser divides exactly); line lengths that leave partial and interior
    i-chunks."""
    rng = np.random.default_rng(sum(shape) + top)
    im = rng.integers(0, top + 1, int(np.prod(shape))).astype(np.float32)
    for qs in (1, 2, 3):
        gpu = host(api.descriptor(cu(im), *shape, qs), np.uint64)
        ref = orc.descriptor(im, *shape, qs)
        assert same_bits(gpu, ref), (shape, qs, int(np.count_nonzero(gpu != ref)))


def test_mind_phantom_vs_oracle(api):
    from deedsbcv_gb300 import phantom
    shape = (96, 80, 128)
    pair = phantom.make_pair(shape, seed=11, max_disp=6.0)
    im = pair["moving"].ravel(order="F") + np.float32(1024)
    for qs in (1, 2, 3):
        gpu = host(api.descriptor(cu(im), *shape, qs), np.uint64)
        ref = orc.descriptor(im, *shape, qs)
        assert same_bits(gpu, ref), (qs, int(np.count_nonzero(gpu != ref)))


def test_data_cost_golden(api, golden):
    g = golden("datacost")
    m, n, o = (int(x) for x in g["dims"])
    F, M = cu(g["F"]), cu(g["M"])
    for (gs, hw, q) in g["cases"]:
        cost = host(api.dataCostCL(F, M, m, n, o, int(gs), int(hw), int(q), float(g["alpha"])))
        assert same_bits(cost, g[f"cost_{gs}_{hw}_{q}"]), (gs, hw, q)


@pytest.mark.parametrize("gs,hw,q", [(8, 8, 5), (7, 7, 4), (6, 6, 3), (5, 5, 2), (4, 4, 1), (4, 3, 2),
                                     (7, 5, 4), (6, 4, 3), (5, 3, 2), (4, 2, 1)])
def test_data_cost_phantom_vs_oracle(api, gs, hw, q):
    # deedsBCV's and linearBCV's default level shapes (compile-time label widths) and one runtime-width shape
    from deedsbcv_gb300 import phantom
    shape = (64, 48, 72)
    pair = phantom.make_pair(shape, seed=12, max_disp=6.0)
    qs = orc.mind_step(q)
    F = orc.descriptor(pair["fixed"].ravel(order="F") + np.float32(1024), *shape, qs)
    M = orc.descriptor(pair["moving"].ravel(order="F") + np.float32(1024), *shape, qs)
    gpu = host(api.dataCostCL(cu(F), cu(M), *shape, gs, hw, q, 1.6))
    ref = orc.data_cost(F, M, *shape, gs, hw, q, 1.6)
    assert same_bits(gpu, ref)


@pytest.mark.parametrize("gs", [4, 5, 6, 8])
def test_mst_golden(api, golden, gs):
    p = golden("prims")
    m, n, o = (int(x) for x in p["dims"])
    im = cu(p["image"])
    sad = host(api.mst_edges(im, m, n, o, gs))
    assert same_bits(sad, orc.edge_sad(p["image"], m, n, o, gs))
    ordered, parents, edgemst = api.primsGraph(im, m, n, o, gs)
    assert np.array_equal(ordered, p[f"ordered_{gs}"])
    assert np.array_equal(parents, p[f"parents_{gs}"])
    assert same_bits(edgemst, p[f"edgemst_{gs}"])


@pytest.mark.parametrize("key", ["4_2_1", "5_3_2", "8_2_3"])
def test_tree_bp_golden(api, golden, key):
    r = golden("reg")
    p = golden("prims")
    m, n, o = (int(x) for x in r["dims"])
    gs, hw, q = (int(x) for x in key.split("_"))
    m1, n1, o1 = m // gs, n // gs, o // gs
    cost = r[f"counts_{key}"].astype(np.float32) * r[f"alpha1_{key}"]
    dcost = cu(cost)
    u1, v1, w1, ai = api.regularisationCL(dcost, cu(r[f"u0_{key}"]), cu(r[f"v0_{key}"]), cu(r[f"w0_{key}"]), m1, n1, o1,
                                          hw, q, p[f"ordered_{gs}"], p[f"parents_{gs}"], p[f"edgemst_{gs}"],
                                          want_allinds=True)
    post = host(dcost)
    ref_post, _, _, _, ref_ai = orc.regularisation(cost, r[f"u0_{key}"], r[f"v0_{key}"], r[f"w0_{key}"], m1, n1, o1, hw,
                                                   q, p[f"ordered_{gs}"], p[f"parents_{gs}"], p[f"edgemst_{gs}"],
                                                   want_allinds=True)
    # the oracle is pinned to the reference's post-sweep state by digest
    assert hashlib.sha256(ref_post.tobytes()).digest() == r[f"post_sha256_{key}"].tobytes()
    np.testing.assert_allclose(post, ref_post, rtol=BP_RTOL, atol=BP_RTOL * np.abs(ref_post).max())
    for name, arr in (("u1", u1), ("v1", v1), ("w1", w1)):
        agree = np.mean(host(arr) == r[f"{name}_{key}"])
        assert agree >= ARGMIN_AGREE, (name, agree)
    # non-root argmin tables are the reference's messageDT outputs
    root = p[f"ordered_{gs}"][0]
    len3 = (2 * hw + 1) ** 3
    mask = np.ones(m1 * n1 * o1, bool)
    mask[root] = False
    got = host(ai).reshape(-1, len3)[mask]
    exp = ref_ai.reshape(-1, len3)[mask]
    assert np.mean(got == exp) >= ARGMIN_AGREE
    # without tables the downward pass evaluates each node's one entry from its stored
    # row: the same fields bit for bit
    lu, lv, lw = api.regularisationCL(cu(cost), cu(r[f"u0_{key}"]), cu(r[f"v0_{key}"]), cu(r[f"w0_{key}"]), m1, n1, o1,
                                      hw, q, p[f"ordered_{gs}"], p[f"parents_{gs}"], p[f"edgemst_{gs}"])
    for a, b in ((lu, u1), (lv, v1), (lw, w1)):
        assert same_bits(host(a), host(b))


def test_tree_bp_bit_exact_on_phantom(api):
    """Same inputs -> identical messages and fields (the arithmetic is the reference's)."""
    from deedsbcv_gb300 import phantom
    shape = (64, 48, 72)
    gs, hw, q = 6, 6, 3
    pair = phantom.make_pair(shape, seed=13, max_disp=6.0)
    fixed = pair["fixed"].ravel(order="F") + np.float32(1024)
    qs = orc.mind_step(q)
    F = orc.descriptor(fixed, *shape, qs)
    M = orc.descriptor(pair["moving"].ravel(order="F") + np.float32(1024), *shape, qs)
    cost = orc.data_cost(F, M, *shape, gs, hw, q, 1.6)
    ordered, parents, edgemst = orc.prims_graph(fixed, *shape, gs)
    m1, n1, o1 = (s // gs for s in shape)
    rng = np.random.default_rng(5)
    u0, v0, w0 = (rng.uniform(-6, 6, m1 * n1 * o1).astype(np.float32) for _ in range(3))
    dcost = cu(cost)
    u1, v1, w1 = api.regularisationCL(dcost, cu(u0), cu(v0), cu(w0), m1, n1, o1, hw, q, ordered, parents, edgemst)
    ref_post, ru, rv, rw = orc.regularisation(cost, u0, v0, w0, m1, n1, o1, hw, q, ordered, parents, edgemst)
    assert same_bits(host(dcost), ref_post)
    assert same_bits(host(u1), ru) and same_bits(host(v1), rv) and same_bits(host(w1), rw)


def test_transforms_golden(api, golden):
    t = golden("transforms")
    m, n, o = (int(x) for x in t["dims"])
    m2, n2, o2 = (int(x) for x in t["grid_dims"])
    up = api.upsampleDeformationsCL(cu(t["grid"][0]), cu(t["grid"][1]), cu(t["grid"][2]), m2, n2, o2, m, n, o)
    for i in range(3):
        assert same_bits(host(up[i]), t["up"][i]), i
    f = [cu(x) for x in t["field"]]
    assert same_bits(host(api.warpAffine(cu(t["image"]), t["X"], *f, m, n, o)), t["warp_affine"])
    assert same_bits(host(api.warpImageCL(cu(t["image"]), *f, m, n, o)), t["warp_image"])
    assert np.array_equal(host(api.warpAffineS(cu(t["seg"]), t["X"], *f, m, n, o)), t["warp_seg"])
    cm, cn, co, cg = (int(x) for x in t["cons_dims"])
    six = [cu(x) for x in t["cons_in"]]
    api.consistentMappingCL(*six, cm, cn, co, cg)
    for i in range(6):
        assert same_bits(host(six[i]), t["cons_out"][i]), i
    js, _ = api.jacobian(*[cu(x) for x in t["cons_in"][:3]], cm, cn, co, cg)
    assert abs(js - float(t["jac_std"])) <= 1e-4 * max(1.0, abs(float(t["jac_std"])))


def test_register_golden_end_to_end(api, golden):
    """Whole 3-level registration against the reference binary's own outputs."""
    from deedsbcv_gb300 import phantom
    e = golden("e2e")
    m, n, o = (int(x) for x in e["dims"])
    params = api.default_params(grid=e["G"], radius=e["L"], quant=e["Q"])
    flow, warped = api.register(e["fixed"].astype(np.float32), e["moving"].astype(np.float32), dims=(m, n, o),
                                params=params)
    agree = np.mean(flow == e["flow"])
    assert agree >= ARGMIN_AGREE, agree
    seg = api.warp_segmentation(e["moving_labels"].astype(np.int16))
    d_gpu = phantom.dice(e["fixed_labels"].ravel(order="F"), seg)
    d_ref = phantom.dice(e["fixed_labels"].ravel(order="F"), e["warped_seg"])
    assert abs(d_gpu - d_ref) <= DICE_TOL, (d_gpu, d_ref)
    # with identical fields the outputs are bit-identical
    if agree == 1.0:
        assert same_bits(flow, e["flow"])
        assert same_bits(warped, e["warped"])
        assert np.array_equal(seg, e["warped_seg"])


def test_register_config1_vs_oracle(api):
    """96x80x128 CT-like pair, default 5 levels: GPU against the oracle."""
    from deedsbcv_gb300 import phantom
    shape = (96, 80, 128)
    pair = phantom.make_pair(shape, seed=21, max_disp=6.0)
    flow, warped = api.register(pair["fixed"], pair["moving"])
    seg = api.warp_segmentation(pair["moving_labels"].astype(np.int16))
    f = pair["fixed"].ravel(order="F") + np.float32(1024)
    mv = pair["moving"].ravel(order="F") + np.float32(1024)
    rflow, ux, vx, wx, rwarped = orc.register(f, mv, *shape, want_full=True)
    agree = np.mean(flow == rflow)
    assert agree >= ARGMIN_AGREE, agree
    rseg = orc.warp_affine_s(pair["moving_labels"].astype(np.int16), np.eye(4, dtype=np.float32).ravel(), ux, vx, wx,
                             *shape)
    lab = pair["fixed_labels"].ravel(order="F")
    d_gpu, d_ref = phantom.dice(lab, seg), phantom.dice(lab, rseg)
    assert abs(d_gpu - d_ref) <= DICE_TOL, (d_gpu, d_ref)
    assert d_gpu > phantom.dice(lab, pair["moving_labels"].ravel(order="F"))  # registration helped


def test_apply_flow_matches_register(api, golden):
    """applyBCV path: upsample + nearest warp of the .dat flow equals the -S output."""
    e = golden("e2e")
    m, n, o = (int(x) for x in e["dims"])
    seg = api.apply_flow(e["flow"], e["moving_labels"].astype(np.int16), dims=(m, n, o))
    assert np.array_equal(seg, e["warped_seg"])
    img = api.apply_flow(e["flow"], e["moving"].astype(np.float32) + np.float32(0), dims=(m, n, o))
    assert img.dtype == np.float32 and img.shape == (m * n * o,)


def _apply_inputs(e):
    m, n, o = (int(x) for x in e["dims"])
    img = (e["moving"].astype(np.float32) * np.float32(0.37) + np.float32(11.125)).astype(np.float32)
    return (m, n, o), img, e["moving_labels"].astype(np.int16)


def test_apply_float_matches_reference_applybcvfloat(api, golden):
    """applyBCVfloat (src/applyBCVfloat.cpp: upsampling + trilinear warpAffine of a
    float image through the .dat) and applyBCV with an affine matrix, against the
    reference binaries' outputs on the e2e flow: bit-exact."""
    e, a = golden("e2e"), golden("apply")
    dims, img, lab = _apply_inputs(e)
    got = api.apply_flow(e["flow"], img, dims=dims)
    assert same_bits(got, a["warped_float"])
    got = api.apply_flow(e["flow"], img, dims=dims, X=a["X"])
    assert same_bits(got, a["warped_float_affine"])
    seg = api.apply_flow(e["flow"], lab, dims=dims, X=a["X"])
    assert np.array_equal(seg, a["warped_seg_affine"])


def test_cli_applybcvfloat_matches_reference(api, golden, tmp_path):
    """The applyBCVfloat / applyBCV executables on NIfTI files, with -A matrix text in
    the reference's layout (line i: X[i] X[i+4] X[i+8] X[i+12])."""
    import subprocess
    from deedsbcv_gb300 import build, nifti
    e, a = golden("e2e"), golden("apply")
    dims, img, lab = _apply_inputs(e)
    stem = str(tmp_path / "out")
    nifti.write_dat(stem + "_displacements.dat", e["flow"])
    ipath, spath = str(tmp_path / "img.nii.gz"), str(tmp_path / "seg.nii.gz")
    nifti.write(ipath, img.ravel(order="F").reshape(dims, order="F"))
    nifti.write(spath, lab)
    mat = str(tmp_path / "matrix.txt")
    with open(mat, "w") as f:
        for i in range(4):
            f.write("  ".join(f"{float(a['X'][i + 4 * k]):.6f}" for k in range(4)) + "\n")
    for exe, src, extra, key in (("applyBCVfloat", ipath, [], "warped_float"),
                                 ("applyBCVfloat", ipath, ["-A", mat], "warped_float_affine"),
                                 ("applyBCV", spath, ["-A", mat], "warped_seg_affine")):
        out = str(tmp_path / (key + ".nii.gz"))
        r = subprocess.run([os.path.join(build.OUT, exe), "-M", src, "-O", stem, "-D", out] + extra,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        vol, _ = nifti.read(out)
        assert same_bits(vol.ravel(order="F").astype(a[key].dtype), a[key]), key


def test_register_device_equals_host(api):
    from deedsbcv_gb300 import phantom
    shape = (48, 40, 56)
    pair = phantom.make_pair(shape, seed=31, max_disp=4.0)
    params = api.default_params(grid=[6, 5, 4], radius=[5, 4, 3], quant=[3, 2, 1])
    flow_h, _ = api.register(pair["fixed"], pair["moving"], params=params)
    flow_d = api.register_device(cu(pair["fixed"]), cu(pair["moving"]), *shape, params=params)
    torch.cuda.synchronize()
    assert same_bits(host(flow_d), flow_h)


def test_register_full_size_properties(api):
    """192x160x256 (7.9 M voxels), default parameters: determinism, output size,
    and that the warped labels overlap the fixed labels better than before."""
    from deedsbcv_gb300 import phantom
    shape = (192, 160, 256)
    pair = phantom.make_pair(shape, seed=2, n_organs=13, max_disp=10.0)
    flow1, _ = api.register(pair["fixed"], pair["moving"], want_warped=False)
    seg = api.warp_segmentation(pair["moving_labels"].astype(np.int16))
    flow2, _ = api.register(pair["fixed"], pair["moving"], want_warped=False)
    assert flow1.size == 3 * (192 // 4) * (160 // 4) * (256 // 4)
    assert same_bits(flow1, flow2)
    lab = pair["fixed_labels"].ravel(order="F")
    assert phantom.dice(lab, seg) > phantom.dice(lab, pair["moving_labels"].ravel(order="F")) + 0.05


def test_invalid_arguments_raise(api):
    from deedsbcv_gb300._lib import DeedsError
    params = api.default_params()
    with pytest.raises(DeedsError):  # grid spacing 8 does not fit a 4^3 volume
        api.register(np.zeros((4, 4, 4), np.float32), np.zeros((4, 4, 4), np.float32), params=params)
    bad = api.default_params(grid=[4], radius=[11], quant=[1])  # label radius above the supported 10
    with pytest.raises(DeedsError):
        api.register(np.zeros((16, 16, 16), np.float32), np.zeros((16, 16, 16), np.float32), params=bad)
    with pytest.raises(DeedsError):
        api.apply_flow(np.zeros(7, np.float32), np.zeros((8, 8, 8), np.int16))


def test_register_batch_matches_single_calls(api):
    """Uneven pair sizes through deeds_register_batch give the per-pair results."""
    from deedsbcv_gb300 import phantom
    shapes = [(48, 40, 56), (56, 48, 40), (40, 56, 48), (64, 40, 48), (48, 48, 48)]
    pairs = []
    for i, sh in enumerate(shapes):
        p = phantom.make_pair(sh, seed=50 + i, n_organs=5, max_disp=4.0)
        pairs.append((p["fixed"], p["moving"]))
    params = api.default_params(grid=[6, 5, 4], radius=[5, 4, 3], quant=[3, 2, 1])
    single = [api.register(f, m, params=params, want_warped=False)[0] for f, m in pairs]
    for lanes in (1, 3):
        batched = api.register_batch(pairs, params=params, lanes=lanes)
        for a, (b, _) in zip(single, batched):
            assert same_bits(a, b)


def test_register_batch_reports_bad_pair(api):
    from deedsbcv_gb300._lib import DeedsError
    rng = np.random.default_rng(3)
    ok = rng.normal(0, 100, (32, 32, 32)).astype(np.float32)
    tiny = rng.normal(0, 100, (2, 2, 2)).astype(np.float32)  # too small for a MIND radius of 1
    with pytest.raises(DeedsError, match="pair 1"):
        api.register_batch([(ok, ok), (tiny, tiny)], params=api.default_params(grid=[2], radius=[2], quant=[1]))


def test_constant_images_follow_reference_nan_semantics(api):
    """A constant image has zero intensity spread, so the MST edge weights are
    -exp(-0/0) = NaN in the reference as well; the registration must still run
    and pick the same labels as the oracle (index 0 where every cost is NaN)."""
    shape = (32, 24, 40)
    flat = np.zeros(shape, np.float32)
    params = api.default_params(grid=[6, 4], radius=[3, 2], quant=[2, 1])
    flow, _ = api.register(flat, flat, params=params, want_warped=False)
    f = flat.ravel(order="F") + np.float32(1024)
    ref = orc.register(f, f, *shape, G=(6, 4), L=(3, 2), Q=(2, 1))
    assert same_bits(flow, ref)


def test_cli_deedsbcv_and_applybcv_match_reference_outputs(api, golden, tmp_path):
    """The drop-in boundary end to end: the deedsBCV binary on NIfTI files with the
    reference's flags writes the reference's displacement file and deformed images;
    applyBCV re-applies the .dat to the labels."""
    import subprocess
    from deedsbcv_gb300 import build, nifti, phantom
    e = golden("e2e")
    f, mv = tmp_path / "f.nii.gz", tmp_path / "m.nii.gz"
    seg = tmp_path / "seg.nii.gz"
    nifti.write(str(f), e["fixed"])
    nifti.write(str(mv), e["moving"])
    nifti.write(str(seg), e["moving_labels"].astype(np.int16))
    stem = str(tmp_path / "out")
    exe = os.path.join(build.OUT, "deedsBCV")
    r = subprocess.run([exe, "-F", str(f), "-M", str(mv), "-O", stem, "-G", "6x5x4", "-L", "5x4x3", "-Q", "3x2x1",
                        "-S", str(seg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    flow = nifti.read_dat(stem + "_displacements.dat")
    assert flow.size == e["flow"].size
    agree = np.mean(flow == e["flow"])
    assert agree >= ARGMIN_AGREE, agree
    wseg, _ = nifti.read(stem + "_deformed_seg.nii.gz")
    lab = e["fixed_labels"].ravel(order="F")
    assert abs(phantom.dice(lab, wseg.ravel(order="F")) - phantom.dice(lab, e["warped_seg"])) <= DICE_TOL
    if agree == 1.0:
        warped, _ = nifti.read(stem + "_deformed.nii.gz")
        assert np.array_equal(warped.ravel(order="F").astype(np.float32), e["warped"])
        assert np.array_equal(wseg.ravel(order="F"), e["warped_seg"])
    # applyBCV: the same labels through the written displacement file
    out = str(tmp_path / "applied.nii.gz")
    r = subprocess.run([os.path.join(build.OUT, "applyBCV"), "-M", str(seg), "-O", stem, "-D", out],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    applied, _ = nifti.read(out)
    assert np.array_equal(applied.ravel(order="F"), wseg.ravel(order="F"))


def test_register_cross_contrast_vs_oracle(api):
    """The cross-contrast workload (per-organ intensity remap, inverted background,
    bias field, Rician noise) at 64x64x72: GPU against the oracle."""
    from deedsbcv_gb300 import phantom
    shape = (64, 64, 72)
    pair = phantom.make_pair(shape, seed=31, max_disp=5.0, contrast="cross")
    flow, _ = api.register(pair["fixed"], pair["moving"])
    f = pair["fixed"].ravel(order="F") + np.float32(1024)
    mv = pair["moving"].ravel(order="F") + np.float32(1024)
    rflow, ux, vx, wx, rwarped = orc.register(f, mv, *shape, want_full=True)
    agree = np.mean(flow == rflow)
    assert agree >= ARGMIN_AGREE, agree
