"""Generate the golden vectors that pin the oracle to the reference.

Runs the UNMODIFIED reference, compiled by ``make -C oracle ref`` into
oracle/_ref/ (the stage harness oracle/_ref/ref_stages around the reference's
own functions, and the reference deedsBCV / applyBCV binaries), on small seeded
inputs and stores inputs and outputs under tests/golden/*.npz.  It needs the
reference sources, so it runs only where they are present; the fixtures it
writes are committed and travel with the tests.

    python tests/golden/make_golden.py                 # every fixture
    python tests/golden/make_golden.py --linear-only   # linear.npz alone
    python tests/golden/make_golden.py --apply-only    # apply.npz alone
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from deedsbcv_gb300 import nifti, phantom  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")


def run(*args, capture=False):
    out = subprocess.run([str(a) for a in args], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"{args[0]} failed: {out.stdout}\n{out.stderr}")
    return out.stdout


def stage(name, *args):
    return run(os.path.join(REF, "ref_stages"), name, *args)


def tofile(d, name, arr):
    p = os.path.join(d, name)
    np.ascontiguousarray(arr).tofile(p)
    return p


def _as_counts(cost, g, q, alpha=1.6):
    """Integer Hamming sums behind a cost volume (cost = float(count) * alpha1)."""
    skip = 2 if g > 4 else 1
    maxsamp = np.float32(np.ceil(g / skip) * np.ceil(g / skip) * g)
    alphai = np.float32(np.float32(g) / (np.float32(alpha) * np.float32(q)))
    alpha1 = np.float32(0.5 * np.float64(alphai) / np.float64(maxsamp))
    counts = np.round(cost / alpha1).astype(np.uint16)
    assert np.array_equal(counts.astype(np.float32) * alpha1, cost), "cost volume is not count*alpha1"
    return counts, alpha1


def shifted_phantom(shape, seed, **kw):
    pair = phantom.make_pair(shape, seed=seed, **kw)
    f = pair["fixed"].ravel(order="F") + np.float32(1024)
    mv = pair["moving"].ravel(order="F") + np.float32(1024)
    return pair, f.astype(np.float32), mv.astype(np.float32)


def lin(name, *args):
    return run(os.path.join(REF, "ref_linear"), name, *args)


def make_linear(d, rng):
    """linearBCV (src/linearBCV.cpp, src/affineLTS1.h, src/QRsolve.h): each stage of
    the reference through oracle/_ref/ref_linear, and the reference binary end to
    end (affine and rigid) on a phantom pair with a seeded affine misalignment."""
    lg = {}
    # affine-only warp (zero outside) and the QR inverse of a near-identity matrix
    m, n, o = 24, 20, 28
    _, fim, _ = shifted_phantom((m, n, o), seed=1, n_organs=6, max_disp=3.0)
    Xw = np.array([0.97, 0.04, -0.03, 1.6, -0.02, 1.03, 0.05, -2.2, 0.03, -0.04, 0.99, 0.9,
                   0.0, 0.0, 0.0, 1.0], np.float32)
    lin("warp", tofile(d, "im", fim), tofile(d, "X", Xw), m, n, o, os.path.join(d, "w"))
    lg["warp_dims"] = np.array([m, n, o]); lg["warp_image"] = fim; lg["warp_X"] = Xw
    lg["warp_out"] = np.fromfile(os.path.join(d, "w"), np.float32)
    lin("qrinv", tofile(d, "X", Xw), os.path.join(d, "xi"))
    lg["qrinv"] = np.fromfile(os.path.join(d, "xi"), np.float32)
    # affineRobust on seeded point sets with 20% outliers (affine and rigid fits)
    npts = 301
    p1 = np.ones((4, npts), np.float32)
    p1[:3] = rng.uniform(0, 60, (3, npts)).astype(np.float32)
    A = np.array([[0.98, 0.05, -0.02, 2.0], [-0.04, 1.02, 0.03, -1.5], [0.02, -0.03, 0.99, 3.0]])
    p2 = np.ones((4, npts), np.float32)
    p2[:3] = (A[:, :3] @ p1[:3] + A[:, 3:]).astype(np.float32) + rng.normal(0, 0.3, (3, npts)).astype(np.float32)
    out_idx = rng.choice(npts, npts // 5, replace=False)
    p2[:3, out_idx] += rng.uniform(-15, 15, (3, out_idx.size)).astype(np.float32)
    lg["robust_p1"] = p1.ravel(); lg["robust_p2"] = p2.ravel()
    for rigid in (0, 1):
        lin("robust", tofile(d, "p1", p1.ravel()), tofile(d, "p2", p2.ravel()), npts, rigid, os.path.join(d, "rt"))
        lg[f"robust_{rigid}"] = np.fromfile(os.path.join(d, "rt"), np.float32)
    # estimateAffine2 on the two cost volumes of a misaligned pair
    em, en, eo = 48, 40, 48
    pair = phantom.make_pair((em, en, eo), seed=5, n_organs=7, max_disp=1.5, affine=(5.0, 0.05, 3.0))
    # whole-HU images (stored as int16), +1024 as the reference shifts them
    fi = np.round(pair["fixed"].ravel(order="F")).astype(np.int16)
    mi = np.round(pair["moving"].ravel(order="F")).astype(np.int16)
    f = fi.astype(np.float32) + np.float32(1024)
    mv = mi.astype(np.float32) + np.float32(1024)
    lg["est_dims"] = np.array([em, en, eo]); lg["est_fixed"] = fi; lg["est_moving"] = mi
    Xp = np.array([1.01, -0.02, 0.01, 0.5, 0.02, 0.99, -0.01, -0.4, -0.01, 0.02, 1.0, 0.3,
                   0.0, 0.0, 0.0, 1.0], np.float32)
    lg["est_Xprev"] = Xp
    for (g, hw, q) in [(5, 3, 2), (4, 2, 1)]:
        qs = int(np.floor(0.5 * q + 1.0))
        for name, img in (("cf", f), ("cm", mv)):
            stage("mind", tofile(d, name + ".f32", img), em, en, eo, qs, os.path.join(d, name + ".u64"))
        cost = {}
        for tag, a, b in (("1", "cf", "cm"), ("2", "cm", "cf")):
            stage("datacost", os.path.join(d, a + ".u64"), os.path.join(d, b + ".u64"), em, en, eo, g, hw, q, "1",
                  os.path.join(d, "cost" + tag))
            cost[tag] = np.fromfile(os.path.join(d, "cost" + tag), np.float32)
        key = f"{g}_{hw}_{q}"
        for tag in ("1", "2"):
            counts, alpha1 = _as_counts(cost[tag], g, q, alpha=1.0)
            lg[f"est_counts{tag}_{key}"] = counts
            lg[f"est_alpha1_{key}"] = alpha1
        for rigid in (0, 1):
            out = lin("estimate", tofile(d, "f", f), tofile(d, "mv", mv), os.path.join(d, "cost1"),
                      os.path.join(d, "cost2"), tofile(d, "xp", Xp), em, en, eo, g, hw, q, rigid,
                      *(os.path.join(d, x) for x in ("X", "s1", "s2")))
            lg[f"est_X_{key}_{rigid}"] = np.fromfile(os.path.join(d, "X"), np.float32)
            lg[f"est_used_{key}_{rigid}"] = np.int32(int(out.split("# points used:")[1].split("/")[0]))
            if rigid == 0:
                for tag, fn in (("1", "s1"), ("2", "s2")):
                    sm = np.fromfile(os.path.join(d, fn), np.float32)
                    lg[f"est_smooth{tag}_sha256_{key}"] = np.frombuffer(hashlib.sha256(sm.tobytes()).digest(), np.uint8)
    # the reference binary end to end (default 4 levels), with a label map
    lm, ln, lo = 64, 48, 64
    pair = phantom.make_pair((lm, ln, lo), seed=8, n_organs=8, max_disp=1.5, affine=(6.0, 0.05, 4.0))
    fpath, mpath, spath = (os.path.join(d, x) for x in ("lf.nii.gz", "lm.nii.gz", "ls.nii.gz"))
    fi = np.round(pair["fixed"]).astype(np.int16)
    mi = np.round(pair["moving"]).astype(np.int16)
    nifti.write(fpath, fi)
    nifti.write(mpath, mi)
    nifti.write(spath, pair["moving_labels"].astype(np.int16))
    lg["e2e_dims"] = np.array([lm, ln, lo])
    lg["e2e_fixed"] = fi.ravel(order="F"); lg["e2e_moving"] = mi.ravel(order="F")
    lg["e2e_moving_labels"] = pair["moving_labels"].ravel(order="F")
    lg["e2e_fixed_labels"] = pair["fixed_labels"].ravel(order="F")
    lg["e2e_true_affine"] = pair["affine"]
    logs = []
    for rigid in (0, 1):
        stem = os.path.join(d, f"lin{rigid}")
        args = ["-F", fpath, "-M", mpath, "-O", stem, "-S", spath] + (["-R", "1"] if rigid else [])
        logs.append(run(os.path.join(REF, "linearBCV"), *args))
        with open(stem + "_matrix.txt") as fh:
            lg[f"e2e_matrix_txt_{rigid}"] = np.frombuffer(fh.read().encode(), np.uint8)
        wseg, _ = nifti.read(stem + "_deformed_seg.nii.gz")
        lg[f"e2e_seg_{rigid}"] = wseg.ravel(order="F").astype(np.int16)
    np.savez_compressed(os.path.join(HERE, "linear.npz"), **lg)
    with open(os.path.join(HERE, "linear_ref_log.txt"), "w") as fh:
        fh.write("\n".join(logs))


def write_matrix(path, X):
    """The affine matrix text file read by -A: line i holds X[i] X[i+4] X[i+8] X[i+12]
    (src/applyBCV.cpp:118-135)."""
    with open(path, "w") as f:
        for i in range(4):
            f.write("  ".join(f"{float(X[i + 4 * k]):.6f}" for k in range(4)) + "\n")


def make_apply(d):
    """applyBCV / applyBCVfloat (src/applyBCV.cpp:54-204, src/applyBCVfloat.cpp): the
    reference deedsBCV binary registers the end-to-end pair of e2e.npz (same inputs
    and flags; its flow must equal the stored one), then the reference
    applyBCVfloat warps a float image with non-integer values (0.37 x the moving
    image + 11.125) through the written displacement file, without and with an
    affine matrix file, and applyBCV warps the moving labels with the matrix."""
    e = np.load(os.path.join(HERE, "e2e.npz"))
    em, en, eo = (int(v) for v in e["dims"])
    fpath, mpath = os.path.join(d, "f.nii.gz"), os.path.join(d, "m.nii.gz")
    nifti.write(fpath, e["fixed"])
    nifti.write(mpath, e["moving"])
    stem = os.path.join(d, "out")
    run(os.path.join(REF, "deedsBCV"), "-F", fpath, "-M", mpath, "-O", stem, "-G", "6x5x4", "-L", "5x4x3",
        "-Q", "3x2x1")
    flow = nifti.read_dat(stem + "_displacements.dat")
    assert np.array_equal(flow, e["flow"]), "the reference's flow on the e2e inputs changed"
    fimg = (e["moving"].astype(np.float32) * np.float32(0.37) + np.float32(11.125)).astype(np.float32)
    ipath = os.path.join(d, "img.nii.gz")
    nifti.write(ipath, fimg)
    X = np.array([0.98, 0.03, -0.02, 1.25, -0.01, 1.02, 0.04, -0.8, 0.02, -0.03, 0.99, 0.6,
                  0.0, 0.0, 0.0, 1.0], np.float32)
    mat = os.path.join(d, "matrix.txt")
    write_matrix(mat, X)
    Xf = np.zeros(16, np.float32)  # the matrix as the reference reads it back (%f text)
    with open(mat) as f:
        for i, line in enumerate(f):
            for k, tok in enumerate(line.split()):
                Xf[i + 4 * k] = np.float32(tok)
    outs = {}
    for key, extra in (("warped_float", []), ("warped_float_affine", ["-A", mat])):
        dst = os.path.join(d, key + ".nii.gz")
        run(os.path.join(REF, "applyBCVfloat"), "-M", ipath, "-O", stem, "-D", dst, *extra)
        outs[key] = nifti.read(dst)[0].ravel(order="F").astype(np.float32)
    spath = os.path.join(d, "seg.nii.gz")
    seg = e["moving_labels"].astype(np.int16)
    nifti.write(spath, seg)
    dst = os.path.join(d, "seg_affine.nii.gz")
    run(os.path.join(REF, "applyBCV"), "-M", spath, "-O", stem, "-D", dst, "-A", mat)
    outs["warped_seg_affine"] = nifti.read(dst)[0].ravel(order="F").astype(np.int16)
    # inputs are those of e2e.npz (flow, moving labels); the float image is derived from its moving image
    np.savez_compressed(os.path.join(HERE, "apply.npz"), X=Xf, **outs)


def main():
    if not os.path.exists(os.path.join(REF, "ref_linear")):
        run("make", "-C", os.path.join(ROOT, "oracle"), "ref")
    if "--linear-only" in sys.argv:  # regenerate linear.npz alone
        with tempfile.TemporaryDirectory() as d:
            make_linear(d, np.random.default_rng(20241204))
        return
    if "--apply-only" in sys.argv:  # regenerate apply.npz alone
        with tempfile.TemporaryDirectory() as d:
            make_apply(d)
        return
    rng = np.random.default_rng(20241203)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        # ---- MIND-SSC (src/MINDSSCbox.h:127) on a 24x20x28 phantom, radii 1..3
        m, n, o = 24, 20, 28
        _, fim, mim = shifted_phantom((m, n, o), seed=1, n_organs=6, max_disp=3.0)
        codes = {}
        for qs in (1, 2, 3):
            stage("mind", tofile(d, "im.f32", fim), m, n, o, qs, os.path.join(d, "c.u64"))
            codes[qs] = np.fromfile(os.path.join(d, "c.u64"), np.uint64)
            stage("mind", tofile(d, "im2.f32", mim), m, n, o, qs, os.path.join(d, "c2.u64"))
            codes[(qs, "m")] = np.fromfile(os.path.join(d, "c2.u64"), np.uint64)
        np.savez_compressed(os.path.join(HERE, "mind.npz"), dims=np.array([m, n, o]), fixed=fim, moving=mim,
                            **{f"codes_q{q}": codes[q] for q in (1, 2, 3)},
                            **{f"mcodes_q{q}": codes[(q, "m")] for q in (1, 2, 3)})
        # ---- dataCostCL (src/dataCostD.h:108) for several (g, hw, q)
        cases = [(4, 2, 1), (5, 2, 2), (6, 2, 3), (8, 3, 2), (7, 1, 4)]
        dc = {"dims": np.array([m, n, o]), "cases": np.array(cases), "alpha": np.float32(1.6)}
        for (g, hw, q) in cases:
            F_ = codes[2]; M_ = codes[(2, "m")]
            stage("datacost", tofile(d, "F.u64", F_), tofile(d, "M.u64", M_), m, n, o, g, hw, q, "1.6",
                  os.path.join(d, "cost.f32"))
            dc[f"cost_{g}_{hw}_{q}"] = np.fromfile(os.path.join(d, "cost.f32"), np.float32)
        dc["F"] = codes[2]; dc["M"] = codes[(2, "m")]
        np.savez_compressed(os.path.join(HERE, "datacost.npz"), **dc)
        # ---- primsGraph (src/primsMST.h:52) on a 32x24x40 phantom, g = 4,5,6,8
        pm, pn, po = 32, 24, 40
        _, pim, pmov = shifted_phantom((pm, pn, po), seed=2, n_organs=8, max_disp=4.0)
        pr = {"dims": np.array([pm, pn, po]), "image": pim}
        for g in (4, 5, 6, 8):
            stage("prims", tofile(d, "p.f32", pim), pm, pn, po, g, *(os.path.join(d, x) for x in ("o.i32", "p.i32", "e.f32")))
            pr[f"ordered_{g}"] = np.fromfile(os.path.join(d, "o.i32"), np.int32)
            pr[f"parents_{g}"] = np.fromfile(os.path.join(d, "p.i32"), np.int32)
            pr[f"edgemst_{g}"] = np.fromfile(os.path.join(d, "e.f32"), np.float32)
        np.savez_compressed(os.path.join(HERE, "prims.npz"), **pr)
        # ---- regularisationCL (src/regularisation.h:115): cost volumes of the 32x24x40 pair
        rg = {"dims": np.array([pm, pn, po])}
        for (g, hw, q) in [(4, 2, 1), (5, 3, 2), (8, 2, 3)]:
            qs = int(np.floor(0.5 * q + 1.0))
            stage("mind", tofile(d, "a.f32", pim), pm, pn, po, qs, os.path.join(d, "a.u64"))
            stage("mind", tofile(d, "b.f32", pmov), pm, pn, po, qs, os.path.join(d, "b.u64"))
            stage("datacost", os.path.join(d, "a.u64"), os.path.join(d, "b.u64"), pm, pn, po, g, hw, q, "1.6",
                  os.path.join(d, "cost.f32"))
            cost = np.fromfile(os.path.join(d, "cost.f32"), np.float32)
            m1, n1, o1 = pm // g, pn // g, po // g
            sz1 = m1 * n1 * o1
            u0 = rng.uniform(-3 * q, 3 * q, sz1).astype(np.float32)
            v0 = rng.uniform(-3 * q, 3 * q, sz1).astype(np.float32)
            w0 = rng.uniform(-3 * q, 3 * q, sz1).astype(np.float32)
            ordered, parents, edgemst = pr[f"ordered_{g}"], pr[f"parents_{g}"], pr[f"edgemst_{g}"]
            stage("reg", os.path.join(d, "cost.f32"), tofile(d, "u0", u0), tofile(d, "v0", v0), tofile(d, "w0", w0),
                  tofile(d, "ord", ordered), tofile(d, "par", parents), tofile(d, "em", edgemst),
                  pm, pn, po, g, hw, q, *(os.path.join(d, x) for x in ("oc", "u1", "v1", "w1")))
            key = f"{g}_{hw}_{q}"
            # the cost volume is float(popcount sum) * alpha1: store the integer sums
            counts, alpha1 = _as_counts(cost, g, q)
            rg[f"counts_{key}"] = counts; rg[f"alpha1_{key}"] = alpha1
            rg[f"u0_{key}"] = u0; rg[f"v0_{key}"] = v0; rg[f"w0_{key}"] = w0
            post = np.fromfile(os.path.join(d, "oc"), np.float32)
            rg[f"post_sha256_{key}"] = np.frombuffer(hashlib.sha256(post.tobytes()).digest(), np.uint8)
            rg[f"post_root_{key}"] = post.reshape(sz1, -1)[ordered[0]]
            for c in ("u1", "v1", "w1"):
                rg[f"{c}_{key}"] = np.fromfile(os.path.join(d, c), np.float32)
        np.savez_compressed(os.path.join(HERE, "reg.npz"), **rg)
        # ---- transforms (src/transformations.h, src/dataCostD.h:213-315)
        tr = {}
        m2, n2, o2 = 5, 4, 6
        gu = rng.uniform(-4, 4, (3, m2 * n2 * o2)).astype(np.float32)
        tm, tn, to = 24, 20, 28
        stage("upsample", *(tofile(d, f"g{i}", gu[i]) for i in range(3)), m2, n2, o2, tm, tn, to,
              *(os.path.join(d, f"up{i}") for i in range(3)))
        tr["grid"] = gu; tr["grid_dims"] = np.array([m2, n2, o2]); tr["dims"] = np.array([tm, tn, to])
        tr["up"] = np.stack([np.fromfile(os.path.join(d, f"up{i}"), np.float32) for i in range(3)])
        # X[0..3] maps to y, X[4..7] to x, X[8..11] to z (src/dataCostD.h:281-283)
        Xf = np.array([1.02, 0.03, -0.02, 0.7, -0.01, 0.98, 0.04, -1.3, 0.02, -0.03, 1.01, 0.4,
                       0.0, 0.0, 0.0, 1.0], np.float32)
        img = fim.copy()
        field = tr["up"] * np.float32(1.7)
        stage("warpaffine", tofile(d, "in", img), tofile(d, "ref", mim), tofile(d, "X", Xf),
              *(tofile(d, f"f{i}", field[i]) for i in (0, 1, 2)), tm, tn, to, os.path.join(d, "wa"))
        tr["X"] = Xf; tr["image"] = img; tr["field"] = field
        tr["warp_affine"] = np.fromfile(os.path.join(d, "wa"), np.float32)
        stage("warpimage", tofile(d, "in", img), tofile(d, "ref", mim),
              *(tofile(d, f"f{i}", field[i]) for i in (0, 1, 2)), tm, tn, to, os.path.join(d, "wi"))
        tr["warp_image"] = np.fromfile(os.path.join(d, "wi"), np.float32)
        seg = rng.integers(0, 14, tm * tn * to).astype(np.int16)
        stage("warpseg", tofile(d, "seg", seg), tofile(d, "X", Xf),
              *(tofile(d, f"f{i}", field[i]) for i in (0, 1, 2)), tm, tn, to, os.path.join(d, "ws"))
        tr["seg"] = seg
        tr["warp_seg"] = np.fromfile(os.path.join(d, "ws"), np.int16)
        cm, cn, co = 8, 6, 7
        six = rng.uniform(-6, 6, (6, cm * cn * co)).astype(np.float32)
        stage("consistent", *(tofile(d, f"c{i}", six[i]) for i in range(6)), cm, cn, co, 4,
              *(os.path.join(d, f"co{i}") for i in range(6)))
        tr["cons_in"] = six; tr["cons_dims"] = np.array([cm, cn, co, 4])
        tr["cons_out"] = np.stack([np.fromfile(os.path.join(d, f"co{i}"), np.float32) for i in range(6)])
        outj = stage("jacobian", *(tofile(d, f"c{i}", six[i]) for i in range(3)), cm, cn, co, 4)
        tr["jac_std"] = np.float32(float(outj.split("JSTD")[1].split()[0]))
        np.savez_compressed(os.path.join(HERE, "transforms.npz"), **tr)
        # ---- end to end: reference deedsBCV binary on a 48x40x48 int16 phantom
        em, en, eo = 48, 40, 48
        pair = phantom.make_pair((em, en, eo), seed=3, n_organs=7, max_disp=4.0)
        fi16 = np.round(pair["fixed"]).astype(np.int16)
        mi16 = np.round(pair["moving"]).astype(np.int16)
        fpath, mpath = os.path.join(d, "f.nii.gz"), os.path.join(d, "m.nii.gz")
        nifti.write(fpath, fi16)
        nifti.write(mpath, mi16)
        spath = os.path.join(d, "seg.nii.gz")
        nifti.write(spath, pair["moving_labels"].astype(np.int16))
        stem = os.path.join(d, "out")
        args = ["-F", fpath, "-M", mpath, "-O", stem, "-G", "6x5x4", "-L", "5x4x3", "-Q", "3x2x1", "-S", spath]
        log = run(os.path.join(REF, "deedsBCV"), *args)
        flow = nifti.read_dat(stem + "_displacements.dat")
        warped, _ = nifti.read(stem + "_deformed.nii.gz")
        wseg, _ = nifti.read(stem + "_deformed_seg.nii.gz")
        np.savez_compressed(os.path.join(HERE, "e2e.npz"), dims=np.array([em, en, eo]), fixed=fi16, moving=mi16,
                            moving_labels=pair["moving_labels"], fixed_labels=pair["fixed_labels"],
                            G=np.array([6, 5, 4]), L=np.array([5, 4, 3]), Q=np.array([3, 2, 1]),
                            flow=flow, warped=warped.ravel(order="F"), warped_seg=wseg.ravel(order="F"))
        with open(os.path.join(HERE, "e2e_ref_log.txt"), "w") as f:
            f.write(log)
    with tempfile.TemporaryDirectory() as d:
        make_linear(d, np.random.default_rng(20241204))
    with tempfile.TemporaryDirectory() as d:
        make_apply(d)
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))


if __name__ == "__main__":
    main()
