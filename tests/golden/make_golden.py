"""Generate the golden vectors that pin the oracle to the reference.

Runs the UNMODIFIED reference, compiled by ``make -C oracle ref`` into
oracle/_ref/ (the stage harness oracle/_ref/ref_stages around the reference's
own functions, and the reference deedsBCV / applyBCV binaries), on small seeded
inputs and stores inputs and outputs under tests/golden/*.npz.  It needs the
reference sources, so it runs only where they are present; the fixtures it
writes are committed and travel with the tests.

    python tests/golden/make_golden.py
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


def main():
    if not os.path.exists(os.path.join(REF, "ref_stages")):
        run("make", "-C", os.path.join(ROOT, "oracle"), "ref")
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
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))


if __name__ == "__main__":
    main()
