"""Generates the golden fixtures of tests/golden/ from the REFERENCE itself.

Run in a container that holds the reference sources (it builds
oracle/_ref/libdcrf_ref.so and libdcrf_ref_scalar.so from them via
oracle/Makefile).  Outputs, all small:

* lattice.npz   -- lattice tables (offset, rank, barycentric, neighbours) of
                   seeded feature sets, from the reference's own
                   Permutohedral::init, x86 (SSE) and scalar builds.
* inference.npz -- marginals after T iterations, startInference, one
                   stepInference and klDivergence of seeded small CRFs covering
                   every compatibility and normalisation type, both builds.
* gradient.npz  -- the reference's own DenseCRF::gradient (log-likelihood of
                   a label map) of seeded small CRFs: objective, dL/dU (through
                   a logistic unary L*I), compatibility and kernel-parameter
                   gradients, for every normalisation, compatibility and kernel
                   type.
* energy.npz    -- the reference's own DenseCRF::unaryEnergy / pairwiseEnergy
                   (debug energies of a labelling) on seeded CRFs covering
                   every normalisation, compatibility and kernel type, both
                   builds.
* utils.npz     -- outputs of the reference's pure-numpy pydensecrf/utils.py
                   (unary and feature builders) on seeded inputs, imported
                   from its source file.
* examples.npz  -- the reference's example images and annotations
                   (examples/im*.png, anno*.png) decoded, with the shipped
                   outputs (out*.png) turned back into label maps, and the
                   reference's MAP of the generic path of examples/inference.py.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT [FIXTURE ...]]
(FIXTURE: lattice, inference, gradient, energy, utils, examples; default all)
"""
from __future__ import annotations

import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

REF_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DCRF_REFERENCE_ROOT", "")
if __name__ == "__main__" and not os.path.isdir(REF_ROOT):
    sys.exit("usage: make_golden.py REFERENCE_ROOT [FIXTURE ...] (or set DCRF_REFERENCE_ROOT): "
             "the root of a pydensecrf checkout")


# ---------------------------------------------------------------------------
# minimal PNG decoder (8-bit RGB and 1/2/4/8-bit palette, non-interlaced)
# ---------------------------------------------------------------------------
def read_png(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", path
    pos, idat, plte = 8, b"", None
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h, bd, ct, _, _, il = struct.unpack(">IIBBBBB", body)
        elif typ == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    assert il == 0, "interlaced PNG not supported"
    raw = zlib.decompress(idat)
    chans = {2: 3, 3: 1, 0: 1, 6: 4}[ct]
    bpp = max(1, chans * bd // 8)
    stride = (w * chans * bd + 7) // 8
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    p = 0
    for y in range(h):
        f = raw[p]
        line = np.frombuffer(raw[p + 1:p + 1 + stride], np.uint8).astype(np.int32)
        p += 1 + stride
        cur = np.zeros(stride, np.int32)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if f == 0:
                v = line[x]
            elif f == 1:
                v = line[x] + a
            elif f == 2:
                v = line[x] + b
            elif f == 3:
                v = line[x] + ((a + b) >> 1)
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                v = line[x] + pr
            cur[x] = v & 255
        out[y] = cur
        prev = cur
    if ct == 3:
        bits = np.unpackbits(out, axis=1)[:, :w * bd].reshape(h, w, bd)
        idx = (bits * (1 << np.arange(bd - 1, -1, -1))).sum(-1)
        return plte[idx]
    return out[:, :w * chans].reshape(h, w, chans)


def gen_lattice():
    rng = np.random.default_rng(20240601)
    cases = {}
    specs = [(1, 7), (2, 1), (2, 9), (2, 300), (3, 257), (4, 300), (5, 13), (5, 400), (7, 200), (9, 100),
             (12, 60), (16, 40)]
    for ci, (d, N) in enumerate(specs):
        f = rng.normal(0, 2.5, size=(N, d)).astype(np.float32)
        cases[f"c{ci}"] = f
    # integer-valued grid features (rounding ties) and image-like bilateral features
    cases["grid"] = np.stack(np.meshgrid(np.arange(23, dtype=np.float32), np.arange(19, dtype=np.float32),
                                         indexing="ij"), -1).reshape(-1, 2) / np.float32(1.0)
    cases["grid3"] = np.stack(np.meshgrid(np.arange(9, dtype=np.float32), np.arange(7, dtype=np.float32),
                                          np.arange(5, dtype=np.float32), indexing="ij"), -1).reshape(-1, 3)
    img = rng.integers(0, 256, size=(17, 21, 3)).astype(np.uint8)
    cases["bilat"] = O.features_bilateral_2d(img, 5.0, 5.0, 13.0, 13.0, 13.0)
    out = {}
    for name, f in cases.items():
        out[f"{name}/feat"] = f
        for vname, var in (("sse", O.VARIANT_SSE), ("scalar", O.VARIANT_SCALAR)):
            lat = O.Lattice(f, "ref", var)
            out[f"{name}/{vname}/offset"] = lat.offset
            out[f"{name}/{vname}/rank"] = lat.rank
            out[f"{name}/{vname}/bary"] = lat.bary
            out[f"{name}/{vname}/neighbors"] = lat.neighbors
    np.savez_compressed(os.path.join(HERE, "lattice.npz"), **out)
    print("lattice.npz", len(cases), "feature sets")


def gen_inference():
    rng = np.random.default_rng(7)
    out = {}
    W, H, M = 20, 14, 5
    N = W * H
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    img[4:11, 6:16] = [200, 40, 40]
    logits = rng.normal(0, 2, size=(N, M)).astype(np.float32)
    U = -np.log(np.exp(logits) / np.exp(logits).sum(1, keepdims=True)).astype(np.float32)  # (N, M)
    fg = O.features_gaussian_2d(W, H, 3.0, 3.0)
    fb = O.features_bilateral_2d(img, 8.0, 8.0, 13.0, 13.0, 13.0)
    diag = rng.uniform(-3, 0, size=M).astype(np.float32)
    mat = rng.uniform(0, 2, size=(M, M)).astype(np.float32)
    cases = []
    for ck, c in (("potts", 3.0), ("diag", diag), ("mat", mat)):
        for nt in range(4):
            cases.append((f"{ck}_n{nt}", [(fg, c, 1, nt), (fb, 5.0, 1, 3)], 1))
    cases.append(("fullk", [(fg, 3.0, 2, 3), (fb, 10.0, 2, 3)], 2))
    out["U"] = U
    out["img"] = img
    out["W"], out["H"], out["M"] = W, H, M
    out["diag"], out["mat"] = diag, mat
    T = 4
    for name, terms, _ in cases:
        for vname, var in (("sse", O.VARIANT_SSE), ("scalar", O.VARIANT_SCALAR)):
            r = O.RefCRF(N, M, variant=var)
            r.set_unary(U)
            for f, c, kt, nt in terms:
                r.add_pairwise(f, c, kt, nt)
            Q = r.inference(T)
            Q0 = r.start()
            Q1 = Q0.copy()
            r.step(Q1)
            out[f"{name}/{vname}/Q"] = Q
            out["Q0"] = Q0
            out[f"{name}/{vname}/Q1"] = Q1
            out[f"{name}/{vname}/kl"] = np.float64(r.kl(Q))
    # two-label and M=2 path (seqCompute for the messages too)
    U2 = U[:, :2].copy()
    for vname, var in (("sse", O.VARIANT_SSE), ("scalar", O.VARIANT_SCALAR)):
        r = O.RefCRF(N, 2, variant=var)
        r.set_unary(U2)
        r.add_pairwise(fb, 4.0, 1, 3)
        out[f"m2/{vname}/Q"] = r.inference(5)
    out["U2"] = U2
    out["T"] = T
    out["cases"] = np.array([c[0] for c in cases])
    np.savez_compressed(os.path.join(HERE, "inference.npz"), **out)
    print("inference.npz", len(cases), "cases")


def gen_gradient():
    rng = np.random.default_rng(99)
    out = {}
    W, H, M, T = 12, 10, 3, 3
    N = W * H
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    img[3:8, 2:9] = [30, 200, 90]
    logits = rng.normal(0, 1.5, size=(N, M)).astype(np.float32)
    U = -np.log(np.exp(logits) / np.exp(logits).sum(1, keepdims=True)).astype(np.float32)  # (N, M)
    gt = rng.integers(0, M, size=N).astype(np.int16)
    fg = O.features_gaussian_2d(W, H, 2.0, 2.0)
    fb = O.features_bilateral_2d(img, 5.0, 5.0, 40.0, 40.0, 40.0)
    diag = rng.uniform(-2, -0.5, size=M).astype(np.float32)
    mat = rng.uniform(-1, 1, size=(M, M)).astype(np.float32)
    cases = []
    for ck, c in (("potts", 2.0), ("diag", diag), ("mat", mat)):
        for nt in range(4):
            for kt in (1, 2):
                cases.append((f"{ck}_n{nt}_k{kt}", c, nt, kt))
    eye = np.eye(N, dtype=np.float32)
    for name, c, nt, kt in cases:
        r = O.RefCRF(N, M)
        lib = r._lib
        Lm = np.ascontiguousarray(U.T)  # L = U^T as M x N (column-major = point-major U), f = I
        lib.ref_crf_set_unary_logistic(r._h, O._p(np.ascontiguousarray(U), O._f32p), O._p(eye, O._f32p), M, N, N)
        r.add_pairwise(fg, c, kt, nt)
        r.add_pairwise(fb, 3.0, kt, 3)
        val, ug, cg, kg = r.gradient(T, gt, want_unary=True, want_compat=True, want_kernel=True)
        out[f"{name}/obj"] = np.float64(val)
        out[f"{name}/dU"] = ug.reshape(N, M)
        out[f"{name}/dcompat"] = cg
        out[f"{name}/dkernel"] = kg
        out[f"{name}/Q"] = r.inference(T)
    out.update(U=U, img=img, gt=gt, W=W, H=H, M=M, T=T, diag=diag, mat=mat,
               cases=np.array([c[0] for c in cases]))
    np.savez_compressed(os.path.join(HERE, "gradient.npz"), **out)
    print("gradient.npz", len(cases), "cases")


def gen_energy():
    rng = np.random.default_rng(4242)
    N, M = 700, 5
    f = rng.normal(0, 1.5, size=(N, 3)).astype(np.float32)
    f2 = rng.normal(0, 2.0, size=(N, 2)).astype(np.float32)
    U = (rng.random((N, M)) * 3).astype(np.float32)  # per point
    mat = rng.uniform(-1, 1, size=(M, M)).astype(np.float32)
    diag = rng.uniform(0, 2, size=M).astype(np.float32)
    lab = rng.integers(-1, M + 1, size=N).astype(np.int16)  # -1 and M: no label
    out = {"f": f, "f2": f2, "U": U, "mat": mat, "diag": diag, "lab": lab}
    # name -> terms [(feature key, compat, kernel type, normalisation)]
    cases = {f"mat_n{nt}": [("f", "mat", 1, nt)] for nt in range(4)}
    cases["potts_n3"] = [("f", 2.5, 1, 3)]
    cases["diag_n1"] = [("f", "diag", 1, 1)]
    cases["full_n3"] = [("f", "mat", 2, 3)]
    cases["two_terms"] = [("f", 2.0, 1, 3), ("f2", "mat", 1, 2)]
    out["cases"] = np.array(list(cases))
    for name, terms in cases.items():
        for vname, var in (("sse", O.VARIANT_SSE), ("scalar", O.VARIANT_SCALAR)):
            r = O.RefCRF(N, M, variant=var)
            r.set_unary(U)
            for fk, ck, kt, nt in terms:
                r.add_pairwise(out[fk], out[ck] if isinstance(ck, str) else ck, kt, nt)
            out[f"{name}/{vname}/unary"] = r.unary_energy(lab)
            out[f"{name}/{vname}/pairwise"] = r.pairwise_energy(lab, -1)
            for k in range(len(terms)):
                out[f"{name}/{vname}/pairwise{k}"] = r.pairwise_energy(lab, k)
    np.savez_compressed(os.path.join(HERE, "energy.npz"), **out)
    print("energy.npz", len(cases), "cases")


def _ref_utils():
    """The reference's pydensecrf/utils.py, loaded from its file alone (its
    package __init__ would import the compiled extension)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("ref_utils", os.path.join(REF_ROOT, "pydensecrf", "utils.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def gen_utils():
    R = _ref_utils()
    rng = np.random.default_rng(515)
    out = {}
    # unary_from_labels: 1-based labels with unknowns, and 0-based labels
    lab = rng.integers(0, 6, size=(13, 17)).astype(np.int32)
    out["lab"] = lab
    for gt in (0.5, 0.7, 0.95):
        out[f"labels_unsure/{gt}"] = R.unary_from_labels(lab, 5, gt, zero_unsure=True)
        out[f"labels_sure/{gt}"] = R.unary_from_labels(lab, 6, gt, zero_unsure=False)
    out["compute_unary"] = R.compute_unary(lab, 5, GT_PROB=0.6)
    # unary_from_softmax / softmax_to_unary on float64 and float32 probabilities
    logits = rng.normal(0, 3, size=(4, 9, 11))
    sm = np.exp(logits - logits.max(0))
    sm /= sm.sum(0)
    sm[0, 0, :3] = 0.0
    out["sm64"] = sm
    out["sm32"] = sm.astype(np.float32)
    for name in ("sm64", "sm32"):
        x = out[name]
        out[f"softmax/{name}/default"] = R.unary_from_softmax(x)
        out[f"softmax/{name}/scale"] = R.unary_from_softmax(x, scale=0.8)
        out[f"softmax/{name}/noclip"] = R.unary_from_softmax(np.maximum(x, 1e-30), clip=None)
        out[f"softmax/{name}/scale_noclip"] = R.unary_from_softmax(x, scale=0.6, clip=None)
        out[f"softmax/{name}/to_unary"] = R.softmax_to_unary(np.maximum(x, 1e-30))
        out[f"softmax/{name}/to_unary_gt"] = R.softmax_to_unary(x, GT_PROB=0.7)
    # feature builders: 2-D and 3-D grids, RGB / single-channel / channels-first images
    out["gauss2"] = R.create_pairwise_gaussian(sdims=(3, 5), shape=(19, 23))
    out["gauss2_frac"] = R.create_pairwise_gaussian(sdims=(0.7, 13.3), shape=(7, 29))
    out["gauss3"] = R.create_pairwise_gaussian(sdims=(2, 3, 7), shape=(5, 6, 7))
    img = rng.integers(0, 256, size=(15, 18, 3)).astype(np.uint8)
    vol = rng.integers(0, 4096, size=(2, 5, 6, 4)).astype(np.uint16)
    gray = rng.random(size=(12, 10)).astype(np.float32)
    out["img"], out["vol"], out["gray"] = img, vol, gray
    out["bilat_rgb"] = R.create_pairwise_bilateral(sdims=(80, 80), schan=(13, 13, 13), img=img, chdim=2)
    out["bilat_rgb_mixed"] = R.create_pairwise_bilateral(sdims=(3.3, 7), schan=(5, 11.5, 0.9), img=img, chdim=2)
    out["bilat_rgb_scalar"] = R.create_pairwise_bilateral(sdims=(4, 4), schan=20, img=img, chdim=2)
    out["bilat_gray"] = R.create_pairwise_bilateral(sdims=(2, 9), schan=0.3, img=gray, chdim=-1)
    out["bilat_vol"] = R.create_pairwise_bilateral(sdims=(1, 2, 3), schan=(100, 250.0), img=vol, chdim=0)
    out["gauss2_loop"] = R._create_pairwise_gaussian_2d(3, 5, (9, 8))
    out["bilat2_loop"] = R._create_pairwise_bilateral_2d(3, 5, 13, 11, 7, img[:9, :8])
    np.savez_compressed(os.path.join(HERE, "utils.npz"), **out)
    print("utils.npz", len(out), "arrays")


def gen_examples():
    ex = os.path.join(REF_ROOT, "examples")
    out = {}
    for k in ("1", "2", "3"):
        img = read_png(os.path.join(ex, f"im{k}.png"))[..., :3]
        anno = read_png(os.path.join(ex, f"anno{k}.png")).astype(np.uint32)
        outp = read_png(os.path.join(ex, f"out{k}.png")).astype(np.uint32)
        lbl = anno[..., 0] + (anno[..., 1] << 8) + (anno[..., 2] << 16)
        colors, labels = np.unique(lbl, return_inverse=True)
        has_unk = 0 in colors
        if has_unk:
            colors = colors[1:]
        n_labels = len(set(labels.flat)) - int(has_unk)
        col_out = (outp[..., 0] + (outp[..., 1] << 8) + (outp[..., 2] << 16)).reshape(-1)
        # shipped output as label indices (-1 where the colour is not a label colour)
        lut = {int(c): i for i, c in enumerate(colors)}
        shipped = np.array([lut.get(int(c), -1) for c in col_out], np.int16)
        H, W = img.shape[:2]
        # the reference's generic path (examples/inference.py:93-119)
        from pydensecrf_gb300 import utils as U

        Uu = U.unary_from_labels(labels, n_labels, gt_prob=0.7, zero_unsure=has_unk)
        fg = U.create_pairwise_gaussian(sdims=(3, 3), shape=img.shape[:2])
        fb = U.create_pairwise_bilateral(sdims=(80, 80), schan=(13, 13, 13), img=img, chdim=2)
        r = O.RefCRF(W * H, n_labels)
        r.set_unary(np.ascontiguousarray(Uu.T))
        r.add_pairwise(np.ascontiguousarray(fg.T), 3.0, 1, 3)
        r.add_pairwise(np.ascontiguousarray(fb.T), 10.0, 1, 3)
        Q = r.inference(5)
        ref_map = Q.argmax(1).astype(np.int16)
        print(f"example {k}: reference MAP vs shipped out{k}.png agreement {(ref_map == shipped).mean():.4%}")
        out[f"{k}/img"] = img.astype(np.uint8)
        out[f"{k}/labels"] = labels.reshape(H, W).astype(np.int16)
        out[f"{k}/has_unk"] = np.bool_(has_unk)
        out[f"{k}/n_labels"] = np.int32(n_labels)
        out[f"{k}/shipped_map"] = shipped
        out[f"{k}/ref_map"] = ref_map
    np.savez_compressed(os.path.join(HERE, "examples.npz"), **out)


if __name__ == "__main__":
    O.build(reference_root=REF_ROOT)
    if not (O.ref_available(O.VARIANT_SSE) and O.ref_available(O.VARIANT_SCALAR)):
        sys.exit("the reference could not be built from " + REF_ROOT)
    gens = {"lattice": gen_lattice, "inference": gen_inference, "gradient": gen_gradient, "energy": gen_energy,
            "utils": gen_utils, "examples": gen_examples}
    for name in (sys.argv[2:] or gens):
        gens[name]()
