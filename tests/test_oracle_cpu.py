"""CPU tests of the oracle: pinned against the reference's golden fixtures and,
where the reference could be compiled here, against the reference itself."""
import numpy as np
import pytest


def _bits(a):
    return np.ascontiguousarray(a).view(np.int32)


VARIANTS = (("sse", 0), ("scalar", 1))


@pytest.mark.parametrize("vname,var", VARIANTS)
def test_oracle_lattice_matches_golden(oracle_mod, golden, vname, var):
    g = golden("lattice.npz")
    names = sorted({k.split("/")[0] for k in g.files})
    for name in names:
        lat = oracle_mod.Lattice(g[f"{name}/feat"], "oracle", var)
        assert np.array_equal(lat.offset, g[f"{name}/{vname}/offset"]), name
        assert np.array_equal(lat.rank, g[f"{name}/{vname}/rank"]), name
        assert np.array_equal(_bits(lat.bary), _bits(g[f"{name}/{vname}/bary"])), name
        assert np.array_equal(lat.neighbors, g[f"{name}/{vname}/neighbors"]), name


@pytest.mark.parametrize("vname,var", VARIANTS)
def test_oracle_inference_matches_golden(oracle_mod, golden, vname, var):
    g = golden("inference.npz")
    O = oracle_mod
    W, H, M, T = int(g["W"]), int(g["H"]), int(g["M"]), int(g["T"])
    N = W * H
    U, img = g["U"], g["img"]
    fg = O.features_gaussian_2d(W, H, 3.0, 3.0)
    fb = O.features_bilateral_2d(img, 8.0, 8.0, 13.0, 13.0, 13.0)
    compat = {"potts": 3.0, "diag": g["diag"], "mat": g["mat"]}
    for name in g["cases"]:
        name = str(name)
        c = O.OracleCRF(N, M, var)
        c.set_unary(U)
        if name == "fullk":
            c.add_pairwise(fg, 3.0, 2, 3)
            c.add_pairwise(fb, 10.0, 2, 3)
        else:
            ck, nt = name.split("_n")
            c.add_pairwise(fg, compat[ck], 1, int(nt))
            c.add_pairwise(fb, 5.0, 1, 3)
        Q = c.inference(T)
        # tolerance 1e-5: the only differences are libm expf vs Eigen's exp and sum order
        assert np.abs(Q - g[f"{name}/{vname}/Q"]).max() < 1e-5, name
        Q0 = c.start()
        assert np.abs(Q0 - g["Q0"]).max() < 1e-6
        c.step(Q0)
        assert np.abs(Q0 - g[f"{name}/{vname}/Q1"]).max() < 1e-5, name
        kl_ref = float(g[f"{name}/{vname}/kl"])
        assert abs(c.kl(g[f"{name}/{vname}/Q"]) - kl_ref) <= 1e-5 * max(1.0, abs(kl_ref)), name


def test_oracle_two_labels_golden(oracle_mod, golden):
    g = golden("inference.npz")
    O = oracle_mod
    W, H = int(g["W"]), int(g["H"])
    fb = O.features_bilateral_2d(g["img"], 8.0, 8.0, 13.0, 13.0, 13.0)
    for vname, var in VARIANTS:
        c = O.OracleCRF(W * H, 2, var)
        c.set_unary(g["U2"])
        c.add_pairwise(fb, 4.0, 1, 3)
        assert np.abs(c.inference(5) - g[f"m2/{vname}/Q"]).max() < 1e-5


def test_oracle_examples_golden(oracle_mod, golden):
    """The reference's own example outputs (examples/out{1,2,3}.png) via the generic path."""
    from pydensecrf_gb300 import utils as U
    g = golden("examples.npz")
    O = oracle_mod
    for k in ("1", "2", "3"):
        img, labels = g[f"{k}/img"], g[f"{k}/labels"]
        n_labels, has_unk = int(g[f"{k}/n_labels"]), bool(g[f"{k}/has_unk"])
        H, W = labels.shape
        Uu = U.unary_from_labels(labels, n_labels, gt_prob=0.7, zero_unsure=has_unk)
        fg = U.create_pairwise_gaussian(sdims=(3, 3), shape=(H, W))
        fb = U.create_pairwise_bilateral(sdims=(80, 80), schan=(13, 13, 13), img=img, chdim=2)
        c = O.OracleCRF(W * H, n_labels)
        c.set_unary(np.ascontiguousarray(Uu.T))
        c.add_pairwise(np.ascontiguousarray(fg.T), 3.0)
        c.add_pairwise(np.ascontiguousarray(fb.T), 10.0)
        m = c.inference(5).argmax(1)
        assert (m == g[f"{k}/shipped_map"]).mean() == 1.0, k


def test_oracle_fp64_close(oracle_mod):
    """The float restatement stays within 1e-5 of the FP64 mean-field on a small case."""
    O = oracle_mod
    rng = np.random.default_rng(3)
    N, M = 500, 4
    f = rng.normal(0, 1.5, size=(N, 3)).astype(np.float32)
    U = (rng.random((N, M)) * 3).astype(np.float32)
    c = O.OracleCRF(N, M)
    c.set_unary(U)
    c.add_pairwise(f, 2.0)
    assert np.abs(c.inference(5) - c.inference_f64(5)).max() < 1e-5


def test_fp64_filter_and_transpose_identity(oracle_mod):
    """The FP64 filter that the full-size GPU filter test measures against:
    within 2e-6 of the oracle's float filter (both sseCompute and seqCompute
    value sizes) on a small bilateral case.  The oracle's reverse filter is the
    transpose of its forward one: <K x, y> = <x, K^T y>."""
    from filter_f64 import filter_f64

    O = oracle_mod
    rng = np.random.default_rng(41)
    W, H = 96, 64
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    lat = O.Lattice(O.features_bilateral_2d(img, 20, 20, 13, 13, 13), "oracle")
    for vs in (1, 2, 21):
        x = rng.random((W * H, vs)).astype(np.float32)
        y = rng.random((W * H, vs)).astype(np.float32)
        Kx = lat.compute(x, False)
        k64 = filter_f64(lat, x)
        assert np.abs(Kx - k64).max() <= 2e-6 * np.abs(k64).max(), vs
        lhs = float((Kx.astype(np.float64) * y).sum())
        rhs = float((x.astype(np.float64) * lat.compute(y, True)).sum())
        assert abs(lhs - rhs) <= 1e-6 * abs(lhs), vs


requires_ref =pytest.mark.skipif("not __import__('oracle').ref_available()",
                                  reason="the reference was not compiled on this machine")


@requires_ref
@pytest.mark.parametrize("vname,var", VARIANTS)
def test_oracle_vs_reference_random(oracle_mod, vname, var):
    O = oracle_mod
    if not O.ref_available(var):
        pytest.skip("variant not built")
    rng = np.random.default_rng(11 + var)
    for d in (1, 2, 3, 5, 6, 8):
        for N in (1, 3, 4, 5, 77, 640):
            f = rng.normal(0, 3, size=(N, d)).astype(np.float32)
            a, b = O.Lattice(f, "oracle", var), O.Lattice(f, "ref", var)
            assert a.L == b.L
            assert np.array_equal(a.offset, b.offset) and np.array_equal(a.rank, b.rank)
            assert np.array_equal(_bits(a.bary), _bits(b.bary)) and np.array_equal(a.neighbors, b.neighbors)
            v = rng.random((N, 3)).astype(np.float32)
            for rev in (False, True):
                assert np.array_equal(_bits(a.compute(v, rev)), _bits(b.compute(v, rev)))


@requires_ref
@pytest.mark.parametrize("vname,var", VARIANTS)
def test_oracle_map_matches_reference(oracle_mod, vname, var):
    """map after T iterations: the first maximum per point, as the reference's
    DenseCRF::map (densecrf.cpp:132-137,202-211).  A CRF with exactly tied
    marginals (no unary, so Q is uniform) must give label 0 everywhere; a
    random one must give the reference's labels (ties are measure-zero there,
    and Q differs from the reference's only at the ulp level)."""
    O = oracle_mod
    if not O.ref_available(var):
        pytest.skip("variant not built")
    rng = np.random.default_rng(77 + var)
    N, M = 900, 6
    f = rng.normal(0, 1.5, size=(N, 3)).astype(np.float32)
    o, r = O.OracleCRF(N, M, var), O.RefCRF(N, M, variant=var)
    for c in (o, r):
        c.add_pairwise(f, 3.0)
    assert np.array_equal(o.map(3), np.zeros(N, np.int16))
    assert np.array_equal(r.map(3), np.zeros(N, np.int16))
    U = (rng.random((N, M)) * 4).astype(np.float32)
    mat = rng.uniform(0, 1, (M, M)).astype(np.float32)
    o, r = O.OracleCRF(N, M, var), O.RefCRF(N, M, variant=var)
    for c in (o, r):
        c.set_unary(U)
        c.add_pairwise(f, 3.0)
        c.add_pairwise(f[:, :2].copy(), mat)
    mo, mr = o.map(4), r.map(4)
    assert mo.dtype == np.int16 and np.array_equal(mo, o.inference(4).argmax(1).astype(np.int16))
    assert (mo == mr).mean() >= 0.999, (mo == mr).mean()


@pytest.mark.parametrize("name", ["potts_n3_k1", "diag_n1_k1", "mat_n3_k1", "mat_n2_k2"])
def test_reference_gradient_vs_fp64_finite_differences(oracle_mod, golden, name):
    """The reference's own DenseCRF::gradient (the golden fixture the GPU
    adjoint is held to) against central differences of the FP64 restatement
    of the same mean-field: objective = mean log Q(gt) (objective.cpp:37-50;
    the cases here keep every Q(gt) far above its 1e-20 clamp).  dL/dU, the
    compatibility of the first term (Potts weight, Diagonal entries, or the
    Matrix's packed upper triangle, labelcompatibility.cpp:101-107, under a
    symmetric perturbation) and the second term's Potts weight.  Steps are
    powers of two, so the perturbed float inputs are exact.  Tolerance 1e-3 of
    the largest magnitude, like the GPU tests."""
    g = golden("gradient.npz")
    O = oracle_mod
    W, H, M, T = int(g["W"]), int(g["H"]), int(g["M"]), int(g["T"])
    N = W * H
    U, gt = g["U"], g["gt"].astype(np.int64)
    fg = O.features_gaussian_2d(W, H, 2.0, 2.0)
    fb = O.features_bilateral_2d(g["img"], 5.0, 5.0, 40.0, 40.0, 40.0)
    ck, rest = name.split("_n")
    nt, kt = (int(x) for x in rest.split("_k"))
    compat = {"potts": np.float32(2.0), "diag": g["diag"], "mat": g["mat"]}[ck]

    def obj(Uv, c=compat, w2=3.0):
        o = O.OracleCRF(N, M)
        o.set_unary(Uv)
        o.add_pairwise(fg, float(c) if np.ndim(c) == 0 else c, kt, nt)
        o.add_pairwise(fb, w2, kt, 3)
        return float(np.log(o.inference_f64(T)[np.arange(N), gt]).mean())

    assert abs(obj(U) - float(g[f"{name}/obj"])) < 1e-5
    dU, dc = g[f"{name}/dU"], g[f"{name}/dcompat"]
    rng = np.random.default_rng(9)
    du = 2.0 ** -10
    fd, ref = [], []
    for n, m in zip(rng.integers(0, N, 10), rng.integers(0, M, 10)):
        up, dn = U.copy(), U.copy()
        up[n, m] += np.float32(du)
        dn[n, m] -= np.float32(du)
        fd.append((obj(up) - obj(dn)) / (2 * du))
        ref.append(dU[n, m])
    assert np.abs(np.array(fd) - ref).max() <= 1e-3 * np.abs(dU).max()

    dw = 2.0 ** -8
    want = []
    if ck == "potts":
        want.append((obj(U, compat + dw) - obj(U, compat - dw)) / (2 * dw))
    elif ck == "diag":
        for m in range(M):
            e = np.zeros(M, np.float32)
            e[m] = dw
            want.append((obj(U, compat + e) - obj(U, compat - e)) / (2 * dw))
    else:
        for i in range(M):
            for j in range(i, M):
                e = np.zeros((M, M), np.float32)
                e[i, j] = e[j, i] = dw
                want.append((obj(U, compat + e) - obj(U, compat - e)) / (2 * dw))
    want.append((obj(U, w2=3.0 + dw) - obj(U, w2=3.0 - dw)) / (2 * dw))
    want = np.array(want)
    assert dc.shape == want.shape
    assert np.abs(dc - want).max() <= 1e-3 * np.abs(want).max(), (dc, want)
