"""GPU mean-field inference against the reference's golden marginals, the
oracle (same seeded inputs) and the FP64 restatement.

Tolerances (float32 path): Q max-abs <= 1e-4 against the reference/oracle,
argmax agreement >= 99.9 %; klDivergence relative 1e-5 (the device sums in
double, the reference's pairwise term in float)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
QTOL = 1e-4
VARIANTS = (("sse", 0), ("scalar", 1))


def _golden_crf(dc, g, name, var, O):
    W, H, M = int(g["W"]), int(g["H"]), int(g["M"])
    N = W * H
    fg = O.features_gaussian_2d(W, H, 3.0, 3.0)
    fb = O.features_bilateral_2d(g["img"], 8.0, 8.0, 13.0, 13.0, 13.0)
    compat = {"potts": 3.0, "diag": g["diag"], "mat": g["mat"]}
    crf = dc.DenseCRF(N, M)
    crf.set_variant(var)
    crf.setUnaryEnergy(np.ascontiguousarray(g["U"].T))
    if name == "fullk":
        crf.addPairwiseEnergy(np.ascontiguousarray(fg.T), 3.0, dc.FULL_KERNEL)
        crf.addPairwiseEnergy(np.ascontiguousarray(fb.T), 10.0, dc.FULL_KERNEL)
    else:
        ck, nt = name.split("_n")
        crf.addPairwiseEnergy(np.ascontiguousarray(fg.T), compat[ck], dc.DIAG_KERNEL, int(nt))
        crf.addPairwiseEnergy(np.ascontiguousarray(fb.T), 5.0)
    return crf


@pytest.mark.parametrize("vname,var", VARIANTS)
def test_inference_matches_reference_golden(engine, oracle_mod, golden, vname, var):
    g = golden("inference.npz")
    T = int(g["T"])
    for name in g["cases"]:
        name = str(name)
        crf = _golden_crf(engine, g, name, var, oracle_mod)
        Q = np.array(crf.inference(T)).T  # (N, M)
        err = np.abs(Q - g[f"{name}/{vname}/Q"]).max()
        assert err < QTOL, (name, err)
        Qs, t1, t2 = crf.startInference()
        assert np.abs(np.array(Qs).T - g["Q0"]).max() < 1e-6
        crf.stepInference(Qs, t1, t2)
        assert np.abs(np.array(Qs).T - g[f"{name}/{vname}/Q1"]).max() < QTOL, name
        kl_ref = float(g[f"{name}/{vname}/kl"])
        kl = crf.klDivergence(engine.MatrixXf().wrap_colmajor(np.ascontiguousarray(g[f"{name}/{vname}/Q"])))
        assert abs(kl - kl_ref) <= 1e-5 * max(1.0, abs(kl_ref)), (name, kl, kl_ref)


def test_two_labels_golden(engine, oracle_mod, golden):
    g = golden("inference.npz")
    O = oracle_mod
    W, H = int(g["W"]), int(g["H"])
    fb = O.features_bilateral_2d(g["img"], 8.0, 8.0, 13.0, 13.0, 13.0)
    for vname, var in VARIANTS:
        crf = engine.DenseCRF(W * H, 2)
        crf.set_variant(var)
        crf.setUnaryEnergy(np.ascontiguousarray(g["U2"].T))
        crf.addPairwiseEnergy(np.ascontiguousarray(fb.T), 4.0)
        assert np.abs(np.array(crf.inference(5)).T - g[f"m2/{vname}/Q"]).max() < QTOL


def test_examples_golden(engine, golden):
    """examples/inference.py generic path on the reference's example images:
    MAP against the reference's shipped out{1,2,3}.png."""
    from pydensecrf_gb300 import utils as U
    g = golden("examples.npz")
    for k in ("1", "2", "3"):
        img, labels = g[f"{k}/img"], g[f"{k}/labels"]
        n_labels, has_unk = int(g[f"{k}/n_labels"]), bool(g[f"{k}/has_unk"])
        H, W = labels.shape
        d = engine.DenseCRF(W * H, n_labels)
        d.setUnaryEnergy(U.unary_from_labels(labels, n_labels, gt_prob=0.7, zero_unsure=has_unk))
        d.addPairwiseEnergy(U.create_pairwise_gaussian(sdims=(3, 3), shape=(H, W)), compat=3,
                            kernel=engine.DIAG_KERNEL, normalization=engine.NORMALIZE_SYMMETRIC)
        d.addPairwiseEnergy(U.create_pairwise_bilateral(sdims=(80, 80), schan=(13, 13, 13), img=img, chdim=2),
                            compat=10, kernel=engine.DIAG_KERNEL, normalization=engine.NORMALIZE_SYMMETRIC)
        m = np.argmax(d.inference(5), axis=0)
        agree = (m == g[f"{k}/shipped_map"]).mean()
        assert agree >= 0.999, (k, agree)


def _cfg1_pair(dc, O, var, seed=0, W=320, H=240, M=5, T=5):
    from pydensecrf_gb300 import synthetic as S
    cfg = S.plain_small(seed, W, H, M)
    d = dc.DenseCRF2D(W, H, M)
    d.set_variant(var)
    d.setUnaryEnergy(cfg["U"])
    d.addPairwiseGaussian(sxy=3, compat=3)
    d.addPairwiseBilateral(sxy=80, srgb=13, rgbim=cfg["img"], compat=10)
    o = O.OracleCRF(W * H, M, var)
    o.set_unary(np.ascontiguousarray(cfg["U"].T))
    o.add_pairwise(O.features_gaussian_2d(W, H, 3, 3), 3.0)
    o.add_pairwise(O.features_bilateral_2d(cfg["img"], 80, 80, 13, 13, 13), 10.0)
    return d, o, cfg


@pytest.mark.parametrize("var", (0, 1))
def test_plain_small_vs_oracle(engine, oracle_mod, var):
    """320x240, 5 labels, Gaussian + bilateral, 5 iterations; error also stated against FP64."""
    d, o, cfg = _cfg1_pair(engine, oracle_mod, var)
    Qg = np.array(d.inference(5)).T
    Qo = o.inference(5)
    Q64 = o.inference_f64(5)
    err = np.abs(Qg - Qo).max()
    agree = (Qg.argmax(1) == Qo.argmax(1)).mean()
    err64 = np.abs(Qg - Q64).max()
    print(f"plain_small variant {var}: |Q-oracle| {err:.2e}, argmax {agree:.5f}, |Q-fp64| {err64:.2e}, "
          f"|oracle-fp64| {np.abs(Qo - Q64).max():.2e}")
    assert err < QTOL and agree >= 0.999 and err64 < QTOL
    m = d.map(5)
    assert (m == Qg.argmax(1)).mean() >= 0.9999


@pytest.mark.parametrize("M", (1, 2, 3, 4, 8, 13, 21, 32))
def test_label_counts_vs_oracle(engine, oracle_mod, M):
    rng = np.random.default_rng(M)
    W, H = 45, 31
    N = W * H
    from pydensecrf_gb300 import synthetic as S
    img = S.rect_image(rng, W, H)
    U = S.neg_log_softmax(rng.normal(0, 2, size=(M, N)).astype(np.float32), axis=0)
    mat = S.random_sym_matrix(rng, M, 2.0, True)
    O = oracle_mod
    for compat in (3.0, rng.uniform(-2, 0, M).astype(np.float32), mat):
        d = engine.DenseCRF2D(W, H, M)
        d.setUnaryEnergy(U)
        d.addPairwiseGaussian(3, compat)
        d.addPairwiseBilateral(20, 13, img, compat)
        o = O.OracleCRF(N, M)
        o.set_unary(np.ascontiguousarray(U.T))
        o.add_pairwise(O.features_gaussian_2d(W, H, 3, 3), compat)
        o.add_pairwise(O.features_bilateral_2d(img, 20, 20, 13, 13, 13), compat)
        err = np.abs(np.array(d.inference(6)).T - o.inference(6)).max()
        assert err < QTOL, (M, err)


def test_norm_and_filter_vs_oracle(engine, oracle_mod):
    rng = np.random.default_rng(9)
    N, M, dd = 3000, 6, 4
    f = rng.normal(0, 2, size=(N, dd)).astype(np.float32)
    for nt in range(4):
        d = engine.DenseCRF(N, M)
        d.addPairwiseEnergy(np.ascontiguousarray(f.T), 1.0, engine.DIAG_KERNEL, nt)
        o = oracle_mod.OracleCRF(N, M)
        o.add_pairwise(f, 1.0, 1, nt)
        a, b = d.term_norm(0), o.term_norm(0)
        assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max(), nt
    lat = oracle_mod.Lattice(f, "oracle")
    for vs in (1, M):
        v = rng.random((vs, N)).astype(np.float32)
        for rev in (False, True):
            got = d.lattice_filter(0, v, rev)
            want = lat.compute(np.ascontiguousarray(v.T), rev).T
            assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max(), (vs, rev)


def test_no_unary_paths(engine, oracle_mod):
    rng = np.random.default_rng(4)
    N, M = 500, 3
    f = rng.normal(0, 1, size=(N, 2)).astype(np.float32)
    d = engine.DenseCRF(N, M)
    d.addPairwiseEnergy(np.ascontiguousarray(f.T), 2.0)
    Q, _, _ = d.startInference()
    assert np.all(np.array(Q) == 0)  # densecrf.cpp:179-184
    o = oracle_mod.OracleCRF(N, M)
    o.add_pairwise(f, 2.0)
    assert np.abs(np.array(d.inference(3)).T - o.inference(3)).max() < QTOL


# ---- the reference's own tests (pydensecrf/tests/test_dcrf.py) -------------
def _simple_unary():
    u1 = np.zeros((10, 10), dtype=np.float32)
    u1[:, [0, -1]] = u1[[0, -1], :] = 1
    u2 = np.zeros((10, 10), dtype=np.float32)
    u2[4:7, 4:7] = 1
    u = np.vstack([u1.flat, u2.flat])
    return (u + 1) / (np.sum(u, axis=0) + 2)


def _simple_img():
    img = np.zeros((10, 10, 3), dtype=np.uint8)
    img[2:8, 2:8, :] = 255
    return img


def test_call_dcrf2d(engine):
    d = engine.DenseCRF2D(10, 10, 2)
    d.setUnaryEnergy(-np.log(_simple_unary()))
    d.addPairwiseBilateral(sxy=2, srgb=2, rgbim=_simple_img(), compat=3)
    np.argmax(d.inference(10), axis=0).reshape(10, 10)


def test_call_dcrf(engine):
    from pydensecrf_gb300 import utils
    d = engine.DenseCRF(100, 2)
    d.setUnaryEnergy(-np.log(_simple_unary()))
    feats = utils.create_pairwise_bilateral(sdims=(2, 2), schan=2, img=_simple_img(), chdim=2)
    d.addPairwiseEnergy(feats, compat=3)
    np.argmax(d.inference(10), axis=0).reshape(10, 10)


def test_call_dcrf_eq_dcrf2d(engine):
    from pydensecrf_gb300 import utils
    d = engine.DenseCRF(100, 2)
    d2 = engine.DenseCRF2D(10, 10, 2)
    d.setUnaryEnergy(-np.log(_simple_unary()))
    d2.setUnaryEnergy(-np.log(_simple_unary()))
    d.addPairwiseEnergy(utils.create_pairwise_bilateral(sdims=(2, 2), schan=2, img=_simple_img(), chdim=2), compat=3)
    d2.addPairwiseBilateral(sxy=2, srgb=2, rgbim=_simple_img(), compat=3)
    r1 = np.argmax(d.inference(10), axis=0).reshape(10, 10)
    r2 = np.argmax(d2.inference(10), axis=0).reshape(10, 10)
    assert np.all(r1 == r2)


def test_compact_wrong(engine):
    d = engine.DenseCRF2D(10, 10, 2)
    d.setUnaryEnergy(np.ones((2, 10 * 10), dtype=np.float32))
    with pytest.raises(ValueError):
        d.addPairwiseBilateral(sxy=(3, 3), srgb=(3, 3, 3), rgbim=np.zeros((10, 10, 3), np.uint8),
                               compat=np.array([1.0, 2.0]))
        d.inference(2)


def test_shape_errors(engine):
    d = engine.DenseCRF2D(10, 10, 2)
    with pytest.raises(ValueError):
        d.setUnaryEnergy(np.ones((3, 100), np.float32))
    # a unary with the right labels but the wrong pixel count raises at
    # setUnaryEnergy, not later (the reference's tests/issue29.py)
    with pytest.raises(ValueError):
        d.setUnaryEnergy(np.ones((2, 99), np.float32))
    with pytest.raises(ValueError):
        d.addPairwiseEnergy(np.ones((2, 99), np.float32), compat=1.0)
    with pytest.raises(ValueError):
        d.addPairwiseBilateral(2, 2, np.zeros((9, 10, 3), np.uint8), 1.0)
    with pytest.raises(ValueError):
        d.addPairwiseBilateral(2, 2, np.zeros((10, 10, 4), np.uint8), 1.0)
    with pytest.raises(TypeError):
        d.addPairwiseEnergy(None, compat=1.0)
    with pytest.raises(ValueError):
        engine.DenseCRF(100, 5000)  # more labels than the engine supports (4096) is an explicit error
