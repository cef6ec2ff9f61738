"""More than 32 labels (DenseCRF(N, M) takes any M, densecrf.cpp:39-40;
sseCompute filters any value size, permutohedral.cpp:529-589): the engine
splits the labels into chunks of 32, filters chunk by chunk and takes the
messages, compatibilities and softmax over all labels in one pass.  Checked
against the oracle on the same seeded inputs: Q max-abs <= 1e-4, argmax
agreement >= 99.9 %, klDivergence relative 1e-5, for Potts, Diagonal and
Matrix compatibilities, both lattice variants, start/stepInference, MAP, the
unary energy and a batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
QTOL = 1e-4


def _problem(seed, W, H, M):
    rng = np.random.default_rng(seed)
    N = W * H
    logits = rng.normal(0, 2, size=(N, M)).astype(np.float32)
    U = (-(logits - logits.max(1, keepdims=True)) + np.log(np.exp(logits - logits.max(1, keepdims=True)).sum(
        1, keepdims=True))).astype(np.float32)  # (N, M) = -log softmax
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    img[H // 4:H // 2, W // 3:2 * W // 3] = [30, 200, 90]
    diag = rng.uniform(-3, 0, size=M).astype(np.float32)
    mat = rng.uniform(0, 2, size=(M, M)).astype(np.float32)
    return rng, N, U, img, diag, mat


def _pair(engine, O, W, H, M, U, img, compat, variant=0, ntype=3):
    N = W * H
    fg = O.features_gaussian_2d(W, H, 3, 3)
    fb = O.features_bilateral_2d(img, 8, 8, 13, 13, 13)
    d = engine.DenseCRF2D(W, H, M)
    d.set_variant(variant)
    d.setUnaryEnergy(np.ascontiguousarray(U.T))
    d.addPairwiseGaussian(3, compat, engine.DIAG_KERNEL, ntype)
    d.addPairwiseBilateral(8, 13, img, 5.0)
    o = O.OracleCRF(N, M, variant)
    o.set_unary(U)
    o.add_pairwise(fg, compat, 1, ntype)
    o.add_pairwise(fb, 5.0)
    return d, o


def _kl_f64(O, Q, U, img, W, H, compat):
    """DenseCRF::klDivergence (densecrf.cpp:214-235) of Q (N, M) for the two
    terms of _pair (symmetric normalisation), accumulated in float64 over the
    oracle's float filter outputs."""
    N = W * H
    Qd = Q.astype(np.float64)
    kl = (Qd * np.log(np.maximum(Qd, 1e-20))).sum() + (U.astype(np.float64) * Qd).sum()
    for f, c in ((O.features_gaussian_2d(W, H, 3, 3), compat), (O.features_bilateral_2d(img, 8, 8, 13, 13, 13), 5.0)):
        lat = O.Lattice(f, "oracle")
        n = lat.compute(np.ones((N, 1), np.float32))[:, 0]
        nrm = (1.0 / np.sqrt(n.astype(np.float64) + 1e-20)).astype(np.float32)[:, None]
        KQ = lat.compute((Q * nrm).astype(np.float32)) * nrm
        if np.ndim(c) == 0:
            msg = -float(c) * KQ
        elif np.ndim(c) == 1:
            msg = KQ * c[None, :]
        else:
            msg = KQ @ (0.5 * (c + c.T)).T
        kl += (Qd * msg.astype(np.float64)).sum()
    return kl


@pytest.mark.parametrize("M", [33, 40, 64, 100])
@pytest.mark.parametrize("ck", ["potts", "diag", "mat"])
def test_wide_inference_vs_oracle(engine, oracle_mod, M, ck):
    W, H, T = 40, 30, 5
    rng, N, U, img, diag, mat = _problem(M, W, H, M)
    compat = {"potts": 3.0, "diag": diag, "mat": mat}[ck]
    d, o = _pair(engine, oracle_mod, W, H, M, U, img, compat)
    Q = np.array(d.inference(T)).T
    Qo = o.inference(T)
    assert np.abs(Q - Qo).max() <= QTOL, (M, ck, np.abs(Q - Qo).max())
    assert (Q.argmax(1) == Qo.argmax(1)).mean() >= 0.999
    # klDivergence of the oracle's marginals.  The reference (and the oracle)
    # add the pairwise part in float over N*M terms, which at these label counts
    # is ~1e-5 relative from the exact sum; the device adds in double.  So the
    # device is held to 1e-6 of the same sum accumulated in float64 from the
    # oracle's own filter outputs, and to 1e-4 of the reference's float sum.
    kl = d.klDivergence(engine.MatrixXf().wrap_colmajor(np.ascontiguousarray(Qo)))
    kl64 = _kl_f64(oracle_mod, Qo, U, img, W, H, compat)
    assert abs(kl - kl64) <= 1e-6 * abs(kl64), (M, ck, kl, kl64)
    kl_ref = o.kl(Qo)
    assert abs(kl - kl_ref) <= 1e-4 * max(1.0, abs(kl_ref)), (M, ck, kl, kl_ref)


@pytest.mark.parametrize("variant", [0, 1], ids=["sse", "scalar"])
def test_wide_variants_start_step_map_energy(engine, oracle_mod, variant):
    W, H, M, T = 64, 48, 72, 4
    rng, N, U, img, diag, mat = _problem(5, W, H, M)
    d, o = _pair(engine, oracle_mod, W, H, M, U, img, mat, variant, ntype=1)
    Q = np.array(d.inference(T)).T
    assert np.abs(Q - o.inference(T)).max() <= QTOL
    Qs, t1, t2 = d.startInference()
    Q0 = o.start()
    assert np.abs(np.array(Qs).T - Q0).max() < 1e-6
    d.stepInference(Qs, t1, t2)
    o.step(Q0)
    assert np.abs(np.array(Qs).T - Q0).max() <= QTOL
    labels = d.map(T)
    want = o.map(T)
    assert (np.asarray(labels) == want).mean() >= 0.999
    lab = rng.integers(-1, M + 1, size=N).astype(np.int16)
    e = d.unaryEnergy(lab)
    ok = (lab >= 0) & (lab < M)
    want_e = np.where(ok, U[np.arange(N), np.clip(lab, 0, M - 1)], 0.0)
    assert np.abs(e - want_e).max() <= 1e-6 * np.abs(want_e).max()


def test_wide_larger_image_and_batch(engine, oracle_mod):
    from pydensecrf_gb300.batch import DenseCRF2DBatch

    O = oracle_mod
    M, T = 150, 3
    sizes = [(160, 120), (57, 91)]
    probs = [_problem(20 + b, W, H, M) for b, (W, H) in enumerate(sizes)]
    mat = probs[0][5]
    b = DenseCRF2DBatch([w for w, _ in sizes], [h for _, h in sizes], M)
    b.setUnaryEnergy([np.ascontiguousarray(p[2].T) for p in probs])
    b.addPairwiseGaussian(3, 3.0)
    b.addPairwiseBilateral(8, 13, [p[3] for p in probs], mat)
    Qs = b.inference(T)
    for (W, H), p, Q in zip(sizes, probs, Qs):
        o = O.OracleCRF(W * H, M)
        o.set_unary(p[2])
        o.add_pairwise(O.features_gaussian_2d(W, H, 3, 3), 3.0)
        o.add_pairwise(O.features_bilateral_2d(p[3], 8, 8, 13, 13, 13), mat)
        Qo = o.inference(T)
        err = np.abs(np.asarray(Q).T - Qo).max()
        assert err <= QTOL, (W, H, err)
        assert (np.asarray(Q).T.argmax(1) == Qo.argmax(1)).mean() >= 0.999


def test_wide_unsupported_calls_are_errors(engine):
    """The adjoint keeps the 32-label limit, as an explicit error."""
    d = engine.DenseCRF2D(16, 12, 40)
    d.setUnaryEnergy(np.ones((40, 16 * 12), np.float32))
    d.addPairwiseGaussian(3, 3.0)
    with pytest.raises(ValueError):
        d.inferenceCheckpointed(2)
    out = d.lattice_filter(0, np.ones((1, 16 * 12), np.float32), False)
    assert np.isfinite(out).all()


@pytest.mark.parametrize("M", [40, 70])
def test_wide_lattice_filter_vs_oracle(engine, oracle_mod, M):
    """The raw filter (Permutohedral::compute, permutohedral.cpp:596-604) with
    value size M above 32, both directions, on both terms: label chunks of 32
    (70 labels: 32 + 32 + a ragged 6 padded to 8) against the oracle's filter of
    the whole rows, within 1e-6 of the output's magnitude like the narrow
    filter tests; value size 1 on the same handle afterwards."""
    rng, N, U, img, diag, mat = _problem(61 + M, 29, 21, M)
    d = engine.DenseCRF2D(29, 21, M)
    d.setUnaryEnergy(np.ascontiguousarray(U.T))
    d.addPairwiseGaussian(3, 3.0)
    d.addPairwiseBilateral(8, 13, img, 5.0)
    lats = [oracle_mod.Lattice(oracle_mod.features_gaussian_2d(29, 21, 3, 3), "oracle"),
            oracle_mod.Lattice(oracle_mod.features_bilateral_2d(img, 8, 8, 13, 13, 13), "oracle")]
    for term in (0, 1):
        for reverse in (False, True):
            for vs in (M, 1):
                v = rng.random((vs, N)).astype(np.float32)
                got = d.lattice_filter(term, v, reverse)
                want = lats[term].compute(np.ascontiguousarray(v.T), reverse).T
                err = np.abs(got - want).max()
                assert err <= 1e-6 * np.abs(want).max(), (term, reverse, vs, err)


def test_wide_logistic_unary_with_matrix_keeps_parameters(engine, oracle_mod):
    """A logistic unary (unary.cpp:48-68) on a handle of 40 labels with a Matrix
    term: the first inference sizes the Matrix terms' message rows, and the
    unary's parameters must survive it -- setUnaryParameters afterwards and a
    second inference give the marginals of a fresh handle built with the new
    parameters and of the oracle solved with U = L2 f."""
    rng = np.random.default_rng(83)
    W, H, M, K, T = 23, 17, 40, 6, 3
    N = W * H
    L = rng.normal(0, 1, (M, K)).astype(np.float32)
    L2 = rng.normal(0, 1, (M, K)).astype(np.float32)
    f = rng.normal(0, 1, (K, N)).astype(np.float32)
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    mat = rng.uniform(0, 2, size=(M, M)).astype(np.float32)

    def crf(Lm):
        d = engine.DenseCRF2D(W, H, M)
        d.setUnaryEnergy(Lm, f)
        d.addPairwiseGaussian(3, mat)
        d.addPairwiseBilateral(8, 13, img, 5.0)
        return d

    d = crf(L)
    d.inference(T)
    d.setUnaryParameters(L2.reshape(-1, order="F"))
    assert np.array_equal(d.unaryParameters(), L2.reshape(-1, order="F"))
    q = np.array(d.inference(T))
    q_fresh = np.array(crf(L2).inference(T))
    assert np.abs(q - q_fresh).max() == 0.0
    U2 = (L2.astype(np.float64) @ f.astype(np.float64)).astype(np.float32)
    o = oracle_mod.OracleCRF(N, M)
    o.set_unary(np.ascontiguousarray(U2.T))
    o.add_pairwise(oracle_mod.features_gaussian_2d(W, H, 3, 3), mat)
    o.add_pairwise(oracle_mod.features_bilateral_2d(img, 8, 8, 13, 13, 13), 5.0)
    assert np.abs(q.T - o.inference(T)).max() < QTOL


@pytest.mark.parametrize("ntype", [0, 1, 2, 3])
def test_wide_pairwise_energy_vs_oracle(engine, oracle_mod, ntype):
    """pairwiseEnergy (densecrf.cpp:160-177) at 40 labels, per term and summed
    over a Matrix, a Potts and a Diagonal term, against the one-hot messages of
    the oracle's lattice filter (1e-5 of the largest magnitude, the energy
    tests' bar); labels outside [0, M) give 0."""
    rng = np.random.default_rng(91 + ntype)
    N, M = 900, 40
    feats = [rng.normal(0, s, size=(N, dd)).astype(np.float32) for s, dd in ((1.5, 3), (2.0, 2), (1.0, 4))]
    compats = [rng.uniform(-1, 1, size=(M, M)).astype(np.float32), 2.5, rng.uniform(-2, 0, size=M).astype(np.float32)]
    d = engine.DenseCRF(N, M)
    d.setUnaryEnergy(rng.random((M, N)).astype(np.float32))
    for f, c in zip(feats, compats):
        d.addPairwiseEnergy(np.ascontiguousarray(f.T), c, normalization=ntype)
    lab = rng.integers(-1, M + 1, size=N).astype(np.int16)  # -1 and M: no label
    ok = (lab >= 0) & (lab < M)
    oh = np.zeros((N, M), np.float32)
    oh[np.arange(N)[ok], lab[ok]] = 1.0
    want_terms = []
    for f, c in zip(feats, compats):
        lat = oracle_mod.Lattice(f, "oracle", 0)
        raw1 = lat.compute(np.ones((N, 1), np.float32), False)[:, 0].astype(np.float64)
        if ntype == 0:
            n_pre = n_post = np.ones(N)
        elif ntype == 3:
            n_pre = n_post = 1.0 / np.sqrt(raw1 + 1e-20)
        else:
            n = 1.0 / (raw1 + 1e-20)
            n_pre, n_post = (n, np.ones(N)) if ntype == 1 else (np.ones(N), n)
        kq = lat.compute(np.ascontiguousarray((oh * n_pre[:, None]).astype(np.float32)), False) * n_post[:, None]
        if np.ndim(c) == 0:
            msg = -float(c) * kq
        elif np.ndim(c) == 1:
            msg = kq * c[None, :]
        else:
            msg = kq @ (0.5 * (c + c.T)).T
        want_terms.append(np.where(ok, -0.5 * msg[np.arange(N), np.clip(lab, 0, M - 1)], 0.0))
    for k, want in enumerate(want_terms):
        got = d.pairwiseEnergy(lab, k)
        assert np.abs(got - want).max() <= 1e-5 * max(1.0, np.abs(want).max()), (k, np.abs(got - want).max())
    want = sum(want_terms)
    got = d.pairwiseEnergy(lab)
    assert np.abs(got - want).max() <= 1e-5 * max(1.0, np.abs(want).max()), np.abs(got - want).max()
    assert (got[~ok] == 0).all()
