"""Batched handles (one lattice per image, every launch over all images)
against one handle per image.  Each image's lattice, splat order and blur
arithmetic are those of its own handle, so results agree exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _images(rng, sizes):
    out = []
    for w, h in sizes:
        img = rng.integers(0, 256, size=(h, w, 3)).astype(np.uint8)
        img[h // 4:h // 2, w // 4:w // 2] = rng.integers(0, 256, size=3)
        out.append(img)
    return out


def _unaries(rng, M, ns):
    out = []
    for n in ns:
        logits = rng.normal(0, 2, size=(M, n)).astype(np.float32)
        p = np.exp(logits - logits.max(0))
        out.append((-np.log(p / p.sum(0))).astype(np.float32))
    return out


SIZES_2D = [(37, 21), (64, 48), (16, 16), (101, 7), (13, 29)]  # ragged edges, N % 4 != 0


@pytest.mark.parametrize("variant", [0, 1])
def test_batch_2d_matches_per_image(engine, variant):
    from pydensecrf_gb300.batch import DenseCRF2DBatch

    rng = np.random.default_rng(11)
    M, T = 5, 4
    imgs = _images(rng, SIZES_2D)
    Us = _unaries(rng, M, [w * h for w, h in SIZES_2D])
    mat = rng.uniform(0, 2, size=(M, M)).astype(np.float32)
    mat = (mat + mat.T) / 2
    np.fill_diagonal(mat, 0)
    bt = DenseCRF2DBatch([w for w, _ in SIZES_2D], [h for _, h in SIZES_2D], M)
    bt.set_variant(variant)
    bt.setUnaryEnergy(Us)
    bt.addPairwiseGaussian(sxy=3, compat=3)
    bt.addPairwiseBilateral(sxy=20, srgb=13, rgbims=imgs, compat=mat)
    Qb = bt.inference(T)
    labels = bt.map(T)
    for b, (w, h) in enumerate(SIZES_2D):
        d = engine.DenseCRF2D(w, h, M)
        d.set_variant(variant)
        d.setUnaryEnergy(Us[b])
        d.addPairwiseGaussian(sxy=3, compat=3)
        d.addPairwiseBilateral(sxy=20, srgb=13, rgbim=imgs[b], compat=mat)
        Q = np.array(d.inference(T))
        assert np.array_equal(Qb[b], Q), (b, np.abs(Qb[b] - Q).max())
        assert np.array_equal(labels[b], d.map(T)), b


def test_batch_generic_matches_per_image(engine):
    from pydensecrf_gb300.batch import DenseCRFBatch

    rng = np.random.default_rng(12)
    M, T = 4, 3
    ns = [300, 1000, 77, 513]
    feats = [rng.normal(0, 2, size=(3, n)).astype(np.float32) for n in ns]
    Us = _unaries(rng, M, ns)
    bt = DenseCRFBatch(ns, M)
    bt.setUnaryEnergy(Us)
    bt.addPairwiseEnergy(feats, compat=np.float32([1.0, 2.0, 0.5, 1.5]), kernel=2, normalization=1)
    Qb = bt.inference(T)
    kl = bt.klDivergence(Qb)
    kls = 0.0
    for b, n in enumerate(ns):
        d = engine.DenseCRF(n, M)
        d.setUnaryEnergy(Us[b])
        d.addPairwiseEnergy(feats[b], compat=np.float32([1.0, 2.0, 0.5, 1.5]), kernel=2, normalization=1)
        Q = np.array(d.inference(T))
        assert np.array_equal(Qb[b], Q), (b, np.abs(Qb[b] - Q).max())
        kls += d.klDivergence(Q)
    assert abs(kl - kls) <= 1e-6 * max(1.0, abs(kls)), (kl, kls)


def test_batch_backward_matches_per_image(engine):
    from pydensecrf_gb300.batch import DenseCRF2DBatch

    rng = np.random.default_rng(13)
    M, T = 3, 3
    sizes = [(24, 17), (40, 12)]
    imgs = _images(rng, sizes)
    Us = _unaries(rng, M, [w * h for w, h in sizes])
    wts = [rng.normal(0, 1, size=(M, w * h)).astype(np.float32) for w, h in sizes]
    bt = DenseCRF2DBatch([w for w, _ in sizes], [h for _, h in sizes], M)
    bt.setUnaryEnergy(Us)
    bt.addPairwiseGaussian(sxy=3, compat=3)
    bt.addPairwiseBilateral(sxy=10, srgb=20, rgbims=imgs, compat=5)
    bt.inferenceCheckpointed(T)
    dUb, dcb, dkb = bt.backward(wts, want_compat=True, want_kernel=True)
    dc_sum = [np.zeros_like(x) for x in dcb]
    dk_sum = [np.zeros_like(x) for x in dkb]
    for b, (w, h) in enumerate(sizes):
        d = engine.DenseCRF2D(w, h, M)
        d.setUnaryEnergy(Us[b])
        d.addPairwiseGaussian(sxy=3, compat=3)
        d.addPairwiseBilateral(sxy=10, srgb=20, rgbim=imgs[b], compat=5)
        d.inferenceCheckpointed(T)
        dU, dc, dk = d.backward(wts[b], want_compat=True, want_kernel=True)
        assert np.array_equal(dUb[b], dU), (b, np.abs(dUb[b] - dU).max())
        for k in range(len(dc)):
            dc_sum[k] += dc[k]
            dk_sum[k] += dk[k]
    for k in range(len(dcb)):
        assert np.allclose(dcb[k], dc_sum[k], rtol=1e-5, atol=1e-9), (k, dcb[k], dc_sum[k])
        assert np.allclose(dkb[k], dk_sum[k], rtol=1e-4, atol=1e-7), (k, dkb[k], dk_sum[k])


def test_batch_shape_errors(engine):
    from pydensecrf_gb300.batch import DenseCRF2DBatch

    bt = DenseCRF2DBatch([8, 9], [4, 5], 3)
    with pytest.raises(ValueError):
        bt.setUnaryEnergy([np.zeros((3, 32), np.float32)])
    with pytest.raises(ValueError):
        bt.setUnaryEnergy([np.zeros((3, 32), np.float32), np.zeros((3, 44), np.float32)])
    with pytest.raises(ValueError):
        bt.addPairwiseBilateral(sxy=3, srgb=3, rgbims=[np.zeros((4, 8, 3), np.uint8)] * 2, compat=1)


def test_autotune_choices_and_results(engine):
    """The autotuner's knobs are in range, a handle given the same knobs
    reproduces the tuned handle exactly, and results stay within 1e-5 of the
    default knobs (only the splat task length regroups sums)."""
    rng = np.random.default_rng(14)
    W, H, M, T = 96, 80, 8, 4
    img = _images(rng, [(W, H)])[0]
    U = _unaries(rng, M, [W * H])[0]

    def make():
        d = engine.DenseCRF2D(W, H, M)
        d.setUnaryEnergy(U)
        d.addPairwiseGaussian(sxy=3, compat=3)
        d.addPairwiseBilateral(sxy=30, srgb=13, rgbim=img, compat=5)
        return d

    ref = np.array(make().inference(T))
    tuned = make()
    knobs = tuned.autotune()
    assert knobs["split"] in (1, 2) and 8 <= knobs["task_len"] <= 32 and knobs["hash_load"] >= 1.5
    assert knobs["smem_kb"] > 0 and knobs["coop_blur"] in (0, 1)
    Qt = np.array(tuned.inference(T))
    same = make()
    same.set_tuning(knobs["split"], knobs["smem_kb"], knobs["task_len"], knobs["hash_load"], knobs["coop_blur"])
    assert np.array_equal(np.array(same.inference(T)), Qt)
    assert np.abs(Qt - ref).max() < 1e-5
    # automatic mode takes the remembered choice for the same configuration
    auto = make()
    auto.set_autotune(True)
    Qa = np.array(auto.inference(T))
    assert auto.tuning() == knobs
    assert np.array_equal(Qa, Qt)


def test_volume_batch_fwd_bwd_matches_per_volume(engine):
    """Generic batch of small volumes with 4-d features (x, y, z, intensity), a
    FULL kernel term and a DIAG Gaussian term, Matrix compatibility: forward and
    adjoint per volume equal separate handles."""
    from pydensecrf_gb300.batch import DenseCRFBatch

    rng = np.random.default_rng(15)
    M, T, S = 4, 3, 10
    ns = [S * S * S, (S - 2) ** 3]
    feats4, feats3, Us, wts = [], [], [], []
    for n in ns:
        s = round(n ** (1 / 3))
        z, y, x = np.mgrid[0:s, 0:s, 0:s].astype(np.float32)
        inten = rng.normal(0, 0.05, size=(s, s, s)).astype(np.float32) + (x > s / 2)
        feats4.append(np.ascontiguousarray(np.stack([x / 5, y / 5, z / 5, inten / np.float32(0.1)]).reshape(4, -1),
                                           np.float32))
        feats3.append(np.ascontiguousarray(np.stack([x / 3, y / 3, z / 3]).reshape(3, -1), np.float32))
        Us.extend(_unaries(rng, M, [n]))
        wts.append(rng.normal(0, 1, size=(M, n)).astype(np.float32))
    mat = rng.uniform(0, 1, size=(M, M)).astype(np.float32)
    mat = (mat + mat.T) / 2
    bt = DenseCRFBatch(ns, M)
    bt.setUnaryEnergy(Us)
    bt.addPairwiseEnergy(feats4, compat=mat, kernel=2)
    bt.addPairwiseEnergy(feats3, compat=2.0, kernel=1)
    Qb = bt.inferenceCheckpointed(T)
    dUb, dcb, dkb = bt.backward(wts, want_compat=True, want_kernel=True)
    dk_sum = [np.zeros_like(x) for x in dkb]
    for b, n in enumerate(ns):
        d = engine.DenseCRF(n, M)
        d.setUnaryEnergy(Us[b])
        d.addPairwiseEnergy(feats4[b], compat=mat, kernel=2)
        d.addPairwiseEnergy(feats3[b], compat=2.0, kernel=1)
        assert np.array_equal(d.inferenceCheckpointed(T), Qb[b])
        dU, dc, dk = d.backward(wts[b], want_compat=True, want_kernel=True)
        assert np.array_equal(dU, dUb[b])
        for k in range(len(dk)):
            dk_sum[k] += dk[k]
    for k in range(len(dkb)):
        assert np.allclose(dkb[k], dk_sum[k], rtol=1e-4, atol=1e-7), (k, dkb[k], dk_sum[k])


def test_two_axis_blur_launches_match_pass_by_pass(engine):
    """The launched blur runs two axes per launch (the first recomputed at the
    second's neighbours); the cooperative blur runs one axis per grid-barrier
    step through a buffer.  Same arithmetic: marginals and gradients agree bit
    for bit."""
    rng = np.random.default_rng(16)
    W, H, M, T = 48, 40, 6, 4
    img = _images(rng, [(W, H)])[0]
    U = _unaries(rng, M, [W * H])[0]
    dQ = rng.normal(0, 1, size=(M, W * H)).astype(np.float32)

    def run(coop):
        d = engine.DenseCRF2D(W, H, M)
        d.set_tuning(2 if M % 8 == 0 else 1, 0, 24, 2.0, coop)
        d.setUnaryEnergy(U)
        d.addPairwiseGaussian(sxy=3, compat=3)
        d.addPairwiseBilateral(sxy=30, srgb=13, rgbim=img, compat=np.float32(np.eye(M) + 1))
        Q = np.array(d.inferenceCheckpointed(T))
        dU, dc, dk = d.backward(dQ, want_compat=True, want_kernel=True)
        return Q, dU, dc, dk

    Qa, dUa, dca, dka = run(0)
    Qb, dUb, dcb, dkb = run(1)
    assert np.array_equal(Qa, Qb)
    assert np.array_equal(dUa, dUb)
    for x, y in zip(dca + dka, dcb + dkb):
        if x is not None:
            assert np.array_equal(x, y)
