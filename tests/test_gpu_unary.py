"""The logistic unary (setUnaryEnergy(L, f) and setUnary(LogisticUnary(L, f)),
densecrf.pyx:44-46,77-89 -> unary.cpp:48-68: U = L f) on the device, its
parameter vector (densecrf.cpp:298-306) and its gradient b f^T
(unary.cpp:64-67).

* Marginals against the oracle solved with U = L f computed in float64 and
  rounded (the device sums each label's products in float with fused
  multiply-adds, so the bar is the inference tolerance, 1e-4 on Q).
* The parameter gradient equals (dL/dU) f^T of the backward's own dL/dU
  (1e-5 relative) and central differences of the FP64 oracle in L (1e-3 of the
  largest magnitude, the gradient tests' bar)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(seed, N=500, M=4, K=7):
    rng = np.random.default_rng(seed)
    L = rng.normal(0, 1, (M, K)).astype(np.float32)
    f = rng.normal(0, 1, (K, N)).astype(np.float32)
    feat = rng.normal(0, 1.5, (3, N)).astype(np.float32)
    return rng, L, f, feat


def test_logistic_unary_matches_constant_and_oracle(engine, oracle_mod):
    rng, L, f, feat = _case(61)
    N, M = f.shape[1], L.shape[0]
    U = (L.astype(np.float64) @ f.astype(np.float64)).astype(np.float32)

    def solve(set_unary):
        d = engine.DenseCRF(N, M)
        set_unary(d)
        d.addPairwiseEnergy(feat, compat=2.0)
        return np.array(d.inference(4))

    q_const = solve(lambda d: d.setUnaryEnergy(U))
    q_lf = solve(lambda d: d.setUnaryEnergy(L, f))
    q_obj = solve(lambda d: d.setUnary(engine.LogisticUnary(L, f)))
    assert np.abs(q_lf - q_const).max() < 1e-4
    assert np.abs(q_obj - q_lf).max() == 0.0
    o = oracle_mod.OracleCRF(N, M)
    o.set_unary(np.ascontiguousarray(U.T))
    o.add_pairwise(np.ascontiguousarray(feat.T), 2.0)
    assert np.abs(q_lf.T - o.inference(4)).max() < 1e-4


def test_logistic_parameters_roundtrip(engine):
    rng, L, f, feat = _case(62, M=5, K=3)
    N, M = f.shape[1], L.shape[0]
    d = engine.DenseCRF(N, M)
    assert d.unaryParameters().size == 0  # no unary yet / constant unary: none (unary.cpp:32-34)
    d.setUnaryEnergy(L, f)
    d.addPairwiseEnergy(feat, compat=1.5)
    v = d.unaryParameters()
    assert np.array_equal(v, L.reshape(-1, order="F"))  # column-major, as Eigen's resize
    L2 = rng.normal(0, 1, L.shape).astype(np.float32)
    d.setUnaryParameters(L2.reshape(-1, order="F"))
    assert np.array_equal(d.unaryParameters(), L2.reshape(-1, order="F"))
    e = engine.DenseCRF(N, M)
    e.setUnary(engine.LogisticUnary(L2, f))
    e.addPairwiseEnergy(feat, compat=1.5)
    assert np.abs(np.array(d.inference(3)) - np.array(e.inference(3))).max() == 0.0
    with pytest.raises(ValueError):
        d.setUnaryParameters(np.ones(3, np.float32))


def test_logistic_parameter_gradient(engine, oracle_mod):
    rng, L, f, feat = _case(63, N=400, M=3, K=4)
    N, M = f.shape[1], L.shape[0]
    T = 3
    wt = rng.normal(0, 1, (M, N))
    d = engine.DenseCRF(N, M)
    d.setUnaryEnergy(L, f)
    d.addPairwiseEnergy(feat, compat=2.0)
    d.inferenceCheckpointed(T)
    dU, _, _ = d.backward(wt.astype(np.float32), want_compat=False)
    g = d.unaryParameterGradient()
    want = (dU.astype(np.float64) @ f.astype(np.float64).T).reshape(-1, order="F")
    assert np.abs(g - want).max() <= 1e-5 * np.abs(want).max()

    def loss(Lv):
        U = (Lv.astype(np.float64) @ f.astype(np.float64)).astype(np.float32)
        o = oracle_mod.OracleCRF(N, M)
        o.set_unary(np.ascontiguousarray(U.T))
        o.add_pairwise(np.ascontiguousarray(feat.T), 2.0)
        return float((o.inference_f64(T) * wt.T).sum())

    h = 2.0 ** -8
    fd = []
    for j in range(L.shape[1]):
        for m in range(M):
            up, dn = L.copy(), L.copy()
            up[m, j] += np.float32(h)
            dn[m, j] -= np.float32(h)
            fd.append((loss(up) - loss(dn)) / (2 * h))
    fd = np.array(fd)  # column-major order, as the parameter vector
    assert np.abs(g - fd).max() <= 1e-3 * np.abs(fd).max(), (g, fd)
