"""The logistic unary (setUnaryEnergy(L, f) and setUnary(LogisticUnary(L, f)),
densecrf.pyx:44-46,77-89 -> unary.cpp:48-52: U = L f) on the device: the
marginals must match those of a CRF given the same U as a constant unary,
computed in float64 and rounded (the product itself is a float32 GEMM, so the
bar is 1e-4 on Q, the inference tolerance)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_logistic_unary_matches_constant(engine):
    rng = np.random.default_rng(61)
    N, M, K = 500, 4, 7
    L = rng.normal(0, 1, (M, K)).astype(np.float32)
    f = rng.normal(0, 1, (K, N)).astype(np.float32)
    feat = rng.normal(0, 1.5, (3, N)).astype(np.float32)
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
    assert np.abs(q_obj - q_lf).max() < 1e-6
