"""The parameter API: the reference's flattened parameter vectors
(DenseCRF::labelCompatibilityParameters / kernelParameters and their setters,
densecrf.cpp:307-360; LabelCompatibility::parameters, labelcompatibility.cpp:
50-100; DenseKernel::parameters / setParameters, pairwise.cpp:129-151) and the
per-term setters.  A CRF whose parameters were changed through them must solve
like the oracle built with those parameters from the start (features scaled as
the kernel parameters say, compatibilities as set): Q within 1e-4."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _full_transform(P, f):
    """P f for a FULL kernel, each output summed over k in order with separately
    rounded float products and sums (the device's feature transform)."""
    d, N = f.shape
    out = np.zeros((d, N), np.float32)
    for j in range(d):
        s = np.zeros(N, np.float32)
        for k in range(d):
            s = (s + (np.float32(P[j, k]) * f[k]).astype(np.float32)).astype(np.float32)
        out[j] = s
    return out


def test_parameters_set_in_place_match_a_fresh_crf(engine):
    rng = np.random.default_rng(62)
    N, M = 600, 4
    U = rng.uniform(0.1, 3.0, (M, N)).astype(np.float32)
    f = rng.normal(0, 1.5, (3, N)).astype(np.float32)
    g = np.ascontiguousarray(f[:2])
    d = engine.DenseCRF(N, M)
    d.setUnaryEnergy(U)
    d.addPairwiseEnergy(f, compat=2.0)
    d.addPairwiseEnergy(g, compat=np.eye(M, dtype=np.float32), kernel=engine.FULL_KERNEL)
    assert d.nTerms() == 2
    assert d.paramCounts(0) == (1, 3)          # Potts weight; DIAG: one scale per feature
    assert d.paramCounts(1) == (M * M, 2 * 2)  # Matrix M x M; FULL: d x d
    mat = rng.uniform(0, 1, (M, M)).astype(np.float32)
    p = np.array([0.5, 2.0, 1.25], np.float32)
    d.setCompatibility(0, 3.5)
    d.setCompatibility(1, mat)
    d.setKernelParameters(0, p)
    q = np.array(d.inference(4))

    e = engine.DenseCRF(N, M)
    e.setUnaryEnergy(U)
    e.addPairwiseEnergy(np.ascontiguousarray(f * p[:, None]), compat=3.5)
    e.addPairwiseEnergy(g, compat=mat, kernel=engine.FULL_KERNEL)
    assert np.abs(q - np.array(e.inference(4))).max() < 1e-5


def test_flattened_parameter_vectors_vs_oracle(engine, oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(64)
    N, M, T = 900, 5, 4
    U = rng.uniform(0.1, 3.0, (M, N)).astype(np.float32)
    fa = rng.normal(0, 1.5, (3, N)).astype(np.float32)
    fb = rng.normal(0, 1.0, (2, N)).astype(np.float32)
    fc = rng.normal(0, 2.0, (2, N)).astype(np.float32)
    diag = rng.uniform(-2, 0, M).astype(np.float32)
    mat = rng.uniform(0, 1, (M, M)).astype(np.float32)
    d = engine.DenseCRF(N, M)
    d.setUnaryEnergy(U)
    d.addPairwiseEnergy(fa, compat=2.0, kernel=engine.DIAG_KERNEL)
    d.addPairwiseEnergy(fb, compat=diag, kernel=engine.CONST_KERNEL)
    d.addPairwiseEnergy(fc, compat=mat, kernel=engine.FULL_KERNEL)
    # the vectors as the reference lays them out
    sym = 0.5 * (mat + mat.T)
    packed = [sym[i, j] for i in range(M) for j in range(i, M)]
    want_c = np.concatenate([[2.0], diag, packed]).astype(np.float32)
    assert np.array_equal(d.labelCompatibilityParameters(), want_c)
    assert np.array_equal(d.kernelParameters(), np.array([1, 1, 1, 1, 0, 0, 1], np.float32))
    # new values through the flattened setters
    new_diag = rng.uniform(-3, 0, M).astype(np.float32)
    new_sym = rng.uniform(0, 2, (M, M)).astype(np.float32)
    new_sym = (0.5 * (new_sym + new_sym.T)).astype(np.float32)
    new_c = np.concatenate([[3.25], new_diag, [new_sym[i, j] for i in range(M) for j in range(i, M)]])
    d.setLabelCompatibilityParameters(new_c.astype(np.float32))
    assert np.array_equal(d.labelCompatibilityParameters(), new_c.astype(np.float32))
    pa = np.array([0.75, 1.5, 0.5], np.float32)
    P = np.array([[1.0, 0.25], [-0.5, 1.5]], np.float32)
    d.setKernelParameters(np.concatenate([pa, P.reshape(-1, order="F")]))
    assert np.array_equal(d.kernelParameters(), np.concatenate([pa, P.reshape(-1, order="F")]))
    q = np.array(d.inference(T)).T

    o = O.OracleCRF(N, M)
    o.set_unary(np.ascontiguousarray(U.T))
    o.add_pairwise(np.ascontiguousarray((fa * pa[:, None]).astype(np.float32).T), 3.25, 1)
    o.add_pairwise(np.ascontiguousarray(fb.T), new_diag, 0)
    o.add_pairwise(np.ascontiguousarray(_full_transform(P, fc).T), new_sym, 2)
    qo = o.inference(T)
    assert np.abs(q - qo).max() < 1e-4, np.abs(q - qo).max()
    with pytest.raises(ValueError):
        d.setLabelCompatibilityParameters(np.ones(3, np.float32))
    with pytest.raises(ValueError):
        d.setKernelParameters(np.ones(2, np.float32))
