"""The parameter API (the reference's DenseCRF / LabelCompatibility /
DenseKernel parameter setters, densecrf.cpp:298-360, pairwise.cpp:129-151,
labelcompatibility.cpp): nTerms, paramCounts, setCompatibility and
setKernelParameters (a DIAG kernel's per-feature scales p, features p_j f_j,
lattice rebuilt).  A CRF whose parameters were changed in place must solve
like a fresh CRF built with those parameters from the start."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
