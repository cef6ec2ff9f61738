"""The debug energies (DenseCRF::unaryEnergy / pairwiseEnergy,
densecrf.cpp:141-177) pinned to the reference's own outputs.

tests/golden/energy.npz holds the reference's energies of a labelling (labels
-1 and M included: they score 0) for every normalisation, Potts / Diagonal /
Matrix compatibilities, DIAG and FULL kernels and a two-term CRF, from both of
its builds.  The restatement below -- the one-hot labelling filtered through
the oracle's lattice with the term's normalisation on either side, the
compatibility applied, -1/2 of the own-label entry -- is the formula the GPU
energy tests hold the device to; here it must reproduce the reference within
1e-5 of the largest magnitude."""
import numpy as np
import pytest

VARIANTS = [("sse", 0), ("scalar", 1)]


def restated_pairwise(O, var, f, compat, ktype, ntype, lab, N, M):
    """-1/2 (C n_post K(n_pre onehot))[l_i, i] for 0 <= l_i < M, else 0."""
    c = O.OracleCRF(N, M, var)
    c.add_pairwise(f, compat, ktype, ntype)
    norm = c.term_norm(0).astype(np.float64)
    ones = np.ones(N)
    n_pre = norm if ntype in (1, 3) else ones
    n_post = norm if ntype in (2, 3) else ones
    ok = (lab >= 0) & (lab < M)
    oh = np.zeros((N, M), np.float32)
    oh[np.arange(N)[ok], lab[ok]] = 1.0
    lat = O.Lattice(f, "oracle", var)
    kq = lat.compute(np.ascontiguousarray((oh * n_pre[:, None]).astype(np.float32)), False) * n_post[:, None]
    if np.isscalar(compat):
        msg = -float(compat) * kq
    elif np.ndim(compat) == 1:
        msg = kq * compat[None, :]
    else:
        msg = kq @ (0.5 * (compat + compat.T)).T
    return np.where(ok, -0.5 * msg[np.arange(N), np.clip(lab, 0, M - 1)], 0.0)


@pytest.mark.parametrize("vname,var", VARIANTS)
def test_energies_match_reference(oracle_mod, golden, vname, var):
    g = golden("energy.npz")
    O = oracle_mod
    U, lab = g["U"], g["lab"]
    N, M = U.shape
    cases = {f"mat_n{nt}": [("f", "mat", 1, nt)] for nt in range(4)}
    cases["potts_n3"] = [("f", 2.5, 1, 3)]
    cases["diag_n1"] = [("f", "diag", 1, 1)]
    cases["full_n3"] = [("f", "mat", 2, 3)]
    cases["two_terms"] = [("f", 2.0, 1, 3), ("f2", "mat", 1, 2)]
    assert sorted(map(str, g["cases"])) == sorted(cases)
    ok = (lab >= 0) & (lab < M)
    want_u = np.where(ok, U[np.arange(N), np.clip(lab, 0, M - 1)], 0.0)
    for name, terms in cases.items():
        assert np.array_equal(g[f"{name}/{vname}/unary"], want_u.astype(np.float32)), name
        total = np.zeros(N)
        for k, (fk, ck, kt, nt) in enumerate(terms):
            compat = g[ck] if isinstance(ck, str) else ck
            e = restated_pairwise(O, var, g[fk], compat, kt, nt, lab, N, M)
            ref = g[f"{name}/{vname}/pairwise{k}"]
            assert np.abs(e - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max()), (name, k, np.abs(e - ref).max())
            total += e
        ref = g[f"{name}/{vname}/pairwise"]
        assert np.abs(total - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max()), name
