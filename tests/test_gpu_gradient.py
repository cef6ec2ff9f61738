"""The hand-written adjoint of T mean-field iterations against (1) the
reference's own C++ DenseCRF::gradient (golden fixtures, log-likelihood of a
label map) and (2) FP64 finite differences of the FP64 restatement of the same
mean-field.  Tolerance: 1e-3 of the gradient's largest magnitude."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-3


def _pack_matrix(G):
    """The reference's packed symmetric-matrix gradient (labelcompatibility.cpp:101-107)."""
    M = G.shape[0]
    return np.array([G[i, j] + (G[j, i] if i != j else 0.0) for i in range(M) for j in range(i, M)])


def _close(a, b, what):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    scale = max(np.abs(b).max(), 1e-12)
    err = np.abs(a - b).max() / scale
    assert err < RTOL, (what, err, a[:6], b[:6])


def test_gradient_matches_reference(engine, oracle_mod, golden):
    g = golden("gradient.npz")
    O = oracle_mod
    W, H, M, T = int(g["W"]), int(g["H"]), int(g["M"]), int(g["T"])
    N = W * H
    U, gt = g["U"], g["gt"].astype(np.int64)
    fg = O.features_gaussian_2d(W, H, 2.0, 2.0)
    fb = O.features_bilateral_2d(g["img"], 5.0, 5.0, 40.0, 40.0, 40.0)
    compat = {"potts": 2.0, "diag": g["diag"], "mat": g["mat"]}
    for name in g["cases"]:
        name = str(name)
        ck, rest = name.split("_n")
        nt, kt = (int(x) for x in rest.split("_k"))
        crf = engine.DenseCRF(N, M)
        crf.setUnaryEnergy(np.ascontiguousarray(U.T))
        crf.addPairwiseEnergy(np.ascontiguousarray(fg.T), compat[ck], kt, nt)
        crf.addPairwiseEnergy(np.ascontiguousarray(fb.T), 3.0, kt, 3)
        Q = crf.inferenceCheckpointed(T)  # (M, N)
        assert np.abs(Q.T - g[f"{name}/Q"]).max() < 1e-4, name
        # d/dQ of the mean log-likelihood, whose probabilities are clamped
        # at 1e-20 (objective.cpp:37-50); the unnormalised Potts cases drive
        # some marginals below the clamp
        dQ = np.zeros((M, N), np.float32)
        dQ[gt, np.arange(N)] = 1.0 / (N * np.maximum(Q[gt, np.arange(N)], np.float32(1e-20)))
        dU, dcs, dks = crf.backward(dQ, want_compat=True, want_kernel=True)
        _close(dU.T, g[f"{name}/dU"], (name, "dU"))
        packed = []
        for k, dc in enumerate(dcs):
            packed.extend(_pack_matrix(dc.reshape(M, M)) if (k == 0 and ck == "mat") else dc)
        _close(packed, g[f"{name}/dcompat"], (name, "dcompat"))
        _close(np.concatenate(dks), g[f"{name}/dkernel"], (name, "dkernel"))


def _fd_setup(O, seed=5):
    rng = np.random.default_rng(seed)
    W, H, M, T = 8, 6, 3, 3
    N = W * H
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    U = (rng.random((N, M)) * 3).astype(np.float32)
    wt = rng.normal(0, 1, size=(N, M))
    fg = O.features_gaussian_2d(W, H, 2.0, 2.0)
    fb = O.features_bilateral_2d(img, 4.0, 4.0, 30.0, 30.0, 30.0)
    return W, H, M, T, N, U, wt, fg, fb, rng


@pytest.mark.parametrize("ntype", [0, 1, 2, 3])
@pytest.mark.parametrize("ckind", ["potts", "diag", "mat"])
def test_gradient_vs_fp64_finite_differences(engine, oracle_mod, ntype, ckind):
    """dL/dU and dL/d(compatibility) against central differences of the FP64
    mean-field, L = sum(w .* Q_T).  The perturbations are powers of two, so the
    perturbed float inputs are exact.  Kernel parameters are not checked this
    way: the lattice is piecewise constant in the features (points change
    simplex under any finite step), so their differences do not converge; they
    are checked against the reference's own gradient above."""
    O = oracle_mod
    W, H, M, T, N, U, wt, fg, fb, rng = _fd_setup(O)
    comp = {"potts": 2.0, "diag": rng.uniform(-2, 0.5, size=M).astype(np.float32),
            "mat": rng.uniform(-1, 1, size=(M, M)).astype(np.float32)}[ckind]
    if ckind == "mat":
        comp = (0.5 * (comp + comp.T)).astype(np.float32)
    crf = engine.DenseCRF(N, M)
    crf.setUnaryEnergy(np.ascontiguousarray(U.T))
    crf.addPairwiseEnergy(np.ascontiguousarray(fg.T), comp, 1, ntype)
    crf.addPairwiseEnergy(np.ascontiguousarray(fb.T), 3.0)
    crf.inferenceCheckpointed(T)
    dU, dcs, _ = crf.backward(np.ascontiguousarray(wt.T).astype(np.float32), want_compat=True)

    def loss(Uv, c=comp):
        o = O.OracleCRF(N, M)
        o.set_unary(Uv)
        o.add_pairwise(fg, c, 1, ntype)
        o.add_pairwise(fb, 3.0)
        return float((o.inference_f64(T) * wt).sum())

    delta = 2.0 ** -10
    idx = [(int(n), int(m)) for n, m in zip(rng.integers(0, N, 12), rng.integers(0, M, 12))]
    fd, got = [], []
    for n, m in idx:
        up, dn = U.copy(), U.copy()
        up[n, m] += np.float32(delta)
        dn[n, m] -= np.float32(delta)
        fd.append((loss(up) - loss(dn)) / (2 * delta))
        got.append(dU[m, n])
    err = np.abs(np.array(got) - np.array(fd)).max() / np.abs(dU).max()
    assert err < RTOL, ("dU", err)

    dw = 2.0 ** -8
    if ckind == "potts":
        want = [(loss(U, comp + dw) - loss(U, comp - dw)) / (2 * dw)]
        have = [dcs[0][0]]
    elif ckind == "diag":
        want, have = [], list(dcs[0])
        for m in range(M):
            e = np.zeros(M, np.float32)
            e[m] = dw
            want.append((loss(U, comp + e) - loss(U, comp - e)) / (2 * dw))
    else:  # symmetric perturbation of entries (i, j) and (j, i): G_ij + G_ji
        G = np.asarray(dcs[0]).reshape(M, M)
        want, have = [], []
        for i in range(M):
            for j in range(i, M):
                e = np.zeros((M, M), np.float32)
                e[i, j] = e[j, i] = dw
                want.append((loss(U, comp + e) - loss(U, comp - e)) / (2 * dw))
                have.append(G[i, j] + (G[j, i] if i != j else 0.0))
    want, have = np.array(want), np.array(have)
    assert np.abs(have - want).max() <= RTOL * max(np.abs(want).max(), 1e-6), (ckind, have, want)


def test_autograd_function(engine, oracle_mod):
    """torch.autograd over mean_field: unary, Matrix compatibility and DIAG kernel
    parameters all receive gradients; the unary gradient matches backward()."""
    import torch

    from pydensecrf_gb300.autograd import mean_field
    O = oracle_mod
    W, H, M, T, N, U, wt, fg, fb, rng = _fd_setup(O, 7)
    crf = engine.DenseCRF(N, M)
    crf.setUnaryEnergy(np.ascontiguousarray(U.T))
    mat = rng.uniform(0, 1, size=(M, M)).astype(np.float32)
    crf.addPairwiseEnergy(np.ascontiguousarray(fg.T), mat)
    crf.addPairwiseEnergy(np.ascontiguousarray(fb.T), 3.0)
    Ut = torch.tensor(np.ascontiguousarray(U.T), device="cuda", requires_grad=True)
    mt = torch.tensor(mat, device="cuda", requires_grad=True)
    pt = torch.ones(5, device="cuda", requires_grad=True)
    Q = mean_field(crf, Ut, T, compat=[mt], kernel_params=[None, pt])
    loss = (Q * torch.tensor(np.ascontiguousarray(wt.T), device="cuda", dtype=torch.float32)).sum()
    loss.backward()
    assert Ut.grad is not None and mt.grad is not None and pt.grad is not None
    assert torch.isfinite(Ut.grad).all() and torch.isfinite(mt.grad).all() and torch.isfinite(pt.grad).all()
    crf.inferenceCheckpointed(T)
    dU, _, _ = crf.backward(np.ascontiguousarray(wt.T).astype(np.float32), want_compat=False)
    assert np.abs(Ut.grad.cpu().numpy() - dU).max() <= 1e-5 * np.abs(dU).max()
    # the matrix gradient is symmetric (W = (m + m^T)/2)
    G = mt.grad.cpu().numpy()
    assert np.abs(G - G.T).max() <= 1e-6 * max(1e-12, np.abs(G).max())


@pytest.mark.parametrize("every", [2, 3, 5, 8])
def test_checkpoint_interval_recompute_matches_full_storage(engine, oracle_mod, every):
    """Keeping only every k-th iterate and recomputing the segments in the
    backward gives the gradients of full storage bit for bit (the recomputed
    iterates are the forward's): unary, Matrix compatibility and DIAG kernel."""
    O = oracle_mod
    W, H, M, T, N, U, wt, fg, fb, rng = _fd_setup(O, 11)
    mat = rng.uniform(0, 1, size=(M, M)).astype(np.float32)
    dQ = np.ascontiguousarray(wt.T).astype(np.float32)
    out = []
    for k in (1, every):
        crf = engine.DenseCRF(N, M)
        crf.setCheckpointInterval(k)
        crf.setUnaryEnergy(np.ascontiguousarray(U.T))
        crf.addPairwiseEnergy(np.ascontiguousarray(fg.T), 3.0)
        crf.addPairwiseEnergy(np.ascontiguousarray(fb.T), mat)
        Q = crf.inferenceCheckpointed(T + 2)
        dU, dcs, dks = crf.backward(dQ, want_compat=True, want_kernel=True)
        out.append((Q, dU, np.concatenate(dcs), np.concatenate(dks)))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b), (every, np.abs(a - b).max())
