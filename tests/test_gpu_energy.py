"""DenseCRF::unaryEnergy / pairwiseEnergy (densecrf.cpp:141-177) on the device
against the same quantities from the oracle's lattice filter (tolerance 1e-5
of the largest magnitude).  That restatement is itself pinned to the
reference's own energies by tests/test_energy_golden.py."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(engine, oracle_mod, seed, ntype):
    rng = np.random.default_rng(seed)
    N, M = 700, 5
    f = rng.normal(0, 1.5, size=(N, 3)).astype(np.float32)
    U = rng.random((M, N)).astype(np.float32) * 3
    mat = rng.uniform(-1, 1, size=(M, M)).astype(np.float32)
    d = engine.DenseCRF(N, M)
    d.setUnaryEnergy(U)
    d.addPairwiseEnergy(np.ascontiguousarray(f.T), mat, normalization=ntype)
    lab = rng.integers(-1, M, size=N).astype(np.int16)  # -1: no label
    lat = oracle_mod.Lattice(f, "oracle", 0)
    return d, U, mat, lab, lat, N, M


@pytest.mark.parametrize("ntype", [0, 1, 2, 3])
def test_energies_match_oracle(engine, oracle_mod, ntype):
    d, U, mat, lab, lat, N, M = _setup(engine, oracle_mod, 31 + ntype, ntype)
    ok = (lab >= 0) & (lab < M)
    want_u = np.where(ok, U[np.clip(lab, 0, M - 1), np.arange(N)], 0.0)
    assert np.allclose(d.unaryEnergy(lab), want_u, rtol=0, atol=1e-6)
    # one-hot message of the term: C (n_post .* K_raw(n_pre .* onehot)), C = (m + m^T) / 2
    oh = np.zeros((N, M), np.float32)
    oh[np.arange(N)[ok], lab[ok]] = 1.0
    raw1 = lat.compute(np.ones((N, 1), np.float32), False)[:, 0].astype(np.float64)
    if ntype == 0:
        n_pre = n_post = np.ones(N)
    elif ntype == 3:
        n = 1.0 / np.sqrt(raw1 + 1e-20)
        n_pre = n_post = n
    else:
        n = 1.0 / (raw1 + 1e-20)
        n_pre, n_post = (n, np.ones(N)) if ntype == 1 else (np.ones(N), n)
    kq = lat.compute(np.ascontiguousarray((oh * n_pre[:, None]).astype(np.float32)), False) * n_post[:, None]
    C = 0.5 * (mat + mat.T)
    msg = kq @ C.T
    want_p = np.where(ok, -0.5 * msg[np.arange(N), np.clip(lab, 0, M - 1)], 0.0)
    got = d.pairwiseEnergy(lab)
    assert np.abs(got - want_p).max() <= 1e-5 * max(1.0, np.abs(want_p).max()), np.abs(got - want_p).max()
    assert np.array_equal(d.pairwiseEnergy(lab, 0), got)


def test_device_pipeline_matches_host(engine):
    """utils builders on CUDA tensors + device-tensor engine inputs reproduce the
    host (numpy) pipeline exactly."""
    import torch

    from pydensecrf_gb300 import utils
    rng = np.random.default_rng(40)
    H, W, M = 40, 56, 4
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    labels = rng.integers(0, M + 1, size=(H, W))
    U_h = utils.unary_from_labels(labels, M, gt_prob=0.7, zero_unsure=True)
    U_d = utils.unary_from_labels(torch.from_numpy(labels).cuda(), M, gt_prob=0.7, zero_unsure=True)
    assert torch.equal(U_d.cpu(), torch.from_numpy(U_h))
    fb_h = utils.create_pairwise_bilateral(sdims=(5, 5), schan=(13, 13, 13), img=img, chdim=2)
    fb_d = utils.create_pairwise_bilateral(sdims=(5, 5), schan=(13, 13, 13), img=torch.from_numpy(img).cuda(), chdim=2)
    assert torch.equal(fb_d.cpu(), torch.from_numpy(fb_h))
    fg_h = utils.create_pairwise_gaussian(sdims=(3, 3), shape=(H, W))
    fg_d = utils.create_pairwise_gaussian(sdims=(3, 3), shape=(H, W), device="cuda")
    assert torch.equal(fg_d.cpu(), torch.from_numpy(fg_h))
    sm = rng.random((M, H, W)).astype(np.float32)
    assert torch.allclose(utils.unary_from_softmax(torch.from_numpy(sm).cuda(), scale=0.8).cpu(),
                          torch.from_numpy(utils.unary_from_softmax(sm, scale=0.8)), rtol=0, atol=1e-6)

    def run(U, fg, fb, device):
        d = engine.DenseCRF(H * W, M)
        d.setUnaryEnergy(U)
        d.addPairwiseEnergy(fg, compat=3)
        d.addPairwiseEnergy(fb, compat=10)
        return d.inference_tensor(5).cpu().numpy() if device else np.array(d.inference(5))

    assert np.array_equal(run(U_d, fg_d, fb_d, True), run(U_h, fg_h, fb_h, False))
    d2 = engine.DenseCRF2D(W, H, M)
    d2.setUnaryEnergy(U_d)
    d2.addPairwiseBilateral(sxy=5, srgb=13, rgbim=torch.from_numpy(img).cuda(), compat=10)
    h2 = engine.DenseCRF2D(W, H, M)
    h2.setUnaryEnergy(U_h)
    h2.addPairwiseBilateral(sxy=5, srgb=13, rgbim=img, compat=10)
    assert np.array_equal(d2.inference_tensor(4).cpu().numpy(), np.array(h2.inference(4)))
