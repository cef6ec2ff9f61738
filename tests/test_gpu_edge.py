"""Degenerate problem sizes against the oracle: a single point, one-pixel-wide
and one-pixel-high images, a tile holding a handful of points, and a 4-d
generic point set smaller than one tile.  They exercise the smallest cases of
every launch (one tile, one partial per vertex, one-element scans and sorts,
one or two blur launches)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QTOL = 1e-4


def _unary(rng, M, N):
    logits = rng.normal(0, 2, size=(M, N))
    p = np.exp(logits - logits.max(0))
    return (-np.log(p / p.sum(0))).astype(np.float32)


@pytest.mark.parametrize("W,H", [(1, 1), (1, 17), (19, 1), (3, 2), (16, 16), (17, 16)])
def test_tiny_images_vs_oracle(engine, oracle_mod, W, H):
    rng = np.random.default_rng(W * 100 + H)
    M, N, T = 4, W * H, 5
    U = _unary(rng, M, N)
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    d = engine.DenseCRF2D(W, H, M)
    d.setUnaryEnergy(U)
    d.addPairwiseGaussian(sxy=3, compat=3)
    d.addPairwiseBilateral(sxy=20, srgb=13, rgbim=img, compat=5)
    Q = np.array(d.inference(T))
    O = oracle_mod
    o = O.OracleCRF(N, M)
    o.set_unary(np.ascontiguousarray(U.T))
    o.add_pairwise(O.features_gaussian_2d(W, H, 3, 3), 3.0)
    o.add_pairwise(O.features_bilateral_2d(img, 20, 20, 13, 13, 13), 5.0)
    err = np.abs(Q.T - o.inference(T)).max()
    assert err < QTOL, (W, H, err)


@pytest.mark.parametrize("N", [1, 2, 5, 255, 257])
def test_small_point_sets_vs_oracle(engine, oracle_mod, N):
    rng = np.random.default_rng(N)
    M, T = 3, 4
    U = _unary(rng, M, N)
    feat = rng.normal(0, 1.5, size=(4, N)).astype(np.float32)
    d = engine.DenseCRF(N, M)
    d.setUnaryEnergy(U)
    d.addPairwiseEnergy(feat, compat=2.0)
    Q = np.array(d.inference(T))
    o = oracle_mod.OracleCRF(N, M)
    o.set_unary(np.ascontiguousarray(U.T))
    o.add_pairwise(np.ascontiguousarray(feat.T), 2.0)
    err = np.abs(Q.T - o.inference(T)).max()
    assert err < QTOL, (N, err)
