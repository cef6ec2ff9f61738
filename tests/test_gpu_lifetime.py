"""Handle lifetimes on pooled device memory: handles are created and destroyed
without device-wide synchronisation, their memory comes back from a pool that
keeps blocks (so a new handle may get an old handle's bytes), and handles of
the same image size share one copy of the tile tables.  Results must not
depend on any of that."""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(rng, W, H, M):
    U = rng.uniform(0.05, 4.0, size=(M, W * H)).astype(np.float32)
    img = rng.integers(0, 256, size=(H, W, 3)).astype(np.uint8)
    return U, img


def _solve(engine, W, H, M, U, img, T=4):
    d = engine.DenseCRF2D(W, H, M)
    d.setUnaryEnergy(U)
    d.addPairwiseGaussian(sxy=3, compat=3)
    d.addPairwiseBilateral(sxy=20, srgb=13, rgbim=img, compat=np.float32(np.eye(M) * 2 + 1))
    return d, np.array(d.inference(T))


def test_fresh_handles_on_reused_memory_reproduce(engine):
    """The same solve in fresh handles, with handles of other sizes created and
    destroyed in between (their pooled blocks are handed out again), gives
    bit-identical marginals."""
    rng = np.random.default_rng(31)
    M = 6
    sizes = [(40, 24), (23, 37), (64, 48), (40, 24), (17, 9), (40, 24)]
    probs = {s: _problem(rng, s[0], s[1], M) for s in set(sizes)}
    first = {}
    for W, H in sizes:
        d, Q = _solve(engine, W, H, M, *probs[(W, H)])
        del d
        gc.collect()
        if (W, H) in first:
            assert np.array_equal(first[(W, H)], Q), (W, H)
        else:
            first[(W, H)] = Q


def test_same_size_handles_share_tables_safely(engine):
    """Two live handles of one size (one shared copy of the tile tables): each
    keeps working after the other is destroyed, and both agree."""
    rng = np.random.default_rng(32)
    W, H, M = 33, 20, 5
    U, img = _problem(rng, W, H, M)
    a, Qa = _solve(engine, W, H, M, U, img)
    b, Qb = _solve(engine, W, H, M, U, img)
    assert np.array_equal(Qa, Qb)
    del a
    gc.collect()
    assert np.array_equal(np.array(b.inference(4)), Qa)
    c, Qc = _solve(engine, W, H, M, U, img)
    del b
    gc.collect()
    assert np.array_equal(np.array(c.inference(4)), Qa)
    assert np.array_equal(Qc, Qa)
