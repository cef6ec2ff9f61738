"""The engine evaluates two of the reference's double-precision steps in
float (double arithmetic is slow on the GB300); these CPU tests check, with
numpy's IEEE float32/float64 arithmetic, that the float formulas the kernels
use give the reference's floats.

* seqCompute's blur step, old + 0.5 * (n1 + n2) with the float sum n1 + n2
  evaluated in double and rounded to float (permutohedral.cpp:505), equals
  the float evaluation x0 + 0.5 * s: bit for bit.
* The kernel norms (pairwise.cpp:54-61): 1.0 / (n + 1e-20) in double equals
  the float division bit for bit; 1.0 / sqrt(n + 1e-20) equals the float-pair
  evaluation (square root and reciprocal carried as hi + lo, low parts from
  exact fused multiply-add residuals, one final rounding) except in rare
  cases, by at most 1 ulp (meanfield.cu, norm_symmetric).
"""
import numpy as np

F32 = np.float32


def _fma(a, b, c):
    # a * b is exact in float64 (24 + 24 bits); the residuals below are exact
    # in float64 too, so one rounding to float32 is the fused result
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def test_seq_blur_step_float_equals_double():
    rng = np.random.default_rng(5)
    n = 1_000_000
    mags = np.exp(rng.uniform(-40, 40, (3, n)))
    x0, x1, x2 = (rng.standard_normal((3, n)) * mags).astype(F32)
    # near-cancellations of the old value and the neighbours' half sum
    x0[: n // 4] = (-0.5 * (x1[: n // 4].astype(np.float64) + x2[: n // 4])).astype(F32) * F32(1 + 1e-6)
    s = (x1 + x2).astype(F32)
    want = (x0.astype(np.float64) + 0.5 * s.astype(np.float64)).astype(F32)
    got = (x0 + (F32(0.5) * s).astype(F32)).astype(F32)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))


def test_one_sided_norm_float_equals_double():
    rng = np.random.default_rng(6)
    n = np.exp(rng.uniform(np.log(1e-4), 30, 1_000_000)).astype(F32)
    want = (1.0 / (n.astype(np.float64) + 1e-20)).astype(F32)
    got = (F32(1) / n).astype(F32)
    assert np.array_equal(got, want)


def test_symmetric_norm_float_pair_matches_double():
    rng = np.random.default_rng(7)
    n = np.concatenate([rng.uniform(0.5, 50, 500_000),
                        np.exp(rng.uniform(np.log(1e-4), 30, 500_000))]).astype(F32)
    want = (1.0 / np.sqrt(n.astype(np.float64) + 1e-20)).astype(F32)
    sh = np.sqrt(n).astype(F32)
    sl = (_fma(-sh, sh, n) / (F32(2) * sh)).astype(F32)
    r = (F32(1) / sh).astype(F32)
    t = _fma(-r, sh, np.ones_like(r))
    got = (r + (r * (t - (r * sl).astype(F32)).astype(F32)).astype(F32)).astype(F32)
    ulp = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32))
    assert ulp.max() <= 1
    assert np.count_nonzero(ulp) <= 2, np.count_nonzero(ulp)
    # the naive float formula is 1 ulp off for about a quarter of the values
    naive = (F32(1) / np.sqrt(n)).astype(F32)
    assert np.count_nonzero(naive != want) > len(n) // 10
