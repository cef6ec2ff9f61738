"""The allocation-free lattice filter (dcrf_lattice_filter_noalloc) against the
regular one (dcrf_lattice_filter), through the C ABI.

The allocation-free entry point exists for callers that must not allocate
device memory while they run (a fixed budget owned by another allocator, or no
cudaMalloc/cudaFree after start-up); its scratch is one static device array
shared by every call.  Two calls in a row with different inputs check that the
contents the first call leaves in that array do not leak into the second.
Same tolerance as the other filter tests: 1e-6 of the output's magnitude,
against the regular filter and against the oracle's restatement of
Permutohedral::compute (permutohedral.cpp:596-604).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_filter(lib, _lib, crf, term, values, reverse, torch, stream=None):
    stream = stream or torch.cuda.current_stream()
    with torch.cuda.stream(stream):
        src = torch.from_numpy(np.ascontiguousarray(values, np.float32)).cuda()
        dst = torch.full_like(src, float("nan"))
        _lib.check(lib.dcrf_lattice_filter_noalloc(crf._h, term, ctypes.c_void_p(src.data_ptr()), values.shape[0],
                                                   int(reverse), ctypes.c_void_p(dst.data_ptr()),
                                                   ctypes.c_void_p(stream.cuda_stream)))
        out = dst.cpu()  # ordered on `stream`
    torch.cuda.synchronize()
    return out.numpy()


def test_noalloc_filter_matches_filter(engine, oracle_mod):
    import torch

    from pydensecrf_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(21)
    N, M = 2500, 6
    feats = [rng.normal(0, 2, size=(N, 4)).astype(np.float32), rng.normal(0, 1.5, size=(N, 2)).astype(np.float32)]
    crf = engine.DenseCRF(N, M)
    for f in feats:
        crf.addPairwiseEnergy(np.ascontiguousarray(f.T), 1.0)
    lats = [oracle_mod.Lattice(f, "oracle") for f in feats]
    for term in (0, 1):
        for vs in (M, 1):
            for reverse in (False, True):
                for call in range(2):  # two calls in a row share the scratch array
                    v = rng.random((vs, N)).astype(np.float32) * (call + 1)
                    want = crf.lattice_filter(term, v, reverse)
                    got = _noalloc_filter(lib, _lib, crf, term, v, reverse, torch)
                    assert np.isfinite(got).all()
                    err = np.abs(got - want).max()
                    assert err <= 1e-6 * np.abs(want).max(), (term, vs, reverse, call, err)
                    orc = lats[term].compute(np.ascontiguousarray(v.T), reverse).T
                    err = np.abs(got - orc).max()
                    assert err <= 1e-6 * np.abs(orc).max(), ("oracle", term, vs, reverse, call, err)


def test_noalloc_filter_above_32_labels(engine, oracle_mod):
    """70 labels: the scratch holds one label chunk of 32 at a time and the
    three chunks (the last one 6 labels padded to 8) go through it in turn; the
    result must match the regular filter and the oracle's filter of the whole
    rows, after a call of value size 1 left other contents in the scratch."""
    import torch

    from pydensecrf_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(27)
    N, M = 3000, 70
    f = rng.normal(0, 2, size=(N, 3)).astype(np.float32)
    crf = engine.DenseCRF(N, M)
    crf.addPairwiseEnergy(np.ascontiguousarray(f.T), 1.0)
    lat = oracle_mod.Lattice(f, "oracle")
    for reverse in (False, True):
        _noalloc_filter(lib, _lib, crf, 0, rng.random((1, N)).astype(np.float32), reverse, torch)
        v = rng.random((M, N)).astype(np.float32)
        got = _noalloc_filter(lib, _lib, crf, 0, v, reverse, torch)
        assert np.isfinite(got).all()
        want = crf.lattice_filter(0, v, reverse)
        err = np.abs(got - want).max()
        assert err <= 1e-6 * np.abs(want).max(), (reverse, err)
        orc = lat.compute(np.ascontiguousarray(v.T), reverse).T
        err = np.abs(got - orc).max()
        assert err <= 1e-6 * np.abs(orc).max(), ("oracle", reverse, err)


def test_noalloc_right_after_build_on_another_stream(engine, oracle_mod):
    """The call is queued on a stream of the caller's own straight after a term
    is added (the build may still be running on the handle's stream), and the
    handle's terms are cleared and rebuilt straight after the call, before
    anything synchronises (the call may still be reading the old tables).  The
    result is read only at the end, and must match the oracle's filter."""
    import torch

    from pydensecrf_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(33)
    N, M = 40000, 8
    side = torch.cuda.Stream()
    for trial in range(3):
        f = rng.normal(0, 3, size=(N, 3)).astype(np.float32)
        v = rng.random((M, N)).astype(np.float32)
        src = torch.from_numpy(v).cuda()
        torch.cuda.synchronize()
        crf = engine.DenseCRF(N, M)
        crf.addPairwiseEnergy(np.ascontiguousarray(f.T), 1.0)
        with torch.cuda.stream(side):
            dst = torch.full_like(src, float("nan"))
            _lib.check(lib.dcrf_lattice_filter_noalloc(crf._h, 0, ctypes.c_void_p(src.data_ptr()), M,
                                                       int(trial == 1), ctypes.c_void_p(dst.data_ptr()),
                                                       ctypes.c_void_p(side.cuda_stream)))
        _lib.check(lib.dcrf_clear_pairwise(crf._h))
        crf.addPairwiseEnergy(np.ascontiguousarray(rng.normal(0, 1, size=(2, N)).astype(np.float32)), 1.0)
        torch.cuda.synchronize()
        got = dst.cpu().numpy()
        want = oracle_mod.Lattice(f, "oracle").compute(np.ascontiguousarray(v.T), trial == 1).T
        err = np.abs(got - want).max()
        assert err <= 1e-6 * np.abs(want).max(), (trial, err)
        del crf


def test_noalloc_rejects_oversized(engine):
    """A problem whose scratch exceeds the static array is refused with a clear error."""
    import torch

    from pydensecrf_gb300 import _lib

    lib = _lib.load()
    W, H, M = 1024, 1024, 21  # 21 x 2^20 slots alone exceed the array
    crf = engine.DenseCRF2D(W, H, M)
    crf.addPairwiseGaussian(3, 3)
    src = torch.zeros((M, W * H), device="cuda")
    dst = torch.zeros_like(src)
    code = lib.dcrf_lattice_filter_noalloc(crf._h, 0, ctypes.c_void_p(src.data_ptr()), M, 0,
                                           ctypes.c_void_p(dst.data_ptr()), None)
    assert code == _lib.DCRF_ERR_INVALID_ARG
    assert "scratch" in _lib.last_error()
