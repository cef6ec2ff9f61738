"""The allocation-free lattice filter (dcrf_lattice_filter_noalloc) against the
regular one (dcrf_lattice_filter), through the C ABI.

The allocation-free entry point exists for callers that must not allocate
device memory while they run (a fixed budget owned by another allocator, or no
cudaMalloc/cudaFree after start-up); its scratch is one static device array
shared by every call.  Two calls in a row with different inputs check that the
contents the first call leaves in that array do not leak into the second.
Same tolerance as the other filter tests: 1e-6 of the output's magnitude.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_filter(lib, _lib, crf, term, values, reverse, torch):
    src = torch.from_numpy(np.ascontiguousarray(values, np.float32)).cuda()
    dst = torch.full_like(src, float("nan"))
    stream = torch.cuda.current_stream()
    _lib.check(lib.dcrf_lattice_filter_noalloc(crf._h, term, ctypes.c_void_p(src.data_ptr()), values.shape[0],
                                               int(reverse), ctypes.c_void_p(dst.data_ptr()),
                                               ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    return dst.cpu().numpy()


def test_noalloc_filter_matches_filter(engine):
    import torch

    from pydensecrf_gb300 import _lib

    lib = _lib.load()
    rng = np.random.default_rng(21)
    N, M = 2500, 6
    feats = [rng.normal(0, 2, size=(N, 4)).astype(np.float32), rng.normal(0, 1.5, size=(N, 2)).astype(np.float32)]
    crf = engine.DenseCRF(N, M)
    for f in feats:
        crf.addPairwiseEnergy(np.ascontiguousarray(f.T), 1.0)
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
