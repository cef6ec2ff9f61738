"""Failure detection without a GPU fault: a device-side wait on a flag that
nothing sets gives up after its bound, the host reads DCRF_ERR_TIMEOUT from the
handle's status block at the next synchronisation, and the handle (and the
CUDA context) keep working afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_crf(engine, rng):
    W, H, M = 24, 16, 4
    d = engine.DenseCRF2D(W, H, M)
    d.setUnaryEnergy(rng.uniform(0.1, 3.0, size=(M, W * H)).astype(np.float32))
    d.addPairwiseGaussian(sxy=3, compat=3)
    return d


def test_bounded_wait_times_out_and_handle_stays_usable(engine):
    from pydensecrf_gb300 import _lib

    lib = _lib.load()
    d = _small_crf(engine, np.random.default_rng(21))
    Q0 = np.array(d.inference(3))
    rc = lib.dcrf_check_bounded_wait(d._h, 2000)
    assert rc == _lib.DCRF_ERR_TIMEOUT, (rc, _lib.last_error())
    assert "gave up" in _lib.last_error()
    # the status was cleared: the same solve runs and gives the same marginals
    Q1 = np.array(d.inference(3))
    assert np.array_equal(Q0, Q1)
    # and a second wait times out again (the flag path is not latched)
    assert lib.dcrf_check_bounded_wait(d._h, 10) == _lib.DCRF_ERR_TIMEOUT


def test_bounded_wait_rejects_bad_bounds(engine):
    from pydensecrf_gb300 import _lib

    lib = _lib.load()
    d = _small_crf(engine, np.random.default_rng(22))
    assert lib.dcrf_check_bounded_wait(d._h, 0) == _lib.DCRF_ERR_INVALID_ARG
    assert lib.dcrf_check_bounded_wait(d._h, (1 << 20) + 1) == _lib.DCRF_ERR_INVALID_ARG
    assert lib.dcrf_check_bounded_wait(None, 10) == _lib.DCRF_ERR_INVALID_ARG
