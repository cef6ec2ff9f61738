"""CPU tests of the host side: the C-ABI library's exports, the eigen buffer
wrappers (reference pydensecrf/tests/test_eigen.py) and the utils helpers
(reference tests/test_utils.py).  No GPU work is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "dcrf.h")).read()
    return sorted(set(re.findall(r"^\s*int\s+(dcrf_\w+)\s*\(", txt, re.M)))


def test_header_and_binding_agree():
    from pydensecrf_gb300 import _lib
    assert _declared_symbols() == _lib.symbols()


def test_library_exports_every_declared_symbol():
    from pydensecrf_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in _declared_symbols():
        assert hasattr(lib, name), name
    assert lib.dcrf_abi_version() == 1


def test_library_errors_without_device_are_explicit():
    """Creating a handle where no GPU is visible returns an error, never a CPU path."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from pydensecrf_gb300 import _lib, densecrf
    _lib.load()
    with pytest.raises(_lib.DenseCRFError):
        densecrf.DenseCRF(100, 2)
    with pytest.raises(_lib.DenseCRFError):
        densecrf.DenseCRF2D(10, 10, 2)


def test_batch_handles_without_device_are_explicit():
    """The batched classes have no CPU path either; their host-side argument
    checks run before any device call."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from pydensecrf_gb300 import _lib, batch
    _lib.load()
    with pytest.raises(_lib.DenseCRFError):
        batch.DenseCRFBatch([100, 37], 3)
    with pytest.raises(_lib.DenseCRFError):
        batch.DenseCRF2DBatch([10, 7], [10, 3], 3)
    with pytest.raises(ValueError):
        batch.DenseCRF2DBatch([10, 7], [10], 3)


def test_bandwidth_grad_chain_rule():
    """dL/ds for features x/s from the DIAG parameter gradient at p = 1."""
    import torch
    from pydensecrf_gb300 import autograd
    dp = torch.tensor([1.0, 2.0, 3.0, 4.0], dtype=torch.float64)
    assert float(autograd.bandwidth_grad(dp, 2.0, (0, 2))) == -(1.0 + 3.0) / 2.0


# ---- eigen (reference: pydensecrf/tests/test_eigen.py) -----------------------
def test_vector_conversion():
    from pydensecrf_gb300 import eigen as e
    v = np.random.randn(3).astype(np.float32)
    assert np.all(np.array(e.vectorXf(v)) == v)


def test_matrix_conversion():
    from pydensecrf_gb300 import eigen as e
    m = np.random.randn(3, 4).astype(np.float32)
    c = e.matrixXf(m)
    assert np.all(np.array(c) == m)
    # column-major memory like the reference's Eigen buffer
    assert memoryview(c).strides == (4, 12)


def test_wrong_dims():
    from pydensecrf_gb300 import eigen as e
    with pytest.raises(ValueError):
        e.matrixXf(np.random.randn(3, 3, 3).astype(np.float32))


def test_wrong_type():
    from pydensecrf_gb300 import eigen as e
    with pytest.raises(ValueError):
        e.matrixXf(np.random.randn(3, 3).astype(np.float64))


def test_none_type():
    from pydensecrf_gb300 import eigen as e
    with pytest.raises(TypeError):
        e.matrixXf(None)


# ---- utils (reference: tests/test_utils.py) -----------------------------------
def test_unary_known_answer():
    from pydensecrf_gb300 import utils
    M = 3
    U, P, N = 1. / M, 0.8, 0.2 / (M - 1)
    labels = np.array([[0, 1, 2, 3], [3, 2, 1, 0]])
    unary = -np.log(np.array([[U, P, N, N, N, N, P, U], [U, N, P, N, N, P, N, U], [U, N, N, P, P, N, N, U]]))
    np.testing.assert_almost_equal(utils.compute_unary(labels, M, GT_PROB=P), unary)


def test_unary_not_zero_unsure():
    from pydensecrf_gb300 import utils
    U = utils.unary_from_labels(np.array([0, 1, 1]), 2, 0.9, zero_unsure=False)
    np.testing.assert_allclose(U, -np.log([[0.9, 0.1, 0.1], [0.1, 0.9, 0.9]]), rtol=1e-6)


def test_unary_from_softmax():
    from pydensecrf_gb300 import utils
    sm = np.array([[0.0, 0.5], [1.0, 0.5]])
    np.testing.assert_allclose(utils.unary_from_softmax(sm), -np.log([[1e-5, 0.5], [1.0, 0.5]]), rtol=1e-6)
    s = utils.unary_from_softmax(sm, scale=0.5, clip=None)
    np.testing.assert_allclose(s, -np.log([[0.25, 0.5], [0.75, 0.5]]), rtol=1e-6)
    assert s.dtype == np.float32


def test_pairwise_builders_match_loop_forms():
    from pydensecrf_gb300 import utils
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, size=(7, 9, 3)).astype(np.uint8)
    a = utils.create_pairwise_gaussian((3, 2), (7, 9))
    b = utils._create_pairwise_gaussian_2d(3, 2, (7, 9))
    assert np.array_equal(a, b)
    a = utils.create_pairwise_bilateral((3, 2), (13, 11, 7), img, chdim=2)
    b = utils._create_pairwise_bilateral_2d(3, 2, 13, 11, 7, img)
    assert np.array_equal(a, b) and a.dtype == np.float32
    one = utils.create_pairwise_bilateral((2, 2), 5, img[..., 0], chdim=-1)
    assert one.shape == (3, 63)


def test_logistic_unary_host_logic():
    """LogisticUnary (densecrf.pyx:44-46) keeps float32 copies of L and f; the
    shapes are checked on the host before the engine is called (U = L f itself
    is computed by the engine on the device)."""
    from pydensecrf_gb300 import densecrf
    rng = np.random.default_rng(60)
    L = rng.normal(0, 1, (4, 7))
    f = rng.normal(0, 1, (7, 50)).astype(np.float32)
    u = densecrf.LogisticUnary(L.astype(np.float32), f)
    assert u.L.dtype == np.float32 and u.f.dtype == np.float32 and u.f is not f
    d = object.__new__(densecrf.DenseCRF)  # argument checks only: no device handle
    d._nlabel, d._nvar = 4, 50
    for bad_L, bad_f in ((np.ones((3, 7), np.float32), f), (np.ones((4, 6), np.float32), f),
                         (np.ones((4, 7), np.float32), np.ones((7, 49), np.float32))):
        with pytest.raises(ValueError):
            d._set_logistic(bad_L, bad_f)