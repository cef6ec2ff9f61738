"""The unary and feature builders against the reference's own utils.py.

tests/golden/utils.npz holds the outputs of pydensecrf/utils.py (the
reference's pure-numpy module, imported from its source file by
tests/golden/make_golden.py) on seeded label maps, softmaxes, images and
volumes.  The numpy forms must reproduce them bit for bit (same dtype, same
shape).  The tensor forms (run here on CPU tensors; the same torch code runs on
CUDA tensors) must too, except where the reference takes a float32 logarithm:
numpy's float32 log is itself up to a few ulp from the exact value and varies
with the host's SIMD dispatch, so there the bar is 3 ulp of the reference value
(the tensor form is correctly rounded on these inputs)."""
import os
import warnings

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def z():
    return np.load(os.path.join(ROOT, "tests", "golden", "utils.npz"))


@pytest.fixture(scope="module")
def U():
    from pydensecrf_gb300 import utils
    return utils


def _np(x):
    try:
        import torch
        if isinstance(x, torch.Tensor):
            return x.numpy()
    except ImportError:
        pass
    return x


def _exact(z, name, ours):
    ref = z[name]
    o = _np(ours)
    assert o.shape == ref.shape and o.dtype == ref.dtype, (name, o.shape, o.dtype, ref.shape, ref.dtype)
    assert np.array_equal(o, ref), (name, np.abs(o.astype(np.float64) - ref).max())


def _ulp(z, name, ours, n):
    ref = z[name]
    o = _np(ours)
    assert o.shape == ref.shape and o.dtype == ref.dtype, name
    err = np.abs(o.astype(np.float64) - ref) / np.spacing(np.abs(ref))
    assert err.max() <= n, (name, err.max())


def _forms():
    forms = [("numpy", lambda a: a)]
    try:
        import torch
        forms.append(("tensor", lambda a: torch.from_numpy(np.ascontiguousarray(a))))
    except ImportError:
        pass
    return forms


@pytest.mark.parametrize("form", [f[0] for f in _forms()])
def test_unary_from_labels(z, U, form):
    f = dict(_forms())[form]
    for gt in (0.5, 0.7, 0.95):
        _exact(z, f"labels_unsure/{gt}", U.unary_from_labels(f(z["lab"]), 5, gt, zero_unsure=True))
        _exact(z, f"labels_sure/{gt}", U.unary_from_labels(f(z["lab"]), 6, gt, zero_unsure=False))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        if form == "numpy":
            _exact(z, "compute_unary", U.compute_unary(z["lab"], 5, GT_PROB=0.6))


@pytest.mark.parametrize("form", [f[0] for f in _forms()])
@pytest.mark.parametrize("src", ["sm64", "sm32"])
def test_unary_from_softmax(z, U, form, src):
    f = dict(_forms())[form]
    x = z[src]
    tiny = np.maximum(x, x.dtype.type(1e-30))
    # float32 input without ``scale``: the reference takes a float32 log
    check = (lambda n, o: _ulp(z, n, o, 3)) if (form == "tensor" and src == "sm32") else (lambda n, o: _exact(z, n, o))
    check(f"softmax/{src}/default", U.unary_from_softmax(f(x)))
    _exact(z, f"softmax/{src}/scale", U.unary_from_softmax(f(x), scale=0.8))
    check(f"softmax/{src}/noclip", U.unary_from_softmax(f(tiny), clip=None))
    _exact(z, f"softmax/{src}/scale_noclip", U.unary_from_softmax(f(x), scale=0.6, clip=None))
    check(f"softmax/{src}/to_unary", U.softmax_to_unary(f(tiny)))
    _exact(z, f"softmax/{src}/to_unary_gt", U.softmax_to_unary(f(x), GT_PROB=0.7))


@pytest.mark.parametrize("form", [f[0] for f in _forms()])
def test_pairwise_gaussian(z, U, form):
    dev = None if form == "numpy" else "cpu"
    _exact(z, "gauss2", U.create_pairwise_gaussian((3, 5), (19, 23), device=dev))
    _exact(z, "gauss2_frac", U.create_pairwise_gaussian((0.7, 13.3), (7, 29), device=dev))
    _exact(z, "gauss3", U.create_pairwise_gaussian((2, 3, 7), (5, 6, 7), device=dev))


@pytest.mark.parametrize("form", [f[0] for f in _forms()])
def test_pairwise_bilateral(z, U, form):
    f = dict(_forms())[form]
    img, gray = z["img"], z["gray"]
    # uint16 is not a torch tensor type: the tensor form takes the volume as int32
    vol = z["vol"] if form == "numpy" else z["vol"].astype(np.int32)
    _exact(z, "bilat_rgb", U.create_pairwise_bilateral((80, 80), (13, 13, 13), f(img), chdim=2))
    _exact(z, "bilat_rgb_mixed", U.create_pairwise_bilateral((3.3, 7), (5, 11.5, 0.9), f(img), chdim=2))
    _exact(z, "bilat_rgb_scalar", U.create_pairwise_bilateral((4, 4), 20, f(img), chdim=2))
    _exact(z, "bilat_gray", U.create_pairwise_bilateral((2, 9), 0.3, f(gray), chdim=-1))
    _exact(z, "bilat_vol", U.create_pairwise_bilateral((1, 2, 3), (100, 250.0), f(vol), chdim=0))


def test_loop_forms(z, U):
    _exact(z, "gauss2_loop", U._create_pairwise_gaussian_2d(3, 5, (9, 8)))
    _exact(z, "bilat2_loop", U._create_pairwise_bilateral_2d(3, 5, 13, 11, 7, z["img"][:9, :8]))
