"""The Python surface a pydensecrf user switches to, checked without a GPU:
enum values (pydensecrf/densecrf.pxd:43-44), method names and defaults
(densecrf.pyx:49-140), the class hierarchy, the compatibility dispatch
(densecrf.pyx:11-20) and the ``pydensecrf`` import alias."""
import inspect
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_enum_values():
    from pydensecrf_gb300 import densecrf as d
    assert (int(d.CONST_KERNEL), int(d.DIAG_KERNEL), int(d.FULL_KERNEL)) == (0, 1, 2)
    assert (int(d.NO_NORMALIZATION), int(d.NORMALIZE_BEFORE), int(d.NORMALIZE_AFTER),
            int(d.NORMALIZE_SYMMETRIC)) == (0, 1, 2, 3)


def test_methods_and_defaults():
    from pydensecrf_gb300 import densecrf as d
    for name in ("addPairwiseEnergy", "setUnary", "setUnaryEnergy", "inference", "startInference",
                 "stepInference", "klDivergence"):
        assert callable(getattr(d.DenseCRF, name)), name
    for name in ("addPairwiseGaussian", "addPairwiseBilateral"):
        assert callable(getattr(d.DenseCRF2D, name)), name
    assert issubclass(d.DenseCRF2D, d.DenseCRF)
    assert issubclass(d.ConstUnary, d.Unary) and issubclass(d.LogisticUnary, d.Unary)

    def defaults(fn):
        return {k: p.default for k, p in inspect.signature(fn).parameters.items()
                if p.default is not inspect.Parameter.empty}

    want = {"kernel": d.DIAG_KERNEL, "normalization": d.NORMALIZE_SYMMETRIC}
    assert defaults(d.DenseCRF.addPairwiseEnergy) == want
    assert defaults(d.DenseCRF2D.addPairwiseGaussian) == want
    assert defaults(d.DenseCRF2D.addPairwiseBilateral) == want
    assert defaults(d.DenseCRF.setUnaryEnergy) == {"f": None}
    # positional order of the reference's signatures
    assert list(inspect.signature(d.DenseCRF2D.addPairwiseBilateral).parameters)[:5] == \
        ["self", "sxy", "srgb", "rgbim", "compat"]
    assert list(inspect.signature(d.DenseCRF.stepInference).parameters) == ["self", "Q", "tmp1", "tmp2"]


def test_compatibility_dispatch():
    from pydensecrf_gb300 import _lib
    from pydensecrf_gb300 import densecrf as d
    kind, v = d._labelcomp(3, 4)
    assert kind == _lib.COMPAT_POTTS and v.tolist() == [3.0]
    kind, v = d._labelcomp(np.arange(4, dtype=np.float32), 4)
    assert kind == _lib.COMPAT_DIAGONAL and v.tolist() == [0, 1, 2, 3]
    kind, v = d._labelcomp(np.eye(4, dtype=np.float32), 4)
    assert kind == _lib.COMPAT_MATRIX and v.shape == (4, 4)
    with pytest.raises(ValueError):
        d._labelcomp(np.ones((2, 2, 2), np.float32), 2)  # "dimension >2 not meaningful"
    with pytest.raises(ValueError):
        d._labelcomp(np.ones(3, np.float64), 3)  # float64 buffer: the typed memoryview rejects it
    with pytest.raises(ValueError):
        d._labelcomp(np.ones(3, np.float32), 4)  # wrong label count


def test_unary_holders_copy_their_inputs():
    from pydensecrf_gb300 import densecrf as d
    u = np.ones((2, 5), np.float32)
    c = d.ConstUnary(u)
    u[:] = 7
    assert np.all(c._matrix(2, 5) == 1)
    with pytest.raises(TypeError):
        d.ConstUnary(None)
    with pytest.raises(ValueError):
        d.ConstUnary(np.ones(5, np.float32))


def test_pydensecrf_alias():
    """Unmodified reference-style imports resolve to this package."""
    code = ("import pydensecrf_gb300 as p; p.install_alias();"
            "import pydensecrf.densecrf as dcrf; from pydensecrf import eigen;"
            "from pydensecrf.utils import unary_from_softmax, create_pairwise_bilateral;"
            "import pydensecrf_gb300.densecrf as ours, pydensecrf_gb300.utils as u;"
            "assert dcrf is ours and unary_from_softmax is u.unary_from_softmax;"
            "assert eigen.MatrixXf is ours.MatrixXf;"
            "print('ok')")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
