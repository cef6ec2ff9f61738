"""GB300-native dense-CRF engine with the Python surface of pydensecrf.

Submodules mirror the reference package:

* :mod:`pydensecrf_gb300.densecrf` -- ``DenseCRF``, ``DenseCRF2D``, unaries, enums
* :mod:`pydensecrf_gb300.eigen`    -- ``MatrixXf`` / ``VectorXf`` buffer wrappers
* :mod:`pydensecrf_gb300.utils`    -- unary and feature builders

``install_alias()`` registers this package under the name ``pydensecrf`` so
that unmodified code doing ``import pydensecrf.densecrf as dcrf`` runs on it.
"""
from __future__ import annotations

import sys

__all__ = ["install_alias"]


def install_alias() -> None:
    """Make ``import pydensecrf[.densecrf|.eigen|.utils]`` resolve to this package."""
    from . import densecrf, eigen, utils

    sys.modules["pydensecrf"] = sys.modules[__name__]
    sys.modules["pydensecrf.densecrf"] = densecrf
    sys.modules["pydensecrf.eigen"] = eigen
    sys.modules["pydensecrf.utils"] = utils
