"""Buffer wrappers with the behaviour of ``pydensecrf.eigen``.

The reference exposes Eigen's column-major ``MatrixXf``/``VectorXf`` through
the buffer protocol (pydensecrf/eigen.pyx:15-98): a matrix of ``rows x cols``
has strides ``(4, 4*rows)``, so ``np.array(Q)`` of the marginals returned by
``inference`` is an ``(M, N)`` array whose memory is point-major.  These
classes keep exactly that memory layout in a numpy buffer and export it with
``__buffer__`` / ``__array__``.
"""
from __future__ import annotations

import numpy as np

__all__ = ["MatrixXf", "VectorXf", "matrixXf", "vectorXf", "as_float_buffer"]


def as_float_buffer(x, ndim: int, name: str = "argument") -> np.ndarray:
    """Accept what a Cython ``float[::1]`` / ``float[:, ::1]`` argument accepts.

    None -> TypeError; wrong dtype, wrong number of dimensions or a
    non-C-contiguous buffer -> ValueError (pydensecrf/eigen.pyx:7-12,49-55).
    """
    if x is None:
        raise TypeError(f"{name} must not be None")
    if isinstance(x, (MatrixXf, VectorXf)):
        x = np.asarray(x)
    try:
        mv = memoryview(x)
    except TypeError as e:
        raise TypeError(f"{name}: object does not support the buffer protocol") from e
    if mv.format not in ("f", "<f", "=f", "@f"):
        raise ValueError(f"Buffer dtype mismatch, expected 'float' but got '{mv.format}'")
    if mv.ndim != ndim:
        raise ValueError(f"Buffer has wrong number of dimensions (expected {ndim}, got {mv.ndim})")
    if not mv.c_contiguous:
        raise ValueError("ndarray is not C-contiguous")
    return np.asarray(x)


class VectorXf:
    """1-D float buffer (the reference's eigen.VectorXf)."""

    def __init__(self):
        self._a = np.zeros((0,), np.float32)

    def wrap(self, a: np.ndarray) -> "VectorXf":
        self._a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
        return self

    @property
    def shape(self):
        return self._a.shape

    def __buffer__(self, flags):
        return memoryview(self._a)

    def __array__(self, dtype=None, copy=None):
        return self._a if dtype is None else self._a.astype(dtype)

    def __len__(self):
        return len(self._a)


class MatrixXf:
    """Column-major float matrix (the reference's eigen.MatrixXf).

    ``data`` is the underlying point-major buffer of shape ``(cols, rows)``;
    the exported view is ``(rows, cols)`` with strides ``(4, 4*rows)``.
    """

    def __init__(self):
        self.data = np.zeros((0, 0), np.float32)

    def wrap_colmajor(self, data: np.ndarray) -> "MatrixXf":
        """Wrap a C-contiguous (cols, rows) float32 buffer without copying."""
        assert data.dtype == np.float32 and data.flags.c_contiguous and data.ndim == 2
        self.data = data
        return self

    @property
    def shape(self):
        return (self.data.shape[1], self.data.shape[0])

    @property
    def rows(self) -> int:
        return self.data.shape[1]

    @property
    def cols(self) -> int:
        return self.data.shape[0]

    def view(self) -> np.ndarray:
        """The (rows, cols) view, sharing memory."""
        return self.data.T

    def __buffer__(self, flags):
        return memoryview(self.data.T)

    def __array__(self, dtype=None, copy=None):
        v = self.data.T
        return v if dtype is None else v.astype(dtype)

    def __repr__(self):
        return f"MatrixXf(shape={self.shape})"


def vectorXf(arr) -> VectorXf:
    """Copy a C-contiguous float32 vector (pydensecrf/eigen.pyx:11-12)."""
    a = as_float_buffer(arr, 1, "arr")
    return VectorXf().wrap(a.copy())


def matrixXf(arr) -> MatrixXf:
    """Copy a C-contiguous float32 matrix into column-major storage (eigen.pyx:54-55)."""
    a = as_float_buffer(arr, 2, "arr")
    return MatrixXf().wrap_colmajor(np.ascontiguousarray(a.T, dtype=np.float32))
