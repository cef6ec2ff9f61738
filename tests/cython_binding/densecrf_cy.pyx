# cython: language_level=3
"""A Cython extension over the engine's C ABI (include/dcrf.h), in the shape of
the reference's own extension module (pydensecrf/densecrf.pyx:49-140, whose
extern block pydensecrf/densecrf.pxd:47-84 binds the C++ core): what a
maintainer of the reference would compile to put this engine behind the same
classes.  Typed memoryviews take the same arguments as the reference's
(float32 C-contiguous unary and features, uint8 H x W x 3 image); errors come
back as the reference's exception types.  Built and exercised by
tests/test_cython_binding.py."""
from numbers import Number

import numpy as np

from libc.stdint cimport uint8_t


cdef extern from "dcrf.h":
    ctypedef struct dcrf_crf:
        pass
    enum:
        DCRF_OK
        DCRF_ERR_INVALID_ARG
        DCRF_ERR_OOM
        DCRF_HOST
        DCRF_LAYOUT_LM
        DCRF_COMPAT_POTTS
        DCRF_COMPAT_DIAGONAL
        DCRF_COMPAT_MATRIX
        DCRF_DIAG_KERNEL
        DCRF_NORMALIZE_SYMMETRIC
    int dcrf_abi_version()
    int dcrf_last_error(char *buf, size_t len)
    int dcrf_create(int N, int M, dcrf_crf **out)
    int dcrf_create_2d(int W, int H, int M, dcrf_crf **out)
    int dcrf_destroy(dcrf_crf *h)
    int dcrf_set_unary(dcrf_crf *h, const float *U, int layout, int where)
    int dcrf_add_pairwise(dcrf_crf *h, const float *feat, int d, int where, int compat_kind, const float *compat,
                          int kernel_type, int normalization_type, int *term_out)
    int dcrf_add_pairwise_gaussian(dcrf_crf *h, float sx, float sy, int compat_kind, const float *compat,
                                   int kernel_type, int normalization_type, int *term_out)
    int dcrf_add_pairwise_bilateral(dcrf_crf *h, float sx, float sy, float sr, float sg, float sb,
                                    const uint8_t *rgb, int where, int compat_kind, const float *compat,
                                    int kernel_type, int normalization_type, int *term_out)
    int dcrf_inference(dcrf_crf *h, int n_iterations, float *Q, int layout, int where)
    int dcrf_start_inference(dcrf_crf *h, float *Q, int layout, int where)
    int dcrf_step_inference(dcrf_crf *h, float *Q, int layout, int where)
    int dcrf_kl_divergence(dcrf_crf *h, const float *Q, int layout, int where, double *kl_out)


NO_NORMALIZATION, NORMALIZE_BEFORE, NORMALIZE_AFTER, NORMALIZE_SYMMETRIC = 0, 1, 2, 3
CONST_KERNEL, DIAG_KERNEL, FULL_KERNEL = 0, 1, 2


def abi_version():
    return dcrf_abi_version()


cdef int _check(int code) except -1:
    """Status code -> the exception the reference raises for the same fault."""
    cdef char buf[512]
    if code == DCRF_OK:
        return 0
    dcrf_last_error(buf, sizeof(buf))
    msg = buf.decode("utf-8", "replace")
    if code == DCRF_ERR_INVALID_ARG:
        raise ValueError(msg)
    if code == DCRF_ERR_OOM:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def compat_buffer(compat, int M):
    """(kind, float32 buffer) for a compatibility given as the reference takes
    it: a Number (Potts), a float32 vector of M (Diagonal) or an M x M float32
    matrix (Matrix); anything else raises ValueError."""
    cdef float[:] v
    cdef float[:, :] m
    if isinstance(compat, Number):
        return DCRF_COMPAT_POTTS, np.array([compat], np.float32)
    cdef int nd = memoryview(compat).ndim
    if nd == 1:
        v = compat  # a float32 buffer, else ValueError (dtype mismatch)
        if v.shape[0] != M:
            raise ValueError("Diagonal compatibility needs one entry per label")
        return DCRF_COMPAT_DIAGONAL, np.ascontiguousarray(np.asarray(v), np.float32)
    if nd == 2:
        m = compat
        if m.shape[0] != M or m.shape[1] != M:
            raise ValueError("Matrix compatibility needs M x M entries")
        return DCRF_COMPAT_MATRIX, np.ascontiguousarray(np.asarray(m), np.float32)
    raise ValueError("LabelCompatibility of dimension >2 not meaningful.")


cdef class DenseCRF:
    cdef dcrf_crf *_h
    cdef readonly int nvar, nlabels

    def __cinit__(self, int nvar, int nlabels, *_, **__):
        self._h = NULL
        # a DenseCRF2D makes its own (2-D) handle in its constructor
        if type(self) is DenseCRF:
            self.nvar, self.nlabels = nvar, nlabels
            _check(dcrf_create(nvar, nlabels, &self._h))

    def __dealloc__(self):
        if self._h != NULL:
            dcrf_destroy(self._h)

    def setUnaryEnergy(self, float[:, ::1] u not None, f=None):
        if f is not None:
            raise NotImplementedError("logistic unaries are not part of this binding")
        if u.shape[0] != self.nlabels or u.shape[1] != self.nvar:
            raise ValueError("Bad shape for unary energy (Need {}, got {})".format(
                (self.nlabels, self.nvar), (u.shape[0], u.shape[1])))
        _check(dcrf_set_unary(self._h, &u[0, 0], DCRF_LAYOUT_LM, DCRF_HOST))

    def addPairwiseEnergy(self, float[:, ::1] features not None, compat, int kernel=DCRF_DIAG_KERNEL,
                          int normalization=DCRF_NORMALIZE_SYMMETRIC):
        if features.shape[1] != self.nvar:
            raise ValueError("Bad shape for pairwise energy (Need (?, {}), got {})".format(
                self.nvar, (features.shape[0], features.shape[1])))
        kind, c = compat_buffer(compat, self.nlabels)
        cdef float[::1] cv = c.reshape(-1)
        _check(dcrf_add_pairwise(self._h, &features[0, 0], features.shape[0], DCRF_HOST, kind, &cv[0], kernel,
                                 normalization, NULL))

    def inference(self, int niter):
        Q = np.empty((self.nlabels, self.nvar), np.float32)
        cdef float[:, ::1] q = Q
        _check(dcrf_inference(self._h, niter, &q[0, 0], DCRF_LAYOUT_LM, DCRF_HOST))
        return Q

    def startInference(self):
        Q = np.empty((self.nlabels, self.nvar), np.float32)
        cdef float[:, ::1] q = Q
        _check(dcrf_start_inference(self._h, &q[0, 0], DCRF_LAYOUT_LM, DCRF_HOST))
        return Q

    def stepInference(self, float[:, ::1] Q not None):
        _check(dcrf_step_inference(self._h, &Q[0, 0], DCRF_LAYOUT_LM, DCRF_HOST))

    def klDivergence(self, float[:, ::1] Q not None):
        cdef double kl = 0
        _check(dcrf_kl_divergence(self._h, &Q[0, 0], DCRF_LAYOUT_LM, DCRF_HOST, &kl))
        return kl


cdef class DenseCRF2D(DenseCRF):
    cdef readonly int w, h

    def __cinit__(self, int w, int h, int nlabels, *_, **__):
        self.w, self.h = w, h
        self.nvar, self.nlabels = w * h, nlabels
        _check(dcrf_create_2d(w, h, nlabels, &self._h))

    def addPairwiseGaussian(self, sxy, compat, int kernel=DCRF_DIAG_KERNEL,
                            int normalization=DCRF_NORMALIZE_SYMMETRIC):
        if isinstance(sxy, Number):
            sxy = (sxy, sxy)
        kind, c = compat_buffer(compat, self.nlabels)
        cdef float[::1] cv = c.reshape(-1)
        _check(dcrf_add_pairwise_gaussian(self._h, sxy[0], sxy[1], kind, &cv[0], kernel, normalization, NULL))

    def addPairwiseBilateral(self, sxy, srgb, unsigned char[:, :, ::1] rgbim not None, compat,
                             int kernel=DCRF_DIAG_KERNEL, int normalization=DCRF_NORMALIZE_SYMMETRIC):
        if isinstance(sxy, Number):
            sxy = (sxy, sxy)
        if isinstance(srgb, Number):
            srgb = (srgb, srgb, srgb)
        if rgbim.shape[0] != self.h or rgbim.shape[1] != self.w:
            raise ValueError("Bad shape for image (Need ({}, {}, 3), got {})".format(
                self.h, self.w, (rgbim.shape[0], rgbim.shape[1], rgbim.shape[2])))
        if rgbim.shape[2] != 3:
            raise ValueError("addPairwiseBilateral needs an RGB image with 3 channels")
        kind, c = compat_buffer(compat, self.nlabels)
        cdef float[::1] cv = c.reshape(-1)
        _check(dcrf_add_pairwise_bilateral(self._h, sxy[0], sxy[1], srgb[0], srgb[1], srgb[2], &rgbim[0, 0, 0],
                                           DCRF_HOST, kind, &cv[0], kernel, normalization, NULL))
