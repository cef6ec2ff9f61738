"""Batches of independent dense CRFs solved together (no reference counterpart).

The reference solves one ``DenseCRF`` per image or point cloud
(densecrf.pyx:49-140).  :class:`DenseCRFBatch` and :class:`DenseCRF2DBatch`
hold many problems of uneven sizes with the same labels and pairwise terms in
one engine handle: each image gets its own lattice (the image index is part of
the lattice key), and every kernel of the build, the normalisation and the
mean-field iterations runs once over all images.  Per image the results are
those of a separate ``DenseCRF`` / ``DenseCRF2D`` with the same inputs.

Unaries, marginals and gradients are lists with one ``(M, N_b)`` array per
image; features are lists of ``(d, N_b)`` arrays; RGB images are lists of
``(H_b, W_b, 3)`` uint8 arrays.
"""
from __future__ import annotations

import ctypes
from numbers import Number

import numpy as np

from . import _lib
from .densecrf import DIAG_KERNEL, NORMALIZE_SYMMETRIC, DenseCRF, _check_enum, _labelcomp, _ptr

__all__ = ["DenseCRFBatch", "DenseCRF2DBatch"]


class DenseCRFBatch:
    """``len(sizes)`` dense CRFs with ``sizes[b]`` variables each and ``nlabels`` labels."""

    def __init__(self, sizes, nlabels: int):
        self._sizes = [int(n) for n in sizes]
        self._nlabel = int(nlabels)
        self._start = np.concatenate([[0], np.cumsum(self._sizes)]).astype(np.int64)
        self._h = ctypes.c_void_p()
        if type(self) is DenseCRFBatch:
            n = np.ascontiguousarray(self._sizes, np.int32)
            _lib.check(_lib.load().dcrf_create_batch(len(self._sizes), _ptr(n), self._nlabel, ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().dcrf_destroy(h)
            except Exception:
                pass
            h.value = None

    def __len__(self) -> int:
        return len(self._sizes)

    @property
    def sizes(self):
        return list(self._sizes)

    # -- buffers: one (rows, N_b) block per image, images one after another --------
    def _pack(self, arrays, rows: int, what: str) -> np.ndarray:
        if len(arrays) != len(self._sizes):
            raise ValueError(f"{what}: expected {len(self._sizes)} arrays, got {len(arrays)}")
        out = np.empty(rows * int(self._start[-1]), np.float32)
        for b, a in enumerate(arrays):
            a = np.asarray(a)
            if a.dtype != np.float32:
                raise ValueError(f"{what}[{b}]: expected float32, got {a.dtype}")
            if a.shape != (rows, self._sizes[b]):
                raise ValueError(f"{what}[{b}]: need shape {(rows, self._sizes[b])}, got {a.shape}")
            out[rows * self._start[b]:rows * self._start[b + 1]] = a.reshape(-1)
        return out

    def _unpack(self, flat: np.ndarray, rows: int):
        return [flat[rows * self._start[b]:rows * self._start[b + 1]].reshape(rows, n)
                for b, n in enumerate(self._sizes)]

    # -- configuration ------------------------------------------------------------
    def set_variant(self, variant: int) -> None:
        _lib.check(_lib.load().dcrf_set_variant(self._h, int(variant)))

    def setUnaryEnergy(self, unaries) -> None:
        """One (M, N_b) float32 unary per image."""
        U = self._pack(unaries, self._nlabel, "unary")
        _lib.check(_lib.load().dcrf_set_unary(self._h, _ptr(U), _lib.LAYOUT_LM, _lib.HOST))

    def addPairwiseEnergy(self, features, compat, kernel=DIAG_KERNEL, normalization=NORMALIZE_SYMMETRIC):
        """One (d, N_b) float32 feature array per image, the same d for all."""
        if len(features) != len(self._sizes):
            raise ValueError(f"features: expected {len(self._sizes)} arrays, got {len(features)}")
        d = int(np.asarray(features[0]).shape[0])
        F = self._pack(features, d, "features")
        # the engine takes features as (d, N) over all points: regroup per dimension
        F = np.ascontiguousarray(np.concatenate(
            [F[d * self._start[b]:d * self._start[b + 1]].reshape(d, n) for b, n in enumerate(self._sizes)], axis=1))
        kernel = _check_enum(kernel, 0, 2, "KernelType")
        normalization = _check_enum(normalization, 0, 3, "NormalizationType")
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_add_pairwise(self._h, _ptr(F), d, _lib.HOST, kind, _ptr(c), kernel,
                                                 normalization, None))

    def setCompatibility(self, term: int, compat) -> None:
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_set_compat(self._h, int(term), kind, _ptr(c)))

    def setKernelParameters(self, term: int, params) -> None:
        p = np.ascontiguousarray(np.asarray(params, np.float32).reshape(-1))
        _lib.check(_lib.load().dcrf_set_kernel_params(self._h, int(term), _ptr(p)))

    def paramCounts(self, term: int):
        nc, nk = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.load().dcrf_param_counts(self._h, int(term), ctypes.byref(nc), ctypes.byref(nk)))
        return nc.value, nk.value

    def nTerms(self) -> int:
        n = ctypes.c_int()
        _lib.check(_lib.load().dcrf_info(self._h, None, None, ctypes.byref(n)))
        return n.value

    # -- autotuning --------------------------------------------------------------------
    set_autotune = DenseCRF.set_autotune
    autotune = DenseCRF.autotune
    tuning = DenseCRF.tuning
    set_tuning = DenseCRF.set_tuning
    setCheckpointInterval = DenseCRF.setCheckpointInterval

    # -- inference ------------------------------------------------------------------
    def _flat(self) -> np.ndarray:
        return np.empty(self._nlabel * int(self._start[-1]), np.float32)

    def inference(self, niter: int):
        """Marginals after ``niter`` iterations: one (M, N_b) array per image."""
        Q = self._flat()
        _lib.check(_lib.load().dcrf_inference(self._h, int(niter), _ptr(Q), _lib.LAYOUT_LM, _lib.HOST))
        return self._unpack(Q, self._nlabel)

    def map(self, niter: int):
        """Argmax labels after ``niter`` iterations: one int16 array per image."""
        out = np.empty(int(self._start[-1]), np.int16)
        _lib.check(_lib.load().dcrf_map(self._h, int(niter), _ptr(out), _lib.HOST))
        return [out[self._start[b]:self._start[b + 1]] for b in range(len(self._sizes))]

    def klDivergence(self, Q) -> float:
        """Sum over the images of DenseCRF::klDivergence (densecrf.cpp:214-235)."""
        data = self._pack(Q, self._nlabel, "Q")
        out = ctypes.c_double()
        _lib.check(_lib.load().dcrf_kl_divergence(self._h, _ptr(data), _lib.LAYOUT_LM, _lib.HOST, ctypes.byref(out)))
        return out.value

    def inferenceCheckpointed(self, niter: int):
        Q = self._flat()
        _lib.check(_lib.load().dcrf_inference_checkpointed(self._h, int(niter), _ptr(Q), _lib.LAYOUT_LM, _lib.HOST))
        return self._unpack(Q, self._nlabel)

    def backward(self, dQ, want_compat: bool = True, want_kernel: bool = False):
        """Adjoint of the last inferenceCheckpointed: given one dL/dQ (M, N_b) per
        image, returns (per-image dL/dU, per-term dL/dcompat, per-term dL/dkernel);
        parameter gradients are summed over the images."""
        g = self._pack(dQ, self._nlabel, "dQ")
        dU = np.empty_like(g)
        counts = [self.paramCounts(k) for k in range(self.nTerms())]
        dc = np.zeros(max(1, sum(c for c, _ in counts)), np.float64) if want_compat else None
        dk = np.zeros(max(1, sum(k for _, k in counts)), np.float64) if want_kernel else None
        _lib.check(_lib.load().dcrf_backward(self._h, _ptr(g), _lib.LAYOUT_LM, _lib.HOST, _ptr(dU),
                                             _ptr(dc) if dc is not None else None,
                                             _ptr(dk) if dk is not None else None))
        cs, ks, oc, ok = [], [], 0, 0
        for c, k in counts:
            cs.append(dc[oc:oc + c].copy() if dc is not None else None)
            ks.append(dk[ok:ok + k].copy() if dk is not None else None)
            oc += c
            ok += k
        return self._unpack(dU, self._nlabel), cs, ks


class DenseCRF2DBatch(DenseCRFBatch):
    """Dense CRFs over ``widths[b] x heights[b]`` pixel grids."""

    def __init__(self, widths, heights, nlabels: int):
        self._wh = [(int(w), int(h)) for w, h in zip(widths, heights)]
        if len(self._wh) != len(widths) or len(widths) != len(heights):
            raise ValueError("widths and heights must have the same length")
        super().__init__([w * h for w, h in self._wh], nlabels)
        W = np.ascontiguousarray([w for w, _ in self._wh], np.int32)
        H = np.ascontiguousarray([h for _, h in self._wh], np.int32)
        _lib.check(_lib.load().dcrf_create_batch_2d(len(self._wh), _ptr(W), _ptr(H), self._nlabel,
                                                    ctypes.byref(self._h)))

    def addPairwiseGaussian(self, sxy, compat, kernel=DIAG_KERNEL, normalization=NORMALIZE_SYMMETRIC):
        """DenseCRF2D.addPairwiseGaussian for every image."""
        if isinstance(sxy, Number):
            sxy = (sxy, sxy)
        kernel = _check_enum(kernel, 0, 2, "KernelType")
        normalization = _check_enum(normalization, 0, 3, "NormalizationType")
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_add_pairwise_gaussian(self._h, float(sxy[0]), float(sxy[1]), kind, _ptr(c),
                                                          kernel, normalization, None))

    def addPairwiseBilateral(self, sxy, srgb, rgbims, compat, kernel=DIAG_KERNEL, normalization=NORMALIZE_SYMMETRIC):
        """DenseCRF2D.addPairwiseBilateral with one (H_b, W_b, 3) uint8 image per image."""
        if isinstance(sxy, Number):
            sxy = (sxy, sxy)
        if isinstance(srgb, Number):
            srgb = (srgb, srgb, srgb)
        if len(rgbims) != len(self._wh):
            raise ValueError(f"expected {len(self._wh)} images, got {len(rgbims)}")
        parts = []
        for b, im in enumerate(rgbims):
            im = np.asarray(im)
            if im.dtype != np.uint8:
                raise ValueError(f"image {b}: expected uint8, got {im.dtype}")
            w, h = self._wh[b]
            if im.shape != (h, w, 3):
                raise ValueError(f"image {b}: need shape {(h, w, 3)}, got {im.shape}")
            parts.append(im.reshape(-1))
        img = np.ascontiguousarray(np.concatenate(parts))
        kernel = _check_enum(kernel, 0, 2, "KernelType")
        normalization = _check_enum(normalization, 0, 3, "NormalizationType")
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_add_pairwise_bilateral(
            self._h, float(sxy[0]), float(sxy[1]), float(srgb[0]), float(srgb[1]), float(srgb[2]), _ptr(img),
            _lib.HOST, kind, _ptr(c), kernel, normalization, None))
