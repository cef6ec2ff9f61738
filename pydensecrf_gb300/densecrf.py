"""Drop-in for ``pydensecrf.densecrf`` backed by the GB300 engine.

Same classes, methods, defaults, enums and argument checks as the reference's
Cython module (pydensecrf/densecrf.pyx, pydensecrf/densecrf.pxd); every call
goes through the C ABI of include/dcrf.h to hand-written sm_103a kernels.
Marginals come back as :class:`pydensecrf_gb300.eigen.MatrixXf` with the
reference's memory layout (column-major ``M x N``).
"""
from __future__ import annotations

import ctypes
from numbers import Number

import numpy as np

from . import _lib
from .eigen import MatrixXf, as_float_buffer

# enums of pydensecrf/densecrf/include/pairwise.h:32-42 (densecrf.pxd:43-44)
NO_NORMALIZATION = 0
NORMALIZE_BEFORE = 1
NORMALIZE_AFTER = 2
NORMALIZE_SYMMETRIC = 3
CONST_KERNEL = 0
DIAG_KERNEL = 1
FULL_KERNEL = 2


class NormalizationType(int):
    NO_NORMALIZATION = NO_NORMALIZATION
    NORMALIZE_BEFORE = NORMALIZE_BEFORE
    NORMALIZE_AFTER = NORMALIZE_AFTER
    NORMALIZE_SYMMETRIC = NORMALIZE_SYMMETRIC


class KernelType(int):
    CONST_KERNEL = CONST_KERNEL
    DIAG_KERNEL = DIAG_KERNEL
    FULL_KERNEL = FULL_KERNEL


def _cuda_tensor(x) -> bool:
    """A torch tensor on a CUDA device (used in place, no host copy)."""
    try:
        import torch
    except ImportError:
        return False
    return isinstance(x, torch.Tensor) and x.is_cuda


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _labelcomp(compat, M: int):
    """Compatibility dispatch of densecrf.pyx:11-20 -> (kind, float32 buffer).

    A Number gives Potts, a 1-D float32 buffer Diagonal, a 2-D float32 buffer
    Matrix; other dtypes raise ValueError like the typed memoryviews do.
    """
    if isinstance(compat, Number):
        return _lib.COMPAT_POTTS, np.array([float(compat)], dtype=np.float32)
    ndim = memoryview(compat).ndim
    if ndim == 1:
        c = as_float_buffer(compat, 1, "compat")
        if c.shape[0] != M:
            raise ValueError(f"Diagonal compatibility needs {M} entries, got {c.shape[0]}")
        return _lib.COMPAT_DIAGONAL, np.ascontiguousarray(c, np.float32)
    if ndim == 2:
        c = as_float_buffer(compat, 2, "compat")
        if c.shape != (M, M):
            raise ValueError(f"Matrix compatibility needs shape {(M, M)}, got {c.shape}")
        return _lib.COMPAT_MATRIX, np.ascontiguousarray(c, np.float32)
    raise ValueError("LabelCompatibility of dimension >2 not meaningful.")


def _check_enum(v, lo, hi, what):
    if not isinstance(v, (int, np.integer)) or not (lo <= int(v) <= hi):
        raise TypeError(f"{what} must be one of the {what} constants")
    return int(v)


class Unary:
    """Base of the unary holders (densecrf.pyx:23-36)."""

    def _matrix(self, M: int, N: int) -> np.ndarray:
        raise NotImplementedError


class ConstUnary(Unary):
    """Constant unary energy (densecrf.pyx:39-41, unary.cpp:42-46)."""

    def __init__(self, u):
        self.u = np.array(as_float_buffer(u, 2, "u"), dtype=np.float32, copy=True)

    def _matrix(self, M, N):
        return self.u


class LogisticUnary(Unary):
    """Logistic unary energy U = L f (densecrf.pyx:44-46, unary.cpp:48-52),
    computed on the device by the engine."""

    def __init__(self, L, f):
        self.L = np.array(as_float_buffer(L, 2, "L"), dtype=np.float32, copy=True)
        self.f = np.array(as_float_buffer(f, 2, "f"), dtype=np.float32, copy=True)


class DenseCRF:
    """Fully connected CRF over ``nvar`` variables and ``nlabels`` labels
    (densecrf.pyx:49-101 -> densecrf.cpp)."""

    def __init__(self, nvar: int, nlabels: int, *_, **__):
        self._nvar = int(nvar)
        self._nlabel = int(nlabels)
        self._h = ctypes.c_void_p()
        if type(self) is DenseCRF:
            lib = _lib.load()
            _lib.check(lib.dcrf_create(self._nvar, self._nlabel, ctypes.byref(self._h)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _lib.load().dcrf_destroy(h)
            except Exception:
                pass
            h.value = None

    def _bind_torch_stream(self) -> None:
        """Order the handle's work on torch's current stream, so device tensors
        written by torch are complete when the engine reads them."""
        import torch
        st = torch.cuda.current_stream().cuda_stream
        if getattr(self, "_stream", None) != st:
            _lib.check(_lib.load().dcrf_set_stream(self._h, ctypes.c_void_p(st)))
            self._stream = st

    def _device_matrix(self, t, rows: int, what: str):
        import torch
        if t.dtype != torch.float32 or t.dim() != 2 or t.shape[0] != rows or t.shape[1] != self._nvar:
            raise ValueError(f"{what}: need a float32 CUDA tensor of shape {(rows, self._nvar)}, got "
                             f"{tuple(t.shape)} {t.dtype}")
        self._bind_torch_stream()
        return t.contiguous()

    # -- configuration ------------------------------------------------------
    def set_variant(self, variant: int) -> None:
        """Lattice arithmetic of the x86 (0, default) or scalar (1) reference build."""
        _lib.check(_lib.load().dcrf_set_variant(self._h, int(variant)))

    def addPairwiseEnergy(self, features, compat, kernel=DIAG_KERNEL, normalization=NORMALIZE_SYMMETRIC):
        """densecrf.pyx:71-75.  ``features`` may be a (d, N) float32 CUDA tensor."""
        if _cuda_tensor(features):
            t = features
            if t.dim() != 2 or t.shape[1] != self._nvar:
                raise ValueError("Bad shape for pairwise energy (Need (?, {}), got {})".format(self._nvar,
                                                                                         tuple(t.shape)))
            t = self._device_matrix(t, t.shape[0], "features")
            kernel = _check_enum(kernel, 0, 2, "KernelType")
            normalization = _check_enum(normalization, 0, 3, "NormalizationType")
            kind, c = _labelcomp(compat, self._nlabel)
            _lib.check(_lib.load().dcrf_add_pairwise(self._h, ctypes.c_void_p(t.data_ptr()), t.shape[0],
                                                     _lib.DEVICE, kind, _ptr(c), kernel, normalization, None))
            return
        feat = as_float_buffer(features, 2, "features")
        kernel = _check_enum(kernel, 0, 2, "KernelType")
        normalization = _check_enum(normalization, 0, 3, "NormalizationType")
        if feat.shape[1] != self._nvar:
            raise ValueError("Bad shape for pairwise energy (Need (?, {}), got {})".format(
                self._nvar, (feat.shape[0], feat.shape[1])))
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_add_pairwise(self._h, _ptr(feat), feat.shape[0], _lib.HOST, kind, _ptr(c),
                                                 kernel, normalization, None))

    def setUnary(self, u: Unary) -> None:
        """densecrf.pyx:77-78."""
        if not isinstance(u, Unary):
            raise TypeError("Argument 'u' has incorrect type (expected Unary)")
        if isinstance(u, LogisticUnary):
            self._set_logistic(u.L, u.f)
        else:
            self._set_unary_matrix(u._matrix(self._nlabel, self._nvar))

    def _set_logistic(self, L: np.ndarray, f: np.ndarray) -> None:
        """LogisticUnaryEnergy(L, f) (unary.cpp:48-52): L is (M, K), f is (K, N)."""
        L = np.ascontiguousarray(L, np.float32)
        f = np.ascontiguousarray(f, np.float32)
        if L.shape[0] != self._nlabel or f.shape != (L.shape[1], self._nvar):
            raise ValueError("Bad shape for logistic unary energy (Need L ({}, K), f (K, {}); got {} and {})".format(
                self._nlabel, self._nvar, L.shape, f.shape))
        _lib.check(_lib.load().dcrf_set_unary_logistic(self._h, _ptr(L), L.shape[1], _ptr(f), _lib.HOST))

    def setUnaryEnergy(self, u, f=None) -> None:
        """densecrf.pyx:80-89; with ``f`` the unary is logistic, U = u f.  ``u``
        may be an (M, N) float32 CUDA tensor (used in place)."""
        if f is None and _cuda_tensor(u):
            t = self._device_matrix(u, self._nlabel, "unary")
            _lib.check(_lib.load().dcrf_set_unary(self._h, ctypes.c_void_p(t.data_ptr()), _lib.LAYOUT_LM,
                                                  _lib.DEVICE))
            return
        u = as_float_buffer(u, 2, "u")
        if u.shape[0] != self._nlabel or (f is None and u.shape[1] != self._nvar):
            raise ValueError("Bad shape for unary energy (Need {}, got {})".format(
                (self._nlabel, self._nvar), (u.shape[0], u.shape[1])))
        if f is None:
            self._set_unary_matrix(u)
        else:
            self._set_logistic(u, as_float_buffer(f, 2, "f"))

    def _set_unary_matrix(self, U: np.ndarray) -> None:
        U = np.ascontiguousarray(U, dtype=np.float32)
        if U.shape != (self._nlabel, self._nvar):
            raise ValueError("Bad shape for unary energy (Need {}, got {})".format(
                (self._nlabel, self._nvar), U.shape))
        _lib.check(_lib.load().dcrf_set_unary(self._h, _ptr(U), _lib.LAYOUT_LM, _lib.HOST))

    # -- inference -------------------------------------------------------------
    def _new_q(self) -> np.ndarray:
        return np.empty((self._nvar, self._nlabel), np.float32)

    def inference(self, niter: int) -> MatrixXf:
        """densecrf.pyx:91-92."""
        Q = self._new_q()
        _lib.check(_lib.load().dcrf_inference(self._h, int(niter), _ptr(Q), _lib.LAYOUT_PM, _lib.HOST))
        return MatrixXf().wrap_colmajor(Q)

    def inference_tensor(self, niter: int):
        """inference(niter) into a new (M, N) float32 CUDA tensor on torch's current stream."""
        import torch
        self._bind_torch_stream()
        Q = torch.empty((self._nlabel, self._nvar), dtype=torch.float32, device="cuda")
        _lib.check(_lib.load().dcrf_inference(self._h, int(niter), ctypes.c_void_p(Q.data_ptr()), _lib.LAYOUT_LM,
                                              _lib.DEVICE))
        return Q

    def startInference(self):
        """densecrf.pyx:94-95: (Q, tmp1, tmp2)."""
        Q = self._new_q()
        _lib.check(_lib.load().dcrf_start_inference(self._h, _ptr(Q), _lib.LAYOUT_PM, _lib.HOST))
        return MatrixXf().wrap_colmajor(Q), MatrixXf(), MatrixXf()

    def stepInference(self, Q: MatrixXf, tmp1: MatrixXf, tmp2: MatrixXf) -> None:
        """densecrf.pyx:97-98: one mean-field update of Q, in place."""
        if not isinstance(Q, MatrixXf):
            raise TypeError("Argument 'Q' has incorrect type (expected MatrixXf)")
        if Q.shape != (self._nlabel, self._nvar):
            raise ValueError(f"Q must have shape {(self._nlabel, self._nvar)}, got {Q.shape}")
        _lib.check(_lib.load().dcrf_step_inference(self._h, _ptr(Q.data), _lib.LAYOUT_PM, _lib.HOST))

    def klDivergence(self, Q) -> float:
        """densecrf.pyx:100-101."""
        if isinstance(Q, MatrixXf):
            data, layout = Q.data, _lib.LAYOUT_PM
        else:
            data, layout = np.ascontiguousarray(np.asarray(Q, np.float32)), _lib.LAYOUT_LM
        if (data.size != self._nlabel * self._nvar):
            raise ValueError("Q has the wrong size")
        out = ctypes.c_double()
        _lib.check(_lib.load().dcrf_kl_divergence(self._h, _ptr(data), layout, _lib.HOST, ctypes.byref(out)))
        return out.value

    def map(self, niter: int) -> np.ndarray:
        """DenseCRF::map (densecrf.cpp:132-137): argmax labels after niter iterations."""
        out = np.empty(self._nvar, np.int16)
        _lib.check(_lib.load().dcrf_map(self._h, int(niter), _ptr(out), _lib.HOST))
        return out

    # -- debug energies (densecrf.cpp:141-177; C++ only in the reference) --------
    def _labels(self, labels) -> np.ndarray:
        lab = np.ascontiguousarray(np.asarray(labels).reshape(-1), np.int16)
        if lab.size != self._nvar:
            raise ValueError(f"labels must have {self._nvar} entries, got {lab.size}")
        return lab

    def unaryEnergy(self, labels) -> np.ndarray:
        """U(l_i, i) per variable (0 where l_i is not a label)."""
        lab = self._labels(labels)
        out = np.empty(self._nvar, np.float32)
        _lib.check(_lib.load().dcrf_unary_energy(self._h, _ptr(lab), _lib.HOST, _ptr(out), _lib.HOST))
        return out

    def pairwiseEnergy(self, labels, term: int = -1) -> np.ndarray:
        """-1/2 the pairwise message of the one-hot labelling at l_i (term -1: all terms)."""
        lab = self._labels(labels)
        out = np.empty(self._nvar, np.float32)
        _lib.check(_lib.load().dcrf_pairwise_energy(self._h, _ptr(lab), _lib.HOST, int(term), _ptr(out), _lib.HOST))
        return out

    # -- autotuning (no reference counterpart) -----------------------------------
    def set_autotune(self, on: bool = True) -> None:
        """Tune the engine's launch and build knobs at the first inference of
        every new configuration (remembered for the process)."""
        _lib.check(_lib.load().dcrf_set_autotune(self._h, int(bool(on))))

    def autotune(self) -> dict:
        """Tune now for the current pairwise terms; returns the chosen knobs."""
        _lib.check(_lib.load().dcrf_autotune(self._h))
        return self.tuning()

    def tuning(self) -> dict:
        sp, sm, tk, hl, co = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()
        _lib.check(_lib.load().dcrf_get_tuning(self._h, ctypes.byref(sp), ctypes.byref(sm), ctypes.byref(tk),
                                               ctypes.byref(hl), ctypes.byref(co)))
        return {"split": sp.value, "smem_kb": sm.value, "task_len": tk.value, "hash_load": hl.value,
                "coop_blur": co.value}

    def set_tuning(self, split: int = 0, smem_kb: int = 0, task_len: int = 24, hash_load: float = 2.0,
                   coop_blur: int = 0) -> None:
        _lib.check(_lib.load().dcrf_set_tuning(self._h, int(split), int(smem_kb), int(task_len), float(hash_load),
                                               int(coop_blur)))

    # -- learning (the parameter API and adjoint of densecrf.cpp:238-360) -------
    def setCompatibility(self, term: int, compat) -> None:
        """Replace term ``term``'s label compatibility (Potts number, Diagonal
        vector or Matrix), like LabelCompatibility::setParameters."""
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_set_compat(self._h, int(term), kind, _ptr(c)))

    def setKernelParameters(self, *args) -> None:
        """``setKernelParameters(v)``: DenseCRF::setKernelParameters
        (densecrf.cpp:348-360), the concatenation over the terms of DIAG
        scales / FULL d x d matrices in column-major order, as kernelParameters()
        returns it.  ``setKernelParameters(term, params)``: one term's
        parameters (DenseKernel::setParameters, pairwise.cpp:140-151): DIAG d
        feature scales, FULL a d x d matrix (row-major, features become P f).
        Either rebuilds the lattices."""
        if len(args) == 1:
            v = np.ascontiguousarray(np.asarray(args[0], np.float32).reshape(-1))
            _lib.check(_lib.load().dcrf_set_kernel_parameters(self._h, _ptr(v), int(v.size)))
            return
        if len(args) != 2:
            raise TypeError("setKernelParameters(v) or setKernelParameters(term, params)")
        term, params = args
        p = np.ascontiguousarray(np.asarray(params, np.float32).reshape(-1))
        _lib.check(_lib.load().dcrf_set_kernel_params(self._h, int(term), _ptr(p)))

    def _vector(self, fn) -> np.ndarray:
        n = ctypes.c_int()
        _lib.check(fn(self._h, None, 0, ctypes.byref(n)))
        out = np.empty(n.value, np.float32)
        if n.value:
            _lib.check(fn(self._h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def _set_vector(self, fn, v) -> None:
        v = np.ascontiguousarray(np.asarray(v, np.float32).reshape(-1))
        _lib.check(fn(self._h, _ptr(v) if v.size else None, int(v.size)))

    def unaryParameters(self) -> np.ndarray:
        """DenseCRF::unaryParameters (densecrf.cpp:298-302): a logistic unary's L
        in column-major order; empty for a constant unary."""
        return self._vector(_lib.load().dcrf_unary_parameters)

    def setUnaryParameters(self, v) -> None:
        """DenseCRF::setUnaryParameters (densecrf.cpp:303-306)."""
        self._set_vector(_lib.load().dcrf_set_unary_parameters, v)

    def labelCompatibilityParameters(self) -> np.ndarray:
        """DenseCRF::labelCompatibilityParameters (densecrf.cpp:307-320): per term
        Potts w / the Diagonal weights / the Matrix's packed upper triangle."""
        return self._vector(_lib.load().dcrf_label_compatibility_parameters)

    def setLabelCompatibilityParameters(self, v) -> None:
        """DenseCRF::setLabelCompatibilityParameters (densecrf.cpp:321-333)."""
        self._set_vector(_lib.load().dcrf_set_label_compatibility_parameters, v)

    def kernelParameters(self) -> np.ndarray:
        """DenseCRF::kernelParameters (densecrf.cpp:334-347)."""
        return self._vector(_lib.load().dcrf_kernel_parameters)

    def unaryParameterGradient(self) -> np.ndarray:
        """After backward(): dL/d(unaryParameters()) = (dL/dU) f^T for a logistic
        unary (LogisticUnaryEnergy::gradient summed over the iterations,
        unary.cpp:64-67); empty for a constant unary."""
        n = ctypes.c_int()
        lib = _lib.load()
        _lib.check(lib.dcrf_unary_gradient(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.float64)
        if n.value:
            _lib.check(lib.dcrf_unary_gradient(self._h, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def paramCounts(self, term: int):
        """(number of compatibility values, number of kernel parameters) of a term."""
        nc, nk = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.load().dcrf_param_counts(self._h, int(term), ctypes.byref(nc), ctypes.byref(nk)))
        return nc.value, nk.value

    def nTerms(self) -> int:
        n = ctypes.c_int()
        _lib.check(_lib.load().dcrf_info(self._h, None, None, ctypes.byref(n)))
        return n.value

    def setCheckpointInterval(self, every: int) -> None:
        """Keep every ``every``-th iterate in inferenceCheckpointed and recompute
        the others segment by segment in backward() (1: keep all)."""
        _lib.check(_lib.load().dcrf_set_checkpoint_interval(self._h, int(every)))

    def inferenceCheckpointed(self, niter: int) -> np.ndarray:
        """inference(niter) keeping every iterate on the device for backward();
        returns Q as an (M, N) array."""
        Q = np.empty((self._nlabel, self._nvar), np.float32)
        _lib.check(_lib.load().dcrf_inference_checkpointed(self._h, int(niter), _ptr(Q), _lib.LAYOUT_LM,
                                                           _lib.HOST))
        return Q

    def backward(self, dQ, want_compat: bool = True, want_kernel: bool = False):
        """Adjoint of the last inferenceCheckpointed: given dL/dQ (M, N), returns
        (dL/dU (M, N), [per-term dL/dcompat], [per-term dL/dkernel params])."""
        dQ = np.ascontiguousarray(dQ, np.float32)
        dU = np.empty_like(dQ)
        counts = [self.paramCounts(k) for k in range(self.nTerms())]
        dc = np.zeros(max(1, sum(c for c, _ in counts)), np.float64) if want_compat else None
        dk = np.zeros(max(1, sum(k for _, k in counts)), np.float64) if want_kernel else None
        _lib.check(_lib.load().dcrf_backward(self._h, _ptr(dQ), _lib.LAYOUT_LM, _lib.HOST, _ptr(dU),
                                             _ptr(dc) if dc is not None else None,
                                             _ptr(dk) if dk is not None else None))
        cs, ks, oc, ok = [], [], 0, 0
        for c, k in counts:
            cs.append(dc[oc:oc + c].copy() if dc is not None else None)
            ks.append(dk[ok:ok + k].copy() if dk is not None else None)
            oc += c
            ok += k
        return dU, cs, ks

    # -- introspection -----------------------------------------------------------
    def lattice(self, term: int) -> dict:
        """Lattice tables of pairwise term ``term`` in the reference's layout."""
        lib = _lib.load()
        d, L = ctypes.c_int(), ctypes.c_int()
        _lib.check(lib.dcrf_lattice_info(self._h, term, ctypes.byref(d), ctypes.byref(L)))
        d, L, N = d.value, L.value, self._nvar
        out = dict(offset=np.empty((N, d + 1), np.int32), rank=np.empty((N, d + 1), np.int32),
                   bary=np.empty((N, d + 1), np.float32), neighbors=np.empty((d + 1, L, 2), np.int32),
                   keys=np.empty((L, d), np.int16), L=L, d=d)
        _lib.check(lib.dcrf_lattice_dump(self._h, term, _ptr(out["offset"]), _ptr(out["rank"]), _ptr(out["bary"]),
                                         _ptr(out["neighbors"]), _ptr(out["keys"])))
        return out

    def term_norm(self, term: int) -> np.ndarray:
        out = np.empty(self._nvar, np.float32)
        _lib.check(_lib.load().dcrf_term_norm(self._h, term, _ptr(out)))
        return out

    def lattice_filter(self, term: int, values: np.ndarray, reverse: bool = False) -> np.ndarray:
        """Raw lattice filter K v of term ``term``; values is (value_size, N)."""
        v = np.ascontiguousarray(values, np.float32)
        out = np.empty_like(v)
        _lib.check(_lib.load().dcrf_lattice_filter(self._h, term, _ptr(v), v.shape[0], int(bool(reverse)),
                                                   _ptr(out)))
        return out


class DenseCRF2D(DenseCRF):
    """CRF over a W x H pixel grid (densecrf.pyx:104-140)."""

    def __init__(self, w: int, h: int, nlabels: int, *_, **__):
        super().__init__(int(w) * int(h), nlabels)
        self._w = int(w)
        self._h2 = int(h)
        if type(self) is DenseCRF2D:
            lib = _lib.load()
            _lib.check(lib.dcrf_create_2d(self._w, self._h2, self._nlabel, ctypes.byref(self._h)))

    def addPairwiseGaussian(self, sxy, compat, kernel=DIAG_KERNEL, normalization=NORMALIZE_SYMMETRIC):
        """densecrf.pyx:120-124."""
        if isinstance(sxy, Number):
            sxy = (sxy, sxy)
        kernel = _check_enum(kernel, 0, 2, "KernelType")
        normalization = _check_enum(normalization, 0, 3, "NormalizationType")
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_add_pairwise_gaussian(self._h, float(sxy[0]), float(sxy[1]), kind, _ptr(c),
                                                          kernel, normalization, None))

    def addPairwiseBilateral(self, sxy, srgb, rgbim, compat, kernel=DIAG_KERNEL, normalization=NORMALIZE_SYMMETRIC):
        """densecrf.pyx:126-140."""
        if isinstance(sxy, Number):
            sxy = (sxy, sxy)
        if isinstance(srgb, Number):
            srgb = (srgb, srgb, srgb)
        if rgbim is None:
            raise TypeError("rgbim must not be None")
        if _cuda_tensor(rgbim):
            import torch
            if rgbim.dtype != torch.uint8 or tuple(rgbim.shape) != (self._h2, self._w, 3):
                raise ValueError("Bad shape for pairwise bilateral (Need {}, got {} {})".format(
                    (self._h2, self._w, 3), tuple(rgbim.shape), rgbim.dtype))
            self._bind_torch_stream()
            img = rgbim.contiguous()
            kernel = _check_enum(kernel, 0, 2, "KernelType")
            normalization = _check_enum(normalization, 0, 3, "NormalizationType")
            kind, c = _labelcomp(compat, self._nlabel)
            _lib.check(_lib.load().dcrf_add_pairwise_bilateral(
                self._h, float(sxy[0]), float(sxy[1]), float(srgb[0]), float(srgb[1]), float(srgb[2]),
                ctypes.c_void_p(img.data_ptr()), _lib.DEVICE, kind, _ptr(c), kernel, normalization, None))
            return
        mv = memoryview(rgbim)
        if mv.format not in ("B", "=B", "<B", "@B"):
            raise ValueError(f"Buffer dtype mismatch, expected 'unsigned char' but got '{mv.format}'")
        if mv.ndim != 3:
            raise ValueError(f"Buffer has wrong number of dimensions (expected 3, got {mv.ndim})")
        if not mv.c_contiguous:
            raise ValueError("ndarray is not C-contiguous")
        img = np.asarray(rgbim)
        if img.shape[0] != self._h2 or img.shape[1] != self._w:
            raise ValueError("Bad shape for pairwise bilateral (Need {}, got {})".format(
                (self._h2, self._w, 3), img.shape))
        if img.shape[2] != 3:
            raise ValueError("addPairwiseBilateral only works for RGB images. For other types, use "
                             "`utils.create_pairwise_bilateral` to construct your own pairwise energy and add it "
                             "through `addPairwiseEnergy`.")
        kernel = _check_enum(kernel, 0, 2, "KernelType")
        normalization = _check_enum(normalization, 0, 3, "NormalizationType")
        kind, c = _labelcomp(compat, self._nlabel)
        _lib.check(_lib.load().dcrf_add_pairwise_bilateral(
            self._h, float(sxy[0]), float(sxy[1]), float(srgb[0]), float(srgb[1]), float(srgb[2]), _ptr(img),
            _lib.HOST, kind, _ptr(c), kernel, normalization, None))
