"""Differentiable mean-field inference (torch.autograd) over the GB300 engine.

``mean_field(crf, U, T, compat=..., kernel_params=...)`` runs T mean-field
iterations of a built :class:`~pydensecrf_gb300.densecrf.DenseCRF` with
per-iteration checkpoints on the device and returns Q; its backward is the
hand-written adjoint of the iterations (the device form of
DenseCRF::gradient, pydensecrf/densecrf/src/densecrf.cpp:238-297), giving
gradients with respect to

* the unary U,
* each term's label compatibility (Potts weight, Diagonal vector, or the raw
  Matrix m -- the engine uses W = (m + m^T)/2),
* each term's kernel parameters (DIAG feature scales p / FULL matrix P, at
  their current values; a bandwidth s of features x/s has dL/ds = -(1/s) *
  sum of dL/dp over the feature dimensions that use s).

Tensors live on the GPU; U is (M, N) float32 (labels major).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .densecrf import _labelcomp

__all__ = ["mean_field", "bandwidth_grad"]


def _ptr(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


class _MeanField(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U, T, crf, n_compat, n_kernel, *params):
        lib = _lib.load()
        h = crf._h
        nt = crf.nTerms()
        compats, kparams = params[:n_compat], params[n_compat:n_compat + n_kernel]
        for k, c in enumerate(compats):
            if c is None:
                continue
            cc = c.detach().float().cpu().numpy()
            kind, buf = _labelcomp(float(cc) if cc.ndim == 0 else np.ascontiguousarray(cc), crf._nlabel)
            _lib.check(lib.dcrf_set_compat(h, k, kind, ctypes.c_void_p(buf.ctypes.data)))
        for k, p in enumerate(kparams):
            if p is None:
                continue
            pp = np.ascontiguousarray(p.detach().float().cpu().numpy().reshape(-1), np.float32)
            _lib.check(lib.dcrf_set_kernel_params(h, k, ctypes.c_void_p(pp.ctypes.data)))
        Uc = U.detach().contiguous().float()
        stream = torch.cuda.current_stream(Uc.device)
        _lib.check(lib.dcrf_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
        _lib.check(lib.dcrf_set_unary(h, _ptr(Uc), _lib.LAYOUT_LM, _lib.DEVICE))
        Q = torch.empty_like(Uc)
        _lib.check(lib.dcrf_inference_checkpointed(h, int(T), _ptr(Q), _lib.LAYOUT_LM, _lib.DEVICE))
        ctx.crf = crf
        ctx.n_compat, ctx.n_kernel, ctx.nt = n_compat, n_kernel, nt
        ctx.param_shapes = [None if p is None else (p.shape, p.dtype, p.device) for p in params]
        ctx.compat_kinds = [None if c is None else c.dim() for c in compats]
        return Q

    @staticmethod
    def backward(ctx, dQ):
        lib = _lib.load()
        crf = ctx.crf
        h = crf._h
        need_u = ctx.needs_input_grad[0]
        need_c = any(ctx.needs_input_grad[5:5 + ctx.n_compat])
        need_k = any(ctx.needs_input_grad[5 + ctx.n_compat:5 + ctx.n_compat + ctx.n_kernel])
        dQc = dQ.detach().contiguous().float()
        dU = torch.empty_like(dQc)
        counts = [crf.paramCounts(k) for k in range(ctx.nt)]
        dc = np.zeros(max(1, sum(c for c, _ in counts)), np.float64)
        dk = np.zeros(max(1, sum(k for _, k in counts)), np.float64)
        _lib.check(lib.dcrf_backward(h, _ptr(dQc), _lib.LAYOUT_LM, _lib.DEVICE, _ptr(dU),
                                     ctypes.c_void_p(dc.ctypes.data) if need_c else None,
                                     ctypes.c_void_p(dk.ctypes.data) if need_k else None))
        grads = [dU if need_u else None, None, None, None, None]
        oc = ok = 0
        for k in range(ctx.n_compat):
            nc, nk = counts[k] if k < len(counts) else (0, 0)
            shp = ctx.param_shapes[k]
            if shp is None or not ctx.needs_input_grad[5 + k]:
                grads.append(None)
            else:
                g = dc[oc:oc + nc]
                if ctx.compat_kinds[k] == 2:  # raw m, W = (m + m^T)/2
                    M = crf._nlabel
                    G = g.reshape(M, M)
                    g = 0.5 * (G + G.T)
                grads.append(torch.as_tensor(np.asarray(g).reshape(shp[0]), dtype=shp[1], device=shp[2]))
            oc += nc
        for k in range(ctx.n_kernel):
            nc, nk = counts[k] if k < len(counts) else (0, 0)
            shp = ctx.param_shapes[ctx.n_compat + k]
            if shp is None or not ctx.needs_input_grad[5 + ctx.n_compat + k]:
                grads.append(None)
            else:
                grads.append(torch.as_tensor(dk[ok:ok + nk].reshape(shp[0]), dtype=shp[1], device=shp[2]))
            ok += nk
        return tuple(grads)


def mean_field(crf, U: torch.Tensor, T: int, compat=None, kernel_params=None) -> torch.Tensor:
    """Q after T differentiable mean-field iterations of ``crf``.

    compat: optional list (one entry per pairwise term, None to keep) of
    tensors -- a 0-d Potts weight, an (M,) Diagonal or an (M, M) raw Matrix.
    kernel_params: optional list of DIAG (d,) / FULL (d, d) parameter tensors.
    """
    nt = crf.nTerms()
    compat = list(compat) if compat is not None else []
    kernel_params = list(kernel_params) if kernel_params is not None else []
    if len(compat) > nt or len(kernel_params) > nt:
        raise ValueError("more parameter tensors than pairwise terms")
    return _MeanField.apply(U, int(T), crf, len(compat), len(kernel_params), *compat, *kernel_params)


def bandwidth_grad(dp: torch.Tensor, s: float, dims) -> torch.Tensor:
    """dL/ds of a bandwidth s used by features f_j = x_j / s (j in dims), from
    the DIAG kernel-parameter gradient dp at p = 1: -(1/s) * sum_j dp[j]."""
    return -dp[list(dims)].sum() / s
