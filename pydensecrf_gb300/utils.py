"""Unary and feature builders with the interface of ``pydensecrf.utils``.

Same functions, arguments and float32 results as pydensecrf/utils.py:6-193.
They prepare inputs for :class:`pydensecrf_gb300.densecrf.DenseCRF`; the
feature arrays are ``(d, N)`` float32, the unaries ``(M, N)`` float32.

Given torch tensors (e.g. CUDA tensors) the builders compute on the tensors'
device with the same arithmetic and return tensors, so that a label map or a
softmax that already lives on the GPU is turned into engine inputs without a
host round trip (``DenseCRF`` accepts CUDA tensors directly).
"""
from __future__ import annotations

from logging import warning
from numbers import Number

import numpy as np


def _is_tensor(x) -> bool:
    try:
        import torch
    except ImportError:  # the numpy forms need no torch
        return False
    return isinstance(x, torch.Tensor)

__all__ = ["unary_from_labels", "compute_unary", "unary_from_softmax", "softmax_to_unary",
           "create_pairwise_gaussian", "create_pairwise_bilateral"]


def unary_from_labels(labels, n_labels, gt_prob, zero_unsure=True):
    """Unary from a label map that is right with probability ``gt_prob``
    (utils.py:6-46).

    Every variable gets -log((1-gt_prob)/(n_labels-1)) for the other labels and
    -log(gt_prob) for its own.  With ``zero_unsure`` the value 0 means "unknown":
    labels are 1-based and 0-labelled variables get the uniform -log(1/n_labels).
    """
    assert 0 < gt_prob < 1, "`gt_prob must be in (0,1)."
    if _is_tensor(labels):
        import torch
        flat = labels.reshape(-1).long()
        n = flat.shape[0]
        other = float(np.float32(-np.log((1.0 - gt_prob) / (n_labels - 1))))
        U = torch.full((n_labels, n), other, dtype=torch.float32, device=labels.device)
        rows = flat - 1 if zero_unsure else flat
        keep = rows >= 0
        idx = torch.arange(n, device=labels.device)
        U[rows[keep], idx[keep]] = float(np.float32(-np.log(gt_prob)))
        if zero_unsure:
            U[:, flat == 0] = float(np.float32(-np.log(1.0 / n_labels)))
        return U
    flat = np.asarray(labels).reshape(-1)
    n = flat.shape[0]
    other = -np.log((1.0 - gt_prob) / (n_labels - 1))
    own = -np.log(gt_prob)
    U = np.full((n_labels, n), other, dtype=np.float32)
    rows = flat - 1 if zero_unsure else flat
    U[rows, np.arange(n)] = own
    if zero_unsure:
        U[:, flat == 0] = -np.log(1.0 / n_labels)
    return U


def compute_unary(labels, M, GT_PROB=0.5):
    """Deprecated alias of :func:`unary_from_labels` (utils.py:49-52)."""
    warning("pydensecrf.compute_unary is deprecated, use unary_from_labels instead.")
    return unary_from_labels(labels, M, GT_PROB)


def unary_from_softmax(sm, scale=None, clip=1e-5):
    """Negative log of class probabilities, classes on axis 0 (utils.py:55-79).

    ``scale`` in (0, 1] mixes the probabilities with the uniform distribution
    (0 -> uniform, 1 -> unchanged); ``clip`` bounds them away from 0.
    """
    n_cls = sm.shape[0]
    if _is_tensor(sm):
        # the numpy form's type promotion: a float32 softmax stays float32
        # unless ``scale`` mixes in the (float64) uniform term
        import torch
        x = sm if sm.is_floating_point() else sm.to(torch.float64)
        if scale is not None:
            assert 0 < scale <= 1, "`scale` needs to be in (0,1]"
            x = (scale * x).to(torch.float64) + (1 - scale) * (1.0 / n_cls)
        if clip is not None:
            x = x.clamp(clip, 1.0)
        return (-torch.log(x)).reshape(n_cls, -1).to(torch.float32)
    if scale is not None:
        assert 0 < scale <= 1, "`scale` needs to be in (0,1]"
        sm = scale * sm + (1 - scale) * (np.ones(sm.shape) / n_cls)
    if clip is not None:
        sm = np.clip(sm, clip, 1.0)
    return -np.log(sm).reshape([n_cls, -1]).astype(np.float32)


def softmax_to_unary(sm, GT_PROB=1):
    """Deprecated alias of :func:`unary_from_softmax` (utils.py:82-86)."""
    warning("pydensecrf.softmax_to_unary is deprecated, use unary_from_softmax instead.")
    return unary_from_softmax(sm, None if GT_PROB == 1 else GT_PROB, clip=None)


def _grid(shape):
    return np.array(np.meshgrid(*[np.arange(s) for s in shape], indexing="ij"), dtype=np.float32)


def _grid_t(shape, device):
    import torch
    axes = [torch.arange(n, dtype=torch.float32, device=device) for n in shape]
    return torch.stack(torch.meshgrid(*axes, indexing="ij"))


def _div_t(x, s):
    """x / s rounded like numpy's float32 division (an elementwise tensor divisor:
    a scalar divisor may be applied as a reciprocal multiply)."""
    import torch
    return torch.div(x, torch.full_like(x, float(np.float32(s))))


def create_pairwise_gaussian(sdims, shape, device=None):
    """Position features of an N-D grid, coordinate k divided by sdims[k]
    (utils.py:89-111).  Axis 0 of ``shape`` is feature 0 (for an image: rows).
    With ``device`` (a torch device) the features are a tensor built there."""
    if device is not None:
        feats = _grid_t(shape, device)
        for k, s in enumerate(sdims):
            feats[k] = _div_t(feats[k], s)
        return feats.reshape(len(sdims), -1)
    feats = _grid(shape)
    for k, s in enumerate(sdims):
        feats[k] /= s
    return feats.reshape([len(sdims), -1])


def create_pairwise_bilateral(sdims, schan, img, chdim=-1):
    """Position + channel features of an N-D image (utils.py:114-162).

    ``chdim`` is the channel axis of ``img`` (-1: single channel, no axis).
    ``schan`` is one scale per channel or a single number for all.
    """
    if _is_tensor(img):
        import torch
        chans = (img.unsqueeze(0) if chdim == -1 else torch.movedim(img, chdim, 0)).to(torch.float32)
        if isinstance(schan, Number):
            chans = _div_t(chans, schan)
        else:
            chans = chans.clone()
            for k, s in enumerate(schan):
                chans[k] = _div_t(chans[k], s)
        pos = _grid_t(chans.shape[1:], img.device)
        for k, s in enumerate(sdims):
            pos[k] = _div_t(pos[k], s)
        feats = torch.cat([pos, chans])
        return feats.reshape(feats.shape[0], -1)
    if chdim == -1:
        chans = img[np.newaxis].astype(np.float32)
    else:
        chans = np.rollaxis(img, chdim).astype(np.float32)
    if isinstance(schan, Number):
        chans /= schan
    else:
        for k, s in enumerate(schan):
            chans[k] /= s
    pos = _grid(chans.shape[1:])
    for k, s in enumerate(sdims):
        pos[k] /= s
    feats = np.concatenate([pos, chans])
    return feats.reshape([feats.shape[0], -1])


def _create_pairwise_gaussian_2d(sx, sy, shape):
    """Loop form of the 2-D Gaussian features (utils.py:165-176)."""
    f = np.zeros((2, shape[0], shape[1]), dtype=np.float32)
    for r in range(shape[0]):
        for c in range(shape[1]):
            f[0, r, c] = r / sx
            f[1, r, c] = c / sy
    return f.reshape([2, -1])


def _create_pairwise_bilateral_2d(sx, sy, sr, sg, sb, img):
    """Loop form of the 2-D bilateral features (utils.py:179-193)."""
    f = np.zeros((5, img.shape[0], img.shape[1]), dtype=np.float32)
    for r in range(img.shape[0]):
        for c in range(img.shape[1]):
            f[0, r, c] = r / sx
            f[1, r, c] = c / sy
            f[2, r, c] = img[r, c, 0] / sr
            f[3, r, c] = img[r, c, 1] / sg
            f[4, r, c] = img[r, c, 2] / sb
    return f.reshape([5, -1])
