"""Unary and feature builders with the interface of ``pydensecrf.utils``.

Same functions, arguments and float32 results as pydensecrf/utils.py:6-193.
They prepare inputs for :class:`pydensecrf_gb300.densecrf.DenseCRF`; the
feature arrays are ``(d, N)`` float32, the unaries ``(M, N)`` float32.
"""
from __future__ import annotations

from logging import warning
from numbers import Number

import numpy as np

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


def create_pairwise_gaussian(sdims, shape):
    """Position features of an N-D grid, coordinate k divided by sdims[k]
    (utils.py:89-111).  Axis 0 of ``shape`` is feature 0 (for an image: rows)."""
    feats = _grid(shape)
    for k, s in enumerate(sdims):
        feats[k] /= s
    return feats.reshape([len(sdims), -1])


def create_pairwise_bilateral(sdims, schan, img, chdim=-1):
    """Position + channel features of an N-D image (utils.py:114-162).

    ``chdim`` is the channel axis of ``img`` (-1: single channel, no axis).
    ``schan`` is one scale per channel or a single number for all.
    """
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
