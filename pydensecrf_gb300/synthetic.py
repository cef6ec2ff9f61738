"""Seeded synthetic inputs for the dense-CRF workloads this package is measured on.

No public dataset is involved: every workload is a seeded numpy generator.
Arrays follow the pydensecrf conventions: unaries ``(M, N)`` float32 (labels
major, as ``DenseCRF.setUnaryEnergy`` takes them), images ``(H, W, 3)`` uint8,
volumes ``(D, H, W)`` float32.

Workloads (sizes as named):

* ``plain_small``  -- 320x240, 5 labels, logits ~ N(0, 2), image of 12 random
  rectangles of uniform colour + N(0, 8) noise; Gaussian(sxy=3, compat=3) +
  bilateral(sxy=80, srgb=13, compat=10), 5 iterations.
* ``plain_vga``    -- 640x480, 21 labels, logits = 4 x (N(0,1) blurred with a
  sigma = 8 px Gaussian, rescaled to unit standard deviation) per label,
  unary = -log(clip(softmax, 1e-5)), image of 40
  Voronoi cells of uniform colour + N(0, 6) noise; same two Potts terms, 10
  iterations.
* ``batch_uneven`` -- 64 images with W, H ~ U[256, 1024], 21 labels, inputs as
  ``plain_small`` per image, one symmetric 21x21 matrix compatibility with
  entries U(0, 2) and zero diagonal, 10 iterations.
* ``train_512``    -- 8 images of 512x512, 21 labels, 5 iterations, a
  30-region Voronoi label map as the cross-entropy target.
* ``volume_96``    -- 8 volumes of 96^3, 4 labels, intensity = 6 Gaussian
  blobs + N(0, 0.05), features (x/5, y/5, z/5, I/0.1), logits ~ N(0, 1.5),
  matrix compatibility U(0, 1) symmetric, 8 iterations.
"""
from __future__ import annotations

import numpy as np


def softmax(logits: np.ndarray, axis: int = 0) -> np.ndarray:
    z = logits - logits.max(axis=axis, keepdims=True)
    e = np.exp(z)
    return e / e.sum(axis=axis, keepdims=True)


def neg_log_softmax(logits: np.ndarray, axis: int = 0) -> np.ndarray:
    z = logits - logits.max(axis=axis, keepdims=True)
    return (np.log(np.exp(z).sum(axis=axis, keepdims=True)) - z).astype(np.float32)


def _gauss_kernel(sigma: float) -> np.ndarray:
    r = int(np.ceil(4 * sigma))
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    return k / k.sum()


def gaussian_blur_2d(a: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian blur of the last two axes (reflect padding)."""
    k = _gauss_kernel(sigma)
    r = len(k) // 2
    out = a.astype(np.float64)
    for axis in (-2, -1):
        pad = [(0, 0)] * out.ndim
        pad[axis] = (r, r)
        p = np.pad(out, pad, mode="reflect")
        acc = np.zeros_like(out)
        n = out.shape[axis]
        for i, w in enumerate(k):
            sl = [slice(None)] * out.ndim
            sl[axis] = slice(i, i + n)
            acc += w * p[tuple(sl)]
        out = acc
    return out


def rect_image(rng: np.random.Generator, W: int, H: int, n_rect: int = 12, noise: float = 8.0) -> np.ndarray:
    img = np.zeros((H, W, 3), np.float32)
    img[:] = rng.uniform(0, 255, size=3)
    for _ in range(n_rect):
        x0, x1 = np.sort(rng.integers(0, W, size=2))
        y0, y1 = np.sort(rng.integers(0, H, size=2))
        img[y0:y1 + 1, x0:x1 + 1] = rng.uniform(0, 255, size=3)
    img += rng.normal(0, noise, size=img.shape)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def voronoi_labels(rng: np.random.Generator, W: int, H: int, n_cells: int) -> np.ndarray:
    sx = rng.uniform(0, W, size=n_cells)
    sy = rng.uniform(0, H, size=n_cells)
    yy, xx = np.mgrid[0:H, 0:W]
    best = np.zeros((H, W), np.int32)
    bd = np.full((H, W), np.inf)
    for c in range(n_cells):
        dd = (xx - sx[c]) ** 2 + (yy - sy[c]) ** 2
        m = dd < bd
        best[m] = c
        bd[m] = dd[m]
    return best


def voronoi_image(rng: np.random.Generator, W: int, H: int, n_cells: int = 40, noise: float = 6.0) -> np.ndarray:
    cell = voronoi_labels(rng, W, H, n_cells)
    colours = rng.uniform(0, 255, size=(n_cells, 3))
    img = colours[cell] + rng.normal(0, noise, size=(H, W, 3))
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def plain_small(seed: int = 0, W: int = 320, H: int = 240, M: int = 5):
    """320x240 x 5 labels: returns dict(U (M,N), img (H,W,3), params)."""
    rng = np.random.default_rng(seed)
    logits = rng.normal(0, 2, size=(M, H * W)).astype(np.float32)
    U = neg_log_softmax(logits, axis=0)
    img = rect_image(rng, W, H)
    return dict(W=W, H=H, M=M, U=np.ascontiguousarray(U, np.float32), img=img, T=5,
                gauss=dict(sxy=3.0, compat=3.0), bilat=dict(sxy=80.0, srgb=13.0, compat=10.0))


def plain_vga(seed: int = 0, W: int = 640, H: int = 480, M: int = 21):
    """640x480 x 21 labels (smooth logits, Voronoi image): dict(U, img, params)."""
    rng = np.random.default_rng(seed)
    noise = rng.normal(0, 1, size=(M, H, W))
    field = gaussian_blur_2d(noise, 8.0)
    # the blurred field is rescaled to unit standard deviation, then x4
    logits = 4.0 * field / max(float(field.std()), 1e-12)
    sm = softmax(logits.reshape(M, -1), axis=0)
    U = -np.log(np.clip(sm, 1e-5, 1.0)).astype(np.float32)
    img = voronoi_image(rng, W, H, 40, 6.0)
    return dict(W=W, H=H, M=M, U=np.ascontiguousarray(U, np.float32), img=img, T=10,
                gauss=dict(sxy=3.0, compat=3.0), bilat=dict(sxy=80.0, srgb=13.0, compat=10.0))


def random_sym_matrix(rng: np.random.Generator, M: int, hi: float, zero_diag: bool) -> np.ndarray:
    a = rng.uniform(0, hi, size=(M, M))
    a = 0.5 * (a + a.T)
    if zero_diag:
        np.fill_diagonal(a, 0.0)
    return a.astype(np.float32)


def batch_uneven(seed: int = 0, B: int = 64, M: int = 21, lo: int = 256, hi: int = 1024):
    """B images of uneven size, per-image inputs as plain_small, shared matrix compat."""
    rng = np.random.default_rng(seed)
    imgs, Us, sizes = [], [], []
    for _ in range(B):
        W = int(rng.integers(lo, hi + 1))
        H = int(rng.integers(lo, hi + 1))
        logits = rng.normal(0, 2, size=(M, H * W)).astype(np.float32)
        Us.append(np.ascontiguousarray(neg_log_softmax(logits, axis=0), np.float32))
        imgs.append(rect_image(rng, W, H))
        sizes.append((W, H))
    compat = random_sym_matrix(rng, M, 2.0, True)
    return dict(M=M, sizes=sizes, U=Us, img=imgs, compat=compat, T=10,
                gauss=dict(sxy=3.0), bilat=dict(sxy=80.0, srgb=13.0))


def train_512(seed: int = 0, B: int = 8, W: int = 512, H: int = 512, M: int = 21):
    rng = np.random.default_rng(seed)
    imgs, Us, gts = [], [], []
    for _ in range(B):
        logits = rng.normal(0, 2, size=(M, H * W)).astype(np.float32)
        Us.append(np.ascontiguousarray(neg_log_softmax(logits, axis=0), np.float32))
        imgs.append(rect_image(rng, W, H))
        cells = voronoi_labels(rng, W, H, 30)
        lab = rng.integers(0, M, size=30)
        gts.append(lab[cells].reshape(-1).astype(np.int64))
    compat = random_sym_matrix(rng, M, 2.0, True)
    return dict(W=W, H=H, M=M, U=Us, img=imgs, gt=gts, compat=compat, T=5,
                gauss=dict(sxy=3.0, compat=3.0), bilat=dict(sxy=80.0, srgb=13.0))


def volume_96(seed: int = 0, B: int = 8, S: int = 96, M: int = 4):
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.mgrid[0:S, 0:S, 0:S].astype(np.float32)
    vols, Us, feats = [], [], []
    for _ in range(B):
        I = np.zeros((S, S, S), np.float32)
        for _ in range(6):
            c = rng.uniform(0, S, size=3)
            s = rng.uniform(4, 16)
            a = rng.uniform(0.3, 1.0)
            I += a * np.exp(-((zz - c[0]) ** 2 + (yy - c[1]) ** 2 + (xx - c[2]) ** 2) / (2 * s * s))
        I += rng.normal(0, 0.05, size=I.shape).astype(np.float32)
        I = I.astype(np.float32)
        f = np.stack([xx / np.float32(5), yy / np.float32(5), zz / np.float32(5), I / np.float32(0.1)], axis=0)
        feats.append(np.ascontiguousarray(f.reshape(4, -1), np.float32))
        logits = rng.normal(0, 1.5, size=(M, S ** 3)).astype(np.float32)
        Us.append(np.ascontiguousarray(neg_log_softmax(logits, axis=0), np.float32))
        vols.append(I)
    compat = random_sym_matrix(rng, M, 1.0, False)
    return dict(S=S, M=M, U=Us, vol=vols, feat=feats, compat=compat, T=8, gauss_sxyz=3.0)
