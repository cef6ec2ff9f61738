"""FP64 lattice filter for the filter parity tests (test infrastructure)."""
import numpy as np


def filter_f64(lat, x):
    """Permutohedral::compute (permutohedral.cpp:476-610) in float64 on the
    oracle's lattice tables (`oracle.Lattice`): x (N, vs) -> (N, vs), forward
    blur order."""
    N, d1 = lat.offset.shape
    d, L = d1 - 1, lat.L
    off = lat.offset + 1  # row 0 is the zero sentinel
    bary = lat.bary.astype(np.float64)
    xd = x.astype(np.float64)
    vals = np.zeros((L + 2, x.shape[1]))
    for k in range(x.shape[1]):
        for r in range(d1):
            vals[:, k] += np.bincount(off[:, r], weights=bary[:, r] * xd[:, k], minlength=L + 2)
    for j in range(d1):
        n1, n2 = lat.neighbors[j, :, 0] + 1, lat.neighbors[j, :, 1] + 1
        nv = vals.copy()
        nv[1:L + 1] = vals[1:L + 1] + 0.5 * (vals[n1] + vals[n2])
        vals = nv
    alpha = 1.0 / (1.0 + 2.0 ** -d)
    out = np.zeros_like(xd)
    for r in range(d1):
        out += (bary[:, r, None] * alpha) * vals[off[:, r]]
    return out
