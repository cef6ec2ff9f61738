"""TEST INFRASTRUCTURE ONLY -- ctypes front-ends of the CPU checkers.

* ``Oracle*`` wrap ``oracle/liboracle.so``, the plain-C restatement of the
  reference's mean-field path (``oracle/dcrf_oracle.c``).
* ``Ref*`` wrap ``oracle/_ref/libdcrf_ref.so``, the reference's own C++
  sources compiled unmodified plus ``oracle/ref_shim.cpp``; it exists only on a
  machine where the reference sources were present at build time.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline arm import
this module.  The product package never does.

Array conventions: unaries / marginals are numpy ``(N, M)`` float32 arrays
(point-major, i.e. the memory of the reference's column-major ``M x N``
MatrixXf); features are ``(N, d)`` float32.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
VARIANT_SSE = 0
VARIANT_SCALAR = 1

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int)
_i16p = ctypes.POINTER(ctypes.c_short)
_u8p = ctypes.POINTER(ctypes.c_ubyte)
_vp = ctypes.c_void_p


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def build(quiet: bool = True, reference_root: str | None = None) -> None:
    """Compile liboracle.so, and _ref when the reference's sources are found:
    under `reference_root` (the root of a pydensecrf checkout), else under the
    DCRF_REFERENCE_ROOT environment variable; without either, _ref is skipped."""
    cmd = ["make", "-C", HERE, "all", "ref"]
    root = reference_root or os.environ.get("DCRF_REFERENCE_ROOT")
    if root:
        cmd.append("DCRF_REFERENCE_ROOT=" + os.path.abspath(root))
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_ORC = None
_REF = {}


def orc_lib():
    global _ORC
    if _ORC is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.orc_lattice_new.restype = _vp
        lib.orc_lattice_new.argtypes = [_f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.orc_lattice_vertices.argtypes = [_vp]
        lib.orc_lattice_phantoms.argtypes = [_vp]
        lib.orc_lattice_dump.argtypes = [_vp, _i32p, _i32p, _f32p, _i32p, _i16p]
        lib.orc_lattice_compute.argtypes = [_vp, _f32p, ctypes.c_int, ctypes.c_int, _f32p]
        lib.orc_lattice_free.argtypes = [_vp]
        lib.orc_crf_new.restype = _vp
        lib.orc_crf_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.orc_crf_free.argtypes = [_vp]
        lib.orc_crf_set_unary.argtypes = [_vp, _f32p]
        lib.orc_crf_add_pairwise.argtypes = [_vp, _f32p, ctypes.c_int, ctypes.c_int, _f32p, ctypes.c_int,
                                             ctypes.c_int]
        lib.orc_crf_inference.argtypes = [_vp, ctypes.c_int, _f32p]
        lib.orc_crf_inference_f64.argtypes = [_vp, ctypes.c_int, _f64p]
        lib.orc_crf_start.argtypes = [_vp, _f32p]
        lib.orc_crf_step.argtypes = [_vp, _f32p]
        lib.orc_crf_kl.restype = ctypes.c_double
        lib.orc_crf_kl.argtypes = [_vp, _f32p]
        lib.orc_crf_map.argtypes = [_vp, ctypes.c_int, _i16p]
        lib.orc_crf_term_vertices.argtypes = [_vp, ctypes.c_int]
        lib.orc_crf_term_norm.argtypes = [_vp, ctypes.c_int, _f32p]
        lib.orc_crf_term_lattice.restype = _vp
        lib.orc_crf_term_lattice.argtypes = [_vp, ctypes.c_int]
        _ORC = lib
    return _ORC


def _ref_path(variant: int) -> str:
    name = "libdcrf_ref.so" if variant == VARIANT_SSE else "libdcrf_ref_scalar.so"
    return os.path.join(HERE, "_ref", name)


def ref_available(variant: int = VARIANT_SSE) -> bool:
    """True when the reference compiled from its sources (that variant) exists."""
    return os.path.exists(_ref_path(variant))


def ref_lib(variant: int = VARIANT_SSE):
    if variant not in _REF:
        path = _ref_path(variant)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        lib.ref_lattice_new.restype = _vp
        lib.ref_lattice_new.argtypes = [_f32p, ctypes.c_int, ctypes.c_int]
        lib.ref_lattice_vertices.argtypes = [_vp]
        lib.ref_lattice_dump.argtypes = [_vp, ctypes.c_int, _i32p, _i32p, _f32p, _i32p]
        lib.ref_lattice_compute.argtypes = [_vp, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f32p]
        lib.ref_lattice_gradient.argtypes = [_vp, _f32p, _f32p, ctypes.c_int, ctypes.c_int, _f32p]
        lib.ref_lattice_free.argtypes = [_vp]
        lib.ref_crf_new.restype = _vp
        lib.ref_crf_new.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.ref_crf2d_new.restype = _vp
        lib.ref_crf2d_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.ref_crf_free.argtypes = [_vp]
        lib.ref_crf_set_unary.argtypes = [_vp, _f32p, ctypes.c_int, ctypes.c_int]
        lib.ref_crf_set_unary_logistic.argtypes = [_vp, _f32p, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.ref_crf_add_pairwise.argtypes = [_vp, _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _f32p,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.ref_crf2d_add_gaussian.argtypes = [_vp, ctypes.c_float, ctypes.c_float, ctypes.c_int, _f32p,
                                               ctypes.c_int, ctypes.c_int, ctypes.c_int]
        lib.ref_crf2d_add_bilateral.argtypes = [_vp] + [ctypes.c_float] * 5 + [_u8p, ctypes.c_int, _f32p,
                                                                                ctypes.c_int, ctypes.c_int,
                                                                                ctypes.c_int]
        lib.ref_crf_inference.argtypes = [_vp, ctypes.c_int, _f32p]
        lib.ref_crf_start.argtypes = [_vp, _f32p]
        lib.ref_crf_step.argtypes = [_vp, _f32p, ctypes.c_int, ctypes.c_int]
        lib.ref_crf_kl.restype = ctypes.c_double
        lib.ref_crf_kl.argtypes = [_vp, _f32p, ctypes.c_int, ctypes.c_int]
        lib.ref_crf_map.argtypes = [_vp, ctypes.c_int, _i16p]
        lib.ref_crf_unary_energy.argtypes = [_vp, _i16p, ctypes.c_int, _f32p]
        lib.ref_crf_pairwise_energy.argtypes = [_vp, _i16p, ctypes.c_int, ctypes.c_int, _f32p]
        lib.ref_crf_compat_param_count.argtypes = [_vp]
        lib.ref_crf_kernel_param_count.argtypes = [_vp]
        lib.ref_crf_unary_param_count.argtypes = [_vp]
        lib.ref_crf_set_kernel_params.argtypes = [_vp, _f32p, ctypes.c_int]
        lib.ref_crf_set_compat_params.argtypes = [_vp, _f32p, ctypes.c_int]
        lib.ref_crf_gradient.restype = ctypes.c_double
        lib.ref_crf_gradient.argtypes = [_vp, ctypes.c_int, _i16p, ctypes.c_int, _f32p, _f32p, _f32p]
        _REF[variant] = lib
    return _REF[variant]


def _compat_args(compat, M):
    """(kind, float32 buffer) for a Potts scalar / Diagonal vector / Matrix."""
    if np.isscalar(compat):
        return 0, np.array([compat], dtype=np.float32)
    c = np.ascontiguousarray(compat, dtype=np.float32)
    if c.ndim == 1:
        return 1, c
    return 2, c


class Lattice:
    """Lattice tables from the oracle (`impl="oracle"`) or the reference."""

    def __init__(self, feat: np.ndarray, impl: str = "oracle", variant: int = VARIANT_SSE):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        self.N, self.d = feat.shape
        self.impl = impl
        d1 = self.d + 1
        if impl == "oracle":
            lib = orc_lib()
            h = lib.orc_lattice_new(_p(feat, _f32p), self.d, self.N, variant)
            self.L = lib.orc_lattice_vertices(h)
            self.n_phantom = lib.orc_lattice_phantoms(h)
            self.offset = np.empty((self.N, d1), np.int32)
            self.rank = np.empty((self.N, d1), np.int32)
            self.bary = np.empty((self.N, d1), np.float32)
            self.neighbors = np.empty((d1, self.L, 2), np.int32)
            self.keys = np.empty((self.L, self.d), np.int16)
            lib.orc_lattice_dump(h, _p(self.offset, _i32p), _p(self.rank, _i32p), _p(self.bary, _f32p),
                                 _p(self.neighbors, _i32p), _p(self.keys, _i16p))
            self._h, self._free, self._lib = h, lib.orc_lattice_free, lib
        else:
            lib = ref_lib(variant)
            h = lib.ref_lattice_new(_p(feat, _f32p), self.d, self.N)
            self.L = lib.ref_lattice_vertices(h)
            self.offset = np.empty((self.N, d1), np.int32)
            self.rank = np.empty((self.N, d1), np.int32)
            self.bary = np.empty((self.N, d1), np.float32)
            self.neighbors = np.empty((d1, self.L, 2), np.int32)
            self.keys = None
            lib.ref_lattice_dump(h, self.N, _p(self.offset, _i32p), _p(self.rank, _i32p), _p(self.bary, _f32p),
                                 _p(self.neighbors, _i32p))
            self._h, self._free, self._lib = h, lib.ref_lattice_free, lib

    def compute(self, values: np.ndarray, reverse: bool = False) -> np.ndarray:
        v = np.ascontiguousarray(values, dtype=np.float32)
        vs = v.shape[1]
        out = np.empty_like(v)
        if self.impl == "oracle":
            self._lib.orc_lattice_compute(self._h, _p(v, _f32p), vs, int(reverse), _p(out, _f32p))
        else:
            self._lib.ref_lattice_compute(self._h, _p(v, _f32p), vs, self.N, int(reverse), _p(out, _f32p))
        return out

    def __del__(self):
        try:
            self._free(self._h)
        except Exception:
            pass


class OracleCRF:
    """The C restatement of DenseCRF (float, reference arithmetic) plus its FP64 twin."""

    def __init__(self, N: int, M: int, variant: int = VARIANT_SSE):
        self.N, self.M = N, M
        self._lib = orc_lib()
        self._h = self._lib.orc_crf_new(N, M, variant)

    def set_unary(self, U: np.ndarray) -> None:
        U = np.ascontiguousarray(U, dtype=np.float32).reshape(self.N, self.M)
        self._lib.orc_crf_set_unary(self._h, _p(U, _f32p))

    def add_pairwise(self, feat, compat, ktype=1, ntype=3) -> int:
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        kind, c = _compat_args(compat, self.M)
        return self._lib.orc_crf_add_pairwise(self._h, _p(feat, _f32p), feat.shape[1], kind, _p(c, _f32p),
                                              ktype, ntype)

    def inference(self, T: int) -> np.ndarray:
        Q = np.empty((self.N, self.M), np.float32)
        self._lib.orc_crf_inference(self._h, T, _p(Q, _f32p))
        return Q

    def inference_f64(self, T: int) -> np.ndarray:
        Q = np.empty((self.N, self.M), np.float64)
        self._lib.orc_crf_inference_f64(self._h, T, _p(Q, _f64p))
        return Q

    def start(self) -> np.ndarray:
        Q = np.empty((self.N, self.M), np.float32)
        self._lib.orc_crf_start(self._h, _p(Q, _f32p))
        return Q

    def step(self, Q: np.ndarray) -> None:
        assert Q.dtype == np.float32 and Q.flags.c_contiguous
        self._lib.orc_crf_step(self._h, _p(Q, _f32p))

    def kl(self, Q: np.ndarray) -> float:
        Q = np.ascontiguousarray(Q, dtype=np.float32)
        return self._lib.orc_crf_kl(self._h, _p(Q, _f32p))

    def map(self, T: int) -> np.ndarray:
        """map (densecrf.cpp:132-137,202-211): labels of the first maximum after T iterations."""
        out = np.empty(self.N, np.int16)
        self._lib.orc_crf_map(self._h, T, _p(out, _i16p))
        return out

    def term_norm(self, k: int) -> np.ndarray:
        out = np.empty(self.N, np.float32)
        self._lib.orc_crf_term_norm(self._h, k, _p(out, _f32p))
        return out

    def __del__(self):
        try:
            self._lib.orc_crf_free(self._h)
        except Exception:
            pass


class RefCRF:
    """The reference's DenseCRF / DenseCRF2D (compiled from its sources)."""

    def __init__(self, N: int, M: int, W: int = 0, H: int = 0, variant: int = VARIANT_SSE):
        self.N, self.M = N, M
        self._lib = ref_lib(variant)
        self._h = self._lib.ref_crf2d_new(W, H, M) if W else self._lib.ref_crf_new(N, M)
        self.is2d = bool(W)

    def set_unary(self, U: np.ndarray) -> None:
        U = np.ascontiguousarray(U, dtype=np.float32).reshape(self.N, self.M)
        self._lib.ref_crf_set_unary(self._h, _p(U, _f32p), self.M, self.N)

    def add_pairwise(self, feat, compat, ktype=1, ntype=3) -> None:
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        kind, c = _compat_args(compat, self.M)
        self._lib.ref_crf_add_pairwise(self._h, _p(feat, _f32p), feat.shape[1], self.N, kind, _p(c, _f32p),
                                       self.M, ktype, ntype)

    def add_gaussian(self, sx, sy, compat, ktype=1, ntype=3) -> None:
        kind, c = _compat_args(compat, self.M)
        self._lib.ref_crf2d_add_gaussian(self._h, sx, sy, kind, _p(c, _f32p), self.M, ktype, ntype)

    def add_bilateral(self, sx, sy, sr, sg, sb, img, compat, ktype=1, ntype=3) -> None:
        img = np.ascontiguousarray(img, dtype=np.uint8)
        kind, c = _compat_args(compat, self.M)
        self._lib.ref_crf2d_add_bilateral(self._h, sx, sy, sr, sg, sb, _p(img, _u8p), kind, _p(c, _f32p),
                                          self.M, ktype, ntype)

    def inference(self, T: int) -> np.ndarray:
        Q = np.empty((self.N, self.M), np.float32)
        self._lib.ref_crf_inference(self._h, T, _p(Q, _f32p))
        return Q

    def start(self) -> np.ndarray:
        Q = np.empty((self.N, self.M), np.float32)
        self._lib.ref_crf_start(self._h, _p(Q, _f32p))
        return Q

    def step(self, Q: np.ndarray) -> None:
        self._lib.ref_crf_step(self._h, _p(Q, _f32p), self.M, self.N)

    def kl(self, Q: np.ndarray) -> float:
        Q = np.ascontiguousarray(Q, dtype=np.float32)
        return self._lib.ref_crf_kl(self._h, _p(Q, _f32p), self.M, self.N)

    def map(self, T: int) -> np.ndarray:
        out = np.empty(self.N, np.int16)
        self._lib.ref_crf_map(self._h, T, _p(out, _i16p))
        return out

    def unary_energy(self, labels: np.ndarray) -> np.ndarray:
        """DenseCRF::unaryEnergy (densecrf.cpp:141-153)."""
        lab = np.ascontiguousarray(labels, dtype=np.int16)
        out = np.empty(self.N, np.float32)
        self._lib.ref_crf_unary_energy(self._h, _p(lab, _i16p), self.N, _p(out, _f32p))
        return out

    def pairwise_energy(self, labels: np.ndarray, term: int = -1) -> np.ndarray:
        """DenseCRF::pairwiseEnergy (densecrf.cpp:154-177); term -1 sums all terms."""
        lab = np.ascontiguousarray(labels, dtype=np.int16)
        out = np.empty(self.N, np.float32)
        self._lib.ref_crf_pairwise_energy(self._h, _p(lab, _i16p), self.N, term, _p(out, _f32p))
        return out

    def gradient(self, T: int, gt: np.ndarray, want_unary=False, want_compat=True, want_kernel=True):
        lib = self._lib
        gt = np.ascontiguousarray(gt, dtype=np.int16)
        nu = lib.ref_crf_unary_param_count(self._h)
        nc = lib.ref_crf_compat_param_count(self._h)
        nk = lib.ref_crf_kernel_param_count(self._h)
        ug = np.zeros(max(nu, 1), np.float32) if want_unary else None
        cg = np.zeros(max(nc, 1), np.float32) if want_compat else None
        kg = np.zeros(max(nk, 1), np.float32) if want_kernel else None
        r = lib.ref_crf_gradient(self._h, T, _p(gt, _i16p), self.N, _p(ug, _f32p), _p(cg, _f32p), _p(kg, _f32p))
        return r, (ug[:nu] if ug is not None else None), (cg[:nc] if cg is not None else None), \
            (kg[:nk] if kg is not None else None)

    def __del__(self):
        try:
            self._lib.ref_crf_free(self._h)
        except Exception:
            pass


def features_gaussian_2d(W: int, H: int, sx: float, sy: float) -> np.ndarray:
    """Features of DenseCRF2D::addPairwiseGaussian (D:61-69): (i/sx, j/sy), point j*W+i."""
    j, i = np.meshgrid(np.arange(H, dtype=np.float32), np.arange(W, dtype=np.float32), indexing="ij")
    f = np.stack([i / np.float32(sx), j / np.float32(sy)], axis=-1)
    return np.ascontiguousarray(f.reshape(W * H, 2), dtype=np.float32)


def features_bilateral_2d(img: np.ndarray, sx, sy, sr, sg, sb) -> np.ndarray:
    """Features of DenseCRF2D::addPairwiseBilateral (D:70-81)."""
    H, W, _ = img.shape
    j, i = np.meshgrid(np.arange(H, dtype=np.float32), np.arange(W, dtype=np.float32), indexing="ij")
    im = img.astype(np.float32)
    f = np.stack([i / np.float32(sx), j / np.float32(sy), im[..., 0] / np.float32(sr), im[..., 1] / np.float32(sg),
                  im[..., 2] / np.float32(sb)], axis=-1)
    return np.ascontiguousarray(f.reshape(W * H, 5), dtype=np.float32)
