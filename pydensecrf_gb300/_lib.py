"""ctypes binding of ``libdcrf_gb300.so`` (the C ABI declared in include/dcrf.h).

The library is built in-tree by :mod:`pydensecrf_gb300.build`.  There is no
CPU fallback: if the library is missing or no GPU is present, the calls fail
with an explicit error.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdcrf_gb300.so")

DCRF_OK = 0
DCRF_ERR_INVALID_ARG = -1
DCRF_ERR_CUDA = -2
DCRF_ERR_OOM = -3
DCRF_ERR_HASH_FULL = -4
DCRF_ERR_KEY_OVERFLOW = -5
DCRF_ERR_NO_DEVICE = -6
DCRF_ERR_STATE = -7
DCRF_ERR_TIMEOUT = -8

HOST, DEVICE = 0, 1
LAYOUT_LM, LAYOUT_PM = 0, 1
VARIANT_SSE, VARIANT_SCALAR = 0, 1
COMPAT_POTTS, COMPAT_DIAGONAL, COMPAT_MATRIX = 0, 1, 2

_vp = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_pf = ctypes.POINTER(ctypes.c_float)
_pi = ctypes.POINTER(ctypes.c_int)

_SIGS = {
    "dcrf_abi_version": ([], _i),
    "dcrf_last_error": ([ctypes.c_char_p, ctypes.c_size_t], _i),
    "dcrf_create": ([_i, _i, ctypes.POINTER(_vp)], _i),
    "dcrf_create_2d": ([_i, _i, _i, ctypes.POINTER(_vp)], _i),
    "dcrf_create_batch": ([_i, _vp, _i, ctypes.POINTER(_vp)], _i),
    "dcrf_create_batch_2d": ([_i, _vp, _vp, _i, ctypes.POINTER(_vp)], _i),
    "dcrf_batch_info": ([_vp, _vp, _vp], _i),
    "dcrf_unary_energy": ([_vp, _vp, _i, _vp, _i], _i),
    "dcrf_pairwise_energy": ([_vp, _vp, _i, _i, _vp, _i], _i),
    "dcrf_set_autotune": ([_vp, _i], _i),
    "dcrf_autotune": ([_vp], _i),
    "dcrf_get_tuning": ([_vp, _vp, _vp, _vp, _vp, _vp], _i),
    "dcrf_set_tuning": ([_vp, _i, _i, _i, ctypes.c_float, _i], _i),
    "dcrf_check_bounded_wait": ([_vp, _i], _i),
    "dcrf_destroy": ([_vp], _i),
    "dcrf_set_stream": ([_vp, _vp], _i),
    "dcrf_set_variant": ([_vp, _i], _i),
    "dcrf_set_unary": ([_vp, _vp, _i, _i], _i),
    "dcrf_add_pairwise": ([_vp, _vp, _i, _i, _i, _vp, _i, _i, _pi], _i),
    "dcrf_add_pairwise_gaussian": ([_vp, _f, _f, _i, _vp, _i, _i, _pi], _i),
    "dcrf_add_pairwise_bilateral": ([_vp, _f, _f, _f, _f, _f, _vp, _i, _i, _vp, _i, _i, _pi], _i),
    "dcrf_inference": ([_vp, _i, _vp, _i, _i], _i),
    "dcrf_start_inference": ([_vp, _vp, _i, _i], _i),
    "dcrf_step_inference": ([_vp, _vp, _i, _i], _i),
    "dcrf_kl_divergence": ([_vp, _vp, _i, _i, ctypes.POINTER(ctypes.c_double)], _i),
    "dcrf_map": ([_vp, _i, _vp, _i], _i),
    "dcrf_synchronize": ([_vp], _i),
    "dcrf_info": ([_vp, _pi, _pi, _pi], _i),
    "dcrf_lattice_info": ([_vp, _i, _pi, _pi], _i),
    "dcrf_lattice_dump": ([_vp, _i, _vp, _vp, _vp, _vp, _vp], _i),
    "dcrf_term_norm": ([_vp, _i, _vp], _i),
    "dcrf_lattice_filter": ([_vp, _i, _vp, _i, _i, _vp], _i),
    "dcrf_clear_pairwise": ([_vp], _i),
    "dcrf_launch_count": ([ctypes.POINTER(ctypes.c_ulonglong)], _i),
    "dcrf_set_profiling": ([_vp, _i], _i),
    "dcrf_profile": ([_vp, _i, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)], _i),
    "dcrf_term_stats": ([_vp, _i, _pi, _pi, _pi], _i),
    "dcrf_term_buffer": ([_vp, _i, _i, _vp, ctypes.c_size_t], _i),
    "dcrf_lattice_filter_noalloc": ([_vp, _i, _vp, _i, _i, _vp, _vp], _i),
    "dcrf_set_compat": ([_vp, _i, _i, _vp], _i),
    "dcrf_set_kernel_params": ([_vp, _i, _vp], _i),
    "dcrf_param_counts": ([_vp, _i, _pi, _pi], _i),
    "dcrf_inference_checkpointed": ([_vp, _i, _vp, _i, _i], _i),
    "dcrf_backward": ([_vp, _vp, _i, _i, _vp, _vp, _vp], _i),
    "dcrf_set_unary_logistic": ([_vp, _vp, _i, _vp, _i], _i),
    "dcrf_unary_parameters": ([_vp, _vp, _i, _pi], _i),
    "dcrf_set_unary_parameters": ([_vp, _vp, _i], _i),
    "dcrf_label_compatibility_parameters": ([_vp, _vp, _i, _pi], _i),
    "dcrf_set_label_compatibility_parameters": ([_vp, _vp, _i], _i),
    "dcrf_kernel_parameters": ([_vp, _vp, _i, _pi], _i),
    "dcrf_set_kernel_parameters": ([_vp, _vp, _i], _i),
    "dcrf_unary_gradient": ([_vp, _vp, _i, _pi], _i),
    "dcrf_set_checkpoint_interval": ([_vp, _i], _i),
}

_LIB = None


class DenseCRFError(RuntimeError):
    """A failure reported by the device engine (carries the status code)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (status {code})")
        self.code = code


def load():
    """Load the engine library; raises ImportError if it was not built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA engine first "
                "(python -m pydensecrf_gb300.build); there is no CPU fallback")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = lib
    return _LIB


def symbols():
    """Names of every entry point this binding expects the library to export."""
    return sorted(_SIGS)


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().dcrf_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code: int) -> None:
    """Raise the Python exception that the reference's binding would raise."""
    if code == DCRF_OK:
        return
    msg = last_error()
    if code in (DCRF_ERR_INVALID_ARG, DCRF_ERR_KEY_OVERFLOW):
        raise ValueError(msg)
    if code == DCRF_ERR_OOM:
        raise MemoryError(msg)
    raise DenseCRFError(code, msg)
