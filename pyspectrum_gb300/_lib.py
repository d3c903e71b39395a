"""ctypes binding of libpyspec_gb300.so (the C ABI declared in include/pyspec_gpu.h).

Every GPU computation of this package goes through these functions.  There is
no CPU fallback: if the library is missing and cannot be built, importing the
binding raises, and every call checks the returned status.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import _build

_lock = threading.Lock()
_lib = None

c_int, c_i64, c_size, c_double, c_float, c_void = (ctypes.c_int, ctypes.c_int64, ctypes.c_size_t,
                                                   ctypes.c_double, ctypes.c_float, ctypes.c_void_p)
_P = c_void  # device pointer / stream

# name -> (restype, argtypes)
SIGNATURES = {
    "pyspec_abi_version": (c_int, []),
    "pyspec_last_error": (c_int, [ctypes.c_char_p, c_size]),
    "pyspec_launch_count": (c_i64, []),
    "pyspec_prepare_positions": (c_int, [_P, c_i64, _P, c_i64, c_int, c_double, _P, c_i64, c_double, _P, _P, _P]),
    "pyspec_assign_pcs_interlaced": (c_int, [_P, _P, c_i64, c_int, c_float, c_float, _P, _P]),
    "pyspec_assign_tiled_workspace": (c_size, [c_i64, c_int, c_int]),
    "pyspec_assign_pcs_interlaced_tiled": (c_int, [_P, _P, c_i64, c_int, c_float, c_float, c_int, _P, _P, c_size,
                                                   _P]),
    "pyspec_fft3d_c2c": (c_int, [_P, c_int, c_int, _P]),
    "pyspec_fft3d_variants": (c_int, [c_int, _P, c_int]),
    "pyspec_fft3d_c2c_variant": (c_int, [_P, c_int, c_int, c_int, _P]),
    "pyspec_fcomb_periodic": (c_int, [_P, c_int, c_double, _P, _P]),
    "pyspec_reflect_delta": (c_int, [_P, c_int, _P, _P]),
    "pyspec_half_from_full": (c_int, [_P, c_int, _P, _P]),
    "pyspec_mode_counts": (c_int, [c_int, c_int, c_int, _P, _P]),
    "pyspec_shell_fields_workspace": (c_size, [c_int, c_int]),
    "pyspec_shell_fields": (c_int, [_P, c_int, c_int, c_int, c_int, _P, _P, _P, c_size, _P]),
    "pyspec_bk_contract_workspace": (c_size, [c_int, c_int, c_int, c_int]),
    "pyspec_bk_contract": (c_int, [_P, c_int, c_int, _P, _P, c_int, c_int, _P, _P, c_size, _P]),
    "pyspec_bk_contract_noalloc": (c_int, [_P, c_int, c_int, _P, c_int, _P, _P]),
    "pyspec_bk_plan_check": (c_int, [c_int, _P, c_int, _P, c_int]),
    "pyspec_bk_plan_check_flags": (c_int, [c_int, _P, c_int, c_int, _P, c_int]),
    "pyspec_bk_counts_workspace": (c_size, [c_int, c_int, c_int, c_int]),
    "pyspec_bk_counts": (c_int, [c_int, c_int, c_int, c_int, _P, c_int, _P, _P, _P, c_size, _P]),
    "pyspec_bk_normalize": (c_int, [_P, _P, _P, _P, _P, c_int, c_int, c_int, c_int, c_int, c_double, c_double, _P, _P]),
    "pyspec_pk_monopole": (c_int, [_P, c_int, c_double, _P, _P]),
    "pyspec_pk_pbox_rsd": (c_int, [_P, c_int, c_int, c_int, c_int, c_int, _P, _P]),
    "pyspec_pk_rsd_python": (c_int, [_P, c_int, c_int, c_double, c_int, _P, _P]),
    "pyspec_cast_positions": (c_int, [_P, c_i64, _P, c_i64, _P, _P, _P]),
    "pyspec_fcomb_survey": (c_int, [_P, c_int, _P, _P]),
    "pyspec_combine_fields": (c_int, [_P, _P, c_double, c_i64, _P, _P]),
}

CONTRACT_FP32 = 0
CONTRACT_BF16X3 = 1
CONTRACT_BF16X6 = 2
CONTRACT_RUN_PLAN = 0x100
CONTRACT_FINE_DRAIN = 0x200
CONTRACT_KC32 = 0x400


class PyspecError(RuntimeError):
    """A C-ABI call returned a negative status."""


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load (and if needed build) the shared library; raises if unavailable."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(_build.LIB_PATH) or not _build.up_to_date():
            if not build_if_missing:
                raise ImportError(f"{_build.LIB_PATH} is missing; run pyspectrum_gb300._build.build()")
            _build.build()
        lib = ctypes.CDLL(_build.LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(512)
    load().pyspec_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise PyspecError(f"{what} failed with status {rc}: {last_error()}")


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def call(name: str, *args):
    """Call a status-returning entry point and raise on failure."""
    rc = getattr(load(), name)(*args)
    check(rc, name)


def launch_count() -> int:
    return int(load().pyspec_launch_count())
