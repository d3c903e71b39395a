"""The C-ABI library builds, loads and exports every symbol include/pyspec_gpu.h
declares.  Only host-side calls (size queries, argument validation that fails
before any CUDA call) run here; nothing touches a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from pyspectrum_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "pyspec_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pyspec_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_loads():
    path = _build.build()
    assert os.path.exists(path)
    lib = _lib.load()
    assert lib.pyspec_abi_version() == 1


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(_build.build())
    names = declared_symbols()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    # and the Python binding knows every declared entry point
    assert set(names) <= set(_lib.SIGNATURES)


def test_workspace_queries_are_host_only():
    lib = _lib.load()
    ws = lib.pyspec_shell_fields_workspace(360, 40)
    nh = 181
    assert ws >= nh * 360 * 360 * 8
    assert lib.pyspec_shell_fields_workspace(1, 1) == 0
    assert lib.pyspec_bk_counts_workspace(360, 3, 1, 40) > 360 ** 3 * 8
    assert lib.pyspec_bk_counts_workspace(360, 3, 0, 40) == 0
    assert lib.pyspec_bk_contract_workspace(360, 40, 6350, 0) > 0


@pytest.mark.parametrize("call", [
    lambda l: l.pyspec_fft3d_c2c(None, 16, 1, None),
    lambda l: l.pyspec_fft3d_c2c(ctypes.c_void_p(16), 14 * 7 * 11, 1, None),
    lambda l: l.pyspec_fcomb_periodic(None, 16, 1.0, None, None),
    lambda l: l.pyspec_shell_fields(ctypes.c_void_p(16), 15, 3, 1, 5, ctypes.c_void_p(16), None, None, 0, None),
    lambda l: l.pyspec_pk_pbox_rsd(ctypes.c_void_p(16), 16, 3, 100, 8, 5, ctypes.c_void_p(16), None),
    lambda l: l.pyspec_pk_pbox_rsd(ctypes.c_void_p(16), 16, 2, 100, 7, 5, ctypes.c_void_p(16), None),
    lambda l: l.pyspec_bk_counts(16, 3, 0, 5, ctypes.c_void_p(16), 1, ctypes.c_void_p(16), None, None, 0, None),
])
def test_invalid_arguments_rejected_before_launch(call):
    lib = _lib.load()
    assert call(lib) == -1
    assert _lib.last_error() != ""


def test_workspace_too_small_reported():
    lib = _lib.load()
    rc = lib.pyspec_shell_fields(ctypes.c_void_p(256), 16, 1, 1, 4, ctypes.c_void_p(256), None,
                                 ctypes.c_void_p(256), 16, None)
    assert rc == -4
    assert "workspace" in _lib.last_error()


@pytest.mark.parametrize("call", [
    lambda l: l.pyspec_fcomb_periodic(ctypes.c_void_p(16), 16, 0.0, ctypes.c_void_p(16), None),
    lambda l: l.pyspec_pk_rsd_python(ctypes.c_void_p(16), 16, 3, 100.0, 5, ctypes.c_void_p(16), None),
    lambda l: l.pyspec_pk_rsd_python(ctypes.c_void_p(16), 16, 2, 100.0, 0, ctypes.c_void_p(16), None),
    lambda l: l.pyspec_pk_rsd_python(ctypes.c_void_p(16), 15, 2, 100.0, 4, ctypes.c_void_p(16), None),
    lambda l: l.pyspec_bk_contract_noalloc(None, 16, 4, None, 1, None, None),
    lambda l: l.pyspec_bk_contract_noalloc(ctypes.c_void_p(16), 16, 0, ctypes.c_void_p(16), 1,
                                           ctypes.c_void_p(16), None),
])
def test_more_invalid_arguments(call):
    lib = _lib.load()
    assert call(lib) == -1
    assert _lib.last_error() != ""


def test_python_layer_rejects_degenerate_catalogues():
    from pyspectrum_gb300 import pyspectrum as P
    with pytest.raises(ValueError, match="empty"):
        P.Bk_periodic(np.zeros((3, 0)), Lbox=100.0, Ngrid=16)
    with pytest.raises(ValueError, match="sum to zero"):
        P.Pk_periodic(np.ones((3, 4)), w=np.zeros(4), Lbox=100.0, Ngrid=16)
    with pytest.raises(ValueError, match="even"):
        P.FFT_periodic(np.ones((3, 4)), Lbox=100.0, Ngrid=15)
