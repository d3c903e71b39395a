"""pyspectrum_gb300: GB300-native periodic-box power spectrum and bispectrum.

A drop-in for the periodic-box path of pySpectrum: ``pyspectrum_gb300.pyspectrum``
mirrors ``pyspectrum.pyspectrum`` (FFT_periodic, Pk_periodic, Pk_periodic_rsd,
Bk_periodic, ...) and ``pyspectrum_gb300.util`` mirrors ``pyspectrum.util``.
All arithmetic runs in libpyspec_gb300.so (sm_103a CUDA, C ABI in
include/pyspec_gpu.h).
"""
import os

from . import _build, _lib  # noqa: F401

__version__ = "0.1.0"


def dat_dir():
    """Directory of cached data (triangle counts); the reference's dat_dir()."""
    from .core import cache_dir
    return cache_dir()


def build(force: bool = False) -> str:
    """Compile libpyspec_gb300.so for sm_103a (in-tree)."""
    return _build.build(force=force)


def lib_path() -> str:
    return _build.LIB_PATH


def native_loaded() -> bool:
    return _lib._lib is not None and os.path.exists(_build.LIB_PATH)
