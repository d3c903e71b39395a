"""Triangle-count caches in the reference's file format.

The reference stores the bispectrum normalisation
counts[i-1, j-1, l-1] = sum_x I_i I_j I_l (= N^3 x the number of closed
k-triangles with k_a in shells i, j, l) as ONE Fortran unformatted sequential
record of float64 values, written and read with ``scipy.io.FortranFile``
(4-byte record-length marker, payload, marker), in its ``dat/`` folder under
``counts.Ngrid{N}.Nmax{S}.Ncut{c}.step{s}.{fft}``:

* ``fft='pyfftw'`` / ``'numpy'`` (pyspectrum.py:962-1030): the (S, S, S)
  array filled for i >= j >= l, serialised in C order and read back with a
  C-order reshape.
* ``fft='fort77'`` (pyspectrum.py:1033-1056, estimator.f:2-102): the Fortran
  routine fills coun(i, j, l) for i <= j <= l of a Fortran-ordered array, the
  record holds that array's C-order bytes, and the reader reshapes in Fortran
  order, which puts the values at [i-1, j-1, l-1] with i >= j >= l again.

This package keeps exact int64 counts (one per loop triangle) instead.  The
functions here convert in both directions, so a user can hand over the
reference's caches (skipping the count computation) or produce caches the
reference reads.
"""
from __future__ import annotations

import os

import numpy as np

from . import core

__all__ = ["reference_counts_name", "read_reference_counts", "write_reference_counts",
           "reference_counts_array", "counts_from_reference_array", "import_reference_counts",
           "mode_counts_host"]

_FORMATS = ("pyfftw", "numpy", "fort77")


def reference_counts_name(Ngrid, Nmax, Ncut, step, fft="pyfftw") -> str:
    """File name convention of pyspectrum.py:966 and :1037."""
    if fft not in _FORMATS:
        raise ValueError(f"fft must be one of {_FORMATS}")
    return f"counts.Ngrid{Ngrid}.Nmax{Nmax}.Ncut{Ncut}.step{step}.{fft}"


def read_reference_counts(path, Nmax, fft="pyfftw") -> np.ndarray:
    """(Nmax, Nmax, Nmax) float64 array exactly as the reference's reader
    returns it (pyspectrum.py:969-973 for pyfftw/numpy, :1040-1043 for fort77)."""
    from scipy.io import FortranFile
    with FortranFile(path, "r") as f:
        flat = f.read_reals(dtype=np.float64)
    if flat.size != Nmax ** 3:
        raise ValueError(f"{path}: record holds {flat.size} values, expected Nmax^3 = {Nmax ** 3}")
    return flat.reshape((Nmax, Nmax, Nmax), order="F" if fft == "fort77" else "C")


def write_reference_counts(path, arr, fft="pyfftw") -> None:
    """Write a cache the reference's reader accepts.  ``arr`` is in the layout
    ``read_reference_counts`` returns (values at i >= j >= l); for fort77 it is
    stored the way the Fortran path writes it (its i <= j <= l array in C order)."""
    from scipy.io import FortranFile
    a = np.asarray(arr, dtype=np.float64)
    if fft == "fort77":
        # the reader reshapes in Fortran order: store the C-order bytes of the
        # array whose Fortran-order reading is `a`, i.e. a's Fortran-order bytes
        payload = np.ascontiguousarray(a.ravel(order="F"))
    else:
        payload = np.ascontiguousarray(a).ravel()
    tmp = str(path) + ".tmp"
    with FortranFile(tmp, "w") as f:
        f.write_record(payload)
    os.replace(tmp, path)


def reference_counts_array(Ngrid, Nmax, Ncut, step, device=None) -> np.ndarray:
    """The (Nmax, Nmax, Nmax) float64 normalisation array of the reference
    (values at [i-1, j-1, l-1] for the loop's i >= j >= l, zero elsewhere) from
    this package's exact counts: counts x Ngrid^3, exact in float64."""
    c, _ = core.triangle_counts(Ngrid, Nmax, Ncut, step, device=device)
    tri = core.triangles(Ncut // step, Nmax)
    out = np.zeros((Nmax, Nmax, Nmax))
    out[tri[0] - 1, tri[1] - 1, tri[2] - 1] = c.astype(np.float64) * float(Ngrid) ** 3
    return out


def counts_from_reference_array(arr, Ngrid, Nmax, Ncut, step, max_dev=1e-3) -> np.ndarray:
    """Exact int64 counts in loop order from a reference array: rint(c / N^3).

    The reference's values are sums of FP32/FP64 FFT products, off the exact
    integers by rounding noise (below 1e-4 in the shipped caches).  A value
    further than ``max_dev`` from an integer means the file is not a count
    cache of this geometry, and raises ValueError."""
    a = np.asarray(arr, dtype=np.float64)
    if a.shape != (Nmax, Nmax, Nmax):
        raise ValueError(f"counts array has shape {a.shape}, expected {(Nmax,) * 3}")
    tri = core.triangles(Ncut // step, Nmax)
    q = a[tri[0] - 1, tri[1] - 1, tri[2] - 1] / float(Ngrid) ** 3
    r = np.rint(q)
    dev = np.abs(q - r)
    if tri.shape[1] and dev.max() > max_dev:
        t = int(dev.argmax())
        raise ValueError(f"count of triangle {tuple(int(x) for x in tri[:, t])} is {q[t]:.6f} x N^3: "
                         f"not an integer within {max_dev}")
    return r.astype(np.int64)


def mode_counts_host(Ngrid, step, Nmax) -> np.ndarray:
    """Nk[0..Nmax]: number of grid modes in each shell (pyspectrum.py:984-987),
    counted on the host with the exact integer shell rule
    n(d2) = max n with (2n-1)^2 step^2 <= 4 d2, d2 = a^2 + b^2 + c^2,
    a = min(i, N - i)."""
    n = int(Ngrid)
    a = np.minimum(np.arange(n), n - np.arange(n)).astype(np.int64)
    sq = a * a
    h1 = np.bincount(sq)                                     # histogram of a^2
    h2 = np.zeros(2 * h1.size - 1, dtype=np.int64)           # of a^2 + b^2
    for v in np.nonzero(h1)[0]:
        h2[v:v + h1.size] += h1[v] * h1
    h3 = np.zeros(h2.size + h1.size - 1, dtype=np.int64)     # of a^2 + b^2 + c^2
    for v in np.nonzero(h1)[0]:
        h3[v:v + h2.size] += h1[v] * h2
    d2 = np.arange(h3.size, dtype=np.int64)
    shell = np.floor(np.sqrt(d2.astype(np.float64)) / step + 0.5).astype(np.int64)
    s2 = step * step
    shell -= ((2 * shell - 1) ** 2 * s2 > 4 * d2) & (shell > 0)   # exact integer correction
    shell += (2 * shell + 1) ** 2 * s2 <= 4 * d2
    keep = shell <= Nmax
    return np.bincount(shell[keep], weights=h3[keep], minlength=Nmax + 1).astype(np.int64)[:Nmax + 1]


def import_reference_counts(path, Ngrid, Nmax, Ncut, step, fft="pyfftw", use_disk=True):
    """Install a reference count cache as this package's count cache for the
    geometry (in memory and, with ``use_disk``, in ``core.cache_dir()``), so
    that Bk_periodic skips the count computation.  Returns (counts, nk)."""
    arr = read_reference_counts(path, Nmax, fft)
    counts = counts_from_reference_array(arr, Ngrid, Nmax, Ncut, step)
    nk = mode_counts_host(Ngrid, step, Nmax)
    core.install_triangle_counts(Ngrid, Nmax, Ncut, step, counts, nk, use_disk=use_disk)
    return counts, nk
