"""Text outputs in the layout of the reference's driver scripts.

run/fastpm/fastpm.py writes the bispectrum as a 10-column text table
(:150-166: i_k1, i_k2, i_k3, p0k1, p0k2, p0k3, b123, q123, counts, b123_sn;
three integer columns, then '%.5e') and the power-spectrum monopole as a
3-column table (:95-103: k, p0k, counts), both with ``np.savetxt`` headers,
and reads them back with ``np.loadtxt(skiprows=1, unpack=True)``.  These
helpers write and read the same files from this package's result
dictionaries, so downstream scripts keep working unchanged.
"""
from __future__ import annotations

import numpy as np

__all__ = ["save_bk", "load_bk", "save_pk", "load_pk", "BK_COLUMNS"]

BK_COLUMNS = ("i_k1", "i_k2", "i_k3", "p0k1", "p0k2", "p0k3", "b123", "q123", "counts", "b123_sn")
_BK_FMT = "%i %i %i %.5e %.5e %.5e %.5e %.5e %.5e %.5e"


def save_bk(path, bispec: dict, Lbox: float, order=None) -> None:
    """The 10-column bispectrum table of run/fastpm/fastpm.py:160-166.
    ``order``: optional triangle permutation (e.g. util.ijl_order(...))."""
    cols = [np.asarray(bispec[k]) for k in BK_COLUMNS]
    if order is not None:
        idx = np.asarray(order).ravel()
        cols = [c[idx] for c in cols]
    hdr = "pyspectrum bispectrum calculation test. k_f = 2pi/%.1f" % Lbox
    hdr += "\n i_k1, i_k2, i_k3, p0k1, p0k2, p0k3, bk, qk, counts, bk_shotnoise"
    np.savetxt(path, np.array(cols).T, fmt=_BK_FMT, delimiter="\t", header=hdr)


def load_bk(path) -> dict:
    """Read a table written by save_bk (or by the reference's driver)."""
    cols = np.loadtxt(path, skiprows=1, unpack=True, usecols=range(10))
    out = dict(zip(BK_COLUMNS, cols))
    for k in ("i_k1", "i_k2", "i_k3"):
        out[k] = out[k].astype(np.int64)
    return out


def save_pk(path, k, p0k, counts, Nhalo: int, Lbox: float, kf: float, nbar: float) -> None:
    """The 3-column monopole table of run/fastpm/fastpm.py:99-102
    (k and p0k in the caller's units, as the driver converts them first)."""
    hdr = "pySpectrum P_l=0(k). Nhalo=%i, Lbox=%.f, k_f=%.5e, SN=%.5e" % (Nhalo, Lbox, kf, 1.0 / nbar)
    hdr += "\n k, p0k, counts"
    np.savetxt(path, np.array([k, p0k, counts]).T, fmt="%.5e %.5e %.5e", delimiter="\t", header=hdr)


def load_pk(path):
    """(k, p0k, counts) from a table written by save_pk or the reference's driver."""
    return np.loadtxt(path, skiprows=1, unpack=True, usecols=[0, 1, 2])
