"""Utilities of the reference (pyspectrum/util.py) used by the periodic-box path."""
from __future__ import annotations

import numpy as np

from .core import efunc


def applyRSD(xyz, vxyz, redshift, h=0.7, omega0_m=0.3, LOS=None, Lbox=None):
    """util.py:54-75: redshift-space positions for a periodic box,
    s_los = (x_los + (1+z)/(100 E(z)) v_los + L) mod L, float64 host arrays.
    E(z) is astropy's FlatLambdaCDM(H0=100h, Om0).efunc with Tcmb0=0 (the
    reference uses that class without importing it, util.py:67)."""
    xyz = np.asarray(xyz)
    vxyz = np.asarray(vxyz)
    assert xyz.shape[0] == 3
    assert vxyz.shape[0] == 3
    if LOS is None:
        raise ValueError("specify line of sight")
    if Lbox is None:
        raise ValueError("specify box size")
    i_los = {'x': 0, 'y': 1, 'z': 2}[LOS]
    rsd_factor = (1 + redshift) / (100 * efunc(redshift, omega0_m))
    xyz_rsd = np.array(xyz, dtype=np.float64, copy=True)
    xyz_rsd[i_los] += rsd_factor * vxyz[i_los] + Lbox
    xyz_rsd[i_los] = (xyz_rsd[i_los] % Lbox)
    return xyz_rsd


def ijl_order(i_k, j_k, l_k, typ='GM'):
    """util.py:8-24: triangle ordering (by l, then j, then i)."""
    i_bq = np.arange(len(i_k))
    if typ != 'GM':
        raise NotImplementedError
    out = []
    for l in np.sort(np.unique(l_k)):
        for j in np.sort(np.unique(j_k[l_k == l])):
            for i in np.sort(np.unique(i_k[(l_k == l) & (j_k == j)])):
                out.append(i_bq[(i_k == i) & (j_k == j) & (l_k == l)])
    return np.array(out)
