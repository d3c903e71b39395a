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


class FlatLambdaCDM:
    """Flat LambdaCDM background without radiation: the part of astropy's
    FlatLambdaCDM(H0, Om0) (default Tcmb0 = 0) that the reference uses --
    efunc, h and comoving_distance in Mpc.  The comoving distance
    (c/H0) int_0^z dz'/E(z') is a 64-point Gauss-Legendre quadrature per
    redshift (relative error < 1e-13 for z < 10)."""

    C_KMS = 299792.458

    def __init__(self, H0=67.6, Om0=0.31):
        self.H0 = float(H0)
        self.Om0 = float(Om0)
        self.h = self.H0 / 100.0
        x, wq = np.polynomial.legendre.leggauss(64)
        self._x, self._w = x, wq

    def efunc(self, z):
        z = np.asarray(z, dtype=np.float64)
        return np.sqrt(self.Om0 * (1.0 + z) ** 3 + (1.0 - self.Om0))

    def comoving_distance(self, z):
        z = np.atleast_1d(np.asarray(z, dtype=np.float64))
        half = 0.5 * z[:, None]
        zz = half * (self._x[None, :] + 1.0)                 # nodes mapped to [0, z]
        integ = (self._w[None, :] / self.efunc(zz)).sum(axis=1) * half[:, 0]
        out = self.C_KMS / self.H0 * integ
        return out if np.ndim(z) else out[0]


def radecz_to_cartesian(radecz, cosmo=None):
    """util.py:25-51: (RA, Dec in degrees, redshift) -> comoving Cartesian
    coordinates in Mpc/h.  Unlike the reference, the input array is not
    modified (the reference converts RA and Dec to radians in place).  Any
    object with comoving_distance(z) [Mpc] and h works as ``cosmo``."""
    radecz = np.asarray(radecz, dtype=np.float64)
    assert radecz.shape[0] == 3, "radecz has to be have shape [3,N]"
    if cosmo is None:
        cosmo = FlatLambdaCDM(H0=67.6, Om0=0.31)
    ra = radecz[0] * np.pi / 180.0
    dec = radecz[1] * np.pi / 180.0
    rad = np.asarray(cosmo.comoving_distance(radecz[2]), dtype=np.float64) * cosmo.h
    return np.array([rad * np.cos(dec) * np.cos(ra), rad * np.cos(dec) * np.sin(ra), rad * np.sin(dec)])
