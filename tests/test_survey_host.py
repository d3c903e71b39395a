"""Host parts of the survey (FKP) path: cosmology and coordinates
(util.py:25-51 with astropy's flat LambdaCDM, Tcmb0 = 0).  CPU only."""
import numpy as np
import pytest
from scipy import integrate

from pyspectrum_gb300 import util


def test_comoving_distance_matches_quadrature():
    c = util.FlatLambdaCDM(H0=67.6, Om0=0.31)
    z = np.array([0.0, 0.01, 0.3, 0.57, 1.0, 2.5, 6.0])
    ref = np.array([integrate.quad(lambda x: 1.0 / np.sqrt(0.31 * (1 + x) ** 3 + 0.69), 0, zz, epsabs=0,
                                   epsrel=1e-13)[0] for zz in z]) * 299792.458 / 67.6
    np.testing.assert_allclose(c.comoving_distance(z), ref, rtol=1e-12, atol=1e-9)
    assert c.h == pytest.approx(0.676)


def test_radecz_to_cartesian_geometry_and_no_mutation():
    c = util.FlatLambdaCDM(H0=70.0, Om0=0.3)
    radecz = np.array([[0.0, 90.0, 45.0, 10.0], [0.0, 0.0, 90.0, -30.0], [0.5, 0.5, 0.5, 1.2]])
    keep = radecz.copy()
    xyz = util.radecz_to_cartesian(radecz, cosmo=c)
    np.testing.assert_array_equal(radecz, keep)
    r = c.comoving_distance(radecz[2]) * c.h
    np.testing.assert_allclose(np.sqrt((xyz ** 2).sum(0)), r, rtol=1e-14)
    np.testing.assert_allclose(xyz[:, 0], [r[0], 0, 0], atol=1e-9)
    np.testing.assert_allclose(xyz[:, 1], [0, r[1], 0], atol=1e-9)
    np.testing.assert_allclose(xyz[:, 2], [0, 0, r[2]], atol=1e-9)
