"""GPU parity of the redshift-space path (applyRSD + Bk_periodic + the P0/P2
multipoles of the same grid) against the oracle: util.py:54-75,
pyspectrum.py:285-356 and :460-538 (code='fortran')."""
import numpy as np
import pytest

from oracle import pyspec_oracle as O
from pyspectrum_gb300 import pyspectrum as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("los", ["x", "z"])
@pytest.mark.parametrize("method", ["fp32", "bf16x3"])
def test_bk_periodic_rsd_matches_oracle(los, method):
    n, L, step, ncut, nmax, npart = 48, 1000.0, 2, 2, 12, 40000
    rng = np.random.default_rng(21)
    # clustered positions (so that B and P2 are not pure shot noise) with
    # Gaussian velocities of 300 km/s per component
    centres = rng.uniform(0, L, size=(3, 400))
    xyz = (centres[:, rng.integers(0, 400, npart)] + rng.normal(0, 15.0, size=(3, npart))) % L
    vxyz = rng.normal(0, 300.0, size=(3, npart))
    z, om = 0.5, 0.3
    got = P.Bk_periodic_rsd(xyz, vxyz, z, h=0.7, omega0_m=om, LOS=los, Lbox=L, Ngrid=n, step=step, Ncut=ncut,
                            Nmax=nmax, Nmubin=5, method=method)
    xs = O.applyRSD(xyz, vxyz, z, h=0.7, omega0_m=om, LOS=los, Lbox=L)
    ref = O.Bk_periodic(xs, Lbox=L, Ngrid=n, step=step, Ncut=ncut, Nmax=nmax)
    for k in ("i_k1", "i_k2", "i_k3"):
        np.testing.assert_array_equal(got[k], ref[k])
    np.testing.assert_allclose(got["counts"], ref["counts"], rtol=1e-12)
    np.testing.assert_allclose(got["p0k1"], ref["p0k1"], rtol=2e-5, atol=1e-6 * np.abs(ref["p0k1"]).max())
    rt = 2e-5 if method == "fp32" else 1e-4
    tot_g = got["b123"] + got["b123_sn"]
    tot_r = ref["b123"] + ref["b123_sn"]
    np.testing.assert_allclose(tot_g, tot_r, rtol=rt, atol=rt * np.abs(tot_r).max())
    assert got["meta"]["LOS"] == los and got["meta"]["N"] == npart
    # multipoles of the same redshift-space grid
    pk = got["pk"]
    pref = O.Pk_periodic_rsd(xs, Lbox=L, Ngrid=n, rsd={"x": 0, "y": 1, "z": 2}[los], Nmubin=5)
    np.testing.assert_array_equal(pk["counts"], pref["counts"])
    for key in ("k", "p0k", "p2k", "p4k"):
        r = pref[key]
        np.testing.assert_allclose(pk[key], r, rtol=3e-5, atol=3e-5 * np.abs(r).max(), err_msg=key)
    # the quadrupole carries the RSD signal: it is not zero along the LOS
    assert np.abs(pk["p2k"][1:8]).max() > 1e-3 * np.abs(pk["p0k"][1:8]).max()
