"""GPU parity: power-spectrum monopole and pk_pbox_rsd multipoles vs the oracle,
and the reference's own smoke tests on its fixture."""
import numpy as np
import pytest

from oracle import pyspec_oracle as O
from pyspectrum_gb300 import pyspectrum as P
from pyspectrum_gb300 import util

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,npart,L", [(32, 20000, 1000.0), (64, 50000, 2600.0)])
def test_pk_periodic_matches_oracle(n, npart, L):
    rng = np.random.default_rng(n)
    xyz = rng.uniform(0, L, size=(3, npart))
    ref = O.Pk_periodic(xyz, Lbox=L, Ngrid=n)
    got = P.Pk_periodic(xyz, Lbox=L, Ngrid=n)
    np.testing.assert_array_equal(got["counts"], ref["counts"])
    np.testing.assert_allclose(got["k"], ref["k"], rtol=1e-6)
    np.testing.assert_allclose(got["p0k"] + got["p0k_sn"], ref["p0k"] + ref["p0k_sn"], rtol=2e-5)


@pytest.mark.parametrize("irsd", [0, 1, 2])
@pytest.mark.parametrize("n,nmu", [(32, 10), (48, 7)])
def test_pk_pbox_rsd_matches_oracle(irsd, n, nmu):
    L = 1500.0
    rng = np.random.default_rng(irsd + n)
    xyz = rng.uniform(0, L, size=(3, 30000))
    half = O.FFT_periodic(xyz, Lbox=L, Ngrid=n)
    ref = O.pk_pbox_rsd(half, irsd, L, n // 2, nmu, n)
    got = P._Pk_periodic_rsd(half.astype(np.complex64), Lbox=L, rsd=irsd, Nmubin=nmu)
    norm = (2 * np.pi) ** 3
    names = ["k", "p0", "p2", "p4", "nk", "km", "mk", "pkm", "nkm"]
    scale = {"p0": norm, "p2": norm, "p4": norm, "pkm": norm}
    for name, r, gv in zip(names, ref, got):
        r = r * scale.get(name, 1.0)
        if name in ("nk", "nkm"):
            np.testing.assert_array_equal(gv, r, err_msg=name)     # exact mode and mu-bin selection
        else:
            np.testing.assert_allclose(gv, r, rtol=3e-5, atol=1e-6 * np.abs(r).max(), err_msg=name)


def _fixture(golden):
    f = golden("test_box_f32.npz")
    return f["xyz"].astype(np.float64), f["vxyz"].astype(np.float64), float(f["Lbox"])


@pytest.mark.parametrize("pt,space", [(2, "real"), (2, "rsd"), (3, "real"), (3, "rsd")])
def test_reference_smoke(golden, pt, space):
    """tests/test_pyspec.py:11-38 of the reference, against this package."""
    xyz, vxyz, Lbox = _fixture(golden)
    Ngrid = 360
    if space == "rsd":
        xyz_s = util.applyRSD(xyz.T, vxyz.T, 0.5, h=0.7, omega0_m=0.3, LOS="z", Lbox=Lbox)
    pos = xyz.T if space == "real" else xyz_s
    if pt == 2:
        spec = P.Pk_periodic(pos, Lbox=Lbox, Ngrid=Ngrid, silent=False)
        assert spec["p0k"].mean() > 0.
    else:
        spec = P.Bk_periodic(pos, Lbox=Lbox, Ngrid=Ngrid, silent=False)
        assert len(spec["b123"]) == 6350
        assert spec["b123"].mean() > 0.
