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


def test_pk_rsd_python_binning_matches_reference(golden):
    """code='python' (pyspectrum.py:545-611) against the reference's own numpy
    binning: mode counts per (k, mu) bin exactly, values to float32 rounding."""
    g = golden("ref_pk_rsd_python.npz")
    names = ("k", "p0k", "p2k", "p4k", "nk", "k_kmu", "mu_kmu", "p_kmu", "n_kmu")
    for n, nmu, rsd in g["cases"]:
        tag = f"n{n}_m{nmu}_r{rsd}"
        got = P._Pk_periodic_rsd(g[tag + "_delta"], Lbox=1000.0, rsd=int(rsd), Nmubin=int(nmu), code="python")
        scale = np.abs(g[tag + "_p0k"]).max()
        for name, v in zip(names, got):
            r = g[tag + "_" + name]
            if name in ("nk", "n_kmu"):
                np.testing.assert_array_equal(v, r, err_msg=tag + name)
            elif name in ("p2k", "p4k"):
                # Legendre-weighted sums cancel: bound the error by the monopole scale
                np.testing.assert_allclose(v, r, rtol=2e-6, atol=2e-6 * scale, err_msg=tag + name)
            else:
                np.testing.assert_allclose(v, r, rtol=2e-6, atol=1e-9 * np.abs(r).max(), err_msg=tag + name)


@pytest.mark.parametrize("rsd", [0, 2])
def test_pk_periodic_rsd_python_code_matches_oracle(rsd):
    n, L, npart = 32, 1000.0, 30000
    rng = np.random.default_rng(40 + rsd)
    xyz = rng.uniform(0, L, size=(3, npart))
    got = P.Pk_periodic_rsd(xyz, Lbox=L, Ngrid=n, rsd=rsd, Nmubin=4, code="python")
    half = O.FFT_periodic(xyz, Lbox=L, Ngrid=n)
    ref = O.pk_rsd_python(O.reflect_delta(half, n), Lbox=L, rsd=rsd, Nmubin=4)
    nbar = npart / L ** 3
    np.testing.assert_array_equal(got["counts"], ref[4])
    np.testing.assert_array_equal(got["counts_kmu"], ref[8])
    np.testing.assert_allclose(got["p0k"] + 1 / nbar, ref[1], rtol=3e-5)
    np.testing.assert_allclose(got["p2k"], ref[2], rtol=3e-5, atol=3e-5 * np.abs(ref[1]).max())
    np.testing.assert_allclose(got["k"], ref[0], rtol=1e-12)
