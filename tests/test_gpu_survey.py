"""GPU parity of the survey-geometry (FKP) bispectrum: pyspectrum.py:13-282,
731-826 and estimator.f:677-745, against the reference's own _B0_survey output
and against the oracle end to end."""
import numpy as np
import pytest

from oracle import pyspec_oracle as O
from pyspectrum_gb300 import pyspectrum as P
from pyspectrum_gb300 import util

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["fp32", "bf16x3"])
def test_b0_survey_stage_matches_reference_golden(golden, method):
    g = golden("ref_b0_survey.npz")
    for n, step, ncut, nmax in g["cases"]:
        tag = f"n{n}_s{step}_c{ncut}_m{nmax}"
        got = P._B0_survey(g[tag + "_delta"], float(g[tag + "_alpha"]), *g[tag + "_ints"], Nmax=int(nmax),
                           Ncut=int(ncut), step=int(step), method=method)
        for k in ("i_k1", "i_k2", "i_k3"):
            np.testing.assert_array_equal(got[k], g[tag + "_" + k])
        rt = 1e-5 if method == "fp32" else 5e-5
        for k in ("p0k1", "b123", "counts"):
            r = g[tag + "_" + k]
            np.testing.assert_allclose(got[k], r, rtol=rt, atol=rt * np.abs(r).max(), err_msg=tag + k)


def _survey_catalogue(rng, npart, zlo, zhi, clustered=False):
    ra = rng.uniform(0, 60.0, npart)
    dec = np.degrees(np.arcsin(rng.uniform(0.0, 0.6, npart)))
    z = rng.uniform(zlo, zhi, npart)
    if clustered:        # objects scattered around 200 centres (structure for the FKP field)
        k = rng.integers(0, 200, npart)
        ra = (ra[k] + rng.normal(0, 0.8, npart)) % 60.0
        dec = np.clip(dec[k] + rng.normal(0, 0.8, npart), 0.0, 36.0)
        z = np.clip(z[k] + rng.normal(0, 0.002, npart), zlo, zhi)
    return np.array([ra, dec, z])


def test_b0_survey_end_to_end_matches_oracle():
    rng = np.random.default_rng(17)
    L, n, step, ncut, nmax = 1200.0, 32, 2, 2, 8
    cosmo = util.FlatLambdaCDM(H0=67.6, Om0=0.31)
    data = _survey_catalogue(rng, 20_000, 0.05, 0.15, clustered=True)
    rand = _survey_catalogue(rng, 80_000, 0.05, 0.15)
    nb_d = np.full(data.shape[1], 3e-4)
    nb_r = np.full(rand.shape[1], 3e-4)
    got = P.B0_survey(data, nb_d, radecz_r=rand, nbar_r=nb_r, P0_fkp=1e4, Lbox=L, Ngrid=n, step=step, Ncut=ncut,
                      Nmax=nmax, cosmo=cosmo)
    # oracle: the same Cartesian positions through the restated FFT_survey_mono and _B0_survey
    hd, Nd, *Id = O.FFT_survey_mono(util.radecz_to_cartesian(data, cosmo), nb_d, P0_fkp=1e4, Lbox=L, Ngrid=n)
    hr, Nr, *Ir = O.FFT_survey_mono(util.radecz_to_cartesian(rand, cosmo), nb_r, P0_fkp=1e4, Lbox=L, Ngrid=n)
    alpha = Nd / Nr
    full = O.reflect_delta(hd, n) - alpha * O.reflect_delta(hr, n)
    ref = O._B0_survey(full, alpha, *(alpha * v for v in Ir), Nmax=nmax, Ncut=ncut, step=step)
    for k in ("i_k1", "i_k2", "i_k3"):
        np.testing.assert_array_equal(got[k], ref[k])
    for k in ("p0k1", "b123", "counts"):
        np.testing.assert_allclose(got[k], ref[k], rtol=2e-4, atol=2e-4 * np.abs(ref[k]).max(), err_msg=k)
    assert got["meta"]["N"] == data.shape[1]
    with pytest.raises(ValueError):
        P.B0_survey(data, nb_d, Lbox=L, Ngrid=n)
