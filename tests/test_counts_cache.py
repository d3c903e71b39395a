"""Count caches in the reference's FortranFile format (pyspectrum.py:962-1056):
reading the reference's shipped cache, writing files its reader accepts, and
installing them as this package's exact counts.  CPU only."""
import os

import numpy as np
import pytest
from scipy.io import FortranFile

from oracle import pyspec_oracle as O
from pyspectrum_gb300 import core, counts_cache as cc
from pyspectrum_gb300 import pyspectrum as P


@pytest.fixture()
def fresh_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("PYSPEC_GB300_CACHE", str(tmp_path / "cache"))
    saved = dict(core._counts_mem)
    core._counts_mem.clear()
    yield tmp_path
    core._counts_mem.clear()
    core._counts_mem.update(saved)


def test_name_convention():
    assert cc.reference_counts_name(360, 40, 3, 3) == "counts.Ngrid360.Nmax40.Ncut3.step3.pyfftw"
    assert cc.reference_counts_name(360, 40, 3, 3, "fort77") == "counts.Ngrid360.Nmax40.Ncut3.step3.fort77"
    with pytest.raises(ValueError):
        cc.reference_counts_name(360, 40, 3, 3, "cufft")


@pytest.mark.parametrize("n,step,nmax", [(16, 1, 8), (48, 2, 20), (90, 3, 40), (64, 3, 40)])
def test_mode_counts_host_matches_oracle(n, step, nmax):
    np.testing.assert_array_equal(cc.mode_counts_host(n, step, nmax), O.mode_counts(n, step, nmax))


def test_reference_cache_roundtrip_and_exact_counts(golden, tmp_path):
    """The shipped Nmax 10 cache (values as the reference's reader returns
    them) written in the reference format, read back bit-identically, and
    rounded to the exact counts."""
    g = golden("counts_ref360.npz")
    raw = g["nmax10_raw"]
    path = tmp_path / cc.reference_counts_name(360, 10, 3, 3)
    cc.write_reference_counts(path, raw, "pyfftw")
    # the file is what the reference's own writer produces (pyspectrum.py:1026-1028)
    ref_path = tmp_path / "ref_writer"
    f = FortranFile(ref_path, "w")
    f.write_record(raw)
    f.close()
    assert path.read_bytes() == ref_path.read_bytes()
    back = cc.read_reference_counts(path, 10, "pyfftw")
    np.testing.assert_array_equal(back, raw)
    counts = cc.counts_from_reference_array(back, 360, 10, 3, 3)
    np.testing.assert_array_equal(counts, g["nmax10"])


def test_fort77_layout(tmp_path):
    """fort77: the Fortran routine's array (filled for i <= j <= l) stored in
    C order; the reader's Fortran-order reshape returns i >= j >= l."""
    S = 6
    rng = np.random.default_rng(3)
    orig = np.zeros((S, S, S), order="F")
    for i in range(S):
        for j in range(i, S):
            for l in range(j, S):
                orig[i, j, l] = rng.integers(1, 100)
    ref_path = tmp_path / "ref_f77"
    f = FortranFile(ref_path, "w")
    f.write_record(orig)                  # as pyspectrum.py:1053-1055 does
    f.close()
    read = cc.read_reference_counts(ref_path, S, "fort77")
    np.testing.assert_array_equal(read, orig.transpose(2, 1, 0))
    assert np.all(read[np.triu_indices(S, 1)[0], np.triu_indices(S, 1)[1], :] == 0)
    mine = tmp_path / "mine_f77"
    cc.write_reference_counts(mine, read, "fort77")
    assert mine.read_bytes() == ref_path.read_bytes()


def test_rejects_non_integer_counts():
    a = np.zeros((5, 5, 5))
    tri = core.triangles(1, 5)
    a[tri[0] - 1, tri[1] - 1, tri[2] - 1] = 16.0 ** 3 * 2
    a[4, 4, 4] += 0.3 * 16 ** 3
    with pytest.raises(ValueError):
        cc.counts_from_reference_array(a, 16, 5, 1, 1)
    with pytest.raises(ValueError):
        cc.counts_from_reference_array(np.zeros((4, 4, 4)), 16, 5, 1, 1)


def test_import_installs_cache(golden, fresh_cache):
    g = golden("counts_ref360.npz")
    path = fresh_cache / cc.reference_counts_name(360, 10, 3, 3)
    cc.write_reference_counts(path, g["nmax10_raw"], "pyfftw")
    counts, nk = cc.import_reference_counts(path, 360, 10, 3, 3)
    np.testing.assert_array_equal(counts, g["nmax10"])
    # served from the in-memory cache and from disk without any GPU work
    c2, nk2 = core.triangle_counts(360, 10, 3, 3)
    np.testing.assert_array_equal(c2, counts)
    core._counts_mem.clear()
    c3, nk3 = core.triangle_counts(360, 10, 3, 3)
    np.testing.assert_array_equal(c3, counts)
    np.testing.assert_array_equal(nk3, nk)
    # and the reference-format array produced from them matches the file up to
    # the reference's rounding noise
    arr = cc.reference_counts_array(360, 10, 3, 3)
    tri = core.triangles(1, 10)
    sel = (tri[0] - 1, tri[1] - 1, tri[2] - 1)
    np.testing.assert_allclose(arr[sel], g["nmax10_raw"][sel], rtol=0, atol=1e-3 * 360 ** 3)


def test_counts_mirror_reads_reference_dat_dir(golden, fresh_cache):
    """_counts_Bk123(dat_dir=...) follows the reference's cache convention:
    an existing file is returned as stored."""
    g = golden("counts_ref360.npz")
    dat = fresh_cache / "dat"
    dat.mkdir()
    cc.write_reference_counts(dat / cc.reference_counts_name(360, 10, 3, 3), g["nmax10_raw"])
    out = P._counts_Bk123(Ngrid=360, Nmax=10, Ncut=3, step=3, dat_dir=str(dat))
    np.testing.assert_array_equal(out, g["nmax10_raw"])
    c, _ = core.triangle_counts(360, 10, 3, 3)
    np.testing.assert_array_equal(c, g["nmax10"])
    assert os.path.exists(core.counts_path(360, 10, 3, 3))
