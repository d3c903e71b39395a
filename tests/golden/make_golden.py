"""Generate the golden fixtures in this folder from the reference pySpectrum.

Run once in a checkout that has the reference source tree (read-only is fine):

    PYSPEC_REFERENCE=<path to pySpectrum checkout> python tests/golden/make_golden.py [pk_rsd_python | b0_survey]

What it produces (all small, committed):

* ``counts_ref360.npz`` -- the reference's shipped triangle-count caches
  ``pyspectrum/dat/counts.Ngrid360.Nmax{10,40,50}.Ncut3.step3.pyfftw`` and the
  ``.fort77`` twin, reduced to the exact integer number of closed k-triangles
  (count / N^3, rounded; the single-precision ``.fort77`` values unrounded) in
  the reference's loop order, plus the raw float64 Nmax=10 cache for
  file-format interop.
* ``ref_bk_small.npz`` -- outputs of the reference's own ``reflect_delta``,
  ``_Bk_periodic`` and ``_counts_Bk123`` (compute path) on seeded delta(k)
  grids at N = 16, 24, 32.
* ``ref_fft_small.npz`` -- the reference's ``_FFT`` (de-interleave +
  unnormalised backward FFT) on a seeded interlaced grid.
* ``ref_rsd.npz`` -- the reference's ``util.applyRSD`` on fixture halos.
* ``ref_b0_survey.npz`` -- the reference's ``_B0_survey`` (survey FKP
  bispectrum from a full delta(k) and normalisation integrals) at N = 16, 24.
* ``ref_pk_rsd_python.npz`` -- the reference's ``_Pk_periodic_rsd`` with
  ``code='python'`` (its numpy (k, mu) binning) on seeded full delta(k)
  grids at N = 16, 24 for every line of sight.
* ``test_box_f32.npz`` -- the reference's test fixture ``dat/test_box.hdf5``
  (73,442 halo positions and velocities, L = 2600), read from its raw HDF5
  data offsets and stored as float32.

The reference imports pyfftw, astropy and its f2py extension at import time;
none is installed here.  The script therefore registers stand-ins before
importing it:

* ``pyfftw``: the FFTW builders are replaced by numpy's DFTs with FFTW's sign
  and normalisation conventions (FFTW_FORWARD = ``fftn``; FFTW_BACKWARD with
  ``normalise_idft=False`` = ``ifftn * N**3``), keeping the input precision.
* ``astropy.cosmology.FlatLambdaCDM``: ``efunc(z) = sqrt(Om0 (1+z)^3 + 1 - Om0)``
  (flat, Tcmb0 = 0, astropy's default).  ``util.py`` uses the name without
  importing it (util.py:67); the stand-in is injected into that module.
* ``estimator`` (the Fortran extension): every routine raises -- nothing
  golden here runs Fortran code.
"""
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("PYSPEC_REFERENCE", "/root/reference")


def _install_stubs():
    pyfftw = types.ModuleType("pyfftw")

    def n_byte_align_empty(shape, align, dtype="complex128"):
        return np.empty(shape, dtype=dtype)

    class _Plan:
        def __init__(self, a, inverse):
            self.a = a
            self.inverse = inverse

        def __call__(self, input_array=None, normalise_idft=True):
            arr = self.a if input_array is None else input_array
            if self.inverse:
                out = np.fft.ifftn(arr)
                if not normalise_idft:
                    out = out * float(np.prod(arr.shape))
            else:
                out = np.fft.fftn(arr)
            return out.astype(arr.dtype if np.iscomplexobj(arr) else np.complex128)

    builders = types.ModuleType("pyfftw.builders")
    builders.fftn = lambda a, planner_effort=None, threads=1, **k: _Plan(a, False)
    builders.ifftn = lambda a, planner_effort=None, threads=1, **k: _Plan(a, True)
    interfaces = types.ModuleType("pyfftw.interfaces")
    cache = types.ModuleType("pyfftw.interfaces.cache")
    cache.enable = lambda: None
    interfaces.cache = cache
    pyfftw.n_byte_align_empty = n_byte_align_empty
    pyfftw.builders = builders
    pyfftw.interfaces = interfaces
    sys.modules.update({"pyfftw": pyfftw, "pyfftw.builders": builders,
                        "pyfftw.interfaces": interfaces, "pyfftw.interfaces.cache": cache})

    class FlatLambdaCDM:
        def __init__(self, H0, Om0):
            self.H0, self.Om0 = H0, Om0

        def efunc(self, z):
            return np.sqrt(self.Om0 * (1.0 + z) ** 3 + (1.0 - self.Om0))

    astropy = types.ModuleType("astropy")
    cosmology = types.ModuleType("astropy.cosmology")
    cosmology.FlatLambdaCDM = FlatLambdaCDM
    astropy.cosmology = cosmology
    sys.modules.update({"astropy": astropy, "astropy.cosmology": cosmology})

    est = types.ModuleType("estimator")

    def _nofortran(*a, **k):
        raise NotImplementedError("the reference's Fortran extension is not built here")

    for name in ("assign_quad", "fcomb_periodic", "pk_pbox_rsd", "bk_counts", "ffting", "fcomb"):
        setattr(est, name, _nofortran)
    sys.modules["estimator"] = est
    return FlatLambdaCDM


def _loop(jmin, nmax):
    return [(i, j, l) for i in range(jmin, nmax + 1) for j in range(jmin, i + 1)
            for l in range(max(i - j, jmin), j + 1)]


def counts_goldens():
    from scipy.io import FortranFile
    dat = os.path.join(REF, "pyspectrum", "dat")
    out = {}
    V = float(360 ** 3)
    for nmax in (10, 40, 50):
        f = FortranFile(os.path.join(dat, f"counts.Ngrid360.Nmax{nmax}.Ncut3.step3.pyfftw"), "r")
        c = f.read_reals(dtype=np.float64).reshape(nmax, nmax, nmax)
        f.close()
        tri = _loop(1, nmax)
        q = np.array([c[i - 1, j - 1, l - 1] for i, j, l in tri]) / V
        out[f"nmax{nmax}"] = np.rint(q).astype(np.int64)
        out[f"nmax{nmax}_maxdev"] = np.array(np.abs(q - np.rint(q)).max())
        if nmax == 10:
            out["nmax10_raw"] = c
    f = FortranFile(os.path.join(dat, "counts.Ngrid360.Nmax40.Ncut3.step3.fort77"), "r")
    c = f.read_reals(dtype=np.float64).reshape(40, 40, 40, order="F")
    f.close()
    # Fortran bk_counts fills coun(i,j,l) for i <= j <= l (estimator.f:90-97); the
    # cache holds that array serialised in C order, so read back in Fortran
    # order it has the reference's (i >= j >= l) layout.
    # (single-precision FFTW: kept unrounded, it agrees only to ~1e-7 relative)
    out["nmax40_fort77"] = np.array([c[i - 1, j - 1, l - 1] for i, j, l in _loop(1, 40)]) / V
    np.savez_compressed(os.path.join(HERE, "counts_ref360.npz"), **out)


def bk_goldens(ref, tmp):
    ref.dat_dir = lambda: tmp            # the count cache is written here
    cases = [(16, 1, 1, 8), (16, 3, 3, 5), (24, 2, 2, 6), (32, 3, 3, 5)]
    out = {"cases": np.array(cases)}
    for n, step, ncut, nmax in cases:
        rng = np.random.default_rng(1000 + n + step)
        field = rng.standard_normal((n, n, n))
        full = (np.fft.ifftn(field) * n ** 3).astype(np.complex64)
        delt = np.ascontiguousarray(full[: n // 2 + 1])
        delta_fft = ref.reflect_delta(delt, Ngrid=n)
        bk = ref._Bk_periodic(delta_fft, Nmax=nmax, Ncut=ncut, step=step, fft="pyfftw")
        counts = ref._counts_Bk123(Ngrid=n, Nmax=nmax, Ncut=ncut, step=step, fft="pyfftw")
        tag = f"n{n}_s{step}_c{ncut}_m{nmax}"
        out[tag + "_delt"] = delt
        out[tag + "_delta_fft"] = delta_fft
        out[tag + "_countscache"] = counts
        for k, v in bk.items():
            out[tag + "_" + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "ref_bk_small.npz"), **out)


def fft_goldens(ref):
    n = 16
    rng = np.random.default_rng(7)
    _delta = np.asfortranarray(rng.standard_normal((2 * n, n, n)).astype(np.float32))
    ifft = ref._FFT(_delta, fft="pyfftw", Ngrid=n)
    np.savez_compressed(os.path.join(HERE, "ref_fft_small.npz"), interlaced=_delta, out=ifft)


def fixture_and_rsd(ref_util, FlatLambdaCDM):
    raw = open(os.path.join(REF, "pyspectrum", "dat", "test_box.hdf5"), "rb").read()
    n = 73442      # rows of the 'xyz' and 'vxyz' datasets, stored contiguously from byte 2048
    xyz = np.frombuffer(raw[2048: 2048 + n * 24], dtype="<f8").reshape(n, 3)
    vxyz = np.frombuffer(raw[2048 + n * 24: 2048 + n * 48], dtype="<f8").reshape(n, 3)
    np.savez_compressed(os.path.join(HERE, "test_box_f32.npz"), xyz=xyz.astype(np.float32),
                        vxyz=vxyz.astype(np.float32), Lbox=np.array(2600.0))
    ref_util.FlatLambdaCDM = FlatLambdaCDM
    xs = xyz[:2000].T.astype(np.float32).astype(np.float64)
    vs = vxyz[:2000].T.astype(np.float32).astype(np.float64)
    out = {"xyz": xs, "vxyz": vs}
    for los in ("x", "y", "z"):
        out["rsd_" + los] = ref_util.applyRSD(xs, vs, 0.5, h=0.7, omega0_m=0.3, LOS=los, Lbox=2600.0)
    np.savez_compressed(os.path.join(HERE, "ref_rsd.npz"), **out)


def pk_rsd_python_goldens(ref):
    import contextlib
    import io
    out = {}
    cases = [(16, 4, 0), (16, 5, 1), (24, 4, 2), (24, 3, 0)]
    out["cases"] = np.array(cases)
    for n, nmu, rsd in cases:
        rng = np.random.default_rng(500 + n + nmu + rsd)
        full = (np.fft.fftn(rng.standard_normal((n, n, n)) + 0.2) / n ** 1.5).astype(np.complex64)
        with contextlib.redirect_stdout(io.StringIO()):      # the reference prints every bin
            res = ref._Pk_periodic_rsd(full, Lbox=1000.0, rsd=rsd, Nmubin=nmu, code="python")
        tag = f"n{n}_m{nmu}_r{rsd}"
        out[tag + "_delta"] = full
        for name, v in zip(("k", "p0k", "p2k", "p4k", "nk", "k_kmu", "mu_kmu", "p_kmu", "n_kmu"), res):
            out[tag + "_" + name] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "ref_pk_rsd_python.npz"), **out)


def b0_survey_goldens(ref, tmp):
    ref.dat_dir = lambda: tmp            # the count cache is written here
    cases = [(16, 1, 1, 6), (24, 2, 2, 6)]
    out = {"cases": np.array(cases)}
    for n, step, ncut, nmax in cases:
        rng = np.random.default_rng(700 + n)
        full = (np.fft.fftn(rng.standard_normal((n, n, n))) / n ** 1.5).astype(np.complex64)
        ints = rng.uniform(0.5, 2.0, size=5)
        alpha = 0.05
        res = ref._B0_survey(full, alpha, *ints, Nmax=nmax, Ncut=ncut, step=step, fft="pyfftw")
        tag = f"n{n}_s{step}_c{ncut}_m{nmax}"
        out[tag + "_delta"] = full
        out[tag + "_ints"] = ints
        out[tag + "_alpha"] = np.array(alpha)
        for k, v in res.items():
            out[tag + "_" + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "ref_b0_survey.npz"), **out)


def main():
    FlatLambdaCDM = _install_stubs()
    sys.path.insert(0, REF)
    from pyspectrum import pyspectrum as ref
    from pyspectrum import util as ref_util
    if sys.argv[1:] == ["pk_rsd_python"]:           # only this fixture
        pk_rsd_python_goldens(ref)
        return
    if sys.argv[1:] == ["b0_survey"]:               # only this fixture
        with tempfile.TemporaryDirectory() as tmp:
            b0_survey_goldens(ref, tmp)
        return
    pk_rsd_python_goldens(ref)
    with tempfile.TemporaryDirectory() as tmp:
        b0_survey_goldens(ref, tmp)
    counts_goldens()
    with tempfile.TemporaryDirectory() as tmp:
        bk_goldens(ref, tmp)
    fft_goldens(ref)
    fixture_and_rsd(ref_util, FlatLambdaCDM)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
