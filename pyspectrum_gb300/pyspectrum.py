"""The reference's periodic-box call surface (pyspectrum/pyspectrum.py) on GB300.

Same function names, arguments, binning and output dictionaries as the
reference; the arithmetic runs in libpyspec_gb300.so (hand-written sm_103a
CUDA behind a C ABI).  Differences from the reference, all deliberate:

* ``Bk_periodic`` does not assert ``Ngrid == 360`` (pyspectrum.py:332).
* Bispectrum outputs keep only triangles with counts > 0, with every array
  aligned (the reference appends zeros to its value arrays but not to its
  index arrays for zero-count triangles, pyspectrum.py:438-445).
* ``Pk_periodic`` bins the reflected grid (the reference indexes the half
  grid with a full-grid mask at pyspectrum.py:713, which raises); so does
  ``Pk_periodic_rsd(code='python')`` (its numpy binning, pyspectrum.py:545-611,
  cannot index the half grid it is handed).
* ``fft`` and ``nthreads`` are accepted and ignored: every FFT is the
  library's own.  ``method`` selects the contraction ('fp32' CUDA cores or
  'bf16x3' tensor cores).
* ``Bk_periodic_rsd`` is new (the reference composes applyRSD + Bk_periodic).
* ``Bk_periodic_batch`` is new: many boxes of mixed grid sizes per call
  (CUDA-graph replay of the per-geometry stages).
* ``Ncut // step`` must be >= 1.
"""
from __future__ import annotations

import os

import numpy as np
import torch

from . import core
from .batch import Bk_periodic_batch  # noqa: F401  (many boxes per call; no reference counterpart)
from .survey import B0_survey, FFT_survey_mono, _B0_survey  # noqa: F401  (pyspectrum.py:13-282, 731-826)
from .util import applyRSD  # noqa: F401  (re-exported as the tests of the reference expect)

__all__ = ["FFT_periodic", "FFTperiodic", "reflect_delta", "Pk_periodic", "Pk_periodic_rsd", "_Pk_periodic_rsd",
           "Bk_periodic", "_Bk_periodic", "Bk_periodic_rsd", "_counts_Bk123", "_counts_Bk123_f77",
           "applyRSD", "Bk_periodic_batch", "B0_survey", "_B0_survey", "FFT_survey_mono"]


def _weight_sum(w, n):
    """Sum of the weights as float64 (the reference sums a float64 weight
    array, pyspectrum.py:921-925); unit weights sum to n exactly, so no array
    is built for them."""
    return float(n) if w is None else float(np.sum(np.asarray(w, dtype=np.float64)))


def _half_to_numpy(half: torch.Tensor) -> np.ndarray:
    """Device [z, y, x] half grid -> numpy [x, y, z] (Fortran-ordered view), complex64."""
    return half.cpu().numpy().transpose(2, 1, 0)


def _half_from_numpy(delt, device=None) -> torch.Tensor:
    """numpy [x, y, z] half grid (N//2+1, N, N) -> device [z, y, x]."""
    a = torch.as_tensor(np.asarray(delt, dtype=np.complex64))
    return a.permute(2, 1, 0).contiguous().to(core._dev(device))


def _delta_half_device(xyz, w, Lbox, Ngrid, vel=None, los=2, rsd_factor=0.0, device=None):
    npart = np.asarray(xyz).shape[1] if not torch.is_tensor(xyz) else xyz.shape[1]
    if npart == 0:
        raise ValueError("empty catalogue: the density contrast needs at least one object")
    if int(Ngrid) < 4 or int(Ngrid) % 2:
        raise ValueError("Ngrid must be even and >= 4")
    wsum = _weight_sum(w, npart)
    if wsum == 0.0:
        raise ValueError("the weights sum to zero (the density is normalised by their sum)")
    dev = core._dev(device)
    xyz_d = core.positions_to_device(xyz, dev)
    w_d = None if w is None else torch.as_tensor(np.asarray(w, dtype=np.float64), device=dev)
    v_d = None if vel is None else core.positions_to_device(vel, dev)
    xyzs, ws = core.prepare_positions(xyz_d, Lbox, w_d, v_d, los, rsd_factor)
    return core.fft_periodic_half(xyzs, ws, Ngrid, Lbox, wsum), npart, wsum


def FFT_periodic(xyz, w=None, Lbox=2600., Ngrid=360, fft='pyfftw', silent=True, device=None):
    """pyspectrum.py:909-959: particles -> half-complex delta(k), shape
    (Ngrid//2+1, Ngrid, Ngrid) complex64, indexed [x, y, z]."""
    half, npart, wsum = _delta_half_device(xyz, w, Lbox, Ngrid, device=device)
    if not silent:
        print('%i positions, Ntot=%.f' % (npart, wsum))
    return _half_to_numpy(half)


FFTperiodic = FFT_periodic   # name used by the reference's run scripts


def reflect_delta(delt, Ngrid=360, silent=True, device=None):
    """pyspectrum.py:1134-1157: half grid -> full (Ngrid, Ngrid, Ngrid) complex64 [x, y, z]."""
    half = _half_from_numpy(delt, device)
    full = core.reflect_half(half)
    return np.ascontiguousarray(full.cpu().numpy().transpose(2, 1, 0))


def _counts_Bk123(Ngrid=360, Nmax=40, Ncut=3, step=3, fft='pyfftw', silent=True, device=None, dat_dir=None):
    """pyspectrum.py:962-1030: (Nmax, Nmax, Nmax) float64 array with
    counts[i-1, j-1, l-1] = sum_x I_i I_j I_l = N^3 x (number of closed
    k-triangles), for the triangle loop's (i, j, l).

    With ``dat_dir`` the reference's cache convention applies: an existing
    ``counts.Ngrid..{fft}`` file there is read and returned as stored (and its
    rounded counts become this package's cache for the geometry); otherwise
    the counts are computed and written there in the reference's format."""
    from . import counts_cache as cc
    if dat_dir is not None:
        path = os.path.join(dat_dir, cc.reference_counts_name(Ngrid, Nmax, Ncut, step, fft))
        if os.path.isfile(path):
            arr = cc.read_reference_counts(path, Nmax, fft)
            counts = cc.counts_from_reference_array(arr, Ngrid, Nmax, Ncut, step)
            core.install_triangle_counts(Ngrid, Nmax, Ncut, step, counts, cc.mode_counts_host(Ngrid, step, Nmax))
            return arr
        if not silent:
            print("--- calculating %s ---" % path)
    out = cc.reference_counts_array(Ngrid, Nmax, Ncut, step, device=device)
    if dat_dir is not None:
        cc.write_reference_counts(path, out, fft)
    return out


def _counts_Bk123_f77(Ngrid=360, Nmax=40, Ncut=3, step=3, silent=True, device=None, dat_dir=None):
    """pyspectrum.py:1033-1056 (Fortran bk_counts, estimator.f:2-102): the same
    normalisation in the layout the reference's fort77 cache reader returns
    (values at [i-1, j-1, l-1] for i >= j >= l).  With ``dat_dir`` the
    ``counts...fort77`` file there is read, or written after computing."""
    return _counts_Bk123(Ngrid, Nmax, Ncut, step, fft='fort77', silent=silent, device=device, dat_dir=dat_dir)


def _bk_from_half(half, Ngrid, step, Ncut, Nmax, method, units=None, device=None):
    plan = core.get_plan(Ngrid, step, Ncut, Nmax, method, device)
    if units is None:
        plan.run(half)
        return plan.result(False)
    nbar, kf = units
    plan.run(half, True, nbar, kf)
    return plan.result(True)


def _Bk_periodic(delta, Nmax=40, Ncut=3, step=3, fft='pyfftw', nthreads=1, silent=True, method='fp32',
                 device=None):
    """pyspectrum.py:359-457 on a full delta(k) grid (N, N, N) [x, y, z]."""
    n = np.asarray(delta).shape[0]
    full = torch.as_tensor(np.asarray(delta, dtype=np.complex64)).permute(2, 1, 0).contiguous().to(core._dev(device))
    half = core.half_from_full(full)
    del full
    return _bk_from_half(half, n, step, Ncut, Nmax, method, device=device)


def Bk_periodic(xyz, w=None, Lbox=2600, Ngrid=360, step=3, Ncut=3, Nmax=40, fft='pyfftw', nthreads=1, silent=True,
                method='fp32', device=None):
    """pyspectrum.py:285-356: B0/Q0 of a periodic box.  Keys 'meta', 'i_k1',
    'i_k2', 'i_k3', 'p0k1', 'p0k2', 'p0k3', 'b123', 'q123', 'counts',
    'p0k_sn', 'b123_sn'."""
    N = np.asarray(xyz).shape[1] if not torch.is_tensor(xyz) else xyz.shape[1]
    half, _, wsum = _delta_half_device(xyz, w, Lbox, Ngrid, device=device)
    nbar = wsum / Lbox ** 3
    kf = 2 * np.pi / Lbox
    if not silent:
        print('------------------')
        print('%i positions in %i box' % (N, Lbox))
        print('sum w_i = %f' % wsum)
        print('nbar = %f' % nbar)
    bispec = _bk_from_half(half, Ngrid, step, Ncut, Nmax, method, units=(nbar, kf), device=device)
    bispec['meta'] = {'Lbox': Lbox, 'Ngrid': Ngrid, 'step': step, 'Ncut': Ncut, 'Nmax': Nmax, 'N': N,
                      'nbar': nbar, 'kf': kf}
    bispec['p0k_sn'] = 1. / nbar
    return bispec


def _Pk_periodic_rsd(delta, Lbox=None, rsd=2, Nmubin=5, code='fortran', device=None):
    """pyspectrum.py:541-641, both binnings; includes the (2 pi)^3 factor.

    code='fortran' (estimator.f:155-264): ``delta`` is the half grid
    (N//2+1, N, N) [x, y, z].  code='python' (pyspectrum.py:545-611): ``delta``
    is a full grid (N, N, N) [x, y, z], binned with the reference's numpy rules
    (float64 mu from folded components, ceil(mu/dmu) bins, no shot noise).
    A CUDA tensor is taken as already on the device in [z, y, x] order."""
    if code == 'python':
        if torch.is_tensor(delta):
            full = delta
        else:
            a = np.asarray(delta, dtype=np.complex64)
            if a.ndim != 3 or not (a.shape[0] == a.shape[1] == a.shape[2]):
                raise ValueError("code='python' bins a full (N, N, N) grid")
            full = torch.as_tensor(a).permute(2, 1, 0).contiguous().to(core._dev(device))
        return core.pk_rsd_python(full, rsd, Lbox, Nmubin)
    if code != 'fortran':
        raise ValueError("code must be 'fortran' or 'python'")
    half = _half_from_numpy(delta, device) if not torch.is_tensor(delta) else delta
    k, p0k, p2k, p4k, nk, k_kmu, mu_kmu, p_kmu, n_kmu = core.pk_pbox_rsd(half, rsd, Lbox, Nmubin)
    norm = (2. * np.pi) ** 3
    return k, p0k * norm, p2k * norm, p4k * norm, nk, k_kmu, mu_kmu, p_kmu * norm, n_kmu


def _pk_rsd_dict(half, N, Lbox, Ngrid, rsd, Nmubin, code):
    nbar = float(N) / Lbox ** 3        # pyspectrum.py:510 (particle count, not sum w)
    kf = 2 * np.pi / Lbox
    # code='python' bins the full grid (the reference hands it FFT_periodic's
    # half grid, which its numpy binning cannot index; the reflected grid is
    # what that code is written for)
    grid = core.reflect_half(half) if code == 'python' else half
    k, p0k, p2k, p4k, n_k, k_kmu, mu_kmu, p_kmu, n_kmu = _Pk_periodic_rsd(grid, Lbox=Lbox, rsd=rsd, Nmubin=Nmubin,
                                                                          code=code)
    return {'meta': {'Lbox': Lbox, 'Ngrid': Ngrid, 'N': N, 'nbar': nbar, 'kf': kf},
            'k': k, 'p0k': p0k - 1. / nbar, 'p2k': p2k, 'p4k': p4k, 'p_sn': np.repeat(1. / nbar, len(k)),
            'counts': n_k, 'k_kmu': k_kmu, 'mu_kmu': mu_kmu, 'p_kmu': p_kmu - 1. / nbar, 'counts_kmu': n_kmu}


def Pk_periodic_rsd(xyz, w=None, Lbox=2600, Ngrid=360, rsd=2, Nmubin=10, fft='pyfftw', code='fortran', silent=True,
                    device=None):
    """pyspectrum.py:460-538: multipoles P0/P2/P4 and P(k, mu)."""
    half, N, _ = _delta_half_device(xyz, w, Lbox, Ngrid, device=device)
    return _pk_rsd_dict(half, N, Lbox, Ngrid, rsd, Nmubin, code)


def Pk_periodic(xyz, w=None, Lbox=2600, Ngrid=360, fft='pyfftw', silent=True, device=None):
    """pyspectrum.py:644-728: monopole in k_f-wide bins.  Keys 'meta', 'k',
    'p0k', 'counts', 'p0k_sn'."""
    half, N, wsum = _delta_half_device(xyz, w, Lbox, Ngrid, device=device)
    nbar = wsum / Lbox ** 3
    kf = 2 * np.pi / Lbox
    k, p0k, counts = core.pk_monopole(half, Lbox)
    return {'meta': {'Lbox': Lbox, 'Ngrid': Ngrid, 'N': N, 'nbar': nbar, 'kf': kf},
            'k': k, 'p0k': p0k - 1. / nbar, 'counts': counts, 'p0k_sn': 1. / nbar}


def Bk_periodic_rsd(xyz, vxyz, redshift, h=0.7, omega0_m=0.3, LOS='z', w=None, Lbox=2600, Ngrid=360, step=3,
                    Ncut=3, Nmax=40, Nmubin=10, method='fp32', pk=True, silent=True, device=None):
    """Redshift-space B0/Q0: util.applyRSD (util.py:54-75) followed by
    Bk_periodic, computed from one delta(k).  With pk=True the result also
    holds 'pk', the Pk_periodic_rsd dictionary (P0, P2, P4, P(k, mu)) of the
    same redshift-space grid.  The reference has no function of this name."""
    los = {'x': 0, 'y': 1, 'z': 2}[LOS]
    half, N, wsum = _delta_half_device(xyz, w, Lbox, Ngrid, vel=vxyz, los=los,
                                       rsd_factor=core.rsd_factor(redshift, omega0_m), device=device)
    nbar = wsum / Lbox ** 3
    kf = 2 * np.pi / Lbox
    bispec = _bk_from_half(half, Ngrid, step, Ncut, Nmax, method, units=(nbar, kf), device=device)
    bispec['meta'] = {'Lbox': Lbox, 'Ngrid': Ngrid, 'step': step, 'Ncut': Ncut, 'Nmax': Nmax, 'N': N,
                      'nbar': nbar, 'kf': kf, 'redshift': redshift, 'h': h, 'omega0_m': omega0_m, 'LOS': LOS}
    bispec['p0k_sn'] = 1. / nbar
    if pk:
        bispec['pk'] = _pk_rsd_dict(half, N, Lbox, Ngrid, los, Nmubin, 'fortran')
    return bispec
