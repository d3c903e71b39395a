"""Survey-geometry (FKP) bispectrum monopole: pyspectrum.py:13-282 (B0_survey,
_B0_survey) and :731-826 (FFT_survey_mono), estimator.f:677-745 (fcomb_survey).

The same device kernels as the periodic box: positions cast to float32
without clipping, PCS + interlaced assignment with the N/2-cell offset that
centres the survey in the box, the backward 3D FFT, the interlacing combine
without the weight-sum normalisation, the shell fields and the triangle
contraction.  The FKP weights and the normalisation integrals I12..I33 are
per-object sums evaluated on the host in float64, as the reference does; the
normalisation of the T triangle sums is a few vector operations.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib, core, tune
from ._lib import call, ptr, stream_ptr
from .util import FlatLambdaCDM, radecz_to_cartesian

__all__ = ["FFT_survey_mono", "_B0_survey", "B0_survey"]


def _fft_survey_half(radecz, nb, w=None, P0_fkp=1e6, Lbox=2600.0, Ngrid=360, cosmo=None, device=None):
    """pyspectrum.py:773-826 on the device.  Returns (half grid [z, y, x]
    complex64, Ntot, I12, I13, I22, I23, I33)."""
    dev = core._dev(device)
    n = int(Ngrid)
    if n < 4 or n % 2:
        raise ValueError("Ngrid must be even and >= 4")
    if cosmo is None:
        cosmo = FlatLambdaCDM(H0=67.6, Om0=0.31)
    radecz = np.asarray(radecz, dtype=np.float64)
    N = radecz.shape[1]
    if N == 0:
        raise ValueError("empty catalogue")
    w = np.ones(N) if w is None else np.array(w, dtype=np.float64, copy=True)
    nb = np.asarray(nb, dtype=np.float64)
    xyz = radecz_to_cartesian(radecz, cosmo=cosmo)
    xyz_max, xyz_min = np.max(xyz, axis=1), np.min(xyz, axis=1)
    if np.sum(xyz_max >= 0.5 * Lbox) + np.sum(np.abs(xyz_min) >= 0.5 * Lbox) != 0:
        raise AssertionError("box not big enough!")
    Ntot = np.sum(w)                                   # total weight without FKP
    w = w * (1.0 / (1.0 + nb * P0_fkp))                # FKP weights
    I12, I13 = np.sum(w ** 2), np.sum(w ** 3)
    I22, I23, I33 = np.sum(nb * w ** 2), np.sum(nb * w ** 3), np.sum(nb ** 2 * w ** 3)
    if not all(v >= 0 for v in (I12, I13, I22, I23, I33)):
        raise AssertionError("negative normalisation integral")
    x_d = torch.as_tensor(xyz, dtype=torch.float64).to(dev).contiguous()
    w_d = torch.as_tensor(w, dtype=torch.float64).to(dev).contiguous()
    xyzs = torch.empty((3, N), dtype=torch.float32, device=dev)
    ws = torch.empty((N,), dtype=torch.float32, device=dev)
    call("pyspec_cast_positions", ptr(x_d), x_d.stride(0), ptr(w_d), N, ptr(xyzs), ptr(ws), stream_ptr())
    grid = torch.zeros((n, n, n), dtype=torch.complex64, device=dev)
    kf_ks = float(np.float32(float(n) / Lbox))        # pyspectrum.py:773
    tune.assign(xyzs, ws, n, kf_ks, 0.5 * n, grid)      # offset N/2 cells (pyspectrum.py:775)
    tune.fft3d(grid, n, 1)
    half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=dev)
    call("pyspec_fcomb_survey", ptr(grid), n, ptr(half), stream_ptr())
    return half, Ntot, I12, I13, I22, I23, I33


def FFT_survey_mono(radecz, nb, w=None, P0_fkp=1e6, Lbox=2600., Ngrid=360, cosmo=None, fft='pyfftw', silent=True,
                    device=None):
    """pyspectrum.py:731-826: FKP-weighted delta_0(k) of a survey catalogue on
    the half grid (N//2+1, N, N) [x, y, z], with Ntot and I12, I13, I22, I23,
    I33.  ``fft`` is accepted and ignored; ``w`` is not modified."""
    half, Ntot, I12, I13, I22, I23, I33 = _fft_survey_half(radecz, nb, w, P0_fkp, Lbox, Ngrid, cosmo, device)
    return half.cpu().numpy().transpose(2, 1, 0), Ntot, I12, I13, I22, I23, I33


def _b0_from_half(half, alpha, I12, I13, I22, I23, I33, Nmax, Ncut, step, method, device):
    n = half.shape[0]
    plan = core.get_plan(n, step, Ncut, Nmax, method, device)
    plan.shells(half)
    plan.contract()
    bsum = plan.bsum.cpu().numpy()
    if plan.method in core.TENSOR_METHODS:
        core.check_contract_status(plan.status_word().item())
    p0sum = plan.p0sum.cpu().numpy()
    V = float(n) ** 3
    jmin = plan.jmin
    # pyspectrum.py:231-236: p0k[j-1] = sum F_j^2 / N^3 / Nk[j], then FKP shot noise
    p0k = np.zeros(Nmax)
    with np.errstate(invalid="ignore", divide="ignore"):
        p0k[jmin - 1:Nmax] = p0sum / V / plan.nk_np[jmin:Nmax + 1]
    p0k /= I22
    p0k -= (1.0 + alpha) * I12 / I22
    keep = plan.counts_np > 0
    tri = plan.tri_np[:, keep]
    i, j, l = tri
    cnt = plan.counts_np[keep].astype(np.float64) * V
    pi, pj, pl = p0k[i - 1], p0k[j - 1], p0k[l - 1]
    # pyspectrum.py:252-262
    b = bsum[keep] / cnt
    b -= (pi + pj + pl) * I23 + (1.0 - alpha ** 2) * I13
    b /= I33
    fac = np.where((i == j) & (j == l), 6.0, np.where((i == j) | (i == l) | (j == l), 2.0, 1.0))
    return {"i_k1": i.astype(np.int64) * step, "i_k2": j.astype(np.int64) * step, "i_k3": l.astype(np.int64) * step,
            "p0k1": pi, "p0k2": pj, "p0k3": pl, "b123": b, "q123": b / (pi * pj + pj * pl + pl * pi),
            "counts": cnt / (fac * V)}


def _B0_survey(delta, alpha, I12, I13, I22, I23, I33, Nmax=40, Ncut=3, step=3, fft='pyfftw', nthreads=1,
               silent=True, method='fp32', device=None):
    """pyspectrum.py:137-282 on a full FKP field delta(k) (N, N, N) [x, y, z]
    (data minus alpha times randoms).  Only triangles with counts > 0 are
    returned, all arrays aligned (see pyspectrum.Bk_periodic)."""
    dev = core._dev(device)
    full = torch.as_tensor(np.asarray(delta, dtype=np.complex64)).permute(2, 1, 0).contiguous().to(dev)
    half = core.half_from_full(full)
    del full
    return _b0_from_half(half, alpha, I12, I13, I22, I23, I33, Nmax, Ncut, step, method, dev)


def B0_survey(radecz, nbar, w=None, radecz_r=None, nbar_r=None, w_r=None, P0_fkp=1e6, Lbox=2600, Ngrid=360, step=3,
              Ncut=3, Nmax=40, cosmo=None, fft='pyfftw', nthreads=1, silent=True, method='fp32', device=None):
    """pyspectrum.py:13-134: bispectrum monopole of a survey (Scoccimarro 2015
    FKP estimator) from (RA, Dec, z) of data and randoms.  The reference's
    ``Ngrid == 360`` assertion (:85) is not kept."""
    if radecz_r is None:
        raise ValueError("a random catalogue (radecz_r, nbar_r) is required")
    if nbar_r is None:
        raise ValueError("specify nbar for random catalog")
    dev = core._dev(device)
    kf = 2 * np.pi / Lbox
    N = np.asarray(radecz).shape[1]
    half_d, Ngtot, *Id = _fft_survey_half(radecz, nbar, w, P0_fkp, Lbox, Ngrid, cosmo, dev)
    half_r, Nrtot, *Ir = _fft_survey_half(radecz_r, nbar_r, w_r, P0_fkp, Lbox, Ngrid, cosmo, dev)
    alpha = Ngtot / Nrtot
    I12, I13, I22, I23, I33 = (alpha * v for v in Ir)
    call("pyspec_combine_fields", ptr(half_d), ptr(half_r), float(alpha), half_d.numel(), ptr(half_d), stream_ptr())
    del half_r
    bispec = _b0_from_half(half_d, alpha, I12, I13, I22, I23, I33, Nmax, Ncut, step, method, dev)
    bispec["meta"] = {"Lbox": Lbox, "Ngrid": Ngrid, "step": step, "Ncut": Ncut, "Nmax": Nmax, "N": N,
                      "nbar": nbar, "kf": kf}
    return bispec
