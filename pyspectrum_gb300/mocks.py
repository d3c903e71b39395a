"""Seeded synthetic periodic-box catalogues (Zel'dovich mocks).

A Gaussian random field with power-law spectrum P(k) ~ k^slope is drawn on an
N^3 grid (white noise from numpy's PCG64 with the given seed, coloured in
Fourier space with this package's own FFT kernels), turned into the
Zel'dovich displacement psi(k) = i k delta(k) / k^2, and applied to particles
placed on a uniform lattice with a random offset inside each lattice cell.
Optional velocities follow linear theory, v = f a H psi, plus an isotropic
Gaussian dispersion.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr
from .core import efunc


def _kvec(n, device):
    k = torch.fft.fftfreq(n, d=1.0 / n, device=device)     # integer wavenumbers
    return k


def displacement_field(ngrid, slope=-1.5, rms_disp=5.0, seed=1, device="cuda"):
    """Zel'dovich displacement psi (3, N, N, N) float32 [d][z][y][x] in Mpc/h with
    rms |psi| = rms_disp.  Uses pyspec_fft3d_c2c for both transforms."""
    n = int(ngrid)
    rng = np.random.default_rng(seed)
    white = torch.from_numpy(rng.standard_normal((n, n, n), dtype=np.float32)).to(device)
    g = torch.complex(white, torch.zeros_like(white)).contiguous()
    call("pyspec_fft3d_c2c", ptr(g), n, -1, stream_ptr())            # forward
    k = _kvec(n, device)
    kz, ky, kx = k.view(n, 1, 1), k.view(1, n, 1), k.view(1, 1, n)
    k2 = kx * kx + ky * ky + kz * kz
    k2[0, 0, 0] = 1.0
    amp = k2 ** (slope / 4.0)            # sqrt(P) ~ k^(slope/2)
    amp[0, 0, 0] = 0.0
    g *= amp
    psi = torch.empty((3, n, n, n), dtype=torch.float32, device=device)
    for d, kd in enumerate((kx, ky, kz)):
        comp = (g * (1j * kd / k2)).to(torch.complex64).contiguous()
        call("pyspec_fft3d_c2c", ptr(comp), n, 1, stream_ptr())      # backward
        psi[d] = comp.real
    rms = torch.sqrt((psi.double() ** 2).sum(0).mean())
    psi *= float(rms_disp / rms)
    return psi


def zeldovich_mock(npart, Lbox, ngrid=360, slope=-1.5, rms_disp=5.0, seed=1, velocities=False, redshift=0.5,
                   omega_m=0.3, sigma_v=300.0, device="cuda"):
    """Particles (3, npart) float64 on `device` (and velocities in km/s when
    requested).  The lattice has m = ceil(npart^(1/3)) cells per side; when
    m^3 > npart a seeded random subset of cells is used."""
    _lib.load()
    npart = int(npart)
    m = int(round(npart ** (1.0 / 3.0)))
    if m ** 3 < npart:
        m += 1
    rng = np.random.default_rng(seed + 1000)
    cells = np.arange(m ** 3) if m ** 3 == npart else np.sort(rng.choice(m ** 3, size=npart, replace=False))
    iz, rem = np.divmod(cells, m * m)
    iy, ix = np.divmod(rem, m)
    q = (np.stack([ix, iy, iz]).astype(np.float64) + rng.uniform(0.0, 1.0, size=(3, npart))) * (Lbox / m)
    q_d = torch.from_numpy(q).to(device)
    psi = displacement_field(ngrid, slope, rms_disp, seed, device)
    idx = torch.clamp((q_d / Lbox * ngrid).long(), 0, ngrid - 1)          # nearest grid point
    disp = psi[:, idx[2], idx[1], idx[0]].double()
    x = torch.remainder(q_d + disp, Lbox)
    if not velocities:
        return x
    a = 1.0 / (1.0 + redshift)
    E = efunc(redshift, omega_m)
    om_z = omega_m * (1.0 + redshift) ** 3 / E ** 2
    f = om_z ** 0.55
    H = 100.0 * E                                   # h km/s / (Mpc/h)
    gen = torch.Generator(device="cpu").manual_seed(seed + 2000)
    noise = torch.randn((3, npart), generator=gen, dtype=torch.float64).to(device) * sigma_v
    v = f * a * H * disp + noise
    return x, v


def uniform_mock(npart, Lbox, seed=0, device="cuda"):
    rng = np.random.default_rng(seed)
    return torch.from_numpy(rng.uniform(0.0, Lbox, size=(3, int(npart)))).to(device)


def mock_info(slope=-1.5, rms_disp=5.0):
    return {"field": f"GRF P(k)~k^{slope}", "displacement": "Zel'dovich, NGP-sampled",
            "rms_disp_mpc_h": rms_disp}
