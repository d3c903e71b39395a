"""CPU oracle for the periodic-box P(k)/B(k) path -- TEST INFRASTRUCTURE ONLY.

This module is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import it.  The product package
``pyspectrum_gb300`` never imports, links or calls anything under ``oracle/``.

It restates, in float64 numpy (plus the small C file ``assign_pcs.c`` for the
particle loop), the arithmetic of the reference pySpectrum estimator:

===========================  ==============================================
reference (file:line)        oracle function
===========================  ==============================================
pyspectrum.py:909-959        ``FFT_periodic``
estimator.f:284-512          ``assign_quad`` (C: ``assign_pcs.c``)
pyspectrum.py:1060-1080      ``fft_backward``
estimator.f:605-675          ``fcomb_periodic``
pyspectrum.py:1134-1157      ``reflect_delta``
pyspectrum.py:373-404        ``shell_index``, ``shell_fields``
pyspectrum.py:962-1030       ``counts_Bk123``
pyspectrum.py:359-457        ``_Bk_periodic``
pyspectrum.py:285-356        ``Bk_periodic``
pyspectrum.py:644-728        ``Pk_periodic``
estimator.f:155-264          ``pk_pbox_rsd``
pyspectrum.py:460-538        ``Pk_periodic_rsd``
util.py:54-75                ``applyRSD``
===========================  ==============================================

Parity status of this oracle
----------------------------
* Pinned: shell binning, mode counts and triangle counts against the
  reference's shipped count caches (``dat/counts.Ngrid360.Nmax{10,40,50}``);
  ``reflect_delta``, the shell/triangle stage (``_Bk_periodic``), the count
  computation (``_counts_Bk123``), ``_FFT`` and ``applyRSD`` against golden
  vectors produced by importing the reference's own Python functions
  (``tests/golden/make_golden.py``).
* Unpinned: the Fortran subroutines ``assign_quad``, ``fcomb_periodic`` and
  ``pk_pbox_rsd`` (no Fortran compiler and no FFTW exist here, so the
  reference's compiled layer cannot be run); they are restated line by line.

FFT convention: the reference calls FFTW 3.x single precision (version not
pinned by the reference; ``setup.py`` mentions 3.3.4 and 3.3.8).  FFTW's
published transforms are the plain DFTs; this oracle evaluates them in
float64 with pocketfft (``scipy.fft``, numpy's FFT on all host cores:
``ifftn * N**3`` for FFTW_BACKWARD unnormalised, ``fftn`` for FFTW_FORWARD).

Array convention: every grid is indexed ``[x, y, z]`` as in the reference's
numpy code; half grids are ``[0..N/2, y, z]``.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB = os.path.join(_BUILD, "liboracle_assign.so")
_lib = None


def build_c(force: bool = False) -> str:
    """Compile ``assign_pcs.c`` (IEEE single precision, no FMA contraction)."""
    src = os.path.join(_HERE, "assign_pcs.c")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        os.makedirs(_BUILD, exist_ok=True)
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math",
                               "-fPIC", "-shared", "-o", _LIB, src])
    return _LIB


def _c():
    global _lib
    if _lib is None:
        build_c()
        _lib = ctypes.CDLL(_LIB)
        _lib.oracle_assign_quad.restype = None
        _lib.oracle_assign_quad.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
            ctypes.c_float, ctypes.c_float, ctypes.c_void_p]
    return _lib


# --------------------------------------------------------------------------
# a1 / a2 / a3 / a4 : particles -> half-complex delta(k)
# --------------------------------------------------------------------------
def _sfft():
    """scipy.fft: numpy's pocketfft algorithm in double precision, on all
    host cores."""
    import scipy.fft
    return scipy.fft


def clip_positions(xyz, Lbox):
    """pyspectrum.py:938-941: clip to [0, L(1-1e-6)] in float64, store float32."""
    xyz = np.asarray(xyz)
    out = np.zeros((3, xyz.shape[1]), dtype=np.float32, order="F")
    for d in range(3):
        out[d, :] = np.clip(xyz[d, :], 0.0, Lbox * (1.0 - 1e-6))
    return out


def assign_quad(xyzs, w, kf_ks, offset, ngrid):
    """estimator.f:284-512 (density mode).  Returns a complex128 grid [x,y,z]:
    real part = PCS grid, imaginary part = half-cell interlaced PCS grid."""
    xyzs = np.asfortranarray(xyzs, dtype=np.float32)
    npart = xyzs.shape[1]
    wf = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
    grid = np.zeros((ngrid, ngrid, ngrid, 2), dtype=np.float64)  # [z][y][x][re/im]
    _c().oracle_assign_quad(xyzs.ctypes.data, None if wf is None else wf.ctypes.data,
                            npart, ngrid, float(np.float32(kf_ks)), float(np.float32(offset)),
                            grid.ctypes.data)
    g = grid[..., 0] + 1j * grid[..., 1]            # [z, y, x]
    return np.ascontiguousarray(g.transpose(2, 1, 0))  # [x, y, z]


def fft_backward(g):
    """pyspectrum.py:1072-1075: FFTW_BACKWARD, ``normalise_idft=False``."""
    n = g.shape[0]
    return _sfft().ifftn(g, workers=-1) * float(n) ** 3


def _fcomb_tables(n):
    lnyq = n // 2 + 1
    idx = np.arange(1, lnyq + 1)                 # Fortran 1-based ix
    ic = np.mod(n - idx + 1, n) + 1              # estimator.f:629,635,641
    rk = 2.0 * np.pi / n * (idx - 1)
    W = np.ones(lnyq)
    nz = rk != 0
    W[nz] = (np.sin(rk[nz] / 2) / (rk[nz] / 2)) ** 4   # estimator.f:632,638,644
    rec = np.exp(-1j * np.pi * (idx - 1) / n)    # recx**(ix-1), estimator.f:620-623,667
    return idx, ic, W, rec


def fcomb_periodic(G, wsum):
    """estimator.f:605-675, including its in-place write order.

    Each Fortran iteration (ix,iy,iz) in [1..N/2+1]^3 reads and writes the
    orbit {ix,icx} x {iy,icy} x {iz,icz}.  Orbits of different iterations are
    disjoint, but inside one orbit the eight writes (lines 658-665) alias when
    ix==icx, iy==icy or iz==icz; the last write wins.  This function replays
    those writes on eight slots per iteration.  Returns the half grid
    [0..N/2, :, :] (complex128)."""
    n = G.shape[0]
    lnyq = n // 2 + 1
    cf = 1.0 / (6.0 ** 3 * 4.0 * float(wsum))     # estimator.f:615
    idx, ic, W, rec = _fcomb_tables(n)
    out = np.zeros((lnyq, n, n), dtype=np.complex128)
    IX, IY = np.meshgrid(np.arange(lnyq), np.arange(lnyq), indexing="ij")
    IX = IX.ravel(); IY = IY.ravel()
    for kz in range(lnyq):
        ix = idx[IX]; iy = idx[IY]; iz = np.full_like(ix, idx[kz])
        icx = ic[IX]; icy = ic[IY]; icz = np.full_like(ix, ic[kz])
        cfac = cf / (W[IX] * W[IY] * W[kz])
        xr = rec[IX]; yr = rec[IY]; zr = rec[kz]
        cma = 1j * xr * yr * zr
        cmb = 1j * xr * yr * np.conj(zr)
        cmc = 1j * xr * np.conj(yr) * zr
        cmd = 1j * xr * np.conj(yr * zr)
        # slot positions (0-based): p0..p3 on column ix, p4..p7 on column icx
        P = [(ix, iy, iz), (ix, iy, icz), (ix, icy, iz), (ix, icy, icz),
             (icx, iy, iz), (icx, iy, icz), (icx, icy, iz), (icx, icy, icz)]
        P = [(a - 1, b - 1, c - 1) for a, b, c in P]
        val = [G[a, b, c].astype(np.complex128) for a, b, c in P]
        same = [[(P[a][0] == P[b][0]) & (P[a][1] == P[b][1]) & (P[a][2] == P[b][2])
                 for b in range(8)] for a in range(8)]

        def write(k, v):
            for k2 in range(8):
                val[k2] = np.where(same[k][k2], v, val[k2])

        c000 = val[0] * (1 - cma) + np.conj(val[7]) * (1 + cma)   # line 652
        c001 = val[1] * (1 - cmb) + np.conj(val[6]) * (1 + cmb)   # line 653
        c010 = val[2] * (1 - cmc) + np.conj(val[5]) * (1 + cmc)   # line 654
        c011 = val[3] * (1 - cmd) + np.conj(val[4]) * (1 + cmd)   # line 655
        write(0, c000 * cfac)                                     # line 658
        write(1, c001 * cfac)
        write(2, c010 * cfac)
        write(3, c011 * cfac)
        write(4, np.conj(val[3]))                                 # line 662
        write(5, np.conj(val[2]))
        write(6, np.conj(val[1]))
        write(7, np.conj(val[0]))                                 # line 665
        for k in range(8):
            a, b, c = P[k]
            m = a < lnyq
            out[a[m], b[m], c[m]] = val[k][m]
    return out


def FFT_periodic(xyz, w=None, Lbox=2600.0, Ngrid=360):
    """pyspectrum.py:909-959 -> half grid delta(k) [0..N/2, :, :]."""
    kf_ks = np.float32(float(Ngrid) / Lbox)
    npart = np.asarray(xyz).shape[1]
    if w is None:
        w = np.ones(npart)
    xyzs = clip_positions(xyz, Lbox)
    g = assign_quad(xyzs, np.asarray(w, dtype=np.float32), kf_ks, 0.0, Ngrid)
    G = fft_backward(g)
    return fcomb_periodic(G, float(np.sum(w)))


def reflect_delta(delt, Ngrid=None):
    """pyspectrum.py:1134-1157 (float64/complex128 version)."""
    n = delt.shape[1] if Ngrid is None else Ngrid
    delta = np.zeros((n, n, n), dtype=np.complex128)
    delta[: n // 2 + 1] = delt
    delta[: n // 2: -1, n:0:-1, n:0:-1] = np.conj(delt[1: n // 2, 1:n, 1:n])
    delta[: n // 2: -1, n:0:-1, 0] = np.conj(delt[1: n // 2, 1:n, 0])
    delta[: n // 2: -1, 0, n:0:-1] = np.conj(delt[1: n // 2, 0, 1:n])
    delta[: n // 2: -1, 0, 0] = np.conj(delt[1: n // 2, 0, 0])
    hg = n // 2
    for c in [(hg, 0, 0), (0, hg, 0), (0, 0, hg), (0, hg, hg), (hg, 0, hg), (hg, hg, 0), (hg, hg, hg)]:
        delta[c] = np.real(delt[c])
    return delta


# --------------------------------------------------------------------------
# a6 / a7 / a8 / a9 / a10 : shells, counts, triangles, units
# --------------------------------------------------------------------------
def _absfreq(n):
    i = np.arange(n)
    return np.minimum(i, n - i)


def shell_index(n, step):
    """pyspectrum.py:373-378: irk = int(|k|/step + 0.5), |k| in units of k_f."""
    a = _absfreq(n).astype(np.float64)
    rk = np.sqrt(a[:, None, None] ** 2 + a[None, :, None] ** 2 + a[None, None, :] ** 2)
    return (rk / step + 0.5).astype(np.int64)


def shell_index_int(d2, step):
    """Integer form of the binning: the largest n with (2n-1)^2 step^2 <= 4 d2.
    Equal to ``int(sqrt(d2)/step + 0.5)`` for every integer d2 (the boundary
    case is exact in float64 and otherwise never within rounding of it)."""
    d2 = np.asarray(d2, dtype=np.int64)
    nn = np.floor(np.sqrt(d2.astype(np.float64)) / step + 0.5).astype(np.int64)
    nn = np.where((nn > 0) & ((2 * nn - 1) ** 2 * step * step > 4 * d2), nn - 1, nn)
    nn = np.where((2 * nn + 1) ** 2 * step * step <= 4 * d2, nn + 1, nn)
    return nn


def mode_counts(n, step, nmax):
    """pyspectrum.py:380: Nk[j] = #{k : irk(k) == j}, j = 0..Nmax."""
    irk = shell_index(n, step)
    return np.array([np.sum(irk == j) for j in range(nmax + 1)], dtype=np.int64)


def triangles(jmin, nmax):
    """pyspectrum.py:415-422: the (i, j, l) loop and its symmetry factor."""
    out = []
    for i in range(jmin, nmax + 1):
        for j in range(jmin, i + 1):
            for l in range(max(i - j, jmin), j + 1):
                fac = 1.0
                if j == l and i == j:
                    fac = 6.0
                if i == j and j != l:
                    fac = 2.0
                if i == l and l != j:
                    fac = 2.0
                if j == l and l != i:
                    fac = 2.0
                out.append((i, j, l, fac))
    return out


def shell_fields(delta_full, step, jmin, nmax):
    """pyspectrum.py:384-404: F_j = Re(fftn(delta * [irk==j])) in float64,
    p0k[j-1] = sum F_j^2 / N^3 / Nk[j].  Returns (F[j], p0k, Nk)."""
    n = delta_full.shape[0]
    irk = shell_index(n, step)
    nk = np.array([np.sum(irk == j) for j in range(nmax + 1)], dtype=np.int64)
    F = {}
    p0k = np.zeros(nmax)
    for j in range(jmin, nmax + 1):
        tmp = np.where(irk == j, delta_full, 0)
        F[j] = np.real(_sfft().fftn(tmp, workers=-1))
        with np.errstate(invalid="ignore", divide="ignore"):
            p0k[j - 1] = np.sum(F[j] ** 2) / float(n) ** 3 / nk[j]
    return F, p0k, nk


def counts_Bk123(Ngrid, Nmax, Ncut, step):
    """pyspectrum.py:976-1023 compute path: counts[i-1,j-1,l-1] =
    sum_x I_i I_j I_l with I_j = FFT(shell indicator), float64.
    Returns (counts (Nmax,Nmax,Nmax) float64, exact integer counts/N^3)."""
    n = Ngrid
    jmin = Ncut // step
    irk = shell_index(n, step)
    I = {}
    for j in range(jmin, Nmax + 1):
        I[j] = np.real(_sfft().fftn((irk == j).astype(np.complex128), workers=-1))
    counts = np.zeros((Nmax, Nmax, Nmax))
    for i, j, l, _ in triangles(jmin, Nmax):
        counts[i - 1, j - 1, l - 1] = np.einsum("i,i,i", I[i].ravel(), I[j].ravel(), I[l].ravel())
    exact = np.rint(counts / float(n) ** 3).astype(np.int64)
    return counts, exact


def _Bk_periodic(delta_full, Nmax=40, Ncut=3, step=3, counts=None):
    """pyspectrum.py:359-457.  ``counts`` is the (Nmax,Nmax,Nmax) array of
    sum_x I_i I_j I_l (the reference's cache content); computed if None.

    Output arrays hold the triangles with counts > 0 (the reference appends
    zeros to its value arrays but not to its index arrays for zero-count
    triangles, pyspectrum.py:438-445; here all arrays stay aligned)."""
    n = delta_full.shape[0]
    jmin = Ncut // step
    F, p0k, nk = shell_fields(delta_full, step, jmin, Nmax)
    if counts is None:
        counts, _ = counts_Bk123(n, Nmax, Ncut, step)
    res = {k: [] for k in ("i_k1", "i_k2", "i_k3", "p0k1", "p0k2", "p0k3", "b123", "q123", "counts")}
    for i, j, l, fac in triangles(jmin, Nmax):
        c = counts[i - 1, j - 1, l - 1]
        if c > 0:
            b = np.einsum("i,i,i", F[i].ravel(), F[j].ravel(), F[l].ravel())
            res["i_k1"].append(i); res["i_k2"].append(j); res["i_k3"].append(l)
            res["p0k1"].append(p0k[i - 1]); res["p0k2"].append(p0k[j - 1]); res["p0k3"].append(p0k[l - 1])
            res["b123"].append(b / c)
            res["q123"].append(b / c / (p0k[i - 1] * p0k[j - 1] + p0k[j - 1] * p0k[l - 1] + p0k[l - 1] * p0k[i - 1]))
            res["counts"].append(c / (fac * float(n) ** 3))
    out = {k: np.array(v) for k, v in res.items()}
    for k in ("i_k1", "i_k2", "i_k3"):
        out[k] = out[k].astype(np.int64) * step
    out["raw_bsum"] = out["b123"] * np.array([counts[i - 1, j - 1, l - 1] for i, j, l in
                                               zip(out["i_k1"] // step, out["i_k2"] // step, out["i_k3"] // step)])
    return out


def _B0_survey(delta_full, alpha, I12, I13, I22, I23, I33, Nmax=40, Ncut=3, step=3, counts=None):
    """pyspectrum.py:137-282 (survey FKP bispectrum) in float64, triangles with
    counts > 0 only (all arrays aligned)."""
    n = delta_full.shape[0]
    jmin = Ncut // step
    F, p0k, nk = shell_fields(delta_full, step, jmin, Nmax)
    p0k = p0k / I22 - (1.0 + alpha) * I12 / I22
    if counts is None:
        counts, _ = counts_Bk123(n, Nmax, Ncut, step)
    res = {k: [] for k in ("i_k1", "i_k2", "i_k3", "p0k1", "p0k2", "p0k3", "b123", "q123", "counts")}
    for i, j, l, fac in triangles(jmin, Nmax):
        c = counts[i - 1, j - 1, l - 1]
        if c > 0:
            b = np.einsum("i,i,i", F[i].ravel(), F[j].ravel(), F[l].ravel()) / c
            b -= (p0k[i - 1] + p0k[j - 1] + p0k[l - 1]) * I23 + (1.0 - alpha ** 2) * I13
            b /= I33
            res["i_k1"].append(i * step); res["i_k2"].append(j * step); res["i_k3"].append(l * step)
            res["p0k1"].append(p0k[i - 1]); res["p0k2"].append(p0k[j - 1]); res["p0k3"].append(p0k[l - 1])
            res["b123"].append(b)
            res["q123"].append(b / (p0k[i - 1] * p0k[j - 1] + p0k[j - 1] * p0k[l - 1] + p0k[l - 1] * p0k[i - 1]))
            res["counts"].append(c / (fac * float(n) ** 3))
    return {k: np.array(v) for k, v in res.items()}


def FFT_survey_mono(xyz, nb, w=None, P0_fkp=1e6, Lbox=2600.0, Ngrid=360):
    """pyspectrum.py:773-826 from Cartesian positions (centred on the origin):
    FKP weights, normalisation integrals, assignment with the N/2-cell offset,
    backward FFT and fcomb_survey (fcomb_periodic with N = 1, estimator.f:686).
    Returns (half grid, Ntot, I12, I13, I22, I23, I33)."""
    npart = xyz.shape[1]
    w = np.ones(npart) if w is None else np.array(w, dtype=np.float64)
    Ntot = np.sum(w)
    w = w * (1.0 / (1.0 + nb * P0_fkp))
    I12, I13 = np.sum(w ** 2), np.sum(w ** 3)
    I22, I23, I33 = np.sum(nb * w ** 2), np.sum(nb * w ** 3), np.sum(nb ** 2 * w ** 3)
    xyzs = np.asarray(xyz, dtype=np.float32)
    g = assign_quad(xyzs, w.astype(np.float32), np.float32(float(Ngrid) / Lbox), 0.5 * Ngrid, Ngrid)
    G = fft_backward(g)
    return fcomb_periodic(G, 1.0), Ntot, I12, I13, I22, I23, I33


def Bk_periodic(xyz, w=None, Lbox=2600.0, Ngrid=360, step=3, Ncut=3, Nmax=40, counts=None):
    """pyspectrum.py:285-356 (the ``Ngrid == 360`` assertion at :332 is not kept)."""
    npart = np.asarray(xyz).shape[1]
    if w is None:
        w = np.ones(npart)
    nbar = np.sum(w) / Lbox ** 3
    kf = 2 * np.pi / Lbox
    delta = FFT_periodic(xyz, w=w, Lbox=Lbox, Ngrid=Ngrid)
    bispec = _Bk_periodic(reflect_delta(delta, Ngrid), Nmax=Nmax, Ncut=Ncut, step=step, counts=counts)
    return bk_postprocess(bispec, Lbox, Ngrid, step, Ncut, Nmax, npart, nbar, kf)


def bk_postprocess(bispec, Lbox, Ngrid, step, Ncut, Nmax, npart, nbar, kf):
    """pyspectrum.py:341-355: units and shot noise."""
    bispec = dict(bispec)
    bispec["meta"] = {"Lbox": Lbox, "Ngrid": Ngrid, "step": step, "Ncut": Ncut, "Nmax": Nmax,
                      "N": npart, "nbar": nbar, "kf": kf}
    for key in ("p0k1", "p0k2", "p0k3"):
        bispec[key] = bispec[key] * (2 * np.pi) ** 3 / kf ** 3 - 1.0 / nbar
    bispec["p0k_sn"] = 1.0 / nbar
    bsn = (bispec["p0k1"] + bispec["p0k2"] + bispec["p0k3"]) / nbar + 1.0 / nbar ** 2
    bispec["b123"] = bispec["b123"] * (2 * np.pi) ** 6 / kf ** 6 - bsn
    bispec["b123_sn"] = bsn
    bispec["q123"] = bispec["b123"] / (bispec["p0k1"] * bispec["p0k2"] + bispec["p0k1"] * bispec["p0k3"]
                                       + bispec["p0k2"] * bispec["p0k3"])
    return bispec


# --------------------------------------------------------------------------
# a11 / a12 / a13 : power spectrum and RSD
# --------------------------------------------------------------------------
def Pk_periodic(xyz, w=None, Lbox=2600.0, Ngrid=360, delta_half=None):
    """pyspectrum.py:644-728 with the binning sum over the reflected grid
    ``delta_fft`` (the reference indexes the half grid ``delta`` with a
    full-grid mask at :713, which raises IndexError; the full grid is the
    evident intent)."""
    npart = np.asarray(xyz).shape[1] if xyz is not None else 0
    if w is None:
        w = np.ones(npart)
    nbar = np.sum(w) / Lbox ** 3
    kf = 2 * np.pi / Lbox
    if delta_half is None:
        delta_half = FFT_periodic(xyz, w=w, Lbox=Lbox, Ngrid=Ngrid)
    out = pk_monopole(reflect_delta(delta_half, Ngrid), Lbox)
    out["meta"] = {"Lbox": Lbox, "Ngrid": Ngrid, "N": npart, "nbar": nbar, "kf": kf}
    out["p0k"] = out["p0k"] - 1.0 / nbar
    out["p0k_sn"] = 1.0 / nbar
    return out


def pk_monopole(delta_fft, Lbox):
    """pyspectrum.py:691-716 on the full grid: returns k, p0k (x (2pi)^3), counts."""
    n = delta_fft.shape[0]
    nbins = n // 2
    kf = 2 * np.pi / float(Lbox)
    a = _absfreq(n)
    d2 = a[:, None, None] ** 2 + a[None, :, None] ** 2 + a[None, None, :] ** 2
    irk = shell_index_int(d2, 1)
    rk = kf * np.sqrt(d2.astype(np.float64))
    p = np.abs(delta_fft) ** 2
    k = np.zeros(nbins); p0k = np.zeros(nbins); cnt = np.zeros(nbins)
    irk = irk.ravel(); rk = rk.ravel(); p = p.ravel()
    sel = (irk >= 1) & (irk <= nbins)
    nk = np.bincount(irk[sel] - 1, minlength=nbins)[:nbins]
    ks = np.bincount(irk[sel] - 1, weights=rk[sel], minlength=nbins)[:nbins]
    ps = np.bincount(irk[sel] - 1, weights=p[sel], minlength=nbins)[:nbins]
    m = nk > 0
    k[m] = ks[m] / nk[m]
    p0k[m] = ps[m] / nk[m] / kf ** 3
    cnt[m] = nk[m]
    return {"k": k, "p0k": p0k * (2.0 * np.pi) ** 3, "counts": cnt}


def _f32(x):
    return np.float32(x)


def rsd_observer_constants(irsd):
    """estimator.f:164,171-181 evaluated in single precision:
    returns (cos(thetaobs), sin(thetaobs), cos(phiobs), sin(phiobs)) as float32."""
    pi = np.float32(3.141592654)
    half_pi = np.float32(np.float32(0.5) * pi)
    theta, phi = {0: (half_pi, np.float32(0)), 1: (half_pi, half_pi), 2: (np.float32(0), np.float32(0))}[irsd]
    c = lambda v: np.float32(math.cos(float(v)))
    s = lambda v: np.float32(math.sin(float(v)))
    return c(theta), s(theta), c(phi), s(phi)


def pk_pbox_rsd(delt, irsd, Lbox, Nbin, Nmu, Ngrid):
    """estimator.f:155-264.  ``delt`` is the half grid [0..N/2, :, :].
    Mode selection and mu-bin assignment follow the Fortran's single-precision
    arithmetic; sums are float64.  Returns the 9 output arrays before the
    (2 pi)^3 factor applied by the Python wrapper (pyspectrum.py:636-640)."""
    n = Ngrid
    f = lambda i: (np.mod(i + n // 2 - 2, n) - n // 2 + 1)       # estimator.f:198 (1-based i)
    fr = f(np.arange(1, n + 1)).astype(np.int64)                 # signed frequency per index
    ix = np.arange(n)
    kx = fr[:, None, None]; ky = fr[None, :, None]; kz = fr[None, None, :]
    d2 = kx * kx + ky * ky + kz * kz
    imk = shell_index_int(d2, 1)            # nint(Nbin*rk/real(N/2)) with Nbin = N/2
    assert Nbin == n // 2, "the periodic wrapper always passes Nbin = Ngrid//2"
    sel = (imk <= Nbin) & (imk != 0)
    rk = np.sqrt(d2.astype(np.float32))                          # real rk (single)
    with np.errstate(invalid="ignore", divide="ignore"):
        cot1 = (kz.astype(np.float32) / rk).astype(np.float32)
        sit1 = np.sqrt((np.float32(1) - cot1 * cot1).astype(np.float32)).astype(np.float32)
        ct, st, cph, sph = rsd_observer_constants(irsd)
        rs = (rk * sit1).astype(np.float32)
        cp = (kx.astype(np.float32) / rs).astype(np.float32)
        sp = (ky.astype(np.float32) / rs).astype(np.float32)
        cc = ((sph * sp).astype(np.float32) + (cph * cp).astype(np.float32)).astype(np.float32)
        cc = np.where(sit1 > 0, cc, np.float32(0))
        mu = ((ct * cot1).astype(np.float32) + ((st * sit1).astype(np.float32) * cc).astype(np.float32)).astype(np.float32)
    mu = np.broadcast_to(mu, d2.shape).astype(np.float64)
    mubin = np.float32(1.0) / np.float32(Nmu)
    imu = np.floor((np.abs(mu) + np.float64(mubin)) / np.float64(mubin)).astype(np.int64)
    le2 = -0.5 + 1.5 * mu ** 2
    le4 = 0.375 - 3.75 * mu ** 2 + 4.375 * mu ** 4
    # |delta|^2 with the conjugate lookup of estimator.f:226-230
    full = np.empty((n, n, n), dtype=np.complex128)
    h = n // 2 + 1
    full[:h] = delt
    icx = (np.mod(n + 1 - (ix + 1), n) + 1) - 1
    icx_hi = icx[h:]
    full[h:] = np.conj(delt[icx_hi][:, (np.mod(n - ix, n))][:, :, (np.mod(n - ix, n))])
    pk = np.abs(full) ** 2
    kf = np.float32(np.float32(2.0 * np.float32(3.141592654)) / np.float32(int(Lbox)))
    kval = (kf * rk).astype(np.float64)
    kval = np.broadcast_to(kval, d2.shape)
    I = imk[sel] - 1
    def bsum(wts):
        return np.bincount(I, weights=wts, minlength=Nbin)[:Nbin]
    nk = bsum(np.ones(I.shape))
    k = bsum(kval[sel]); p0 = bsum(pk[sel]); p2 = bsum(pk[sel] * 5.0 * le2[sel]); p4 = bsum(pk[sel] * 9.0 * le4[sel])
    selm = sel & (imu <= Nmu) & (imu > 0)
    J = (imk[selm] - 1) * Nmu + (imu[selm] - 1)
    def bsum2(wts):
        return np.bincount(J, weights=wts, minlength=Nbin * Nmu)[: Nbin * Nmu].reshape(Nbin, Nmu)
    nkm = bsum2(np.ones(J.shape)); km = bsum2(kval[selm]); mk = bsum2(np.abs(mu[selm])); pkm = bsum2(pk[selm])
    kf3 = float(kf) ** 3
    m = nk > 0
    k[m] /= nk[m]; p0[m] = p0[m] / nk[m] / kf3; p2[m] = p2[m] / nk[m] / kf3; p4[m] = p4[m] / nk[m] / kf3
    mm = nkm > 0
    km[mm] /= nkm[mm]; mk[mm] /= nkm[mm]; pkm[mm] = pkm[mm] / nkm[mm] / kf3
    return k, p0, p2, p4, nk, km, mk, pkm, nkm


def pk_rsd_python(delta, Lbox=None, rsd=2, Nmubin=5):
    """pyspectrum.py:545-611 (_Pk_periodic_rsd with code='python') on a full
    grid delta [x, y, z]: |k| bins irk = int(Nbins |k| / k_Nyq + 0.5) and
    mu from the folded components |k_x|, |k_y|, |k_z| in float64 (so mu >= 0),
    mu bins imu = ceil(mu / dmu); modes with imu = 0 count in Nk but add to
    neither the (k, mu) table nor P2, P4 (the reference sums those inside its
    mu-bin loop).  |delta| is the float32 modulus squared in float32, as
    np.absolute on complex64.  Returns the 9 arrays after the (2 pi)^3 factor."""
    n = delta.shape[0]
    nb = n // 2
    dmu = 1.0 / float(Nmubin)
    kf = 1.0 if Lbox is None else 2 * np.pi / float(Lbox)
    nyq = kf * float(n) / 2.0
    a = np.minimum(np.arange(n), n - np.arange(n))
    d2 = a[:, None, None] ** 2 + a[None, :, None] ** 2 + a[None, None, :] ** 2
    rk = kf * np.sqrt(d2.astype(np.float64))
    irk = (nb * rk / nyq + 0.5).astype(np.int64)
    th = [0.5 * np.pi, 0.5 * np.pi, 0.0][rsd]
    ph = [0.0, 0.5 * np.pi, 0.0][rsd]
    rkx = kf * a[:, None, None]
    rky = kf * a[None, :, None]
    rkz = kf * a[None, None, :]
    with np.errstate(invalid="ignore", divide="ignore"):
        cos_t = rkz / rk
        sin_t = np.sqrt(1.0 - cos_t ** 2)
        cos_p = rkx / (rk * sin_t)
        sin_p = rky / (rk * sin_t)
        cc = np.where(sin_t > 0, np.sin(ph) * sin_p + np.cos(ph) * cos_p, 0.0)
        mu = np.cos(th) * cos_t + np.sin(th) * sin_t * cc
        imu = np.where(d2 == 0, -999, np.ceil(mu / dmu)).astype(np.int64)
    leg2 = -0.5 + 1.5 * mu ** 2
    leg4 = 0.375 - 3.75 * mu ** 2 + 4.375 * mu ** 4
    p = (np.absolute(delta.astype(np.complex64)) ** 2).astype(np.float32).astype(np.float64)
    sel = (irk >= 1) & (irk <= nb)
    I = irk[sel] - 1
    bs = lambda w: np.bincount(I, weights=w, minlength=nb)[:nb]
    nk = bs(np.ones(I.shape))
    ks = bs(rk[sel]); p0 = bs(p[sel])
    selm = sel & (imu >= 1) & (imu <= Nmubin)
    J = (irk[selm] - 1) * Nmubin + imu[selm] - 1
    bm = lambda w: np.bincount(J, weights=w, minlength=nb * Nmubin)[: nb * Nmubin].reshape(nb, Nmubin)
    nkm = bm(np.ones(J.shape)); km = bm(rk[selm]); mm = bm(mu[selm]); pkm = bm(p[selm])
    Ik = irk[selm] - 1
    p2 = np.bincount(Ik, weights=p[selm] * leg2[selm], minlength=nb)[:nb]
    p4 = np.bincount(Ik, weights=p[selm] * leg4[selm], minlength=nb)[:nb]
    kf3 = kf ** 3
    norm = (2.0 * np.pi) ** 3
    m = nk > 0
    ks[m] /= nk[m]; p0[m] = p0[m] / nk[m] / kf3
    p2[m] = p2[m] / nk[m] / kf3 * 5.0; p4[m] = p4[m] / nk[m] / kf3 * 9.0
    p2[~m] = 0; p4[~m] = 0
    q = nkm > 0
    km[q] /= nkm[q]; mm[q] /= nkm[q]; pkm[q] = pkm[q] / nkm[q] / kf3
    return ks, p0 * norm, p2 * norm, p4 * norm, nk, km, mm, pkm * norm, nkm


def Pk_periodic_rsd(xyz, w=None, Lbox=2600, Ngrid=360, rsd=2, Nmubin=10, delta_half=None):
    """pyspectrum.py:460-538 with code='fortran' (pyspectrum.py:628-641)."""
    npart = np.asarray(xyz).shape[1] if xyz is not None else 0
    nbar = float(npart) / Lbox ** 3
    kf = 2 * np.pi / Lbox
    if delta_half is None:
        delta_half = FFT_periodic(xyz, w=w, Lbox=Lbox, Ngrid=Ngrid)
    k, p0k, p2k, p4k, nk, kkmu, mukmu, pkmu, nkmu = pk_pbox_rsd(delta_half, rsd, Lbox, Ngrid // 2, Nmubin, Ngrid)
    norm = (2.0 * np.pi) ** 3
    return {"meta": {"Lbox": Lbox, "Ngrid": Ngrid, "N": npart, "nbar": nbar, "kf": kf},
            "k": k, "p0k": p0k * norm - 1.0 / nbar, "p2k": p2k * norm, "p4k": p4k * norm,
            "p_sn": np.repeat(1.0 / nbar, len(k)), "counts": nk, "k_kmu": kkmu, "mu_kmu": mukmu,
            "p_kmu": pkmu * norm - 1.0 / nbar, "counts_kmu": nkmu}


def efunc(z, omega0_m):
    """E(z) of a flat LambdaCDM model without radiation (astropy's FlatLambdaCDM
    with its default Tcmb0=0, as used at util.py:67)."""
    return math.sqrt(omega0_m * (1.0 + z) ** 3 + (1.0 - omega0_m))


def applyRSD(xyz, vxyz, redshift, h=0.7, omega0_m=0.3, LOS=None, Lbox=None):
    """util.py:54-75."""
    assert xyz.shape[0] == 3 and vxyz.shape[0] == 3
    if LOS is None:
        raise ValueError("specify line of sight")
    if Lbox is None:
        raise ValueError("specify box size")
    i_los = {"x": 0, "y": 1, "z": 2}[LOS]
    rsd_factor = (1 + redshift) / (100 * efunc(redshift, omega0_m))
    out = np.array(xyz, dtype=np.float64, copy=True)
    out[i_los] += rsd_factor * vxyz[i_los] + Lbox
    out[i_los] = out[i_los] % Lbox
    return out
