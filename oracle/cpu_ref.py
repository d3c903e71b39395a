"""All-core CPU restatement of the reference's Bk_periodic -- TEST
INFRASTRUCTURE and the timed CPU baseline only.

Only ``tests/``, ``__graft_entry__`` (build) and ``bench.py`` (its CPU
baseline and ``--impl reference`` arm) may import this module; the product
package never does.  It imports nothing from ``pyspectrum_gb300``.

``bk_periodic_cpu`` follows the reference's own CPU path step by step
(pyspectrum.py:285-457 with the Fortran parts of estimator.f), structured as
the reference is -- single-precision grid, complex64 FFTs, one full 3D FFT
per shell, float64 triangle sums -- but running every stage on all host
cores:

===============================  ===========================================
reference (file:line)            here
===============================  ===========================================
pyspectrum.py:938-945            clip + float32 cast (numpy)
estimator.f:284-512 assign_quad  ``cpu_assign_pcs`` (C, OpenMP, z slabs)
pyspectrum.py:1060-1080 _FFT     ``scipy.fft.ifftn`` complex64, unnormalised
                                 (pocketfft on all cores stands in for
                                 threaded FFTW, which this machine lacks)
estimator.f:605-675 fcomb        ``cpu_fcomb_periodic`` (C, OpenMP)
pyspectrum.py:1134-1157          ``cpu_reflect`` (C, OpenMP)
pyspectrum.py:387-404 shells     ``cpu_shell_extract`` + ``scipy.fft.fftn``
                                 complex64 + ``cpu_real_part`` (p0k sums)
pyspectrum.py:407 counts         read from a cache, as the reference does
pyspectrum.py:415-445 triangles  ``cpu_triangle_sums_f32`` (C, OpenMP)
pyspectrum.py:341-356 units      numpy
===============================  ===========================================
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB = os.path.join(_BUILD, "liboracle_cpu.so")
_SRCS = ("cpu_mesh.c", "cpu_tri.c")
_lib = None


def build(force: bool = False) -> str:
    """Compile the OpenMP CPU restatement.  cpu_mesh.c follows the Fortran's
    IEEE single-precision arithmetic, so it is built without multiply-add
    contraction; the float64 triangle sums may contract."""
    srcs = [os.path.join(_HERE, s) for s in _SRCS]
    if (not force and os.path.exists(_LIB)
            and all(os.path.getmtime(_LIB) >= os.path.getmtime(s) for s in srcs)):
        return _LIB
    os.makedirs(_BUILD, exist_ok=True)
    objs = []
    for src, fp in zip(srcs, ("-ffp-contract=off", "-ffp-contract=fast")):
        obj = os.path.join(_BUILD, os.path.basename(src)[:-2] + ".o")
        subprocess.check_call(["gcc", "-O3", "-std=gnu11", fp, "-fno-fast-math", "-fopenmp", "-fPIC", "-c", src,
                               "-o", obj])
        objs.append(obj)
    tmp = _LIB + ".tmp"
    subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", tmp] + objs + ["-lm"])
    os.replace(tmp, _LIB)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        P, I64, I, F, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float, ctypes.c_double
        sig = {
            "cpu_assign_pcs": (None, [P, P, I64, I, F, F, P, I]),
            "cpu_fcomb_periodic": (None, [P, I, F, I]),
            "cpu_reflect": (None, [P, I, P, I]),
            "cpu_shell_extract": (None, [P, I, I, I, P, I]),
            "cpu_real_part": (D, [P, I64, P, I]),
            "cpu_triangle_sums_f32": (None, [P, I64, I, P, I, P, I]),
            "cpu_triangle_sums_f64": (None, [P, I64, I, P, I, P, P, I]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def triangles(jmin, nmax):
    """pyspectrum.py:415-422 loop as an int32 (3, T) array and its fac."""
    out, fac = [], []
    for i in range(jmin, nmax + 1):
        for j in range(jmin, i + 1):
            for l in range(max(i - j, jmin), j + 1):
                out.append((i, j, l))
                f = 1.0
                if j == l and i == j:
                    f = 6.0
                if i == j and j != l:
                    f = 2.0
                if i == l and l != j:
                    f = 2.0
                if j == l and l != i:
                    f = 2.0
                fac.append(f)
    return np.array(out, dtype=np.int32).T.copy(), np.array(fac)


def delta_half(xyz, Lbox, Ngrid, w=None, threads=None):
    """FFT_periodic (pyspectrum.py:909-959): half grid delta(k) complex64
    [z][y][x <= N/2] and the stage times."""
    import scipy.fft as sfft
    L = lib()
    th = threads or cores()
    n = int(Ngrid)
    t = {}
    t0 = time.perf_counter()
    xyz = np.asarray(xyz, dtype=np.float64)
    npart = xyz.shape[1]
    r = np.empty((npart, 3), dtype=np.float32)          # Fortran r(3, np): r[3 i + d]
    r[:] = np.clip(xyz, 0.0, Lbox * (1.0 - 1e-6)).T      # pyspectrum.py:938-941
    wf = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
    wsum = float(npart) if w is None else float(np.sum(np.asarray(w, dtype=np.float64)))
    kf_ks = np.float32(float(n) / Lbox)
    grid = np.zeros((n, n, n), dtype=np.complex64)
    L.cpu_assign_pcs(r.ctypes.data, None if wf is None else wf.ctypes.data, npart, n, float(kf_ks), 0.0,
                     grid.ctypes.data, th)
    t["assign_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    grid = sfft.ifftn(grid, norm="forward", workers=th, overwrite_x=True)   # FFTW_BACKWARD, unnormalised
    t["fft_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    grid = np.ascontiguousarray(grid, dtype=np.complex64)
    L.cpu_fcomb_periodic(grid.ctypes.data, n, float(np.float32(wsum)), th)
    half = np.ascontiguousarray(grid[:, :, : n // 2 + 1])
    t["fcomb_s"] = time.perf_counter() - t0
    return half, t


def shell_fields_f32(full, step, jmin, nmax, threads=None):
    """Shell fields (pyspectrum.py:387-404) as float32 (S, N^3) -- the values
    FFTW single precision produces, which the reference keeps in float64 --
    and the sums of squares per shell (float64)."""
    import scipy.fft as sfft
    L = lib()
    th = threads or cores()
    n = full.shape[0]
    S = nmax - jmin + 1
    F = np.empty((S, n ** 3), dtype=np.float32)
    p0 = np.zeros(S)
    work = np.empty((n, n, n), dtype=np.complex64)
    for s in range(S):
        L.cpu_shell_extract(full.ctypes.data, n, step, jmin + s, work.ctypes.data, th)
        out = sfft.fftn(work, workers=th)
        out = np.ascontiguousarray(out, dtype=np.complex64)
        p0[s] = L.cpu_real_part(out.ctypes.data, n ** 3, F[s].ctypes.data, th)
    return F, p0


def triangle_sums(F, tri_slots, threads=None):
    """bsum[t] = sum_v F_i F_j F_l over the rows of F (float32 or float64);
    for float64 fields also sum_v |F_i F_j F_l|."""
    L = lib()
    th = threads or cores()
    tri = np.ascontiguousarray(tri_slots, dtype=np.int32)
    T = tri.shape[1]
    bsum = np.zeros(T)
    if F.dtype == np.float32:
        L.cpu_triangle_sums_f32(F.ctypes.data, F.shape[1], F.shape[0], tri.ctypes.data, T, bsum.ctypes.data, th)
        return bsum
    F = np.ascontiguousarray(F, dtype=np.float64)
    absum = np.zeros(T)
    L.cpu_triangle_sums_f64(F.ctypes.data, F.shape[1], F.shape[0], tri.ctypes.data, T, bsum.ctypes.data,
                            absum.ctypes.data, th)
    return bsum, absum


def reflect(half, threads=None):
    L = lib()
    n = half.shape[0]
    full = np.empty((n, n, n), dtype=np.complex64)
    L.cpu_reflect(np.ascontiguousarray(half, dtype=np.complex64).ctypes.data, n, full.ctypes.data,
                  threads or cores())
    return full


def mode_counts(n, step, nmax):
    """Nk[j] (pyspectrum.py:380) from the exact integer shell rule."""
    a = np.minimum(np.arange(n), n - np.arange(n)).astype(np.int64)
    d2 = (a[:, None, None] ** 2 + a[None, :, None] ** 2 + a[None, None, :] ** 2).ravel()
    m = np.floor(np.sqrt(d2.astype(np.float64)) / step + 0.5).astype(np.int64)
    m -= ((2 * m - 1) ** 2 * step * step > 4 * d2) & (m > 0)
    m += (2 * m + 1) ** 2 * step * step <= 4 * d2
    return np.bincount(m[m <= nmax], minlength=nmax + 1)[: nmax + 1].astype(np.int64)


def bk_periodic_cpu(xyz, Lbox, Ngrid, step, Ncut, Nmax, counts, w=None, threads=None, nk=None):
    """Bk_periodic (pyspectrum.py:285-356) on the host cores.

    counts: exact integer triangle counts in loop order (the reference reads
    them from its cache, pyspectrum.py:407).  Returns (output dict with the
    reference's keys for the triangles with counts > 0, stage times)."""
    n = int(Ngrid)
    jmin = Ncut // step
    half, t = delta_half(xyz, Lbox, n, w, threads)
    t0 = time.perf_counter()
    full = reflect(half, threads)
    t["reflect_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    F, p0 = shell_fields_f32(full, step, jmin, Nmax, threads)
    t["shells_s"] = time.perf_counter() - t0
    del full
    tri, fac = triangles(jmin, Nmax)
    t0 = time.perf_counter()
    bsum = triangle_sums(F, tri - jmin, threads)
    t["triangles_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    V = float(n) ** 3
    if nk is None:
        nk = mode_counts(n, step, Nmax)
    p0k = np.zeros(Nmax)
    with np.errstate(invalid="ignore", divide="ignore"):
        p0k[jmin - 1:Nmax] = p0 / V / nk[jmin:Nmax + 1]                   # pyspectrum.py:404
    counts = np.asarray(counts, dtype=np.float64)
    keep = counts > 0
    i, j, l = (tri[k][keep] for k in range(3))
    c = counts[keep] * V                                                  # sum_x I_i I_j I_l
    b = bsum[keep] / c
    p1, p2, p3 = p0k[i - 1], p0k[j - 1], p0k[l - 1]
    npart = np.asarray(xyz).shape[1]
    wsum = float(npart) if w is None else float(np.sum(w))
    nbar = wsum / Lbox ** 3
    out = {"i_k1": i.astype(np.int64) * step, "i_k2": j.astype(np.int64) * step, "i_k3": l.astype(np.int64) * step,
           "p0k1": p1, "p0k2": p2, "p0k3": p3, "b123": b, "q123": b / (p1 * p2 + p2 * p3 + p3 * p1),
           "counts": counts[keep] / fac[keep]}
    # pyspectrum.py:341-355: units and shot noise
    kf = 2 * np.pi / Lbox
    for k in ("p0k1", "p0k2", "p0k3"):
        out[k] = out[k] * (2 * np.pi) ** 3 / kf ** 3 - 1.0 / nbar
    out["p0k_sn"] = 1.0 / nbar
    b_sn = (out["p0k1"] + out["p0k2"] + out["p0k3"]) / nbar + 1.0 / nbar ** 2
    out["b123"] = out["b123"] * (2 * np.pi) ** 6 / kf ** 6 - b_sn
    out["b123_sn"] = b_sn
    out["q123"] = out["b123"] / (out["p0k1"] * out["p0k2"] + out["p0k1"] * out["p0k3"] + out["p0k2"] * out["p0k3"])
    out["meta"] = {"Lbox": Lbox, "Ngrid": n, "step": step, "Ncut": Ncut, "Nmax": Nmax, "N": npart, "nbar": nbar,
                   "kf": kf}
    out["raw_bsum"] = bsum[keep]
    t["normalize_s"] = time.perf_counter() - t0
    return out, t
