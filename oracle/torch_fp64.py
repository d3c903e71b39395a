"""Float64 bispectrum sums with plain PyTorch -- TEST INFRASTRUCTURE ONLY.

The double-precision counterpart of the shell + triangle stages
(pyspectrum.py:373-404 and :415-430), written with nothing but torch tensor
operations (torch.fft on complex128, elementwise products and float64
matrix-vector products), so it runs on the GPU machine's device at the full
360^3 / Nmax 40 size in seconds and on the CPU in the small tests that pin
it against ``pyspec_oracle``.  It uses no code of the product package.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s accuracy
check may import it.

Grids here are indexed [z, y, x] (x fastest), like the device library; the
half grid holds x in [0, N/2].
"""
from __future__ import annotations

import numpy as np
import torch


def reflect_half(half: torch.Tensor) -> torch.Tensor:
    """pyspectrum.py:1134-1157 in complex128: full grid from the half grid,
    delta(-k) = conj(delta(k)), the seven Nyquist corners real."""
    n = half.shape[0]
    h = n // 2
    half = half.to(torch.complex128)
    full = torch.empty((n, n, n), dtype=torch.complex128, device=half.device)
    full[:, :, : h + 1] = half
    neg = (-torch.arange(n, device=half.device)) % n
    mirrored = half.index_select(0, neg).index_select(1, neg)      # [-z, -y, x]
    full[:, :, h + 1:] = torch.conj(mirrored[:, :, 1:h].flip(-1))   # x > N/2 <- conj at N - x
    for z in (0, h):
        for y in (0, h):
            for x in (0, h):
                if x + y + z:
                    full[z, y, x] = full[z, y, x].real.to(torch.complex128)
    return full


def shell_index(n: int, step: int, device) -> torch.Tensor:
    """irk = int(|k|/step + 0.5) (pyspectrum.py:373-378) as the exact integer
    rule: the largest m with (2m-1)^2 step^2 <= 4|k|^2."""
    i = torch.arange(n, device=device)
    a = torch.minimum(i, n - i).to(torch.int64)
    d2 = a.view(n, 1, 1) ** 2 + a.view(1, n, 1) ** 2 + a.view(1, 1, n) ** 2
    m = torch.floor(torch.sqrt(d2.to(torch.float64)) / step + 0.5).to(torch.int64)
    m = m - (((2 * m - 1) ** 2 * step * step > 4 * d2) & (m > 0)).to(torch.int64)
    m = m + ((2 * m + 1) ** 2 * step * step <= 4 * d2).to(torch.int64)
    return m


def shell_fields(full: torch.Tensor, step: int, jmin: int, nmax: int):
    """F[s] = Re(fftn(delta * [irk == jmin + s])) in float64, (S, N^3), and
    sum_v F[s]^2 per shell (pyspectrum.py:387-404 in double precision)."""
    n = full.shape[0]
    irk = shell_index(n, step, full.device)
    S = nmax - jmin + 1
    F = torch.empty((S, n ** 3), dtype=torch.float64, device=full.device)
    zero = torch.zeros((), dtype=torch.complex128, device=full.device)
    for s in range(S):
        tmp = torch.where(irk == jmin + s, full, zero)
        F[s] = torch.fft.fftn(tmp).real.reshape(-1)
        del tmp
    p0 = (F * F).sum(dim=1)
    return F, p0


def triangle_sums(F: torch.Tensor, tri_slots, with_abs: bool = True):
    """For each triangle t of tri_slots (int (3, T) rows of F):
    bsum[t] = sum_v F_i F_j F_l and absum[t] = sum_v |F_i F_j F_l|, float64.
    Triangles sharing their two largest shells share one pair product."""
    tri = np.asarray(tri_slots, dtype=np.int64)
    T = tri.shape[1]
    srt = -np.sort(-tri, axis=0)                   # per column: largest, middle, smallest
    groups: dict = {}
    for t in range(T):
        groups.setdefault((int(srt[0, t]), int(srt[1, t])), []).append((int(srt[2, t]), t))
    bsum = np.zeros(T)
    absum = np.zeros(T)
    Fa = F.abs() if with_abs else None
    for (a, b), lst in groups.items():
        P = F[a] * F[b]
        Pa = P.abs() if with_abs else None
        ls = torch.tensor([l for l, _ in lst], device=F.device)
        ts = [t for _, t in lst]
        lo, hi = int(ls.min()), int(ls.max())
        if hi - lo + 1 == len(lst) and bool((ls == torch.arange(lo, hi + 1, device=F.device)).all()):
            rows = slice(lo, hi + 1)               # a contiguous run of columns: no copy
            v = (F[rows] @ P).cpu().numpy()
            va = (Fa[rows] @ Pa).cpu().numpy() if with_abs else None
            order = [l - lo for l, _ in lst]
        else:
            v = (F.index_select(0, ls) @ P).cpu().numpy()
            va = (Fa.index_select(0, ls) @ Pa).cpu().numpy() if with_abs else None
            order = list(range(len(lst)))
        for k, t in enumerate(ts):
            bsum[t] = v[order[k]]
            if with_abs:
                absum[t] = va[order[k]]
        del P, Pa
    return bsum, absum


def error_report(got, exact, absum):
    """Accuracy metrics of raw triangle sums against float64 ones: median and
    maximum |dB/B|, the maximum over triangles with condition number
    sum|FFF| / |sum FFF| < 1e3, and the maximum error normalised by
    sum|FFF|."""
    got = np.asarray(got, dtype=np.float64)
    err = np.abs(got - exact)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = err / np.abs(exact)
        cond = absum / np.abs(exact)
    well = cond < 1e3
    return {"triangles": int(len(exact)), "median_rel": float(np.median(rel)), "max_rel": float(rel.max()),
            "max_rel_cond_lt_1e3": float(rel[well].max()) if well.any() else 0.0,
            "n_cond_lt_1e3": int(well.sum()), "normalised_max": float((err / absum).max())}
