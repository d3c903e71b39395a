"""Error of both contraction forms against float64 at the full 360^3 / step 3 /
Nmax 40 size, on a 1,000,000-particle Zel'dovich box (L = 2500).

Both sides start from the same delta(k) (this package's FFT_periodic):
the float64 side builds the sampled shell fields with complex128 FFTs
(pyspectrum.py:387-404 in double precision) and sums F_i F_j F_l in float64
(pyspectrum.py:424-426); the GPU side is Bk_periodic's shell + contraction
stages.  Reported per method: raw-B relative error, error normalised by
sum |F_i F_j F_l|, the maximum relative error over triangles with condition
number sum|FFF| / |sum FFF| < 1e3, and the raw maximum."""
import numpy as np
import pytest
import scipy.fft as sfft

from oracle import pyspec_oracle as O

pytestmark = pytest.mark.gpu

SHELLS = (1, 2, 3, 5, 8, 13, 20, 27, 34, 40)


def _fp64_sums(half_xyz, n, step, tri):
    full = O.reflect_delta(half_xyz, n).astype(np.complex128)
    irk = O.shell_index(n, step)
    F = {}
    for j in sorted({int(v) for t in tri for v in t}):
        F[j] = np.real(sfft.fftn(np.where(irk == j, full, 0), workers=-1)).ravel()
    out = []
    for i, j, l in tri:
        prod = F[i] * F[j] * F[l]
        out.append((prod.sum(), np.abs(prod).sum()))
    return np.array(out)


def test_contraction_error_vs_float64_full_size():
    import torch
    from pyspectrum_gb300 import core, mocks
    n, L, step, ncut, nmax = 360, 2500.0, 3, 3, 40
    x = mocks.zeldovich_mock(1_000_000, L, ngrid=n, seed=2)
    xyzs, ws = core.prepare_positions(x, L)
    half = core.fft_periodic_half(xyzs, ws, n, L, float(x.shape[1]))
    half_xyz = half.cpu().numpy().transpose(2, 1, 0)
    loop = core.triangles(ncut // step, nmax)
    sel = [t for t in range(loop.shape[1]) if all(int(v) in SHELLS for v in loop[:, t])]
    tri = [tuple(int(v) for v in loop[:, t]) for t in sel]
    ref = _fp64_sums(half_xyz, n, step, tri)
    exact, absum = ref[:, 0], ref[:, 1]
    cond = absum / np.abs(exact)
    report = {}
    for method in ("fp32", "bf16x3"):
        plan = core.get_plan(n, step, ncut, nmax, method)
        plan.run(half)
        torch.cuda.synchronize()
        got = plan.bsum.cpu().numpy()[sel]
        err = np.abs(got - exact)
        rel = err / np.abs(exact)
        report[method] = {"median_rel": float(np.median(rel)), "normalised_max": float((err / absum).max()),
                          "max_rel_cond_lt_1e3": float(rel[cond < 1e3].max()), "max_rel": float(rel.max())}
    print("triangles", len(sel), "cond median", float(np.median(cond)), report)
    assert report["fp32"]["normalised_max"] < 2e-6
    assert report["bf16x3"]["normalised_max"] < 2e-5
    assert report["fp32"]["max_rel_cond_lt_1e3"] < 1e-3
    assert report["bf16x3"]["max_rel_cond_lt_1e3"] < 1e-2
