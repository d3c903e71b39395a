"""The CPU-side checkers agree with the oracle (no GPU).

``oracle/cpu_ref.py`` (the all-core C restatement that bench.py times as the
reference's CPU path) and ``oracle/torch_fp64.py`` (float64 shell fields and
triangle sums in plain torch, used by the full-size accuracy checks) are
pinned here against ``oracle/pyspec_oracle.py`` on small boxes."""
import numpy as np
import pytest
import torch

from oracle import cpu_ref as C
from oracle import pyspec_oracle as O
from oracle import torch_fp64 as TF


@pytest.fixture(scope="module")
def box():
    n, L = 32, 1000.0
    rng = np.random.default_rng(7)
    centres = rng.uniform(0, L, (3, 60))
    xyz = (centres[:, rng.integers(0, 60, 30000)] + rng.normal(0, 30.0, (3, 30000))) % L
    half = O.FFT_periodic(xyz, Lbox=L, Ngrid=n)          # [x, y, z] complex128
    return n, L, xyz, half


def test_cpu_delta_matches_oracle(box):
    n, L, xyz, half = box
    got, _ = C.delta_half(xyz, L, n, threads=3)          # single precision, [z, y, x]
    ref = half.transpose(2, 1, 0)
    assert np.abs(got - ref).max() <= 2e-6 * np.abs(ref).max()
    full = C.reflect(got, threads=2)
    fref = O.reflect_delta(half, n).transpose(2, 1, 0)
    assert np.abs(full - fref).max() <= 2e-6 * np.abs(fref).max()


def test_cpu_assignment_independent_of_thread_count(box):
    n, L, xyz, _ = box
    a, _ = C.delta_half(xyz, L, n, threads=1)
    b, _ = C.delta_half(xyz, L, n, threads=5)
    np.testing.assert_array_equal(a, b)


def test_cpu_bk_matches_oracle(box):
    n, L, xyz, half = box
    step, ncut, nmax = 2, 2, 8
    ref = O._Bk_periodic(O.reflect_delta(half, n), Nmax=nmax, Ncut=ncut, step=step)
    counts_raw, exact = O.counts_Bk123(n, nmax, ncut, step)
    tri, _ = C.triangles(1, nmax)
    cnt = np.array([exact[i - 1, j - 1, l - 1] for i, j, l in tri.T])
    got, _ = C.bk_periodic_cpu(xyz, L, n, step, ncut, nmax, cnt, threads=4)
    np.testing.assert_array_equal(got["i_k1"], ref["i_k1"])
    np.testing.assert_array_equal(got["i_k3"], ref["i_k3"])
    np.testing.assert_allclose(got["raw_bsum"], ref["raw_bsum"], rtol=1e-5,
                               atol=1e-5 * np.abs(ref["raw_bsum"]).max())
    nbar = xyz.shape[1] / L ** 3
    np.testing.assert_allclose(got["p0k1"] + 1 / nbar, ref["p0k1"] * L ** 3, rtol=1e-5)


def test_cpu_triangle_sums_exact_order_free():
    rng = np.random.default_rng(3)
    F = rng.standard_normal((9, 1000)).astype(np.float32)
    tri, _ = C.triangles(1, 9)
    slots = tri - 1
    perm = rng.permutation(slots.shape[1])
    a = C.triangle_sums(F, slots, threads=2)
    b = C.triangle_sums(F, slots[:, perm], threads=7)
    np.testing.assert_array_equal(a[perm], b)
    F64 = F.astype(np.float64)
    ref = np.array([np.sum(F64[i] * F64[j] * F64[l]) for i, j, l in slots.T])
    np.testing.assert_allclose(a, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    s, ab = C.triangle_sums(F64, slots, threads=3)
    np.testing.assert_allclose(s, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    aref = np.array([np.sum(np.abs(F64[i] * F64[j] * F64[l])) for i, j, l in slots.T])
    np.testing.assert_allclose(ab, aref, rtol=1e-12)


def test_torch_fp64_matches_oracle(box):
    n, L, xyz, half = box
    step, jmin, nmax = 2, 1, 8
    full_o = O.reflect_delta(half, n)                     # [x, y, z]
    full_t = TF.reflect_half(torch.from_numpy(np.ascontiguousarray(half.transpose(2, 1, 0))))
    np.testing.assert_array_equal(full_t.numpy(), full_o.transpose(2, 1, 0))
    F, p0 = TF.shell_fields(full_t, step, jmin, nmax)
    Fo, p0o, nk = O.shell_fields(full_o, step, jmin, nmax)
    for j in range(jmin, nmax + 1):
        ref = Fo[j].transpose(2, 1, 0).ravel()
        np.testing.assert_allclose(F[j - jmin].numpy(), ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    tri, _ = C.triangles(jmin, nmax)
    bsum, absum = TF.triangle_sums(F, tri - jmin)
    Fn = F.numpy()
    ref = np.array([np.sum(Fn[i - 1] * Fn[j - 1] * Fn[l - 1]) for i, j, l in tri.T])
    aref = np.array([np.sum(np.abs(Fn[i - 1] * Fn[j - 1] * Fn[l - 1])) for i, j, l in tri.T])
    np.testing.assert_allclose(bsum, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(absum, aref, rtol=1e-11)
    # an arbitrary (non-loop) order of the same triangles
    perm = np.random.default_rng(0).permutation(tri.shape[1])
    b2, _ = TF.triangle_sums(F, (tri - jmin)[:, perm], with_abs=False)
    np.testing.assert_allclose(b2, bsum[perm], rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    rep = TF.error_report(bsum * (1 + 1e-9), bsum, absum)
    assert rep["median_rel"] == pytest.approx(1e-9, rel=1e-3)
