"""GPU parity: shells, triangle counts, contraction and the bispectrum API vs
the oracle and the reference's golden vectors."""
import numpy as np
import pytest
import torch

from oracle import pyspec_oracle as O
from pyspectrum_gb300 import core, pyspectrum as P
from pyspectrum_gb300._lib import call, ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _zyx(a):
    return np.ascontiguousarray(np.asarray(a).transpose(2, 1, 0))


@pytest.fixture(autouse=True)
def _private_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("PYSPEC_GB300_CACHE", str(tmp_path))
    core._counts_mem.clear()
    core.release_plans()
    yield
    core.release_plans()


@pytest.mark.parametrize("n,step,jmin,nmax", [(16, 1, 1, 8), (24, 2, 1, 6), (32, 3, 1, 5), (30, 2, 2, 7)])
def test_shell_fields_match_oracle(n, step, jmin, nmax):
    rng = np.random.default_rng(n)
    full = np.fft.ifftn(rng.standard_normal((n, n, n))) * n ** 3
    half = full[: n // 2 + 1]
    df = O.reflect_delta(half, n)
    F, p0k, nk = O.shell_fields(df, step, jmin, nmax)
    S = nmax - jmin + 1
    h = torch.from_numpy(_zyx(half.astype(np.complex64))).cuda()
    fields = torch.empty((S, n ** 3), dtype=torch.float32, device="cuda")
    p0 = torch.empty(S, dtype=torch.float64, device="cuda")
    lib = core._lib.load()
    ws = torch.empty(lib.pyspec_shell_fields_workspace(n, S), dtype=torch.uint8, device="cuda")
    call("pyspec_shell_fields", ptr(h), n, step, jmin, nmax, ptr(fields), ptr(p0), ptr(ws), ws.numel(), stream_ptr())
    got = fields.cpu().numpy().reshape(S, n, n, n)
    p0g = p0.cpu().numpy()
    for s in range(S):
        j = jmin + s
        ref = F[j].transpose(2, 1, 0)
        scale = max(np.abs(ref).max(), 1e-30)
        assert np.abs(got[s] - ref).max() < 2e-6 * scale, (j, np.abs(got[s] - ref).max() / scale)
        np.testing.assert_allclose(p0g[s], np.sum(F[j] ** 2), rtol=1e-5)


@pytest.mark.parametrize("n,step,shells", [(192, 3, (1, 17, 40)), (256, 4, (2, 31))])
def test_shell_fields_large_grids(n, step, shells):
    """Grid sizes with compile-time FFT plans, checked against numpy on a few shells."""
    rng = np.random.default_rng(n)
    half = (rng.standard_normal((n // 2 + 1, n, n)) + 1j * rng.standard_normal((n // 2 + 1, n, n))) / n ** 1.5
    half[0] = half[0].real
    df = O.reflect_delta(half, n)
    irk = O.shell_index(n, step)
    jmin, nmax = min(shells), max(shells)
    S = nmax - jmin + 1
    h = torch.from_numpy(_zyx(half.astype(np.complex64))).cuda()
    fields = torch.empty((S, n ** 3), dtype=torch.float32, device="cuda")
    p0 = torch.empty(S, dtype=torch.float64, device="cuda")
    ws = torch.empty(core._lib.load().pyspec_shell_fields_workspace(n, S), dtype=torch.uint8, device="cuda")
    call("pyspec_shell_fields", ptr(h), n, step, jmin, nmax, ptr(fields), ptr(p0), ptr(ws), ws.numel(), stream_ptr())
    for j in shells:
        ref = np.real(np.fft.fftn(np.where(irk == j, df, 0))).transpose(2, 1, 0)
        got = fields[j - jmin].cpu().numpy().reshape(n, n, n)
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() < 3e-6 * scale, (j, np.abs(got - ref).max() / scale)
        np.testing.assert_allclose(p0[j - jmin].item(), np.sum(ref.astype(np.float64) ** 2), rtol=1e-5)


@pytest.mark.parametrize("n,step,ncut,nmax", [(16, 1, 1, 8), (16, 3, 3, 5), (24, 2, 2, 6), (32, 3, 3, 5)])
def test_counts_match_reference_compute_path(golden, n, step, ncut, nmax):
    g = golden("ref_bk_small.npz")
    ref = g[f"n{n}_s{step}_c{ncut}_m{nmax}_countscache"]
    got = P._counts_Bk123(Ngrid=n, Nmax=nmax, Ncut=ncut, step=step)
    exact_ref = np.rint(ref / n ** 3)
    np.testing.assert_array_equal(np.rint(got / n ** 3), exact_ref)
    np.testing.assert_array_equal(got, exact_ref * float(n) ** 3)
    c, nk = core.triangle_counts(n, nmax, ncut, step)
    np.testing.assert_array_equal(nk, O.mode_counts(n, step, nmax))


@pytest.mark.parametrize("nmax", [10, 40, 50])
def test_counts_match_reference_cache_360(golden, nmax):
    """Bit-exact triangle counts against the reference's shipped caches."""
    g = golden("counts_ref360.npz")
    c, nk = core.triangle_counts(360, nmax, 3, 3)
    np.testing.assert_array_equal(c, g[f"nmax{nmax}"])
    np.testing.assert_array_equal(nk, O.mode_counts(360, 3, nmax))


def test_bk_stage_matches_reference_golden(golden):
    """_Bk_periodic on the reference's own delta(k) grids vs its outputs."""
    g = golden("ref_bk_small.npz")
    for n, step, ncut, nmax in g["cases"]:
        n, step, ncut, nmax = int(n), int(step), int(ncut), int(nmax)
        tag = f"n{n}_s{step}_c{ncut}_m{nmax}"
        bk = P._Bk_periodic(g[tag + "_delta_fft"], Nmax=nmax, Ncut=ncut, step=step)
        cache = g[tag + "_countscache"]
        loop = O.triangles(ncut // step, nmax)
        cv = np.array([cache[i - 1, j - 1, l - 1] for i, j, l, _ in loop])
        real = np.rint(cv / n ** 3) > 0            # exact count > 0
        tri = np.array([(i, j, l) for i, j, l, _ in loop])[real]
        np.testing.assert_array_equal(bk["i_k1"], tri[:, 0] * step)
        np.testing.assert_array_equal(bk["i_k3"], tri[:, 2] * step)
        keep = cv > 0
        sel = real[keep]
        for k in ("p0k1", "p0k2", "p0k3", "b123", "q123", "counts"):
            r = g[tag + "_" + k][keep][sel]
            np.testing.assert_allclose(bk[k], r, rtol=1e-5, atol=2e-6 * np.abs(r).max(), err_msg=k)


def _bk_oracle_subset(xyz, L, n, step, ncut, nmax, tri_idx):
    half = O.FFT_periodic(xyz, Lbox=L, Ngrid=n)
    df = O.reflect_delta(half, n)
    F, p0k, nk = O.shell_fields(df, step, ncut // step, nmax)
    loop = O.triangles(ncut // step, nmax)
    out = []
    for t in tri_idx:
        i, j, l, _ = loop[t]
        prod = F[i] * F[j] * F[l]
        out.append((prod.sum(), np.abs(prod).sum()))
    return np.array(out), p0k, nk


@pytest.mark.parametrize("method", ["fp32", "bf16x3"])
def test_bk_periodic_matches_oracle(method):
    """Bk_periodic end to end on uniform particles (N=48, step 2, Nmax 12)."""
    n, L, step, ncut, nmax = 48, 1000.0, 2, 2, 12
    rng = np.random.default_rng(11)
    xyz = rng.uniform(0, L, size=(3, 40000))
    bk = P.Bk_periodic(xyz, Lbox=L, Ngrid=n, step=step, Ncut=ncut, Nmax=nmax, method=method)
    plan = core.get_plan(n, step, ncut, nmax, method)
    loop = O.triangles(1, nmax)
    keep = plan.counts_np > 0
    idx = np.nonzero(keep)[0]
    ref, p0k, nk = _bk_oracle_subset(xyz, L, n, step, ncut, nmax, idx)
    bsum = plan.bsum.cpu().numpy()[idx]
    # raw triangle sums: error normalised by sum |F_i F_j F_l|
    err = np.abs(bsum - ref[:, 0]) / ref[:, 1]
    assert err.max() < (1e-5 if method == "fp32" else 3e-5), err.max()
    # API values: recompute the reference formulas from the oracle sums
    nbar = xyz.shape[1] / L ** 3
    kf = 2 * np.pi / L
    counts = plan.counts_np[idx].astype(np.float64) * n ** 3
    tri = np.array([loop[t][:3] for t in idx])
    pp = p0k[tri - 1] * (2 * np.pi) ** 3 / kf ** 3 - 1 / nbar
    bsn = pp.sum(1) / nbar + 1 / nbar ** 2
    b = ref[:, 0] / counts * (2 * np.pi) ** 6 / kf ** 6 - bsn
    # compare before the shot-noise subtraction: uniform particles have P ~ 1/nbar,
    # so the subtracted values are small differences of large numbers
    np.testing.assert_allclose(bk["p0k1"] + 1 / nbar, pp[:, 0] + 1 / nbar, rtol=1e-5)
    np.testing.assert_allclose(bk["b123_sn"], bsn, rtol=1e-5)
    rt = 1e-5 if method == "fp32" else 1e-4
    np.testing.assert_allclose(bk["b123"] + bk["b123_sn"], b + bsn, rtol=rt, atol=rt * np.abs(b + bsn).max())
    assert bk["meta"]["Ngrid"] == n and len(bk["b123"]) == len(idx)
