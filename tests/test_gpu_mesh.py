"""GPU parity: particles -> delta(k) (assignment, FFT, fcomb, reflection) vs the oracle."""
import numpy as np
import pytest
import torch

from oracle import pyspec_oracle as O
from pyspectrum_gb300 import core, pyspectrum as P
from pyspectrum_gb300._lib import call, ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _zyx(a_xyz):
    return np.ascontiguousarray(np.asarray(a_xyz).transpose(2, 1, 0))


@pytest.mark.parametrize("n", [8, 16, 24, 30, 40, 64, 96, 192, 256])
@pytest.mark.parametrize("sign", [1, -1])
def test_fft3d_c2c_matches_numpy(n, sign):
    rng = np.random.default_rng(n)
    a = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex64)
    t = torch.from_numpy(a).cuda()
    call("pyspec_fft3d_c2c", ptr(t), n, sign, stream_ptr())
    got = t.cpu().numpy()
    ref = np.fft.fftn(a.astype(np.complex128)) if sign < 0 else np.fft.ifftn(a.astype(np.complex128)) * n ** 3
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-6, err


@pytest.mark.parametrize("n", [360, 512])
def test_fft3d_roundtrip_large(n):
    """Forward then backward transform returns N^3 times the input (sizes with
    compile-time plans), and Parseval holds."""
    g = torch.Generator(device="cuda").manual_seed(n)
    a = torch.complex(torch.randn((n, n, n), device="cuda", generator=g),
                      torch.randn((n, n, n), device="cuda", generator=g))
    t = a.clone()
    call("pyspec_fft3d_c2c", ptr(t), n, -1, stream_ptr())
    e_k = (t.abs() ** 2).double().sum().item()
    call("pyspec_fft3d_c2c", ptr(t), n, 1, stream_ptr())
    err = ((t / float(n) ** 3 - a).abs().max() / a.abs().max()).item()
    assert err < 2e-6, err
    e_x = (a.abs() ** 2).double().sum().item()
    assert abs(e_k / float(n) ** 3 - e_x) / e_x < 1e-5


def test_fft_matches_reference_golden(golden):
    """The reference's _FFT (de-interleave + unnormalised backward FFT)."""
    g = golden("ref_fft_small.npz")
    inter = g["interlaced"]           # (2N, N, N) Fortran array [slot, y, z]
    n = inter.shape[1]
    grid = (inter[0::2] + 1j * inter[1::2]).astype(np.complex64)     # [x, y, z]
    t = torch.from_numpy(_zyx(grid)).cuda()
    call("pyspec_fft3d_c2c", ptr(t), n, 1, stream_ptr())
    got = t.cpu().numpy().transpose(2, 1, 0)
    ref = g["out"]
    assert np.abs(got - ref).max() < 2e-6 * np.abs(ref).max()


def _particles(npart, L, seed):
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(0, L, size=(3, npart))
    xyz[:, :4] = [[0.0, L, L * (1 - 1e-7), 1e-9]] * 3          # edges: 0, L (clipped), just below L
    return xyz


@pytest.mark.parametrize("n,npart", [(16, 3000), (32, 20000), (48, 5000)])
def test_assignment_matches_oracle(n, npart):
    L = 500.0
    xyz = _particles(npart, L, n)
    w = np.random.default_rng(1).uniform(0.5, 2.0, npart)
    xs = O.clip_positions(xyz, L)
    kf_ks = np.float32(n / L)
    ref = O.assign_quad(xs, w.astype(np.float32), kf_ks, 0.0, n)
    xyz_d = core.positions_to_device(xyz)
    xyzs, ws = core.prepare_positions(xyz_d, L, torch.as_tensor(w, device="cuda"))
    np.testing.assert_array_equal(xyzs.cpu().numpy(), xs)
    grid = torch.zeros((n, n, n), dtype=torch.complex64, device="cuda")
    call("pyspec_assign_pcs_interlaced", ptr(xyzs), ptr(ws), npart, n, float(kf_ks), 0.0, ptr(grid), stream_ptr())
    got = grid.cpu().numpy().transpose(2, 1, 0)
    assert np.abs(got - ref).max() < 1e-5 * np.abs(ref).max()
    # mass: every particle deposits 6^3 w on each of the two grids
    np.testing.assert_allclose(got.real.sum(), 216.0 * w.astype(np.float32).sum(), rtol=1e-5)


@pytest.mark.parametrize("n", [8, 16, 18, 32])
def test_fcomb_matches_oracle(n):
    rng = np.random.default_rng(5 + n)
    G = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n)))
    ref = O.fcomb_periodic(G, 1234.5)
    g = torch.from_numpy(_zyx(G.astype(np.complex64))).cuda()
    half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device="cuda")
    call("pyspec_fcomb_periodic", ptr(g), n, 1234.5, ptr(half), stream_ptr())
    got = half.cpu().numpy().transpose(2, 1, 0)
    assert np.abs(got - ref).max() < 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("n,npart,L", [(32, 5000, 1000.0), (64, 30000, 2600.0), (60, 8000, 700.0)])
def test_fft_periodic_matches_oracle(n, npart, L):
    xyz = _particles(npart, L, 7)
    ref = O.FFT_periodic(xyz, Lbox=L, Ngrid=n)
    got = P.FFT_periodic(xyz, Lbox=L, Ngrid=n)
    assert got.shape == (n // 2 + 1, n, n)
    # float32 grid sums and FFT against the float64 oracle
    err = np.abs(got - ref).max() / np.abs(ref[1:]).max()
    assert err < 3e-5, err


def test_reflect_delta_matches_reference(golden):
    g = golden("ref_bk_small.npz")
    for n, step, ncut, nmax in g["cases"]:
        tag = f"n{n}_s{step}_c{ncut}_m{nmax}"
        got = P.reflect_delta(g[tag + "_delt"], Ngrid=int(n))
        np.testing.assert_array_equal(got, g[tag + "_delta_fft"])


def test_half_from_full_roundtrip(golden):
    g = golden("ref_bk_small.npz")
    tag = "n24_s2_c2_m6"
    full = torch.from_numpy(_zyx(g[tag + "_delta_fft"])).cuda()
    half = core.half_from_full(full).cpu().numpy().transpose(2, 1, 0)
    delt = g[tag + "_delt"]
    # away from x = 0, N/2 the reflected grid is exactly Hermitian, so the average is the input
    np.testing.assert_allclose(half[1:-1], delt[1:-1], rtol=0, atol=1e-6 * np.abs(delt).max())
    np.testing.assert_array_equal(half[0], g[tag + "_delta_fft"][0])
