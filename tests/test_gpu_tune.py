"""Tunable variants and the autotuner (GPU).

Every candidate the tuner may pick must compute what the default does:
* tiled mass assignment (shared-memory tiles of 4^3, 8^3, 16^3 cells) against
  the direct kernel and the oracle (estimator.f:284-512), including tiles cut
  by the grid edge, the survey's N/2-cell offset, weights and dense clusters;
* every radix-plan variant of the 3D FFT against numpy
  (pyspectrum.py:1073-1075, FFTW_BACKWARD unnormalised, and FFTW_FORWARD);
* the run tile plan of the tensor-core contraction against the cover plan;
and the tuner keeps its choices per key, on disk, and can be switched off."""
import ctypes
import json

import numpy as np
import pytest
import torch

from oracle import pyspec_oracle as O

pytestmark = pytest.mark.gpu


def _assign(kind, xyz32, w32, n, kf, offset):
    from pyspectrum_gb300 import _lib
    from pyspectrum_gb300._lib import call, ptr, stream_ptr
    npart = xyz32.shape[1]
    grid = torch.zeros((n, n, n, 2), dtype=torch.float32, device="cuda")
    if kind == "direct":
        call("pyspec_assign_pcs_interlaced", ptr(xyz32), ptr(w32), npart, n, kf, offset, ptr(grid), stream_ptr())
    else:
        tile = int(kind[5:])
        ws = torch.empty(_lib.load().pyspec_assign_tiled_workspace(npart, n, tile), dtype=torch.uint8, device="cuda")
        call("pyspec_assign_pcs_interlaced_tiled", ptr(xyz32), ptr(w32), npart, n, kf, offset, tile, ptr(grid),
             ptr(ws), ws.numel(), stream_ptr())
    torch.cuda.synchronize()
    return grid.cpu().numpy()


@pytest.mark.parametrize("n,L,offset_cells,clustered,weights", [
    (36, 500.0, 0.0, False, False),      # 36 = 2*16 + 4: tiles of 16 cut by the edge
    (48, 700.0, 0.0, True, True),        # dense clusters, weights
    (40, 800.0, 20.0, True, False),      # survey form: offset N/2, positions centred on 0
])
def test_tiled_assignment_matches_direct_and_oracle(n, L, offset_cells, clustered, weights):
    rng = np.random.default_rng(n)
    npart = 150_000
    if clustered:
        c = rng.uniform(0, L, (3, 30))
        xyz = (c[:, rng.integers(0, 30, npart)] + rng.normal(0, 10.0, (3, npart))) % L
    else:
        xyz = rng.uniform(0, L, (3, npart))
    if offset_cells:
        xyz = xyz - L / 2                # centred, as the survey positions
    w = rng.uniform(0.5, 1.5, npart) if weights else None
    kf = float(np.float32(n / L))
    xyz32 = torch.from_numpy(xyz.astype(np.float32)).cuda()
    w32 = None if w is None else torch.from_numpy(w.astype(np.float32)).cuda()
    # the oracle: float64 sums of the same single-precision weights.  Every
    # device variant sums in float32 in its own order; a cell with m
    # contributions is within ~m ulp of the exact sum (dense clusters put
    # thousands of particles in a cell), hence the relative tolerance.
    xyz_f = np.asfortranarray(xyz.astype(np.float32))
    g = O.assign_quad(xyz_f, None if w is None else w.astype(np.float32), np.float32(kf), offset_cells, n)
    ora = np.stack([g.real, g.imag], axis=-1).transpose(2, 1, 0, 3)     # [z, y, x, re/im]
    scale = np.abs(ora).max()
    ref = _assign("direct", xyz32, w32, n, kf, offset_cells)
    np.testing.assert_allclose(ref, ora, rtol=2e-5, atol=2e-7 * scale, err_msg="direct")
    for kind in ("tiled4", "tiled8", "tiled16"):
        got = _assign(kind, xyz32, w32, n, kf, offset_cells)
        np.testing.assert_allclose(got, ora, rtol=2e-5, atol=2e-7 * scale, err_msg=kind)
        np.testing.assert_allclose(got, ref, rtol=4e-5, atol=4e-7 * scale, err_msg=kind)
        # the cells touched are exactly the same
        np.testing.assert_array_equal(got != 0, ref != 0, err_msg=kind)
    # mass: every particle deposits its weight (x 6^3 per grid) on both grids
    tot = ref.astype(np.float64).sum(axis=(0, 1, 2)) / 216.0
    wsum = npart if w is None else float(np.sum(w.astype(np.float32)))
    np.testing.assert_allclose(tot, [wsum, wsum], rtol=1e-5)


def test_tiled_assignment_rejects_small_grid_and_bad_tile():
    from pyspectrum_gb300 import _lib
    from pyspectrum_gb300._lib import ptr, stream_ptr
    lib = _lib.load()
    xyz = torch.zeros((3, 10), dtype=torch.float32, device="cuda")
    grid = torch.zeros((16, 16, 16, 2), dtype=torch.float32, device="cuda")
    ws = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    assert lib.pyspec_assign_pcs_interlaced_tiled(ptr(xyz), None, 10, 16, 1.0, 0.0, 16, ptr(grid), ptr(ws),
                                                  ws.numel(), stream_ptr()) == -1          # 16 < 16 + 4
    assert lib.pyspec_assign_pcs_interlaced_tiled(ptr(xyz), None, 10, 16, 1.0, 0.0, 5, ptr(grid), ptr(ws),
                                                  ws.numel(), stream_ptr()) == -1          # tile 5
    assert lib.pyspec_assign_pcs_interlaced_tiled(ptr(xyz), None, 10, 16, 1.0, 0.0, 8, ptr(grid), ptr(ws), 16,
                                                  stream_ptr()) == -4                      # workspace


@pytest.mark.parametrize("n", [128, 192, 360])
def test_every_fft_variant_matches_numpy(n):
    import scipy.fft as sfft
    from pyspectrum_gb300 import tune
    from pyspectrum_gb300._lib import call, ptr, stream_ptr
    rng = np.random.default_rng(n)
    a = (rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))).astype(np.complex64)
    back = sfft.ifftn(a.astype(np.complex128), workers=-1) * float(n) ** 3
    fwd = sfft.fftn(a.astype(np.complex128), workers=-1)
    variants = tune.fft_variants(n)
    assert variants[-1][1] == (0, 0)                  # the Stockham form is always offered
    for v, split in variants:
        for sign, ref in ((1, back), (-1, fwd)):
            g = torch.from_numpy(a).cuda()
            call("pyspec_fft3d_c2c_variant", ptr(g), n, sign, v, stream_ptr())
            got = g.cpu().numpy()
            err = np.abs(got - ref).max() / np.abs(ref).max()
            assert err < 2e-6, (n, split, sign, err)
    # the plain entry point runs the default variant
    g = torch.from_numpy(a).cuda()
    call("pyspec_fft3d_c2c", ptr(g), n, 1, stream_ptr())
    g2 = torch.from_numpy(a).cuda()
    call("pyspec_fft3d_c2c_variant", ptr(g2), n, 1, tune.fft_default(n), stream_ptr())
    assert torch.equal(g, g2)


def test_plan_and_chunk_forms_agree():
    """Cover and run plans, 64- and 32-voxel chunks: the same sums to the
    split-BF16 accuracy."""
    from pyspectrum_gb300 import _lib, core
    from pyspectrum_gb300._lib import call, ptr, stream_ptr
    n, nmax = 48, 40
    rng = np.random.default_rng(5)
    fields = torch.from_numpy(rng.standard_normal((nmax, n ** 3)).astype(np.float32)).cuda()
    slots = np.ascontiguousarray(core.triangles(1, nmax) - 1, dtype=np.int32)
    T = slots.shape[1]
    tri_d = torch.from_numpy(slots).cuda()
    info = {}
    combos = (0, _lib.CONTRACT_KC32, _lib.CONTRACT_RUN_PLAN, _lib.CONTRACT_RUN_PLAN | _lib.CONTRACT_KC32)
    for flags in combos:
        v = np.zeros(9, dtype=np.int64)
        call("pyspec_bk_plan_check_flags", nmax, slots.ctypes.data_as(ctypes.c_void_p), T, flags, v.ctypes.data, 9)
        info[flags] = v
    assert info[0][2] == 1 and info[_lib.CONTRACT_RUN_PLAN][2] == 0      # cover vs run plan
    assert info[0][8] == 64 and info[_lib.CONTRACT_KC32][8] == 32        # 64- vs 32-voxel chunks
    out = {}
    lib = _lib.load()
    for flags in combos:
        ws = torch.zeros(lib.pyspec_bk_contract_workspace(n, nmax, T, 1 | flags), dtype=torch.uint8, device="cuda")
        b = torch.zeros(T, dtype=torch.float64, device="cuda")
        call("pyspec_bk_contract", ptr(fields), n, nmax, ptr(tri_d), slots.ctypes.data_as(ctypes.c_void_p), T,
             _lib.CONTRACT_BF16X3 | flags, ptr(b), ptr(ws), ws.numel(), stream_ptr())
        torch.cuda.synchronize()
        assert int(ws[:4].view(torch.int32).item()) == 0
        out[flags] = b.cpu().numpy()
    F = fields.double()
    ref = np.array([float((F[i] * F[j] * F[l]).sum()) for i, j, l in slots.T[::97]])
    ab = np.array([float((F[i] * F[j] * F[l]).abs().sum()) for i, j, l in slots.T[::97]])
    for flags, b in out.items():
        assert np.max(np.abs(b[::97] - ref) / ab) < 3e-6, flags
    # the FP32 method takes no plan flag
    ws = torch.zeros(lib.pyspec_bk_contract_workspace(n, nmax, T, 0), dtype=torch.uint8, device="cuda")
    b = torch.zeros(T, dtype=torch.float64, device="cuda")
    assert lib.pyspec_bk_contract(ptr(fields), n, nmax, ptr(tri_d), slots.ctypes.data_as(ctypes.c_void_p), T,
                                  _lib.CONTRACT_RUN_PLAN, ptr(b), ptr(ws), ws.numel(), stream_ptr()) == -1


def test_tuner_caches_choices(tmp_path, monkeypatch):
    from pyspectrum_gb300 import core, tune
    monkeypatch.setenv("PYSPEC_GB300_CACHE", str(tmp_path))
    monkeypatch.setattr(tune, "_mem", {})
    monkeypatch.setattr(tune, "_loaded", False)
    n, L = 64, 1000.0
    rng = np.random.default_rng(2)
    x = torch.from_numpy(rng.uniform(0, L, (3, 300_000))).cuda()
    xyzs, ws = core.prepare_positions(x, L)
    h1 = core.fft_periodic_half(xyzs, ws, n, L, 300_000.0).clone()
    with open(tmp_path / "tune.json") as f:
        saved = json.load(f)
    kinds = sorted(k.split("|")[0] for k in saved)
    assert kinds == ["assign", "fft3d"]
    for k, v in saved.items():
        # 64^3 has one FFT form (Stockham); the assignment has four candidates
        assert len(v["ms"]) >= (4 if k.startswith("assign") else 1) and str(v["choice"]) in v["ms"]
    # a second call reuses the choices (no new keys) and gives the same delta(k)
    h2 = core.fft_periodic_half(xyzs, ws, n, L, 300_000.0)
    with open(tmp_path / "tune.json") as f:
        assert json.load(f) == saved
    torch.testing.assert_close(h1, h2, rtol=0, atol=1e-6 * float(h1.abs().max()))
    # switched off: the fixed defaults, same delta(k)
    monkeypatch.setenv("PYSPEC_GB300_TUNE", "0")
    h3 = core.fft_periodic_half(xyzs, ws, n, L, 300_000.0)
    torch.testing.assert_close(h1, h3, rtol=0, atol=1e-6 * float(h1.abs().max()))
