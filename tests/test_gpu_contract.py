"""GPU parity of the triangle contraction: FP32 CUDA-core and BF16x3 tensor-core
forms against a float64 sum over the same shell fields."""
import ctypes

import numpy as np
import pytest
import torch

from pyspectrum_gb300 import core
from pyspectrum_gb300._lib import call, load, ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _fields(n, step, jmin, nmax, seed):
    """Shell fields of a random delta(k) via the library's own shell kernel."""
    rng = np.random.default_rng(seed)
    full = np.fft.ifftn(rng.standard_normal((n, n, n)) + 0.3) * n ** 3
    half = np.ascontiguousarray(full[: n // 2 + 1].transpose(2, 1, 0)).astype(np.complex64)
    S = nmax - jmin + 1
    h = torch.from_numpy(half).cuda()
    fields = torch.empty((S, n ** 3), dtype=torch.float32, device="cuda")
    ws = torch.empty(load().pyspec_shell_fields_workspace(n, S), dtype=torch.uint8, device="cuda")
    call("pyspec_shell_fields", ptr(h), n, step, jmin, nmax, ptr(fields), None, ptr(ws), ws.numel(), stream_ptr())
    return fields


def _contract(fields, n, tri_slots, method):
    S = fields.shape[0]
    T = tri_slots.shape[1]
    tri_d = torch.from_numpy(tri_slots).cuda()
    bsum = torch.zeros(T, dtype=torch.float64, device="cuda")
    ws = torch.zeros(load().pyspec_bk_contract_workspace(n, S, T, method), dtype=torch.uint8, device="cuda")
    call("pyspec_bk_contract", ptr(fields), n, S, ptr(tri_d), tri_slots.ctypes.data_as(ctypes.c_void_p), T, method,
         ptr(bsum), ptr(ws), ws.numel(), stream_ptr())
    torch.cuda.synchronize()
    status = int(ws[:4].view(torch.int32).item()) if (method & 0xff) in (1, 2) else 0
    return bsum.cpu().numpy(), status


def _reference(fields, tri_slots):
    F = fields.double()
    out = np.zeros(tri_slots.shape[1]); mag = np.zeros(tri_slots.shape[1])
    for t in range(tri_slots.shape[1]):
        i, j, l = tri_slots[:, t]
        p = F[i] * F[j] * F[l]
        out[t] = p.sum().item(); mag[t] = p.abs().sum().item()
    return out, mag


@pytest.mark.parametrize("n,step,nmax", [(32, 1, 12), (48, 1, 40), (96, 3, 16), (40, 1, 60), (40, 1, 30)])
def test_contraction_fp32_and_bf16x3(n, step, nmax):
    jmin = 1
    fields = _fields(n, step, jmin, nmax, seed=n + nmax)
    tri = core.triangles(jmin, nmax)
    slots = np.ascontiguousarray(tri - jmin, dtype=np.int32)
    ref, mag = _reference(fields, slots)
    mag = np.maximum(mag, 1e-300)
    got32, _ = _contract(fields, n, slots, 0)
    err32 = np.abs(got32 - ref) / mag
    assert err32.max() < 1e-6, err32.max()
    got16, status = _contract(fields, n, slots, 1)
    assert status == 0
    err16 = np.abs(got16 - ref) / mag
    # hi+lo bf16 operands keep ~16 mantissa bits: error per term ~2^-16, normalised
    assert err16.max() < 3e-5, err16.max()
    assert np.median(err16) < 3e-6


def test_bf16x3_rejects_unsupported():
    n = 16
    fields = torch.zeros((70, n ** 3), dtype=torch.float32, device="cuda")
    slots = np.ascontiguousarray(core.triangles(1, 70) - 1, dtype=np.int32)
    lib = load()
    T = slots.shape[1]
    tri_d = torch.from_numpy(slots).cuda()
    bsum = torch.zeros(T, dtype=torch.float64, device="cuda")
    ws = torch.zeros(lib.pyspec_bk_contract_workspace(n, 70, T, 1), dtype=torch.uint8, device="cuda")
    rc = lib.pyspec_bk_contract(ptr(fields), n, 70, ptr(tri_d), slots.ctypes.data_as(ctypes.c_void_p), T, 1,
                                ptr(bsum), ptr(ws), ws.numel(), stream_ptr())
    assert rc == -3


def test_arbitrary_triangle_lists():
    """A shuffled subset of the loop's triangles, with the shells of each
    triangle in any order and gaps in each pair's column range: both planned
    methods against float64."""
    n, step, nmax, jmin = 48, 1, 24, 1
    fields = _fields(n, step, jmin, nmax, seed=7)
    tri = core.triangles(jmin, nmax) - jmin
    rng = np.random.default_rng(3)
    keep = rng.permutation(tri.shape[1])[: tri.shape[1] // 3]
    sub = tri[:, keep]
    for t in range(sub.shape[1]):
        sub[:, t] = sub[rng.permutation(3), t]
    slots = np.ascontiguousarray(sub, dtype=np.int32)
    ref, mag = _reference(fields, slots)
    mag = np.maximum(mag, 1e-300)
    for method, tol in ((0, 1e-6), (1, 3e-5)):
        got, status = _contract(fields, n, slots, method)
        assert status == 0
        assert (np.abs(got - ref) / mag).max() < tol, method


@pytest.mark.parametrize("n,nmax", [(30, 12), (50, 30), (18, 12)])
def test_chunk_tails(n, nmax):
    """Voxel counts that are not a multiple of 64 (N = 30, 50, 18: the last
    64-voxel chunk is partly past the end and the copies fill it with zeros;
    N = 50, Nmax 30 also has empty shells past the Nyquist shell) and grids
    with fewer chunks than CTAs (N = 18, 30): the 64- and 32-voxel
    tensor-core forms and the FP32 form (128-voxel chunks, the last one
    partial at all three sizes) against float64."""
    jmin = 1
    fields = _fields(n, 1, jmin, nmax, seed=n)
    slots = np.ascontiguousarray(core.triangles(jmin, nmax) - jmin, dtype=np.int32)
    info = np.zeros(9, dtype=np.int64)
    call("pyspec_bk_plan_check", nmax, slots.ctypes.data_as(ctypes.c_void_p), slots.shape[1],
         info.ctypes.data_as(ctypes.c_void_p), 9)
    assert info[8] == 64
    ref, mag = _reference(fields, slots)
    mag = np.maximum(mag, 1e-300)
    for flags in (0, 0x400):                 # 64-voxel chunks, then PYSPEC_CONTRACT_KC32
        got, status = _contract(fields, n, slots, 1 | flags)
        assert status == 0
        err = np.abs(got - ref) / mag
        assert err.max() < 3e-5 and np.median(err) < 3e-6, flags
    got32, _ = _contract(fields, n, slots, 0)
    assert (np.abs(got32 - ref) / mag).max() < 1e-6


def test_cover_plan_narrow_three_tiles():
    """The Nmax 40 loop moved to shells 7..46 of 48: its pair cover still fits
    3 tiles, but columns up to 46 exceed the wide form's TMEM budget, so the
    3-tile narrow form (three MMAs per tile and k-step) runs."""
    n, step, nmax, jmin = 64, 1, 48, 1
    fields = _fields(n, step, jmin, nmax, seed=11)
    slots = np.ascontiguousarray(core.triangles(1, 40) - 1 + 7, dtype=np.int32)
    info = np.zeros(8, dtype=np.int64)
    call("pyspec_bk_plan_check", nmax, slots.ctypes.data_as(ctypes.c_void_p), slots.shape[1],
         info.ctypes.data_as(ctypes.c_void_p), 8)
    assert info[1] == 3 and info[2] == 1 and info[5] == 0   # 3 tiles, pair cover, narrow form
    ref, mag = _reference(fields, slots)
    mag = np.maximum(mag, 1e-300)
    got, status = _contract(fields, n, slots, 1)
    assert status == 0
    err = np.abs(got - ref) / mag
    assert err.max() < 3e-5 and np.median(err) < 3e-6


@pytest.mark.parametrize("method", [0, 1])
def test_repeated_triangle_rejected(method):
    n = 16
    fields = torch.zeros((8, n ** 3), dtype=torch.float32, device="cuda")
    slots = np.ascontiguousarray(core.triangles(1, 8) - 1, dtype=np.int32)
    slots = np.ascontiguousarray(np.concatenate([slots, slots[:, 5:6][[2, 0, 1]]], axis=1))
    lib = load()
    T = slots.shape[1]
    tri_d = torch.from_numpy(slots).cuda()
    bsum = torch.zeros(T, dtype=torch.float64, device="cuda")
    ws = torch.zeros(lib.pyspec_bk_contract_workspace(n, 8, T, method), dtype=torch.uint8, device="cuda")
    rc = lib.pyspec_bk_contract(ptr(fields), n, 8, ptr(tri_d), slots.ctypes.data_as(ctypes.c_void_p), T, method,
                                ptr(bsum), ptr(ws), ws.numel(), stream_ptr())
    assert rc == -1


@pytest.mark.parametrize("n,step,nmax", [(48, 1, 40), (40, 1, 60)])
def test_six_product_form_against_float64(n, step, nmax):
    """PYSPEC_CONTRACT_BF16X6 (the split-BF16 sums drained every 8 chunks plus
    a residual pass with the operands' third bf16 parts) on the pair-cover
    plan (Nmax 40, wide first pass) and a run plan (Nmax 60, narrow first
    pass): its error, normalised by sum |F_i F_j F_l|, is well below the
    three-product form's and near the FP32 form's."""
    jmin = 1
    fields = _fields(n, step, jmin, nmax, seed=7 * n + nmax)
    slots = np.ascontiguousarray(core.triangles(jmin, nmax) - jmin, dtype=np.int32)
    ref, mag = _reference(fields, slots)
    mag = np.maximum(mag, 1e-300)
    live = mag > 1e-300                      # triangles whose shells hold modes on this grid
    err = {}
    for name, method in (("fp32", 0), ("bf16x3", 1), ("bf16x6", 2)):
        got, status = _contract(fields, n, slots, method)
        assert status == 0
        err[name] = (np.abs(got - ref) / mag)[live]
    print({k: (float(np.median(v)), float(v.max())) for k, v in err.items()})
    assert err["bf16x6"].max() < 0.5 * err["bf16x3"].max()
    assert err["bf16x6"].max() < 5e-7
    assert np.median(err["bf16x6"]) < 0.25 * np.median(err["bf16x3"])
