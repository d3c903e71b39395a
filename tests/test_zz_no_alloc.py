"""The contraction entry point that allocates no device memory.

pyspec_bk_contract_noalloc serves callers that cannot allocate device memory
where they run (a framework's custom-call hook that only receives operands,
or code inside a stream capture).  It keeps its scratch in a fixed device
array; this test calls it through the C ABI twice in a row and checks both
results against the workspace-based pyspec_bk_contract (FP32 method).  It is
collected last on purpose, and also passes on its own in a fresh process."""
import ctypes

import numpy as np
import pytest
import torch

from pyspectrum_gb300 import core
from pyspectrum_gb300._lib import call, load, ptr, stream_ptr

pytestmark = pytest.mark.gpu


def _fields(n, S, seed):
    rng = np.random.default_rng(seed)
    return torch.from_numpy(rng.standard_normal((S, n ** 3)).astype(np.float32)).cuda()


@pytest.mark.parametrize("n,nmax", [(32, 12), (64, 40)])
def test_noalloc_matches_workspace_contraction(n, nmax):
    lib = load()
    S = nmax
    fields = _fields(n, S, seed=n)
    slots = np.ascontiguousarray(core.triangles(1, nmax) - 1, dtype=np.int32)
    T = slots.shape[1]
    tri_d = torch.from_numpy(slots).cuda()
    ref = torch.zeros(T, dtype=torch.float64, device="cuda")
    ws = torch.zeros(lib.pyspec_bk_contract_workspace(n, S, T, 0), dtype=torch.uint8, device="cuda")
    call("pyspec_bk_contract", ptr(fields), n, S, ptr(tri_d), slots.ctypes.data_as(ctypes.c_void_p), T, 0,
         ptr(ref), ptr(ws), ws.numel(), stream_ptr())
    refh = ref.cpu().numpy()
    scale = np.abs(refh).max()
    for _ in range(2):     # the shared scratch keeps the previous call's contents
        out = torch.full((T,), np.nan, dtype=torch.float64, device="cuda")
        call("pyspec_bk_contract_noalloc", ptr(fields), n, S, slots.ctypes.data_as(ctypes.c_void_p), T, ptr(out),
             stream_ptr())
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, refh, rtol=1e-12, atol=1e-12 * scale)


def test_noalloc_rejects_oversized_request():
    lib = load()
    n, S = 16, 120
    fields = _fields(n, S, seed=1)
    slots = np.ascontiguousarray(core.triangles(1, S) - 1, dtype=np.int32)
    out = torch.zeros(slots.shape[1], dtype=torch.float64, device="cuda")
    rc = lib.pyspec_bk_contract_noalloc(ptr(fields), n, S, slots.ctypes.data_as(ctypes.c_void_p), slots.shape[1],
                                        ptr(out), stream_ptr())
    assert rc == -1


def _list(nmax):
    return np.ascontiguousarray(core.triangles(1, nmax) - 1, dtype=np.int32)


def test_noalloc_call_allocates_no_device_memory():
    n, S = 32, 12
    fields = _fields(n, S, seed=5)
    slots = _list(S)
    out = torch.zeros(slots.shape[1], dtype=torch.float64, device="cuda")
    args = (ptr(fields), n, S, slots.ctypes.data_as(ctypes.c_void_p), slots.shape[1], ptr(out), stream_ptr())
    call("pyspec_bk_contract_noalloc", *args)      # first call: address lookup, plan, module load
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for _ in range(3):
        call("pyspec_bk_contract_noalloc", *args)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert torch.cuda.memory_allocated() == alloc0
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes across no-alloc calls"


def test_noalloc_inside_stream_capture():
    lib = load()
    n, S = 32, 12
    fields = _fields(n, S, seed=6)
    slots = _list(S)
    T = slots.shape[1]
    tri_d = torch.from_numpy(slots).cuda()
    ref = torch.zeros(T, dtype=torch.float64, device="cuda")
    ws = torch.zeros(lib.pyspec_bk_contract_workspace(n, S, T, 0), dtype=torch.uint8, device="cuda")
    call("pyspec_bk_contract", ptr(fields), n, S, ptr(tri_d), slots.ctypes.data_as(ctypes.c_void_p), T, 0,
         ptr(ref), ptr(ws), ws.numel(), stream_ptr())
    refh = ref.cpu().numpy()
    out = torch.full((T,), np.nan, dtype=torch.float64, device="cuda")
    # one call outside the capture plans this list and looks the array up
    call("pyspec_bk_contract_noalloc", ptr(fields), n, S, slots.ctypes.data_as(ctypes.c_void_p), T, ptr(out),
         stream_ptr())
    torch.cuda.synchronize()
    fresh = np.ascontiguousarray(slots[:, ::-1])   # the list reversed: never planned by this process
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            rc = lib.pyspec_bk_contract_noalloc(ptr(fields), n, S, slots.ctypes.data_as(ctypes.c_void_p), T,
                                                ptr(out), stream_ptr(s))
            rc_fresh = lib.pyspec_bk_contract_noalloc(ptr(fields), n, S, fresh.ctypes.data_as(ctypes.c_void_p),
                                                      fresh.shape[1], ptr(out), stream_ptr(s))
    torch.cuda.current_stream().wait_stream(s)
    assert rc == 0
    assert rc_fresh == -1            # planning inside the capture is refused, the capture stays valid
    scale = np.abs(refh).max()
    for _ in range(2):
        out.fill_(np.nan)
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), refh, rtol=1e-12, atol=1e-12 * scale)
