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
