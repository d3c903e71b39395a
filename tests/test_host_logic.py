"""Host-side logic of the package (no GPU)."""
import numpy as np

from oracle import pyspec_oracle as O
from pyspectrum_gb300 import core, util


def test_triangle_table_matches_reference_loop():
    for jmin, nmax in [(1, 5), (1, 40), (2, 7), (1, 60)]:
        t = core.triangles(jmin, nmax)
        ref = np.array([(i, j, l) for i, j, l, _ in O.triangles(jmin, nmax)]).T
        assert np.array_equal(t, ref)
    assert core.triangles(1, 40).shape[1] == 6350
    assert core.triangles(1, 60).shape[1] == 20275
    assert core.triangles(1, 50).shape[1] == 12000


def test_rsd_factor_and_applyrsd(golden):
    g = golden("ref_rsd.npz")
    for los in "xyz":
        out = util.applyRSD(g["xyz"], g["vxyz"], 0.5, h=0.7, omega0_m=0.3, LOS=los, Lbox=2600.0)
        np.testing.assert_allclose(out, g["rsd_" + los], rtol=0, atol=1e-9)
    assert abs(core.rsd_factor(0.5, 0.3) - 1.5 / (100 * np.sqrt(0.3 * 1.5 ** 3 + 0.7))) < 1e-15


def test_ijl_order_groups_by_l_then_j():
    i = np.array([3, 2, 2, 1]); j = np.array([1, 2, 1, 1]); l = np.array([1, 1, 1, 1])
    order = util.ijl_order(i, j, l).ravel()
    assert list(order) == [3, 2, 0, 1]


def test_counts_cache_path_naming(tmp_path, monkeypatch):
    monkeypatch.setenv("PYSPEC_GB300_CACHE", str(tmp_path))
    p = core.counts_path(360, 40, 3, 3)
    assert p.startswith(str(tmp_path)) and "Ngrid360.Nmax40.Ncut3.step3" in p


def _plan_with_status(word, method="bf16x3"):
    """A BkPlan whose buffers are host tensors, with its contraction status
    word preset (BkPlan.result only reads these on the host)."""
    import torch
    p = object.__new__(core.BkPlan)
    p.method, p.step = method, 3
    p.tri_np = core.triangles(1, 3)
    p.counts_np = np.ones(p.tri_np.shape[1], dtype=np.int64)
    p.out = torch.zeros((7, p.tri_np.shape[1]), dtype=torch.float64)
    p.ws_con = torch.zeros(256, dtype=torch.uint8)
    p.ws_con[:4].view(torch.int32)[0] = word
    return p


def test_timed_out_contraction_raises():
    import pytest
    core.check_contract_status(0)
    for word in (1, 2, 3, 4, 5, 77):
        with pytest.raises(core.ContractTimeout, match=f"status {word}"):
            core.check_contract_status(word)
    # the result of a plan whose tensor-core contraction stopped early is refused
    with pytest.raises(core.ContractTimeout):
        _plan_with_status(3).result(True)
    T = core.triangles(1, 3).shape[1]
    assert _plan_with_status(0).result(True)["b123"].shape == (T,)
    # the FP32 method has no status word: its workspace bytes are not read
    assert _plan_with_status(3, method="fp32").result(False)["b123"].shape == (T,)
