"""Many boxes per call (Bk_periodic_batch): the same results as one
Bk_periodic call per box, with the per-geometry stages replayed from a CUDA
graph after the first box of each grid size."""
import numpy as np
import pytest

from pyspectrum_gb300 import batch
from pyspectrum_gb300 import pyspectrum as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["fp32", "bf16x3"])
def test_batch_matches_single_calls(method):
    L, step, ncut, nmax = 1000.0, 2, 2, 12
    rng = np.random.default_rng(5)
    mocks = []
    for k, n in enumerate((32, 48, 32, 48, 32, 48)):
        npart = int(rng.integers(20_000, 60_000))
        centres = rng.uniform(0, L, size=(3, 200))
        xyz = (centres[:, rng.integers(0, 200, npart)] + rng.normal(0, 20.0, size=(3, npart))) % L
        mocks.append((xyz, n))
    runner = batch.BkBatch(Lbox=L, step=step, Ncut=ncut, Nmax=nmax, method=method, graphs=True)
    got = runner.run(mocks)
    assert runner.geometry(32).graph is not None and runner.geometry(48).graph is not None
    for (xyz, n), g in zip(mocks, got):
        ref = P.Bk_periodic(xyz, Lbox=L, Ngrid=n, step=step, Ncut=ncut, Nmax=nmax, method=method)
        for k in ("i_k1", "i_k2", "i_k3", "counts"):
            np.testing.assert_array_equal(g[k], ref[k])
        assert g["meta"]["N"] == ref["meta"]["N"] and g["meta"]["Ngrid"] == n
        # float atomics in the assignment make repeated runs differ at ~1e-7;
        # compare the raw (pre-shot-noise) power, a small difference otherwise
        sn = ref["p0k_sn"]
        np.testing.assert_allclose(g["p0k1"] + sn, ref["p0k1"] + sn, rtol=1e-5)
        np.testing.assert_allclose(g["b123_sn"], ref["b123_sn"], rtol=1e-5)
        tot_g, tot_r = g["b123"] + g["b123_sn"], ref["b123"] + ref["b123_sn"]
        np.testing.assert_allclose(tot_g, tot_r, rtol=1e-5, atol=1e-5 * np.abs(tot_r).max())
    # a second pass replays the graphs and reproduces the first
    again = runner.run(mocks[:2])
    for a, b in zip(again, got[:2]):
        np.testing.assert_allclose(a["b123"] + a["b123_sn"], b["b123"] + b["b123_sn"], rtol=1e-5,
                                   atol=1e-5 * np.abs(b["b123"] + b["b123_sn"]).max())


def test_batch_accepts_device_and_weighted_inputs():
    import torch
    L, n = 1000.0, 32
    rng = np.random.default_rng(8)
    xyz = rng.uniform(0, L, size=(3, 30_000))
    w = rng.uniform(0.5, 1.5, size=30_000)
    out = P.Bk_periodic_batch([(torch.as_tensor(xyz, device="cuda"), n), (xyz, n, w)], Lbox=L, step=2, Ncut=2,
                              Nmax=8, method="fp32")
    ref0 = P.Bk_periodic(xyz, Lbox=L, Ngrid=n, step=2, Ncut=2, Nmax=8)
    ref1 = P.Bk_periodic(xyz, w=w, Lbox=L, Ngrid=n, step=2, Ncut=2, Nmax=8)
    for g, r in ((out[0], ref0), (out[1], ref1)):
        np.testing.assert_allclose(g["b123"] + g["b123_sn"], r["b123"] + r["b123_sn"], rtol=1e-5,
                                   atol=1e-5 * np.abs(r["b123"] + r["b123_sn"]).max())
        assert g["meta"]["nbar"] == pytest.approx(r["meta"]["nbar"])
