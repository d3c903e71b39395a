"""GPU parity at the benchmark configurations, at their stated sizes.

* Uniform box (200,000 particles, L = 1000, 128^3, step 3, Ncut 3, Nmax 40):
  Bk_periodic and Pk_periodic against the float64 oracle run end to end from
  the same particles (assignment estimator.f:284-512, backward FFT
  pyspectrum.py:1060-1080, combine estimator.f:605-675, reflection
  :1134-1157, shells :387-404, triangles :415-445, units :341-356).  Shells
  38-40 hold no mode at 128^3, so only 4420 of the 6350 loop triangles have
  counts; the counts are exact integers.
* Zel'dovich box at 360^3 (1,000,000 particles, L = 2500, Nmax 40): both
  contraction forms against float64 sums over all 6350 triangles, from the
  device's own delta(k) (the contraction's error) and from the oracle's
  float64 delta(k) of the same particles (end to end).
* Redshift-space Zel'dovich box at 360^3 (2,000,000 particles with linear
  velocities + 300 km/s dispersion, z = 0.5, Omega_m = 0.3, LOS z):
  Bk_periodic_rsd's B0/Q0 and P0/P2 against the oracle (applyRSD util.py:54-75,
  pk_pbox_rsd estimator.f:155-264).

Accuracy metrics (raw B before shot noise): |dB/B| over triangles with
condition number sum|F_iF_jF_l| / |sum F_iF_jF_l| < 1e3, the error normalised
by sum|F_iF_jF_l|, and the median; the float64 sums are oracle/torch_fp64.py.
Bounds: split-BF16 max |dB/B| <= 1e-5 over condition number < 1e3 and
normalised error <= 2e-7 for the contraction; FP32 tighter."""
import json
import os

import numpy as np
import pytest
import torch

from oracle import pyspec_oracle as O
from oracle import torch_fp64 as TF

pytestmark = pytest.mark.gpu

REPORT = {}


def _report(name, rep):
    REPORT[name] = rep
    print(name, json.dumps(rep))
    out = os.environ.get("PYSPEC_ACCURACY_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(REPORT, f, indent=1)


def _loop(jmin, nmax):
    tri = np.array([(i, j, l) for i, j, l, _ in O.triangles(jmin, nmax)], dtype=np.int64).T
    fac = np.array([f for *_, f in O.triangles(jmin, nmax)])
    return tri, fac


def _fp64_sums(half_zyx, step, jmin, nmax, tri):
    """float64 shell fields of a half grid [z, y, x] on the device, and the
    float64 triangle sums (raw and absolute) and sums of squares."""
    full = TF.reflect_half(half_zyx.to("cuda"))
    F, p0 = TF.shell_fields(full, step, jmin, nmax)
    del full
    bsum, absum = TF.triangle_sums(F, tri - jmin)
    p0 = p0.cpu().numpy()
    del F
    torch.cuda.empty_cache()
    return bsum, absum, p0


def _units(bsum, p0sum, counts, nk, tri, fac, n, L, step, jmin, nmax, wsum):
    """pyspectrum.py:404, :435-437 and :341-355 from raw sums, in float64."""
    V = float(n) ** 3
    p0k = np.zeros(nmax)
    with np.errstate(invalid="ignore", divide="ignore"):
        p0k[jmin - 1:nmax] = p0sum / V / nk[jmin:nmax + 1]
    keep = counts > 0
    i, j, l = (tri[k][keep] for k in range(3))
    b = bsum[keep] / (counts[keep] * V)
    nbar = wsum / L ** 3
    kf = 2 * np.pi / L
    p1, p2, p3 = (p0k[a - 1] * (2 * np.pi) ** 3 / kf ** 3 - 1.0 / nbar for a in (i, j, l))
    bsn = (p1 + p2 + p3) / nbar + 1.0 / nbar ** 2
    b = b * (2 * np.pi) ** 6 / kf ** 6 - bsn
    return {"i_k1": i * step, "i_k2": j * step, "i_k3": l * step, "p0k1": p1, "p0k2": p2, "p0k3": p3,
            "b123": b, "b123_sn": bsn, "q123": b / (p1 * p2 + p1 * p3 + p2 * p3),
            "counts": counts[keep] / fac[keep]}


def _fresh():
    from pyspectrum_gb300 import core
    core.release_plans()
    torch.cuda.empty_cache()


def test_config1_uniform_128_end_to_end():
    from pyspectrum_gb300 import core
    from pyspectrum_gb300 import pyspectrum as P
    n, L, step, ncut, nmax, npart = 128, 1000.0, 3, 3, 40, 200_000
    jmin = ncut // step
    rng = np.random.default_rng(1)
    xyz = rng.uniform(0.0, L, size=(3, npart))
    tri, fac = _loop(jmin, nmax)
    # exact counts: float64 shell-indicator fields (pyspectrum.py:976-1023)
    ind = torch.ones((n, n, n), dtype=torch.complex128, device="cuda")
    I, _ = TF.shell_fields(ind, step, jmin, nmax)
    craw, _ = TF.triangle_sums(I, tri - jmin, with_abs=False)
    del I, ind
    counts = np.rint(craw / float(n) ** 3).astype(np.int64)
    assert np.abs(craw / float(n) ** 3 - counts).max() < 1e-3      # float64 sums of ~1e11: integers to ~1e-5
    assert int((counts > 0).sum()) == 4420
    nk = O.mode_counts(n, step, nmax)
    assert nk[38:41].sum() == 0                         # shells 38-40 are empty at 128^3
    # the oracle, float64 from the particles
    half_o = O.FFT_periodic(xyz, Lbox=L, Ngrid=n)       # [x, y, z]
    half_zyx = torch.from_numpy(np.ascontiguousarray(half_o.transpose(2, 1, 0)))
    bsum, absum, p0sum = _fp64_sums(half_zyx, step, jmin, nmax, tri)
    ref = _units(bsum, p0sum, counts, nk, tri, fac, n, L, step, jmin, nmax, float(npart))
    keep = counts > 0
    # the device's own delta(k), for the error of the shells + contraction alone
    x_d = torch.from_numpy(xyz).cuda()
    xyzs, ws = core.prepare_positions(x_d, L)
    half_d = core.fft_periodic_half(xyzs, ws, n, L, float(npart)).clone()
    bsum_d, absum_d, _ = _fp64_sums(half_d, step, jmin, nmax, tri)
    _fresh()
    for method in ("fp32", "bf16x3", "bf16x3_fine", "bf16x6"):
        got = P.Bk_periodic(xyz, Lbox=L, Ngrid=n, step=step, Ncut=ncut, Nmax=nmax, method=method)
        plan = core.get_plan(n, step, ncut, nmax, method)
        np.testing.assert_array_equal(plan.counts_np, counts)
        np.testing.assert_array_equal(plan.nk_np, nk)
        for k in ("i_k1", "i_k2", "i_k3"):
            np.testing.assert_array_equal(got[k], ref[k])
        np.testing.assert_array_equal(got["counts"], ref["counts"])
        for k in ("p0k1", "p0k2", "p0k3", "b123", "q123", "counts", "b123_sn"):
            assert np.isfinite(got[k]).all(), k          # no NaN from the empty shells
        # end to end: the float32 delta(k) (single precision like the
        # reference's FFTW) against the float64 oracle
        raw = plan.bsum.cpu().numpy()[keep]
        rep = TF.error_report(raw, bsum[keep], absum[keep])
        rep["p0_max_rel"] = float(np.abs(plan.p0sum.cpu().numpy() - p0sum)[:37].max()
                                  / np.abs(p0sum[:37]).max())
        tot_g, tot_r = got["b123"] + got["b123_sn"], ref["b123"] + ref["b123_sn"]
        rel = np.abs(tot_g - tot_r) / np.abs(tot_r)
        cond = absum[keep] / np.abs(bsum[keep])
        rep["b0_total_max_rel_cond_lt_100"] = float(rel[cond < 100].max())
        # the shells + contraction alone, from the same delta(k)
        plan.run(half_d)
        con = TF.error_report(plan.bsum.cpu().numpy()[keep], bsum_d[keep], absum_d[keep])
        rep.update({"contraction_" + k: v for k, v in con.items()})
        _report(f"config1_{method}", rep)
        assert rep["p0_max_rel"] <= 1e-5
        # the float32 delta(k) floor; the mesh accumulates particles with float
        # atomics, so it moves from run to run (measured 1.5e-6 - 2.1e-6)
        assert rep["normalised_max"] <= 4e-6
        assert rep["b0_total_max_rel_cond_lt_100"] <= 1e-4
        np.testing.assert_allclose(got["p0k1"], ref["p0k1"], rtol=1e-5, atol=1e-5 * np.abs(ref["p0k1"]).max())
        # the shot-noise field of the uniform box is less forgiving than the
        # clustered 360^3 box (where split-BF16 stays below 1e-5 / 2e-7): here
        # the worst triangles of condition number ~1e3 reach 1.3e-5 with
        # either drain interval (measured 1.30e-5 / 1.24e-5), so the bound is 2e-5.
        # FP32: the mesh accumulates particles with float atomics, so delta(k)
        # -- and with it the worst triangle -- changes in its last bits from
        # run to run (measured 1.78e-6 and 2.36e-6 on two runs of one build)
        bound = {"fp32": (4e-6, 3e-8), "bf16x3": (2e-5, 3e-7), "bf16x3_fine": (2e-5, 1e-7),
                 "bf16x6": (1e-5, 1e-7)}[method]
        assert con["max_rel_cond_lt_1e3"] <= bound[0]
        assert con["normalised_max"] <= bound[1]
    pk = P.Pk_periodic(xyz, Lbox=L, Ngrid=n)
    pref = O.Pk_periodic(xyz, Lbox=L, Ngrid=n, delta_half=half_o)
    np.testing.assert_array_equal(pk["counts"], pref["counts"])
    np.testing.assert_allclose(pk["k"], pref["k"], rtol=1e-6)
    np.testing.assert_allclose(pk["p0k"] + pk["p0k_sn"], pref["p0k"] + pref["p0k_sn"], rtol=1e-5)
    _fresh()


def test_config2_all_triangles_fp64():
    from pyspectrum_gb300 import core, mocks
    n, L, step, ncut, nmax = 360, 2500.0, 3, 3, 40
    jmin = ncut // step
    x = mocks.zeldovich_mock(1_000_000, L, ngrid=n, seed=2)
    xyz_np = x.cpu().numpy()
    xyzs, ws = core.prepare_positions(x, L)
    half = core.fft_periodic_half(xyzs, ws, n, L, float(x.shape[1]))
    del xyzs, ws
    tri, fac = _loop(jmin, nmax)
    assert tri.shape[1] == 6350
    bsum, absum, p0sum = _fp64_sums(half, step, jmin, nmax, tri)
    got = {}
    for method in ("fp32", "bf16x3", "bf16x3_fine", "bf16x6"):
        plan = core.get_plan(n, step, ncut, nmax, method)
        plan.run(half)
        got[method] = plan.bsum.cpu().numpy()
        if method in core.TENSOR_METHODS:
            core.check_contract_status(plan.status_word().item())
        rep = TF.error_report(got[method], bsum, absum)
        rep["p0_max_rel"] = float(np.max(np.abs(plan.p0sum.cpu().numpy() - p0sum) / p0sum))
        _report(f"config2_contraction_{method}", rep)
    # end to end: float64 oracle delta(k) from the same particles
    half_o = O.FFT_periodic(xyz_np, Lbox=L, Ngrid=n)            # [x, y, z] complex128
    hz = np.ascontiguousarray(half_o.transpose(2, 1, 0))
    del half_o
    dh = half.cpu().numpy()
    d_rep = {"delta_max_abs_over_max": float(np.abs(dh - hz).max() / np.abs(hz).max()),
             "delta_rel_l2": float(np.linalg.norm(dh - hz) / np.linalg.norm(hz))}
    del dh
    _fresh()
    bsum_o, absum_o, _ = _fp64_sums(torch.from_numpy(hz), step, jmin, nmax, tri)
    del hz
    for method in ("fp32", "bf16x3", "bf16x3_fine", "bf16x6"):
        rep = TF.error_report(got[method], bsum_o, absum_o)
        rep.update(d_rep)
        _report(f"config2_end_to_end_{method}", rep)
    c2 = REPORT
    assert c2["config2_contraction_bf16x3"]["max_rel_cond_lt_1e3"] <= 1e-5
    assert c2["config2_contraction_bf16x3"]["normalised_max"] <= 2e-7
    assert c2["config2_contraction_bf16x3_fine"]["max_rel_cond_lt_1e3"] <= 1e-5
    assert c2["config2_contraction_bf16x3_fine"]["normalised_max"] <= 1e-7
    assert c2["config2_contraction_bf16x6"]["max_rel_cond_lt_1e3"] <= 1e-5
    assert c2["config2_contraction_bf16x6"]["normalised_max"] <= 1e-7
    assert c2["config2_contraction_fp32"]["max_rel_cond_lt_1e3"] <= 2e-6
    assert c2["config2_contraction_fp32"]["normalised_max"] <= 1e-8
    assert c2["config2_contraction_fp32"]["p0_max_rel"] <= 1e-5
    assert d_rep["delta_max_abs_over_max"] <= 1e-5
    for method in ("fp32", "bf16x3"):
        assert c2[f"config2_end_to_end_{method}"]["normalised_max"] <= 1e-6
    _fresh()


def test_config3_rsd_360_2M():
    from pyspectrum_gb300 import core, mocks
    from pyspectrum_gb300 import pyspectrum as P
    n, L, step, ncut, nmax, z, om = 360, 2500.0, 3, 3, 40, 0.5, 0.3
    jmin = ncut // step
    x, v = mocks.zeldovich_mock(2_000_000, L, ngrid=n, seed=3, velocities=True, redshift=z, omega_m=om)
    xyz_np, v_np = x.cpu().numpy(), v.cpu().numpy()
    got = P.Bk_periodic_rsd(x, v, z, h=0.7, omega0_m=om, LOS="z", Lbox=L, Ngrid=n, step=step, Ncut=ncut,
                            Nmax=nmax, Nmubin=10, method="bf16x3")
    plan = core.get_plan(n, step, ncut, nmax, "bf16x3")
    raw = plan.bsum.cpu().numpy()
    _fresh()
    xs = O.applyRSD(xyz_np, v_np, z, h=0.7, omega0_m=om, LOS="z", Lbox=L)
    half_o = O.FFT_periodic(xs, Lbox=L, Ngrid=n)
    pref = O.Pk_periodic_rsd(xs, Lbox=L, Ngrid=n, rsd=2, Nmubin=10, delta_half=half_o)
    pk = got["pk"]
    np.testing.assert_array_equal(pk["counts"], pref["counts"])
    np.testing.assert_array_equal(pk["counts_kmu"], pref["counts_kmu"])
    prep = {}
    for key in ("p0k", "p2k"):
        r = pref[key]
        prep[key + "_max_rel"] = float(np.max(np.abs(pk[key] - r) / np.abs(r).max()))
    tri, fac = _loop(jmin, nmax)
    hz = torch.from_numpy(np.ascontiguousarray(half_o.transpose(2, 1, 0)))
    del half_o
    bsum, absum, p0sum = _fp64_sums(hz, step, jmin, nmax, tri)
    counts = plan.counts_np
    nk = O.mode_counts(n, step, nmax)
    ref = _units(bsum, p0sum, counts, nk, tri, fac, n, L, step, jmin, nmax, float(xyz_np.shape[1]))
    rep = TF.error_report(raw, bsum, absum)
    rep.update(prep)
    tot_g, tot_r = got["b123"] + got["b123_sn"], ref["b123"] + ref["b123_sn"]
    rep["b0_total_max_rel"] = float(np.max(np.abs(tot_g - tot_r) / np.abs(tot_r)))
    rep["q0_max_abs"] = float(np.max(np.abs(got["q123"] - ref["q123"])))
    _report("config3_rsd_end_to_end_bf16x3", rep)
    for k in ("i_k1", "i_k2", "i_k3", "counts"):
        np.testing.assert_array_equal(got[k], ref[k])
    assert prep["p0k_max_rel"] <= 1e-5 and prep["p2k_max_rel"] <= 1e-5
    # end to end (float32 delta(k) like the reference's FFTW): the normalised
    # error and the relative error of triangles with condition number < 1e3;
    # the raw maximum sits on cancelling triangles (reported, not bounded)
    assert rep["normalised_max"] <= 1e-6
    assert rep["max_rel_cond_lt_1e3"] <= 5e-5
    _fresh()
