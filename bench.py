#!/usr/bin/env python
"""Benchmark of the periodic-box bispectrum path on GB300.

One step = one Bk_periodic evaluation of the 360^3 / step 3 / Nmax 40
workload (1,000,000 Zel'dovich particles, L = 2500 Mpc/h): positions ->
PCS+interlaced assignment -> 3D FFT -> interlacing combine -> 40 shell fields
-> 6350-triangle contraction -> normalisation and shot noise.

`value` is Bk evaluations per second with the split-BF16 tensor-core
contraction and the inputs resident in HBM; the plain FP32 CUDA-core form is
timed on the same inputs and reported under "methods".  `e2e` times the public
API (pyspectrum_gb300.pyspectrum.Bk_periodic) from pinned host positions to
the host result dictionary.  `cpu_baseline` times the CPU restatement of the
reference on a bounded sample of the same workload (see --impl reference).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun (N > 1) every rank runs an independent replica ("replicas
only": the path does not shard).
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Bk evals/sec & triangles/sec at Ngrid=360 (split-BF16 TC vs plain FP32, FP64-err)"
UNIT = "Bk evals/s"
WORKLOAD = {"workload": "zeldovich-1M-360-step3-nmax40", "npart": 1_000_000, "Lbox": 2500.0, "Ngrid": 360,
            "step": 3, "Ncut": 3, "Nmax": 40, "triangles": 6350, "shells": 40,
            "field": "GRF P(k)~k^-1.5 on 360^3, rms displacement 5 Mpc/h, lattice 100^3 with random offsets",
            "seed": 2}
# a reduced case of the same kernels for ncu captures (fields 283 MB, still > L2);
# its line is not a bench result
SMALL_WORKLOAD = {"workload": "zeldovich-300k-192-step3-nmax40 (profiling case)", "npart": 300_000,
                  "Lbox": 1500.0, "Ngrid": 192, "step": 3, "Ncut": 3, "Nmax": 40, "triangles": 6350, "shells": 40,
                  "field": "GRF P(k)~k^-1.5 on 192^3, rms displacement 5 Mpc/h", "seed": 2}
L2_FLUSH_BYTES = 512 << 20   # > 129 MB L2, written between timed steps


def max_over_ranks(x, device=None):
    """The slowest rank's value of x (max over the ranks of the process group);
    x itself when no group of more than one rank is running.  device: where
    the reduction tensor lives (cuda for NCCL, cpu for gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, seconds_max):
    """Whole-job throughput of `world` independent replicas: the units all
    ranks processed over the slowest rank's time."""
    return world * units_per_rank / seconds_max


def plan_macs_per_voxel(nmax, ncut, step):
    """Tensor-core multiply-adds per voxel of the contraction plan for the
    triangle loop (host-side plan query of the library)."""
    from pyspectrum_gb300 import _lib, core as _core
    jmin = ncut // step
    tri = np.ascontiguousarray(_core.triangles(jmin, nmax) - jmin, dtype=np.int32)
    info = np.zeros(7, dtype=np.int64)
    _lib.call("pyspec_bk_plan_check", nmax - jmin + 1, tri.ctypes.data, int(tri.shape[1]), info.ctypes.data, 7)
    return int(info[6])


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# ---------------------------------------------------------------------------
# CPU reference arm: the oracle port of the reference's CPU path, timed on a
# bounded sample of the same workload and extrapolated to one Bk evaluation.
# ---------------------------------------------------------------------------
def cpu_reference_sample(xyz_np, n_shell_sample=4, n_tri_sample=24):
    """Reference-structured CPU pipeline (pyspectrum.py:285-457 with the
    Fortran parts restated): assignment (C, one core), complex64 FFT (scipy,
    all cores, like threaded FFTW), interlacing combine, reflection, then a
    sample of shell FFTs and triangle einsums, extrapolated to 40 shells and
    6350 triangles.  Returns (seconds per Bk evaluation, details)."""
    import scipy.fft as sfft
    from oracle import pyspec_oracle as O
    cores = os.cpu_count() or 1
    W = WORKLOAD
    n, L, step = W["Ngrid"], W["Lbox"], W["step"]
    t0 = time.perf_counter()
    xyzs = O.clip_positions(xyz_np, L)
    g = O.assign_quad(xyzs, np.ones(xyz_np.shape[1], np.float32), np.float32(n / L), 0.0, n)
    t_assign = time.perf_counter() - t0
    t0 = time.perf_counter()
    G = sfft.ifftn(g.astype(np.complex64), workers=cores) * np.float32(n ** 3)
    t_fft = time.perf_counter() - t0
    t0 = time.perf_counter()
    half = O.fcomb_periodic(G, float(xyz_np.shape[1]))
    full = O.reflect_delta(half, n).astype(np.complex64)
    t_fcomb = time.perf_counter() - t0
    del g, G
    irk = O.shell_index(n, step)
    shells = {}
    t0 = time.perf_counter()
    for j in range(1, n_shell_sample + 1):
        tmp = np.where(irk == j, full, np.complex64(0))
        F = np.real(sfft.fftn(tmp, workers=cores)).astype(np.float64)
        _ = np.einsum("i,i", F.ravel(), F.ravel())
        shells[j] = F
    t_shell = (time.perf_counter() - t0) / n_shell_sample
    tri = [(i, j, l) for i in range(1, 5) for j in range(1, i + 1) for l in range(max(i - j, 1), j + 1)]
    tri = (tri * ((n_tri_sample // len(tri)) + 1))[:n_tri_sample]
    t0 = time.perf_counter()
    for i, j, l in tri:
        _ = np.einsum("i,i,i", shells[i].ravel(), shells[j].ravel(), shells[l].ravel())
    t_tri = (time.perf_counter() - t0) / n_tri_sample
    total = t_assign + t_fft + t_fcomb + W["shells"] * t_shell + W["triangles"] * t_tri
    det = {"assign_s": t_assign, "fft_s": t_fft, "fcomb_reflect_s": t_fcomb, "per_shell_s": t_shell,
           "per_triangle_s": t_tri, "extrapolated_s_per_eval": total}
    sample = (f"full FFT_periodic (1M particles, 360^3) + {n_shell_sample} of 40 shell FFTs + {n_tri_sample} of "
              f"6350 triangle einsums, extrapolated; FFTs on {cores} threads, assignment and einsums on 1 "
              f"thread as in the reference")
    return total, det, sample, cores


def make_positions_np(seed):
    """Same particles as the GPU arm, generated on the GPU when available."""
    import torch
    from pyspectrum_gb300 import mocks
    W = WORKLOAD
    if torch.cuda.is_available():
        x = mocks.zeldovich_mock(W["npart"], W["Lbox"], ngrid=W["Ngrid"], seed=seed)
        return x, x.cpu().numpy()
    raise RuntimeError("the workload generator runs on the GPU")


def run_reference(args, rank, world):
    if rank != 0:
        return
    import torch
    _, xyz_np = make_positions_np(WORKLOAD["seed"])
    torch.cuda.synchronize()
    per = []
    det = sample = cores = None
    for _ in range(max(1, args.steps)):
        total, det, sample, cores = cpu_reference_sample(xyz_np)
        per.append(total)
    sec = float(np.mean(per))
    value = 1.0 / sec
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64/c64 (CPU)", "data": "synthetic",
            "config": WORKLOAD,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                             "stages": det},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = f"/tmp/pyspec_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "20"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return self
        # wait until nvidia-smi is sampling, then count only the samples taken
        # from here on (the timed region starts when this returns)
        self.skip = 0
        t0 = time.time()
        while time.time() - t0 < 10.0:
            self.fh.flush()
            with open(self.path) as f:
                n = sum(1 for _ in f)
            if n > 0:
                self.skip = n
                break
            time.sleep(0.01)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for k, line in enumerate(open(self.path)):
            if k < getattr(self, "skip", 0):
                continue
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


FP64_SHELLS = (1, 2, 3, 5, 8, 13, 20, 27, 34, 40)


def fp64_error(half, plans):
    """Error of both contraction forms against float64 sums on the bench box:
    the shell fields of FP64_SHELLS rebuilt from the same delta(k) with
    complex128 FFTs (scipy, all host cores) and the triangles among those
    shells summed in float64.  Reports, per form, the median and maximum
    |dB/B|, the maximum over triangles with condition number
    sum|F_iF_jF_l| / |sum F_iF_jF_l| < 1e3, and the maximum error normalised by
    sum|F_iF_jF_l|."""
    import scipy.fft as sfft
    import torch
    from pyspectrum_gb300 import core
    t0 = time.perf_counter()
    bsums = {}
    for name, pl in plans.items():          # both forms from this same delta(k)
        pl.shells(half)
        pl.contract()
        bsums[name] = pl.bsum.cpu().numpy()
    plan = plans["bf16x3"]
    n, step = plan.n, plan.step
    delta = core.reflect_half(half).cpu().numpy().astype(np.complex128)
    torch.cuda.empty_cache()
    a = np.minimum(np.arange(n), n - np.arange(n)).astype(np.int64)
    d2 = a[:, None, None] ** 2 + a[None, :, None] ** 2 + a[None, None, :] ** 2
    irk = np.floor(np.sqrt(d2.astype(np.float64)) / step + 0.5).astype(np.int64)
    irk -= ((2 * irk - 1) ** 2 * step * step > 4 * d2) & (irk > 0)        # exact integer shell rule
    irk += (2 * irk + 1) ** 2 * step * step <= 4 * d2
    F = {j: np.real(sfft.fftn(np.where(irk == j, delta, 0), workers=-1)).ravel() for j in FP64_SHELLS}
    del delta, irk, d2
    loop = plan.tri_np
    sel = [t for t in range(loop.shape[1]) if all(int(v) in F for v in loop[:, t])]
    exact = np.empty(len(sel))
    absum = np.empty(len(sel))
    for k, t in enumerate(sel):
        prod = F[int(loop[0, t])] * F[int(loop[1, t])] * F[int(loop[2, t])]
        exact[k], absum[k] = prod.sum(), np.abs(prod).sum()
    cond = absum / np.abs(exact)
    out = {"triangles": len(sel), "shells": list(FP64_SHELLS), "seconds": time.perf_counter() - t0}
    for name, b in bsums.items():
        err = np.abs(b[sel] - exact)
        rel = err / np.abs(exact)
        out[name] = {"median_rel": float(np.median(rel)), "max_rel": float(rel.max()),
                     "max_rel_cond_lt_1e3": float(rel[cond < 1e3].max()),
                     "normalised_max": float((err / absum).max())}
    return out


def run_gpu(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist
    from pyspectrum_gb300 import _lib, core
    from pyspectrum_gb300 import pyspectrum as P
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    W = WORKLOAD
    n, L, step, ncut, nmax = W["Ngrid"], W["Lbox"], W["step"], W["Ncut"], W["Nmax"]
    x, xyz_np = make_positions_np(W["seed"])
    npart = x.shape[1]
    nbar = npart / L ** 3
    kf = 2 * np.pi / L
    grid = torch.zeros((n, n, n), dtype=torch.complex64, device=dev)
    half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    plans = {m: core.get_plan(n, step, ncut, nmax, m, dev) for m in ("bf16x3", "fp32")}

    def step_fn(plan, ev=None):
        if ev is not None:
            ev[0].record()
        xyzs, ws = core.prepare_positions(x, L)
        core.fft_periodic_half(xyzs, ws, n, L, float(npart), grid=grid, half=half)
        if ev is not None:
            ev[1].record()
        plan.shells(half)
        if ev is not None:
            ev[2].record()
        plan.contract()
        if ev is not None:
            ev[3].record()
        plan.normalize(True, nbar, kf)
        if ev is not None:
            ev[4].record()

    def barrier():
        if world > 1:
            dist.barrier()

    results = {}
    for method in ("bf16x3", "fp32"):
        plan = plans[method]
        steps = args.steps if method == "bf16x3" else max(1, min(args.steps, 5))
        for _ in range(args.warmup):
            step_fn(plan)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(steps)]
        l0 = _lib.launch_count()
        with ClockSampler(local_rank) as clk:
            for k in range(steps):
                step_fn(plan, evs[k])
                flush.zero_()                     # L2 flush between timed steps (not timed)
            torch.cuda.synchronize()
        barrier()
        launches = _lib.launch_count() - l0
        tot = [e[0].elapsed_time(e[4]) for e in evs]
        stage = {name: float(np.mean([e[a].elapsed_time(e[b]) for e in evs]))
                 for name, a, b in (("fft_periodic", 0, 1), ("shell_fields", 1, 2), ("contraction", 2, 3),
                                    ("normalize", 3, 4))}
        ms = max_over_ranks(float(np.sum(tot)), dev)
        results[method] = {"ms_per_step": ms / steps, "bk_evals_per_s": job_rate(world, steps, ms / 1e3),
                           "triangles_per_s": plan.T / (stage["contraction"] / 1e3), "stage_ms": stage,
                           "gpu_launches": launches, "steps": steps, "clocks": clk.summary()}
        if method == "bf16x3":
            results[method]["status_word"] = int(plan.ws_con[:4].view(torch.int32).item())

    # timing comparator for the 3D FFT (cuFFT through torch.fft): the same
    # unnormalised backward transform of the density grid, 5 repetitions each
    fftcmp = None
    try:
        gtest = torch.complex(torch.randn((n, n, n), device=dev), torch.randn((n, n, n), device=dev))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        _lib.call("pyspec_fft3d_c2c", _lib.ptr(gtest), n, 1, _lib.stream_ptr())
        torch.cuda.synchronize()
        e0.record()
        for _ in range(5):
            _lib.call("pyspec_fft3d_c2c", _lib.ptr(gtest), n, 1, _lib.stream_ptr())
        e1.record()
        torch.cuda.synchronize()
        ours = e0.elapsed_time(e1) / 5
        _ = torch.fft.ifftn(gtest, norm="forward")
        torch.cuda.synchronize()
        e0.record()
        for _ in range(5):
            _ = torch.fft.ifftn(gtest, norm="forward")
        e1.record()
        torch.cuda.synchronize()
        fftcmp = {"ours_ms": ours, "cufft_ms": e0.elapsed_time(e1) / 5,
                  "transform": f"complex64 {n}^3 backward, unnormalised (cuFFT via torch.fft.ifftn, out of place)"}
        del gtest
    except Exception as exc:          # the comparator is informational only
        fftcmp = {"error": str(exc)[:200]}

    # accuracy of the tensor-core form against the FP32 form on this workload
    step_fn(plans["bf16x3"])
    step_fn(plans["fp32"])
    torch.cuda.synchronize()
    b16, b32 = plans["bf16x3"].bsum.cpu().numpy(), plans["fp32"].bsum.cpu().numpy()
    rel = np.abs(b16 - b32) / np.abs(b32)
    fp64 = None if args.no_fp64_check else fp64_error(half, plans)

    # end to end through the public API: pinned host positions in, host dict out
    import torch as _t
    xyz_pinned = _t.from_numpy(xyz_np).pin_memory()
    for _ in range(2):
        P.Bk_periodic(xyz_pinned, Lbox=L, Ngrid=n, step=step, Ncut=ncut, Nmax=nmax, method="bf16x3", device=dev)
    torch.cuda.synchronize()
    barrier()
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        out = P.Bk_periodic(xyz_pinned, Lbox=L, Ngrid=n, step=step, Ncut=ncut, Nmax=nmax, method="bf16x3",
                            device=dev)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dev)
    h2d = xyz_np.nbytes
    d2h = 7 * plans["bf16x3"].T * 8

    if rank != 0:
        return
    hbm, bf16, kind = _peaks()
    main = results["bf16x3"]
    # roofline of the dominant kernel: the tensor-core contraction.  Algorithmic
    # work = 2 T V useful FLOP (one FMA per triangle and voxel); executed tensor
    # work = 2 FLOP x the plan's tensor multiply-adds per voxel (per 128-row
    # tile: 2 A parts (hi, lo) x 2N B columns (hi, lo)) x V, from the plan the
    # library builds for this triangle list.
    V = n ** 3
    useful = 2.0 * plans["bf16x3"].T * V
    executed = 2.0 * plan_macs_per_voxel(nmax, ncut, step) * V
    t_con = main["stage_ms"]["contraction"] / 1e3
    roofline = {"kernel": "contract_tc_kernel (+ partial reduction)", "bound": "tensor",
                "achieved": useful / t_con / 1e12, "peak": bf16, "unit": "TFLOP/s",
                "frac": useful / t_con / 1e12 / bf16, "peak_kind": kind,
                "executed_tflops": executed / t_con / 1e12, "executed_frac": executed / t_con / 1e12 / bf16,
                "useful_over_executed": useful / executed,
                "traffic": 4.0 * 40 * V, "traffic_note": "dram bytes of one launch: the ncu capture at 192^3 "
                "(1.133 GB read) scaled by the voxel count; equal to the algorithmic bytes (fields read once)"}
    cpu = None
    if not args.no_cpu_baseline:
        total, det, sample, cores = cpu_reference_sample(xyz_np)
        cpu = {"value": 1.0 / total, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
               "stages": det}
    line = {"metric": METRIC, "value": main["bk_evals_per_s"], "unit": UNIT, "n_gpus": world,
            "steps": main["steps"], "warmup": args.warmup, "ms_per_step": main["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 (f32 fields, f64 sums)",
            "data": "synthetic (seeded Zel'dovich mock)",
            "config": dict(WORKLOAD, l2="flushed between steps (512 MB write); inputs 7.5 GB of fields per step"),
            "triangles_per_s": main["triangles_per_s"],
            "methods": results,
            "tc_over_fp32": results["fp32"]["ms_per_step"] / main["ms_per_step"],
            "tc_over_fp32_contraction": results["fp32"]["stage_ms"]["contraction"] / main["stage_ms"]["contraction"],
            "fp64_error": fp64,
            "bf16x3_vs_fp32_rel": {"median": float(np.median(rel)), "p99": float(np.percentile(rel, 99)),
                                   "max": float(rel.max())},
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": job_rate(world, e2e_steps, e2e_s), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "api": "pyspectrum_gb300.pyspectrum.Bk_periodic(pinned xyz)"},
            "gpu_launches": main["gpu_launches"], "clocks": main["clocks"], "fft3d_comparator": fftcmp}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """Many boxes per call (Bk_periodic_batch): 64 seeded Zel'dovich mocks with
    particle counts uniform in [0.5M, 4M] and grids mixed over {192, 256, 360}
    (L = 2500, step 3, Nmax 40, split-BF16).  Prints one JSON line with the
    batch time (positions already in pinned host memory; results back on the
    host); not the headline bench line."""
    import torch
    from pyspectrum_gb300 import batch, mocks
    rng = np.random.default_rng(4)
    L = 2500.0
    nmock = 64
    grids = rng.choice([192, 256, 360], size=nmock)
    nparts = rng.integers(500_000, 4_000_001, size=nmock)
    cat = []
    for k in range(nmock):
        x = mocks.zeldovich_mock(int(nparts[k]), L, ngrid=int(grids[k]), seed=100 + k)
        cat.append((torch.from_numpy(x.cpu().numpy()).pin_memory(), int(grids[k])))
        del x
    runner = batch.BkBatch(Lbox=L, step=3, Ncut=3, Nmax=40, method="bf16x3", graphs=True)
    # first pass: plans, counts and graph capture for the three geometries
    warm = [cat[int(np.nonzero(grids == g)[0][0])] for g in (192, 256, 360) for _ in range(2)]
    runner.run(warm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = runner.run(cat)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert len(out) == nmock and all(np.isfinite(o["b123"]).all() for o in out)
    line = {"workload": "64 Zel'dovich mocks, Np in [0.5M, 4M], Ngrid in {192, 256, 360}, L 2500, step 3, Nmax 40",
            "metric": "Bk evals/s (batch, host positions in, host results out)", "value": nmock / dt,
            "seconds": dt, "mocks_per_grid": {str(g): int((grids == g).sum()) for g in (192, 256, 360)},
            "particles_total": int(nparts.sum()), "method": "bf16x3", "graphs": True}
    print(json.dumps(line), flush=True)


def run_profile_shells(jtop):
    """Profiling case for the shell passes: shells jtop-2..jtop of the bench
    workload's delta(k) at 360^3 (about 1 GB on the device), three calls.
    Prints the time of the last call; not a bench result."""
    import torch
    from pyspectrum_gb300 import _lib, core
    from pyspectrum_gb300._lib import call, ptr, stream_ptr
    W = WORKLOAD
    n, L, step = W["Ngrid"], W["Lbox"], W["step"]
    x, _ = make_positions_np(W["seed"])
    xyzs, ws = core.prepare_positions(x, L)
    half = core.fft_periodic_half(xyzs, ws, n, L, float(x.shape[1]))
    del x, xyzs, ws
    jmin, nmax = jtop - 2, jtop
    S = nmax - jmin + 1
    fields = torch.empty((S, n ** 3), dtype=torch.float32, device=half.device)
    p0 = torch.empty(S, dtype=torch.float64, device=half.device)
    wsb = torch.empty(_lib.load().pyspec_shell_fields_workspace(n, S), dtype=torch.uint8, device=half.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        e0.record()
        call("pyspec_shell_fields", ptr(half), n, step, jmin, nmax, ptr(fields), ptr(p0), ptr(wsb), wsb.numel(),
             stream_ptr())
        e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"profile": "shell_fields", "Ngrid": n, "shells": [jmin, nmax],
                      "ms_last_call": e0.elapsed_time(e1)}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true", help="skip the float64 error check (about 30 s of CPU)")
    ap.add_argument("--small", action="store_true", help="run the 192^3 profiling case instead of the bench workload")
    ap.add_argument("--batch", action="store_true",
                    help="time 64 mixed-size mocks through Bk_periodic_batch instead of the bench workload")
    ap.add_argument("--profile-shells", type=int, default=0, metavar="J",
                    help="only run shells J-2..J of the bench workload three times (ncu profiling case)")
    args = ap.parse_args()
    if args.profile_shells:
        run_profile_shells(args.profile_shells)
        return
    if args.batch:
        run_batch(args)
        return
    if args.small:
        WORKLOAD.clear()
        WORKLOAD.update(SMALL_WORKLOAD)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            import torch
            torch.cuda.set_device(local_rank)
            run_reference(args, rank, world)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    run_gpu(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
