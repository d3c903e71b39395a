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
the host result dictionary.  `cpu_baseline` times one full evaluation of the
same workload by the all-core C/OpenMP restatement of the reference's CPU
path (oracle/cpu_ref.py); `--impl reference` times full evaluations of it
(no extrapolation) and loads no library of this package.  `fp64_error` gives
both contraction forms' error against float64 sums over all triangles.

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
DATA = "synthetic (seeded Zel'dovich mock)"


def bench_config():
    """The workload description both arms print (the same dict on both)."""
    W = WORKLOAD
    gb = W["shells"] * W["Ngrid"] ** 3 * 4 / 1e9
    return dict(W, l2=f"device arm: L2 flushed between steps (512 MB write); {gb:.1f} GB of shell fields per step")


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


def plan_info(nmax, ncut, step):
    """Host-side plan query of the library for the triangle loop: tensor-core
    multiply-adds per voxel of the contraction plan and its voxels per chunk
    (64: contract_tc64_kernel, 32: contract_tc_kernel)."""
    from pyspectrum_gb300 import _lib, core as _core
    jmin = ncut // step
    tri = np.ascontiguousarray(_core.triangles(jmin, nmax) - jmin, dtype=np.int32)
    info = np.zeros(9, dtype=np.int64)
    _lib.call("pyspec_bk_plan_check", nmax - jmin + 1, tri.ctypes.data, int(tri.shape[1]), info.ctypes.data, 9)
    return int(info[6]), int(info[8])


def fp32_tiles(nmax, ncut, step):
    """Micro-tiles (4 pair rows x 8 shells) of the FP32 contraction's plan for
    the triangle loop: pairs (i, j) sorted by (j, i) in groups of 4, one tile
    per aligned 8-wide window of l (l0 a multiple of 8) that meets the group's
    l range."""
    jmin = ncut // step
    pairs = {}
    for i in range(jmin, nmax + 1):
        for j in range(jmin, i + 1):
            for l in range(max(i - j, jmin), j + 1):
                pairs.setdefault((i - jmin, j - jmin), []).append(l - jmin)
    order = sorted(pairs, key=lambda p: (p[1], p[0]))
    tiles = 0
    for g in range(0, len(order), 4):
        ls = [l for p in order[g:g + 4] for l in pairs[p]]
        lo, hi = min(ls), max(ls)
        tiles += hi // 8 - lo // 8 + 1
    return tiles


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# ---------------------------------------------------------------------------
# Workload generator (numpy/scipy only, shared by both arms)
# ---------------------------------------------------------------------------
def zeldovich_positions(npart, Lbox, ngrid, seed, slope=-1.5, rms_disp=5.0):
    """Seeded Zel'dovich box: a Gaussian random field with P(k) ~ k^slope on
    an ngrid^3 grid (white noise from numpy's PCG64), its displacement
    psi(k) = i k delta(k) / k^2 scaled to rms |psi| = rms_disp Mpc/h, applied
    (nearest grid point) to a lattice of ceil(npart^(1/3))^3 cells with a
    random offset inside each cell.  Returns float64 (3, npart) positions in
    [0, Lbox).  numpy/scipy only, so the reference arm loads no library of
    this package; the device arm uses the same particles."""
    import scipy.fft as sfft
    n = int(ngrid)
    rng = np.random.default_rng(seed)
    g = sfft.fftn(rng.standard_normal((n, n, n), dtype=np.float32).astype(np.complex128), workers=-1)
    k = np.fft.fftfreq(n, d=1.0 / n)
    kz, ky, kx = k.reshape(n, 1, 1), k.reshape(1, n, 1), k.reshape(1, 1, n)
    k2 = kx * kx + ky * ky + kz * kz
    k2[0, 0, 0] = 1.0
    amp = k2 ** (slope / 4.0)
    amp[0, 0, 0] = 0.0
    g *= amp
    psi = np.empty((3, n, n, n), dtype=np.float32)
    for d, kd in enumerate((kx, ky, kz)):
        psi[d] = sfft.ifftn(g * (1j * kd / k2), workers=-1).real * float(n) ** 3
    del g
    psi *= np.float32(rms_disp / np.sqrt((psi.astype(np.float64) ** 2).sum(0).mean()))
    npart = int(npart)
    m = int(round(npart ** (1.0 / 3.0)))
    if m ** 3 < npart:
        m += 1
    rng = np.random.default_rng(seed + 1000)
    cells = np.arange(m ** 3) if m ** 3 == npart else np.sort(rng.choice(m ** 3, size=npart, replace=False))
    iz, rem = np.divmod(cells, m * m)
    iy, ix = np.divmod(rem, m)
    q = (np.stack([ix, iy, iz]).astype(np.float64) + rng.uniform(0.0, 1.0, size=(3, npart))) * (Lbox / m)
    idx = np.clip((q / Lbox * n).astype(np.int64), 0, n - 1)
    disp = psi[:, idx[2], idx[1], idx[0]].astype(np.float64)
    return np.mod(q + disp, Lbox)


def make_positions_np(seed=None):
    W = WORKLOAD
    return zeldovich_positions(W["npart"], W["Lbox"], W["Ngrid"], W["seed"] if seed is None else seed)


def reference_counts():
    """Exact triangle counts of the workload's geometry, read the way the
    reference reads its count cache (pyspectrum.py:407, 962-973): from the
    reference's own shipped cache for Ngrid 360 / Nmax 40 / Ncut 3 / step 3
    (stored in tests/golden as integers); other geometries (the profiling
    case) are counted by the oracle's float64 shell-indicator sums."""
    W = WORKLOAD
    if (W["Ngrid"], W["Nmax"], W["Ncut"], W["step"]) == (360, 40, 3, 3):
        return np.load(os.path.join(ROOT, "tests", "golden", "counts_ref360.npz"))["nmax40"]
    import torch
    from oracle import torch_fp64 as TF
    from oracle import cpu_ref
    n, step, jmin, nmax = W["Ngrid"], W["step"], W["Ncut"] // W["step"], W["Nmax"]
    tri, _ = cpu_ref.triangles(jmin, nmax)
    I, _ = TF.shell_fields(torch.ones((n, n, n), dtype=torch.complex128), step, jmin, nmax)
    craw, _ = TF.triangle_sums(I, tri - jmin, with_abs=False)
    return np.rint(craw / float(n) ** 3).astype(np.int64)


# ---------------------------------------------------------------------------
# CPU reference arm: the all-core C restatement of the reference's CPU path
# (oracle/cpu_ref.py), full Bk_periodic evaluations, no extrapolation.
# ---------------------------------------------------------------------------
def cpu_reference_eval(xyz_np, counts):
    """One full Bk_periodic evaluation of the workload on all host cores
    (pyspectrum.py:285-457 structure: float32 grid, complex64 FFTs, one full
    3D FFT per shell, float64 triangle sums).  Returns (seconds, stages)."""
    from oracle import cpu_ref
    W = WORKLOAD
    t0 = time.perf_counter()
    _, stages = cpu_ref.bk_periodic_cpu(xyz_np, W["Lbox"], W["Ngrid"], W["step"], W["Ncut"], W["Nmax"], counts)
    return time.perf_counter() - t0, stages


def cpu_sample_text(cores):
    W = WORKLOAD
    return (f"full Bk_periodic evaluations ({W['npart']} particles, {W['Ngrid']}^3, {W['shells']} shells, "
            f"{W['triangles']} triangles), no extrapolation: C/OpenMP assignment, fcomb and triangle sums, "
            f"complex64 pocketfft FFTs, on {cores} host threads")


REF_BUDGET_S = 150.0     # the reference arm times at most this much CPU work


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import cpu_ref
    xyz_np = make_positions_np()
    counts = reference_counts()
    cores = cpu_ref.cores()
    per = []
    for _ in range(min(args.warmup, 1)):             # page-in, FFT plans, OpenMP pool
        cpu_reference_eval(xyz_np, counts)
    det = None
    for k in range(max(1, args.steps)):
        sec, det = cpu_reference_eval(xyz_np, counts)
        per.append(sec)
        if sum(per) + sec > REF_BUDGET_S:            # bounded: never run past the budget
            break
    total = float(np.sum(per))
    value = len(per) / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": len(per), "steps_requested": args.steps, "warmup": min(args.warmup, 1),
            "ms_per_step": total / len(per) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 grid and FFTs, f64 sums (CPU)", "data": DATA,
            "config": bench_config(),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": cpu_sample_text(cores), "stages_s": det},
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


def fp64_error(half, plans):
    """Error of both contraction forms against float64 sums over ALL the
    workload's triangles: the shell fields rebuilt from the same delta(k)
    with complex128 FFTs and the triangle sums taken in float64
    (oracle/torch_fp64.py, plain torch on the device).  Per form: median and
    maximum |dB/B|, the maximum over triangles with condition number
    sum|F_iF_jF_l| / |sum F_iF_jF_l| < 1e3, and the maximum error normalised
    by sum|F_iF_jF_l|."""
    import torch
    from oracle import torch_fp64 as TF
    t0 = time.perf_counter()
    bsums = {}
    for name, pl in plans.items():          # both forms from this same delta(k)
        pl.shells(half)
        pl.contract()
        bsums[name] = pl.bsum.cpu().numpy()
    plan = plans["bf16x3"]
    full = TF.reflect_half(half)
    F, _ = TF.shell_fields(full, plan.step, plan.jmin, plan.nmax)
    del full
    exact, absum = TF.triangle_sums(F, plan.tri_np - plan.jmin)
    del F
    torch.cuda.empty_cache()
    out = {"triangles": int(plan.T), "shells": f"{plan.jmin}..{plan.nmax}", "seconds": time.perf_counter() - t0,
           "reference": "float64 fields (complex128 FFTs) and float64 sums from the same delta(k)"}
    for name, b in bsums.items():
        out[name] = TF.error_report(b, exact, absum)
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
    xyz_np = make_positions_np()
    x = torch.from_numpy(xyz_np).to(dev)
    npart = x.shape[1]
    nbar = npart / L ** 3
    kf = 2 * np.pi / L
    grid = torch.zeros((n, n, n), dtype=torch.complex64, device=dev)
    half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    plans = {m: core.get_plan(n, step, ncut, nmax, m, dev) for m in ("bf16x3", "fp32", "bf16x3_fine", "bf16x6")}

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
    for method in ("bf16x3", "fp32", "bf16x3_fine", "bf16x6"):
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
        if method in core.TENSOR_METHODS:
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
    macs, chunk = plan_info(nmax, ncut, step)
    executed = 2.0 * macs * V
    kname = "contract_tc64_kernel" if chunk == 64 else "contract_tc_kernel"
    t_con = main["stage_ms"]["contraction"] / 1e3
    roofline = {"kernel": kname + " (+ partial reduction)", "bound": "tensor",
                "achieved": useful / t_con / 1e12, "peak": bf16, "unit": "TFLOP/s",
                "frac": useful / t_con / 1e12 / bf16, "peak_kind": kind,
                "executed_tflops": executed / t_con / 1e12, "executed_frac": executed / t_con / 1e12 / bf16,
                "useful_over_executed": useful / executed,
                "traffic": 4.0 * 40 * V, "traffic_note": "dram bytes of one launch: the ncu capture at 192^3 "
                "(1.133 GB read) scaled by the voxel count; equal to the algorithmic bytes (fields read once)"}
    # the FP32 CUDA-core comparator against the FP32 SIMT peak (nominal: 152
    # SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz; no measured FP32 peak exists)
    t32 = results["fp32"]["stage_ms"]["contraction"] / 1e3
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    results["fp32"]["roofline"] = {
        "kernel": "contract_fp32_kernel (+ partial reduction)", "bound": "fp32 simt", "unit": "TFLOP/s",
        "achieved": useful / t32 / 1e12, "peak": fp32_peak, "peak_kind": "nominal", "frac": useful / t32 / 1e12 / fp32_peak,
        "executed_tflops": 2.0 * 32 * fp32_tiles(nmax, ncut, step) * V / t32 / 1e12,
        "note": "executed = 2 FLOP x 32 products per micro-tile (4 pairs x 8 shells) x tiles x voxels"}
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cpu_ref
        cores = cpu_ref.cores()
        sec, det = cpu_reference_eval(xyz_np, reference_counts())
        cpu = {"value": 1.0 / sec, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": cpu_sample_text(cores).replace("evaluations", "evaluation (one)"), "stages_s": det}
    line = {"metric": METRIC, "value": main["bk_evals_per_s"], "unit": UNIT, "n_gpus": world,
            "steps": main["steps"], "warmup": args.warmup, "ms_per_step": main["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 (f32 fields, f64 sums)",
            "data": DATA,
            "config": bench_config(),
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
    from pyspectrum_gb300 import tune
    line["tuned"] = {k.split("|", 2)[0] + "|" + k.split("|", 2)[2]: v for k, v in tune.choices().items()
                     if f"|n{n}|" in k or k.endswith(f"|n{n}")}
    if not args.no_batch:
        try:
            line["batch_64_mocks"] = batch_rate()
        except Exception as exc:        # informational; the headline line still prints
            line["batch_64_mocks"] = {"error": str(exc)[:300]}
    print(json.dumps(line), flush=True)


def batch_rate():
    """Many boxes per call (Bk_periodic_batch), the many-mock workload: 64
    seeded Zel'dovich mocks with particle counts uniform in [0.5M, 4M] and
    grids mixed over {192, 256, 360} (L = 2500, step 3, Nmax 40, split-BF16,
    graph replay).  Positions start in pinned host memory and the results end
    on the host.  The first pass (plans, counts, tuning, graph capture of the
    three geometries) is untimed; the second is timed by the host clock."""
    import torch
    from pyspectrum_gb300 import batch, mocks, tune
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
    warm = [cat[int(np.nonzero(grids == g)[0][0])] for g in (192, 256, 360) for _ in range(2)]
    runner.run(warm)
    runner.run(cat)                      # tunes the assignment at every density bucket met
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = runner.run(cat)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert len(out) == nmock and all(np.isfinite(o["b123"]).all() for o in out)
    tuned = {k.split("|", 2)[0] + "|" + k.split("|", 2)[2]: v["choice"] for k, v in tune.choices().items()
             if any(f"|n{g}|" in k for g in (192, 256, 360))}
    return {"workload": "64 Zel'dovich mocks, Np uniform in [0.5M, 4M], Ngrid in {192, 256, 360}, L 2500, step 3, "
                        "Nmax 40", "metric": "Bk evals/s (batch, pinned host positions in, host results out)",
            "value": nmock / dt, "seconds": dt, "mocks_per_grid": {str(g): int((grids == g).sum()) for g in
                                                                   (192, 256, 360)},
            "particles_total": int(nparts.sum()), "method": "bf16x3", "graphs": True, "tuned": tuned}


def run_batch(args):
    """Prints the many-mock batch line alone (not the headline bench line)."""
    print(json.dumps(batch_rate()), flush=True)


def run_profile_delta(reps=3):
    """Profiling case for the delta(k) and P(k) kernels on the bench workload
    (1M particles, 360^3): `reps` rounds of clip/cast, the direct and the
    16^3-tiled mass assignment, the 3D FFT (default radix plan), the
    interlacing combine, the P(k) monopole and the pk_pbox_rsd multipoles.
    About 1.2 GB on the device; prints the last round's event times (not a
    bench result)."""
    import torch
    from pyspectrum_gb300 import _lib, core
    from pyspectrum_gb300._lib import call, ptr, stream_ptr
    W = WORKLOAD
    n, L = W["Ngrid"], W["Lbox"]
    x = torch.from_numpy(make_positions_np()).cuda()
    npart = x.shape[1]
    grid = torch.zeros((n, n, n), dtype=torch.complex64, device="cuda")
    half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device="cuda")
    kf_ks = float(np.float32(float(n) / L))
    wst = torch.empty(_lib.load().pyspec_assign_tiled_workspace(npart, n, 16), dtype=torch.uint8, device="cuda")
    nbin, nmu = n // 2, 10
    pko = torch.empty(6 * nbin, dtype=torch.float64, device="cuda")
    rso = torch.empty(2 * (5 * nbin + 4 * nbin * nmu), dtype=torch.float64, device="cuda")
    names = ["prepare", "assign_direct", "assign_tiled16", "fft3d", "fcomb", "pk_mono", "pk_rsd"]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
    for _ in range(reps):
        ev[0].record()
        xyzs, ws = core.prepare_positions(x, L)
        ev[1].record()
        grid.zero_()
        call("pyspec_assign_pcs_interlaced", ptr(xyzs), ptr(ws), npart, n, kf_ks, 0.0, ptr(grid), stream_ptr())
        ev[2].record()
        grid.zero_()
        call("pyspec_assign_pcs_interlaced_tiled", ptr(xyzs), ptr(ws), npart, n, kf_ks, 0.0, 16, ptr(grid),
             ptr(wst), wst.numel(), stream_ptr())
        ev[3].record()
        call("pyspec_fft3d_c2c", ptr(grid), n, 1, stream_ptr())
        ev[4].record()
        call("pyspec_fcomb_periodic", ptr(grid), n, float(npart), ptr(half), stream_ptr())
        ev[5].record()
        call("pyspec_pk_monopole", ptr(half), n, float(L), ptr(pko), stream_ptr())
        ev[6].record()
        call("pyspec_pk_pbox_rsd", ptr(half), n, 2, int(L), nbin, nmu, ptr(rso), stream_ptr())
        ev[7].record()
    torch.cuda.synchronize()
    print(json.dumps({"profile": "delta_k_and_pk", "Ngrid": n, "npart": npart,
                      "ms_last_round": {nm: ev[k].elapsed_time(ev[k + 1]) for k, nm in enumerate(names)}}),
          flush=True)


def run_assign_sweep():
    """The mass-assignment variants (direct L2 atomics; shared-memory tiles of
    4^3, 8^3, 16^3 cells) timed at three densities of Zel'dovich boxes: the
    bench box (1M particles on 360^3), the densest mock of the many-mock
    workload (4M on 192^3) and the large grid (16M on 512^3).  Best of 5
    CUDA-event timings each (the grid zeroing excluded).  Prints one JSON line."""
    import torch
    from pyspectrum_gb300 import core, mocks, tune
    out = {}
    for n, npart, L in ((360, 1_000_000, 2500.0), (192, 4_000_000, 2500.0), (512, 16_000_000, 3000.0)):
        x = mocks.zeldovich_mock(npart, L, ngrid=n, seed=5)
        xyzs, ws = core.prepare_positions(x, L)
        del x
        grid = torch.zeros((n, n, n), dtype=torch.complex64, device="cuda")
        kf_ks = float(np.float32(float(n) / L))
        wsbuf = {b: tune._assign_workspace(npart, n, b, grid.device) for b in (4, 8, 16)}
        res = {}
        for c in tune.assign_candidates(n):
            best = float("inf")
            for _ in range(6):
                grid.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                tune._assign_run(c, xyzs, ws, n, kf_ks, 0.0, grid, wsbuf)
                e1.record()
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            res[c] = round(best, 4)
        out[f"{npart // 1_000_000}M_on_{n}^3"] = {"particles_per_cell": npart / n ** 3, "ms": res,
                                                   "fastest": min(res, key=res.get)}
        del xyzs, ws, grid, wsbuf
        torch.cuda.empty_cache()
    print(json.dumps({"assign_sweep": out}), flush=True)


def run_profile_shells(jtop):
    """Profiling case for the shell passes: shells jtop-2..jtop of the bench
    workload's delta(k) at 360^3 (about 1 GB on the device), three calls.
    Prints the time of the last call; not a bench result."""
    import torch
    from pyspectrum_gb300 import _lib, core
    from pyspectrum_gb300._lib import call, ptr, stream_ptr
    W = WORKLOAD
    n, L, step = W["Ngrid"], W["Lbox"], W["step"]
    x = torch.from_numpy(make_positions_np()).cuda()
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
    ap.add_argument("--no-fp64-check", action="store_true", help="skip the float64 error check of all triangles")
    ap.add_argument("--small", action="store_true", help="run the 192^3 profiling case instead of the bench workload")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-mock batch measurement on the main line")
    ap.add_argument("--batch", action="store_true",
                    help="time 64 mixed-size mocks through Bk_periodic_batch instead of the bench workload")
    ap.add_argument("--assign-sweep", action="store_true",
                    help="only time the mass-assignment variants at three particle densities")
    ap.add_argument("--profile-delta", action="store_true",
                    help="only run the delta(k) and P(k) kernels of the bench workload (ncu profiling case)")
    ap.add_argument("--profile-shells", type=int, default=0, metavar="J",
                    help="only run shells J-2..J of the bench workload three times (ncu profiling case)")
    args = ap.parse_args()
    if args.profile_shells:
        run_profile_shells(args.profile_shells)
        return
    if args.profile_delta:
        run_profile_delta()
        return
    if args.assign_sweep:
        run_assign_sweep()
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
        run_reference(args, rank, world)      # host cores only; other ranks exit without work
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
