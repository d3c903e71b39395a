"""Autotuner of the launch variants: mass-assignment tile, FFT radix plan and
contraction tile plan.

Each tunable stage has interchangeable device implementations that compute
the same result (to float32 rounding):

* mass assignment (estimator.f:284-512): direct L2 atomics
  (``pyspec_assign_pcs_interlaced``) or shared-memory tiles of 4^3, 8^3 or
  16^3 cells (``pyspec_assign_pcs_interlaced_tiled``); which wins depends on
  how many particles share cells, so the key is the grid size and the
  particles per cell (rounded to a power of two);
* 3D FFT (pyspectrum.py:1073-1075): the two-stage register radix splits of
  the grid size and the shared-memory Stockham form
  (``pyspec_fft3d_variants`` / ``pyspec_fft3d_c2c_variant``); key: grid size;
* tensor-core contraction (pyspectrum.py:415-437): the pair-cover tile plan
  or the run plan (``PYSPEC_CONTRACT_RUN_PLAN``); key: grid size, shell count
  and the triangle list.

The first time a key is met, every candidate is timed with CUDA events on
the current stream (one untimed call, then the best of ``REPS`` timed calls)
and the fastest is kept, in memory and in ``<cache_dir>/tune.json`` (keyed
also by the device name), so later processes skip the search.  Set
``PYSPEC_GB300_TUNE=0`` to skip tuning and use the fixed defaults.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import math
import os
import threading

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr, stream_ptr

REPS = 3
_lock = threading.Lock()
_mem: dict = {}
_loaded = False


def enabled() -> bool:
    return os.environ.get("PYSPEC_GB300_TUNE", "1") not in ("0", "false", "no", "")


def cache_file() -> str:
    from . import core
    return os.path.join(core.cache_dir(), "tune.json")


_dev_names: dict = {}


def _device_key(device) -> str:
    """Device name for cache keys, looked up once per device index (the
    driver query costs more than the rest of a cached lookup)."""
    d = torch.device(device) if not isinstance(device, int) else torch.device("cuda", device)
    idx = d.index if d.index is not None else torch.cuda.current_device()
    name = _dev_names.get(idx)
    if name is None:
        name = torch.cuda.get_device_name(idx).replace(" ", "_")
        _dev_names[idx] = name
    return name


def _load():
    global _loaded
    if _loaded:
        return
    _loaded = True
    try:
        with open(cache_file()) as f:
            _mem.update(json.load(f))
    except (OSError, ValueError):
        pass


def _store(key, value):
    with _lock:
        _mem[key] = value
        try:
            os.makedirs(os.path.dirname(cache_file()), exist_ok=True)
            tmp = cache_file() + ".tmp"
            with open(tmp, "w") as f:
                json.dump(_mem, f, indent=1, sort_keys=True)
            os.replace(tmp, cache_file())
        except OSError:
            pass


def choices() -> dict:
    """Every choice made so far (this process and the on-disk cache)."""
    _load()
    return dict(_mem)


def _time(fn, reps=REPS) -> float:
    """Best of `reps` timed calls of fn (ms), after one untimed call."""
    fn()
    best = math.inf
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def _cached(key, candidates):
    """The stored choice for key if it is one of the candidates, else None."""
    _load()
    got = _mem.get(key)
    if got is not None and got.get("choice") in candidates:
        return got["choice"]
    return None


def _pick(key, candidates, run):
    """The stored choice for key, or the fastest candidate (timed with `run`)."""
    got = _cached(key, candidates)
    if got is not None:
        return got
    times = {}
    for c in candidates:
        try:
            times[c] = _time(lambda: run(c))
        except _lib.PyspecError:
            continue                      # a candidate the library refuses for this size
    best = min(times, key=times.get)
    _store(key, {"choice": best, "ms": {str(k): round(v, 4) for k, v in times.items()}})
    return best


# ---------------------------------------------------------------------------
# mass assignment
# ---------------------------------------------------------------------------
ASSIGN_DEFAULT = "direct"


def assign_candidates(n):
    return ["direct"] + [f"tiled{b}" for b in (4, 8, 16) if n >= b + 4]


def _assign_run(choice, xyzs, ws, n, kf_ks, offset, grid, wsbuf):
    if choice == "direct":
        call("pyspec_assign_pcs_interlaced", ptr(xyzs), ptr(ws), xyzs.shape[1], n, kf_ks, offset, ptr(grid),
             stream_ptr())
        return
    tile = int(choice[5:])
    call("pyspec_assign_pcs_interlaced_tiled", ptr(xyzs), ptr(ws), xyzs.shape[1], n, kf_ks, offset, tile,
         ptr(grid), ptr(wsbuf[tile]), wsbuf[tile].numel(), stream_ptr())


_assign_ws: dict = {}


def _assign_workspace(npart, n, tile, device):
    lib = _lib.load()
    need = int(lib.pyspec_assign_tiled_workspace(npart, n, tile))
    key = (str(device), tile)
    buf = _assign_ws.get(key)
    if buf is None or buf.numel() < need:
        buf = torch.empty(max(need, 256), dtype=torch.uint8, device=device)
        _assign_ws[key] = buf
    return buf


def assign(xyzs, ws, n, kf_ks, offset, grid):
    """Add the particles onto the (zeroed) interlaced grid with the tuned
    variant.  While tuning, each candidate runs on the same grid, which is
    zeroed again before the kept call."""
    npart = xyzs.shape[1]
    dev = xyzs.device
    if npart == 0:
        return ASSIGN_DEFAULT
    cands = assign_candidates(n)
    if not enabled():
        choice = ASSIGN_DEFAULT
    else:
        density = npart / float(n) ** 3
        key = f"assign|{_device_key(dev)}|n{n}|ppc2^{int(round(math.log2(max(density, 1e-9))))}"
        choice = _cached(key, cands)
        if choice is None:                 # tune: every candidate on the same grid, zeroed before each
            wsbuf = {int(c[5:]): _assign_workspace(npart, n, int(c[5:]), dev) for c in cands if c != "direct"}

            def run(c):
                grid.zero_()
                _assign_run(c, xyzs, ws, n, kf_ks, offset, grid, wsbuf)
            choice = _pick(key, cands, run)
            grid.zero_()
    wsbuf = {} if choice == "direct" else {int(choice[5:]): _assign_workspace(npart, n, int(choice[5:]), dev)}
    _assign_run(choice, xyzs, ws, n, kf_ks, offset, grid, wsbuf)
    return choice


# ---------------------------------------------------------------------------
# 3D FFT radix plan
# ---------------------------------------------------------------------------
def fft_variants(n):
    """[(variant, (r1, r2))]; (0, 0) is the shared-memory Stockham form."""
    lib = _lib.load()
    cnt = int(lib.pyspec_fft3d_variants(n, None, 0))
    buf = (ctypes.c_int32 * (2 * cnt))()
    lib.pyspec_fft3d_variants(n, buf, cnt)
    return [(v, (buf[2 * v], buf[2 * v + 1])) for v in range(cnt)]


def fft_default(n):
    """The variant pyspec_fft3d_c2c runs for this size."""
    vs = fft_variants(n)
    return 0 if n in (192, 256, 360) else len(vs) - 1


def fft_variant(n, device=None) -> int:
    """The tuned radix-plan variant of the 3D FFT for size n, timed on a
    scratch grid of random values the first time."""
    if not enabled():
        return fft_default(n)
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    key = f"fft3d|{_device_key(device)}|n{n}"
    _load()
    if key in _mem:
        return int(_mem[key]["choice"])
    vs = [v for v, _ in fft_variants(n)]
    g = torch.randn((n, n, n, 2), dtype=torch.float32, device=device)

    def run(v):
        call("pyspec_fft3d_c2c_variant", ptr(g), n, 1, int(v), stream_ptr())
    best = _pick(key, vs, run)
    del g
    return int(best)


def fft3d(grid, n, sign=1):
    """The unnormalised 3D FFT of a complex64 grid, in place, with the tuned variant."""
    call("pyspec_fft3d_c2c_variant", ptr(grid), n, int(sign), fft_variant(n, grid.device), stream_ptr())


# ---------------------------------------------------------------------------
# contraction tile plan
# ---------------------------------------------------------------------------
def contract_flags(plan) -> int:
    """Method flags of the tuned tile plan for a BkPlan's triangle list
    (0: the default, pair cover where it needs fewer tiles and 64-voxel
    chunks where the plan allows them; CONTRACT_KC32: 32-voxel chunks;
    CONTRACT_RUN_PLAN, with either), timed on the plan's current fields the
    first time."""
    from .core import METHODS, TENSOR_METHODS
    if plan.method not in TENSOR_METHODS or not enabled():
        return 0
    digest = hashlib.sha1(plan.slots_host.tobytes()).hexdigest()[:16]
    key = f"contract|{_device_key(plan.device)}|{plan.method}|n{plan.n}|S{plan.S}|T{plan.T}|{digest}"
    cands = [0, _lib.CONTRACT_KC32, _lib.CONTRACT_RUN_PLAN, _lib.CONTRACT_RUN_PLAN | _lib.CONTRACT_KC32]

    def run(flags):
        call("pyspec_bk_contract", ptr(plan.fields), plan.n, plan.S, ptr(plan.slots),
             plan.slots_host.ctypes.data_as(ctypes.c_void_p), plan.T, METHODS[plan.method] | flags,
             ptr(plan.bsum), ptr(plan.ws_con), plan.ws_con.numel(), stream_ptr())
    return int(_pick(key, cands, run))


def summary() -> dict:
    """Choices of this process and the cache, for reports (ms per candidate included)."""
    return {k: v for k, v in choices().items()}
