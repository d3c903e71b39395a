"""Device-side pipeline of the periodic-box estimator.

Functions here take and return torch CUDA tensors and drive the C ABI of
libpyspec_gb300.so (see ``_lib``).  ``pyspectrum.py`` wraps them in the
reference's call surface (numpy in, dict of numpy arrays out).

Device layouts
--------------
* positions: float32 (3, Np), rows x, y, z;  weights float32 (Np,)
* density grid: complex64 (N, N, N) indexed [z, y, x]
* half grid delta(k): complex64 (N, N, N//2+1) indexed [z, y, x]
* shell fields: float32 (S, N^3), S = Nmax - Ncut//step + 1
"""
from __future__ import annotations

import ctypes
import math
import os
import threading

import numpy as np
import torch

from . import _lib, tune
from ._lib import call, ptr, stream_ptr

# contraction methods: FP32 CUDA cores; split-BF16 tensor cores with the
# accumulators drained every 32 chunks ('bf16x3') or every 8 ('bf16x3_fine':
# about 4x smaller error, the drains cost more time); and 'bf16x6', which adds
# a second tensor-core pass with the operands' third bf16 parts (6 products)
METHODS = {"fp32": _lib.CONTRACT_FP32, "bf16x3": _lib.CONTRACT_BF16X3,
           "bf16x3_fine": _lib.CONTRACT_BF16X3 | _lib.CONTRACT_FINE_DRAIN, "bf16x6": _lib.CONTRACT_BF16X6}
TENSOR_METHODS = ("bf16x3", "bf16x3_fine", "bf16x6")


def _dev(device=None) -> torch.device:
    if device is None:
        device = torch.device("cuda", torch.cuda.current_device())
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError("pyspectrum_gb300 computes on a CUDA device; got %s" % device)
    return device


def _workspace(nbytes: int, device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


# ---------------------------------------------------------------------------
# particles -> delta(k)
# ---------------------------------------------------------------------------
def positions_to_device(xyz, device=None) -> torch.Tensor:
    """(3, Np) float64 contiguous CUDA tensor from a numpy array or tensor."""
    device = _dev(device)
    t = torch.as_tensor(xyz)
    if t.dim() != 2 or t.shape[0] != 3:
        raise ValueError("positions must be a 3 x N array")
    # from page-locked memory the copy is queued on the stream (every public
    # entry point reads its result back, which orders it before return)
    pinned = t.device.type == "cpu" and t.is_pinned() and t.dtype == torch.float64
    return t.to(device=device, dtype=torch.float64, non_blocking=pinned).contiguous()


def prepare_positions(xyz_d: torch.Tensor, Lbox: float, w_d=None, vel_d=None, los: int = 2,
                      rsd_factor: float = 0.0):
    """Clip/cast positions (pyspectrum.py:938-945); optional RSD shift (util.py:72-74)."""
    npart = xyz_d.shape[1]
    xyzs = torch.empty((3, npart), dtype=torch.float32, device=xyz_d.device)
    ws = torch.empty((npart,), dtype=torch.float32, device=xyz_d.device)
    if w_d is not None:
        w_d = w_d.to(dtype=torch.float64).contiguous()
    if vel_d is not None:
        vel_d = vel_d.to(dtype=torch.float64).contiguous()
    call("pyspec_prepare_positions", ptr(xyz_d), xyz_d.stride(0), ptr(vel_d),
         0 if vel_d is None else vel_d.stride(0), int(los), float(rsd_factor), ptr(w_d), npart,
         float(Lbox), ptr(xyzs), ptr(ws), stream_ptr())
    return xyzs, ws


_grids: dict = {}


def _assign_grid(n: int, device) -> torch.Tensor:
    """The interlaced assignment grid (N^3 complex64), kept per device and N:
    it is scratch, fully rewritten by every call on the same stream."""
    key = (n, str(device))
    g = _grids.get(key)
    if g is None:
        g = torch.empty((n, n, n), dtype=torch.complex64, device=device)
        _grids[key] = g
    return g


def fft_periodic_half(xyzs: torch.Tensor, ws, Ngrid: int, Lbox: float, wsum: float,
                      grid: torch.Tensor | None = None, half: torch.Tensor | None = None) -> torch.Tensor:
    """FFT_periodic (pyspectrum.py:909-959) on device: assign -> FFT -> fcomb.
    Returns the half grid delta(k), complex64 (N, N, N//2+1) [z, y, x]."""
    n = int(Ngrid)
    dev = xyzs.device
    if grid is None:
        grid = _assign_grid(n, dev)
    grid.zero_()
    kf_ks = float(np.float32(float(n) / Lbox))          # pyspectrum.py:931
    tune.assign(xyzs, ws, n, kf_ks, 0.0, grid)          # direct or tiled, as tuned for this density
    tune.fft3d(grid, n, 1)                              # the tuned radix plan
    if half is None:
        half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=dev)
    call("pyspec_fcomb_periodic", ptr(grid), n, float(wsum), ptr(half), stream_ptr())
    return half


def half_from_full(full_zyx: torch.Tensor) -> torch.Tensor:
    n = full_zyx.shape[0]
    half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=full_zyx.device)
    call("pyspec_half_from_full", ptr(full_zyx), n, ptr(half), stream_ptr())
    return half


def reflect_half(half: torch.Tensor) -> torch.Tensor:
    n = half.shape[0]
    full = torch.empty((n, n, n), dtype=torch.complex64, device=half.device)
    call("pyspec_reflect_delta", ptr(half), n, ptr(full), stream_ptr())
    return full


# ---------------------------------------------------------------------------
# triangles and counts
# ---------------------------------------------------------------------------
def triangles(jmin: int, nmax: int) -> np.ndarray:
    """The (i, j, l) loop of pyspectrum.py:415-417 as an int32 (3, T) array."""
    out = [(i, j, l) for i in range(jmin, nmax + 1) for j in range(jmin, i + 1)
           for l in range(max(i - j, jmin), j + 1)]
    return np.array(out, dtype=np.int32).T.copy() if out else np.zeros((3, 0), np.int32)


def cache_dir() -> str:
    return os.environ.get("PYSPEC_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "pyspectrum_gb300"))


_counts_mem: dict = {}
_counts_lock = threading.Lock()


def counts_path(Ngrid, Nmax, Ncut, step) -> str:
    return os.path.join(cache_dir(), f"counts.Ngrid{Ngrid}.Nmax{Nmax}.Ncut{Ncut}.step{step}.int64.npz")


def triangle_counts(Ngrid: int, Nmax: int, Ncut: int, step: int, device=None, use_disk: bool = True):
    """Exact integer triangle counts (loop order) and mode counts Nk[0..Nmax].

    Computed on the GPU in float64 (pyspec_bk_counts) once per geometry and
    cached in memory and on disk (``cache_dir()``).  Returns numpy int64
    arrays (counts[T], nk[Nmax+1])."""
    key = (int(Ngrid), int(Nmax), int(Ncut), int(step))
    with _counts_lock:
        if key in _counts_mem:
            return _counts_mem[key]
    path = counts_path(*key)
    if use_disk and os.path.exists(path):
        z = np.load(path)
        res = (z["counts"].astype(np.int64), z["nk"].astype(np.int64))
        with _counts_lock:
            _counts_mem[key] = res
        return res
    res = compute_triangle_counts(*key, device=device)
    install_triangle_counts(*key, res[0], res[1], use_disk=use_disk)
    return res


def install_triangle_counts(Ngrid, Nmax, Ncut, step, counts, nk, use_disk: bool = True) -> None:
    """Make (counts[T] in loop order, nk[Nmax+1]) the cached counts of a
    geometry, in memory and (``use_disk``) in ``cache_dir()``."""
    key = (int(Ngrid), int(Nmax), int(Ncut), int(step))
    counts = np.asarray(counts, dtype=np.int64)
    nk = np.asarray(nk, dtype=np.int64)
    T = triangles(Ncut // step, Nmax).shape[1]
    if counts.shape != (T,) or nk.shape != (Nmax + 1,):
        raise ValueError(f"counts must have shape ({T},) and nk ({Nmax + 1},)")
    if use_disk:
        path = counts_path(*key)
        try:
            os.makedirs(cache_dir(), exist_ok=True)
            tmp = path + ".tmp.npz"
            np.savez(tmp, counts=counts, nk=nk)
            os.replace(tmp, path)
        except OSError:
            pass
    with _counts_lock:
        _counts_mem[key] = (counts, nk)


def compute_triangle_counts(Ngrid, Nmax, Ncut, step, device=None):
    device = _dev(device)
    jmin = Ncut // step
    tri = torch.from_numpy(triangles(jmin, Nmax)).to(device)
    T = tri.shape[1]
    counts = torch.zeros(T, dtype=torch.int64, device=device)
    nk = torch.zeros(Nmax + 1, dtype=torch.int64, device=device)
    nbytes = _lib.load().pyspec_bk_counts_workspace(Ngrid, step, jmin, Nmax)
    ws = _workspace(nbytes, device)
    call("pyspec_bk_counts", Ngrid, step, jmin, Nmax, ptr(tri), T, ptr(counts), ptr(nk), ptr(ws), ws.numel(),
         stream_ptr())
    return counts.cpu().numpy(), nk.cpu().numpy()


# ---------------------------------------------------------------------------
# shells, contraction, normalisation
# ---------------------------------------------------------------------------
class BkPlan:
    """Device buffers for one (Ngrid, step, Ncut, Nmax, method) geometry,
    reused across calls (fields, workspaces, triangle tables, counts)."""

    def __init__(self, Ngrid, step=3, Ncut=3, Nmax=40, method="fp32", device=None):
        self.device = _dev(device)
        self.n, self.step, self.ncut, self.nmax = int(Ngrid), int(step), int(Ncut), int(Nmax)
        self.jmin = self.ncut // self.step
        if self.jmin < 1:
            raise ValueError("Ncut//step must be >= 1 (shell 0 holds k = 0)")
        if self.nmax < self.jmin:
            raise ValueError("Nmax must be >= Ncut//step")
        if method not in METHODS:
            raise ValueError(f"method must be one of {sorted(METHODS)}")
        self.method = method
        self.S = self.nmax - self.jmin + 1
        n = self.n
        V = n ** 3
        lib = _lib.load()
        tri = triangles(self.jmin, self.nmax)
        self.tri_np = tri
        self.T = tri.shape[1]
        self.tri = torch.from_numpy(tri).to(self.device)
        self.slots = (self.tri - self.jmin).contiguous()
        self.slots_host = np.ascontiguousarray(tri - self.jmin, dtype=np.int32)
        c, nk = triangle_counts(n, self.nmax, self.ncut, self.step, device=self.device)
        self.counts_np, self.nk_np = c, nk
        self.counts = torch.from_numpy(c).to(self.device)
        self.nk = torch.from_numpy(nk).to(self.device)
        self.fields = torch.empty((self.S, V), dtype=torch.float32, device=self.device)
        self.p0sum = torch.empty(self.S, dtype=torch.float64, device=self.device)
        self.bsum = torch.empty(self.T, dtype=torch.float64, device=self.device)
        self.out = torch.empty((7, self.T), dtype=torch.float64, device=self.device)
        self.ws_shell = _workspace(lib.pyspec_shell_fields_workspace(n, self.S), self.device)
        self.ws_con = _workspace(lib.pyspec_bk_contract_workspace(n, self.S, self.T, METHODS[method]), self.device)
        self.contract_flags = None          # tile plan chosen by the tuner at the first contraction

    def shells(self, half: torch.Tensor):
        call("pyspec_shell_fields", ptr(half), self.n, self.step, self.jmin, self.nmax, ptr(self.fields),
             ptr(self.p0sum), ptr(self.ws_shell), self.ws_shell.numel(), stream_ptr())

    def contract(self):
        if self.contract_flags is None:
            self.contract_flags = tune.contract_flags(self)
        call("pyspec_bk_contract", ptr(self.fields), self.n, self.S, ptr(self.slots),
             self.slots_host.ctypes.data_as(ctypes.c_void_p), self.T, METHODS[self.method] | self.contract_flags,
             ptr(self.bsum), ptr(self.ws_con), self.ws_con.numel(), stream_ptr())

    def normalize(self, apply_units=False, nbar=1.0, kf=1.0):
        call("pyspec_bk_normalize", ptr(self.bsum), ptr(self.counts), ptr(self.p0sum), ptr(self.nk),
             ptr(self.tri), self.T, self.n, self.jmin, self.nmax, int(bool(apply_units)), float(nbar), float(kf),
             ptr(self.out), stream_ptr())

    def run(self, half: torch.Tensor, apply_units=False, nbar=1.0, kf=1.0):
        """Shells -> contraction -> normalisation, all enqueued on the current stream."""
        self.shells(half)
        self.contract()
        self.normalize(apply_units, nbar, kf)
        return self.out

    def status_word(self) -> torch.Tensor:
        """The contraction's int32 status word on the device (tensor-core
        method: 0, or the code of a bounded wait that timed out)."""
        return self.ws_con[:4].view(torch.int32)

    def _readback(self):
        """The output arrays and the contraction's status word, copied to
        page-locked host buffers on the current stream and read after one
        synchronisation (status 0 for the FP32 method)."""
        tensor = self.method in TENSOR_METHODS
        if self.out.device.type != "cuda":          # host-side buffers (plan logic without a device)
            return self.out.numpy().copy(), int(self.status_word()[0]) if tensor else 0
        if getattr(self, "_host_out", None) is None:
            self._host_out = torch.empty(tuple(self.out.shape), dtype=torch.float64).pin_memory()
            self._host_status = torch.zeros(1, dtype=torch.int32).pin_memory()
        self._host_out.copy_(self.out, non_blocking=True)
        if tensor:
            self._host_status.copy_(self.status_word(), non_blocking=True)
        torch.cuda.current_stream(self.out.device).synchronize()
        return self._host_out.numpy(), int(self._host_status[0]) if tensor else 0

    def result(self, apply_units=False):
        """Copy the normalised arrays to the host as the reference's output dict.
        Only triangles with counts > 0 are returned (all arrays aligned).
        Raises ContractTimeout if the tensor-core contraction stopped early."""
        out, status = self._readback()
        if self.method in TENSOR_METHODS:
            check_contract_status(status)
        if getattr(self, "_keep", None) is None:      # the kept triangles and their k indices, once per plan
            self._keep = np.nonzero(self.counts_np > 0)[0]
            self._ik = self.tri_np[:, self._keep].astype(np.int64) * self.step
        # every triangle kept (the usual case at the common grid sizes): one copy
        o = out.copy() if len(self._keep) == out.shape[1] else np.take(out, self._keep, axis=1)
        res = {
            "i_k1": self._ik[0].copy(), "i_k2": self._ik[1].copy(), "i_k3": self._ik[2].copy(),
            "p0k1": o[0], "p0k2": o[1], "p0k3": o[2],
            "b123": o[3], "q123": o[4], "counts": o[5],
        }
        if apply_units:
            res["b123_sn"] = o[6]
        return res


_plans: dict = {}

# Codes the tensor-core contraction leaves in the int32 at workspace offset 0
# when one of its bounded waits gives up (the kernel then stops early and its
# sums are incomplete).
CONTRACT_STATUS = {1: "producer wait for a field copy or a free stage", 2: "accumulator drain",
                   3: "MMA wait for the operands", 4: "MMA wait for the drain", 5: "copy wait for a free buffer"}


class ContractTimeout(RuntimeError):
    """A bounded wait inside the tensor-core contraction timed out."""


def check_contract_status(word: int) -> None:
    """Raise ContractTimeout if the contraction's status word is not 0."""
    word = int(word)
    if word != 0:
        what = CONTRACT_STATUS.get(word, "unknown wait")
        raise ContractTimeout(f"tensor-core contraction stopped early (status {word}: {what} timed out); "
                              "its triangle sums are incomplete")


def get_plan(Ngrid, step, Ncut, Nmax, method="fp32", device=None) -> BkPlan:
    device = _dev(device)
    key = (int(Ngrid), int(step), int(Ncut), int(Nmax), method, str(device))
    p = _plans.get(key)
    if p is None:
        p = BkPlan(Ngrid, step, Ncut, Nmax, method, device)
        _plans[key] = p
    return p


def release_plans():
    """Drop cached plans and scratch grids (and their device buffers)."""
    _plans.clear()
    _grids.clear()


# ---------------------------------------------------------------------------
# power spectra
# ---------------------------------------------------------------------------
def pk_monopole(half: torch.Tensor, Lbox: float) -> np.ndarray:
    n = half.shape[0]
    out = torch.empty((6, n // 2), dtype=torch.float64, device=half.device)
    call("pyspec_pk_monopole", ptr(half), n, float(Lbox), ptr(out), stream_ptr())
    return out[:3].cpu().numpy()


def pk_rsd_python(full: torch.Tensor, irsd: int, Lbox, Nmu: int):
    """The code='python' (k, mu) binning of pyspectrum.py:545-611 on a full
    grid complex64 (N, N, N) [z, y, x]; the 9 arrays with (2 pi)^3 applied."""
    n = full.shape[0]
    nbin = n // 2
    tot = 5 * nbin + 4 * nbin * Nmu
    out = torch.empty(2 * tot, dtype=torch.float64, device=full.device)
    call("pyspec_pk_rsd_python", ptr(full), n, int(irsd), -1.0 if Lbox is None else float(Lbox), int(Nmu), ptr(out),
         stream_ptr())
    o = out[:tot].cpu().numpy()
    k, p0, p2, p4, nk = (o[i * nbin:(i + 1) * nbin] for i in range(5))
    M = nbin * Nmu
    base = 5 * nbin
    km, mk, pkm, nkm = (o[base + i * M: base + (i + 1) * M].reshape(nbin, Nmu) for i in range(4))
    return k, p0, p2, p4, nk, km, mk, pkm, nkm


def pk_pbox_rsd(half: torch.Tensor, irsd: int, Lbox, Nmu: int):
    n = half.shape[0]
    nbin = n // 2
    tot = 5 * nbin + 4 * nbin * Nmu
    out = torch.empty(2 * tot, dtype=torch.float64, device=half.device)
    call("pyspec_pk_pbox_rsd", ptr(half), n, int(irsd), int(Lbox), nbin, int(Nmu), ptr(out), stream_ptr())
    o = out[:tot].cpu().numpy()
    k, p0, p2, p4, nk = (o[i * nbin:(i + 1) * nbin] for i in range(5))
    M = nbin * Nmu
    base = 5 * nbin
    km, mk, pkm, nkm = (o[base + i * M: base + (i + 1) * M].reshape(nbin, Nmu) for i in range(4))
    return k, p0, p2, p4, nk, km, mk, pkm, nkm


def efunc(z: float, omega0_m: float) -> float:
    """E(z) of flat LambdaCDM without radiation (astropy FlatLambdaCDM, Tcmb0=0)."""
    return math.sqrt(omega0_m * (1.0 + z) ** 3 + (1.0 - omega0_m))


def rsd_factor(redshift: float, omega0_m: float) -> float:
    """util.py:70: (1+z) / (100 E(z))."""
    return (1.0 + redshift) / (100.0 * efunc(redshift, omega0_m))
