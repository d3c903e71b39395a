"""Bispectra of many periodic boxes in one call.

A survey-style analysis evaluates B0/Q0 on tens of mocks of different
particle counts and grid sizes.  ``Bk_periodic_batch`` runs them back to back
on one GPU with per-geometry state kept across mocks:

* one plan per grid size (shell fields, workspaces, triangle tables, exact
  counts computed once per geometry);
* the geometry-only part of each evaluation (40 masked inverse FFTs -> shell
  fields -> triangle contraction, about 125 kernel launches at Nmax 40) is
  captured once into a CUDA graph and replayed for every later mock of that
  geometry; the particle-dependent part (clip/cast, PCS assignment, FFT,
  interlacing combine) and the normalisation (whose shot-noise terms depend on
  the particle count) stay ordinary launches;
* the next mock's positions are copied from page-locked host memory on a
  second stream while the current mock computes, and each result is read back
  asynchronously into page-locked memory.

Each result dict has the keys of ``pyspectrum.Bk_periodic`` (pyspectrum.py:
285-356), computed by the same kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import core


class _Geometry:
    def __init__(self, n, step, ncut, nmax, method, device, graphs):
        self.plan = core.get_plan(n, step, ncut, nmax, method, device)
        self.grid = torch.zeros((n, n, n), dtype=torch.complex64, device=device)
        self.half = torch.empty((n, n, n // 2 + 1), dtype=torch.complex64, device=device)
        self.graphs = graphs
        self.graph = None
        self.runs = 0

    def device_part(self):
        """Shells + contraction from self.half (graph-replayed after the first run)."""
        if not self.graphs:
            self.plan.shells(self.half)
            self.plan.contract()
            return
        if self.graph is None and self.runs >= 1:
            # captured after one eager run: plans, kernel attributes and the
            # page-locked table images already exist
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream(device=self.half.device)
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    self.plan.shells(self.half)
                    self.plan.contract()
            torch.cuda.current_stream().wait_stream(s)
            self.graph = g
        if self.graph is not None:
            self.graph.replay()
        else:
            self.plan.shells(self.half)
            self.plan.contract()
        self.runs += 1


class BkBatch:
    """Reusable runner: keeps the per-geometry plans, buffers and graphs."""

    def __init__(self, Lbox=2500.0, step=3, Ncut=3, Nmax=40, method="bf16x3", graphs=True, device=None):
        self.device = core._dev(device)
        self.Lbox, self.step, self.ncut, self.nmax = float(Lbox), int(step), int(Ncut), int(Nmax)
        self.method = method
        self.graphs = bool(graphs)
        self._geo: dict = {}
        self._copy_stream = torch.cuda.Stream(device=self.device)

    def geometry(self, n) -> _Geometry:
        g = self._geo.get(int(n))
        if g is None:
            g = _Geometry(int(n), self.step, self.ncut, self.nmax, self.method, self.device, self.graphs)
            self._geo[int(n)] = g
        return g

    def _upload(self, xyz):
        """Start the host->device copy of one mock's positions on the copy stream."""
        t = torch.as_tensor(xyz)
        if t.dim() != 2 or t.shape[0] != 3:
            raise ValueError("positions must be a 3 x N array")
        if t.is_cuda:
            return t.to(self.device, torch.float64).contiguous(), None
        t = t.to(torch.float64).contiguous()
        if not t.is_pinned():
            t = t.pin_memory()
        with torch.cuda.stream(self._copy_stream):
            d = t.to(self.device, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self._copy_stream)
        return d, (ev, t)

    def run(self, mocks):
        """mocks: sequence of (xyz (3, Np), Ngrid) or (xyz, Ngrid, w).  Returns
        a list of Bk_periodic dictionaries, in order."""
        mocks = list(mocks)
        L = self.Lbox
        kf = 2 * np.pi / L
        cur = torch.cuda.current_stream(self.device)
        pending = self._upload(mocks[0][0]) if mocks else None
        staged = []
        for idx, m in enumerate(mocks):
            xyz, n = m[0], int(m[1])
            w = m[2] if len(m) > 2 else None
            xyz_d, guard = pending
            if guard is not None:
                cur.wait_event(guard[0])
                xyz_d.record_stream(cur)
            pending = self._upload(mocks[idx + 1][0]) if idx + 1 < len(mocks) else None
            npart = xyz_d.shape[1]
            wsum = float(npart) if w is None else float(np.sum(np.asarray(w, dtype=np.float64)))
            nbar = wsum / L ** 3
            w_d = None if w is None else torch.as_tensor(np.asarray(w, dtype=np.float64), device=self.device)
            geo = self.geometry(n)
            xyzs, ws = core.prepare_positions(xyz_d, L, w_d)
            core.fft_periodic_half(xyzs, ws, n, L, wsum, grid=geo.grid, half=geo.half)
            geo.device_part()
            geo.plan.normalize(True, nbar, kf)
            host = torch.empty(geo.plan.out.shape, dtype=torch.float64, pin_memory=True)
            host.copy_(geo.plan.out, non_blocking=True)
            status = None
            if self.method in core.TENSOR_METHODS:     # the contraction's status word of this mock
                status = torch.empty(1, dtype=torch.int32, pin_memory=True)
                status.copy_(geo.plan.status_word(), non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(cur)
            staged.append((ev, host, status, geo, n, npart, nbar))
        results = []
        for ev, host, status, geo, n, npart, nbar in staged:
            ev.synchronize()
            if status is not None:
                core.check_contract_status(int(status[0]))
            results.append(_result_dict(geo.plan, host.numpy(), L, n, self.step, self.ncut, self.nmax, npart,
                                        nbar, kf))
        return results


def _result_dict(plan, out, Lbox, n, step, ncut, nmax, npart, nbar, kf):
    keep = plan.counts_np > 0
    tri = plan.tri_np[:, keep]
    return {
        "i_k1": tri[0].astype(np.int64) * step, "i_k2": tri[1].astype(np.int64) * step,
        "i_k3": tri[2].astype(np.int64) * step,
        "p0k1": out[0, keep], "p0k2": out[1, keep], "p0k3": out[2, keep],
        "b123": out[3, keep], "q123": out[4, keep], "counts": out[5, keep], "b123_sn": out[6, keep],
        "p0k_sn": 1.0 / nbar,
        "meta": {"Lbox": Lbox, "Ngrid": n, "step": step, "Ncut": ncut, "Nmax": nmax, "N": npart, "nbar": nbar,
                 "kf": kf},
    }


def Bk_periodic_batch(mocks, Lbox=2500.0, step=3, Ncut=3, Nmax=40, method="bf16x3", graphs=True, device=None):
    """B0/Q0 of many periodic boxes (positions in [0, Lbox)^3, one grid size
    per mock).  ``mocks``: sequence of (xyz, Ngrid) or (xyz, Ngrid, w)."""
    return BkBatch(Lbox, step, Ncut, Nmax, method, graphs, device).run(mocks)
