"""Continuous-batching request loop over the batched engine.

Requests (one system each: positions, cell, cutoff, pbc) arrive over time.
The server keeps per-slot device arenas resident -- positions, workspace,
cell-list arrays and pair buffers, grown on demand and then reused -- and
runs up to ``slots`` batches at once, each on its own CUDA stream.  Whenever a
slot is free, every queued request that fits is admitted into one new batch:
admission is bounded by the predicted pair-buffer bytes of all in-flight
batches (``pair_budget_bytes``) and by the batch's atom and system limits, in
arrival order.  Requests that arrive while batches are on the GPU wait only
until a slot and budget free up; their batch then overlaps with the batches
still running.  A finished batch hands each request its own views of the
outputs (or copies, with ``copy_results``); a batch whose pairs exceed the
prediction is re-run with larger buffers.

``mode="plain"`` serves every request alone through the single-system entry
point on the same slots (the per-request baseline).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Deque, List, Optional

import numpy as np
import torch

from . import _lib
from ._lib import check, lib
from .api import _colmajor, _index_bytes, _pbc, _ptr, _tdtype, analyze_cell

_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)


@dataclass
class Request:
    rid: int
    X: object                  # (n, 3) positions of the server's dtype: numpy array, or a pinned torch tensor
    cell: np.ndarray           # 3x3, rows are lattice vectors
    cutoff: float
    pbc: tuple
    t_arrive: float = 0.0      # server clock (s)
    t_done: Optional[float] = None
    npairs: Optional[int] = None
    _res: Optional[tuple] = field(default=None, repr=False)

    @property
    def result(self) -> Optional[dict]:
        """first, i, j, S, R of this request (device tensors; host tensors from
        a server with ``host_results``).  Views into the slot's arenas are
        valid until that slot runs its next batch; a server with
        ``copy_results`` hands out copies."""
        if self._res is None:
            return None
        if isinstance(self._res, dict):
            return self._res
        first, i, j, S, R, f0, p0, p1 = self._res
        return {"first": first[f0:f0 + self.nat + 1], "i": i[p0:p1], "j": j[p0:p1],
                "S": S[3 * p0:3 * p1].view(-1, 3), "R": R[3 * p0:3 * p1].view(-1, 3) if R is not None else None}

    @property
    def nat(self) -> int:
        return int(self.X.shape[0])

    def predicted_pairs(self) -> int:
        """Expected pairs of a homogeneous system plus headroom."""
        p = self.__dict__.get("_pred")
        if p is None:
            vol = abs(float(np.linalg.det(np.asarray(self.cell, dtype=np.float64))))
            n = self.nat
            exp = n * (n / vol) * 4.0 / 3.0 * math.pi * self.cutoff ** 3 if vol > 0 else 0.0
            p = int(1.3 * exp + 8 * math.sqrt(exp + 1.0)) + 64
            self.__dict__["_pred"] = p
        return p


class _Slot:
    """One in-flight batch: stream, completion events and resident arenas
    (device buffers, and pinned host buffers for results copied back)."""

    def __init__(self, device, dtype=torch.float64):
        self.device = device
        self.dtype = dtype  # positions
        self.stream = torch.cuda.Stream(device=device)
        self.event = torch.cuda.Event()
        self.copy_event = torch.cuda.Event()
        self.bufs = {}
        self.hbufs = {}
        self.h_X = None
        self.reqs: List[Request] = []
        self.handle = None
        self.pred_bytes = 0
        self.busy = False
        self.copying = False  # the batch's results are on their way to the host

    def hbuf(self, name, numel, dtype):
        t = self.hbufs.get(name)
        if t is None or t.numel() < numel or t.dtype != dtype:
            t = torch.empty(max(int(numel * 1.25), 1), dtype=dtype).pin_memory()
            self.hbufs[name] = t
        return t

    def buf(self, name, numel, dtype):
        t = self.bufs.get(name)
        if t is None or t.numel() < numel or t.dtype != dtype:
            t = torch.empty(max(int(numel * 1.25), 1), dtype=dtype, device=self.device)
            self.bufs[name] = t
        return t

    def host_X(self, n):
        if self.h_X is None or self.h_X.shape[0] < n:
            self.h_X = torch.empty((max(int(n * 1.25), 1), 3), dtype=self.dtype).pin_memory()
        return self.h_X


class NeighbourListServer:
    def __init__(self, pair_budget_bytes: float = 40e9, slots: int = 3, max_batch_atoms: int = 4_000_000,
                 max_batch_systems: int = 8192, int_type=torch.int32, with_R: bool = True, device="cuda",
                 mode: str = "batched", copy_results: bool = False, host_results: bool = False,
                 dtype=torch.float64):
        """host_results: every batch's results (first, i, j, S, R) are copied
        into pinned host memory on the slot's stream, and a request is done --
        its latency stops -- when its results are on the host; the request's
        ``result`` is then host tensors.  dtype: float64, or float32 for the
        reference with T = Float32 (positions, cell, cutoff and R in Float32)."""
        if mode not in ("batched", "plain"):
            raise ValueError("mode must be 'batched' or 'plain'")
        if dtype not in (torch.float64, torch.float32):
            raise TypeError("positions must be float64 or float32")
        self.fdt = dtype
        self.f32 = dtype == torch.float32
        self.ib = _index_bytes(int_type)
        self.ti = _tdtype(self.ib)
        self.with_R = with_R
        self.device = torch.device(device)
        self.mode = mode
        self.copy_results = copy_results
        self.host_results = host_results
        self.direct_copy_atoms = 8192  # pinned requests at least this large skip the staging copy
        self.budget = float(pair_budget_bytes)
        self.max_atoms = int(max_batch_atoms)
        self.max_systems = int(max_batch_systems) if mode == "batched" else 1
        self.bytes_per_pair = 2 * self.ib + 3 * self.ib + ((12 if self.f32 else 24) if with_R else 0)
        self.slots = [_Slot(self.device, dtype) for _ in range(slots)]
        self.queue: Deque[Request] = deque()
        self.inflight_bytes = 0
        self.batches = 0
        self.reruns = 0

    # ----------------------------------------------------------- requests --
    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def busy(self) -> bool:
        return bool(self.queue) or any(s.busy for s in self.slots)

    def poll(self, now_fn=time.perf_counter) -> List[Request]:
        """Finishes every slot whose batch completed (with host_results: whose
        results reached the host); returns its requests."""
        done = []
        for s in self.slots:
            if s.busy and s.copying and s.copy_event.query():
                done.extend(self._release(s, now_fn()))
            elif s.busy and not s.copying and s.event.query():
                done.extend(self._finish(s, now_fn()))
        return done

    def admit(self) -> int:
        """Launches queued requests on free slots; returns requests admitted."""
        n = 0
        for s in self.slots:
            if s.busy or not self.queue:
                continue
            reqs, atoms, pred = [], 0, 0
            while self.queue and len(reqs) < self.max_systems:
                r = self.queue[0]
                rb = r.predicted_pairs() * self.bytes_per_pair
                if reqs and (atoms + r.nat > self.max_atoms or self.inflight_bytes + pred + rb > self.budget):
                    break
                if not reqs and self.inflight_bytes + rb > self.budget and any(x.busy for x in self.slots):
                    break  # wait for memory to free up
                reqs.append(self.queue.popleft())
                atoms += r.nat
                pred += rb
            if not reqs:
                break
            self._launch(s, reqs, pred)
            n += len(reqs)
        return n

    # ------------------------------------------------------------ batches --
    def _launch(self, s: _Slot, reqs: List[Request], pred_bytes: int) -> None:
        s.reqs, s.pred_bytes, s.busy = reqs, pred_bytes, True
        self.inflight_bytes += pred_bytes
        self.batches += 1
        nat = sum(r.nat for r in reqs)
        Xd = s.buf("X", 3 * max(nat, 1), self.fdt)
        with torch.cuda.stream(s.stream):
            if nat:
                # small requests are gathered into the slot's pinned staging
                # buffer and copied at once; large pinned ones are copied
                # directly (DMA, no host copy)
                hX = s.host_X(nat)
                hXn = hX.numpy()
                o, run0 = 0, 0
                for r in reqs:
                    direct = r.nat >= self.direct_copy_atoms and isinstance(r.X, torch.Tensor) and r.X.is_pinned()
                    if direct:
                        if o > run0:
                            Xd[3 * run0:3 * o].view(o - run0, 3).copy_(hX[run0:o], non_blocking=True)
                        Xd[3 * o:3 * (o + r.nat)].view(r.nat, 3).copy_(r.X, non_blocking=True)
                        run0 = o + r.nat
                    else:
                        hXn[o:o + r.nat] = r.X.numpy() if isinstance(r.X, torch.Tensor) else r.X
                    o += r.nat
                if o > run0:
                    Xd[3 * run0:3 * o].view(o - run0, 3).copy_(hX[run0:o], non_blocking=True)
            cap = max(sum(r.predicted_pairs() for r in reqs), 1)
            if self.mode == "batched":
                self._launch_batched(s, reqs, nat, cap)
            else:
                self._launch_plain(s, reqs[0], cap)
            s.event.record(s.stream)

    def _outputs(self, s: _Slot, cap: int):
        i = s.buf("i", cap, self.ti)
        j = s.buf("j", cap, self.ti)
        S = s.buf("S", 3 * cap, self.ti)
        R = s.buf("R", 3 * cap, self.fdt) if self.with_R else None
        return i, j, S, R, min(i.numel(), j.numel(), S.numel() // 3, R.numel() // 3 if R is not None else 1 << 62)

    def _launch_batched(self, s: _Slot, reqs: List[Request], nat: int, cap: int) -> None:
        L = lib()
        n = len(reqs)
        fnp = np.float32 if self.f32 else np.float64
        cells = np.ascontiguousarray(np.concatenate([_colmajor(r.cell) for r in reqs]).astype(fnp))
        cut = np.array([r.cutoff for r in reqs], dtype=fnp)
        pb = np.concatenate([_pbc(r.pbc) for r in reqs])
        nats = np.array([r.nat for r in reqs], dtype=np.int64)
        if s.handle is not None:
            L.nl_batch_destroy(s.handle)
            s.handle = None
        h = C.c_void_p()
        create = L.nl_batch_create_auto_f32 if self.f32 else L.nl_batch_create_auto
        check(create(C.c_void_p(cells.ctypes.data), C.c_void_p(cut.ctypes.data), pb.ctypes.data_as(_U8),
                     nats.ctypes.data_as(_I64), n, self.ib, C.byref(h)))
        s.handle = h
        na, nc = C.c_int64(), C.c_int64()
        check(L.nl_batch_sizes(h, C.byref(na), C.byref(nc)))
        ws = s.buf("ws", int(L.nl_batch_workspace_bytes(h)), torch.uint8)
        st = C.c_void_p(s.stream.cuda_stream)
        check(L.nl_batch_upload(h, _ptr(ws), ws.numel(), st))
        s.nc = int(nc.value)
        perm = s.buf("perm", max(nat, 1), self.ti)
        Xs = s.buf("Xs", 3 * max(nat, 1), self.fdt)
        cid = s.buf("cid", max(nat, 1), self.ti)
        offs = s.buf("offs", s.nc + n, self.ti)
        first = s.buf("first", nat + n, self.ti)
        po = s.buf("po", n + 1, torch.int64)
        i, j, S, R, capacity = self._outputs(s, cap)
        s.launch_args = (perm, Xs, cid, offs, first, po, ws)
        s.capacity = capacity
        run = L.nl_batch_neighbour_list_f32 if self.f32 else L.nl_batch_neighbour_list
        check(run(h, _ptr(s.bufs["X"]), _ptr(perm), _ptr(Xs), _ptr(cid), C.c_void_p(offs.data_ptr()),
                  C.c_void_p(first.data_ptr()), C.c_void_p(po.data_ptr()), capacity, _ptr(i), _ptr(j), _ptr(S), _ptr(R),
                  None, _ptr(ws), ws.numel(), st))

    def _launch_plain(self, s: _Slot, r: Request, cap: int) -> None:
        L = lib()
        plan = analyze_cell(r.cell, r.cutoff, self.ti, float32=self.f32)
        nat = r.nat
        ws = s.buf("ws", int(L.nl_workspace_bytes(nat, plan.ncells_total)), torch.uint8)
        perm = s.buf("perm", max(nat, 1), self.ti)
        Xs = s.buf("Xs", 3 * max(nat, 1), self.fdt)
        cid = s.buf("cid", max(nat, 1), self.ti)
        offs = s.buf("offs", plan.ncells_total + 1, self.ti)
        first = s.buf("first", nat + 1, self.ti)
        i, j, S, R, capacity = self._outputs(s, cap)
        pb = _pbc(r.pbc)
        s.launch_args = (plan, ws, first)
        s.capacity = capacity
        one = L.nl_neighbour_list_f32 if self.f32 else L.nl_neighbour_list
        rc = float(np.float32(r.cutoff)) if self.f32 else float(r.cutoff)
        fp = C.POINTER(C.c_float) if self.f32 else _D
        check(one(_ptr(s.bufs["X"]), nat, plan.cell_cm.ctypes.data_as(fp), plan.inv_cm.ctypes.data_as(fp),
                  plan.ncells.ctypes.data_as(_I64), plan.nxyz.ctypes.data_as(_I64), pb.ctypes.data_as(_U8), rc,
                  self.ib, _ptr(perm), _ptr(Xs), _ptr(cid), C.c_void_p(offs.data_ptr()), C.c_void_p(first.data_ptr()),
                  capacity, _ptr(i), _ptr(j), _ptr(S), _ptr(R), None, _ptr(ws), ws.numel(),
                  C.c_void_p(s.stream.cuda_stream)))

    def _finish(self, s: _Slot, t_done: float) -> List[Request]:
        L = lib()
        st = C.c_void_p(s.stream.cuda_stream)
        if self.mode == "batched":
            perm, Xs, cid, offs, first, po, ws = s.launch_args
            n = len(s.reqs)
            po_h = po[:n + 1].cpu().numpy()
            total = int(po_h[-1])
        else:
            plan, ws, first = s.launch_args
            total = int(first[s.reqs[0].nat].item()) - 1
            po_h = np.array([0, total], dtype=np.int64)
        status = L.nl_sync_status(_ptr(ws), st)
        if status == _lib.NL_ERR_CAPACITY or total > s.capacity:
            # more pairs than predicted: run the batch again with room for all
            self.reruns += 1
            with torch.cuda.stream(s.stream):
                if self.mode == "batched":
                    nat = sum(r.nat for r in s.reqs)
                    self._launch_batched(s, s.reqs, nat, total)
                else:
                    self._launch_plain(s, s.reqs[0], total)
            s.stream.synchronize()
            return self._finish(s, t_done)
        check(status)
        i, j, S, R = s.bufs["i"], s.bufs["j"], s.bufs["S"], s.bufs.get("R")
        if self.host_results:
            # one copy per array for the whole batch into the slot's pinned arenas
            nf = sum(r.nat for r in s.reqs) + (len(s.reqs) if self.mode == "batched" else 1)
            hf = s.hbuf("first", nf, self.ti)
            hi, hj = s.hbuf("i", max(total, 1), self.ti), s.hbuf("j", max(total, 1), self.ti)
            hS = s.hbuf("S", 3 * max(total, 1), self.ti)
            hR = s.hbuf("R", 3 * max(total, 1), self.fdt) if R is not None else None
            with torch.cuda.stream(s.stream):
                hf[:nf].copy_(first[:nf], non_blocking=True)
                if total:
                    hi[:total].copy_(i[:total], non_blocking=True)
                    hj[:total].copy_(j[:total], non_blocking=True)
                    hS[:3 * total].copy_(S[:3 * total], non_blocking=True)
                    if hR is not None:
                        hR[:3 * total].copy_(R[:3 * total], non_blocking=True)
                s.copy_event.record(s.stream)
            s.copying = True
            s.po_h = po_h
            s.host = (hf, hi, hj, hS, hR)
            return []
        a0 = 0
        for k, r in enumerate(s.reqs):
            p0, p1 = int(po_h[k]), int(po_h[k + 1])
            f0 = a0 + k if self.mode == "batched" else 0
            r._res = (first, i, j, S, R, f0, p0, p1)  # views are made on access
            if self.copy_results:
                r._res = {key: (v.clone() if v is not None else None) for key, v in r.result.items()}
            r.npairs, r.t_done = p1 - p0, t_done
            a0 += r.nat
        return self._free(s)

    def _release(self, s: _Slot, t_done: float) -> List[Request]:
        """The batch's results are on the host: hand each request its slices."""
        hf, hi, hj, hS, hR = s.host
        a0 = 0
        for k, r in enumerate(s.reqs):
            p0, p1 = int(s.po_h[k]), int(s.po_h[k + 1])
            f0 = a0 + k if self.mode == "batched" else 0
            r._res = (hf, hi, hj, hS, hR, f0, p0, p1)
            if self.copy_results:  # the pinned arenas are reused by the slot's next batch
                r._res = {key: (v.clone() if v is not None else None) for key, v in r.result.items()}
            r.npairs, r.t_done = p1 - p0, t_done
            a0 += r.nat
        s.copying = False
        return self._free(s)

    def _free(self, s: _Slot) -> List[Request]:
        done = s.reqs
        s.reqs, s.busy = [], False
        self.inflight_bytes -= s.pred_bytes
        s.pred_bytes = 0
        return done

    def close(self) -> None:
        for s in self.slots:
            if s.handle is not None:
                lib().nl_batch_destroy(s.handle)
                s.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- traces --
    def run_trace(self, requests: List[Request], idle_sleep: float = 20e-6) -> dict:
        """Serves requests whose t_arrive are offsets (s) from the start, with
        the wall clock as the arrival clock.  Returns latency / throughput."""
        reqs = sorted(requests, key=lambda r: r.t_arrive)
        t0 = time.perf_counter()
        k = 0
        while k < len(reqs) or self.busy():
            now = time.perf_counter() - t0
            while k < len(reqs) and reqs[k].t_arrive <= now:
                self.submit(reqs[k])
                k += 1
            finished = self.poll(lambda: time.perf_counter() - t0)
            launched = self.admit()
            if launched or finished:
                continue
            if not self.busy() and k < len(reqs):
                # idle until the next arrival
                time.sleep(max(0.0, min(reqs[k].t_arrive - (time.perf_counter() - t0), 1e-3)))
            else:
                time.sleep(idle_sleep)
        wall = time.perf_counter() - t0
        lat = np.array([r.t_done - r.t_arrive for r in reqs]) * 1e3
        pairs = sum(r.npairs for r in reqs)
        span = max(r.t_done for r in reqs) - min(r.t_arrive for r in reqs)
        return {"requests": len(reqs), "batches": self.batches, "reruns": self.reruns,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "systems_per_s": len(reqs) / span, "pairs_per_s": pairs / span,
                "wall_s": wall}


def poisson_trace(systems, rate: float, seed: int = 0) -> List[Request]:
    """Requests for (X, cell, cutoff, pbc) tuples with Poisson arrivals."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=len(systems)))
    return [Request(k, x, c, rc, p, float(t[k])) for k, (x, c, rc, p) in enumerate(systems)]
