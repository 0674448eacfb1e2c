"""Reusable materialised neighbour-list pipeline (one system, fixed size).

Keeps the workspace, the SortedCellList arrays and the pair buffers resident
on the device between calls, as an MD loop that rebuilds its list every step
would.  One call of ``launch`` enqueues the whole path (nl_neighbour_list:
binning, sort, count, scan, fill) on a stream with no host synchronisation;
``run`` additionally checks the pair count and grows the buffers when needed.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import _lib
from ._lib import check, lib
from .api import PairList, SortedCellList, _index_bytes, _pbc, _ptr, _stream_handle, _tdtype, analyze_cell

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I64 = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)


class NeighbourListEngine:
    """``dtype=torch.float32`` runs the single-precision path (positions, cell,
    cutoff and R in Float32, the reference with T = Float32)."""

    def __init__(self, nat: int, cell, cutoff: float, pbc, int_type=torch.int32, with_R: bool = True,
                 capacity: Optional[int] = None, device="cuda", half: bool = False, dtype=torch.float64):
        if dtype not in (torch.float64, torch.float32):
            raise TypeError("dtype must be torch.float64 or torch.float32")
        self.f32 = dtype == torch.float32
        self.dtype = dtype
        self.nat = int(nat)
        self.cell = np.asarray(cell, dtype=np.float64).reshape(3, 3).astype(np.float32 if self.f32 else np.float64)
        self.cutoff = np.float32(cutoff).item() if self.f32 else float(cutoff)
        self.pbc = _pbc(pbc)
        self.ib = _index_bytes(int_type)
        self.ti = _tdtype(self.ib)
        self.with_R = with_R
        self.half = bool(half)  # keep each unordered pair once (nl_neighbour_list_half[_f32])
        self.device = torch.device(device)
        self.plan = analyze_cell(self.cell, self.cutoff, int_type, float32=self.f32)
        p = self.plan
        nbytes = int(lib().nl_workspace_bytes(self.nat, p.ncells_total))
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.perm = torch.empty(self.nat, dtype=self.ti, device=self.device)
        self.Xs = torch.empty((self.nat, 3), dtype=dtype, device=self.device)
        self.cid = torch.empty(self.nat, dtype=self.ti, device=self.device)
        self.offs = torch.empty(p.ncells_total + 1, dtype=self.ti, device=self.device)
        self.first = torch.empty(self.nat + 1, dtype=self.ti, device=self.device)
        self.capacity = 0
        self.i = self.j = self.S = self.R = None
        if capacity is None:
            # expected pairs for a homogeneous system plus headroom
            vol = abs(float(np.linalg.det(self.cell.astype(np.float64))))
            rho = self.nat / vol if vol > 0 else 0.0
            capacity = int(1.15 * self.nat * rho * 4.0 / 3.0 * np.pi * self.cutoff ** 3 / (2 if half else 1)) + 1024
        self._alloc(capacity)
        self.last_total = None
        self.tuning = _lib.Tuning(0, 0, 0)
        self._graph = None

    def _alloc(self, capacity: int):
        capacity = max(int(capacity), 1)
        self.capacity = capacity
        self.i = torch.empty(capacity, dtype=self.ti, device=self.device)
        self.j = torch.empty(capacity, dtype=self.ti, device=self.device)
        self.S = torch.empty((capacity, 3), dtype=self.ti, device=self.device)
        self.R = torch.empty((capacity, 3), dtype=self.dtype, device=self.device) if self.with_R else None

    def _call(self, X: torch.Tensor, total_ptr, stream, outputs=None):
        p = self.plan
        check(lib().nl_set_tuning(C.byref(self.tuning)))
        if self.f32:
            entry, fp = (lib().nl_neighbour_list_half_f32 if self.half else lib().nl_neighbour_list_f32), _F
        else:
            entry, fp = (lib().nl_neighbour_list_half if self.half else lib().nl_neighbour_list), _D
        if X.dtype != self.dtype:
            raise TypeError(f"positions must be {self.dtype}")
        i, j, S, R, cap = outputs if outputs is not None else (self.i, self.j, self.S, self.R, self.capacity)
        return entry(
            _ptr(X), self.nat, p.cell_cm.ctypes.data_as(fp), p.inv_cm.ctypes.data_as(fp), p.ncells.ctypes.data_as(_I64),
            p.nxyz.ctypes.data_as(_I64), self.pbc.ctypes.data_as(_U8), self.cutoff, self.ib, _ptr(self.perm),
            _ptr(self.Xs), _ptr(self.cid), C.c_void_p(self.offs.data_ptr()), C.c_void_p(self.first.data_ptr()),
            cap, _ptr(i), _ptr(j), _ptr(S), _ptr(R), total_ptr, _ptr(self.ws),
            self.ws.numel(), _stream_handle(stream))

    def launch(self, X: torch.Tensor, stream=None) -> None:
        """Enqueue the whole pipeline; no host synchronisation."""
        check(self._call(X, None, stream))

    def run(self, X: torch.Tensor, stream=None) -> int:
        """Run the pipeline, check errors, grow the pair buffers if needed."""
        total = C.c_int64(0)
        s = self._call(X, C.byref(total), stream)
        if s == _lib.NL_ERR_CAPACITY:
            self._alloc(int(total.value * 1.1) + 1024)
            s = self._call(X, C.byref(total), stream)
        check(s)
        self.last_total = int(total.value)
        return self.last_total

    def set_tuning(self, pair_blocks_per_sm: int = 0, emit_blocks_per_sm: int = 0, count_kernel: int = 0) -> None:
        """Launch shapes of this engine's calls (nl_set_tuning; 0 = default).
        count_kernel: 0 the symmetric pass where the stencil allows it, else 1;
        1 one warp per home cell; 2 one thread per home atom; 3 symmetric where
        it applies.  Results never depend on them."""
        self.tuning = _lib.Tuning(int(pair_blocks_per_sm), int(emit_blocks_per_sm), int(count_kernel))

    def capture(self, X: torch.Tensor) -> torch.cuda.CUDAGraph:
        """Captures one launch on X in a CUDA graph; ``replay()`` re-runs it."""
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.launch(X)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(X)
        self._graph = g
        return g

    def replay(self) -> None:
        self._graph.replay()

    def launch_host(self, hX: torch.Tensor, out: dict, copy_streams: int = 4, stream=None,
                    direct: bool = False) -> None:
        """End to end with host buffers: copies pinned positions ``hX`` in,
        runs the pipeline, and brings first / i / j / S / R back into the
        pinned host tensors of ``out`` (keys "first", "i", "j", "S", "R"; the
        pair arrays sized for the expected pair count).

        direct=False: the pairs are written to the device buffers and copied
        out, spread over ``copy_streams`` streams so that several copy engines
        run at once.  direct=True: the write pass stores i, j, S, R straight
        into the pinned host tensors (they are addressable from the GPU) and
        only ``first`` is copied.  ``stream`` (default: current) waits for
        everything, so work or events recorded on it afterwards see the
        finished outputs."""
        main = stream if stream is not None else torch.cuda.current_stream(self.device)
        if getattr(self, "_Xdev", None) is None or self._Xdev.shape[0] != self.nat:
            self._Xdev = torch.empty((self.nat, 3), dtype=self.dtype, device=self.device)
        if direct:
            P = out["i"].shape[0]
            for key in ("i", "j", "S", "R"):
                t = out.get(key)
                if t is not None and not t.is_pinned():
                    raise ValueError("direct output needs pinned host tensors")
            with torch.cuda.stream(main):
                self._Xdev.copy_(hX, non_blocking=True)
                check(self._call(self._Xdev, None, main, outputs=(out["i"], out["j"], out["S"], out.get("R"), P)))
                out["first"].copy_(self.first, non_blocking=True)
            return
        if len(getattr(self, "_copy_streams", [])) != copy_streams:
            self._copy_streams = [torch.cuda.Stream(device=self.device) for _ in range(copy_streams)]
        with torch.cuda.stream(main):
            self._Xdev.copy_(hX, non_blocking=True)
            self.launch(self._Xdev, main)
            done = torch.cuda.Event()
            done.record(main)
        P = out["i"].shape[0]
        jobs = [(out["first"], self.first), (out["i"], self.i[:P]), (out["j"], self.j[:P]), (out["S"], self.S[:P])]
        if out.get("R") is not None:
            h = P // 2  # the largest array goes in two halves
            jobs += [(out["R"][:h], self.R[:h]), (out["R"][h:], self.R[h:P])]
        for k, (dst, src) in enumerate(jobs):
            cs = self._copy_streams[k % copy_streams]
            cs.wait_event(done)
            with torch.cuda.stream(cs):
                dst.copy_(src, non_blocking=True)
        for cs in self._copy_streams:
            main.wait_stream(cs)

    def sync_status(self, stream=None) -> None:
        check(lib().nl_sync_status(_ptr(self.ws), _stream_handle(stream)))

    def total_pairs(self) -> int:
        """Pair count of the last launch (reads the device; synchronises)."""
        return int(self.first[-1].item()) - 1

    def rechecks(self, stream=None) -> int:
        r = C.c_int64(0)
        check(lib().nl_last_recheck_count(_ptr(self.ws), _stream_handle(stream), C.byref(r)))
        return int(r.value)

    def cell_list(self, X: torch.Tensor) -> SortedCellList:
        """The SortedCellList of the last launch (shares the workspace, whose
        records lazy_reduce reuses)."""
        p = self.plan
        return SortedCellList(self.Xs, X, self.perm, self.cid, self.offs, self.cell.copy(), p.inv_cell,
                              tuple(bool(b) for b in self.pbc), self.cutoff, p.ncells, p.ncells_total, p, self.ws,
                              True)

    def pairlist(self, X: torch.Tensor) -> PairList:
        P = self.total_pairs()
        return PairList(X, self.cell.copy(), self.cutoff, self.i[:P], self.j[:P], self.S[:P], self.first,
                        self.R[:P] if self.R is not None else None)
