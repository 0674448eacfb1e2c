"""Many independent systems in one pass per stage (nl_batch_* of the C ABI).

The reference handles one system per ``neighbour_list`` call
(src/cell_list.jl:897-916).  A batch runs binning, sorting, counting and
filling of every system with one launch per stage: the systems' atoms and
cells are concatenated, each warp looks up the system of its home cell, and
every per-system output keeps the reference's layout and 1-based,
system-local values (see include/nlgpu.h).  ``system(s)`` returns system s's
SortedCellList / PairList views, bit-identical to a single-system call.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import check, lib
from .api import PairList, SortedCellList, _index_bytes, _pbc, _ptr, _stream_handle, _tdtype, analyze_cell

_I64 = C.POINTER(C.c_int64)


class BatchNeighbourList:
    """Materialised neighbour lists of a fixed set of systems.

    ``systems`` is a sequence of (nat, cell, cutoff, pbc); the positions of
    all systems are passed concatenated, system after system, as one (N, 3)
    CUDA tensor of ``dtype``: float64, or float32 for the reference with
    T = Float32 (cell and cutoff converted to Float32, every operation in
    single precision, R in float32; test/test_gpu.jl:14).
    """

    def __init__(self, systems: Sequence[Tuple[int, object, float, object]], int_type=torch.int32,
                 with_R: bool = True, capacity: Optional[int] = None, device="cuda", dtype=torch.float64):
        if dtype not in (torch.float64, torch.float32):
            raise TypeError("positions must be float64 or float32")
        self.ib = _index_bytes(int_type)
        self.ti = _tdtype(self.ib)
        self.with_R = with_R
        self.device = torch.device(device)
        self.dtype = dtype
        self.f32 = dtype == torch.float32
        n = len(systems)
        arr = ((_lib.SystemF32 if self.f32 else _lib.System) * max(n, 1))()
        self.cells, self.cutoffs, self.pbcs, self.nats = [], [], [], []
        exp_pairs = 0.0
        for s, (nat, cell, cutoff, pbc) in enumerate(systems):
            cellm = np.asarray(cell, dtype=np.float64).reshape(3, 3).copy()
            if self.f32:
                cellm = cellm.astype(np.float32)
            plan = analyze_cell(cellm, cutoff, int_type, float32=self.f32)
            pb = _pbc(pbc)
            y = arr[s]
            y.nat = int(nat)
            y.cell[:] = plan.cell_cm.tolist()
            y.inv_cell[:] = plan.inv_cm.tolist()
            y.ncells[:] = plan.ncells.tolist()
            y.nxyz[:] = plan.nxyz.tolist()
            y.pbc[:] = pb.tolist()
            y.cutoff = float(np.float32(cutoff)) if self.f32 else float(cutoff)
            self.cells.append(cellm)
            self.cutoffs.append(float(cutoff))
            self.pbcs.append(tuple(bool(b) for b in pb))
            self.nats.append(int(nat))
            vol = abs(float(np.linalg.det(cellm)))
            if vol > 0:
                exp_pairs += nat * (nat / vol) * 4.0 / 3.0 * np.pi * float(cutoff) ** 3
        h = C.c_void_p()
        create = lib().nl_batch_create_f32 if self.f32 else lib().nl_batch_create
        check(create(arr, n, self.ib, C.byref(h)))
        self._h = h
        self.nsys = n
        na, nc = C.c_int64(), C.c_int64()
        check(lib().nl_batch_sizes(h, C.byref(na), C.byref(nc)))
        self.nat_total, self.ncells_total = int(na.value), int(nc.value)
        self.atom0 = np.concatenate([[0], np.cumsum(self.nats)]).astype(np.int64)
        ncs = [int(arr[s].ncells[0] * arr[s].ncells[1] * arr[s].ncells[2]) for s in range(n)]
        self.cell0 = np.concatenate([[0], np.cumsum(ncs)]).astype(np.int64)
        dev = self.device
        self.ws = torch.empty(int(lib().nl_batch_workspace_bytes(h)), dtype=torch.uint8, device=dev)
        with torch.cuda.device(dev):
            check(lib().nl_batch_upload(h, _ptr(self.ws), self.ws.numel(), _stream_handle(None)))
        N = self.nat_total
        self.perm = torch.empty(N, dtype=self.ti, device=dev)
        self.Xs = torch.empty((N, 3), dtype=dtype, device=dev)
        self.cid = torch.empty(N, dtype=self.ti, device=dev)
        self.offs = torch.empty(self.ncells_total + n, dtype=self.ti, device=dev)
        self.first = torch.empty(N + n, dtype=self.ti, device=dev)
        self.pair_offsets = torch.empty(n + 1, dtype=torch.int64, device=dev)
        if capacity is None:
            capacity = int(1.2 * exp_pairs) + 4096
        self._alloc(capacity)
        self.last_total = None
        self._po_host = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().nl_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def _alloc(self, capacity: int):
        capacity = max(int(capacity), 1)
        self.capacity = capacity
        dev = self.device
        self.i = torch.empty(capacity, dtype=self.ti, device=dev)
        self.j = torch.empty(capacity, dtype=self.ti, device=dev)
        self.S = torch.empty((capacity, 3), dtype=self.ti, device=dev)
        self.R = torch.empty((capacity, 3), dtype=self.dtype, device=dev) if self.with_R else None

    def _call(self, X: torch.Tensor, total_ptr, stream):
        if X.dtype != self.dtype or tuple(X.shape) != (self.nat_total, 3) or not X.is_cuda:
            raise ValueError(f"positions must be a ({self.nat_total}, 3) {str(self.dtype)[6:]} CUDA tensor")
        X = X.contiguous()
        run = lib().nl_batch_neighbour_list_f32 if self.f32 else lib().nl_batch_neighbour_list
        return run(
            self._h, _ptr(X), _ptr(self.perm), _ptr(self.Xs), _ptr(self.cid), C.c_void_p(self.offs.data_ptr()),
            C.c_void_p(self.first.data_ptr()), C.c_void_p(self.pair_offsets.data_ptr()), self.capacity, _ptr(self.i),
            _ptr(self.j), _ptr(self.S), _ptr(self.R), total_ptr, _ptr(self.ws), self.ws.numel(),
            _stream_handle(stream))

    def launch(self, X: torch.Tensor, stream=None) -> None:
        """Enqueue every stage for every system; no host synchronisation."""
        self._po_host = None
        check(self._call(X, None, stream))

    def run(self, X: torch.Tensor, stream=None) -> int:
        """Run, check device-side errors, grow the pair buffers if needed."""
        self._po_host = None
        total = C.c_int64(0)
        s = self._call(X, C.byref(total), stream)
        if s == _lib.NL_ERR_CAPACITY:
            self._alloc(int(total.value * 1.1) + 4096)
            s = self._call(X, C.byref(total), stream)
        check(s)
        self.last_total = int(total.value)
        return self.last_total

    def set_tuning(self, pair_blocks_per_sm: int = 0, emit_blocks_per_sm: int = 0, count_kernel: int = 0) -> None:
        """Launch shapes (nl_batch_set_tuning; 0 = default).  count_kernel: 1
        one warp per home cell, 2 one thread per home atom, 0 or 3 the
        symmetric pass for the systems whose 27-cell stencil has distinct cells
        (the per-cell pass for the others).  Results never depend on them."""
        t = _lib.Tuning(int(pair_blocks_per_sm), int(emit_blocks_per_sm), int(count_kernel))
        check(lib().nl_batch_set_tuning(self._h, C.byref(t)))

    def capture(self, X: torch.Tensor) -> torch.cuda.CUDAGraph:
        """Captures one launch on X in a CUDA graph (the buffers stay fixed);
        ``replay()`` re-runs every stage of every system with one graph launch."""
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.launch(X)  # first launch outside the capture
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(X)
        self._graph = g
        return g

    def replay(self) -> None:
        self._po_host = None
        self._graph.replay()

    def sync_status(self, stream=None) -> None:
        check(lib().nl_sync_status(_ptr(self.ws), _stream_handle(stream)))

    def pair_offsets_host(self) -> np.ndarray:
        if self._po_host is None:
            self._po_host = self.pair_offsets.cpu().numpy()
        return self._po_host

    def system(self, s: int, X: Optional[torch.Tensor] = None):
        """(SortedCellList, PairList) of system s: views into the batch buffers."""
        a0, a1 = int(self.atom0[s]), int(self.atom0[s + 1])
        c0 = int(self.cell0[s]) + s
        c1 = int(self.cell0[s + 1]) + s + 1
        po = self.pair_offsets_host()
        p0, p1 = int(po[s]), int(po[s + 1])
        Xo = X[a0:a1] if X is not None else None
        plan = analyze_cell(self.cells[s], self.cutoffs[s], self.ti, float32=self.f32)
        clist = SortedCellList(self.Xs[a0:a1], Xo, self.perm[a0:a1], self.cid[a0:a1], self.offs[c0:c1],
                               self.cells[s], plan.inv_cell, self.pbcs[s], self.cutoffs[s], plan.ncells,
                               plan.ncells_total, plan)
        pl = PairList(Xo, self.cells[s], self.cutoffs[s], self.i[p0:p1], self.j[p0:p1], self.S[p0:p1],
                      self.first[a0 + s:a1 + s + 1], self.R[p0:p1] if self.R is not None else None)
        return clist, pl
