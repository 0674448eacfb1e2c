"""Host-side mirror of the NeighbourLists.jl API for the GPU path.

Same names, argument meaning and error behaviour as the reference's unified
API (src/cell_list.jl:839-927) and data types (src/types.jl:34-82):

    neighbour_list(X, cutoff, cell, pbc; lazy, int_type) -> PairList | SortedCellList
    build_cell_list(X, cutoff, cell, pbc; int_type)       -> SortedCellList
    materialize_pairlist(clist)                           -> PairList
    npairs, nsites, nneigs, maxneigs/max_neighbours, neigs, neigss, neighbours,
    num_neighbours, count_neighbours, for_each_neighbour

Differences a caller sees:
  * arrays live on the GPU as torch tensors (the reference's CuArrays);
  * indices (i, j, perm, cell_id, cell_offsets, first) are 1-based, as in the
    reference, in int32 (Int32, default) or int64 (Int64);
  * PairList additionally carries R (npairs x 3 float64), bit-equal to the
    reference's _getR (cell_list.jl:525-531).

``cell`` is 3x3 with ROWS = lattice vectors (``cell[k, :]`` is vector k),
exactly like the reference.  Every call goes through libnlgpu.so; there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Callable, Optional, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import NLError, check, lib

__all__ = [
    "SortedCellList", "PairList", "NLError", "analyze_cell", "build_cell_list", "materialize_pairlist",
    "neighbour_list", "npairs", "nsites", "nneigs", "maxneigs", "max_neighbours", "neigs", "neigss", "neighbours",
    "num_neighbours", "count_neighbours", "for_each_neighbour", "lazy_reduce", "cutoff", "pairs", "sites",
    "PairIterator", "SiteIterator", "pair_vectors", "legacy_pairlist", "query_neighbours",
]

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I64 = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)


# ----------------------------------------------------------------- helpers --
def _index_bytes(int_type) -> int:
    if int_type in (torch.int32, np.int32, "Int32", "int32"):
        return 4
    if int_type in (torch.int64, np.int64, "Int64", "int64"):
        return 8
    raise ValueError(f"int_type must be Int32 or Int64, got {int_type!r}")


def _tdtype(index_bytes: int):
    return torch.int32 if index_bytes == 4 else torch.int64


def _colmajor(cell) -> np.ndarray:
    c = np.asarray(cell, dtype=np.float64)
    if c.shape != (3, 3):
        raise ValueError("cell must be a 3x3 matrix (rows are lattice vectors)")
    return np.ascontiguousarray(c.T).reshape(9)


def _pbc(pbc) -> np.ndarray:
    p = [bool(b) for b in pbc]
    if len(p) != 3:
        raise ValueError("pbc must have 3 entries")
    return np.array([1 if b else 0 for b in p], dtype=np.uint8)


def _ptr(t: Optional[torch.Tensor]):
    return C.c_void_p(t.data_ptr()) if t is not None and t.numel() > 0 else C.c_void_p(0)


def _stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _device_positions(X, f32_ok: bool = False) -> torch.Tensor:
    """(N,3) float64 contiguous CUDA tensor -- or float32 where the call has a
    single-precision path (f32_ok); host arrays are copied to the GPU."""
    if isinstance(X, torch.Tensor):
        t = X
    else:
        a = np.asarray(X)
        dt = np.float32 if (f32_ok and a.dtype == np.float32) else np.float64
        t = torch.from_numpy(np.ascontiguousarray(a.astype(dt, copy=False).reshape(-1, 3)))
    if t.dtype != torch.float64 and not (f32_ok and t.dtype == torch.float32):
        raise TypeError("positions must be Float64 (float64)" + (" or Float32 (float32)" if f32_ok else ""))
    t = t.reshape(-1, 3)
    if not t.is_cuda:
        t = t.to("cuda", non_blocking=False)
    return t.contiguous()


@dataclass
class CellPlan:
    """analyze_cell (cell_list.jl:152-170) + nxyz (gpu_kernels.jl:315-316)."""
    cell_cm: np.ndarray        # 9 doubles, column-major
    inv_cm: np.ndarray         # 9 doubles, column-major
    lens: np.ndarray
    ncells: np.ndarray         # int64[3]
    nxyz: np.ndarray           # int64[3]
    ncells_total: int
    band: float

    @property
    def inv_cell(self) -> np.ndarray:
        return self.inv_cm.reshape(3, 3).T.copy()


def analyze_cell(cell, cutoff: float, int_type=torch.int32, float32: bool = False) -> CellPlan:
    """``float32=True``: the analysis with T = Float32 -- cell and cutoff
    converted to Float32 as build_cell_list does (cell_list.jl:637-639), every
    operation in single precision; the plan's arrays are then float32."""
    cm = _colmajor(cell)
    if float32:
        plan32 = _lib.CellPlanF32()
        cm32 = cm.astype(np.float32)
        check(lib().nl_analyze_cell_f32(cm32.ctypes.data_as(_F), np.float32(cutoff).item(), _index_bytes(int_type),
                                        C.byref(plan32)))
        return CellPlan(cm32, np.array(plan32.inv_cell[:], dtype=np.float32), np.array(plan32.lens[:], dtype=np.float32),
                        np.array(plan32.ncells[:], dtype=np.int64), np.array(plan32.nxyz[:], dtype=np.int64),
                        int(plan32.ncells_total), 0.0)
    plan = _lib.CellPlan()
    check(lib().nl_analyze_cell(cm.ctypes.data_as(_D), float(cutoff), _index_bytes(int_type), C.byref(plan)))
    return CellPlan(cm, np.array(plan.inv_cell[:]), np.array(plan.lens[:]), np.array(plan.ncells[:], dtype=np.int64),
                    np.array(plan.nxyz[:], dtype=np.int64), int(plan.ncells_total), float(plan.band))


# ------------------------------------------------------------------- types --
@dataclass
class SortedCellList:
    """Mirror of SortedCellList (src/types.jl:70-82)."""
    X: torch.Tensor              # positions sorted by cell id (N,3)
    X_orig: torch.Tensor         # original positions (N,3)
    perm: torch.Tensor           # sorted index -> original index (1-based)
    cell_id: torch.Tensor        # cell id per sorted atom (1-based)
    cell_offsets: torch.Tensor   # CSR over cells (1-based, ncells_total+1)
    cell: np.ndarray             # 3x3, rows = lattice vectors
    inv_cell: np.ndarray         # 3x3
    pbc: Tuple[bool, bool, bool]
    cutoff: float
    ncells: np.ndarray           # int64[3]
    ncells_total: int
    _plan: CellPlan = field(repr=False, default=None)
    _ws: torch.Tensor = field(repr=False, default=None)
    _records: bool = field(repr=False, default=False)

    @property
    def index_bytes(self) -> int:
        return 4 if self.perm.dtype == torch.int32 else 8

    def to(self, device) -> "SortedCellList":
        """The arrays on another device (Adapt.adapt_structure, adapt.jl:20-33);
        scalar and matrix fields are kept.  A list moved off the GPU is data
        only: the engine's calls take CUDA tensors."""
        return SortedCellList(self.X.to(device), self.X_orig.to(device), self.perm.to(device), self.cell_id.to(device),
                              self.cell_offsets.to(device), self.cell.copy(), self.inv_cell.copy(), self.pbc,
                              self.cutoff, self.ncells.copy(), self.ncells_total, self._plan, None, False)


@dataclass
class PairList:
    """Mirror of PairList (src/types.jl:34-43) plus the pair vectors R."""
    X: torch.Tensor              # positions the list refers to (original order)
    C: np.ndarray                # 3x3 cell
    cutoff: float
    i: torch.Tensor              # 1-based
    j: torch.Tensor              # 1-based
    S: torch.Tensor              # (npairs, 3) integer cell shifts
    first: torch.Tensor          # 1-based CSR per atom (nsites+1)
    R: Optional[torch.Tensor] = None   # (npairs, 3) float64, R = X[j]-X[i]+C'S
    rechecks: int = 0            # candidates decided in FP64 (statistics)

    def __post_init__(self):
        self._first_host = None

    def _first_np(self) -> np.ndarray:
        if self._first_host is None:
            self._first_host = self.first.cpu().numpy().astype(np.int64)
        return self._first_host

    def to(self, device) -> "PairList":
        """The arrays on another device (Adapt.adapt_structure, adapt.jl:35-44)."""
        mv = lambda t: t.to(device) if t is not None else None
        return PairList(mv(self.X), self.C.copy(), self.cutoff, mv(self.i), mv(self.j), mv(self.S), mv(self.first),
                        mv(self.R), self.rechecks)


# --------------------------------------------------------------- building --
def _plan_args(clist: SortedCellList):
    p = clist._plan
    fp = _F if p.cell_cm.dtype == np.float32 else _D
    return (p.cell_cm.ctypes.data_as(fp), p.inv_cm.ctypes.data_as(fp), p.ncells.ctypes.data_as(_I64),
            p.nxyz.ctypes.data_as(_I64))


def _is_f32(clist: SortedCellList) -> bool:
    return clist.X.dtype == torch.float32


def _new_workspace(nat: int, ncells_total: int, device) -> torch.Tensor:
    nbytes = int(lib().nl_workspace_bytes(nat, ncells_total))
    if nbytes == 0:
        raise NLError(_lib.NL_ERR_ARG, "invalid workspace size")
    return torch.empty(nbytes, dtype=torch.uint8, device=device)


def build_cell_list(X, cutoff: float, cell, pbc, int_type=torch.int32, stream=None) -> SortedCellList:
    """build_cell_list(X, cutoff, cell, pbc; int_type) (cell_list.jl:632-679).
    Float32 positions take the single-precision path (the reference with
    T = Float32: cell and cutoff converted to Float32, every operation in
    single precision)."""
    ib = _index_bytes(int_type)
    Xd = _device_positions(X, f32_ok=True)
    f32 = Xd.dtype == torch.float32
    nat = int(Xd.shape[0])
    plan = analyze_cell(cell, cutoff, int_type, float32=f32)
    dev = Xd.device
    ti = _tdtype(ib)
    perm = torch.empty(nat, dtype=ti, device=dev)
    Xs = torch.empty((nat, 3), dtype=Xd.dtype, device=dev)
    cid = torch.empty(nat, dtype=ti, device=dev)
    offs = torch.empty(plan.ncells_total + 1, dtype=ti, device=dev)
    ws = _new_workspace(nat, plan.ncells_total, dev)
    pb = _pbc(pbc)
    rc = np.float32(cutoff).item() if f32 else float(cutoff)
    with torch.cuda.device(dev):
        if f32:
            check(lib().nl_build_cell_list_f32(_ptr(Xd), nat, plan.cell_cm.ctypes.data_as(_F),
                                               plan.inv_cm.ctypes.data_as(_F), plan.ncells.ctypes.data_as(_I64),
                                               pb.ctypes.data_as(_U8), rc, ib, _ptr(perm), _ptr(Xs), _ptr(cid),
                                               C.c_void_p(offs.data_ptr()), _ptr(ws), ws.numel(), _stream_handle(stream)))
        else:
            check(lib().nl_build_cell_list(_ptr(Xd), nat, plan.cell_cm.ctypes.data_as(_D),
                                           plan.inv_cm.ctypes.data_as(_D), plan.ncells.ctypes.data_as(_I64),
                                           pb.ctypes.data_as(_U8), rc, ib, _ptr(perm), _ptr(Xs), _ptr(cid),
                                           C.c_void_p(offs.data_ptr()), _ptr(ws), ws.numel(), _stream_handle(stream)))
        check(lib().nl_sync_status(_ptr(ws), _stream_handle(stream)))
    cellm = np.asarray(cell, dtype=np.float64).reshape(3, 3).astype(np.float32 if f32 else np.float64)
    return SortedCellList(Xs, Xd, perm, cid, offs, cellm, plan.inv_cell, tuple(bool(b) for b in pb), rc,
                          plan.ncells.copy(), plan.ncells_total, plan, ws, True)


def materialize_pairlist(clist: SortedCellList, with_R: bool = True, stream=None) -> PairList:
    """materialize_pairlist(clist) (gpu_kernels.jl:299-364) + R."""
    nat = int(clist.X_orig.shape[0])
    ib = clist.index_bytes
    dev = clist.X_orig.device
    ti = _tdtype(ib)
    if clist._ws is None:
        clist._ws = _new_workspace(nat, clist.ncells_total, dev)
        clist._records = False
    ws = clist._ws
    pb = _pbc(clist.pbc)
    cm, im, nc, nx = _plan_args(clist)
    first = torch.empty(nat + 1, dtype=ti, device=dev)
    total = C.c_int64(0)
    sh = _stream_handle(stream)
    if _is_f32(clist):
        return _materialize_f32(clist, with_R, ws, pb, (cm, im, nc, nx), first, sh)
    with torch.cuda.device(dev):
        check(lib().nl_count_pairs(_ptr(clist.X), _ptr(clist.perm), _ptr(clist.cell_id),
                                   C.c_void_p(clist.cell_offsets.data_ptr()), nat, cm, im, nc, nx,
                                   pb.ctypes.data_as(_U8), clist.cutoff, ib, 1 if clist._records else 0,
                                   C.c_void_p(first.data_ptr()), C.byref(total), _ptr(ws), ws.numel(), sh))
        clist._records = True
        rechecks = C.c_int64(0)
        check(lib().nl_last_recheck_count(_ptr(ws), sh, C.byref(rechecks)))
        P = int(total.value)
        i = torch.empty(P, dtype=ti, device=dev)
        j = torch.empty(P, dtype=ti, device=dev)
        S = torch.empty((P, 3), dtype=ti, device=dev)
        R = torch.empty((P, 3), dtype=torch.float64, device=dev) if with_R else None
        if P > 0:
            check(lib().nl_fill_pairs(_ptr(clist.X), _ptr(clist.perm), C.c_void_p(clist.cell_offsets.data_ptr()), nat,
                                      cm, im, nc, nx, pb.ctypes.data_as(_U8), clist.cutoff, ib,
                                      C.c_void_p(first.data_ptr()), P, _ptr(i), _ptr(j), _ptr(S), _ptr(R), _ptr(ws),
                                      ws.numel(), sh))
            check(lib().nl_sync_status(_ptr(ws), sh))
    return PairList(clist.X_orig, clist.cell.copy(), clist.cutoff, i, j, S, first, R, int(rechecks.value))


def _materialize_f32(clist: SortedCellList, with_R: bool, ws, pb, plan_args, first, sh) -> PairList:
    """materialize_pairlist with T = Float32: i, j, S, first and R (float32)."""
    nat = int(clist.X_orig.shape[0])
    ib = clist.index_bytes
    dev = clist.X_orig.device
    ti = _tdtype(ib)
    total = C.c_int64(0)
    with torch.cuda.device(dev):
        check(lib().nl_count_pairs_f32(_ptr(clist.X), _ptr(clist.perm), _ptr(clist.cell_id),
                                       C.c_void_p(clist.cell_offsets.data_ptr()), nat, *plan_args,
                                       pb.ctypes.data_as(_U8), clist.cutoff, ib, 1 if clist._records else 0,
                                       C.c_void_p(first.data_ptr()), C.byref(total), _ptr(ws), ws.numel(), sh))
        clist._records = True
        P = int(total.value)
        i = torch.empty(P, dtype=ti, device=dev)
        j = torch.empty(P, dtype=ti, device=dev)
        S = torch.empty((P, 3), dtype=ti, device=dev)
        R = torch.empty((P, 3), dtype=torch.float32, device=dev) if with_R else None
        if P > 0:
            check(lib().nl_fill_pairs_f32(_ptr(clist.X), _ptr(clist.perm), C.c_void_p(clist.cell_offsets.data_ptr()),
                                          nat, *plan_args, pb.ctypes.data_as(_U8), clist.cutoff, ib,
                                          C.c_void_p(first.data_ptr()), P, _ptr(i), _ptr(j), _ptr(S), _ptr(R),
                                          _ptr(ws), ws.numel(), sh))
            check(lib().nl_sync_status(_ptr(ws), sh))
    return PairList(clist.X_orig, clist.cell.copy(), clist.cutoff, i, j, S, first, R, 0)


def neighbour_list(X, cutoff: float, cell, pbc, lazy: bool = False, int_type=torch.int32, with_R: bool = True,
                   stream=None, half: bool = False):
    """neighbour_list(X, cutoff, cell, pbc; lazy, int_type) (cell_list.jl:897-916).
    ``half=True`` returns a half list (each unordered pair once: j > i, or
    j == i with S > 0 lexicographically), which the reference does not have."""
    if half:
        if lazy:
            raise ValueError("a half list is a materialised list (lazy=False)")
        from .engine import NeighbourListEngine

        Xd = _device_positions(X, f32_ok=True)
        eng = NeighbourListEngine(int(Xd.shape[0]), cell, cutoff, pbc, int_type=int_type, with_R=with_R,
                                  device=Xd.device, half=True, dtype=Xd.dtype)
        eng.run(Xd, stream)
        return eng.pairlist(Xd)
    clist = build_cell_list(X, cutoff, cell, pbc, int_type=int_type, stream=stream)
    if lazy:
        return clist
    return materialize_pairlist(clist, with_R=with_R, stream=stream)


def legacy_pairlist(X, cutoff: float, cell, pbc, int_type=torch.int32, fixcell: bool = True, with_R: bool = False,
                    stream=None) -> PairList:
    """The reference's legacy linked-list constructor
    PairList(X::Vector{SVec}, cutoff, cell, pbc; int_type, fixcell)
    (cell_list.jl:11-20, 369-385), on the GPU.

    With ``fixcell`` the positions are first moved into the cell and the cell
    enlarged along open axes as _fix_cell_ does (:459-505); the returned
    PairList refers to those positions (``X``) and that cell (``C``), like the
    reference's.  i, j, S and first equal the reference's legacy list: its own
    distance arithmetic and shift formula, each atom's neighbours sorted by j.
    ``with_R`` adds R = X[j] - X[i] + C'S (_getR) for the returned X and C."""
    ib = _index_bytes(int_type)
    ti = _tdtype(ib)
    Xd = _device_positions(X)
    nat = int(Xd.shape[0])
    dev = Xd.device
    pb = _pbc(pbc)
    sh = _stream_handle(stream)
    cm = _colmajor(cell)
    with torch.cuda.device(dev):
        if fixcell:
            Xf = torch.empty_like(Xd)
            cfix = np.zeros(9)
            scratch = torch.empty(_lib.NL_LEGACY_FIX_WORKSPACE_BYTES, dtype=torch.uint8, device=dev)
            check(lib().nl_legacy_fix_cell(_ptr(Xd), nat, cm.ctypes.data_as(_D), pb.ctypes.data_as(_U8), _ptr(Xf),
                                           cfix.ctypes.data_as(_D), _ptr(scratch), scratch.numel(), sh))
            cellm = cfix.reshape(3, 3).T.copy()
        else:
            Xf = Xd
            cellm = np.asarray(cell, dtype=np.float64).reshape(3, 3).copy()
        plan = analyze_cell(cellm, cutoff, int_type)
        nbytes = int(lib().nl_legacy_workspace_bytes(nat, plan.ncells_total, ib))
        if nbytes == 0:
            raise NLError(_lib.NL_ERR_ARG, "invalid workspace size")
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        first = torch.empty(nat + 1, dtype=ti, device=dev)
        total = C.c_int64(0)
        args = (plan.cell_cm.ctypes.data_as(_D), plan.inv_cm.ctypes.data_as(_D), plan.ncells.ctypes.data_as(_I64),
                plan.nxyz.ctypes.data_as(_I64), pb.ctypes.data_as(_U8), float(cutoff), ib)
        check(lib().nl_legacy_count_pairs(_ptr(Xf), nat, *args, C.c_void_p(first.data_ptr()), C.byref(total),
                                          _ptr(ws), ws.numel(), sh))
        rechecks = C.c_int64(0)
        check(lib().nl_last_recheck_count(_ptr(ws), sh, C.byref(rechecks)))
        P = int(total.value)
        i = torch.empty(P, dtype=ti, device=dev)
        j = torch.empty(P, dtype=ti, device=dev)
        S = torch.empty((P, 3), dtype=ti, device=dev)
        if P > 0:
            check(lib().nl_legacy_fill_pairs(nat, *args, C.c_void_p(first.data_ptr()), P, _ptr(i), _ptr(j), _ptr(S),
                                             _ptr(ws), ws.numel(), sh))
            check(lib().nl_sync_status(_ptr(ws), sh))
        R = None
        if with_R:
            R = pair_vectors(Xf, cellm, i, j, S, stream=stream) if P > 0 else torch.empty((0, 3), dtype=torch.float64,
                                                                                          device=dev)
    return PairList(Xf, cellm, float(cutoff), i, j, S, first, R, int(rechecks.value))


def _count_f32(clist: SortedCellList, stream=None) -> torch.Tensor:
    """first (pair offsets) of a Float32 cell list from the count pass."""
    nat = int(clist.X.shape[0])
    dev = clist.X.device
    if clist._ws is None:
        clist._ws = _new_workspace(nat, clist.ncells_total, dev)
        clist._records = False
    ws = clist._ws
    first = torch.empty(nat + 1, dtype=_tdtype(clist.index_bytes), device=dev)
    sh = _stream_handle(stream)
    with torch.cuda.device(dev):
        check(lib().nl_count_pairs_f32(_ptr(clist.X), _ptr(clist.perm), _ptr(clist.cell_id),
                                       C.c_void_p(clist.cell_offsets.data_ptr()), nat, *_plan_args(clist),
                                       _pbc(clist.pbc).ctypes.data_as(_U8), clist.cutoff, clist.index_bytes,
                                       1 if clist._records else 0, C.c_void_p(first.data_ptr()), None, _ptr(ws),
                                       ws.numel(), sh))
        clist._records = True
        check(lib().nl_sync_status(_ptr(ws), sh))
    return first


def lazy_reduce(clist: SortedCellList, op: str = "count", stream=None, out: Optional[torch.Tensor] = None,
                sync: bool = True) -> torch.Tensor:
    """Built-in reductions of the lazy traversal over every atom:
    "count" -> int32 neighbour count per atom (count_neighbours for all i);
    "inv_r6" -> float64 per-atom sum of 1/r^6 in the reference's order
    (bit-identical to a sequential for_each_neighbour sum);
    "inv_r6_fast" -> the same sums from the neighbour masks, each unordered
    pair once with exact fixed-point R (relative error at most 1e-12, last bits
    not reproducible run to run).
    ``out`` reuses an output tensor; ``sync=False`` leaves the error check to
    a later nl_sync_status on the cell list's workspace."""
    nat = int(clist.X.shape[0])
    dev = clist.X.device
    if _is_f32(clist):
        # Float32 positions: the count pass of the single-precision path
        if op != "count":
            raise ValueError("the built-in Σ r^-6 reduction takes Float64 positions; Float32 lists support 'count'")
        first = _count_f32(clist, stream)
        counts = (first[1:] - first[:-1]).to(torch.int32)
        if out is None:
            return counts
        out.copy_(counts)
        return out
    if op == "count":
        code, dt = _lib.NL_REDUCE_COUNT, torch.int32
    elif op == "inv_r6":
        code, dt = _lib.NL_REDUCE_INV_R6, torch.float64
    elif op == "inv_r6_fast":
        code, dt = _lib.NL_REDUCE_INV_R6_FAST, torch.float64
    else:
        raise ValueError("op must be 'count', 'inv_r6' or 'inv_r6_fast'")
    if out is None:
        out = torch.zeros(nat, dtype=dt, device=dev)
    elif out.dtype != dt or out.numel() != nat or not out.is_cuda:
        raise ValueError(f"out must be a CUDA {dt} tensor of {nat} entries")
    if clist._ws is None:
        clist._ws = _new_workspace(nat, clist.ncells_total, dev)
        clist._records = False
    ws = clist._ws
    pb = _pbc(clist.pbc)
    cm, im, nc, nx = _plan_args(clist)
    sh = _stream_handle(stream)
    with torch.cuda.device(dev):
        check(lib().nl_lazy_reduce(_ptr(clist.X), _ptr(clist.perm), _ptr(clist.cell_id),
                                   C.c_void_p(clist.cell_offsets.data_ptr()), nat, cm, im, nc, nx,
                                   pb.ctypes.data_as(_U8), clist.cutoff, clist.index_bytes,
                                   1 if clist._records else 0, code, _ptr(out), _ptr(ws), ws.numel(), sh))
        clist._records = True
        if sync:
            check(lib().nl_sync_status(_ptr(ws), sh))
    return out


# --------------------------------------------------------------- accessors --
def npairs(nlist: PairList) -> int:
    return int(nlist.i.shape[0])


def nsites(x) -> int:
    if isinstance(x, PairList):
        return int(x.first.shape[0]) - 1
    return int(x.X_orig.shape[0])


def cutoff(x) -> float:
    return float(x.cutoff)


def nneigs(nlist: PairList, i0: int) -> int:
    f = nlist._first_np()
    return int(f[i0] - f[i0 - 1])


def maxneigs(nlist: PairList) -> int:
    if nsites(nlist) == 0:
        raise ValueError("maxneigs of an empty PairList")
    f = nlist._first_np()
    return int(np.max(np.diff(f)))


max_neighbours = maxneigs


def neigss(nlist: PairList, i0: int):
    """neigss(nlist, i0) -> (j, R, S) (cell_list.jl:583-598): views of atom i0's
    neighbours (i0 is 1-based).  R comes from the device R buffer, bit-equal to
    the reference's _getR."""
    f = nlist._first_np()
    a, b = int(f[i0 - 1]) - 1, int(f[i0]) - 1
    R = nlist.R[a:b] if nlist.R is not None else _getR(nlist, a, b)
    return nlist.j[a:b], R, nlist.S[a:b]


def neigs(nlist: PairList, i0: int):
    j, R, _ = neigss(nlist, i0)
    return j, R


def pair_vectors(X: torch.Tensor, cell, i: torch.Tensor, j: torch.Tensor, S: torch.Tensor,
                 out: Optional[torch.Tensor] = None, stream=None) -> torch.Tensor:
    """R = (X[j] - X[i]) + C'S for every pair (the reference's _getR,
    cell_list.jl:525-531), bit-equal to the R of a materialised list; float32
    positions take the reference's single-precision operations (T = Float32)."""
    P = int(i.shape[0])
    f32 = X.dtype == torch.float32
    if out is None:
        out = torch.empty((P, 3), dtype=X.dtype, device=X.device)
    cm = _colmajor(cell)
    ib = 4 if i.dtype == torch.int32 else 8
    if f32:
        cm32 = np.ascontiguousarray(cm.astype(np.float32))
        check(lib().nl_pair_vectors_f32(_ptr(X), int(X.shape[0]), cm32.ctypes.data_as(_F), ib, _ptr(i), _ptr(j),
                                        _ptr(S), P, _ptr(out), _stream_handle(stream)))
    else:
        check(lib().nl_pair_vectors(_ptr(X), int(X.shape[0]), cm.ctypes.data_as(_D), ib, _ptr(i), _ptr(j), _ptr(S),
                                    P, _ptr(out), _stream_handle(stream)))
    return out


def _getR(nlist: PairList, a: int, b: int) -> torch.Tensor:
    """R of pairs a..b-1 of a list materialised without R, on the device."""
    if nlist.X is None:
        raise NLError(_lib.NL_ERR_ARG, "this PairList has neither R nor the positions to compute it")
    if nlist.X.dtype == torch.float32:
        raise NLError(_lib.NL_ERR_ARG, "a Float32 list carries R only when materialised with_R=True")
    X = nlist.X.to(torch.float64).contiguous()
    return pair_vectors(X, nlist.C, nlist.i[a:b], nlist.j[a:b], nlist.S[a:b].contiguous())


def query_neighbours(clist: SortedCellList, atoms, with_R: bool = True, stream=None):
    """Neighbours of a set of atoms (1-based original indices) by the lazy
    traversal on the device (nl_query_neighbours: for_each_neighbour,
    cell_list.jl:779-833, per atom), without materialising the system's list.
    Returns (first, j, S, R): first[k] .. first[k+1]-1 (1-based, int64) are the
    pairs of atoms[k], in the reference's traversal order."""
    if _is_f32(clist):
        raise TypeError("the per-atom lazy traversal takes a Float64 cell list")
    dev = clist.X.device
    ti = clist.perm.dtype
    at = torch.as_tensor(np.asarray(atoms, dtype=np.int64).reshape(-1), device=dev).to(ti).contiguous()
    nq = int(at.numel())
    ws = _query_workspace(clist)
    pb = _pbc(clist.pbc)
    cm, im, nc, nx = _plan_args(clist)
    sh = _stream_handle(stream)
    nat = int(clist.X.shape[0])
    counts = torch.zeros(nq, dtype=torch.int64, device=dev)

    def call(offsets, cap, j, S, R, cnt):
        return lib().nl_query_neighbours(
            _ptr(clist.X_orig), _ptr(clist.X), _ptr(clist.perm), C.c_void_p(clist.cell_offsets.data_ptr()), nat, cm,
            im, nc, nx, pb.ctypes.data_as(_U8), clist.cutoff, clist.index_bytes, _ptr(at), nq, _ptr(cnt),
            _ptr(offsets), int(cap), _ptr(j), _ptr(S), _ptr(R), _ptr(ws), ws.numel(), sh)

    with torch.cuda.device(dev):
        check(call(None, 0, None, None, None, counts))
        check(lib().nl_sync_status(_ptr(ws), sh))
        first = torch.zeros(nq + 1, dtype=torch.int64, device=dev)
        torch.cumsum(counts, 0, out=first[1:])
        P = int(first[-1].item())
        j = torch.empty(P, dtype=ti, device=dev)
        S = torch.empty((P, 3), dtype=ti, device=dev)
        R = torch.empty((P, 3), dtype=torch.float64, device=dev) if with_R else None
        if P:
            check(call(first, P, j, S, R, None))
            check(lib().nl_sync_status(_ptr(ws), sh))
    return first + 1, j, S, R


def _query_workspace(clist: SortedCellList) -> torch.Tensor:
    """The error word of the per-atom traversal: the cell list's workspace
    when it has one (the traversal touches only its first word), else a small
    buffer of its own."""
    if clist._ws is not None:
        return clist._ws
    w = getattr(clist, "_qws", None)
    if w is None:
        w = torch.zeros(128, dtype=torch.uint8, device=clist.X.device)
        object.__setattr__(clist, "_qws", w)
    return w


def count_neighbours(clist: SortedCellList, i: int) -> int:
    """count_neighbours(clist, i) (cell_list.jl:808-814), i 1-based: the lazy
    traversal of atom i alone on the device."""
    if _is_f32(clist):
        return int(lazy_reduce(clist, "count")[i - 1].item())
    first, _, _, _ = query_neighbours(clist, [i], with_R=False)
    return int(first[1].item() - first[0].item())


def neighbours(x, i: int):
    """neighbours(nlist, i) = neigss; neighbours(clist, i) -> (js, Rs, Ss)
    (cell_list.jl:606, 821-833): for a SortedCellList, the lazy traversal of
    atom i alone on the device, in the reference's order."""
    if isinstance(x, PairList):
        return neigss(x, i)
    if _is_f32(x):
        return neigss(_lazy_pairlist(x), i)
    _, j, S, R = query_neighbours(x, [i])
    return j, R, S


def _lazy_pairlist(clist: SortedCellList) -> PairList:
    cached = getattr(clist, "_lazy_nl", None)
    if cached is None:
        cached = materialize_pairlist(clist)
        object.__setattr__(clist, "_lazy_nl", cached)
    return cached


def num_neighbours(x, i: int) -> int:
    """num_neighbours (cell_list.jl:926-927)."""
    if isinstance(x, PairList):
        return nneigs(x, i)
    return count_neighbours(x, i)


def for_each_neighbour(f: Callable, clist: SortedCellList, i: int) -> None:
    """for_each_neighbour(f, clist, i) (cell_list.jl:779-801): calls
    f(j, R, S) for each neighbour of atom i (1-based) in the reference's order.
    The traversal runs on the GPU; f runs on the host."""
    js, Rs, Ss = neighbours(clist, i)
    js, Rs, Ss = js.cpu().numpy(), Rs.cpu().numpy(), Ss.cpu().numpy()
    for k in range(js.shape[0]):
        f(int(js[k]), Rs[k], Ss[k])


# --------------------------------------------------------------- iterators --
class PairIterator:
    """pairs(nlist) (iterators.jl:12-26): yields (i, j, R) for every pair in
    list order (1-based i, j; R a float64[3]).  The device buffers are read in
    host blocks of ``block`` pairs."""

    def __init__(self, nlist: PairList, block: int = 1 << 16):
        self.nlist, self.block = nlist, int(block)

    def __len__(self) -> int:
        return npairs(self.nlist)

    def __iter__(self):
        nl = self.nlist
        for a in range(0, npairs(nl), self.block):
            b = min(a + self.block, npairs(nl))
            i = nl.i[a:b].cpu().numpy()
            j = nl.j[a:b].cpu().numpy()
            R = (nl.R[a:b] if nl.R is not None else _getR(nl, a, b)).cpu().numpy()
            for k in range(b - a):
                yield int(i[k]), int(j[k]), R[k]


class SiteIterator:
    """sites(nlist) (iterators.jl:28-40): yields (i, j, R) per site, with j and
    R the device views of site i's neighbours (neigs)."""

    def __init__(self, nlist: PairList):
        self.nlist = nlist

    def __len__(self) -> int:
        return nsites(self.nlist)

    def __iter__(self):
        for i in range(1, nsites(self.nlist) + 1):
            j, R = neigs(self.nlist, i)
            yield i, j, R


def pairs(nlist: PairList) -> PairIterator:
    return PairIterator(nlist)


def sites(nlist: PairList) -> SiteIterator:
    return SiteIterator(nlist)
