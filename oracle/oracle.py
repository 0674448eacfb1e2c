"""ctypes front-end of the CPU oracle (``nl_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by the test suite, the smoke check and the
CPU-baseline leg of ``bench.py``.  The product never imports this module.

Every function restates a function of NeighbourLists.jl v0.6.2 (see the
file:line citations in ``nl_oracle.c``).  Index arrays are 1-based int64, as in
the reference.  ``cell`` is a 3x3 array whose ROWS are the lattice vectors
(``cell[k, :]`` is lattice vector k), as in the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libnl_oracle.so")
_lib = None

ERR_TOO_MANY_CELLS = 2


class OracleError(RuntimeError):
    pass


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE, "libnl_oracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        newest = max(os.path.getmtime(os.path.join(_HERE, f)) for f in ("nl_oracle.c", "nl_oracle_f32.c", "Makefile"))
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < newest:
            build()
        _lib = C.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


class _Result(C.Structure):
    _fields_ = [
        ("nat", C.c_int64),
        ("npairs", C.c_int64),
        ("ncells", C.c_int64),
        ("perm", C.POINTER(C.c_int64)),
        ("cell_id", C.POINTER(C.c_int64)),
        ("cell_offsets", C.POINTER(C.c_int64)),
        ("first", C.POINTER(C.c_int64)),
        ("i", C.POINTER(C.c_int64)),
        ("j", C.POINTER(C.c_int64)),
        ("S", C.POINTER(C.c_int64)),
        ("X_sorted", C.POINTER(C.c_double)),
        ("R", C.POINTER(C.c_double)),
    ]


class _ResultF32(C.Structure):
    _fields_ = [
        ("nat", C.c_int64),
        ("npairs", C.c_int64),
        ("ncells", C.c_int64),
        ("perm", C.POINTER(C.c_int64)),
        ("cell_id", C.POINTER(C.c_int64)),
        ("cell_offsets", C.POINTER(C.c_int64)),
        ("first", C.POINTER(C.c_int64)),
        ("i", C.POINTER(C.c_int64)),
        ("j", C.POINTER(C.c_int64)),
        ("S", C.POINTER(C.c_int64)),
        ("X_sorted", C.POINTER(C.c_float)),
        ("R", C.POINTER(C.c_float)),
    ]


_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)


def _declare(L):
    L.orc_analyze_cell.argtypes = [_D, C.c_double, C.c_int, _D, _I, _D, _I]
    L.orc_analyze_cell.restype = C.c_int
    L.orc_lengths.argtypes = [_D, _D]
    L.orc_build_cell_list.argtypes = [_D, C.c_int64, _D, _U8, C.c_double, C.c_int, _I, _I, _I, _D]
    L.orc_build_cell_list.restype = C.c_int
    L.orc_count.argtypes = [_D, C.c_int64, _D, _U8, C.c_double, _I, _I, C.c_int, _I]
    L.orc_count.restype = C.c_int
    L.orc_pair_offsets.argtypes = [_I, C.c_int64, _I]
    L.orc_fill.argtypes = [_D, C.c_int64, _D, _U8, C.c_double, _I, _I, _I, C.c_int, _I, _I, _I, _D]
    L.orc_fill.restype = C.c_int
    L.orc_lazy_r6.argtypes = [_D, C.c_int64, _D, _U8, C.c_double, _I, _I, C.c_int, _D]
    L.orc_lazy_r6.restype = C.c_int
    L.orc_neighbours.argtypes = [_D, C.c_int64, _D, _U8, C.c_double, _I, _I, C.c_int64, C.c_int64, _I, _I, _D]
    L.orc_neighbours.restype = C.c_int64
    L.orc_getR.argtypes = [_D, _D, C.c_int64, _I, _I, _I, _D]
    L.orc_neighbour_list.argtypes = [_D, C.c_int64, _D, _U8, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(_Result)]
    L.orc_neighbour_list.restype = C.c_int
    L.orc_free.argtypes = [C.POINTER(_Result)]
    L.orc_legacy_pairlist.argtypes = [_D, C.c_int64, _D, _U8, C.c_double, C.c_int, C.c_int, C.POINTER(_Result), _D]
    L.orc_legacy_pairlist.restype = C.c_int64
    L.orc_fix_cell.argtypes = [_D, C.c_int64, _D, _U8]
    L.orc_analyze_cell_f32.argtypes = [_F, C.c_float, C.c_int, _F, _I, _F, _I]
    L.orc_analyze_cell_f32.restype = C.c_int
    L.orc_neighbour_list_f32.argtypes = [_F, C.c_int64, _F, _U8, C.c_float, C.c_int, C.POINTER(_ResultF32)]
    L.orc_neighbour_list_f32.restype = C.c_int
    L.orc_free_f32.argtypes = [C.POINTER(_ResultF32)]


def _colmajor(cell) -> np.ndarray:
    """3x3 (rows = lattice vectors) -> 9 doubles in column-major order."""
    c = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    return np.ascontiguousarray(c.T).reshape(9)


def _pos(X) -> np.ndarray:
    X = np.ascontiguousarray(np.asarray(X, dtype=np.float64).reshape(-1, 3))
    return X


def _pbc(pbc) -> np.ndarray:
    return np.ascontiguousarray(np.array([1 if bool(b) else 0 for b in pbc], dtype=np.uint8))


def _p(a, t):
    return a.ctypes.data_as(t)


@dataclass
class CellInfo:
    inv_cell: np.ndarray  # 3x3, row-major numpy view of the reference's inv(cell)
    ncells: np.ndarray  # int64[3]
    lens: np.ndarray  # float64[3] (abs'ed perpendicular heights)
    nxyz: np.ndarray  # int64[3]


def analyze_cell(cell, cutoff, ti_bytes=4) -> CellInfo:
    """analyze_cell (cell_list.jl:152-170) + nxyz (gpu_kernels.jl:315-316)."""
    L = lib()
    cm = _colmajor(cell)
    inv = np.zeros(9)
    ns = np.zeros(3, dtype=np.int64)
    lens = np.zeros(3)
    nxyz = np.zeros(3, dtype=np.int64)
    st = L.orc_analyze_cell(_p(cm, _D), float(cutoff), int(ti_bytes), _p(inv, _D), _p(ns, _I), _p(lens, _D), _p(nxyz, _I))
    if st:
        raise OracleError(f"analyze_cell failed with status {st}")
    return CellInfo(inv.reshape(3, 3).T.copy(), ns, lens, nxyz)


@dataclass
class OraclePairList:
    i: np.ndarray  # int64[P], 1-based
    j: np.ndarray  # int64[P], 1-based
    S: np.ndarray  # int64[P,3]
    first: np.ndarray  # int64[nat+1], 1-based
    R: np.ndarray | None  # float64[P,3]
    X: np.ndarray  # positions the list refers to
    cell: np.ndarray  # 3x3 rows = lattice vectors

    @property
    def npairs(self) -> int:
        return int(self.i.shape[0])


@dataclass
class OracleCellList:
    X: np.ndarray  # sorted positions
    X_orig: np.ndarray
    perm: np.ndarray  # 1-based
    cell_id: np.ndarray  # 1-based, sorted
    cell_offsets: np.ndarray  # 1-based, ncells+1
    cell: np.ndarray
    pbc: np.ndarray
    cutoff: float


def _arr(ptr, n, dtype, shape=None):
    if n == 0:
        out = np.zeros(0, dtype=dtype)
    else:
        out = np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)
    return out.reshape(shape) if shape is not None else out


def build_cell_list(X, cutoff, cell, pbc, ti_bytes=4) -> OracleCellList:
    """build_cell_list on the CPU backend (cell_list.jl:632-748)."""
    L = lib()
    X = _pos(X)
    nat = X.shape[0]
    info = analyze_cell(cell, cutoff, ti_bytes)
    ncells = int(np.prod(info.ncells))
    perm = np.zeros(max(nat, 1), dtype=np.int64)
    cid = np.zeros(max(nat, 1), dtype=np.int64)
    offs = np.zeros(ncells + 1, dtype=np.int64)
    Xs = np.zeros((max(nat, 1), 3))
    cm = _colmajor(cell)
    pb = _pbc(pbc)
    st = L.orc_build_cell_list(_p(X, _D), nat, _p(cm, _D), _p(pb, _U8), float(cutoff), ti_bytes, _p(perm, _I), _p(cid, _I),
                               _p(offs, _I), _p(Xs, _D))
    if st:
        raise OracleError(f"build_cell_list failed with status {st}")
    return OracleCellList(Xs[:nat].copy(), X.copy(), perm[:nat].copy(), cid[:nat].copy(), offs,
                          np.asarray(cell, dtype=np.float64).reshape(3, 3).copy(), pb.astype(bool), float(cutoff))


def neighbour_list(X, cutoff, cell, pbc, ti_bytes=4, nthreads=1, with_R=True) -> OraclePairList:
    """build_cell_list + materialize_pairlist on the CPU backend (sort-based)."""
    L = lib()
    X = _pos(X)
    nat = X.shape[0]
    cm = _colmajor(cell)
    pb = _pbc(pbc)
    res = _Result()
    st = L.orc_neighbour_list(_p(X, _D), nat, _p(cm, _D), _p(pb, _U8), float(cutoff), int(ti_bytes), int(nthreads),
                              1 if with_R else 0, C.byref(res))
    if st:
        L.orc_free(C.byref(res))
        raise OracleError(f"neighbour_list failed with status {st}")
    try:
        P = res.npairs
        out = OraclePairList(
            i=_arr(res.i, P, np.int64),
            j=_arr(res.j, P, np.int64),
            S=_arr(res.S, 3 * P, np.int64, (P, 3)),
            first=_arr(res.first, nat + 1, np.int64),
            R=_arr(res.R, 3 * P, np.float64, (P, 3)) if with_R else None,
            X=X.copy(),
            cell=np.asarray(cell, dtype=np.float64).reshape(3, 3).copy(),
        )
    finally:
        L.orc_free(C.byref(res))
    return out


def timed_neighbour_list(X, cutoff, cell, pbc, nthreads, with_R=False) -> int:
    """Runs the whole sort-based CPU path once (allocations included, like the
    reference) and returns the pair count.  Used by the CPU baseline timing."""
    L = lib()
    X = _pos(X)
    cm = _colmajor(cell)
    pb = _pbc(pbc)
    res = _Result()
    st = L.orc_neighbour_list(_p(X, _D), X.shape[0], _p(cm, _D), _p(pb, _U8), float(cutoff), 4, int(nthreads),
                              1 if with_R else 0, C.byref(res))
    n = res.npairs
    L.orc_free(C.byref(res))
    if st:
        raise OracleError(f"neighbour_list failed with status {st}")
    return int(n)


def legacy_pairlist(X, cutoff, cell, pbc, ti_bytes=4, fixcell=True) -> OraclePairList:
    """Legacy linked-list PairList (cell_list.jl:11-20, 369-384)."""
    L = lib()
    X = _pos(X)
    nat = X.shape[0]
    cm = _colmajor(cell)
    pb = _pbc(pbc)
    res = _Result()
    cout = np.zeros(9)
    n = L.orc_legacy_pairlist(_p(X, _D), nat, _p(cm, _D), _p(pb, _U8), float(cutoff), int(ti_bytes), 1 if fixcell else 0,
                              C.byref(res), _p(cout, _D))
    if n < 0:
        raise OracleError(f"legacy pairlist failed with status {-n}")
    try:
        out = OraclePairList(
            i=_arr(res.i, n, np.int64),
            j=_arr(res.j, n, np.int64),
            S=_arr(res.S, 3 * n, np.int64, (n, 3)),
            first=_arr(res.first, nat + 1, np.int64),
            R=None,
            X=_arr(res.X_sorted, 3 * nat, np.float64, (nat, 3)),
            cell=cout.reshape(3, 3).T.copy(),
        )
    finally:
        L.orc_free(C.byref(res))
    if out.npairs:
        R = np.zeros((out.npairs, 3))
        cm2 = _colmajor(out.cell)
        Xf = np.ascontiguousarray(out.X)
        L.orc_getR(_p(Xf, _D), _p(cm2, _D), out.npairs, _p(out.i, _I), _p(out.j, _I), _p(np.ascontiguousarray(out.S), _I),
                   _p(R, _D))
        out.R = R
    else:
        out.R = np.zeros((0, 3))
    return out


def count_neighbours(clist: OracleCellList, nthreads=1) -> np.ndarray:
    """count_neighbours_kernel! over all atoms (gpu_kernels.jl:132-152)."""
    L = lib()
    X = _pos(clist.X_orig)
    nat = X.shape[0]
    cnt = np.zeros(max(nat, 1), dtype=np.int64)
    cm = _colmajor(clist.cell)
    pb = _pbc(clist.pbc)
    perm = np.ascontiguousarray(clist.perm, dtype=np.int64)
    offs = np.ascontiguousarray(clist.cell_offsets, dtype=np.int64)
    st = L.orc_count(_p(X, _D), nat, _p(cm, _D), _p(pb, _U8), clist.cutoff, _p(perm, _I), _p(offs, _I), int(nthreads),
                     _p(cnt, _I))
    if st:
        raise OracleError(f"count failed with status {st}")
    return cnt[:nat]


def lazy_sum_r6(clist: OracleCellList, nthreads=1) -> np.ndarray:
    """Per-atom sum over for_each_neighbour of 1/((r2*r2)*r2), r2 = dot(R,R),
    accumulated in traversal order (cell_list.jl:779-801)."""
    L = lib()
    X = _pos(clist.X_orig)
    nat = X.shape[0]
    out = np.zeros(max(nat, 1))
    cm = _colmajor(clist.cell)
    pb = _pbc(clist.pbc)
    perm = np.ascontiguousarray(clist.perm, dtype=np.int64)
    offs = np.ascontiguousarray(clist.cell_offsets, dtype=np.int64)
    st = L.orc_lazy_r6(_p(X, _D), nat, _p(cm, _D), _p(pb, _U8), clist.cutoff, _p(perm, _I), _p(offs, _I), int(nthreads),
                       _p(out, _D))
    if st:
        raise OracleError(f"lazy reduction failed with status {st}")
    return out[:nat]


def neighbours(clist: OracleCellList, i: int):
    """neighbours(clist, i) -> (js, Rs, Ss) (cell_list.jl:821-833); i is 1-based."""
    L = lib()
    X = _pos(clist.X_orig)
    nat = X.shape[0]
    cm = _colmajor(clist.cell)
    pb = _pbc(clist.pbc)
    perm = np.ascontiguousarray(clist.perm, dtype=np.int64)
    offs = np.ascontiguousarray(clist.cell_offsets, dtype=np.int64)
    cap = 64
    while True:
        oj = np.zeros(cap, dtype=np.int64)
        oS = np.zeros((cap, 3), dtype=np.int64)
        oR = np.zeros((cap, 3))
        n = L.orc_neighbours(_p(X, _D), nat, _p(cm, _D), _p(pb, _U8), clist.cutoff, _p(perm, _I), _p(offs, _I), int(i), cap,
                             _p(oj, _I), _p(oS, _I), _p(oR, _D))
        if n < 0:
            raise OracleError("neighbours failed")
        if n <= cap:
            return oj[:n].copy(), oR[:n].copy(), oS[:n].copy()
        cap = int(n)


def canonical(i, j, S, R=None):
    """Canonical (i, j, S) order used by the reference's get_sorted_pairs
    (test/test_utils.jl:68-70).  Returns sorted copies (and R permuted alike)."""
    i = np.asarray(i, dtype=np.int64).reshape(-1)
    j = np.asarray(j, dtype=np.int64).reshape(-1)
    S = np.asarray(S, dtype=np.int64).reshape(-1, 3)
    order = np.lexsort((S[:, 2], S[:, 1], S[:, 0], j, i))
    out = (i[order], j[order], S[order])
    if R is not None:
        out = out + (np.asarray(R).reshape(-1, 3)[order],)
    return out


# ------------------------------------------------------------ T = Float32 --
@dataclass
class OracleF32Result:
    """build_cell_list + materialize_pairlist with T = Float32 (nl_oracle_f32.c)."""
    perm: np.ndarray          # int64[nat], 1-based
    cell_id: np.ndarray       # int64[nat], sorted
    cell_offsets: np.ndarray  # int64[ncells+1]
    X_sorted: np.ndarray      # float32[nat, 3]
    i: np.ndarray
    j: np.ndarray
    S: np.ndarray             # int64[P, 3]
    first: np.ndarray         # int64[nat+1]
    R: np.ndarray             # float32[P, 3]

    @property
    def npairs(self) -> int:
        return int(self.i.shape[0])


def _f32_inputs(X, cutoff, cell):
    X32 = np.ascontiguousarray(np.asarray(X).astype(np.float32).reshape(-1, 3))
    cm32 = np.ascontiguousarray(np.asarray(cell, dtype=np.float64).reshape(3, 3).astype(np.float32).T).reshape(9)
    return X32, cm32, np.float32(cutoff)


def analyze_cell_f32(cell, cutoff, ti_bytes=4):
    """analyze_cell + nxyz with T = Float32: (inv (3x3 float32), ncells, lens, nxyz)."""
    L = lib()
    _, cm, rc = _f32_inputs(np.zeros((0, 3)), cutoff, cell)
    inv = np.zeros(9, dtype=np.float32)
    ns = np.zeros(3, dtype=np.int64)
    lens = np.zeros(3, dtype=np.float32)
    nxyz = np.zeros(3, dtype=np.int64)
    st = L.orc_analyze_cell_f32(_p(cm, _F), float(rc), int(ti_bytes), _p(inv, _F), _p(ns, _I), _p(lens, _F),
                                _p(nxyz, _I))
    if st:
        raise OracleError(f"analyze_cell (Float32) failed with status {st}")
    return inv.reshape(3, 3).T.copy(), ns, lens, nxyz


def neighbour_list_f32(X, cutoff, cell, pbc, ti_bytes=4) -> OracleF32Result:
    """The reference's sort-based path with positions, cell and cutoff in
    Float32 (cell and cutoff converted as build_cell_list does, cell_list.jl:637-639)."""
    L = lib()
    X32, cm, rc = _f32_inputs(X, cutoff, cell)
    nat = X32.shape[0]
    pb = _pbc(pbc)
    res = _ResultF32()
    st = L.orc_neighbour_list_f32(_p(X32, _F), nat, _p(cm, _F), _p(pb, _U8), float(rc), int(ti_bytes), C.byref(res))
    if st:
        L.orc_free_f32(C.byref(res))
        raise OracleError(f"neighbour_list (Float32) failed with status {st}")
    try:
        P = res.npairs
        out = OracleF32Result(
            perm=_arr(res.perm, nat, np.int64),
            cell_id=_arr(res.cell_id, nat, np.int64),
            cell_offsets=_arr(res.cell_offsets, res.ncells + 1, np.int64),
            X_sorted=_arr(res.X_sorted, 3 * nat, np.float32, (nat, 3)),
            i=_arr(res.i, P, np.int64),
            j=_arr(res.j, P, np.int64),
            S=_arr(res.S, 3 * P, np.int64, (P, 3)),
            first=_arr(res.first, nat + 1, np.int64),
            R=_arr(res.R, 3 * P, np.float32, (P, 3)),
        )
    finally:
        L.orc_free_f32(C.byref(res))
    return out
