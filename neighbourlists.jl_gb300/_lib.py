"""ctypes binding of libnlgpu.so (the C ABI declared in include/nlgpu.h).

The library is built in-tree by build.py.  Loading fails loudly if it is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnlgpu.so")

NL_OK = 0
NL_ERR_ARG = 1
NL_ERR_TOO_MANY_CELLS = 2
NL_ERR_NOMEM = 3
NL_ERR_CUDA = 4
NL_ERR_TIMEOUT = 5
NL_ERR_BAD_POSITION = 6
NL_ERR_CAPACITY = 7
NL_ERR_INDEX_OVERFLOW = 8
NL_ERR_INCONSISTENT = 9

NL_LEGACY_FIX_WORKSPACE_BYTES = 256

NL_REDUCE_COUNT = 0
NL_REDUCE_INV_R6 = 1
NL_REDUCE_INV_R6_FAST = 2

# every symbol include/nlgpu.h declares
EXPORTED = [
    "nl_analyze_cell",
    "nl_workspace_bytes",
    "nl_workspace_min_bytes",
    "nl_build_cell_list",
    "nl_count_pairs",
    "nl_fill_pairs",
    "nl_neighbour_list",
    "nl_neighbour_list_static",
    "nl_static_sync_status",
    "nl_neighbour_list_half",
    "nl_lazy_reduce",
    "nl_query_neighbours",
    "nl_pair_vectors",
    "nl_max_displacement_sq",
    "nl_pair_vectors_f32",
    "nl_max_displacement_sq_f32",
    "nl_batch_create",
    "nl_batch_create_auto",
    "nl_batch_destroy",
    "nl_batch_workspace_bytes",
    "nl_batch_sizes",
    "nl_batch_upload",
    "nl_batch_neighbour_list",
    "nl_neighbour_list_half_f32",
    "nl_batch_create_f32",
    "nl_batch_create_auto_f32",
    "nl_batch_neighbour_list_f32",
    "nl_analyze_cell_f32",
    "nl_build_cell_list_f32",
    "nl_count_pairs_f32",
    "nl_fill_pairs_f32",
    "nl_neighbour_list_f32",
    "nl_legacy_fix_cell",
    "nl_legacy_workspace_bytes",
    "nl_legacy_count_pairs",
    "nl_legacy_fill_pairs",
    "nl_set_tuning",
    "nl_batch_set_tuning",
    "nl_sync_status",
    "nl_last_recheck_count",
    "nl_status_string",
    "nl_last_error",
    "nl_version",
]


class CellPlan(C.Structure):
    _fields_ = [
        ("inv_cell", C.c_double * 9),
        ("lens", C.c_double * 3),
        ("ncells", C.c_int64 * 3),
        ("nxyz", C.c_int64 * 3),
        ("ncells_total", C.c_int64),
        ("band", C.c_double),
    ]


class CellPlanF32(C.Structure):
    _fields_ = [
        ("inv_cell", C.c_float * 9),
        ("lens", C.c_float * 3),
        ("ncells", C.c_int64 * 3),
        ("nxyz", C.c_int64 * 3),
        ("ncells_total", C.c_int64),
    ]


class System(C.Structure):
    """nl_system: one system of a batch."""
    _fields_ = [
        ("nat", C.c_int64),
        ("cell", C.c_double * 9),
        ("inv_cell", C.c_double * 9),
        ("ncells", C.c_int64 * 3),
        ("nxyz", C.c_int64 * 3),
        ("pbc", C.c_uint8 * 3),
        ("cutoff", C.c_double),
    ]


class SystemF32(C.Structure):
    """nl_system_f32: one system of a Float32 batch."""
    _fields_ = [
        ("nat", C.c_int64),
        ("cell", C.c_float * 9),
        ("inv_cell", C.c_float * 9),
        ("ncells", C.c_int64 * 3),
        ("nxyz", C.c_int64 * 3),
        ("pbc", C.c_uint8 * 3),
        ("cutoff", C.c_float),
    ]


class Tuning(C.Structure):
    """nl_tuning: grid sizes of the pair kernels (0 = default)."""
    _fields_ = [("pair_blocks_per_sm", C.c_int), ("emit_blocks_per_sm", C.c_int), ("count_kernel", C.c_int)]


class NLError(RuntimeError):
    """Raised for any non-zero status of the C ABI."""

    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


_lib = None

_vp = C.c_void_p
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)


def _declare(L):
    L.nl_analyze_cell.argtypes = [_D, C.c_double, C.c_int, C.POINTER(CellPlan)]
    L.nl_analyze_cell.restype = C.c_int
    L.nl_workspace_bytes.argtypes = [C.c_int64, C.c_int64]
    L.nl_workspace_bytes.restype = C.c_size_t
    L.nl_workspace_min_bytes.argtypes = [C.c_int64, C.c_int64]
    L.nl_workspace_min_bytes.restype = C.c_size_t
    L.nl_build_cell_list.argtypes = [_vp, C.c_int64, _D, _D, _I64, _U8, C.c_double, C.c_int, _vp, _vp, _vp, _vp, _vp,
                                     C.c_size_t, _vp]
    L.nl_build_cell_list.restype = C.c_int
    L.nl_count_pairs.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, C.c_int,
                                 _vp, _I64, _vp, C.c_size_t, _vp]
    L.nl_count_pairs.restype = C.c_int
    L.nl_fill_pairs.argtypes = [_vp, _vp, _vp, C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, _vp, C.c_int64,
                                _vp, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    L.nl_fill_pairs.restype = C.c_int
    L.nl_neighbour_list.argtypes = [_vp, C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, _vp, _vp, _vp, _vp, _vp,
                                    C.c_int64, _vp, _vp, _vp, _vp, _I64, _vp, C.c_size_t, _vp]
    L.nl_neighbour_list.restype = C.c_int
    L.nl_neighbour_list_half.argtypes = L.nl_neighbour_list.argtypes
    L.nl_neighbour_list_half.restype = C.c_int
    L.nl_neighbour_list_static.argtypes = [_vp, C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, _vp, _vp,
                                           _vp, _vp, _vp, C.c_int64, _vp, _vp, _vp, _vp, _I64, _vp]
    L.nl_neighbour_list_static.restype = C.c_int
    L.nl_static_sync_status.argtypes = [_I64, _vp]
    L.nl_static_sync_status.restype = C.c_int
    L.nl_lazy_reduce.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, C.c_int,
                                 C.c_int, _vp, _vp, C.c_size_t, _vp]
    L.nl_lazy_reduce.restype = C.c_int
    L.nl_query_neighbours.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, _vp,
                                      C.c_int64, _vp, _vp, C.c_int64, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    L.nl_query_neighbours.restype = C.c_int
    L.nl_batch_create.argtypes = [C.POINTER(System), C.c_int, C.c_int, C.POINTER(_vp)]
    L.nl_batch_create.restype = C.c_int
    L.nl_batch_create_auto.argtypes = [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.POINTER(_vp)]
    L.nl_batch_create_auto.restype = C.c_int
    L.nl_batch_destroy.argtypes = [_vp]
    L.nl_batch_destroy.restype = None
    L.nl_batch_workspace_bytes.argtypes = [_vp]
    L.nl_batch_workspace_bytes.restype = C.c_size_t
    L.nl_batch_sizes.argtypes = [_vp, _I64, _I64]
    L.nl_batch_sizes.restype = C.c_int
    L.nl_batch_upload.argtypes = [_vp, _vp, C.c_size_t, _vp]
    L.nl_batch_upload.restype = C.c_int
    L.nl_batch_neighbour_list.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int64, _vp, _vp, _vp, _vp, _I64,
                                          _vp, C.c_size_t, _vp]
    L.nl_batch_neighbour_list.restype = C.c_int
    L.nl_batch_create_f32.argtypes = [C.POINTER(SystemF32), C.c_int, C.c_int, C.POINTER(_vp)]
    L.nl_batch_create_f32.restype = C.c_int
    L.nl_batch_create_auto_f32.argtypes = [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.POINTER(_vp)]
    L.nl_batch_create_auto_f32.restype = C.c_int
    L.nl_batch_neighbour_list_f32.argtypes = [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int64, _vp, _vp, _vp, _vp,
                                              _I64, _vp, C.c_size_t, _vp]
    L.nl_batch_neighbour_list_f32.restype = C.c_int
    _F = C.POINTER(C.c_float)
    L.nl_analyze_cell_f32.argtypes = [_F, C.c_float, C.c_int, C.POINTER(CellPlanF32)]
    L.nl_analyze_cell_f32.restype = C.c_int
    L.nl_build_cell_list_f32.argtypes = [_vp, C.c_int64, _F, _F, _I64, _U8, C.c_float, C.c_int, _vp, _vp, _vp, _vp,
                                         _vp, C.c_size_t, _vp]
    L.nl_build_cell_list_f32.restype = C.c_int
    L.nl_count_pairs_f32.argtypes = [_vp, _vp, _vp, _vp, C.c_int64, _F, _F, _I64, _I64, _U8, C.c_float, C.c_int,
                                     C.c_int, _vp, _I64, _vp, C.c_size_t, _vp]
    L.nl_count_pairs_f32.restype = C.c_int
    L.nl_fill_pairs_f32.argtypes = [_vp, _vp, _vp, C.c_int64, _F, _F, _I64, _I64, _U8, C.c_float, C.c_int, _vp,
                                    C.c_int64, _vp, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    L.nl_fill_pairs_f32.restype = C.c_int
    L.nl_neighbour_list_f32.argtypes = [_vp, C.c_int64, _F, _F, _I64, _I64, _U8, C.c_float, C.c_int, _vp, _vp, _vp,
                                        _vp, _vp, C.c_int64, _vp, _vp, _vp, _vp, _I64, _vp, C.c_size_t, _vp]
    L.nl_neighbour_list_f32.restype = C.c_int
    L.nl_neighbour_list_half_f32.argtypes = L.nl_neighbour_list_f32.argtypes
    L.nl_neighbour_list_half_f32.restype = C.c_int
    L.nl_legacy_fix_cell.argtypes = [_vp, C.c_int64, _D, _U8, _vp, _D, _vp, C.c_size_t, _vp]
    L.nl_legacy_fix_cell.restype = C.c_int
    L.nl_legacy_workspace_bytes.argtypes = [C.c_int64, C.c_int64, C.c_int]
    L.nl_legacy_workspace_bytes.restype = C.c_size_t
    L.nl_legacy_count_pairs.argtypes = [_vp, C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, _vp, _I64, _vp,
                                        C.c_size_t, _vp]
    L.nl_legacy_count_pairs.restype = C.c_int
    L.nl_legacy_fill_pairs.argtypes = [C.c_int64, _D, _D, _I64, _I64, _U8, C.c_double, C.c_int, _vp, C.c_int64, _vp,
                                       _vp, _vp, _vp, C.c_size_t, _vp]
    L.nl_legacy_fill_pairs.restype = C.c_int
    L.nl_set_tuning.argtypes = [C.POINTER(Tuning)]
    L.nl_set_tuning.restype = C.c_int
    L.nl_batch_set_tuning.argtypes = [_vp, C.POINTER(Tuning)]
    L.nl_batch_set_tuning.restype = C.c_int
    L.nl_pair_vectors.argtypes = [_vp, C.c_int64, _D, C.c_int, _vp, _vp, _vp, C.c_int64, _vp, _vp]
    L.nl_pair_vectors.restype = C.c_int
    L.nl_max_displacement_sq.argtypes = [_vp, _vp, C.c_int64, _vp, _vp]
    L.nl_max_displacement_sq.restype = C.c_int
    L.nl_pair_vectors_f32.argtypes = [_vp, C.c_int64, C.POINTER(C.c_float), C.c_int, _vp, _vp, _vp, C.c_int64, _vp,
                                      _vp]
    L.nl_pair_vectors_f32.restype = C.c_int
    L.nl_max_displacement_sq_f32.argtypes = [_vp, _vp, C.c_int64, _vp, _vp]
    L.nl_max_displacement_sq_f32.restype = C.c_int
    L.nl_sync_status.argtypes = [_vp, _vp]
    L.nl_sync_status.restype = C.c_int
    L.nl_last_recheck_count.argtypes = [_vp, _vp, _I64]
    L.nl_last_recheck_count.restype = C.c_int
    L.nl_status_string.argtypes = [C.c_int]
    L.nl_status_string.restype = C.c_char_p
    L.nl_last_error.argtypes = []
    L.nl_last_error.restype = C.c_char_p
    L.nl_version.argtypes = []
    L.nl_version.restype = C.c_int


def lib():
    """Loads libnlgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python neighbourlists.jl_gb300/build.py` "
                "(the GPU neighbour list has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != NL_OK:
        L = lib()
        detail = L.nl_last_error().decode(errors="replace")
        raise NLError(status, f"{L.nl_status_string(status).decode()}: {detail}")
