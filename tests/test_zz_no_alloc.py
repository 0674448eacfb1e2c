"""nl_neighbour_list_static: the materialised pipeline for callers that cannot
allocate device memory (its scratch is a fixed 32 MiB array inside the
library instead of a caller-provided workspace).

Checked through the C ABI against the workspace entry point nl_neighbour_list
on the same inputs, bit for bit, on two calls in a row with different systems
(the second call reuses the shared scratch the first one left behind).  This
file is collected last so that a failure here cannot hide other failures."""
import ctypes as C

import numpy as np
import pytest
import torch

import configs as cf

pytestmark = pytest.mark.gpu

_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_U8 = C.POINTER(C.c_uint8)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None and t.numel() else C.c_void_p(0)


def _run(nlpkg, X, cell, rc, pbc, static):
    L = nlpkg.lib()
    plan = nlpkg.analyze_cell(cell, rc)
    nat = X.shape[0]
    dev = torch.device("cuda")
    ti = torch.int32
    Xd = torch.from_numpy(np.ascontiguousarray(X)).to(dev)
    out = {
        "perm": torch.empty(nat, dtype=ti, device=dev),
        "X_sorted": torch.empty((nat, 3), dtype=torch.float64, device=dev),
        "cell_id": torch.empty(nat, dtype=ti, device=dev),
        "cell_offsets": torch.empty(plan.ncells_total + 1, dtype=ti, device=dev),
        "first": torch.empty(nat + 1, dtype=ti, device=dev),
    }
    cap = 200 * nat + 1024
    out.update(i=torch.empty(cap, dtype=ti, device=dev), j=torch.empty(cap, dtype=ti, device=dev),
               S=torch.empty((cap, 3), dtype=ti, device=dev), R=torch.empty((cap, 3), dtype=torch.float64, device=dev))
    pb = np.array([1 if p else 0 for p in pbc], dtype=np.uint8)
    total = C.c_int64(-1)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [_p(Xd), nat, plan.cell_cm.ctypes.data_as(_D), plan.inv_cm.ctypes.data_as(_D),
            plan.ncells.ctypes.data_as(_I64), plan.nxyz.ctypes.data_as(_I64), pb.ctypes.data_as(_U8), float(rc), 4,
            _p(out["perm"]), _p(out["X_sorted"]), _p(out["cell_id"]), _p(out["cell_offsets"]), _p(out["first"]),
            cap, _p(out["i"]), _p(out["j"]), _p(out["S"]), _p(out["R"]), C.byref(total)]
    if static:
        st = L.nl_neighbour_list_static(*args, stream)
    else:
        ws = torch.empty(int(L.nl_workspace_bytes(nat, plan.ncells_total)), dtype=torch.uint8, device=dev)
        st = L.nl_neighbour_list(*args, _p(ws), ws.numel(), stream)
    assert st == 0, L.nl_last_error().decode()
    P = int(total.value)
    for k in ("i", "j", "S", "R"):
        out[k] = out[k][:P]
    return {k: v.cpu().numpy() for k, v in out.items()}


def _same(a, b):
    for k in a:
        x, y = a[k], b[k]
        if x.dtype == np.float64:
            x, y = x.view(np.int64), y.view(np.int64)
        assert np.array_equal(x, y), k


def test_static_scratch_matches_workspace_path_twice(nlpkg):
    X1, C1, _ = cf.rand_config(20000, seed=41)
    X2, C2, pbc2 = cf.fcc_sheared(n=8, seed=42)
    cases = [(X1, C1, 5.0, (True, True, True)), (X2, C2, 5.0, pbc2)]
    refs = [_run(nlpkg, *c, static=False) for c in cases]
    for (case, ref) in zip(cases, refs):  # two calls in a row on the shared scratch
        got = _run(nlpkg, *case, static=True)
        assert got["i"].shape[0] > 0
        _same(got, ref)


def test_static_scratch_rejects_oversize_systems(nlpkg):
    L = nlpkg.lib()
    cell = np.diag([300.0] * 3)
    plan = nlpkg.analyze_cell(cell, 5.0)
    pb = np.ones(3, dtype=np.uint8)
    total = C.c_int64(-1)
    st = L.nl_neighbour_list_static(C.c_void_p(0), 5_000_000, plan.cell_cm.ctypes.data_as(_D),
                                    plan.inv_cm.ctypes.data_as(_D), plan.ncells.ctypes.data_as(_I64),
                                    plan.nxyz.ctypes.data_as(_I64), pb.ctypes.data_as(_U8), 5.0, 4, None, None, None,
                                    None, None, 0, None, None, None, None, C.byref(total), None)
    assert st == 3  # NL_ERR_NOMEM
    assert "32 MiB" in L.nl_last_error().decode()
