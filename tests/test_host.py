"""Host-side checks of the C ABI that need no GPU: the library loads and
exports every declared symbol, the restated cell analysis is bit-equal to the
oracle's, argument errors map to the reference's error behaviour, and the
FP32 screen band is wide enough (numpy emulation of the kernel arithmetic)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import configs as cf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "nlgpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|void|const char\*)\s+(nl_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(nlpkg):
    L = nlpkg.lib()
    decl = declared_symbols()
    assert len(decl) >= 12
    for name in decl:
        assert hasattr(L, name), name
    assert sorted(decl) == sorted(nlpkg._lib.EXPORTED)
    assert L.nl_version() >= 1


CELLS = [
    np.diag([58.48, 58.48, 58.48]),
    cf.triclinic_cell(),
    cf.fcc_sheared(n=20)[1],
    cf.diamond_primitive()[1],
    np.array([[7.0, 0.3, -0.2], [1.1, 6.5, 0.4], [-0.7, 2.2, 9.1]]),
    np.array([[3.0, 0.0, 0.0], [2.9, 0.5, 0.0], [0.1, 0.2, 40.0]]),
]


@pytest.mark.parametrize("k", range(len(CELLS)))
@pytest.mark.parametrize("rc", [1.7, 3.0, 5.0, 6.0])
def test_analyze_cell_bit_equal_to_oracle(nlpkg, orc, k, rc):
    cell = CELLS[k]
    p = nlpkg.analyze_cell(cell, rc)
    o = orc.analyze_cell(cell, rc)
    assert np.array_equal(p.inv_cell.view(np.int64), o.inv_cell.view(np.int64))
    assert np.array_equal(p.lens.view(np.int64), o.lens.view(np.int64))
    assert np.array_equal(p.ncells, o.ncells)
    assert np.array_equal(p.nxyz, o.nxyz)
    assert p.ncells_total == int(np.prod(o.ncells))


@pytest.mark.parametrize("k,rc", [(0, 5.0), (1, 3.0), (2, 6.0), (3, 0.7), (4, 2.5)])
def test_analyze_cell_f32_bit_equal_to_oracle(nlpkg, orc, k, rc):
    """analyze_cell with T = Float32 (cell and cutoff converted to Float32,
    every operation in single precision) equals the oracle's restatement."""
    cells = [np.diag([58.48] * 3), cf.triclinic_cell(), np.array([[5.43 / 2 * a for a in r] for r in
                                                                  [(0, 1, 1), (1, 0, 1), (1, 1, 0)]]),
             np.array([[3.3, 0.4, 0.1], [0.2, 2.9, 0.7], [0.0, 0.3, 4.1]]), np.diag([72.2, 72.2, 92.2])]
    plan = nlpkg.analyze_cell(cells[k], rc, float32=True)
    inv, ns, lens, nxyz = orc.analyze_cell_f32(cells[k], rc)
    assert plan.inv_cm.dtype == np.float32
    assert np.array_equal(plan.inv_cell.view(np.int32), inv.view(np.int32))
    assert np.array_equal(plan.lens.view(np.int32), lens.view(np.int32))
    assert plan.ncells.tolist() == ns.tolist() and plan.nxyz.tolist() == nxyz.tolist()


def test_too_many_cells_error(nlpkg):
    cell = np.diag([1e6, 1e6, 1e6])
    with pytest.raises(nlpkg.NLError) as e:
        nlpkg.analyze_cell(cell, 1e-3)
    assert e.value.status == 2 and "very large" in str(e.value)
    # Int64 lifts the index-type limit but not the engine's 2^31-2 cell limit
    with pytest.raises(nlpkg.NLError):
        nlpkg.analyze_cell(cell, 1e-3, int_type="Int64")


def test_argument_errors_before_any_device_work(nlpkg):
    L = nlpkg.lib()
    D = C.POINTER(C.c_double)
    I64 = C.POINTER(C.c_int64)
    U8 = C.POINTER(C.c_uint8)
    cell = np.ascontiguousarray(np.diag([10.0, 10.0, 10.0]).T).reshape(9)
    inv = np.ascontiguousarray(np.diag([0.1, 0.1, 0.1]).T).reshape(9)
    ns = np.array([3, 3, 3], dtype=np.int64)
    pbc = np.ones(3, dtype=np.uint8)
    # workspace too small
    st = L.nl_build_cell_list(C.c_void_p(8), 10, cell.ctypes.data_as(D), inv.ctypes.data_as(D),
                              ns.ctypes.data_as(I64), pbc.ctypes.data_as(U8), 3.0, 4, C.c_void_p(8), C.c_void_p(8),
                              C.c_void_p(8), C.c_void_p(8), C.c_void_p(8), 16, None)
    assert st == 3
    # bad index type
    plan = nlpkg._lib.CellPlan()
    assert L.nl_analyze_cell(cell.ctypes.data_as(D), 3.0, 2, C.byref(plan)) == 1
    assert L.nl_analyze_cell(cell.ctypes.data_as(D), -1.0, 4, C.byref(plan)) == 1
    assert L.nl_workspace_bytes(-1, 1) == 0
    assert L.nl_workspace_bytes(1000, 27) > 1000 * 48


# ---------------------------------------------------------------- screen --
def _f32(x):
    return np.asarray(x, dtype=np.float64).astype(np.float32)


def _fma32(a, b, c):
    return _f32(np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64))


def _bin(inv_cm, ns, pbc, X):
    """Restates the kernel binning: returns cell (1-based), winding, t (FP64)."""
    f = np.stack([(inv_cm[3 * k] * X[:, 0] + inv_cm[3 * k + 1] * X[:, 1]) + inv_cm[3 * k + 2] * X[:, 2]
                  for k in range(3)], 1)
    y = f * ns
    c0 = np.floor(y + 1.0).astype(np.int64)
    c = np.empty_like(c0)
    w = np.zeros_like(c0)
    for k in range(3):
        if pbc[k]:
            w[:, k] = np.floor_divide(c0[:, k] - 1, ns[k])
            c[:, k] = c0[:, k] - w[:, k] * ns[k]
        else:
            c[:, k] = np.clip(c0[:, k], 1, ns[k])
    m = (c - 1) + w * ns
    return c, w, y - m


def _screen_errors(cell, rc, pbc, X, pairs_per=400, seed=0):
    """Max |r2_fp32 - r2_fp64| over random candidate pairs, and the band."""
    from neighbourlists_gb300 import analyze_cell  # noqa: F401  (package loaded by fixture)

    rng = np.random.default_rng(seed)
    cm = np.ascontiguousarray(cell.T).reshape(9)
    import oracle as orc_mod

    info = orc_mod.analyze_cell(cell, rc)
    inv_cm = np.ascontiguousarray(info.inv_cell.T).reshape(9)
    ns = info.ncells
    nx = info.nxyz
    c, w, t = _bin(inv_cm, ns, pbc, X)
    b = np.array([[cell[k, r] / ns[k] for r in range(3)] for k in range(3)])  # b[k, r]
    b32 = _f32(b)
    t32 = _f32(t)
    u = np.stack([_fma32(t32[:, 2], b32[2, r], _fma32(t32[:, 1], b32[1, r], _f32(t32[:, 0] * b32[0, r])))
                  for r in range(3)], 1)
    ok = (np.abs(t) <= 2.0).all(1)
    n = X.shape[0]
    worst = 0.0
    for _ in range(pairs_per):
        i, j = rng.integers(0, n, 2)
        if not (ok[i] and ok[j]):
            continue
        d = c[j] - c[i]
        # bring d into the stencil like the traversal does (wrapped cell offsets)
        for k in range(3):
            if pbc[k]:
                d[k] = ((d[k] + ns[k] // 2) % ns[k]) - ns[k] // 2
        if np.any(np.abs(d) > nx):
            continue
        sl = np.zeros(3, dtype=np.int64)
        for k in range(3):
            if pbc[k]:
                sl[k] = np.floor_divide(c[i, k] + d[k] - 1, ns[k])
        S = sl + w[i] - w[j]
        R64 = (X[j] - X[i]) + np.array([(cell[0, r] * S[0] + cell[1, r] * S[1]) + cell[2, r] * S[2] for r in range(3)])
        r2_64 = (R64[0] * R64[0] + R64[1] * R64[1]) + R64[2] * R64[2]
        if r2_64 > 4 * rc * rc:
            continue
        fd = d.astype(np.float32)
        off = np.array([_fma32(fd[2], b32[2, r], _fma32(fd[1], b32[1, r], _f32(fd[0] * b32[0, r]))) for r in range(3)])
        v = _f32(u[j] + off)
        R32 = _f32(v - u[i])
        r2_32 = _fma32(R32[2], R32[2], _fma32(R32[1], R32[1], _f32(R32[0] * R32[0])))
        err = abs(float(r2_32) - r2_64) if r2_64 < rc * rc * 1.1 else 0.0
        worst = max(worst, err)
    return worst


@pytest.mark.parametrize("case", ["cubic", "triclinic", "sheared", "outside"])
def test_screen_band_bounds_fp32_error(nlpkg, orc, case):
    rng = np.random.default_rng(5)
    if case == "cubic":
        X, cell, _ = cf.rand_config(3000, seed=1)
        pbc, rc = (True, True, True), 5.0
    elif case == "triclinic":
        X, cell = cf.rand_config_triclinic(2000, seed=2)
        pbc, rc = (True, False, True), 3.0
    elif case == "sheared":
        X, cell, pbc = cf.fcc_sheared(n=6, seed=3)
        rc = 5.0
    else:  # atoms on cell corners and shifted by whole periods
        X, cell, L = cf.rand_config(2000, seed=4)
        X = np.round(X / (L / 11)) * (L / 11) + rng.integers(-2, 3, X.shape) * L
        pbc, rc = (True, True, True), 5.0
    band = nlpkg.analyze_cell(cell, rc).band
    worst = _screen_errors(cell, rc, pbc, X, pairs_per=6000)
    assert worst <= band / 2, (worst, band)


# ---------------------------------------------------------- legacy screen --
def _legacy_band(cell_cm, ns, nxyz, rc, Df):
    """The legacy kernel's band (nl_legacy.cu): e = 6u(2M + O), B = 2(4u rc^2
    + 2 sqrt(3)(rc + e) e + 3 e^2), M = max |D| in FP32 rounded up."""
    u = 2.0 ** -24
    bins = np.array([[cell_cm[k + 3 * r] / ns[k] for k in range(3)] for r in range(3)])  # bins[r, k]
    O = max(sum(abs(bins[r, k]) * nxyz[k] for k in range(3)) for r in range(3)) * (1 + 1e-12)
    M = float(np.max(np.abs(Df))) if Df.size else 0.0
    e = 6 * u * (2 * M + O) * 1.0001
    return bins, 2 * (4 * u * rc * rc + 2 * np.sqrt(3) * (rc + e) * e + 3 * e * e)


@pytest.mark.parametrize("case", ["cubic", "triclinic", "open_outside"])
def test_legacy_screen_band_bounds_fp32_error(nlpkg, case):
    """Every candidate whose FP32 legacy distance lies outside rc^2 -+ B is
    decided the same way by the reference's FP64 legacy arithmetic
    (cell_list.jl:346-352), so the FP64 recheck of the band is enough."""
    rng = np.random.default_rng(9)
    if case == "cubic":
        X, cell, _ = cf.rand_config(700, seed=31)
        pbc, rc = (True, True, True), 5.0
    elif case == "triclinic":
        X, cell = cf.rand_config_triclinic(500, seed=32)
        pbc, rc = (True, False, True), 3.0
    else:  # fixcell = false: atoms far outside along the open axis
        X, cell = cf.rand_config_triclinic(500, seed=33)
        X = X + np.outer(rng.normal(0, 8.0, len(X)), [0.0, 0.0, 1.0])
        pbc, rc = (True, True, False), 3.0
    plan = nlpkg.analyze_cell(cell, rc)
    cm, inv, ns, nxyz = plan.cell_cm, plan.inv_cm, plan.ncells, plan.nxyz
    f = np.stack([(inv[3 * k] * X[:, 0] + inv[3 * k + 1] * X[:, 1]) + inv[3 * k + 2] * X[:, 2] for k in range(3)], 1)
    c0 = np.floor(f * ns + 1.0).astype(np.int64)
    ct = np.stack([c0[:, k] if pbc[k] else np.clip(c0[:, k], 1, ns[k]) for k in range(3)], 1)
    bins0 = np.array([[cm[k + 3 * r] / ns[k] for k in range(3)] for r in range(3)])
    v = (ct - 1).astype(np.float64)
    D = np.stack([X[:, r] - ((bins0[r, 0] * v[:, 0] + bins0[r, 1] * v[:, 1]) + bins0[r, 2] * v[:, 2])
                  for r in range(3)], 1)
    Df = D.astype(np.float32)
    bins, B = _legacy_band(cm, ns, nxyz, rc, np.abs(D).astype(np.float32))
    worst_ratio = 0.0
    for x in range(-nxyz[0], nxyz[0] + 1):
        for y in range(-nxyz[1], nxyz[1] + 1):
            for z in range(-nxyz[2], nxyz[2] + 1):
                off = np.array([(bins[r, 0] * x + bins[r, 1] * y) + bins[r, 2] * z for r in range(3)])
                d64 = (D[None, :, :] - D[:, None, :]) + off
                r64 = (d64[..., 0] * d64[..., 0] + d64[..., 1] * d64[..., 1]) + d64[..., 2] * d64[..., 2]
                # the kernel's FP32 offset: fma(b6, z, fma(b3, y, b0 * x)) on the FP32 bins
                bf = bins.astype(np.float32)
                off32 = np.array([np.float32(np.float64(bf[r, 2]) * z + np.float64(
                    np.float32(np.float64(bf[r, 1]) * y + np.float64(np.float32(bf[r, 0] * np.float32(x))))))
                    for r in range(3)], dtype=np.float32)
                d32 = (Df[None, :, :] - Df[:, None, :]) + off32
                r32 = (d32[..., 0] * d32[..., 0] + d32[..., 1] * d32[..., 1]) + d32[..., 2] * d32[..., 2]
                near = r64 < 4 * rc * rc
                err = np.abs(r32[near].astype(np.float64) - r64[near])
                if err.size:
                    worst_ratio = max(worst_ratio, float(err.max()) / B)
                assert not np.any((r64 < rc * rc) & (r32.astype(np.float64) > rc * rc + B))
                assert not np.any((r64 >= rc * rc) & (r32.astype(np.float64) < rc * rc - B))
    assert worst_ratio < 0.5, worst_ratio


def test_legacy_argument_errors_before_any_device_work(nlpkg):
    L = nlpkg.lib()
    D = C.POINTER(C.c_double)
    I64 = C.POINTER(C.c_int64)
    U8 = C.POINTER(C.c_uint8)
    cell = np.ascontiguousarray(np.diag([10.0, 10.0, 10.0]).T).reshape(9)
    inv = np.ascontiguousarray(np.diag([0.1, 0.1, 0.1]).T).reshape(9)
    ns = np.array([3, 3, 3], dtype=np.int64)
    nx = np.array([1, 1, 1], dtype=np.int64)
    pbc = np.ones(3, dtype=np.uint8)
    out = np.zeros(9)
    assert L.nl_legacy_workspace_bytes(-1, 1, 4) == 0
    assert L.nl_legacy_workspace_bytes(10, 27, 3) == 0
    assert L.nl_legacy_workspace_bytes(1000, 27, 8) > L.nl_workspace_min_bytes(1000, 27) + 1000 * 80
    # null cell / too small workspace for the cell fix
    assert L.nl_legacy_fix_cell(C.c_void_p(8), 10, None, pbc.ctypes.data_as(U8), C.c_void_p(8),
                                out.ctypes.data_as(D), C.c_void_p(8), 256, None) == 1
    assert L.nl_legacy_fix_cell(C.c_void_p(8), 10, cell.ctypes.data_as(D), pbc.ctypes.data_as(U8), C.c_void_p(8),
                                out.ctypes.data_as(D), C.c_void_p(8), 16, None) == 3
    # workspace smaller than nl_legacy_workspace_bytes
    need = L.nl_legacy_workspace_bytes(10, 27, 4)
    total = C.c_int64(0)
    assert L.nl_legacy_count_pairs(C.c_void_p(8), 10, cell.ctypes.data_as(D), inv.ctypes.data_as(D),
                                   ns.ctypes.data_as(I64), nx.ctypes.data_as(I64), pbc.ctypes.data_as(U8), 3.0, 4,
                                   C.c_void_p(8), C.byref(total), C.c_void_p(8), need - 1, None) == 3
    assert L.nl_legacy_fill_pairs(10, cell.ctypes.data_as(D), inv.ctypes.data_as(D), ns.ctypes.data_as(I64),
                                  nx.ctypes.data_as(I64), pbc.ctypes.data_as(U8), 3.0, 4, C.c_void_p(8), 10,
                                  None, None, None, C.c_void_p(8), need, None) == 1


def test_batch_plan_on_host(nlpkg):
    """nl_batch_create validates systems and sizes the workspace without a GPU."""
    import ctypes as C
    L = nlpkg._lib.lib()
    arr = (nlpkg._lib.System * 2)()
    for s, n in enumerate((10, 0)):
        p = nlpkg.analyze_cell(np.diag([10.0, 12.0, 14.0]), 3.0)
        arr[s].nat = n
        arr[s].cell[:] = p.cell_cm.tolist()
        arr[s].inv_cell[:] = p.inv_cm.tolist()
        arr[s].ncells[:] = p.ncells.tolist()
        arr[s].nxyz[:] = p.nxyz.tolist()
        arr[s].pbc[:] = [1, 1, 0]
        arr[s].cutoff = 3.0
    h = C.c_void_p()
    assert L.nl_batch_create(arr, 2, 4, C.byref(h)) == 0
    na, nc = C.c_int64(), C.c_int64()
    assert L.nl_batch_sizes(h, C.byref(na), C.byref(nc)) == 0
    assert na.value == 10 and nc.value == 2 * 3 * 4 * 4
    # the single-system layout for all atoms and cells, plus the system of every cell
    assert L.nl_batch_workspace_bytes(h) >= L.nl_workspace_bytes(10, nc.value) + 4 * nc.value
    L.nl_batch_destroy(h)
    arr[1].nxyz[0] = 63
    assert L.nl_batch_create(arr, 2, 4, C.byref(h)) == nlpkg._lib.NL_ERR_ARG
    assert b"system 1" in L.nl_last_error()
    assert L.nl_batch_create(arr, 0, 4, C.byref(h)) == nlpkg._lib.NL_ERR_ARG


def test_lists_move_between_devices(nlpkg):
    """PairList / SortedCellList .to(device) (the reference's Adapt rules,
    adapt.jl:20-44) move every array field and keep the rest."""
    import torch

    P = nlpkg.PairList(torch.zeros((3, 3), dtype=torch.float64), np.eye(3), 2.0, torch.tensor([1, 1, 2], dtype=torch.int32),
                       torch.tensor([2, 3, 1], dtype=torch.int32), torch.zeros((3, 3), dtype=torch.int32),
                       torch.tensor([1, 3, 4, 4], dtype=torch.int32), torch.ones((3, 3), dtype=torch.float64))
    Q = P.to("cpu")
    assert Q.i.tolist() == [1, 1, 2] and Q.first.tolist() == [1, 3, 4, 4] and Q.cutoff == 2.0
    assert nlpkg.nneigs(Q, 1) == 2 and nlpkg.npairs(Q) == 3


def test_autotune_candidates_and_choice(nlpkg, monkeypatch):
    """The tuner times every (pair blocks, emit blocks, count kernel) set --
    the symmetric count pass among them for any runner, single system or
    batch -- and leaves the fastest on the runner (the CUDA-event timer is
    replaced by a fixed cost per set here)."""
    import sys

    tuning = sys.modules[nlpkg.__name__ + ".tuning"]

    class Runner:
        def __init__(self):
            self.t = None

        def run(self, X):
            return 0

        def set_tuning(self, p, e, k):
            self.t = (p, e, k)

        def launch(self, X):
            pass

        def sync_status(self):
            pass

    r = Runner()
    cost = lambda t: abs(t[0] - 7) + abs(t[1] - 16) / 8 + (0 if t[2] == 3 else 1)  # noqa: E731
    monkeypatch.setattr(tuning, "_time_ms", lambda fn, reps: (fn(), cost(r.t))[1])
    res = tuning.autotune(r, None, reps=1)
    assert len(res["trials"]) == len(tuning.PAIR_BLOCKS) * len(tuning.EMIT_BLOCKS) * len(tuning.COUNT_KERNELS)
    assert {t["count_kernel"] for t in res["trials"]} == {1, 2, 3}
    assert r.t == (7, 16, 3)
    assert (res["pair_blocks_per_sm"], res["emit_blocks_per_sm"], res["count_kernel"]) == (7, 16, 3)
    res = tuning.autotune(r, None, candidates=[(4, 8), (14, 32, 2)], reps=1)
    assert [(t["pair_blocks_per_sm"], t["emit_blocks_per_sm"], t["count_kernel"]) for t in res["trials"]] == \
        [(4, 8, 0), (14, 32, 2)]


def test_numa_helpers_on_the_host(nlpkg):
    """The NUMA helpers of the end-to-end buffers: CPU lists parse, and a
    buffer's pages are reported on an existing node."""
    import torch
    from neighbourlists_gb300 import numa

    nodes = numa.cpu_nodes()
    if not nodes:
        pytest.skip("no NUMA information on this host")
    for node, cpus in nodes.items():
        assert cpus and cpus == numa.node_cpus(node)
    t = torch.zeros(1 << 22, dtype=torch.uint8)
    where = numa.page_nodes(t)
    assert where and sum(where.values()) > 0
    assert numa.node_cpus(10**6) == set()
