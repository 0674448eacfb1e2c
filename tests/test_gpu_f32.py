"""GPU parity of the single-precision path (positions, cell and cutoff in
Float32) against the oracle's Float32 restatement of the reference
(oracle/nl_oracle_f32.c): the SortedCellList arrays and i, j, S, first and
the bits of R identical in the reference's order.  The reference runs its GPU
tests for Float64 and Float32 (test/test_gpu.jl:14, test/test_utils.jl:239);
the cases follow those tests plus atoms outside the cell (windings) and
cutoff-boundary lattices."""
import numpy as np
import pytest
import torch

import configs as cf

pytestmark = pytest.mark.gpu


def to_np(t):
    return t.detach().cpu().numpy()


def run_both(nlpkg, orc, X, rc, cell, pbc, int_type=torch.int32):
    X32 = np.ascontiguousarray(np.asarray(X).astype(np.float32).reshape(-1, 3))
    clist = nlpkg.build_cell_list(torch.from_numpy(X32).cuda(), rc, cell, pbc, int_type=int_type)
    g = nlpkg.materialize_pairlist(clist)
    o = orc.neighbour_list_f32(X32, rc, cell, pbc, ti_bytes=4 if int_type == torch.int32 else 8)
    return clist, g, o


def assert_identical(clist, g, o):
    np.testing.assert_array_equal(to_np(clist.perm).astype(np.int64), o.perm)
    np.testing.assert_array_equal(to_np(clist.cell_id).astype(np.int64), o.cell_id)
    np.testing.assert_array_equal(to_np(clist.cell_offsets).astype(np.int64), o.cell_offsets)
    assert np.array_equal(to_np(clist.X).view(np.int32), o.X_sorted.view(np.int32))
    assert g.R.dtype == torch.float32 and int(g.i.shape[0]) == o.npairs
    np.testing.assert_array_equal(to_np(g.first).astype(np.int64), o.first)
    np.testing.assert_array_equal(to_np(g.i).astype(np.int64), o.i)
    np.testing.assert_array_equal(to_np(g.j).astype(np.int64), o.j)
    np.testing.assert_array_equal(to_np(g.S).astype(np.int64), o.S)
    assert np.array_equal(to_np(g.R).view(np.int32), o.R.view(np.int32)), "R bits differ"


@pytest.mark.parametrize("seed", range(5))
def test_random_configs(nlpkg, orc, seed):
    N = 50 + 37 * seed
    X, C, L = cf.rand_config(N, seed=500 + seed)
    assert_identical(*run_both(nlpkg, orc, X, L / 3, C, (True, True, True)))


@pytest.mark.parametrize("pbc", cf.ALL_PBC)
def test_all_pbc(nlpkg, orc, pbc):
    X, C, L = cf.rand_config(50, seed=57)
    assert_identical(*run_both(nlpkg, orc, X, 0.33 * L, C, pbc))
    X, C, L = cf.rand_config(3000, seed=58)
    assert_identical(*run_both(nlpkg, orc, X, 5.0, C, pbc))


def test_triclinic_and_elongated(nlpkg, orc):
    X, C = cf.rand_config_triclinic(80, seed=59)
    assert_identical(*run_both(nlpkg, orc, X, 3.0, C, (True, True, True)))
    C2 = np.diag([5.0, 5.0, 20.0])
    X2 = np.random.default_rng(60).random((80, 3)) @ C2
    assert_identical(*run_both(nlpkg, orc, X2, 3.0, C2, (True, True, True)))
    X3, C3 = cf.fcc_sheared(n=6, seed=61)[:2]
    assert_identical(*run_both(nlpkg, orc, X3, 5.0, C3, (True, True, False)))


def test_known_answers(nlpkg, orc):
    X, C = cf.diamond_primitive()
    clist, g, o = run_both(nlpkg, orc, X, 6.0, C, (True, True, True))
    assert o.npairs == 92 and list(np.diff(to_np(g.first))) == [46, 46]
    assert_identical(clist, g, o)
    X, C = cf.fcc_cubic(3.61, (3, 3, 3))
    clist, g, o = run_both(nlpkg, orc, X, 3.5, C, (True, True, True))
    assert np.all(np.diff(to_np(g.first)) == 12)
    assert_identical(clist, g, o)


def test_atoms_outside_the_cell(nlpkg, orc):
    X, C, L = cf.rand_config(600, seed=62)
    X = X + np.random.default_rng(63).integers(-4, 5, X.shape) * L
    for pbc in [(True, True, True), (True, False, True), (False, False, False)]:
        assert_identical(*run_both(nlpkg, orc, X, 0.2 * L, C, pbc))


def test_cutoff_boundary_lattice(nlpkg, orc):
    X, C = cf.fcc_cubic(3.61, (4, 4, 4))
    rc = np.float32(3.61) / np.sqrt(np.float32(2))
    for r in (np.nextafter(rc, np.float32(0)), rc, np.nextafter(rc, np.float32(10))):
        assert_identical(*run_both(nlpkg, orc, X, float(r), C, (True, True, True)))


def test_int64_and_sizes(nlpkg, orc):
    X, C, L = cf.rand_config(20000, seed=64)
    assert_identical(*run_both(nlpkg, orc, X, 5.0, C, (True, True, True), int_type=torch.int64))
    assert_identical(*run_both(nlpkg, orc, X, 5.0, C, (True, False, True)))


def test_edge_cases(nlpkg, orc):
    C = np.diag([10.0] * 3)
    for X, pbc in [(np.zeros((0, 3)), (1, 1, 1)), (np.array([[5.0, 5.0, 5.0]]), (1, 1, 1)),
                   (np.array([[5.0, 5.0, 5.0], [5.0, 5.0, 6.0]]), (1, 1, 1)),
                   (np.array([[1.0, 1.0, 1.0], [8.0, 8.0, 8.0]]), (0, 0, 0))]:
        assert_identical(*run_both(nlpkg, orc, X, 3.0, C, pbc))


def test_lazy_and_unified_api(nlpkg, orc):
    X, C, L = cf.rand_config(1000, seed=65)
    X32 = X.astype(np.float32)
    o = orc.neighbour_list_f32(X32, 0.25 * L, C, (1, 1, 1))
    nl = nlpkg.neighbour_list(torch.from_numpy(X32).cuda(), 0.25 * L, C, (True, True, True))
    np.testing.assert_array_equal(to_np(nl.j).astype(np.int64), o.j)
    clist = nlpkg.neighbour_list(torch.from_numpy(X32).cuda(), 0.25 * L, C, (True, True, True), lazy=True)
    np.testing.assert_array_equal(to_np(nlpkg.lazy_reduce(clist, "count")).astype(np.int64), np.diff(o.first))
    js, Rs, Ss = nlpkg.neighbours(clist, 7)
    a, b = o.first[6] - 1, o.first[7] - 1
    np.testing.assert_array_equal(to_np(js).astype(np.int64), o.j[a:b])
    assert np.array_equal(to_np(Rs).view(np.int32), o.R[a:b].view(np.int32))


def test_bad_positions_raise(nlpkg):
    X = torch.tensor([[1.0, 2.0, 3.0], [float("inf"), 0.0, 0.0]], dtype=torch.float32, device="cuda")
    with pytest.raises(nlpkg.NLError):
        nlpkg.build_cell_list(X, 2.0, np.diag([10.0] * 3), (True, True, True))


def test_engine_float32(nlpkg, orc):
    """The resident pipeline (nl_neighbour_list_f32, no host synchronisation)
    gives the same arrays, also when captured in a CUDA graph."""
    X, C, L = cf.rand_config(5000, seed=66)
    X32 = np.ascontiguousarray(X.astype(np.float32))
    o = orc.neighbour_list_f32(X32, 5.0, C, (1, 1, 1))
    Xd = torch.from_numpy(X32).cuda()
    eng = nlpkg.NeighbourListEngine(X.shape[0], C, 5.0, (True, True, True), dtype=torch.float32)
    assert eng.run(Xd) == o.npairs
    for _ in range(2):
        g = eng.pairlist(Xd)
        np.testing.assert_array_equal(to_np(g.first).astype(np.int64), o.first)
        np.testing.assert_array_equal(to_np(g.j).astype(np.int64), o.j)
        np.testing.assert_array_equal(to_np(g.S).astype(np.int64), o.S)
        assert np.array_equal(to_np(g.R).view(np.int32), o.R.view(np.int32))
        eng.R.zero_()
        eng.capture(Xd)
        eng.replay()
        torch.cuda.synchronize()
    with pytest.raises(TypeError):
        eng.launch(Xd.double())


def test_symmetric_pass_and_fallback(nlpkg, orc):
    """The symmetric count with neighbour masks (distinct 27-cell stencils),
    atoms with more than 64 pairs, and crowded cells (> 32 atoms: the
    per-cell passes run instead), all identical to the oracle."""
    X, C, L = cf.rand_config(4000, seed=55)
    assert_identical(*run_both(nlpkg, orc, X, 6.0, C, (True, True, False)))
    Xd = np.random.default_rng(7).random((3000, 3)) * 4.0
    assert_identical(*run_both(nlpkg, orc, Xd, 1.1, np.diag([4.0] * 3), (True, True, True)))
    for k in (1, 2):  # per-cell passes forced
        X32 = np.ascontiguousarray(X.astype(np.float32))
        eng = nlpkg.NeighbourListEngine(X.shape[0], C, 5.0, (True, True, True), dtype=torch.float32)
        eng.set_tuning(0, 0, k)
        eng.run(torch.from_numpy(X32).cuda())
        o = orc.neighbour_list_f32(X32, 5.0, C, (True, True, True))
        np.testing.assert_array_equal(to_np(eng.pairlist(None).j).astype(np.int64), o.j)


def test_batch_float32_every_system(nlpkg, orc):
    """A Float32 batch (nl_batch_create_f32 / nl_batch_neighbour_list_f32):
    uneven triclinic systems with mixed boundaries, a one-atom and an empty
    system, atoms outside their cell -- every system's SortedCellList arrays,
    first, i, j, S and the bits of R equal the oracle's Float32 restatement,
    as for a single-system call; Int32 and Int64 indices."""
    systems = cf.batch_systems(60, seed=31, nmin=1, nmax=700)
    rng = np.random.default_rng(32)
    systems[3] = (np.zeros((0, 3)), systems[3][1], systems[3][2], systems[3][3])
    x, c, rc, p = systems[7]
    x = x.copy()
    x[: max(1, len(x) // 5)] += rng.uniform(-1.5, 1.5, (max(1, len(x) // 5), 3)) @ np.asarray(c)  # windings
    systems[7] = (x, c, rc, p)
    X32 = [np.ascontiguousarray(np.asarray(x, dtype=np.float32).reshape(-1, 3)) for (x, _, _, _) in systems]
    for int_type in (torch.int32, torch.int64):
        b = nlpkg.BatchNeighbourList([(len(x), c, rc, p) for (x, (_, c, rc, p)) in zip(X32, systems)],
                                     int_type=int_type, dtype=torch.float32)
        b.run(torch.from_numpy(np.concatenate(X32)).cuda())
        po = b.pair_offsets_host().astype(np.int64)
        h = {k: to_np(getattr(b, k)) for k in ("perm", "Xs", "cid", "offs", "first", "i", "j", "S", "R")}
        assert h["Xs"].dtype == np.float32 and h["R"].dtype == np.float32
        for s, (x, (_, c, rc, p)) in enumerate(zip(X32, systems)):
            o = orc.neighbour_list_f32(x, rc, c, p, ti_bytes=4 if int_type == torch.int32 else 8)
            a0, a1 = int(b.atom0[s]), int(b.atom0[s + 1])
            c0, c1 = int(b.cell0[s]) + s, int(b.cell0[s + 1]) + s + 1
            p0, p1 = int(po[s]), int(po[s + 1])
            assert p1 - p0 == o.npairs, s
            np.testing.assert_array_equal(h["perm"][a0:a1].astype(np.int64), o.perm)
            np.testing.assert_array_equal(h["cid"][a0:a1].astype(np.int64), o.cell_id)
            np.testing.assert_array_equal(h["offs"][c0:c1].astype(np.int64), o.cell_offsets)
            assert np.array_equal(h["Xs"][a0:a1].view(np.int32), o.X_sorted.view(np.int32)), s
            np.testing.assert_array_equal(h["first"][a0 + s:a1 + s + 1].astype(np.int64), o.first)
            np.testing.assert_array_equal(h["i"][p0:p1].astype(np.int64), o.i)
            np.testing.assert_array_equal(h["j"][p0:p1].astype(np.int64), o.j)
            np.testing.assert_array_equal(h["S"][p0:p1].astype(np.int64), o.S)
            assert np.array_equal(h["R"][p0:p1].view(np.int32), o.R.view(np.int32)), s
        clist, pl = b.system(7)  # the per-system views carry the Float32 plan
        assert clist.X.dtype == torch.float32 and pl.R.dtype == torch.float32


def _half_keep(i, j, S):
    s = S.astype(np.int64)
    return (j > i) | ((j == i) & ((s[:, 0] > 0) | ((s[:, 0] == 0) & ((s[:, 1] > 0) | ((s[:, 1] == 0) & (s[:, 2] > 0))))))


@pytest.mark.parametrize("case", range(3))
def test_half_list_float32(nlpkg, orc, case):
    """Float32 half lists (nl_neighbour_list_half_f32): the oracle's Float32
    full list filtered by the half rule (j > i, or j == i and S > 0
    lexicographically), in the reference's order, bits of R included."""
    if case == 0:
        X, C, L = cf.rand_config(3000, seed=61)
        rc, pbc = 5.0, (True, True, True)
    elif case == 1:
        X, C = cf.rand_config_triclinic(400, seed=62)
        rc, pbc = 3.0, (True, False, True)
    else:
        X, C = cf.diamond_primitive()
        rc, pbc = 6.0, (True, True, True)
    X32 = np.ascontiguousarray(np.asarray(X, dtype=np.float32).reshape(-1, 3))
    pl = nlpkg.neighbour_list(torch.from_numpy(X32).cuda(), rc, C, pbc, half=True)
    o = orc.neighbour_list_f32(X32, rc, C, pbc)
    keep = _half_keep(o.i, o.j, o.S)
    assert pl.R.dtype == torch.float32 and int(pl.i.shape[0]) == int(keep.sum())
    np.testing.assert_array_equal(to_np(pl.i).astype(np.int64), o.i[keep])
    np.testing.assert_array_equal(to_np(pl.j).astype(np.int64), o.j[keep])
    np.testing.assert_array_equal(to_np(pl.S).astype(np.int64), o.S[keep])
    assert np.array_equal(to_np(pl.R).view(np.int32), o.R[keep].view(np.int32))
    counts = np.bincount(o.i[keep] - 1, minlength=X32.shape[0])
    np.testing.assert_array_equal(np.diff(to_np(pl.first).astype(np.int64)), counts)


def test_verlet_reuse_float32(nlpkg, orc):
    """Verlet reuse with Float32 positions: R of the kept pairs recomputed with
    the reference's single-precision operations (bit-equal to a numpy float32
    restatement of _getR), every pair within the cutoff equal to the oracle's
    Float32 list, rebuild once atoms moved beyond skin / 2."""
    X0, C, L = cf.rand_config(5000, seed=95)
    rc, skin, pbc = 5.0, 1.0, (True, True, True)
    v = nlpkg.VerletList(X0.shape[0], C, rc, skin, pbc, dtype=torch.float32)
    C32 = np.asarray(C, dtype=np.float32)
    rng = np.random.default_rng(96)
    X = X0.astype(np.float32)
    for step in range(4):
        rebuilt = v.update(torch.from_numpy(X).cuda())
        assert rebuilt == (step in (0, 3))
        P = v.engine.total_pairs()
        i, j, S = (t[:P].cpu().numpy().astype(np.int64) for t in (v.engine.i, v.engine.j, v.engine.S))
        R = v.engine.R[:P].cpu().numpy()
        assert R.dtype == np.float32
        Sf = S.astype(np.float32)
        cs = (Sf[:, 0:1] * C32[0] + Sf[:, 1:2] * C32[1]) + Sf[:, 2:3] * C32[2]  # float32, left fold, no FMA
        ref = (X[j - 1] - X[i - 1]) + cs
        assert np.array_equal(R.view(np.int32), ref.view(np.int32))
        o = orc.neighbour_list_f32(X, rc, C, pbc)
        inside = ((R[:, 0] * R[:, 0] + R[:, 1] * R[:, 1]) + R[:, 2] * R[:, 2]) < np.float32(rc) * np.float32(rc)
        got = set(zip(i[inside].tolist(), j[inside].tolist(), map(tuple, S[inside].tolist())))
        want = set(zip(o.i.tolist(), o.j.tolist(), map(tuple, o.S.tolist())))
        assert got == want
        X = (X + rng.uniform(-0.12, 0.12, size=X.shape) * (1.0 if step < 2 else 4.0)).astype(np.float32)
