"""GPU parity: the sm_103a kernels, called through the C ABI, against the CPU
oracle on the same seeded inputs.  i, j, S, first and the bits of R must be
identical -- not only after canonical (i, j, S) ordering but in the
reference's own output order -- and the SortedCellList arrays must equal the
reference's stable sort.  Cases follow the reference's tests
(test/test_sortbased.jl, test/test_gpu.jl, test/test_unified_api.jl,
test/test_atoms_base.jl) and the benchmark configurations."""
import numpy as np
import pytest
import torch

import configs as cf
import golden_io

pytestmark = pytest.mark.gpu


def to_np(t):
    return t.detach().cpu().numpy()


def assert_identical(g, o, with_R=True):
    assert int(g.i.shape[0]) == o.npairs
    np.testing.assert_array_equal(to_np(g.first).astype(np.int64), o.first)
    np.testing.assert_array_equal(to_np(g.i).astype(np.int64), o.i)
    np.testing.assert_array_equal(to_np(g.j).astype(np.int64), o.j)
    np.testing.assert_array_equal(to_np(g.S).astype(np.int64), o.S)
    if with_R:
        gr = to_np(g.R)
        assert np.array_equal(gr.view(np.int64), o.R.view(np.int64)), "R bits differ"


def run_both(nlpkg, orc, X, rc, cell, pbc, int_type=torch.int32):
    g = nlpkg.neighbour_list(torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).cuda(), rc, cell, pbc,
                             int_type=int_type)
    o = orc.neighbour_list(X, rc, cell, pbc, nthreads=8)
    return g, o


def test_golden_fixtures_bit_identical(nlpkg):
    for case in golden_io.load_all():
        g = nlpkg.neighbour_list(torch.from_numpy(case["X"]).cuda(), case["cutoff"], case["cell"], case["pbc"])
        assert int(g.i.shape[0]) == case["i"].shape[0], case["name"]
        for key in ("i", "j", "S", "first"):
            assert np.array_equal(to_np(getattr(g, key)).astype(np.int64), case[key]), (case["name"], key)
        assert np.array_equal(to_np(g.R).view(np.int64), case["R"].view(np.int64)), case["name"]


@pytest.mark.parametrize("seed", range(5))
def test_random_configs(nlpkg, orc, seed):
    N = 50 + 37 * seed
    X, C, L = cf.rand_config(N, seed=100 + seed)
    assert_identical(*run_both(nlpkg, orc, X, 0.33 * L, C, (True, True, True)))


@pytest.mark.parametrize("pbc", cf.ALL_PBC)
def test_all_pbc(nlpkg, orc, pbc):
    X, C, L = cf.rand_config(50, seed=7)
    assert_identical(*run_both(nlpkg, orc, X, 0.33 * L, C, pbc))
    X, C, L = cf.rand_config(3000, seed=8)
    assert_identical(*run_both(nlpkg, orc, X, 5.0, C, pbc))


def test_triclinic_elongated_large_cutoff(nlpkg, orc):
    X, C = cf.rand_config_triclinic(80, seed=3)
    assert_identical(*run_both(nlpkg, orc, X, 3.0, C, (True, True, True)))
    C2 = np.diag([5.0, 5.0, 20.0])
    X2 = np.random.default_rng(4).random((80, 3)) @ C2
    assert_identical(*run_both(nlpkg, orc, X2, 3.0, C2, (True, True, True)))
    X3, C3, L3 = cf.rand_config(30, seed=5)
    assert_identical(*run_both(nlpkg, orc, X3, 0.6 * L3, C3, (True, True, True)))


@pytest.mark.parametrize("N", [500, 1000, 2000])
def test_sizes(nlpkg, orc, N):
    X, C, L = cf.rand_config(N, seed=N)
    assert_identical(*run_both(nlpkg, orc, X, 0.25 * L, C, (True, True, True)))


def test_high_density(nlpkg, orc):
    """test/test_gpu.jl:78-86: 200 atoms in a 5 A box, cutoff 2."""
    X = np.random.default_rng(6).random((200, 3)) * 5.0
    assert_identical(*run_both(nlpkg, orc, X, 2.0, np.diag([5.0] * 3), (True, True, True)))


def test_dense_big_cells(nlpkg, orc):
    """Cells with hundreds / thousands of atoms (the shared-memory and
    ordered-scan fix-up paths of the sort)."""
    X = np.random.default_rng(7).random((3000, 3)) * 4.0
    assert_identical(*run_both(nlpkg, orc, X, 1.1, np.diag([4.0] * 3), (True, True, True)))
    X = np.random.default_rng(8).random((9000, 3)) * 2.0
    assert_identical(*run_both(nlpkg, orc, X, 0.3, np.diag([2.0] * 3), (True, False, True)))


def test_edge_cases(nlpkg, orc):
    C = np.diag([10.0] * 3)
    for X, pbc in (([[5.0, 5.0, 5.0]], (1, 1, 1)), ([[5.0, 5.0, 5.0], [5.0, 5.0, 6.0]], (1, 1, 1)),
                   ([[1.0, 1.0, 1.0], [8.0, 8.0, 8.0]], (0, 0, 0))):
        g, o = run_both(nlpkg, orc, np.array(X), 3.0, C, pbc)
        assert_identical(g, o)
    g = nlpkg.neighbour_list(torch.zeros((0, 3), dtype=torch.float64, device="cuda"), 3.0, C, (1, 1, 1))
    assert nlpkg.npairs(g) == 0 and to_np(g.first).tolist() == [1]
    clist = nlpkg.build_cell_list(torch.zeros((0, 3), dtype=torch.float64, device="cuda"), 3.0, C, (1, 1, 1))
    assert set(to_np(clist.cell_offsets).tolist()) == {1}
    two = nlpkg.neighbour_list(torch.tensor([[5.0, 5.0, 5.0], [5.0, 5.0, 6.0]], dtype=torch.float64).cuda(), 3.0, C,
                               (1, 1, 1))
    assert nlpkg.max_neighbours(two) == 1


def test_kats(nlpkg):
    X, C = cf.fcc_cubic(3.61, (4, 2, 3))
    g = nlpkg.neighbour_list(torch.from_numpy(X).cuda(), 3.5, C, (True, True, True))
    assert all(nlpkg.num_neighbours(g, i) == 12 for i in range(1, nlpkg.nsites(g) + 1))
    X = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.0], [0.0, 10.0, 0.0]])
    g = nlpkg.neighbour_list(torch.from_numpy(X).cuda(), 5.0, np.diag(X.max(0) - X.min(0) + 1), (False,) * 3)
    j, R, S = nlpkg.neighbours(g, 1)
    assert to_np(j).tolist() == [2] and to_np(R).tolist() == [[0.0, 0.0, 2.0]]
    j, R, S = nlpkg.neighbours(g, 3)
    assert len(j) == 0


def test_diamond_multi_image(nlpkg, orc):
    X, C = cf.diamond_primitive()
    g, o = run_both(nlpkg, orc, X, 6.0, C, (True, True, True))
    assert o.npairs == 92
    assert_identical(g, o)


def test_issue6_outside_box(nlpkg, orc):
    for pbc in cf.ALL_PBC:
        X, C, L = cf.rand_config(600, seed=31)
        idx = np.arange(1, 601)
        sh = np.stack([(idx % 3) - 1, ((idx + 1) % 3) - 1, ((idx + 2) % 3) - 1], 1).astype(float)
        Xp = X + sh * L * np.array([1.0 if p else 0.0 for p in pbc])
        assert_identical(*run_both(nlpkg, orc, Xp, 5.0, C, pbc))
    # far outside on open axes (clamped cells, FP64-only "exact" atoms)
    X, C, L = cf.rand_config(500, seed=32)
    X[::7, 2] -= 3 * L
    X[::11, 0] += 2.5 * L
    assert_identical(*run_both(nlpkg, orc, X, 5.0, C, (False, True, False)))


def test_config_10k(nlpkg, orc):
    X, C, _ = cf.rand_config(10000, seed=0)
    g, o = run_both(nlpkg, orc, X, 5.0, C, (True, True, True))
    assert abs(o.npairs - 261800) < 3000
    assert_identical(g, o)


def test_config_fcc_sheared_32k(nlpkg, orc):
    X, C, pbc = cf.fcc_sheared(n=20, seed=0)
    assert_identical(*run_both(nlpkg, orc, X, 5.0, C, pbc))


def test_int64_and_no_R(nlpkg, orc):
    X, C = cf.rand_config_triclinic(700, seed=13)
    g, o = run_both(nlpkg, orc, X, 3.3, C, (True, False, True), int_type=torch.int64)
    assert g.i.dtype == torch.int64 and g.S.dtype == torch.int64
    assert_identical(g, o)
    g2 = nlpkg.neighbour_list(torch.from_numpy(X).cuda(), 3.3, C, (True, False, True), with_R=False)
    assert g2.R is None
    assert_identical(g2, o, with_R=False)


def test_sorted_cell_list_fields(nlpkg, orc):
    X, C, pbc = cf.fcc_sheared(n=6, seed=4)
    for it in (torch.int32, torch.int64):
        g = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), 5.0, C, pbc, int_type=it)
        o = orc.build_cell_list(X, 5.0, C, pbc)
        np.testing.assert_array_equal(to_np(g.perm).astype(np.int64), o.perm)
        np.testing.assert_array_equal(to_np(g.cell_id).astype(np.int64), o.cell_id)
        np.testing.assert_array_equal(to_np(g.cell_offsets).astype(np.int64), o.cell_offsets)
        assert np.array_equal(to_np(g.X).view(np.int64), o.X.view(np.int64))


def test_materialize_foreign_cell_list(nlpkg, orc):
    """A SortedCellList produced elsewhere (here by the oracle, i.e. the
    reference's CPU build) is materialised by the GPU kernels."""
    X, C, L = cf.rand_config(4000, seed=14)
    o = orc.build_cell_list(X, 5.0, C, (True, True, False))
    plan = nlpkg.analyze_cell(C, 5.0)
    dev = "cuda"
    clist = nlpkg.SortedCellList(
        torch.from_numpy(o.X).to(dev), torch.from_numpy(o.X_orig).to(dev),
        torch.from_numpy(o.perm.astype(np.int32)).to(dev), torch.from_numpy(o.cell_id.astype(np.int32)).to(dev),
        torch.from_numpy(o.cell_offsets.astype(np.int32)).to(dev), C, plan.inv_cell, (True, True, False), 5.0,
        plan.ncells, plan.ncells_total, plan, None, False)
    g = nlpkg.materialize_pairlist(clist)
    assert_identical(g, orc.neighbour_list(X, 5.0, C, (True, True, False)))


def test_lazy_reductions(nlpkg, orc):
    X, C, L = cf.rand_config(5000, seed=15)
    Xd = torch.from_numpy(X).cuda()
    clist = nlpkg.neighbour_list(Xd, 5.0, C, (True, True, True), lazy=True)
    assert isinstance(clist, nlpkg.SortedCellList)
    o = orc.neighbour_list(X, 5.0, C, (True, True, True))
    cnt = to_np(nlpkg.lazy_reduce(clist, "count"))
    np.testing.assert_array_equal(cnt, np.diff(o.first))
    s = to_np(nlpkg.lazy_reduce(clist, "inv_r6"))
    ref = orc.lazy_sum_r6(orc.build_cell_list(X, 5.0, C, (True, True, True)))
    # per-atom sums follow the reference's traversal order: bit-identical
    assert np.array_equal(s.view(np.int64), ref.view(np.int64))
    assert nlpkg.count_neighbours(clist, 17) == int(np.diff(o.first)[16])
    js, Rs, Ss = nlpkg.neighbours(clist, 17)
    a, b = o.first[16] - 1, o.first[17] - 1
    np.testing.assert_array_equal(to_np(js).astype(np.int64), o.j[a:b])
    seen = []
    nlpkg.for_each_neighbour(lambda j, R, S: seen.append(j), clist, 17)
    assert seen == o.j[a:b].tolist()


def test_engine_reuse_and_capacity(nlpkg, orc):
    X, C, L = cf.rand_config(20000, seed=16)
    Xd = torch.from_numpy(X).cuda()
    eng = nlpkg.NeighbourListEngine(20000, C, 5.0, (True, True, True), capacity=1000)
    total = eng.run(Xd)  # grows the buffers after NL_ERR_CAPACITY
    o = orc.neighbour_list(X, 5.0, C, (True, True, True), nthreads=8)
    assert total == o.npairs and eng.capacity >= total
    assert_identical(eng.pairlist(Xd), o)
    for _ in range(3):
        eng.launch(Xd)
    eng.sync_status()
    assert_identical(eng.pairlist(Xd), o)
    assert eng.rechecks() >= 0


def test_bad_position_reported(nlpkg):
    X = torch.rand((100, 3), dtype=torch.float64, device="cuda") * 10
    X[5, 1] = float("nan")
    with pytest.raises(nlpkg.NLError) as e:
        nlpkg.neighbour_list(X, 3.0, np.diag([10.0] * 3), (True, True, True))
    assert e.value.status == 6


def test_binning_on_cell_boundaries(nlpkg, orc):
    """Positions exactly on, and one ulp either side of, cell faces; tiny
    negatives; zeros; large windings.  The fast double-float binning must
    fall back to the reference's FP64 binning wherever it cannot decide."""
    L = 30.0
    C = np.diag([L, L, L])
    n = 6  # cells per axis at rc = 5
    faces = np.arange(-2 * n, 3 * n + 1) * (L / n)
    vals = np.concatenate([faces, np.nextafter(faces, -np.inf), np.nextafter(faces, np.inf),
                           [0.0, -0.0, -5e-17 * L, 5e-17 * L, 1e-300, -1e-300]])
    rng = np.random.default_rng(17)
    X = rng.choice(vals, size=(3000, 3))
    for pbc in [(True, True, True), (False, True, False)]:
        g = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), 5.0, C, pbc)
        o = orc.build_cell_list(X, 5.0, C, pbc)
        np.testing.assert_array_equal(to_np(g.perm).astype(np.int64), o.perm)
        np.testing.assert_array_equal(to_np(g.cell_id).astype(np.int64), o.cell_id)
        Xs = X[rng.choice(3000, 400, replace=False)] + rng.normal(0, 0.5, (400, 3))
        assert_identical(*run_both(nlpkg, orc, Xs, 5.0, C, pbc))
    # triclinic cell, points on sheared faces
    C2 = cf.fcc_sheared(n=4)[1]
    F = rng.choice(np.arange(-4, 9) / 4.0, size=(2000, 3))
    X2 = F @ C2
    g = nlpkg.build_cell_list(torch.from_numpy(X2).cuda(), 3.0, C2, (True, True, False))
    o = orc.build_cell_list(X2, 3.0, C2, (True, True, False))
    np.testing.assert_array_equal(to_np(g.cell_id).astype(np.int64), o.cell_id)
    np.testing.assert_array_equal(to_np(g.perm).astype(np.int64), o.perm)


@pytest.mark.parametrize("case", ["10k", "fcc"])
def test_minimal_workspace_screening_write(nlpkg, orc, case):
    """A workspace without room for the pair lists: every cell goes through
    the screening write pass; results are identical."""
    if case == "10k":
        X, C, L = cf.rand_config(10000, seed=0)
        pbc, rc = (True, True, True), 5.0
    else:
        X, C, pbc = cf.fcc_sheared(n=6, seed=2)
        rc = 5.0
    eng = nlpkg.NeighbourListEngine(X.shape[0], C, rc, pbc)
    lib = nlpkg._lib.lib()
    full = int(lib.nl_workspace_bytes(X.shape[0], eng.plan.ncells_total))
    small = int(lib.nl_workspace_min_bytes(X.shape[0], eng.plan.ncells_total))
    assert 0 < small < full
    eng.ws = torch.empty(small, dtype=torch.uint8, device="cuda")
    eng.run(torch.from_numpy(X).cuda())
    o = orc.neighbour_list(X, rc, C, pbc, nthreads=8)
    assert_identical(eng.pairlist(None), o)


@pytest.mark.parametrize("case", ["dense", "fcc", "min_workspace"])
def test_lazy_inv_r6_paths(nlpkg, orc, case):
    """Lazy sum 1/r^6: from the per-atom lists, through the screening pass for
    overflowed cells (dense, with a clump of atoms of more than 192 pairs),
    and with no lists at all (minimal workspace) -- bit-identical to the
    oracle in every case."""
    if case == "dense":
        rng = np.random.default_rng(6)
        X = np.concatenate([rng.random((400, 3)) * 6.0, 3.0 + (rng.random((150, 3)) - 0.5) * 1.2])
        C, pbc, rc = np.diag([6.0] * 3), (True, True, True), 2.2
    else:
        X, C, pbc = cf.fcc_sheared(n=5, seed=4)
        rc = 5.0
    clist = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), rc, C, pbc)
    if case == "min_workspace":
        lib = nlpkg._lib.lib()
        clist._ws = torch.empty(int(lib.nl_workspace_min_bytes(X.shape[0], clist.ncells_total)),
                                dtype=torch.uint8, device="cuda")
        clist._records = False
    s = to_np(nlpkg.lazy_reduce(clist, "inv_r6"))
    ref = orc.lazy_sum_r6(orc.build_cell_list(X, rc, C, pbc))
    assert np.array_equal(s.view(np.int64), ref.view(np.int64))


def test_pair_and_site_iterators(nlpkg, orc):
    """pairs / sites (iterators.jl:12-40) over the device buffers."""
    X, C, L = cf.rand_config(300, seed=41)
    nl = nlpkg.neighbour_list(torch.from_numpy(X).cuda(), 0.3 * L, C, (True, True, True))
    o = orc.neighbour_list(X, 0.3 * L, C, (True, True, True))
    items = list(nlpkg.pairs(nl))
    assert len(items) == o.npairs == len(nlpkg.pairs(nl))
    assert [t[0] for t in items] == o.i.tolist() and [t[1] for t in items] == o.j.tolist()
    assert np.array_equal(np.stack([t[2] for t in items]).view(np.int64), o.R.view(np.int64))
    sites = list(nlpkg.sites(nl))
    assert len(sites) == 300
    for i, j, R in sites[::37]:
        a, b = o.first[i - 1] - 1, o.first[i] - 1
        assert np.array_equal(to_np(j).astype(np.int64), o.j[a:b])
        assert np.array_equal(to_np(R).view(np.int64), o.R[a:b].view(np.int64))


@pytest.mark.parametrize("count_kernel", [1, 2, 3])
def test_both_count_kernels(nlpkg, orc, count_kernel):
    """The warp-per-cell, thread-per-atom and symmetric (neighbour masks)
    count passes give the same bits (open and periodic axes, triclinic, a
    one-cell multi-image system, dense cells that overflow the lists)."""
    Xd_, Cd = cf.diamond_primitive()
    Xf, Cf, pf = cf.fcc_sheared(n=5, seed=9)
    cases = [
        (cf.rand_config(3000, seed=51)[0], np.diag([cf.rand_config(3000, seed=51)[2]] * 3), 5.0, (True, False, True)),
        (Xf, Cf, 5.0, pf),
        (Xd_, Cd, 6.0, (True, True, True)),
        (np.random.default_rng(52).random((400, 3)) * 6.0, np.diag([6.0] * 3), 2.2, (True, True, True)),
        (cf.rand_config_triclinic(200, seed=53)[0], cf.triclinic_cell(), 3.0, (True, True, False)),
    ]
    for X, C, rc, pbc in cases:
        eng = nlpkg.NeighbourListEngine(X.shape[0], C, rc, pbc)
        eng.set_tuning(0, 0, count_kernel)
        eng.run(torch.from_numpy(np.ascontiguousarray(X)).cuda())
        o = orc.neighbour_list(X, rc, C, pbc, nthreads=8)
        assert_identical(eng.pairlist(None), o)


def test_count_pass_edge_cases(nlpkg, orc):
    """Exact atoms far outside an open axis, lists that overflow (> 192
    pairs: those cells go to the screening write pass) next to cells that do
    not, in cells of at most 32 atoms (symmetric pass) and in crowded cells
    (> 32 atoms: the symmetric pass falls back), open
    boundaries, Int64; and the symmetric and per-atom count passes giving
    identical lists on 20k atoms."""
    rng = np.random.default_rng(54)
    X, C, L = cf.rand_config(4000, seed=55)
    Xo = X.copy()
    Xo[:30, 2] += rng.choice([-1, 1], 30) * rng.uniform(2.0, 40.0, 30) * L  # far outside the open z axis
    dense = np.concatenate([X, rng.random((40, 3)) * 0.5 + L / 2])              # one crowded cell
    Xc5, Cc, _ = cf.corner_clump(4000, 5.0, seed=55)
    Xc6 = cf.corner_clump(4000, 6.0, seed=55)[0]
    Xm = cf.corner_clump(4000, 5.0, per_octant=20, seed=57)[0]  # 65..192 pairs decoded from the masks
    clump = np.concatenate([X, L / 3 + (rng.random((250, 3)) - 0.5) * 1.5])  # > 192 pairs, one crowded cell
    cases = [(X, C, 5.0, (True, True, True)), (Xo, C, 5.0, (True, True, False)), (X, C, 6.0, (True, True, True)),
             (dense, C, 5.0, (True, True, True)), (X, C, 5.0, (False, False, False)),
             (Xc5, Cc, 5.0, (True, True, True)), (Xc6, Cc, 6.0, (True, True, False)), (clump, C, 5.0, (True, True, True)),
             (Xm, Cc, 5.0, (True, True, True))]
    for X_, C_, rc, pbc in cases:
        for it in (torch.int32, torch.int64):
            g = nlpkg.neighbour_list(torch.from_numpy(np.ascontiguousarray(X_)).cuda(), rc, C_, pbc, int_type=it)
            o = orc.neighbour_list(X_, rc, C_, pbc, nthreads=8)
            assert_identical(g, o)
    X, C, L = cf.rand_config(20000, seed=56)
    Xd = torch.from_numpy(X).cuda()
    lists = []
    for k in (3, 2):
        eng = nlpkg.NeighbourListEngine(X.shape[0], C, 5.0, (True, True, True))
        eng.set_tuning(0, 0, k)
        eng.run(Xd)
        lists.append(eng.pairlist(Xd))
    for key in ("first", "i", "j", "S"):
        assert torch.equal(getattr(lists[0], key), getattr(lists[1], key))
    assert torch.equal(lists[0].R.view(torch.int64), lists[1].R.view(torch.int64))


def test_system_entry_points(nlpkg, orc):
    """AtomsBase-style systems (ext/NeighbourListsAtomsBaseExt.jl): periodic
    cell with a unit scale, and an isolated cluster whose cell is its
    bounding box diag(max - min + 1) with positions left in place."""
    X, C = cf.fcc_cubic(3.61, (3, 3, 3))
    sysp = nlpkg.System(X / 8.0, C / 8.0, (True, True, True))  # a unit 8x larger; exact rescaling
    nl = nlpkg.neighbour_list_system(sysp, 0.625, length_unit=8.0)
    o = orc.neighbour_list(X, 5.0, C, (True, True, True))
    assert_identical(nl, o)
    rng = np.random.default_rng(61)
    Xc = rng.random((120, 3)) * 12.0 + np.array([40.0, -5.0, 3.0])
    iso = nlpkg.System(Xc, None, (False, False, False))
    Ci = nlpkg.isolated_cell(Xc)
    assert np.array_equal(Ci, np.diag((Xc.max(0) - Xc.min(0)) + 1.0))
    nl = nlpkg.neighbour_list_system(iso, 4.0)
    assert_identical(nl, orc.neighbour_list(Xc, 4.0, Ci, (False, False, False)))
    clist = nlpkg.neighbour_list_system(iso, 4.0, lazy=True)
    assert isinstance(clist, nlpkg.SortedCellList)


def test_engine_launch_host(nlpkg, orc):
    """End to end with pinned host buffers on several copy streams."""
    X, C, L = cf.rand_config(30000, seed=71)
    eng = nlpkg.NeighbourListEngine(X.shape[0], C, 5.0, (True, True, True))
    t = eng.run(torch.from_numpy(X).cuda())
    hX = torch.from_numpy(X).pin_memory()
    out = {"first": torch.empty(X.shape[0] + 1, dtype=torch.int32).pin_memory(),
           "i": torch.empty(t, dtype=torch.int32).pin_memory(), "j": torch.empty(t, dtype=torch.int32).pin_memory(),
           "S": torch.empty((t, 3), dtype=torch.int32).pin_memory(),
           "R": torch.empty((t, 3), dtype=torch.float64).pin_memory()}
    eng.launch_host(hX, out)
    torch.cuda.synchronize()
    eng.sync_status()
    o = orc.neighbour_list(X, 5.0, C, (True, True, True), nthreads=8)
    assert np.array_equal(out["first"].numpy().astype(np.int64), o.first)
    assert np.array_equal(out["j"].numpy().astype(np.int64), o.j)
    assert np.array_equal(out["S"].numpy().astype(np.int64), o.S)
    assert np.array_equal(out["R"].numpy().view(np.int64), o.R.view(np.int64))


def half_of(o):
    """The oracle's full list filtered to a half list: j > i, or j == i and
    S > 0 lexicographically (order kept)."""
    S = o.S
    pos = (S[:, 0] > 0) | ((S[:, 0] == 0) & ((S[:, 1] > 0) | ((S[:, 1] == 0) & (S[:, 2] > 0))))
    keep = (o.j > o.i) | ((o.j == o.i) & pos)
    counts = np.bincount(o.i[keep] - 1, minlength=o.first.shape[0] - 1)
    first = np.concatenate([[1], 1 + np.cumsum(counts)])
    return keep, first


@pytest.mark.parametrize("case", ["10k", "fcc", "diamond", "dense", "triclinic", "crowded"])
@pytest.mark.parametrize("count_kernel", [1, 2, 3])
def test_half_lists(nlpkg, orc, case, count_kernel):
    """nl_neighbour_list_half == the full list filtered to j > i (or the
    periodic images of an atom itself with S > 0), in the reference's order;
    the per-cell, per-atom and symmetric count passes (the last keeps one
    direction of each pair in the masks); dense cells take the screening
    write pass."""
    if case == "10k":
        X, C, L = cf.rand_config(10000, seed=0)
        rc, pbc = 5.0, (True, True, True)
    elif case == "fcc":
        X, C, pbc = cf.fcc_sheared(n=5, seed=3)
        rc = 5.0
    elif case == "diamond":
        X, C = cf.diamond_primitive()
        rc, pbc = 6.0, (True, True, True)
    elif case == "dense":
        X, C, pbc, rc = np.random.default_rng(81).random((400, 3)) * 6.0, np.diag([6.0] * 3), (True, True, True), 2.2
    elif case == "triclinic":
        X, C = cf.rand_config_triclinic(300, seed=82)
        rc, pbc = 3.0, (True, False, True)
    else:  # > 192 pairs for some atoms, cells of <= 32 atoms: masks plus the screening write pass
        X, C, L = cf.corner_clump(4000, 6.0, seed=55)
        rc, pbc = 6.0, (True, True, False)
    eng = nlpkg.NeighbourListEngine(X.shape[0], C, rc, pbc, half=True)
    eng.set_tuning(0, 0, count_kernel)
    t = eng.run(torch.from_numpy(np.ascontiguousarray(X)).cuda())
    o = orc.neighbour_list(X, rc, C, pbc, nthreads=8)
    keep, first = half_of(o)
    assert t == int(keep.sum())
    assert np.array_equal(eng.first.cpu().numpy().astype(np.int64), first)
    assert np.array_equal(eng.i[:t].cpu().numpy().astype(np.int64), o.i[keep])
    assert np.array_equal(eng.j[:t].cpu().numpy().astype(np.int64), o.j[keep])
    assert np.array_equal(eng.S[:t].cpu().numpy().astype(np.int64), o.S[keep])
    assert np.array_equal(eng.R[:t].cpu().numpy().view(np.int64), o.R[keep].view(np.int64))


def test_pair_vectors_and_lists_without_R(nlpkg, orc):
    """R of a list built without R comes from nl_pair_vectors, bit-equal."""
    X, C, L = cf.rand_config(4000, seed=91)
    nl = nlpkg.neighbour_list(torch.from_numpy(X).cuda(), 5.0, C, (True, False, True), with_R=False)
    o = orc.neighbour_list(X, 5.0, C, (True, False, True))
    for i in (1, 17, 4000):
        j, R, S = nlpkg.neigss(nl, i)
        a, b = o.first[i - 1] - 1, o.first[i] - 1
        assert np.array_equal(to_np(R).view(np.int64), o.R[a:b].view(np.int64))
    R = nlpkg.pair_vectors(nl.X, C, nl.i, nl.j, nl.S)
    assert np.array_equal(to_np(R).view(np.int64), o.R.view(np.int64))


def test_verlet_reuse(nlpkg, orc):
    """Lists built at cutoff + skin are reused while atoms move less than
    skin / 2: R is recomputed for the new positions (bit-equal to the
    reference formula) and every pair within the cutoff is in the list."""
    X0, C, L = cf.rand_config(6000, seed=92)
    rc, skin, pbc = 5.0, 1.0, (True, True, True)
    v = nlpkg.VerletList(X0.shape[0], C, rc, skin, pbc)
    rng = np.random.default_rng(93)
    X = X0.copy()
    for step in range(4):
        Xd = torch.from_numpy(X).cuda()
        rebuilt = v.update(Xd)
        assert rebuilt == (step in (0, 3))
        P = v.engine.total_pairs()
        i, j, S = (t[:P].cpu().numpy().astype(np.int64) for t in (v.engine.i, v.engine.j, v.engine.S))
        R = v.engine.R[:P].cpu().numpy()
        Sf = S.astype(np.float64)
        cs = (Sf[:, 0:1] * C[0] + Sf[:, 1:2] * C[1]) + Sf[:, 2:3] * C[2]  # C'S, left fold, no FMA
        ref = (X[j - 1] - X[i - 1]) + cs  # _getR (cell_list.jl:525-531)
        assert np.array_equal(R.view(np.int64), ref.view(np.int64))
        o = orc.neighbour_list(X, rc, C, pbc)
        inside = np.einsum("ij,ij->i", R, R) < rc * rc
        got = set(zip(i[inside].tolist(), j[inside].tolist(), map(tuple, S[inside].tolist())))
        want = set(zip(o.i.tolist(), o.j.tolist(), map(tuple, o.S.tolist())))
        assert got == want
        X = X + rng.uniform(-0.12, 0.12, size=X.shape) * (1.0 if step < 2 else 4.0)


def test_verlet_displacement_on_a_side_stream(nlpkg):
    """The displacement test launched on a non-current stream is read back on
    that stream: it sees the new positions, not a stale value."""
    X0, C, L = cf.rand_config(20000, seed=94)
    v = nlpkg.VerletList(X0.shape[0], C, 4.0, 1.0, (True, True, True))
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        Xd0 = torch.from_numpy(X0).cuda()
    side.synchronize()
    v.update(Xd0, stream=side)
    X1 = X0.copy()
    X1[123] += 0.3  # one atom moves by 0.3 * sqrt(3)
    with torch.cuda.stream(side):
        Xd1 = torch.from_numpy(X1).cuda()
    d = v.max_displacement(Xd1, stream=side)  # launched on side, the current stream is the default one
    assert abs(d - 0.3 * np.sqrt(3.0)) < 1e-12


def test_half_int64_and_verlet_half(nlpkg, orc):
    """Half lists in Int64, and Verlet reuse of a half list."""
    X, C, L = cf.rand_config(5000, seed=101)
    pbc = (True, True, False)
    eng = nlpkg.NeighbourListEngine(X.shape[0], C, 5.0, pbc, int_type=torch.int64, half=True)
    t = eng.run(torch.from_numpy(X).cuda())
    o = orc.neighbour_list(X, 5.0, C, pbc, ti_bytes=8, nthreads=8)
    keep, first = half_of(o)
    assert t == int(keep.sum()) and eng.i.dtype == torch.int64
    assert np.array_equal(eng.j[:t].cpu().numpy(), o.j[keep])
    assert np.array_equal(eng.R[:t].cpu().numpy().view(np.int64), o.R[keep].view(np.int64))
    v = nlpkg.VerletList(X.shape[0], C, 4.0, 1.0, pbc, half=True)
    v.update(torch.from_numpy(X).cuda())
    X2 = X + np.random.default_rng(102).uniform(-0.1, 0.1, size=X.shape)
    assert not v.update(torch.from_numpy(X2).cuda())
    P = v.engine.total_pairs()
    i, j, S = (t_[:P].cpu().numpy().astype(np.int64) for t_ in (v.engine.i, v.engine.j, v.engine.S))
    R = v.engine.R[:P].cpu().numpy()
    inside = np.einsum("ij,ij->i", R, R) < 16.0
    o2 = orc.neighbour_list(X2, 4.0, C, pbc)
    keep2, _ = half_of(o2)
    got = set(zip(i[inside].tolist(), j[inside].tolist(), map(tuple, S[inside].tolist())))
    want = set(zip(o2.i[keep2].tolist(), o2.j[keep2].tolist(), map(tuple, o2.S[keep2].tolist())))
    assert got == want


def test_fill_follows_the_count_choice(nlpkg, orc):
    """The write pass follows the count pass recorded in the workspace, even
    when the calling thread's tuning changed in between (symmetric count then
    list-mode tuning, and the reverse)."""
    import ctypes as C

    from neighbourlists_gb300 import _lib
    from neighbourlists_gb300.api import _plan_args, _pbc, _ptr, _stream_handle

    X, Cm, L = cf.rand_config(6000, seed=91)
    o = orc.neighbour_list(X, 5.0, Cm, (True, True, True), nthreads=8)
    L_ = nlpkg.lib()
    for before, after in ((3, 1), (1, 3), (2, 0)):
        clist = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), 5.0, Cm, (True, True, True))
        nat = X.shape[0]
        first = torch.empty(nat + 1, dtype=torch.int32, device="cuda")
        total = C.c_int64(0)
        cm, im, nc, nx = _plan_args(clist)
        pb = _pbc(clist.pbc)
        sh = _stream_handle(None)
        _lib.check(L_.nl_set_tuning(C.byref(_lib.Tuning(0, 0, before))))
        _lib.check(L_.nl_count_pairs(_ptr(clist.X), _ptr(clist.perm), _ptr(clist.cell_id),
                                     C.c_void_p(clist.cell_offsets.data_ptr()), nat, cm, im, nc, nx,
                                     pb.ctypes.data_as(C.POINTER(C.c_uint8)), 5.0, 4, 1,
                                     C.c_void_p(first.data_ptr()), C.byref(total), _ptr(clist._ws), clist._ws.numel(), sh))
        P = int(total.value)
        i = torch.empty(P, dtype=torch.int32, device="cuda")
        j = torch.empty_like(i)
        S = torch.empty((P, 3), dtype=torch.int32, device="cuda")
        R = torch.empty((P, 3), dtype=torch.float64, device="cuda")
        _lib.check(L_.nl_set_tuning(C.byref(_lib.Tuning(0, 0, after))))
        _lib.check(L_.nl_fill_pairs(_ptr(clist.X), _ptr(clist.perm), C.c_void_p(clist.cell_offsets.data_ptr()), nat,
                                    cm, im, nc, nx, pb.ctypes.data_as(C.POINTER(C.c_uint8)), 5.0, 4,
                                    C.c_void_p(first.data_ptr()), P, _ptr(i), _ptr(j), _ptr(S), _ptr(R), _ptr(clist._ws),
                                    clist._ws.numel(), sh))
        _lib.check(L_.nl_sync_status(_ptr(clist._ws), sh))
        _lib.check(L_.nl_set_tuning(None))
        assert P == o.npairs
        np.testing.assert_array_equal(to_np(j).astype(np.int64), o.j)
        np.testing.assert_array_equal(to_np(S).astype(np.int64), o.S)
        assert np.array_equal(to_np(R).view(np.int64), o.R.view(np.int64))


@pytest.mark.parametrize("int_type", [torch.int32, torch.int64])
def test_unaligned_output_arrays(nlpkg, orc, int_type):
    """Pair arrays that do not start on 16-byte boundaries (views one element
    into larger buffers) take the write pass's word-by-word stores: same
    bits as the oracle, nothing written outside the views."""
    import ctypes as C
    X, Cm, L = cf.rand_config(20000, seed=95)
    pbc = (True, True, True)
    plan = nlpkg.analyze_cell(Cm, 5.0, int_type)
    nat = X.shape[0]
    dev = torch.device("cuda")
    ib = 4 if int_type == torch.int32 else 8
    o = orc.neighbour_list(X, 5.0, Cm, pbc, ti_bytes=ib, nthreads=8)
    P = o.npairs
    bufs = {k: torch.zeros((P + 8) * w, dtype=dt, device=dev) for k, w, dt in
            (("i", 1, int_type), ("j", 1, int_type), ("S", 3, int_type), ("R", 3, torch.float64))}
    views = {"i": bufs["i"][1:P + 1], "j": bufs["j"][1:P + 1], "S": bufs["S"][3:3 * P + 3],
             "R": bufs["R"][3:3 * P + 3]}
    ws = torch.empty(int(nlpkg.lib().nl_workspace_bytes(nat, plan.ncells_total)), dtype=torch.uint8, device=dev)
    perm, cid = torch.empty(nat, dtype=int_type, device=dev), torch.empty(nat, dtype=int_type, device=dev)
    Xs = torch.empty((nat, 3), dtype=torch.float64, device=dev)
    offs = torch.empty(plan.ncells_total + 1, dtype=int_type, device=dev)
    first = torch.empty(nat + 1, dtype=int_type, device=dev)
    pb = np.ones(3, dtype=np.uint8)
    total = C.c_int64(-1)
    D, I64, U8 = C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_uint8)
    Xd = torch.from_numpy(X).cuda()
    torch.cuda.synchronize()

    def p(t):
        return C.c_void_p(t.data_ptr())

    st = nlpkg.lib().nl_neighbour_list(p(Xd), nat, plan.cell_cm.ctypes.data_as(D), plan.inv_cm.ctypes.data_as(D),
                                       plan.ncells.ctypes.data_as(I64), plan.nxyz.ctypes.data_as(I64),
                                       pb.ctypes.data_as(U8), 5.0, ib, p(perm), p(Xs), p(cid), p(offs), p(first), P,
                                       p(views["i"]), p(views["j"]), p(views["S"]), p(views["R"]), C.byref(total),
                                       p(ws), ws.numel(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0 and total.value == P
    assert np.array_equal(views["i"].cpu().numpy().astype(np.int64), o.i)
    assert np.array_equal(views["j"].cpu().numpy().astype(np.int64), o.j)
    assert np.array_equal(views["S"].cpu().numpy().reshape(-1, 3).astype(np.int64), o.S)
    assert np.array_equal(views["R"].cpu().numpy().reshape(-1, 3).view(np.int64), o.R.view(np.int64))
    for k, w in (("i", 1), ("j", 1), ("S", 3), ("R", 3)):  # nothing written outside the views
        assert torch.all(bufs[k][:w] == 0) and torch.all(bufs[k][w * (P + 1):] == 0), k
