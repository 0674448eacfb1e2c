"""Pins the CPU oracle against the reference's own known answers and
cross-checks (CPU only).

Sources of the expectations (paths inside the reference project):
  * FCC Cu has 12 neighbours at 3.5 A and 2.6 A, more at 3.7 A, none at 1.0 A
    (test/test_atoms_base.jl:150-171, 243-257);
  * isolated H3: R = (0,0,+-2) (test/test_atoms_base.jl:208-241);
  * two-atom / single-atom edge cases and max_neighbours
    (test/test_utils.jl:480-494, test/test_unified_api.jl:296-312, 393-404);
  * legacy linked-list == sort-based (i,j,S) sets on the reference's test
    configurations (test/test_sortbased.jl:17-71, test/test_utils.jl:319-349);
  * lazy traversal == materialised list (test/test_sortbased.jl:74-115);
  * issue #6: atoms outside [0,L) (test/test_sortbased.jl:143-228);
  * brute force over periodic images (test/nn_list.jl, test/test_celllist.jl).
"""
import numpy as np
import pytest

import configs as cf


def sets_equal(a, b, orc):
    ca = orc.canonical(a.i, a.j, a.S)
    cb = orc.canonical(b.i, b.j, b.S)
    return all(np.array_equal(x, y) for x, y in zip(ca, cb))


def brute_force(X, cell, pbc, rc, kmax=3):
    """All (i, j, S) with |X[j] - X[i] + cell'S| < rc, S in [-kmax,kmax]^3 on
    periodic axes, excluding (i, i, 0)."""
    X = np.asarray(X)
    rng = [range(-kmax, kmax + 1) if p else range(0, 1) for p in pbc]
    out = []
    for s0 in rng[0]:
        for s1 in rng[1]:
            for s2 in rng[2]:
                S = np.array([s0, s1, s2])
                sh = S @ cell
                D = X[None, :, :] - X[:, None, :] + sh
                d2 = (D * D).sum(-1)
                ii, jj = np.nonzero(d2 < rc * rc)
                for a, b in zip(ii, jj):
                    if a == b and not S.any():
                        continue
                    out.append((a + 1, b + 1, s0, s1, s2))
    return sorted(out)


def as_tuples(nl):
    return sorted(zip(nl.i.tolist(), nl.j.tolist(), *[nl.S[:, k].tolist() for k in range(3)]))


# ----------------------------------------------------------------- KATs --
@pytest.mark.parametrize("reps,rc,expect", [((4, 2, 3), 3.5, 12), ((3, 3, 3), 3.5, 12), ((2, 2, 2), 3.5, 12),
                                            ((3, 3, 3), 2.6, 12)])
def test_fcc_cu_coordination(orc, reps, rc, expect):
    X, C = cf.fcc_cubic(3.61, reps)
    nl = orc.neighbour_list(X, rc, C, (True, True, True))
    assert np.all(np.diff(nl.first) == expect)
    lg = orc.legacy_pairlist(X, rc, C, (True, True, True))
    assert np.all(np.diff(lg.first) == expect)


def test_fcc_cu_cutoffs(orc):
    X, C = cf.fcc_cubic(3.61, (3, 3, 3))
    assert np.diff(orc.neighbour_list(X, 3.7, C, (1, 1, 1)).first)[0] > 12
    assert orc.neighbour_list(X, 1.0, C, (1, 1, 1)).npairs == 0


def test_isolated_h3(orc):
    X = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.0], [0.0, 10.0, 0.0]])
    C = np.diag(X.max(0) - X.min(0) + 1)  # bounding box, ext/NeighbourListsAtomsBaseExt.jl:17-31
    nl = orc.neighbour_list(X, 5.0, C, (False, False, False))
    assert nl.npairs == 2
    assert list(np.diff(nl.first)) == [1, 1, 0]
    assert nl.j.tolist() == [2, 1]
    assert nl.R.tolist() == [[0.0, 0.0, 2.0], [0.0, 0.0, -2.0]]


def test_edge_cases(orc):
    C = np.diag([10.0] * 3)
    assert orc.neighbour_list([[5.0, 5.0, 5.0]], 3.0, C, (1, 1, 1)).npairs == 0
    nl = orc.neighbour_list([[5.0, 5.0, 5.0], [5.0, 5.0, 6.0]], 3.0, C, (1, 1, 1))
    assert nl.npairs == 2 and np.max(np.diff(nl.first)) == 1
    assert orc.neighbour_list([[1.0, 1.0, 1.0], [8.0, 8.0, 8.0]], 3.0, C, (0, 0, 0)).npairs == 0
    empty = orc.neighbour_list(np.zeros((0, 3)), 3.0, C, (1, 1, 1))
    assert empty.npairs == 0 and empty.first.tolist() == [1]


def test_diamond_multi_image(orc):
    """cutoff 6.0 > cell height 3.135: nxyz = 2, 125 stencil cells; shells
    4/12/12/6/12 per atom at 2.351/3.840/4.502/5.430/5.917 A (crystallography)."""
    X, C = cf.diamond_primitive()
    info = orc.analyze_cell(C, 6.0)
    assert info.nxyz.tolist() == [2, 2, 2] and info.ncells.tolist() == [1, 1, 1]
    nl = orc.neighbour_list(X, 6.0, C, (1, 1, 1))
    assert nl.npairs == 92 and list(np.diff(nl.first)) == [46, 46]
    r = np.round(np.linalg.norm(nl.R, axis=1), 3)
    shells, counts = np.unique(r, return_counts=True)
    assert shells.tolist() == [2.351, 3.84, 4.502, 5.43, 5.917]
    assert counts.tolist() == [8, 24, 24, 12, 24]
    assert sets_equal(nl, orc.legacy_pairlist(X, 6.0, C, (1, 1, 1)), orc)


# ------------------------------------------------- legacy == sort-based --
@pytest.mark.parametrize("seed", range(5))
def test_legacy_vs_sortbased_random(orc, seed):
    N = 50 + 37 * seed
    X, C, L = cf.rand_config(N, seed=seed)
    a = orc.neighbour_list(X, L / 4, C, (1, 1, 1))
    b = orc.legacy_pairlist(X, L / 4, C, (1, 1, 1))
    assert a.npairs == b.npairs and sets_equal(a, b, orc)


@pytest.mark.parametrize("pbc", cf.ALL_PBC)
def test_legacy_vs_sortbased_all_pbc(orc, pbc):
    X, C, L = cf.rand_config(50, seed=7)
    a = orc.neighbour_list(X, 0.33 * L, C, pbc)
    b = orc.legacy_pairlist(X, 0.33 * L, C, pbc)
    assert sets_equal(a, b, orc)


def test_legacy_vs_sortbased_triclinic_elongated_large_cutoff(orc):
    X, C = cf.rand_config_triclinic(80, seed=3)
    assert sets_equal(orc.neighbour_list(X, 3.0, C, (1, 1, 1)), orc.legacy_pairlist(X, 3.0, C, (1, 1, 1)), orc)
    C2 = np.diag([5.0, 5.0, 20.0])
    X2 = np.random.default_rng(4).random((80, 3)) @ C2
    assert sets_equal(orc.neighbour_list(X2, 3.0, C2, (1, 1, 1)), orc.legacy_pairlist(X2, 3.0, C2, (1, 1, 1)), orc)
    X3, C3, L3 = cf.rand_config(30, seed=5)
    assert sets_equal(orc.neighbour_list(X3, 0.6 * L3, C3, (1, 1, 1)),
                      orc.legacy_pairlist(X3, 0.6 * L3, C3, (1, 1, 1)), orc)


@pytest.mark.parametrize("N", [500, 1000, 2000])
def test_legacy_vs_sortbased_sizes(orc, N):
    X, C, L = cf.rand_config(N, seed=N)
    a = orc.neighbour_list(X, 0.25 * L, C, (1, 1, 1))
    b = orc.legacy_pairlist(X, 0.25 * L, C, (1, 1, 1))
    assert a.npairs == b.npairs and sets_equal(a, b, orc)


@pytest.mark.parametrize("pbc", [(1, 1, 1), (0, 0, 0), (1, 0, 1)])
def test_brute_force(orc, pbc):
    X, C = cf.rand_config_triclinic(60, seed=11)
    nl = orc.neighbour_list(X, 4.0, C, pbc)
    assert as_tuples(nl) == brute_force(X, C, pbc, 4.0)


# ------------------------------------------------------- lazy traversal --
def test_lazy_matches_materialised(orc):
    X, C, L = cf.rand_config(100, seed=2)
    clist = orc.build_cell_list(X, L / 3, C, (1, 1, 1))
    nl = orc.neighbour_list(X, L / 3, C, (1, 1, 1))
    counts = orc.count_neighbours(clist)
    assert counts.sum() == nl.npairs
    assert np.array_equal(counts, np.diff(nl.first))
    for i in (1, 17, 100):
        js, Rs, Ss = orc.neighbours(clist, i)
        a, b = nl.first[i - 1] - 1, nl.first[i] - 1
        assert np.array_equal(js, nl.j[a:b]) and np.array_equal(Ss, nl.S[a:b])
        assert np.array_equal(Rs.view(np.int64), nl.R[a:b].view(np.int64))


def test_lazy_r6_sums(orc):
    X, C, L = cf.rand_config(300, seed=9)
    clist = orc.build_cell_list(X, 5.0, C, (1, 1, 1))
    nl = orc.neighbour_list(X, 5.0, C, (1, 1, 1))
    s = orc.lazy_sum_r6(clist)
    r2 = (nl.R * nl.R).sum(1)
    ref = np.zeros(300)
    np.add.at(ref, nl.i - 1, 1.0 / r2 ** 3)
    np.testing.assert_allclose(s, ref, rtol=1e-12)


# ------------------------------------------------------------ issue #6 --
def _pair_multiset(orc, X, rc, C, pbc):
    nl = orc.neighbour_list(X, rc, C, pbc)
    d = np.round(np.sqrt((nl.R ** 2).sum(1)), 10)
    return sorted(zip(np.minimum(nl.i, nl.j).tolist(), np.maximum(nl.i, nl.j).tolist(), d.tolist()))


def test_issue6_two_atoms(orc):
    C = np.diag([8.0] * 3)
    ref = _pair_multiset(orc, [[0.5, 0.5, 0.5], [0.5, 1.5, 0.5]], 1.5, C, (1, 1, 1))
    assert len(ref) == 2
    assert _pair_multiset(orc, [[0.5, 0.5, 0.5], [0.5, -0.5, 0.5]], 1.5, C, (1, 1, 1)) == ref
    assert _pair_multiset(orc, [[0.5, 0.5, 0.5], [0.5, -6.5, 0.5]], 1.5, C, (1, 1, 1)) == ref


@pytest.mark.parametrize("pbc", cf.ALL_PBC)
def test_issue6_shift_by_L_is_noop(orc, pbc):
    X, C, L = cf.rand_config(60, seed=21)
    rc = 0.25 * L
    ref = _pair_multiset(orc, X, rc, C, pbc)
    idx = np.arange(1, 61)
    shifts = np.stack([(idx % 3) - 1, ((idx + 1) % 3) - 1, ((idx + 2) % 3) - 1], 1).astype(float)
    Xp = X + shifts * L * np.array([1.0 if p else 0.0 for p in pbc])
    assert _pair_multiset(orc, Xp, rc, C, pbc) == ref


def test_issue6_fp_boundary(orc):
    L = 8.0
    tiny = -5e-17 * L
    assert (tiny / L) - np.floor(tiny / L) == 1.0
    X = np.array([[0.5, L - 0.3, 0.5], [0.5, tiny, 0.5]])
    C = np.diag([L] * 3)
    clist = orc.build_cell_list(X, 1.5, C, (1, 1, 1))
    js, Rs, Ss = orc.neighbours(clist, 1)
    k = list(js).index(2)
    assert abs(np.sqrt((Rs[k] ** 2).sum()) - 0.3) < 1e-9
    np.testing.assert_allclose(X[1] - X[0] + C.T @ Ss[k], Rs[k], atol=1e-12)


# ------------------------------------------------------- golden fixtures --
def test_golden_fixtures(orc):
    """The oracle reproduces the committed fixtures bit for bit (this also
    checks that gcc on another ISA compiled it without FP contraction)."""
    import golden_io

    for case in golden_io.load_all():
        out = orc.neighbour_list(case["X"], case["cutoff"], case["cell"], case["pbc"])
        assert out.npairs == case["i"].shape[0], case["name"]
        for key in ("i", "j", "S", "first"):
            assert np.array_equal(getattr(out, key), case[key]), (case["name"], key)
        assert np.array_equal(out.R.view(np.int64), case["R"].view(np.int64)), case["name"]
    for dig in golden_io.load_digests():
        X, C, pbc, rc = golden_io.digest_input(dig)
        out = orc.neighbour_list(X, rc, C, pbc, nthreads=4)
        assert golden_io.digest(out) == dig["sha256"], dig["name"]


# ------------------------------------------------------------ T = Float32 --
def test_f32_known_answers(orc):
    """The known answers of the reference's tests hold for the Float32
    restatement: FCC Cu coordination 12, diamond primitive cell 92 pairs
    (46 per atom) with rc larger than the cell, isolated H3."""
    X, C = cf.fcc_cubic(3.61, (3, 3, 3))
    assert np.all(np.diff(orc.neighbour_list_f32(X, 3.5, C, (1, 1, 1)).first) == 12)
    assert orc.neighbour_list_f32(X, 1.0, C, (1, 1, 1)).npairs == 0
    X, C = cf.diamond_primitive()
    nl = orc.neighbour_list_f32(X, 6.0, C, (1, 1, 1))
    assert nl.npairs == 92 and list(np.diff(nl.first)) == [46, 46]
    X = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.0], [0.0, 10.0, 0.0]])
    nl = orc.neighbour_list_f32(X, 5.0, np.diag(X.max(0) - X.min(0) + 1), (0, 0, 0))
    assert nl.j.tolist() == [2, 1] and nl.R.tolist() == [[0.0, 0.0, 2.0], [0.0, 0.0, -2.0]]


@pytest.mark.parametrize("pbc", cf.ALL_PBC)
def test_f32_equals_f64_sets(orc, pbc):
    """Away from the cutoff, the Float32 and Float64 lists hold the same
    (i, j, S) for the same (Float32-representable) positions."""
    X, C, L = cf.rand_config(400, seed=71)
    X = X.astype(np.float32).astype(np.float64)
    a = orc.neighbour_list_f32(X, 0.3 * L, C, pbc)
    b = orc.neighbour_list(X, 0.3 * L, C, pbc)
    r = np.linalg.norm(b.R, axis=1)
    near = np.abs(r - 0.3 * L) < 1e-4 * L
    key = lambda nl, m: set(zip(nl.i[m].tolist(), nl.j[m].tolist(), *[nl.S[m, k].tolist() for k in range(3)]))
    ra = np.linalg.norm(a.R.astype(np.float64), axis=1)
    assert key(a, np.abs(ra - 0.3 * L) >= 1e-4 * L) == key(b, ~near)
    # the sorted cell lists agree too (binning away from cell faces)
    assert np.array_equal(a.cell_offsets, orc.build_cell_list(X, 0.3 * L, C, pbc).cell_offsets)


@pytest.mark.parametrize("rc,per_octant,pbc,lo,hi", [
    (5.0, 28, (True, True, True), 193, 10**9),    # lists overflow the 192-entry capacity
    (6.0, 28, (True, True, False), 193, 10**9),
    (5.0, 20, (True, True, True), 65, 192),       # more than 64 pairs, decoded from the masks
])
def test_corner_clump_generator(orc, rc, per_octant, pbc, lo, hi):
    """The GPU overflow cases rest on these properties of the corner-clump
    generator: its clump atoms have lo..hi pairs and no cell holds more than
    32 atoms (so the symmetric count pass still applies)."""
    X, C, L = cf.corner_clump(4000, rc, per_octant=per_octant, seed=55 if per_octant == 28 else 57)
    o = orc.neighbour_list(X, rc, C, pbc, nthreads=8)
    cl = orc.build_cell_list(X, rc, C, pbc)
    npair = np.diff(o.first)
    assert np.diff(cl.cell_offsets).max() <= 32
    clump = npair[-8 * per_octant:]
    assert clump.min() >= lo and clump.max() <= hi
    assert npair[:-8 * per_octant].max() < lo  # the background stays below
