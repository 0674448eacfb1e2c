"""GPU parity of the legacy linked-list PairList (cell_list.jl:11-20, 185-505)
against the oracle's restatement of it: the fixed positions and cell of
_fix_cell_, and i, j, S, first of _pairlist_ + sort_neigs!, identical array
for array.  Cases follow the reference's legacy comparisons
(test/test_sortbased.jl, test/test_utils.jl) plus the situations the legacy
code handles differently: atoms outside the cell on periodic and open axes
(wrap, shift, enlarged cell), multi-image stencils whose sort has ties in j,
neighbour lists longer than the in-shared-memory sort, and cutoff-boundary
pairs decided by the FP64 recheck."""
import numpy as np
import pytest
import torch

import configs as cf

pytestmark = pytest.mark.gpu


def to_np(t):
    return t.detach().cpu().numpy()


def run_both(nlpkg, orc, X, rc, cell, pbc, int_type=torch.int32, fixcell=True, with_R=False):
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)).cuda()
    g = nlpkg.legacy_pairlist(Xd, rc, cell, pbc, int_type=int_type, fixcell=fixcell, with_R=with_R)
    o = orc.legacy_pairlist(X, rc, cell, pbc, ti_bytes=4 if int_type == torch.int32 else 8, fixcell=fixcell)
    return g, o


def assert_identical(g, o, with_R=False):
    assert int(g.i.shape[0]) == o.npairs
    assert np.array_equal(to_np(g.X).view(np.int64), o.X.view(np.int64)), "fixed positions differ"
    assert np.array_equal(np.asarray(g.C).view(np.int64), o.cell.view(np.int64)), "fixed cell differs"
    np.testing.assert_array_equal(to_np(g.first).astype(np.int64), o.first)
    np.testing.assert_array_equal(to_np(g.i).astype(np.int64), o.i)
    np.testing.assert_array_equal(to_np(g.j).astype(np.int64), o.j)
    np.testing.assert_array_equal(to_np(g.S).astype(np.int64), o.S)
    if with_R:
        assert np.array_equal(to_np(g.R).view(np.int64), o.R.view(np.int64)), "R bits differ"


@pytest.mark.parametrize("seed", range(4))
def test_random_configs(nlpkg, orc, seed):
    N = 50 + 37 * seed
    X, C, L = cf.rand_config(N, seed=300 + seed)
    assert_identical(*run_both(nlpkg, orc, X, 0.33 * L, C, (True, True, True)))


@pytest.mark.parametrize("pbc", cf.ALL_PBC)
def test_all_pbc(nlpkg, orc, pbc):
    X, C, L = cf.rand_config(50, seed=17)
    assert_identical(*run_both(nlpkg, orc, X, 0.33 * L, C, pbc))
    X, C, L = cf.rand_config(3000, seed=18)
    assert_identical(*run_both(nlpkg, orc, X, 5.0, C, pbc), with_R=False)


def test_triclinic_and_elongated(nlpkg, orc):
    X, C = cf.rand_config_triclinic(80, seed=13)
    assert_identical(*run_both(nlpkg, orc, X, 3.0, C, (True, True, True), with_R=True), with_R=True)
    C2 = np.diag([5.0, 5.0, 20.0])
    X2 = np.random.default_rng(14).random((80, 3)) @ C2
    assert_identical(*run_both(nlpkg, orc, X2, 3.0, C2, (True, True, True)))


def test_multi_image_ties(nlpkg, orc):
    """cutoff larger than the cell: the same j appears under several shifts,
    and sort_neigs!'s stable sort keeps those in traversal order."""
    X, C = cf.diamond_primitive()
    g, o = run_both(nlpkg, orc, X, 6.0, C, (True, True, True), with_R=True)
    assert o.npairs == 92
    assert_identical(g, o, with_R=True)
    X3, C3, L3 = cf.rand_config(30, seed=15)
    assert_identical(*run_both(nlpkg, orc, X3, 0.6 * L3, C3, (True, True, True)))
    X4, C4 = cf.rand_config_triclinic(7, seed=16)
    assert_identical(*run_both(nlpkg, orc, X4, 9.0, C4, (True, False, True)))


def test_fcc_coordination(nlpkg, orc):
    X, C = cf.fcc_cubic(3.61, (3, 3, 3))
    g, o = run_both(nlpkg, orc, X, 3.5, C, (True, True, True))
    assert np.all(np.diff(to_np(g.first)) == 12)
    assert_identical(g, o)


def test_atoms_outside_periodic_axes_are_wrapped(nlpkg, orc):
    X, C, L = cf.rand_config(400, seed=21)
    rng = np.random.default_rng(22)
    X = X + rng.integers(-3, 4, size=X.shape) * L  # whole periods away
    X[:5, 0] = -1e-17                               # mod(-tiny, 1) rounds to 1.0
    X[5:10, 1] = L * (1 - 1e-16)
    for pbc in [(True, True, True), (True, True, False), (False, True, True)]:
        assert_identical(*run_both(nlpkg, orc, X, 0.2 * L, C, pbc, with_R=True), with_R=True)


def test_open_axes_shift_and_enlarge(nlpkg, orc):
    X, C = cf.rand_config_triclinic(300, seed=23)
    Xo = X.copy()
    Xo[:40] -= np.array([0.0, 0.0, 6.0])   # below the cell along z
    Xo[40:60] += np.array([11.0, 0.0, 0.0])  # beyond it along x
    for pbc in [(True, True, False), (False, True, False), (False, False, False)]:
        g, o = run_both(nlpkg, orc, Xo, 3.0, C, pbc, with_R=True)
        assert_identical(g, o, with_R=True)


def test_without_fixcell(nlpkg, orc):
    X, C, L = cf.rand_config(500, seed=24)
    X = X + np.random.default_rng(25).normal(0, 0.3 * L, X.shape)  # many atoms outside
    for pbc in [(True, True, True), (True, False, True), (False, False, False)]:
        assert_identical(*run_both(nlpkg, orc, X, 0.2 * L, C, pbc, fixcell=False))


def test_int64(nlpkg, orc):
    X, C, L = cf.rand_config(800, seed=26)
    g, o = run_both(nlpkg, orc, X, 0.25 * L, C, (True, False, True), int_type=torch.int64)
    assert g.i.dtype == torch.int64 and g.S.dtype == torch.int64
    assert_identical(g, o)


def test_long_neighbour_lists(nlpkg, orc):
    """more than 256 pairs per atom: the two-traversal sort (here with two
    cells per axis, so every neighbouring bin is visited twice and the lists
    hold ties in j)."""
    X, C, L = cf.rand_config(1500, density=0.2, seed=27)
    g, o = run_both(nlpkg, orc, X, 6.6, C, (True, True, True))
    assert np.max(np.diff(o.first)) > 256 and np.min(np.diff(o.first)) < 256
    assert_identical(g, o)
    g, o = run_both(nlpkg, orc, X, 6.6, C, (True, True, False), int_type=torch.int64)
    assert_identical(g, o)


def test_cutoff_boundary_pairs_decided_in_fp64(nlpkg, orc):
    """Pairs at (and one ulp around) the cutoff on a lattice: the FP32 screen
    cannot decide them, the FP64 recheck must reproduce the reference."""
    X, C = cf.fcc_cubic(3.61, (4, 4, 4))
    rc = 3.61 / np.sqrt(2)
    for r in (np.nextafter(rc, 0), rc, np.nextafter(rc, 10)):
        g, o = run_both(nlpkg, orc, X, r, C, (True, True, True))
        assert_identical(g, o)
        assert g.rechecks > 0


def test_unsorted_legacy_equals_sortbased_set(nlpkg, orc):
    """The legacy list and the sort-based list hold the same (i, j, S) for
    atoms inside the cell (the reference's test/test_sortbased.jl checks)."""
    X, C, L = cf.rand_config(1000, seed=28)
    g = nlpkg.legacy_pairlist(torch.from_numpy(X).cuda(), 0.25 * L, C, (True, True, True))
    s = nlpkg.neighbour_list(torch.from_numpy(X).cuda(), 0.25 * L, C, (True, True, True))
    key = lambda nl: sorted(zip(to_np(nl.i).tolist(), to_np(nl.j).tolist(), *[to_np(nl.S[:, k]).tolist() for k in range(3)]))
    assert key(g) == key(s)


def test_edge_cases(nlpkg, orc):
    C = np.diag([10.0] * 3)
    for X, pbc in [(np.zeros((0, 3)), (1, 1, 1)), (np.array([[5.0, 5.0, 5.0]]), (1, 1, 1)),
                   (np.array([[5.0, 5.0, 5.0], [5.0, 5.0, 6.0]]), (1, 1, 1)),
                   (np.array([[1.0, 1.0, 1.0], [8.0, 8.0, 8.0]]), (0, 0, 0)),
                   (np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.0], [0.0, 10.0, 0.0]]), (0, 0, 0))]:
        g, o = run_both(nlpkg, orc, X, 3.0, C, pbc)
        assert_identical(g, o)


def test_bad_positions_raise(nlpkg):
    X = torch.tensor([[1.0, 2.0, 3.0], [float("nan"), 0.0, 0.0]], dtype=torch.float64, device="cuda")
    with pytest.raises(nlpkg.NLError):
        nlpkg.legacy_pairlist(X, 2.0, np.diag([10.0] * 3), (True, True, True))
