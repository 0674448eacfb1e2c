"""The lazy per-atom traversal on the device (nl_query_neighbours):
neighbours(clist, i), count_neighbours(clist, i) and for_each_neighbour
(cell_list.jl:779-833) for single atoms and for sets of atoms, against the
oracle's traversal of the same cell list -- j, S and the bits of R in the
reference's order -- without the system's list being materialised.  Cases:
cubic, triclinic, mixed and open boundaries, a one-cell system whose
stencil reaches several periodic images (diamond primitive, rc 6), atoms
far outside an open axis, Int64, and an out-of-range atom index."""
import numpy as np
import pytest
import torch

import configs as cf

pytestmark = pytest.mark.gpu


def _cases():
    Xd, Cd = cf.diamond_primitive()
    Xf, Cf, pf = cf.fcc_sheared(n=5, seed=11)
    X, C, L = cf.rand_config(3000, seed=12)
    Xo = X.copy()
    Xo[:20, 2] += np.random.default_rng(13).uniform(2.0, 30.0, 20) * L  # far outside the open z axis
    Xt, Ct = cf.rand_config_triclinic(400, seed=14)
    return [
        (X, C, 5.0, (True, True, True)),
        (Xo, C, 5.0, (True, True, False)),
        (Xf, Cf, 5.0, pf),
        (Xd, Cd, 6.0, (True, True, True)),
        (Xt, Ct, 3.0, (False, True, False)),
        (X[:500], C, 5.0, (False, False, False)),
    ]


@pytest.mark.parametrize("case", range(6))
def test_neighbours_of_single_atoms(nlpkg, orc, case):
    X, C, rc, pbc = _cases()[case]
    clist = nlpkg.build_cell_list(torch.from_numpy(np.ascontiguousarray(X)).cuda(), rc, C, pbc)
    oc = orc.build_cell_list(X, rc, C, pbc)
    for i in sorted({1, 2, X.shape[0], (X.shape[0] + 1) // 2, min(17, X.shape[0])}):
        js, Rs, Ss = nlpkg.neighbours(clist, i)
        oj, oR, oS = orc.neighbours(oc, i)
        assert np.array_equal(js.cpu().numpy().astype(np.int64), oj), i
        assert np.array_equal(Ss.cpu().numpy().astype(np.int64), oS), i
        assert np.array_equal(Rs.cpu().numpy().view(np.int64), oR.view(np.int64)), i
        assert nlpkg.count_neighbours(clist, i) == oj.shape[0]
        seen = []
        nlpkg.for_each_neighbour(lambda j, R, S: seen.append((j, tuple(S))), clist, i)
        assert seen == [(int(a), tuple(int(v) for v in b)) for a, b in zip(oj, oS)]


@pytest.mark.parametrize("int_type", [torch.int32, torch.int64])
def test_query_sets_match_the_full_list(nlpkg, orc, int_type):
    X, C, L = cf.rand_config(20000, seed=15)
    pbc = (True, False, True)
    clist = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), 5.0, C, pbc, int_type=int_type)
    o = orc.neighbour_list(X, 5.0, C, pbc, ti_bytes=4 if int_type == torch.int32 else 8, nthreads=8)
    atoms = np.random.default_rng(16).choice(X.shape[0], 500, replace=False) + 1
    first, j, S, R = nlpkg.query_neighbours(clist, atoms)
    first = first.cpu().numpy()
    j, S, R = j.cpu().numpy().astype(np.int64), S.cpu().numpy().astype(np.int64), R.cpu().numpy()
    assert j.dtype == np.int64 and first[0] == 1
    for k, a in enumerate(atoms):
        lo, hi = o.first[a - 1] - 1, o.first[a] - 1
        g0, g1 = first[k] - 1, first[k + 1] - 1
        assert np.array_equal(j[g0:g1], o.j[lo:hi]), a
        assert np.array_equal(S[g0:g1], o.S[lo:hi]), a
        assert np.array_equal(R[g0:g1].view(np.int64), o.R[lo:hi].view(np.int64)), a


def test_query_rejects_out_of_range_atoms(nlpkg):
    X, C, L = cf.rand_config(1000, seed=17)
    clist = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), 5.0, C, (True, True, True))
    with pytest.raises(nlpkg.NLError):
        nlpkg.query_neighbours(clist, [1, 1001])
    assert nlpkg.count_neighbours(clist, 1000) >= 0  # the error word was cleared


LAZY_RTOL = 1e-12  # the fast sum's stated relative tolerance on the per-atom sums


@pytest.mark.parametrize("case", range(6))
def test_fused_lazy_sum_and_count(nlpkg, orc, case):
    """The fast lazy sum (NL_REDUCE_INV_R6_FAST: the mask pass, then each
    unordered pair once with fixed-point R) and the fused lazy count: per-atom
    sums of 1/r^6 within 1e-12 of the oracle's FP64 traversal, per-atom
    counts equal to the oracle's, on geometries they take (cubic, mixed and
    open boundaries, sheared triclinic, atoms far outside an open axis: FP64
    R) and on ones they hand to the traversal-order passes (the diamond
    cell's 5x5x5 stencil)."""
    X, C, rc, pbc = _cases()[case]
    clist = nlpkg.build_cell_list(torch.from_numpy(np.ascontiguousarray(X)).cuda(), rc, C, pbc)
    oc = orc.build_cell_list(X, rc, C, pbc)
    ref = orc.lazy_sum_r6(oc)
    got = nlpkg.lazy_reduce(clist, "inv_r6_fast").cpu().numpy()
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    assert rel.max() <= LAZY_RTOL, rel.max()
    o = orc.neighbour_list(X, rc, C, pbc, nthreads=8)
    cnt = nlpkg.lazy_reduce(clist, "count").cpu().numpy().astype(np.int64)
    assert np.array_equal(cnt, np.diff(o.first))


def test_fused_lazy_crowded_cell_falls_back(nlpkg, orc):
    """A cell of more than 32 atoms: the mask pass gives up and the
    traversal-order passes produce every sum (then bit-identical)."""
    rng = np.random.default_rng(18)
    X, C, L = cf.rand_config(3000, seed=19)
    X = np.concatenate([X, L / 2 + (rng.random((60, 3)) - 0.5) * 0.8])
    clist = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), 5.0, C, (True, True, True))
    ref = orc.lazy_sum_r6(orc.build_cell_list(X, 5.0, C, (True, True, True)))
    got = nlpkg.lazy_reduce(clist, "inv_r6_fast").cpu().numpy()
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))
    o = orc.neighbour_list(X, 5.0, C, (True, True, True), nthreads=8)
    assert np.array_equal(nlpkg.lazy_reduce(clist, "count").cpu().numpy().astype(np.int64), np.diff(o.first))


def test_fused_lazy_close_pairs(nlpkg, orc):
    """Pairs at distances down to 1e-9 A and coincident atoms: the close ones
    are evaluated in FP64 with the reference's formula (an exact zero
    distance gives +Inf, as 1/0 does in the reference)."""
    X, C, L = cf.rand_config(4000, seed=20)
    X = X.copy()
    for k, d in enumerate([1e-9, 1e-6, 1e-3, 0.05, 0.5]):
        X[2 * k + 1] = X[2 * k] + np.array([d, 0.0, 0.0])
    X[20] = X[21]  # coincident
    clist = nlpkg.build_cell_list(torch.from_numpy(X).cuda(), 5.0, C, (True, True, True))
    ref = orc.lazy_sum_r6(orc.build_cell_list(X, 5.0, C, (True, True, True)))
    got = nlpkg.lazy_reduce(clist, "inv_r6_fast").cpu().numpy()
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got), fin) and np.all(got[~fin] == ref[~fin])
    rel = np.abs(got[fin] - ref[fin]) / np.abs(ref[fin])
    assert rel.max() <= LAZY_RTOL, rel.max()


def test_fast_lazy_sum_windings_and_far_positions(nlpkg, orc):
    """The fast sum's two position paths: atoms wound once around periodic
    axes (fixed-point R, S from the windings), a chain of atoms reaching
    beyond 2000 A along an open axis (outside the fixed-point range: R with
    the reference's FP64 operations), and a long periodic box whose wound
    atoms give shifts C'S beyond 2048 A (fixed point modulo 2^64)."""
    X, C, L = cf.rand_config(3000, seed=21)
    Xw = X.copy()
    Xw[:200, 0] += L          # winding +1 on x
    Xw[200:400, 1] -= 2 * L   # winding -2 on y
    rng = np.random.default_rng(22)
    n = 1300
    Xc = np.stack([np.arange(n) * 2.0 + rng.uniform(-0.3, 0.3, n), rng.uniform(0, 16, n), rng.uniform(0, 16, n)], 1)
    Cc = np.diag([2.0 * n, 16.0, 16.0])  # 3 cells across y and z: the mask pass takes it
    # a 1100 A periodic chain whose ends are wound +1 and -2: pairs across the
    # x boundary have C'S = 2200 A (beyond 2^11 A: the fixed-point shift
    # wraps modulo 2^64 together with Xj - Xi)
    m = 2200
    Xl = np.stack([np.arange(m) * 0.5 + rng.uniform(-0.2, 0.2, m), rng.uniform(0, 16, m), rng.uniform(0, 16, m)], 1)
    Xl[Xl[:, 0] < 50.0, 0] += 1100.0
    Xl[Xl[:, 0] > 1050.0, 0] -= 2200.0
    Xl[(np.arange(m) % 7 == 3) & (Xl[:, 0] > 100.0) & (Xl[:, 0] < 800.0), 0] += 1100.0
    Cl = np.diag([1100.0, 16.0, 16.0])
    for Xs, Cs, pbc in ((Xw, C, (True, True, True)), (Xc, Cc, (False, True, True))):
        clist = nlpkg.build_cell_list(torch.from_numpy(np.ascontiguousarray(Xs)).cuda(), 5.0, Cs, pbc)
        ref = orc.lazy_sum_r6(orc.build_cell_list(Xs, 5.0, Cs, pbc))
        got = nlpkg.lazy_reduce(clist, "inv_r6_fast").cpu().numpy()
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
        assert rel.max() <= LAZY_RTOL, rel.max()
    # at |X| ~ 1900 A and C'S = 2200 A the reference's own FP64 R is off by a
    # few 1e-13 A (about 1.4e-12 on the sums): the fast sum is held to 1e-12 of
    # the exact sums, and to the oracle within 1e-12 plus the oracle's own error
    clist = nlpkg.build_cell_list(torch.from_numpy(np.ascontiguousarray(Xl)).cuda(), 5.0, Cl, (True, True, True))
    ref = orc.lazy_sum_r6(orc.build_cell_list(Xl, 5.0, Cl, (True, True, True)))
    got = nlpkg.lazy_reduce(clist, "inv_r6_fast").cpu().numpy()
    ex = _exact_sum_r6(Xl, Cl, orc.neighbour_list(Xl, 5.0, Cl, (True, True, True), nthreads=8))
    den = np.maximum(np.abs(ex), 1e-300)
    assert (np.abs(got - ex) / den).max() <= LAZY_RTOL
    assert (np.abs(got - ref) / den).max() <= LAZY_RTOL + (np.abs(ref - ex) / den).max()


def _exact_sum_r6(X, C, o):
    """Per-atom sums of 1/r^6 over the list's pairs with R = Xj - Xi + C'S and
    r^2 in exact rational arithmetic (each term correctly rounded, summed
    with math.fsum)."""
    from fractions import Fraction
    import math

    I, J, S = np.asarray(o.i) - 1, np.asarray(o.j) - 1, np.asarray(o.S)
    Xf = [[Fraction(float(v)) for v in row] for row in X]
    Cf = [[Fraction(float(v)) for v in row] for row in C]
    terms = [[] for _ in range(len(X))]
    for p in range(len(I)):
        i, j, s = int(I[p]), int(J[p]), [int(v) for v in S[p]]
        r2 = Fraction(0)
        for k in range(3):
            d = Xf[j][k] - Xf[i][k] + sum(Cf[l][k] * s[l] for l in range(3))
            r2 += d * d
        terms[i].append(float(1 / r2 ** 3))
    return np.array([math.fsum(t) for t in terms])
