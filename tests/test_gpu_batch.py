"""Batches of independent systems (nl_batch_neighbour_list) against the
oracle, system by system: every per-system SortedCellList array, first, i, j,
S and the bits of R must equal the single-system reference results."""
import numpy as np
import pytest
import torch

import configs as cf

pytestmark = pytest.mark.gpu


def to_np(t):
    return t.detach().cpu().numpy()


def check_batch(nlpkg, orc, systems, int_type=torch.int32, capacity=None, count_kernel=None):
    b = nlpkg.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems], int_type=int_type,
                                 capacity=capacity)
    if count_kernel is not None:
        b.set_tuning(0, 0, count_kernel)
    X = np.concatenate([x for (x, _, _, _) in systems]) if systems else np.zeros((0, 3))
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).cuda()
    total = b.run(Xd)
    ti = 4 if int_type == torch.int32 else 8
    po = b.pair_offsets_host()
    assert po[0] == 0 and po[-1] == total
    for s, (x, c, rc, p) in enumerate(systems):
        clist, pl = b.system(s, Xd)
        oc = orc.build_cell_list(x, rc, c, p, ti_bytes=ti)
        assert np.array_equal(to_np(clist.perm).astype(np.int64), oc.perm), s
        assert np.array_equal(to_np(clist.cell_id).astype(np.int64), oc.cell_id), s
        assert np.array_equal(to_np(clist.cell_offsets).astype(np.int64), oc.cell_offsets), s
        assert np.array_equal(to_np(clist.X).view(np.int64), oc.X.view(np.int64)), s
        o = orc.neighbour_list(x, rc, c, p, ti_bytes=ti, nthreads=8)
        assert int(pl.i.shape[0]) == o.npairs, s
        assert np.array_equal(to_np(pl.first).astype(np.int64), o.first), s
        assert np.array_equal(to_np(pl.i).astype(np.int64), o.i), s
        assert np.array_equal(to_np(pl.j).astype(np.int64), o.j), s
        assert np.array_equal(to_np(pl.S).astype(np.int64), o.S), s
        assert np.array_equal(to_np(pl.R).view(np.int64), o.R.view(np.int64)), s
    return b, total


@pytest.mark.parametrize("seed", [0, 1])
def test_batch_random_systems(nlpkg, orc, seed):
    check_batch(nlpkg, orc, cf.batch_systems(40, seed=seed, nmax=700))


def test_batch_int64(nlpkg, orc):
    check_batch(nlpkg, orc, cf.batch_systems(12, seed=5, nmax=500), int_type=torch.int64)


def test_batch_edge_systems(nlpkg, orc):
    """Empty and one-atom systems, a one-cell system with a 5x5x5 stencil
    (diamond primitive, rc 6), open boundaries, a dense cell (> 256 atoms in
    one cell) and a triclinic cell, mixed in one batch."""
    rng = np.random.default_rng(3)
    Xd, Cd = cf.diamond_primitive()
    Cbox = np.diag([7.0, 7.0, 7.0])
    dense = rng.random((600, 3)) * 7.0
    Xt, Ct = cf.rand_config_triclinic(80, seed=3)
    Xf, Cf, pf = cf.fcc_sheared(n=4, seed=1)
    systems = [
        (np.zeros((0, 3)), np.diag([10.0, 10.0, 10.0]), 3.0, (True, True, True)),
        (np.array([[1.0, 2.0, 3.0]]), np.diag([10.0, 10.0, 10.0]), 3.0, (True, True, True)),
        (Xd, Cd, 6.0, (True, True, True)),
        (rng.random((50, 3)) * 20.0, np.diag([20.0, 20.0, 20.0]), 4.0, (False, False, False)),
        (dense, Cbox, 2.5, (True, True, True)),
        (Xt, Ct, 3.0, (True, True, True)),
        (Xf, Cf, 5.0, pf),
        (np.zeros((0, 3)), np.diag([5.0, 5.0, 5.0]), 2.0, (False, True, False)),
    ]
    b, total = check_batch(nlpkg, orc, systems)
    assert total == sum(orc.neighbour_list(x, rc, c, p).npairs for (x, c, rc, p) in systems)


def test_batch_matches_single_calls_and_repeats(nlpkg, orc):
    systems = cf.batch_systems(16, seed=9, nmax=400)
    b = nlpkg.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems])
    X = torch.from_numpy(np.concatenate([s[0] for s in systems])).cuda()
    t1 = b.run(X)
    i1, R1 = b.i[:t1].clone(), b.R[:t1].clone()
    b.launch(X)  # second run into the same buffers, no host synchronisation
    b.sync_status()
    assert torch.equal(b.i[:t1], i1) and torch.equal(b.R[:t1].view(torch.int64), R1.view(torch.int64))
    for s, (x, c, rc, p) in enumerate(systems):
        _, pl = b.system(s, X)
        g = nlpkg.neighbour_list(torch.from_numpy(x).cuda(), rc, c, p)
        assert torch.equal(pl.i, g.i) and torch.equal(pl.j, g.j) and torch.equal(pl.S, g.S)
        assert torch.equal(pl.R.view(torch.int64), g.R.view(torch.int64))


def test_batch_capacity_growth(nlpkg, orc):
    systems = cf.batch_systems(10, seed=11, nmax=300)
    check_batch(nlpkg, orc, systems, capacity=5)


def test_batch_graph_replay_and_autotune(nlpkg, orc):
    """A captured CUDA graph and every tuned launch shape give the same bits."""
    systems = cf.batch_systems(24, seed=13, nmax=500)
    b = nlpkg.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems])
    X = torch.from_numpy(np.concatenate([s[0] for s in systems])).cuda()
    t = b.run(X)
    ref = [x[:t].clone() for x in (b.i, b.j, b.S)] + [b.R[:t].clone().view(torch.int64), b.first.clone()]
    res = nlpkg.autotune(b, X, candidates=[(3, 4), (7, 16), (5, 8)], reps=1)
    assert len(res["trials"]) == 3
    b.capture(X)
    for _ in range(2):
        b.replay()
    torch.cuda.synchronize()
    b.sync_status()
    got = [x[:t] for x in (b.i, b.j, b.S)] + [b.R[:t].view(torch.int64), b.first]
    for u, v in zip(ref, got):
        assert torch.equal(u, v)


def test_engine_graph_replay(nlpkg, orc):
    X, C, L = cf.rand_config(20000, seed=21)
    eng = nlpkg.NeighbourListEngine(X.shape[0], C, 5.0, (True, True, True))
    Xd = torch.from_numpy(X).cuda()
    t = eng.run(Xd)
    eng.set_tuning(3, 4)
    eng.capture(Xd)
    eng.i[:t].zero_()
    eng.replay()
    torch.cuda.synchronize()
    eng.sync_status()
    o = orc.neighbour_list(X, 5.0, C, (True, True, True), nthreads=8)
    assert np.array_equal(eng.i[:t].cpu().numpy().astype(np.int64), o.i)
    assert np.array_equal(eng.R[:t].cpu().numpy().view(np.int64), o.R.view(np.int64))


@pytest.mark.parametrize("count_kernel", [1, 2, 3])
def test_batch_both_count_kernels(nlpkg, orc, count_kernel):
    systems = cf.batch_systems(30, seed=17, nmax=600)
    b = nlpkg.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems])
    b.set_tuning(0, 0, count_kernel)
    X = torch.from_numpy(np.concatenate([s[0] for s in systems])).cuda()
    b.run(X)
    for s, (x, c, rc, p) in enumerate(systems):
        _, pl = b.system(s, X)
        o = orc.neighbour_list(x, rc, c, p, nthreads=8)
        assert np.array_equal(to_np(pl.j).astype(np.int64), o.j), s
        assert np.array_equal(to_np(pl.S).astype(np.int64), o.S), s
        assert np.array_equal(to_np(pl.R).view(np.int64), o.R.view(np.int64)), s


@pytest.mark.parametrize("count_kernel", [0, 1, 3])
def test_batch_symmetric_count_mixed(nlpkg, orc, count_kernel):
    """Systems that take the symmetric count pass (27 distinct stencil cells)
    next to systems that cannot (fewer than 3 cells on a periodic axis) and
    one that gives it up (a cell of more than 32 atoms): atoms of more than
    192 pairs (screening write pass), of 65..192 pairs decoded from the masks,
    open axes and windings, all equal to the oracle."""
    rng = np.random.default_rng(60)
    Xc, Cc, Lc = cf.corner_clump(4000, 5.0, seed=55)
    Xm = cf.corner_clump(4000, 5.0, per_octant=20, seed=57)[0]
    X6 = cf.corner_clump(4000, 6.0, seed=55)[0]
    Xr, Cr, Lr = cf.rand_config(3000, seed=61)
    crowded = np.concatenate([Xr, Lr / 2 + rng.random((40, 3)) * 0.5])
    Xo, Co, Lo = cf.rand_config(2000, seed=62)
    Xw, Cw, Lw = cf.rand_config(600, seed=63)
    Xw = Xw + rng.integers(-3, 4, Xw.shape) * Lw
    Xs, Cs, Ls = cf.rand_config(100, seed=64)
    Xt, Ct = cf.rand_config_triclinic(300, seed=65)
    systems = [
        (Xc, Cc, 5.0, (True, True, True)),
        (np.zeros((0, 3)), np.diag([10.0] * 3), 3.0, (True, True, True)),
        (Xm, Cc, 5.0, (True, True, True)),
        (crowded, Cr, 5.0, (True, True, True)),
        (Xs, Cs, 0.4 * Ls, (True, True, True)),
        (Xo, Co, 5.0, (True, True, False)),
        (Xw, Cw, 0.2 * Lw, (True, True, True)),
        (Xt, Ct, 3.0, (True, False, True)),
        (X6, Cc, 6.0, (True, True, False)),
    ]
    check_batch(nlpkg, orc, systems, count_kernel=count_kernel)


@pytest.mark.parametrize("count_kernel", [0, 1])
def test_batch_large_single_cells_in_rounds(nlpkg, orc, count_kernel):
    """Systems whose cells the per-cell passes take in rounds of 32 home
    atoms: one-cell periodic systems of 150 and 70 atoms (their stencils
    images of the one cell), a symmetric-pass system with a crowded cell of
    80 atoms (failed and handed to the per-cell passes with its cells and
    slot chunks), and symmetric-pass systems around them."""
    rng = np.random.default_rng(71)
    X1 = rng.random((150, 3)) * 9.0
    X2 = rng.random((70, 3)) * 7.0
    Xr, Cr, Lr = cf.rand_config(2500, seed=72)
    crowded = np.concatenate([Xr, Lr / 3 + rng.random((80, 3)) * 1.2])
    Xa, Ca, La = cf.rand_config(1200, seed=73)
    Xb, Cb, Lb = cf.rand_config(900, seed=74)
    systems = [
        (Xa, Ca, 5.0, (True, True, True)),
        (X1, np.diag([9.0, 9.0, 9.0]), 6.0, (True, True, True)),
        (crowded, Cr, 5.0, (True, True, True)),
        (X2, np.diag([7.0, 7.0, 7.0]), 6.5, (True, True, False)),
        (Xb, Cb, 5.0, (True, False, True)),
    ]
    check_batch(nlpkg, orc, systems, count_kernel=count_kernel)
