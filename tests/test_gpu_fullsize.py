"""Parity at the benchmark configurations' full sizes, bit for bit against the
oracle (the C restatement of the reference's sort-based CPU path, run on all
host threads):

* 1,000,000 and 4,000,000 atoms uniform at density 0.05, rc 5 A, full pbc:
  every array of the PairList (first, i, j, S) and the bits of R, in the
  reference's own order (a stronger check than the canonical (i, j, S)
  comparison of the reference's tests, test/test_utils.jl:68-70), and every
  SortedCellList array of the same call;
* the lazy per-atom reduction sum_j 1/r^6 on the 1M-atom cell list against
  the oracle's FP64 traversal, relative tolerance 1e-12 (the reduction order
  is the reference's per-atom traversal order, so it is expected bit-equal);
* the 4,096-system batch of uneven systems: every system's SortedCellList
  arrays, first, i, j, S and the bits of R.

Reference: src/gpu_kernels.jl:299-364 (materialize_pairlist),
src/cell_list.jl:632-679 (build_cell_list), :779-833 (lazy traversal)."""
import concurrent.futures as cfut
import os

import numpy as np
import pytest
import torch

import configs as cf

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
LAZY_RTOL = 1e-12


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def _assert_pairlist_equal(eng, total, ref):
    assert total == ref.npairs
    np.testing.assert_array_equal(eng.first.cpu().numpy().astype(np.int64), ref.first)
    for name, got, want in (("i", eng.i, ref.i), ("j", eng.j, ref.j), ("S", eng.S, ref.S)):
        g = got[:total].cpu().numpy().astype(np.int64)
        assert np.array_equal(g, want), name
        del g
    R = eng.R[:total].cpu().numpy()
    assert np.array_equal(_bits(R), _bits(ref.R)), "R bits"


@pytest.mark.parametrize("n_atoms", [1_000_000, 4_000_000])
def test_full_list_bit_exact(nlpkg, orc, n_atoms):
    X, C, L = cf.uniform_system(n_atoms, seed=0)
    Xd = torch.from_numpy(X).cuda()
    eng = nlpkg.NeighbourListEngine(n_atoms, C, 5.0, (True, True, True))
    total = eng.run(Xd)
    ref = orc.neighbour_list(X, 5.0, C, (True, True, True), nthreads=THREADS)
    _assert_pairlist_equal(eng, total, ref)
    # the cell list of the same call, field by field
    oc = orc.build_cell_list(X, 5.0, C, (True, True, True))
    assert np.array_equal(eng.perm.cpu().numpy().astype(np.int64), oc.perm)
    assert np.array_equal(eng.cid.cpu().numpy().astype(np.int64), oc.cell_id)
    assert np.array_equal(eng.offs.cpu().numpy().astype(np.int64), oc.cell_offsets)
    assert np.array_equal(_bits(eng.Xs.cpu().numpy()), _bits(oc.X))
    del eng, ref
    torch.cuda.empty_cache()


def test_lazy_r6_1m_against_fp64_oracle(nlpkg, orc):
    X, C, L = cf.uniform_system(1_000_000, seed=0)
    Xd = torch.from_numpy(X).cuda()
    eng = nlpkg.NeighbourListEngine(X.shape[0], C, 5.0, (True, True, True))
    eng.run(Xd)
    clist = eng.cell_list(Xd)
    got = nlpkg.lazy_reduce(clist, "inv_r6").cpu().numpy()
    ref = orc.lazy_sum_r6(orc.build_cell_list(X, 5.0, C, (True, True, True)), nthreads=THREADS)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    assert rel.max() <= LAZY_RTOL, rel.max()
    fast = nlpkg.lazy_reduce(clist, "inv_r6_fast").cpu().numpy()  # the fused symmetric pass
    rel = np.abs(fast - ref) / np.maximum(np.abs(ref), 1e-300)
    assert rel.max() <= LAZY_RTOL, rel.max()
    cnt = nlpkg.lazy_reduce(clist, "count").cpu().numpy().astype(np.int64)
    assert np.array_equal(cnt, np.diff(eng.first.cpu().numpy().astype(np.int64)))
    del eng
    torch.cuda.empty_cache()


def test_batch_4096_every_system_bit_exact(nlpkg, orc):
    systems = cf.batch_systems(4096, seed=0)
    X = np.ascontiguousarray(np.concatenate([x for (x, _, _, _) in systems]))
    Xd = torch.from_numpy(X).cuda()
    b = nlpkg.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems])
    total = b.run(Xd)
    po = b.pair_offsets_host().astype(np.int64)
    assert po[0] == 0 and po[-1] == total
    # the whole batch on the host once, then per-system slices
    h = {k: getattr(b, k).cpu().numpy() for k in ("perm", "Xs", "cid", "offs", "first", "i", "j", "S", "R")}

    def oracle(s):
        x, c, rc, p = systems[s]
        return orc.build_cell_list(x, rc, c, p), orc.neighbour_list(x, rc, c, p, nthreads=1)

    with cfut.ThreadPoolExecutor(max_workers=THREADS) as ex:  # the oracle's C calls release the GIL
        refs = list(ex.map(oracle, range(len(systems))))
    for s, (oc, o) in enumerate(refs):
        a0, a1 = int(b.atom0[s]), int(b.atom0[s + 1])
        c0, c1 = int(b.cell0[s]) + s, int(b.cell0[s + 1]) + s + 1
        p0, p1 = int(po[s]), int(po[s + 1])
        assert p1 - p0 == o.npairs, s
        assert np.array_equal(h["perm"][a0:a1].astype(np.int64), oc.perm), s
        assert np.array_equal(h["cid"][a0:a1].astype(np.int64), oc.cell_id), s
        assert np.array_equal(h["offs"][c0:c1].astype(np.int64), oc.cell_offsets), s
        assert np.array_equal(_bits(h["Xs"][a0:a1]), _bits(oc.X)), s
        assert np.array_equal(h["first"][a0 + s:a1 + s + 1].astype(np.int64), o.first), s
        assert np.array_equal(h["i"][p0:p1].astype(np.int64), o.i), s
        assert np.array_equal(h["j"][p0:p1].astype(np.int64), o.j), s
        assert np.array_equal(h["S"][p0:p1].astype(np.int64), o.S), s
        assert np.array_equal(_bits(h["R"][p0:p1]), _bits(o.R)), s
