"""The continuous-batching server: every result is the same alone and in the
mix (bit for bit: integer outputs and the bits of R), equal to the oracle,
with budget-bounded admission and re-runs when the pair prediction is low."""
import numpy as np
import pytest
import torch

import configs as cf

pytestmark = pytest.mark.gpu


def mixed_systems():
    systems = cf.batch_systems(40, seed=31, nmax=900)
    X, C, L = cf.rand_config(20000, seed=32)
    systems.insert(17, (X, C, 5.0, (True, True, True)))
    return systems


def serve(nlpkg, systems, rate=1e6, **kw):
    srv = nlpkg.NeighbourListServer(copy_results=True, **kw)
    reqs = nlpkg.poisson_trace(systems, rate=rate, seed=1)
    stats = srv.run_trace(reqs)
    srv.close()
    return reqs, stats, srv


def same(a, b):
    return (torch.equal(a["first"], b["first"]) and torch.equal(a["i"], b["i"]) and torch.equal(a["j"], b["j"])
            and torch.equal(a["S"], b["S"]) and torch.equal(a["R"].view(torch.int64), b["R"].view(torch.int64)))


def test_same_alone_and_in_mix(nlpkg, orc):
    systems = mixed_systems()
    mix, stats, srv = serve(nlpkg, systems, slots=2)
    assert stats["requests"] == len(systems) and srv.batches < len(systems)  # requests were batched
    for r in mix:
        alone, _, _ = serve(nlpkg, [(r.X, r.cell, r.cutoff, r.pbc)], slots=1)
        assert same(alone[0].result, r.result), r.rid
    for r in mix:  # every request, every field, against the oracle
        o = orc.neighbour_list(r.X, r.cutoff, r.cell, r.pbc, nthreads=8)
        res = r.result
        assert np.array_equal(res["first"].cpu().numpy().astype(np.int64), o.first), r.rid
        for k in ("i", "j", "S"):
            assert np.array_equal(res[k].cpu().numpy().astype(np.int64), getattr(o, k)), (r.rid, k)
        assert np.array_equal(res["R"].cpu().numpy().view(np.int64), o.R.view(np.int64)), r.rid


def test_plain_mode_matches_batched(nlpkg):
    systems = mixed_systems()[:12]
    pinned = [(torch.from_numpy(x).pin_memory(), c, rc, p) for (x, c, rc, p) in systems]
    a, _, _ = serve(nlpkg, pinned, slots=2)  # pinned request buffers, copied per request
    b, _, srv = serve(nlpkg, systems, slots=2, mode="plain")
    assert srv.batches == len(systems)
    for x, y in zip(a, b):
        assert same(x.result, y.result)


def test_budget_bounds_admission_and_reruns(nlpkg, monkeypatch):
    systems = mixed_systems()[:16]
    ref, _, _ = serve(nlpkg, systems, slots=2)
    # a budget below one batch's worth serialises admission
    _, stats, srv = serve(nlpkg, systems, slots=3, pair_budget_bytes=2e5)
    assert srv.batches > 3
    # a prediction far too low forces re-runs; results do not change
    monkeypatch.setattr(nlpkg.Request, "predicted_pairs", lambda self: 1)
    got, stats, srv = serve(nlpkg, systems, slots=2)
    assert stats["reruns"] > 0
    for x, y in zip(ref, got):
        assert same(x.result, y.result)


def test_host_results_match_device_results(nlpkg):
    """With host_results the latency stops when a request's results are in
    pinned host memory: the same bits as the device results, every request."""
    systems = mixed_systems()[:14]
    dev, _, _ = serve(nlpkg, systems, slots=2)
    host, stats, _ = serve(nlpkg, systems, slots=2, host_results=True)
    assert stats["requests"] == len(systems)
    for a, b in zip(dev, host):
        assert not b.result["i"].is_cuda
        assert same({k: v.cpu() for k, v in a.result.items()}, b.result), a.rid
    plain, _, _ = serve(nlpkg, systems, slots=2, mode="plain", host_results=True)
    for a, b in zip(dev, plain):
        assert same({k: v.cpu() for k, v in a.result.items()}, b.result), a.rid


def test_float32_server_batched_and_plain(nlpkg, orc):
    """A Float32 server (dtype=torch.float32: Float32 batches, or plain
    nl_neighbour_list_f32 calls): every request, every field and the bits of
    R equal the oracle's Float32 restatement, in both modes."""
    systems = [(np.asarray(x, dtype=np.float32), c, rc, p) for (x, c, rc, p) in mixed_systems()[:24]]
    a, _, srv = serve(nlpkg, systems, slots=2, dtype=torch.float32)
    assert srv.batches < len(systems)
    b, _, _ = serve(nlpkg, systems, slots=2, mode="plain", dtype=torch.float32)
    for ra, rb in zip(a, b):
        o = orc.neighbour_list_f32(ra.X, ra.cutoff, ra.cell, ra.pbc)
        for res in (ra.result, rb.result):
            assert res["R"].dtype == torch.float32
            assert np.array_equal(res["first"].cpu().numpy().astype(np.int64), o.first), ra.rid
            for k in ("i", "j", "S"):
                assert np.array_equal(res[k].cpu().numpy().astype(np.int64), getattr(o, k)), (ra.rid, k)
            assert np.array_equal(res["R"].cpu().numpy().view(np.int32), o.R.view(np.int32)), ra.rid
