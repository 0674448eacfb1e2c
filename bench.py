"""Benchmark of the materialised neighbour-list path on one GB300.

Workload: 1,000,000 atoms uniform at density 0.05 A^-3 in a cubic periodic
box, cutoff 5 A, Float64 positions, Int32 indices (seeded synthetic input with
the shape of the reference's benchmark, scripts/benchmark.jl).  One step is
build_cell_list + materialize_pairlist with R: binning, sort, count, scan and
fill, all on the device, inputs resident in HBM.  L2 is flushed (256 MiB
write, untimed) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  Besides the headline keys it carries the
other configurations as sections: "lazy" (sum of 1/r^6 per atom at 1M),
"batched" (4,096 uneven systems, CUDA graph, autotuned, against plain
per-system launches), "atoms_4m", "half" (half list), "verlet" (skin reuse)
and "serving" (Poisson arrivals, p50/p99); --no-extra skips them.
--impl reference times the reference's sort-based CPU path (the C
restatement in oracle/, since Julia is not available) on the host cores for
the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

N_ATOMS = 1_000_000
DENSITY = 0.05
CUTOFF = 5.0
SEED = 0
METRIC = "pairs/s (1M atoms, rc 5 A, density 0.05, full pbc, Float64, build_cell_list + materialize_pairlist)"
WORKLOAD = "uniform 1,000,000 atoms, density 0.05 A^-3, cubic pbc box (L=271.44 A), cutoff 5 A, Float64, Int32 indices"
ALGO_BYTES_PER_ATOM = 24  # positions read
ALGO_BYTES_PER_PAIR = 44  # i 4 + j 4 + S 12 + R 24 written
# kernels of one step: k_bin, k_scan_offsets (cells), k_scatter, k_fix, k_fix_big (build);
# k_sym_count, k_pairs<count> (returns at once after the symmetric pass), k_scan_offsets
# (pairs) (count); k_cs_table, k_emit<lists> and k_pairs<fill> (both return at once),
# k_emit_orig (write)
LAUNCHES_PER_STEP = 12  # kernels of one step: build 5, count 3 (with its scan), write 4


def bench_config(n_atoms, pairs):
    """The workload description both arms print (identical dicts)."""
    return {"workload": WORKLOAD if n_atoms == N_ATOMS else f"uniform {n_atoms} atoms (profiling size)",
            "atoms": int(n_atoms), "pairs": int(pairs), "cutoff": CUTOFF, "density": DENSITY, "pbc": "TTT",
            "index_type": "Int32", "with_R": True,
            "l2": "GPU arm: 256 MiB write (untimed) before every timed step; CPU arm: positions and pair "
                  "arrays far larger than the host caches"}


def workload(n_atoms=N_ATOMS):
    import configs as cf

    X, C, L = cf.uniform_system(n_atoms, DENSITY, SEED)
    return X, C, (True, True, True)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the write kernel (k_emit_orig) at 1M atoms from the
    committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_emit_orig_1M_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(X, C, pbc, seconds_target=12.0, max_runs=3):
    """Oracle (C restatement of the reference's sort-based CPU path) on all
    host cores, on the full workload, a bounded number of runs."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    threads = os.cpu_count() or 1
    runs, t0 = 0, time.perf_counter()
    pairs = 0
    while runs < max_runs:
        pairs = orc.timed_neighbour_list(X, CUTOFF, C, pbc, threads, with_R=True)
        runs += 1
        if time.perf_counter() - t0 > seconds_target:
            break
    dt = (time.perf_counter() - t0) / runs
    return {"value": pairs / dt, "unit": "pairs/s", "cores": threads, "kind": "port",
            "sample": f"{runs} full run(s) of the 1M-atom workload (build + count + fill + R), {dt:.3f} s each"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    X, C, pbc = workload()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    orc.build()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        orc.timed_neighbour_list(X, CUTOFF, C, pbc, threads, with_R=True)
    t0 = time.perf_counter()
    pairs = 0
    for _ in range(args.steps):
        pairs = orc.timed_neighbour_list(X, CUTOFF, C, pbc, threads, with_R=True)
    dt = (time.perf_counter() - t0) / args.steps
    val = pairs / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "pairs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(N_ATOMS, pairs),
        "cpu_baseline": {"value": val, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} timed full runs of the workload after {args.warmup} warm-up runs"},
        "e2e": {"value": val, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Julia is not installed on either machine; the reference arm is the C restatement of the "
                "reference's sort-based CPU path (oracle/nl_oracle.c) on all host threads",
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch

    import __graft_entry__ as graft

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    nl = graft.load_package()
    n_atoms = args.atoms
    X, C, pbc = workload(n_atoms)
    Xd = torch.from_numpy(X).to(dev)
    eng = nl.NeighbourListEngine(n_atoms, C, CUTOFF, pbc, device=dev)
    total = eng.run(Xd)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    for _ in range(args.warmup):
        eng.launch(Xd)
    torch.cuda.synchronize(dev)
    # the step as an MD loop runs it: every kernel of the step captured once
    # in a CUDA graph over fixed buffers, one graph launch per step
    eng.capture(Xd)
    eng.replay()
    torch.cuda.synchronize(dev)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(dev.index or 0) as clk:
        barrier()
        torch.cuda.synchronize(dev)
        for k in range(args.steps):
            flush.fill_(k & 0xFF)  # untimed L2 flush (256 MiB > 129 MB L2)
            starts[k].record(stream)
            eng.replay()
            ends[k].record(stream)
        torch.cuda.synchronize(dev)
        barrier()
    eng.sync_status()
    step_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / args.steps
    # the same step issued kernel by kernel (no graph), for reference
    launch_ms = timed_steps(lambda: eng.launch(Xd), max(3, min(args.steps, 10)), flush, stream)
    eng.sync_status()
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    assert eng.total_pairs() == total
    rechecks = eng.rechecks()

    # ---- fill kernel alone (same stream, records from the last step)
    import ctypes as Cc

    from neighbourlists_gb300 import _lib
    from neighbourlists_gb300.api import _ptr, _stream_handle

    L = _lib.lib()
    p = eng.plan
    D, I64, U8 = Cc.POINTER(Cc.c_double), Cc.POINTER(Cc.c_int64), Cc.POINTER(Cc.c_uint8)

    def fill():
        _lib.check(L.nl_fill_pairs(_ptr(eng.Xs), _ptr(eng.perm), Cc.c_void_p(eng.offs.data_ptr()), n_atoms,
                                   p.cell_cm.ctypes.data_as(D), p.inv_cm.ctypes.data_as(D),
                                   p.ncells.ctypes.data_as(I64), p.nxyz.ctypes.data_as(I64),
                                   eng.pbc.ctypes.data_as(U8), CUTOFF, eng.ib, Cc.c_void_p(eng.first.data_ptr()),
                                   eng.capacity, _ptr(eng.i), _ptr(eng.j), _ptr(eng.S), _ptr(eng.R), _ptr(eng.ws),
                                   eng.ws.numel(), _stream_handle(stream)))

    fill()
    fs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    fe = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        fs[k].record(stream)
        fill()
        fe[k].record(stream)
    torch.cuda.synchronize(dev)
    eng.sync_status()
    fill_ms = sum(s.elapsed_time(e) for s, e in zip(fs, fe)) / args.steps

    # ---- end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(eng, X, Xd, total, stream, dev, args)
    extra = {}
    if not args.no_extra and n_atoms == N_ATOMS and rank == 0:
        extra_steps = max(3, min(args.steps, 10))
        extra["lazy"] = bench_lazy(nl, eng, Xd, X, C, pbc, stream, flush, extra_steps)
        del eng
        torch.cuda.empty_cache()
        extra["batched"] = bench_batched(nl, dev, stream, flush, extra_steps)
        torch.cuda.empty_cache()
        extra["atoms_4m"] = bench_4m(nl, dev, stream, flush, extra_steps)
        torch.cuda.empty_cache()
        extra.update(bench_half_and_verlet(nl, dev, stream, flush, extra_steps))
        torch.cuda.empty_cache()
        extra.update(bench_float32_and_legacy(nl, dev, stream, flush, extra_steps))
        torch.cuda.empty_cache()
        extra["serving"] = bench_serving(nl, dev)
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    algo_bytes = ALGO_BYTES_PER_ATOM * n_atoms + ALGO_BYTES_PER_PAIR * total
    achieved = algo_bytes / (fill_ms * 1e-3) / 1e9
    traffic = ncu_traffic() if n_atoms == N_ATOMS else None
    cpu = cpu_baseline(X, C, pbc) if not args.no_cpu_baseline else None
    value = world * total / (step_ms * 1e-3)
    if e2e is not None:
        e2e["value"] = world * total / (e2e["ms_per_step"] * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(n_atoms, total),
        "timing": {"cuda_graph": True, "ms_per_step_without_graph": launch_ms,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "kernel": "write pass (k_emit_orig + k_cs_table; k_emit<lists>, k_pairs<fill> return at once)",
                     "algorithmic_bytes": algo_bytes, "kernel_ms": fill_ms,
                     "traffic": (traffic or {}).get("dram_bytes_per_launch")},
        "step_roofline_frac": algo_bytes / (step_ms * 1e-3) / 1e9 / peak,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk.summary(),
        "gpu_launches": LAUNCHES_PER_STEP * args.steps,
        "rechecks": rechecks,
        "recheck_band_rel": float(p.band / (CUTOFF * CUTOFF)),
        **extra,
    }
    print(json.dumps(line))


def timed_steps(fn, steps, flush, stream):
    """Mean CUDA-event time (ms) of fn over `steps` calls, L2 flushed before each."""
    import torch

    ts = []
    for k in range(steps):
        flush.fill_(k & 0xFF)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        ts.append((s, e))
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in ts) / steps


def bench_batched(nl, dev, stream, flush, steps):
    """4,096 uneven systems: one batched pass (captured in a CUDA graph, launch
    shapes autotuned) against the plain per-system launches of the same
    systems on the same GPU; outputs compared bit for bit."""
    import torch
    import configs as cf

    systems = cf.batch_systems(4096, seed=0)
    X = np.ascontiguousarray(np.concatenate([x for (x, _, _, _) in systems]))
    Xd = torch.from_numpy(X).to(dev)
    b = nl.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems], device=dev)
    total = b.run(Xd)
    tune = nl.autotune(b, Xd, reps=2)
    b.capture(Xd)
    batch_ms = timed_steps(b.replay, steps, flush, stream)
    b.sync_status()
    # plain: one engine and one nl_neighbour_list call per system
    engines, views = [], []
    for s, (x, c, rc, p) in enumerate(systems):
        a0, a1 = int(b.atom0[s]), int(b.atom0[s + 1])
        engines.append(nl.NeighbourListEngine(x.shape[0], c, rc, p, device=dev, capacity=x.shape[0] * 64 + 64))
        views.append(Xd[a0:a1])
    for e, v in zip(engines, views):
        e.run(v)

    def plain():
        for e, v in zip(engines, views):
            e.launch(v)

    plain_steps = max(1, min(steps, 2))
    plain_ms = timed_steps(plain, plain_steps, flush, stream)
    # the same per-system calls with the host out of the way: every system's
    # call captured in its own CUDA graph, the graphs replayed one after
    # another on one stream, and round-robin on eight streams (systems overlap
    # on the device)
    for e, v in zip(engines, views):
        e.capture(v)
    torch.cuda.synchronize(dev)

    def plain_graphs():
        for e in engines:
            e.replay()

    plain_graph_ms = timed_steps(plain_graphs, plain_steps, flush, stream)
    side = [torch.cuda.Stream(device=dev) for _ in range(8)]

    def plain_streams():
        for st in side:
            st.wait_stream(stream)
        for k, e in enumerate(engines):
            with torch.cuda.stream(side[k % 8]):
                e.replay()
        for st in side:
            stream.wait_stream(st)

    plain_streams_ms = timed_steps(plain_streams, plain_steps, flush, stream)
    # bit-identical outputs (every system)
    po = b.pair_offsets_host()
    same = True
    for s, e in enumerate(engines):
        p0, p1 = int(po[s]), int(po[s + 1])
        t = e.total_pairs()
        same &= (t == p1 - p0 and torch.equal(e.i[:t], b.i[p0:p1]) and torch.equal(e.j[:t], b.j[p0:p1])
                 and torch.equal(e.S[:t], b.S[p0:p1])
                 and torch.equal(e.R[:t].view(torch.int64), b.R[p0:p1].view(torch.int64)))
    nsys = len(systems)
    # the same systems with Float32 positions, cells and cutoffs (one CUDA graph)
    del engines, views
    X32 = torch.from_numpy(X.astype(np.float32)).to(dev)
    b32 = nl.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems], device=dev,
                                dtype=torch.float32)
    total32 = b32.run(X32)
    b32.capture(X32)
    f32_ms = timed_steps(b32.replay, steps, flush, stream)
    b32.sync_status()
    del b32
    return {"workload": "4,096 systems, atoms log-uniform [8, 4096] (2,740,812 atoms), triclinic, density "
                        "U[0.03,0.10], off-diagonals U(+-0.15 diag), pbc per axis p=0.8, cutoff U[3,6] A, seed 0",
            "systems": nsys, "atoms": int(X.shape[0]), "pairs": int(total),
            "systems_per_s": nsys / (batch_ms * 1e-3), "ms_per_batch": batch_ms,
            "pairs_per_s": total / (batch_ms * 1e-3),
            "plain_systems_per_s": nsys / (plain_ms * 1e-3), "plain_ms": plain_ms,
            "plain_graphs_ms": plain_graph_ms, "plain_graphs_8_streams_ms": plain_streams_ms,
            "plain_note": "plain_ms: one engine.launch per system from Python; plain_graphs_ms: each system's "
                          "call as its own CUDA graph, replayed back to back on one stream; "
                          "plain_graphs_8_streams_ms: the same graphs round-robin on eight streams",
            "speedup_vs_plain": plain_ms / batch_ms,
            "speedup_vs_plain_graphs": min(plain_graph_ms, plain_streams_ms) / batch_ms,
            "identical_to_plain": bool(same),
            "cuda_graph": True, "autotune": {k: tune[k] for k in ("pair_blocks_per_sm", "emit_blocks_per_sm", "count_kernel", "ms")},
            "float32": {"ms_per_batch": f32_ms, "systems_per_s": nsys / (f32_ms * 1e-3), "pairs": int(total32),
                        "note": "the same systems in Float32 (cell, cutoff, positions, R), CUDA graph, default "
                                "launch shapes"},
            "l2": "flushed before every timed step"}


def bench_lazy(nl, eng, Xd, X, C, pbc, stream, flush, steps):
    """Lazy traversal with the built-in per-atom reduction sum_j 1/r^6 on the
    1M-atom cell list, against the FP64 oracle."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    eng.launch(Xd)
    clist = eng.cell_list(Xd)
    ref = orc.lazy_sum_r6(orc.build_cell_list(X, CUTOFF, C, pbc), nthreads=os.cpu_count() or 1)
    res = {"workload": "lazy per-atom reductions over the same 1M-atom cell list, no pair list written",
           "tolerance": 1e-12}
    # "inv_r6": traversal-order passes (bit-identical sums); "inv_r6_fast": the
    # fused symmetric screen-and-reduce pass; "count": neighbours per atom
    for kind in ("inv_r6", "inv_r6_fast", "count"):
        out = nl.lazy_reduce(clist, kind)
        ms = timed_steps(lambda: nl.lazy_reduce(clist, kind, out=out, sync=False), steps, flush, stream)
        eng.sync_status()
        leg = {"ms": ms, "pairs_per_s": eng.last_total / (ms * 1e-3)}
        if kind == "count":
            leg["equal_to_list_counts"] = bool(np.array_equal(
                out.cpu().numpy().astype(np.int64), np.diff(eng.first.cpu().numpy().astype(np.int64))))
        else:
            got = out.cpu().numpy()
            rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
            leg["max_rel_err_vs_oracle"] = float(rel.max())
            leg["bit_identical"] = bool(np.array_equal(got.view(np.int64), ref.view(np.int64)))
        res[kind] = leg
    # the first leg's figures stay at the top level as well
    res.update({k: res["inv_r6"][k] for k in ("ms", "pairs_per_s", "max_rel_err_vs_oracle", "bit_identical")})
    return res


def serving_requests(n_req, seed=7):
    """Requests drawn from the batched distribution, 5% replaced by large
    systems of 50k-200k atoms (density 0.05, cutoff 5 A, full pbc)."""
    import configs as cf

    systems = cf.batch_systems(n_req, seed=seed)
    rng = np.random.default_rng(seed + 1)
    for k in rng.choice(n_req, size=max(1, n_req // 20), replace=False):
        n = int(rng.uniform(50_000, 200_000))
        X, C, _ = cf.rand_config(n, DENSITY, seed=10_000 + int(k))
        systems[int(k)] = (X, C, CUTOFF, (True, True, True))
    return systems


def bench_serving(nl, dev, rates=(1_000, 5_000, 20_000, 50_000), n_req=1_500):
    """Poisson arrivals at each rate through the continuous-batching server
    (40 GB pair budget) and through plain per-request launches."""
    import torch

    # clients hand over pinned position buffers (copied to the device per request)
    systems = [(torch.from_numpy(x).pin_memory(), c, rc, p) for (x, c, rc, p) in serving_requests(n_req)]
    out = {"workload": f"{n_req} requests per rate: the batched distribution (4,096-system config) with 5% "
                       "large systems of 50k-200k atoms (density 0.05, rc 5 A); Poisson arrivals; 40 GB pair "
                       "budget; pinned request buffers; latency = arrival to results on the device, and for the "
                       "*_to_host modes arrival to results (first, i, j, S, R) copied into pinned host memory",
           "rates": {}}
    for mode in ("batched", "plain"):
        for host in (False, True):
            srv = nl.NeighbourListServer(device=dev, mode=mode, host_results=host)
            key = mode + ("_to_host" if host else "")
            # warm-up at the highest rate: the arenas grow to their working size once
            srv.run_trace(nl.poisson_trace(systems, rates[-1], seed=1))
            for rate in rates:
                srv.batches = srv.reruns = 0
                st = srv.run_trace(nl.poisson_trace(systems, rate, seed=int(rate)))
                out["rates"].setdefault(str(rate), {})[key] = {k: st[k] for k in (
                    "p50_ms", "p99_ms", "systems_per_s", "pairs_per_s", "batches", "reruns")}
            srv.close()
            del srv
            torch.cuda.empty_cache()
    top = out["rates"][str(rates[-1])]
    out["speedup_vs_plain_at_max_rate"] = top["batched"]["systems_per_s"] / top["plain"]["systems_per_s"]
    out["speedup_vs_plain_at_max_rate_to_host"] = (top["batched_to_host"]["systems_per_s"] /
                                                   top["plain_to_host"]["systems_per_s"])
    return out


def bench_half_and_verlet(nl, dev, stream, flush, steps):
    """The same 1M-atom system as a half list, and Verlet reuse at cutoff +
    skin 0.5 A: a reuse step (displacement test + R for the kept pairs)
    against a rebuild."""
    import torch

    X, C, pbc = workload()
    Xd = torch.from_numpy(X).to(dev)
    eng = nl.NeighbourListEngine(X.shape[0], C, CUTOFF, pbc, device=dev, half=True)
    total = eng.run(Xd)
    half_ms = timed_steps(lambda: eng.launch(Xd), steps, flush, stream)
    eng.sync_status()
    del eng
    skin = 0.5
    v = nl.VerletList(X.shape[0], C, CUTOFF, skin, pbc, device=dev)
    v.update(Xd)
    vpairs = v.engine.total_pairs()
    rng = np.random.default_rng(5)
    Xm = torch.from_numpy(X + rng.uniform(-0.05, 0.05, size=X.shape)).to(dev)
    reuse_ms = timed_steps(lambda: v.update(Xm), steps, flush, stream)
    rebuild_ms = timed_steps(lambda: v.engine.launch(Xm), steps, flush, stream)
    v.engine.sync_status()
    return {"half": {"workload": "1M-atom workload as a half list (j > i)", "pairs": int(total), "ms_per_step": half_ms,
                     "pairs_per_s": total / (half_ms * 1e-3)},
            "verlet": {"workload": f"1M-atom workload, list at cutoff + {skin} A skin, atoms moved by up to 0.05 A",
                       "pairs": int(vpairs), "reuse_ms": reuse_ms, "rebuild_ms": rebuild_ms,
                       "reuses": v.reuses, "rebuilds": v.rebuilds}}


def bench_float32_and_legacy(nl, dev, stream, flush, steps):
    """The 1M-atom workload with Float32 positions (the reference with
    T = Float32: build, count and fill with R in single precision), and the
    reference's legacy linked-list PairList (cell fix, legacy screen, j sort)
    timed as a whole synchronising call, as a user makes it."""
    import time

    import torch

    X, C, pbc = workload()
    X32 = torch.from_numpy(X.astype(np.float32)).to(dev)
    eng = nl.NeighbourListEngine(X.shape[0], C, CUTOFF, pbc, device=dev, dtype=torch.float32)
    total = eng.run(X32)
    f32_ms = timed_steps(lambda: eng.launch(X32), steps, flush, stream)
    eng.sync_status()
    del eng
    torch.cuda.empty_cache()
    Xd = torch.from_numpy(X).to(dev)
    lg = nl.legacy_pairlist(Xd, CUTOFF, C, pbc)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(steps):
        lg = nl.legacy_pairlist(Xd, CUTOFF, C, pbc)
    torch.cuda.synchronize(dev)
    legacy_ms = (time.perf_counter() - t0) / steps * 1e3
    return {"float32": {"workload": "1M-atom workload, Float32 positions, cell and cutoff", "pairs": int(total),
                        "ms_per_step": f32_ms, "pairs_per_s": total / (f32_ms * 1e-3)},
            "legacy": {"workload": "1M-atom workload, legacy linked-list PairList (fixcell = true)",
                       "pairs": int(lg.i.numel()), "ms_per_call": legacy_ms,
                       "timing": "host clock around the whole synchronising call (allocations included)"}}


def bench_4m(nl, dev, stream, flush, steps):
    import torch

    X, C, pbc = workload(4_000_000)
    Xd = torch.from_numpy(X).to(dev)
    eng = nl.NeighbourListEngine(X.shape[0], C, CUTOFF, pbc, device=dev)
    total = eng.run(Xd)
    ms = timed_steps(lambda: eng.launch(Xd), steps, flush, stream)
    eng.sync_status()
    return {"workload": "uniform 4,000,000 atoms, density 0.05, cubic pbc box, cutoff 5 A", "pairs": int(total),
            "ms_per_step": ms, "pairs_per_s": total / (ms * 1e-3), "rechecks": eng.rechecks()}


def measure_e2e(eng, X, Xd, total, stream, dev, args):
    """Same metric through the engine with HOST buffers (launch_host): pinned
    positions copied in, every output array (first, i, j, S, R) copied back
    on several copy streams, every step.  Two engines (own buffers) on two
    streams take the steps in turn, so one step's copies back overlap the
    next step's kernels; each step still moves its own inputs and outputs."""
    import torch

    from neighbourlists_gb300 import numa

    n_atoms = X.shape[0]
    ti = eng.ti
    node = numa.gpu_numa_node(dev)  # host buffers on the GPU's own NUMA node
    hX = numa.pinned_on_node((n_atoms, 3), torch.float64, node)
    hX.copy_(torch.from_numpy(X))

    def host_outputs():
        return {"first": numa.pinned_on_node(n_atoms + 1, ti, node),
                "i": numa.pinned_on_node(total, ti, node), "j": numa.pinned_on_node(total, ti, node),
                "S": numa.pinned_on_node((total, 3), ti, node),
                "R": numa.pinned_on_node((total, 3), torch.float64, node)}

    eng2 = type(eng)(n_atoms, eng.cell, eng.cutoff, tuple(bool(b) for b in eng.pbc), int_type=ti, device=dev,
                     capacity=eng.capacity)
    engines = [(eng, stream, host_outputs()), (eng2, torch.cuda.Stream(device=dev), host_outputs())]
    h_f, h_i, h_j, h_S, h_R = (engines[0][2][k] for k in ("first", "i", "j", "S", "R"))
    step_no = [0]

    def e2e_step():
        e, st, out = engines[step_no[0] % 2]
        e.launch_host(hX, out, stream=st)
        step_no[0] += 1

    e2e_step()
    e2e_step()
    torch.cuda.synchronize(dev)
    e2e_steps = max(2, args.steps)  # the same K steps as the device-side number
    es, ee = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    es.record(stream)
    engines[1][1].wait_stream(stream)
    for _ in range(e2e_steps):
        e2e_step()
    stream.wait_stream(engines[1][1])
    ee.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = es.elapsed_time(ee) / e2e_steps
    eng.sync_status()
    eng2.sync_status()
    assert int(h_f[-1]) - 1 == total
    assert int(engines[1][2]["first"][-1]) - 1 == total
    h2d = X.nbytes
    d2h = (h_i.numel() * h_i.element_size() + h_j.numel() * h_j.element_size() + h_S.numel() * h_S.element_size()
           + h_R.numel() * 8 + h_f.numel() * h_f.element_size())
    return {"value": None, "unit": "pairs/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": e2e_ms, "api": "NeighbourListEngine.launch_host, two engines taking steps in turn",
            "placement": {"gpu_numa_node": node, "output_R_pages_by_node": numa.page_nodes(h_R),
                          "d2h_gbs_by_host_node": d2h_by_node(dev, stream)}}


def d2h_bandwidth(dev, stream, host):
    """GB/s of one device-to-host copy of 1 GiB into a pinned buffer."""
    import torch

    src = torch.empty(host.numel(), dtype=torch.uint8, device=dev)
    host.copy_(src, non_blocking=True)
    torch.cuda.synchronize(dev)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(3):
        host.copy_(src, non_blocking=True)
    e.record(stream)
    torch.cuda.synchronize(dev)
    return 3 * host.numel() / (s.elapsed_time(e) * 1e-3) / 1e9


def d2h_by_node(dev, stream):
    """Device-to-host copy bandwidth into pinned memory placed on each NUMA
    node that has CPUs (the placement the end-to-end number depends on)."""
    import torch
    from neighbourlists_gb300 import numa

    out = {}
    for node in sorted(numa.cpu_nodes()):
        h = numa.pinned_on_node(1 << 30, torch.uint8, node)
        out[str(node)] = {"gbs": d2h_bandwidth(dev, stream, h), "pages_by_node": numa.page_nodes(h)}
        del h
    if not out:
        out["unknown"] = {"gbs": d2h_bandwidth(dev, stream, torch.empty(1 << 30, dtype=torch.uint8).pin_memory())}
    return out


def run_path(args):
    """Profiling runs of the Float32 and legacy paths on the benchmark's
    workload shape (``--atoms`` sets the size) and of the 4,096-system batch.
    Prints one JSON line that is not the benchmark line."""
    import time

    import torch

    import __graft_entry__ as graft

    nl = graft.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    X, C, pbc = workload(args.atoms)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    steps = max(args.steps, 1)
    if args.path == "batched":
        import configs as cf

        systems = cf.batch_systems(args.systems, seed=0)
        Xb = torch.from_numpy(np.ascontiguousarray(np.concatenate([x for (x, _, _, _) in systems]))).to(dev)
        b = nl.BatchNeighbourList([(x.shape[0], c, rc, p) for (x, c, rc, p) in systems], device=dev)
        total = b.run(Xb)
        for _ in range(args.warmup):
            b.launch(Xb)
        ms = timed_steps(lambda: b.launch(Xb), steps, flush, stream)
        b.sync_status()
        out = {"atoms": int(Xb.shape[0]), "pairs": int(total), "ms_per_batch": ms, "systems": len(systems),
               "timing": "CUDA events, default launch shapes, no graph, L2 flushed before every batch"}
    elif args.path == "lazy":
        Xd = torch.from_numpy(X).to(dev)
        eng = nl.NeighbourListEngine(X.shape[0], C, CUTOFF, pbc, device=dev)
        total = eng.run(Xd)
        clist = eng.cell_list(Xd)
        out = {"pairs": int(total)}
        for kind in ("inv_r6_fast", "count", "inv_r6"):
            res = nl.lazy_reduce(clist, kind)
            for _ in range(args.warmup):
                nl.lazy_reduce(clist, kind, out=res, sync=False)
            out[kind + "_ms"] = timed_steps(lambda: nl.lazy_reduce(clist, kind, out=res, sync=False), steps, flush,
                                            stream)
            eng.sync_status()
        out["timing"] = "CUDA events, L2 flushed before every call"
    elif args.path == "float32":
        X32 = torch.from_numpy(X.astype(np.float32)).to(dev)
        eng = nl.NeighbourListEngine(X.shape[0], C, CUTOFF, pbc, device=dev, dtype=torch.float32)
        total = eng.run(X32)
        for _ in range(args.warmup):
            eng.launch(X32)
        ms = timed_steps(lambda: eng.launch(X32), steps, flush, stream)
        eng.sync_status()
        out = {"pairs": int(total), "ms_per_step": ms, "timing": "CUDA events, L2 flushed before every step"}
    else:
        Xd = torch.from_numpy(X).to(dev)
        for _ in range(args.warmup):
            nl.legacy_pairlist(Xd, CUTOFF, C, pbc)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(steps):
            lg = nl.legacy_pairlist(Xd, CUTOFF, C, pbc)
        torch.cuda.synchronize(dev)
        out = {"pairs": int(lg.i.numel()), "ms_per_call": (time.perf_counter() - t0) / steps * 1e3,
               "timing": "host clock around the whole synchronising call"}
    print(json.dumps({"metric": "profiling run (not the benchmark line)", "path": args.path,
                      **{"atoms": args.atoms, **out}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the lazy / batched / 4M sections")
    ap.add_argument("--atoms", type=int, default=N_ATOMS, help="system size (profiling runs use a smaller one)")
    ap.add_argument("--systems", type=int, default=4096, help="batched profiling runs: systems in the batch")
    ap.add_argument("--path", default="headline", choices=["headline", "float32", "legacy", "batched", "lazy"],
                    help="float32 / legacy / batched / lazy: profiling runs of those paths (not the benchmark line)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.path != "headline":
        run_path(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
