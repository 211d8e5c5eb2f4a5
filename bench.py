"""Benchmark: full k-truss decomposition of R-MAT scale 20 (edge factor 16) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload rmat20]

One step = one decomposition (device CSR build from the COO entries, support count, peeling,
per-entry truss numbers) of the whole graph.  Prints one JSON line.

  value       edges/s = m / t_step with the COO input already in HBM (engine API, device buffers)
  e2e         edges/s through the host-buffer C ABI call kt_decompose: the pinned input entries
              are copied host->device and the per-entry truss numbers device->host every step
  roofline    the dominant kernel, the persistent peel (one launch per decomposition): algorithmic
              bytes per launch = the bytes of the reference's full-recount schedule for the
              passes that launch covers, sum over passes p of 4(n+1) + 12 E+_p (row pointers,
              column array, support written and read once per pass), over the kernel's CUDA-event
              time, against the measured HBM copy bandwidth; the support-count kernel's figure
              (4(n+1) + 12m per launch) is reported beside it
  cpu_baseline  the reference algorithm (oracle port of its CPU path: chained count-and-prune
              passes over k) timed on a bounded sample of passes on one host core, scaled to the
              whole decomposition by the workload's exact pass volume (sum of alive edges over
              all passes of the reference schedule)

--impl reference times only that CPU port (building the reference's own executable needs its
sources, which this package does not ship) and prints the same line with impl "reference".
Under torchrun, each rank decomposes its own replica (the single-graph path does not shard).
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
sys.path.insert(0, os.path.join(ROOT, "ktruss-explorer_gb300"))

WORKLOADS = {
    # R-MAT scale 20, edge factor 16, (a,b,c,d) = (0.57,0.19,0.19,0.05), symmetrized, deduplicated,
    # self loops removed; seed 1
    "rmat20": dict(scale=20, ef=16, a=0.57, b=0.19, c=0.19, seed=1),
    "rmat22": dict(scale=22, ef=16, a=0.57, b=0.19, c=0.19, seed=1),
    "rmat21": dict(scale=21, ef=16, a=0.57, b=0.19, c=0.19, seed=1),
    "rmat18": dict(scale=18, ef=16, a=0.57, b=0.19, c=0.19, seed=1),
    "rmat16": dict(scale=16, ef=16, a=0.57, b=0.19, c=0.19, seed=1),
    # stress: R-MAT scale 24, edge factor 32, same (a,b,c,d), plus 16 planted cliques of 64-512
    # random vertices (deep peeling, k_max >= 64)
    "rmat24": dict(scale=24, ef=32, a=0.57, b=0.19, c=0.19, seed=1, cliques=(16, 64, 512)),
}

# Batched workloads: num_graphs graphs, sizes log-uniform in [n_min, n_max], half Barabasi-Albert
# (m in {2,4,8,16}), half Watts-Strogatz (k in {6,10,20}, p = 0.1), each with 0-3 planted cliques
# of 8-64 vertices; all decomposed in one call.
BATCHES = {
    "batch4096": dict(num_graphs=4096, n_min=500, n_max=50000, seed=1),
    "batch256": dict(num_graphs=256, n_min=500, n_max=50000, seed=1),
}
# The autotuner times its candidate schedules on a separate sample of the same distribution
# (other seed), never on the graphs that are measured.
TUNE_SAMPLE = dict(num_graphs=256, seed=1001)

# Exact pass volume of the reference schedule for each workload (number of count-and-prune
# passes of the chained single-k runs and the sum of their alive oriented edges).  The engine
# recomputes both every run and bench.py checks them; the reference arm needs them to scale its
# bounded sample to the whole decomposition.
PASS_VOLUME = {"rmat20": {"plain_passes": 2470, "plain_alive_sum": 7079259210}}

FALLBACK_HBM_GBS = 6800.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def make_graph(name):
    import ktruss_gb300 as kt

    w = WORKLOADS[name]
    n, u, v = kt.gen_rmat(w["scale"], w["ef"], w["a"], w["b"], w["c"], w["seed"])
    if "cliques" in w:
        count, lo, hi = w["cliques"]
        n, u, v = kt.plant_cliques(n, u, v, count, lo, hi, w["seed"] + 7)
    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    return n, len(u), src, dst


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, td=None, device="cpu") -> float:
    """The slowest rank's value (the job time of N independent replicas); `td` is
    torch.distributed when the process group is initialised, else the value is returned."""
    if td is None or not td.is_initialized() or td.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def shard_seed(seed: int, rank: int) -> int:
    """Seed of rank `rank`'s shard of a batch workload (rank 0 keeps the workload's own seed)."""
    return seed + 7919 * rank


def replica_throughput(m: int, world: int, ms: float) -> float:
    """Edges per second of `world` replicas that each decomposed m edges in at most `ms`."""
    return m * world / (ms * 1e-3)


def cpu_sample(n, src, dst, budget_s, pass_volume):
    """Times the oracle port of the reference's CPU algorithm on a bounded prefix of its passes."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    s = oracle.chain_sample(n, src, dst, budget_s)
    rate = s["alive_sum"] / s["seconds"]  # alive oriented edges processed per second
    return s, rate


def run_reference(args, world, rank):
    if rank != 0:
        return
    if args.workload not in WORKLOADS:
        print(json.dumps({"impl": "reference", "unavailable": "the reference CPU arm is timed on the single-graph "
                                                              "workloads (the reference has no batch or selector)"}))
        return
    n, m, src, dst = make_graph(args.workload)
    vol = PASS_VOLUME.get(args.workload)
    # untimed warm-up on a small graph (the sample's first pass alone is the full-graph count)
    nw, mw, sw, dw = make_graph("rmat16")
    for _ in range(args.warmup):
        cpu_sample(nw, sw, dw, 0.0, None)
    budget = max(1.0, 60.0 / max(1, args.steps))
    rates, samples = [], []
    t0 = time.time()
    for _ in range(args.steps):
        s, rate = cpu_sample(n, src, dst, budget, vol)
        rates.append(rate)
        samples.append(s)
    wall = time.time() - t0
    rate = statistics.median(rates)
    if vol:
        t_full = vol["plain_alive_sum"] / rate
        value = m / t_full
        unit = "edges/s"
        desc = (f"the start of the reference's chained decomposition: {samples[0]['passes']} complete of "
                f"{vol['plain_passes']} count-and-prune passes plus the edges a cut pass had counted "
                f"({samples[0]['alive_sum']} of {vol['plain_alive_sum']} alive-edge visits, graph set-up "
                f"included), {samples[0]['seconds']:.1f} s per step; scaled by alive-edge volume")
    else:
        value, unit, t_full = rate, "alive-edge-visits/s", None
        desc = "first passes of the chained decomposition (pass volume unknown: not scaled)"
    line = {"metric": "k-truss decomposition edges/s", "value": value, "unit": unit, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": (t_full * 1e3) if t_full else None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"{args.workload} full truss decomposition", "m": m, "n": n},
            "cpu_baseline": {"value": value, "unit": unit, "cores": 1, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line), flush=True)


def parse_schedule(text):
    """'default', 'auto', 'learned' or 'G,W,C,R[,B]' (support group, chunk width, compaction
    percent, recount percent, peel blocks per SM; B defaults to 0 = by L2 fit)."""
    if text in ("default", "auto", "learned"):
        return text
    vals = [int(x) for x in text.split(",")]
    return tuple(vals + [0] * (5 - len(vals)))


def train_selector(kt):
    """The learned selector, trained by the library's CUDA kernels on the GB300 timing data."""
    sys.path.insert(0, os.path.join(ROOT, "ktruss-explorer_gb300"))
    import selector

    t0 = time.perf_counter()
    data = selector.load_training()
    sel, losses = selector.train(data)
    return sel, {"training_s": time.perf_counter() - t0, "training_graphs": int(len(data["times"])),
                 "loss_first_last": [float(losses[0]), float(losses[-1])]}


def choose_schedule(args, eng, kt, sample, target):
    """Sets the engine's schedule (and the host-buffer engine's) from --schedule; 'auto' runs the
    autotuner on `sample()` = (n, src, dst) device tensors of other graphs of the same
    distribution; 'learned' trains the selector and applies it to the features of `target()`, the
    measured graph.  Returns the config record."""
    import torch

    choice = parse_schedule(args.schedule)
    rec = {"mode": args.schedule if isinstance(choice, str) else "fixed"}
    if choice == "learned":
        sel, info = train_selector(kt)
        rec.update(info)
        n, d_src, d_dst = target()
        torch.cuda.synchronize()
        feats = eng.features(d_src.data_ptr(), d_dst.data_ptr(), d_src.numel(), n)
        choice = sel.predict(feats)[0].as_tuple()
        sel.close()
    if choice == "auto":
        n, d_src, d_dst = sample()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        best, table = eng.autotune(d_src.data_ptr(), d_dst.data_ptr(), d_src.numel(), n)
        rec["tuning_s"] = time.perf_counter() - t0
        rec["candidates"] = len(table)
        rec["default_ms"] = next(ms for s, ms in table if s.as_tuple() == kt.schedule_default().as_tuple())
        rec["best_ms"] = min(ms for _, ms in table)
        choice = best.as_tuple()
    elif choice == "default":
        choice = kt.schedule_default().as_tuple()
    eng.set_schedule(*choice)
    kt.set_schedule(*choice)
    (rec["support_group"], rec["chunk_width"], rec["compact_percent"], rec["recount_percent"],
     rec["peel_blocks"]) = choice
    return rec


def run_batch(args, world, rank, local):
    """graphs/s of the batched decomposition (device buffers; e2e through kt_decompose_batch)."""
    import torch

    import ktruss_gb300 as kt

    dist = world > 1
    if dist:
        import torch.distributed as td

        td.init_process_group("nccl")
    else:
        td = None
    torch.cuda.set_device(local)
    b = BATCHES[args.workload]
    t0 = time.time()
    # under torchrun each rank takes its own shard of num_graphs * world graphs (its own seed): the
    # graphs are independent units, so the shards need no exchange (weak scaling)
    n, u, v, off = kt.gen_batch(b["num_graphs"], b["n_min"], b["n_max"], shard_seed(b["seed"], rank))
    gen_s = time.time() - t0
    G = b["num_graphs"]
    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    N, m = len(src), len(u)
    eng = kt.Engine(local)
    eng.reserve(n, N)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
    d_src, d_dst, d_off = dev(src), dev(dst), dev(off)
    d_out = torch.empty(N, dtype=torch.int32, device="cuda")
    d_k = torch.empty(G, dtype=torch.int32, device="cuda")
    stream = torch.cuda.ExternalStream(eng.stream)

    def tune_sample():
        ns, us, vs, _ = kt.gen_batch(TUNE_SAMPLE["num_graphs"], b["n_min"], b["n_max"], TUNE_SAMPLE["seed"])
        return ns, dev(np.concatenate([us, vs])), dev(np.concatenate([vs, us]))

    sched = choose_schedule(args, eng, kt, tune_sample, lambda: (n, d_src, d_dst))
    torch.cuda.synchronize()

    def step():
        eng.decompose_batch(d_src.data_ptr(), d_dst.data_ptr(), N, n, d_off.data_ptr(), G, d_out.data_ptr(),
                            d_k.data_ptr(), sync=False)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = eng.stats().kernel_launches
    if dist:
        td.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, td, "cuda")
    st = eng.stats()
    launches = st.kernel_launches - launches0
    kmax = d_k.cpu().numpy()
    h_src = torch.from_numpy(src.view(np.int32)).pin_memory().numpy().view(np.uint32)
    h_dst = torch.from_numpy(dst.view(np.int32)).pin_memory().numpy().view(np.uint32)
    h_out = torch.empty(N, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    kt.decompose_batch(h_src, h_dst, n, off, out=h_out)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        _, k2 = kt.decompose_batch(h_src, h_dst, n, off, out=h_out)
    e2e_s = max_over_ranks((time.perf_counter() - t1) / args.steps, td, "cuda")
    ls = kt.last_stats()
    if not np.array_equal(k2, kmax.view(np.uint32)):
        raise RuntimeError("host-buffer and device-buffer batches differ")
    single = single_graph_path(kt, torch, eng, n, u, v, off, kmax.view(np.uint32), args.single_graphs)
    line = {"metric": "batched k-truss decomposition graphs/s", "value": G * world / (ms * 1e-3),
            "unit": "graphs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": f"{args.workload}: {G} graphs, n log-uniform in [{b['n_min']}, {b['n_max']}], "
                                   "half Barabasi-Albert, half Watts-Strogatz, 0-3 planted cliques each, "
                                   "one call", "n": n, "m": m, "edges_per_s": m * world / (ms * 1e-3),
                       "k_max_max": int(kmax.max()), "peel_rounds": st.num_rounds, "peel_levels": st.num_levels,
                       "phase_ms": {"build": st.build_ms, "support": st.support_ms, "peel": st.peel_ms},
                       "generation_s": gen_s,
                       "parallelism": f"graph shards x{world}" if world > 1 else "one GPU", "schedule": sched,
                       "single_graph_path": single,
                       "l2": "input entries 2x4x2m bytes > L2 (129 MB)"},
            "e2e": {"value": G * world / e2e_s, "unit": "graphs/s", "h2d_bytes_per_step": 8 * N + 4 * (G + 1),
                    "d2h_bytes_per_step": 4 * N + 4 * G, "ms_per_step": e2e_s * 1e3,
                    "last_call_device_ms": {"copy_in": ls.copy_in_ms, "decompose": ls.last_ms,
                                            "copy_out_and_kmax": ls.copy_out_ms}},
            "gpu_launches": launches, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        td.destroy_process_group()


def single_graph_path(kt, torch, eng, n, u, v, off, kmax, count):
    """The plain path on the same graphs: the first `count` graphs of the batch decomposed one call
    each (device buffers, default schedule, calls back to back), as graphs/s."""
    G = min(count, len(off) - 1)
    if G <= 0:
        return None
    lo = np.searchsorted(u, off[:G], side="left")
    hi = np.searchsorted(u, off[1:G + 1], side="left")
    parts_s, parts_d, spans = [], [], []
    pos = 0
    for g in range(G):
        ug, vg = u[lo[g]:hi[g]] - off[g], v[lo[g]:hi[g]] - off[g]
        parts_s += [ug, vg]
        parts_d += [vg, ug]
        spans.append((pos, 2 * len(ug), int(off[g + 1] - off[g])))
        pos += 2 * len(ug)
    dev = lambda a: torch.from_numpy(np.concatenate(a).astype(np.uint32).view(np.int32)).cuda()
    d_s, d_d = dev(parts_s), dev(parts_d)
    d_out = torch.empty(max(pos, 1), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(G, dtype=torch.int32, device="cuda")
    saved = eng.schedule().as_tuple()
    eng.set_schedule(*kt.schedule_default().as_tuple())
    torch.cuda.synchronize()

    def one_pass():
        for g, (p0, N, ng) in enumerate(spans):
            eng.decompose(d_s.data_ptr() + 4 * p0, d_d.data_ptr() + 4 * p0, N, ng, d_out.data_ptr() + 4 * p0,
                          d_k.data_ptr() + 4 * g, sync=False)
        torch.cuda.synchronize()

    one_pass()
    t0 = time.perf_counter()
    one_pass()
    secs = time.perf_counter() - t0
    if not np.array_equal(d_k.cpu().numpy().view(np.uint32), kmax[:G]):
        raise RuntimeError("single-graph calls and the batch disagree on k_max")
    eng.set_schedule(*saved)
    return {"graphs": G, "graphs_per_s": G / secs, "seconds": secs, "calls": G,
            "note": "one kt_engine_decompose call per graph, default schedule, wall time of back-to-back calls"}


def run_selector(args, world, rank, local):
    """Learned selector on the 200 held-out graphs, live on this GPU: per graph, the support+peel
    device time with the network's schedule against exhaustive autotuning of the same graph
    (best of the 36 schedules) and the default schedule."""
    import torch

    import ktruss_gb300 as kt

    if rank != 0:
        return
    torch.cuda.set_device(local)
    sys.path.insert(0, os.path.join(ROOT, "ktruss-explorer_gb300"))
    import selector

    held = selector.load(os.path.join(selector.DATA, "selector_heldout.npz"))
    sel, info = train_selector(kt)
    eng = kt.Engine(local)
    eng.set_selector(sel)
    graphs = []
    for spec in held["specs"]:
        n, u, v = selector.make_graph(json.loads(str(spec)))
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
        graphs.append((n, len(u), dev(np.concatenate([u, v])), dev(np.concatenate([v, u]))))
    torch.cuda.synchronize()
    grid = kt.schedule_grid()
    d_idx = kt.schedule_index(kt.schedule_default())
    tuned = np.zeros(len(graphs))
    default = np.zeros(len(graphs))
    for i, (n, m, s_, d_) in enumerate(graphs):
        eng.set_selector(None)
        _, table = eng.autotune(s_.data_ptr(), d_.data_ptr(), s_.numel(), n, candidates=grid, repeats=args.steps)
        ms = np.array([t for _, t in table])
        tuned[i], default[i] = ms.min(), ms[d_idx]
    eng.set_selector(sel)
    out = torch.empty(max(s_.numel() for _, _, s_, _ in graphs), dtype=torch.int32, device="cuda")
    kk = torch.zeros(1, dtype=torch.int32, device="cuda")
    learned = np.full(len(graphs), np.inf)
    for _ in range(args.warmup):
        for n, m, s_, d_ in graphs:
            eng.decompose(s_.data_ptr(), d_.data_ptr(), s_.numel(), n, out.data_ptr(), kk.data_ptr())
    for _ in range(args.steps):
        for i, (n, m, s_, d_) in enumerate(graphs):
            eng.decompose(s_.data_ptr(), d_.data_ptr(), s_.numel(), n, out.data_ptr(), kk.data_ptr())
            st = eng.stats()
            learned[i] = min(learned[i], st.select_ms + st.support_ms + st.peel_ms)
    ratio = learned.sum() / tuned.sum()
    line = {"metric": "learned-selector time / exhaustively tuned time", "value": ratio, "unit": "ratio",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": learned.sum(),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32 network, u32 peel",
            "data": "synthetic",
            "config": {"workload": "200 held-out graphs (Erdos-Renyi, R-MAT 12-18, Barabasi-Albert, random "
                                   "geometric, planted cliques), support count + peel device time, best of "
                                   f"{args.steps} runs per graph (the learned time includes the selector's "
                                   "features, inference and read-back); selector trained on 2000 other graphs' "
                                   "GB300 timings", "learned_ms": learned.sum(), "tuned_ms": tuned.sum(),
                       "default_ms": default.sum(), "default_over_tuned": default.sum() / tuned.sum(),
                       "gain_vs_default": default.sum() / learned.sum(), "tuning_runs": 36 * args.steps, **info}}
    print(json.dumps(line), flush=True)
    eng.close()


def run_ingest(args, world, rank, local):
    """Device-side TSV ingest: the R-MAT 20 graph as a 'dst src x' text file, parsed on the GPU
    (text already in HBM: value; from the file through pinned staging: e2e) against the host
    reader (cpu_baseline)."""
    import tempfile

    import torch

    import ktruss_gb300 as kt

    if rank != 0:
        return
    torch.cuda.set_device(local)
    n, m, src, dst = make_graph("rmat20")
    N = len(src)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "rmat20.tsv")
        kt.write_coo_graph_to_file(kt.COOGraph(n, src, dst), path)
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        h = kt.create_coo_from_file(path)
        host_s = time.perf_counter() - t0
        eng = kt.Engine(local)
        with open(path, "rb") as f:
            text = torch.frombuffer(bytearray(f.read()), dtype=torch.uint8).cuda()
        d_src = torch.empty(N, dtype=torch.int32, device="cuda")
        d_dst = torch.empty(N, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        stream = torch.cuda.ExternalStream(eng.stream)
        for _ in range(args.warmup):
            eng.parse_tsv(text.data_ptr(), size, d_src.data_ptr(), d_dst.data_ptr(), N)
        launches0 = eng.stats().kernel_launches
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            ev0.record(stream)
            for _ in range(args.steps):
                ne, nv = eng.parse_tsv(text.data_ptr(), size, d_src.data_ptr(), d_dst.data_ptr(), N)
            ev1.record(stream)
            torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
        launches = eng.stats().kernel_launches - launches0
        if ne != N or nv != h.num_nodes or not np.array_equal(d_src.cpu().numpy().view(np.uint32), h.src_idx):
            raise RuntimeError("device and host readers differ")
        t0 = time.perf_counter()
        for _ in range(args.steps):
            eng.read_tsv(path, d_src.data_ptr(), d_dst.data_ptr(), N)
        e2e_s = (time.perf_counter() - t0) / args.steps
        eng.close()
    hbm, hbm_kind = peaks()
    alg = 2 * size + 8 * N  # text read by both passes, entries written once
    gbs = alg / (ms * 1e-3) / 1e9
    line = {"metric": "TSV ingest GB/s of text", "value": size / (ms * 1e-3) / 1e9, "unit": "GB/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8 text, u32 entries", "data": "synthetic",
            "config": {"workload": f"R-MAT 20 as a 'dst src x' TSV file ({size} bytes, {N} entries), parsed into "
                                   "device entries", "bytes": size, "entries": N,
                       "l2": "text larger than L2 (129 MB)"},
            "e2e": {"value": size / e2e_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": size, "d2h_bytes_per_step": 0,
                    "note": "file (page cache) -> pinned staging -> device -> parse, wall time"},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": "k_tsv_count + k_tsv_parse + k_tsv_finish", "achieved": gbs,
                         "peak": hbm, "peak_kind": hbm_kind, "unit": "GB/s", "frac": gbs / hbm, "traffic": None,
                         "algorithmic_bytes": alg},
            "cpu_baseline": {"value": size / host_s / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                             "sample": "the whole file through kt_read_tsv (the host restatement of "
                                       "createCOOFromFile), once"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch

    import ktruss_gb300 as kt

    dist = world > 1
    if dist:
        import torch.distributed as td

        td.init_process_group("nccl")
    torch.cuda.set_device(local)
    n, m, src, dst = make_graph(args.workload)
    N = len(src)
    eng = kt.Engine(local)
    eng.reserve(n, N)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_out = torch.empty(N, dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.ExternalStream(eng.stream)

    def tune_sample():
        w = WORKLOADS[args.workload]
        ns, us, vs = kt.gen_rmat(w["scale"] - 2, w["ef"], w["a"], w["b"], w["c"], w["seed"] + 1000)
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
        return ns, dev(np.concatenate([us, vs])), dev(np.concatenate([vs, us]))

    sched = choose_schedule(args, eng, kt, tune_sample, lambda: (n, d_src, d_dst))
    torch.cuda.synchronize()  # the engine stream does not order after torch's copies

    def step():
        eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), N, n, d_out.data_ptr(), d_k.data_ptr(), sync=False)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    st = eng.stats()
    launches0 = st.kernel_launches
    if dist:
        td.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    support_ms, build_ms, peel_ms, peel_kernel_ms = [], [], [], []
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
            s = eng.stats()
            support_ms.append(s.support_ms)
            build_ms.append(s.build_ms)
            peel_ms.append(s.peel_ms)
            peel_kernel_ms.append(s.peel_kernel_ms)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    st = eng.stats()
    launches = st.kernel_launches - launches0
    if dist:
        ms = max_over_ranks(ms, td, "cuda")
    k_max = int(d_k.item())

    # the same steps as repeat runs on unchanged input: the CUDA graph of the whole device
    # pipeline (kt_engine_replay), captured at the first replay
    ref_out = d_out.clone()
    eng.replay(sync=False)
    torch.cuda.synchronize()
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev2.record(stream)
    for _ in range(args.steps):
        eng.replay(sync=False)
    ev3.record(stream)
    torch.cuda.synchronize()
    replay_ms = ev2.elapsed_time(ev3) / args.steps
    try:
        replay_mode = eng.replay_mode()
    except Exception as exc:  # informational only
        replay_mode = f"unknown ({exc})"
    if not torch.equal(d_out, ref_out):
        raise RuntimeError("replayed decomposition differs")

    # end to end through the host-buffer C ABI (pinned host memory)
    h_src = torch.from_numpy(src.view(np.int32)).pin_memory()
    h_dst = torch.from_numpy(dst.view(np.int32)).pin_memory()
    h_out = torch.empty(N, dtype=torch.int32).pin_memory()
    g = kt.COOGraph(n, h_src.numpy().view(np.uint32), h_dst.numpy().view(np.uint32))
    out_np = h_out.numpy().view(np.uint32)
    kt.decompose(g, out=out_np)
    if dist:
        td.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, k2 = kt.decompose(g, out=out_np)
    e2e_s = (time.perf_counter() - t0) / args.steps
    ls = kt.last_stats()
    if dist:
        e2e_s = max_over_ranks(e2e_s, td, "cuda")
    assert k2 == k_max
    if not np.array_equal(out_np, d_out.cpu().numpy().view(np.uint32)):
        raise RuntimeError("host-buffer and device-buffer decompositions differ")

    hbm, hbm_kind = peaks()
    traffic = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(args.workload, {})
    except Exception:
        pass
    sup_ms = statistics.mean(support_ms)
    sup_bytes = 4 * (n + 1) + 12 * m
    sup_gbs = sup_bytes / (sup_ms * 1e-3) / 1e9
    pk_ms = statistics.mean(peel_kernel_ms)
    plain_bytes = 4 * (n + 1) * st.plain_passes + 12 * st.plain_alive_sum
    pk_gbs = plain_bytes / (pk_ms * 1e-3) / 1e9
    vol = PASS_VOLUME.get(args.workload)
    if vol and (vol["plain_passes"] != st.plain_passes or vol["plain_alive_sum"] != st.plain_alive_sum):
        raise RuntimeError(f"pass volume changed: {st.plain_passes}/{st.plain_alive_sum} vs {vol}")
    line = {"metric": "k-truss decomposition edges/s", "value": replica_throughput(m, world, ms), "unit": "edges/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": f"{args.workload} full truss decomposition", "n": n, "m": m, "k_max": k_max,
                       "triangles": st.triangles, "peel_rounds": st.num_rounds, "peel_levels": st.num_levels,
                       "parallelism": f"replicas{world}", "l2": "input entries 2x4x2m bytes > L2 (129 MB)",
                       "phase_ms": {"build": statistics.mean(build_ms), "support": sup_ms,
                                    "peel": statistics.mean(peel_ms)},
                       "peel_phase_ms": st.as_dict()["peel_phase_ms"], "compactions": st.compactions,
                       "walk_entries": st.walk_entries,
                       "replay": {"ms_per_step": replay_ms, "mode": replay_mode,
                                  "how": "kt_engine_replay: the same steps through a CUDA graph of the device "
                                         "pipeline (repeat runs on unchanged input, no host-side input checks)"},
                       "schedule": sched},
            "e2e": {"value": replica_throughput(m, world, e2e_s * 1e3), "unit": "edges/s", "h2d_bytes_per_step": 8 * N,
                    "d2h_bytes_per_step": 4 * N, "ms_per_step": e2e_s * 1e3,
                    "last_call_device_ms": {"copy_in": ls.copy_in_ms, "decompose": ls.last_ms,
                                            "copy_out": ls.copy_out_ms}},
            "gpu_launches": launches // args.steps * args.steps,
            "roofline": {"bound": "hbm", "kernel": "k_peel", "achieved": pk_gbs, "peak": hbm,
                         "peak_kind": hbm_kind, "unit": "GB/s", "frac": pk_gbs / hbm,
                         "traffic": traffic.get("k_peel"), "algorithmic_bytes": plain_bytes,
                         "kernel_ms": pk_ms, "passes": st.plain_passes, "alive_sum": st.plain_alive_sum},
            "roofline_support": {"bound": "hbm", "kernel": "k_support", "achieved": sup_gbs, "peak": hbm,
                                 "unit": "GB/s", "frac": sup_gbs / hbm, "traffic": traffic.get("k_support"),
                                 "algorithmic_bytes": sup_bytes, "kernel_ms": sup_ms},
            "clocks": clk.summary()}
    if rank == 0 and world == 1 and not args.no_cpu:
        s, rate = cpu_sample(n, src, dst, args.cpu_budget, None)
    else:
        rate = None
    if rate == 0:
        line["cpu_baseline"] = {"value": None, "unit": "edges/s", "cores": 1, "kind": "port",
                                "sample": f"no triangle count of the reference's first pass finished its first "
                                          f"4096 edges within {args.cpu_budget:.0f} s (graph set-up included)"}
    elif rate:
        t_full = st.plain_alive_sum / rate
        line["cpu_baseline"] = {"value": m / t_full, "unit": "edges/s", "cores": 1, "kind": "port",
                                "sample": (f"first {s['passes']} complete of {st.plain_passes} count-and-prune "
                                           f"passes of the reference's chained decomposition ({s['alive_sum']} of "
                                           f"{st.plain_alive_sum} alive-edge visits, a cut pass's merged edges "
                                           f"included) in {s['seconds']:.1f} s with graph set-up, scaled by "
                                           f"alive-edge volume")}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        td.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="rmat20",
                    choices=sorted(WORKLOADS) + sorted(BATCHES) + ["selector", "ingest"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--single-graphs", type=int, default=4096,
                    help="batch workloads: graphs of the batch also decomposed one call each")
    ap.add_argument("--schedule", default=None,
                    help="kernel schedule: default, auto (autotune on a separate sample of the same "
                         "distribution), learned (the selector trained on the GB300 timing data) or G,W,C,R; "
                         "default: auto for batches, default for single graphs")
    args = ap.parse_args()
    if args.schedule is None:
        args.schedule = "auto" if args.workload in BATCHES else "default"
    parse_schedule(args.schedule)
    world, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "selector":
        run_selector(args, world, rank, local)
    elif args.workload == "ingest":
        run_ingest(args, world, rank, local)
    elif args.workload in BATCHES:
        run_batch(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
