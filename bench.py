"""Benchmark: k-truss on R-MAT scale 20 (edge factor 16, seed 1) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload rmat20]

Prints one JSON line.  Both arms print the same `metric` ("k-truss edges/s") and `config` (the
graph); `work` says what one step computes.

ours (one step = one full truss decomposition: device CSR build from the COO entries, support
count, peeling of every level, per-entry truss numbers)
  value       edges/s = m / t_step with the COO input already in HBM (engine API, device buffers)
  e2e         the same through the host-buffer C ABI call kt_decompose: the pinned input entries
              are copied host->device and the per-entry truss numbers device->host every step
  roofline    the dominant kernel, the persistent peel (one launch per decomposition): algorithmic
              bytes per launch = the bytes of the reference's full-recount schedule for the
              passes that launch covers, sum over passes p of 4(n+1) + 12 E+_p (row pointers,
              column array, support written and read once per pass), with the pass counts taken
              from the oracle fixture (tests/golden/rmat20_seed1.json), over the kernel's
              CUDA-event time, against the measured HBM copy bandwidth; the support-count
              kernel's figure (4(n+1) + 12m per launch) is reported beside it
  single_k3   the reference's own unit of work on the same graph - one single-k run at k = 3 -
              through kt_engine_ktruss, for a like-for-like comparison with the reference arm
  cpu_baseline  that unit on the host cores: the oracle port of the reference loop
              (kernel_hdc.cu:107-201, count and mark sweeps split over all host threads), complete
              runs timed like the reference's k-truss timer

reference (--impl reference; one step = one complete single-k run at k = 3 on the whole graph,
the span the reference's k-truss timer measures, kernel_hdc.cu:213-229): the oracle port of the
reference's CPU loop on all host threads, after W warm-up runs, as the reference's -w/-x repeat
runs.  The graph comes from the oracle's own generator; the product library is not loaded.  A
complete CPU decomposition of this graph takes hours (a stratified estimate is made by
--decomposition-estimate and recorded separately, never as `value`).
Under torchrun, each rank decomposes its own replica (the single-graph path does not shard).
"""
from __future__ import annotations

import argparse
import gc
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

# Oracle fixtures of the single-graph workloads (tests/golden/make_headline_fixture.py and
# make_stress_fixture.py): truss-number
# hash and histogram, k_max, and the pass statistics of the reference schedule (per level k the
# count-and-prune passes and their alive oriented edges).  The roofline's algorithmic bytes come
# from these, and every run is checked against them.
FIXTURES = {"rmat20": os.path.join(ROOT, "tests", "golden", "rmat20_seed1.json"),
            "rmat24": os.path.join(ROOT, "tests", "golden", "rmat24_seed1.json")}


def fixture(name):
    path = FIXTURES.get(name)
    if not path or not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def workload_config(name, n, m):
    """The `config` both arms print for a single-graph workload (the graph, not the method)."""
    w = WORKLOADS[name]
    desc = (f"{name}: R-MAT scale {w['scale']}, edge factor {w['ef']}, (a,b,c,d) = ({w['a']},{w['b']},{w['c']},"
            f"{round(1 - w['a'] - w['b'] - w['c'], 2)}), seed {w['seed']}, symmetrized, deduplicated, self loops "
            "removed")
    if "cliques" in w:
        desc += f", {w['cliques'][0]} planted cliques of {w['cliques'][1]}-{w['cliques'][2]} vertices"
    return {"workload": desc, "n": n, "m": m, "l2": "input entries 2x4x2m bytes > L2 (129 MB)"}


FALLBACK_HBM_GBS = 6800.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def make_graph(name, with_oracle=False):
    """(n, m, src, dst) of a single-graph workload; with_oracle: made by the oracle's generator
    (the same graph, without loading the product library)."""
    w = WORKLOADS[name]
    if with_oracle:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        if "cliques" in w:
            raise ValueError(f"{name}: the oracle has no clique planter")
        n, u, v = oracle.gen_rmat(w["scale"], w["ef"], w["a"], w["b"], w["c"], w["seed"])
    else:
        import ktruss_gb300 as kt

        n, u, v = kt.gen_rmat(w["scale"], w["ef"], w["a"], w["b"], w["c"], w["seed"])
        if "cliques" in w:
            count, lo, hi = w["cliques"]
            n, u, v = kt.plant_cliques(n, u, v, count, lo, hi, w["seed"] + 7)
    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    return n, len(u), src, dst


def load_er4096():
    """The Erdos-Renyi G(4096, 16/4095) graph of the golden fixtures (the plain method's small
    configuration): (n, src, dst, truss per edge, k_max)."""
    import gzip

    with open(os.path.join(ROOT, "tests", "golden", "manifest.json")) as f:
        man = json.load(f)["graphs"]["er4096"]
    with gzip.open(os.path.join(ROOT, "tests", "golden", "er4096.tsv.gz"), "rt") as f:
        data = np.loadtxt(f, dtype=np.int64, ndmin=2)
    u, v, t = data[:, 0].astype(np.uint32), data[:, 1].astype(np.uint32), data[:, 2].astype(np.uint32)
    return man["num_nodes"], np.concatenate([u, v]), np.concatenate([v, u]), t, man["k_max"]


def gpu_local_cpus(index):
    """CPUs of the GPU's own NUMA node (sysfs local_cpulist of its PCI device), or None."""
    try:
        bus = subprocess.run(["nvidia-smi", f"--id={index}", "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30).stdout.strip().lower()
        dom, rest = bus.split(":", 1)
        base = f"/sys/bus/pci/devices/{dom[-4:]}:{rest}"
        with open(os.path.join(base, "local_cpulist")) as f:
            text = f.read().strip()
        node = None
        try:
            with open(os.path.join(base, "numa_node")) as f:
                node = int(f.read().strip())
        except Exception:
            pass
        cpus = set()
        for part in text.split(","):
            if "-" in part:
                a, b = part.split("-")
                cpus.update(range(int(a), int(b) + 1))
            elif part:
                cpus.add(int(part))
        return {"cpus": sorted(cpus), "numa_node": node, "cpulist": text}
    except Exception:
        return None


def bind_near_gpu(index):
    """Runs the calling thread (and the pinned host buffers it allocates, placed on first touch) on
    the GPU's own NUMA node, so that host<->device copies do not cross sockets.  Returns a record
    of what was done."""
    info = gpu_local_cpus(index)
    if not info or not info["cpus"]:
        return {"bound": False, "why": "no local CPU list for the GPU"}
    try:
        avail = os.sched_getaffinity(0)
        cpus = [c for c in info["cpus"] if c in avail]
        if not cpus or len(cpus) == len(avail):
            return {"bound": False, "numa_node": info["numa_node"], "cpulist": info["cpulist"],
                    "why": "the GPU's CPUs are all this process's CPUs"}
        os.sched_setaffinity(0, cpus)
        return {"bound": True, "numa_node": info["numa_node"], "cpulist": info["cpulist"], "cpus": len(cpus)}
    except Exception as exc:
        return {"bound": False, "why": str(exc)}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


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


def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    return oracle


def k3_runs_cpu(n, src, dst, warmup, runs, threads):
    """The reference's timed unit on the host cores: single-k runs at k = 3 on the whole graph by the
    oracle port of its loop (count and mark sweeps split over `threads` threads), `warmup` untimed
    runs first.  Returns (seconds per timed run, passes per run, edges kept by the last run)."""
    oracle = oracle_module()
    os_, _, secs, passes = oracle.ktruss_runs(n, src, dst, 3, warmup + runs, threads)
    return secs[warmup:], passes[warmup:], len(os_) // 2


def er4096_chain_cpu():
    """The plain method's small configuration (Erdos-Renyi G(4096, 16/4095)) decomposed completely by
    the reference algorithm (chained single-k runs, one host thread), checked against its fixture."""
    oracle = oracle_module()
    n, src, dst, t, k_max = load_er4096()
    t0 = time.perf_counter()
    r = oracle.decompose(n, src, dst, method="chain", threads=1)
    secs = time.perf_counter() - t0
    if r["k_max"] != k_max or not np.array_equal(r["truss"][: len(t)], t):
        raise RuntimeError("oracle chain differs from the er4096 fixture")
    m = len(t)
    return {"ms": secs * 1e3, "edges_per_s": m / secs, "m": m, "k_max": k_max, "passes": r["plain_passes"],
            "how": "complete decomposition, chained single-k runs k = 3, 4, ... (reference algorithm), one host "
                   "thread"}


def decomposition_estimate(n, m, src, dst, threads, strata):
    """Stratified estimate of the reference's complete chained decomposition on the host cores: the
    chain's levels (k = 3 .. k_max+1, each a single-k run on the (k-1)-truss) are cut into `strata`
    groups of equal alive-edge volume; from each group the level at its volume midpoint runs once,
    completely, on its chain input; a group's time is the run's time scaled by the group's volume
    over the level's.  An extrapolation, reported apart from `value`."""
    oracle = oracle_module()
    t0 = time.perf_counter()
    r = oracle.decompose(n, src, dst, levels=True, threads=threads)
    truss = r["truss"][:m]
    u, v = src[:m], dst[:m]
    lp, la = r["level_passes"], r["level_alive"]
    ks = [k for k in range(len(lp)) if lp[k]]
    vol = np.array([float(la[k]) for k in ks])
    total = vol.sum()
    cum = np.cumsum(vol)
    groups, start = [], 0
    for gi in range(strata):
        end = int(np.searchsorted(cum, total * (gi + 1) / strata - 1e-9)) + 1
        end = max(end, start + 1)
        if start >= len(ks):
            break
        groups.append((start, min(end, len(ks))))
        start = min(end, len(ks))
    rows, est = [], 0.0
    for a, b in groups:
        gvol = vol[a:b].sum()
        mid = cum[a] - vol[a] + gvol / 2  # volume midpoint of the group
        i = min(int(np.searchsorted(cum, mid)), b - 1)
        k = ks[i]
        sel = truss >= k - 1 if k > 3 else np.ones(m, bool)
        s_in = np.concatenate([u[sel], v[sel]])
        d_in = np.concatenate([v[sel], u[sel]])
        _, _, secs, passes = oracle.ktruss_runs(n, s_in, d_in, k, 1, threads)
        if int(passes[0]) != int(lp[k]):
            raise RuntimeError(f"level {k}: {int(passes[0])} passes, the peel says {int(lp[k])}")
        est += float(secs[0]) * gvol / vol[i]
        rows.append({"k": int(k), "levels": [int(ks[a]), int(ks[b - 1])], "input_edges": int(sel.sum()),
                     "passes": int(passes[0]), "seconds": float(secs[0]), "group_volume_share": gvol / total})
    return {"chain_seconds_extrapolated": est, "threads": threads, "strata": rows,
            "levels_total": len(ks), "timed_volume_share": sum(float(la[x["k"]]) for x in rows) / total,
            "edges_per_s_extrapolated": m / est, "setup_s": time.perf_counter() - t0,
            "how": "stratified by alive-edge volume; one complete single-k run per stratum on its chain input "
                   "(the (k-1)-truss from the oracle peel), scaled by the stratum's volume"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    w = WORKLOADS.get(args.workload)
    if w is None or "cliques" in w:
        print(json.dumps({"impl": "reference", "unavailable": "the reference CPU arm runs the single-graph R-MAT "
                                                              "workloads without planted cliques (the reference has "
                                                              "no batch or selector; the oracle plants no cliques)"}))
        return
    n, m, src, dst = make_graph(args.workload, with_oracle=True)
    fx = fixture(args.workload)
    threads = host_threads()
    t0 = time.time()
    secs, passes, kept = k3_runs_cpu(n, src, dst, args.warmup, args.steps, threads)
    wall = time.time() - t0
    if fx and kept != fx["chained_checks"][0]["truss_edges"]:
        raise RuntimeError(f"k = 3 kept {kept} edges, the fixture says {fx['chained_checks'][0]['truss_edges']}")
    ms = float(np.mean(secs)) * 1e3
    value = m / (ms * 1e-3)
    sample = (f"{args.steps} complete single-k runs at k = 3 on the whole graph (after {args.warmup} warm-up "
              f"runs): the oracle port of the reference's count-and-prune loop (kernel_hdc.cu:107-201, "
              f"{int(passes[0])} pass, count and mark sweeps split over {threads} host threads), each timed alone "
              "like the reference's k-truss timer (kernel_hdc.cu:213-229); relabel and CSR build once, untimed")
    line = {"metric": "k-truss edges/s", "value": value, "unit": "edges/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "impl": "reference", "config": workload_config(args.workload, n, m),
            "work": "one complete single-k run at k = 3 on the whole graph (the reference's timed unit)",
            "cpu_baseline": {"value": value, "unit": "edges/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "run_ms": [float(x) * 1e3 for x in secs], "kept_edges": kept,
            "er4096_full_decomposition": er4096_chain_cpu(), "wall_s": wall}
    if args.decomposition_estimate:
        line["decomposition_estimate"] = decomposition_estimate(n, m, src, dst, threads, args.decomposition_estimate)
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


def choose_schedule(args, eng, kt, sample, target, batch=False):
    """Sets the engine's schedule (and the host-buffer engine's) from --schedule; 'auto' runs the
    autotuner on `sample()` = (n, src, dst) device tensors of other graphs of the same
    distribution (as a batch union when `batch`); 'learned' trains the selector and applies it to
    the features of `target()`, the measured graph.  Returns the config record."""
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
        # the least of three runs per candidate: candidates within a few percent of each other on
        # the sample otherwise trade places from run to run
        best, table = eng.autotune(d_src.data_ptr(), d_dst.data_ptr(), d_src.numel(), n, repeats=3, batch=batch)
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

    sched = choose_schedule(args, eng, kt, tune_sample, lambda: (n, d_src, d_dst), batch=True)
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
    for _ in range(max(1, args.warmup)):  # the same warm-up as the device-buffer steps
        kt.decompose_batch(h_src, h_dst, n, off, out=h_out)
    gc.disable()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        _, k2 = kt.decompose_batch(h_src, h_dst, n, off, out=h_out)
    e2e_s = (time.perf_counter() - t1) / args.steps
    gc.enable()
    e2e_s = max_over_ranks(e2e_s, td, "cuda")
    ls = kt.last_stats()
    if not np.array_equal(k2, kmax.view(np.uint32)):
        raise RuntimeError("host-buffer and device-buffer batches differ")
    single = single_graph_path(kt, torch, eng, n, u, v, off, kmax.view(np.uint32), args.single_graphs)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = batch_cpu_baseline(u, v, off, h_out, kmax.view(np.uint32))
    line = {"metric": "batched k-truss decomposition graphs/s", "value": G * world / (ms * 1e-3),
            "unit": "graphs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": f"{args.workload}: {G} graphs, n log-uniform in [{b['n_min']}, {b['n_max']}], "
                                   "half Barabasi-Albert, half Watts-Strogatz, 0-3 planted cliques each, "
                                   "one call", "n": n, "m": m, "edges_per_s": m * world / (ms * 1e-3),
                       "k_max_max": int(kmax.max()), "peel_rounds": st.num_rounds, "peel_levels": st.num_levels,
                       "phase_ms": {"build": st.build_ms, "support": st.support_ms, "peel": st.peel_ms},
                       "peel_phase_ms": st.as_dict()["peel_phase_ms"], "walk_entries": st.walk_entries,
                       "generation_s": gen_s,
                       "parallelism": f"graph shards x{world}" if world > 1 else "one GPU", "schedule": sched,
                       "single_graph_path": single,
                       "l2": "input entries 2x4x2m bytes > L2 (129 MB)"},
            "e2e": {"value": G * world / e2e_s, "unit": "graphs/s", "h2d_bytes_per_step": 8 * N + 4 * (G + 1),
                    "d2h_bytes_per_step": 4 * N + 4 * G, "ms_per_step": e2e_s * 1e3,
                    "last_call_device_ms": {"copy_in": ls.copy_in_ms, "decompose": ls.last_ms,
                                            "copy_out_and_kmax": ls.copy_out_ms}},
            "gpu_launches": launches, "clocks": clk.summary()}
    if cpu:
        line["cpu_baseline"], line["detail_parity"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        td.destroy_process_group()


def batch_cpu_baseline(u, v, off, truss, kmax):
    """The reference algorithm on the host cores for the whole batch: every graph decomposed by
    chained single-k runs (the oracle port of kernel_hdc.cu), one single-threaded process per graph
    at a time on all host cores; each graph's k_max and truss numbers (sha256) are compared with the
    GPU's batch output."""
    import hashlib

    oracle = oracle_module()
    res, secs, workers = oracle.decompose_batch_processes(u, v, off)
    G = len(off) - 1
    lo = np.searchsorted(u, off[:-1], side="left")
    hi = np.searchsorted(u, off[1:], side="left")
    bad = 0
    for g, k_ref, sha_ref in res:
        got = hashlib.sha256(np.ascontiguousarray(truss[lo[g]:hi[g]]).astype("<u4").tobytes()).hexdigest()
        if got != sha_ref or int(kmax[g]) != k_ref:
            bad += 1
    if len(res) != G or bad:
        raise RuntimeError(f"batch: {bad} of {G} graphs differ from the reference algorithm on the CPU")
    base = {"value": G / secs, "unit": "graphs/s", "cores": workers, "kind": "port",
            "sample": f"all {G} graphs of the batch, each decomposed completely by the reference algorithm "
                      "(chained count-and-prune single-k runs, the oracle port of kernel_hdc.cu), one "
                      f"single-threaded process per graph at a time on {workers} host processes ({secs:.1f} s)"}
    parity = (f"all {G} graphs: per-edge truss numbers (sha256) and k_max equal the reference algorithm's "
              "(CPU chain)")
    return base, parity


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
    graphs, host = [], []
    for spec in held["specs"]:
        n, u, v = selector.make_graph(json.loads(str(spec)))
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
        graphs.append((n, len(u), dev(np.concatenate([u, v])), dev(np.concatenate([v, u]))))
        host.append((n, u, v))
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
            # the autotuner's span (support count and peel, no per-entry output) plus the selector
            learned[i] = min(learned[i], st.select_ms + st.support_ms + st.peel_ms - st.emit_ms)
    ratio = learned.sum() / tuned.sum()
    line = {"metric": "learned-selector time / exhaustively tuned time", "value": ratio, "unit": "ratio",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": learned.sum(),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32 network, u32 peel",
            "data": "synthetic",
            "config": {"workload": "200 held-out graphs (Erdos-Renyi, R-MAT 12-18, Barabasi-Albert, random "
                                   "geometric, planted cliques), support count + peel device time, best of "
                                   f"{args.steps} runs per graph (the learned time includes the selector's "
                                   "statistics, features and inference, one launch; no time includes the per-entry "
                                   "output); selector trained on 2000 other graphs' GB300 timings", "learned_ms": learned.sum(), "tuned_ms": tuned.sum(),
                       "default_ms": default.sum(), "default_over_tuned": default.sum() / tuned.sum(),
                       "gain_vs_default": default.sum() / learned.sum(), "tuning_runs": 36 * args.steps, **info}}
    if not args.no_cpu:
        line["cpu_baseline"], line["detail_parity"] = heldout_cpu_baseline(eng, torch, graphs, host, out, kk,
                                                                           learned.sum())
    print(json.dumps(line), flush=True)
    eng.close()


def heldout_cpu_baseline(eng, torch, graphs, host, out, kk, learned_ms):
    """The 200 held-out graphs on the host cores: each decomposed by the oracle's exact peel, one
    single-threaded process per graph at a time on all host cores (the chained reference algorithm
    would take hours on the R-MAT 16-18 graphs of the set); every graph's truss numbers (sha256)
    and k_max are compared with the engine's under the learned schedule."""
    import hashlib

    oracle = oracle_module()
    shas, kmaxes = [], []
    for n, m, s_, d_ in graphs:
        eng.decompose(s_.data_ptr(), d_.data_ptr(), s_.numel(), n, out.data_ptr(), kk.data_ptr())
        t = out[:m].cpu().numpy().view(np.uint32)
        shas.append(hashlib.sha256(np.ascontiguousarray(t).astype("<u4").tobytes()).hexdigest())
        kmaxes.append(int(kk.item()))
    us, vs, off = [], [], [0]
    for n, u, v in host:
        us.append(np.asarray(u, np.uint64) + off[-1])
        vs.append(np.asarray(v, np.uint64) + off[-1])
        off.append(off[-1] + n)
    res, secs, workers = oracle.decompose_batch_processes(np.concatenate(us), np.concatenate(vs),
                                                          np.array(off, np.uint32), per_task=1, method="peel")
    bad = sum(1 for g, k_ref, sha_ref in res if sha_ref != shas[g] or k_ref != kmaxes[g])
    if len(res) != len(graphs) or bad:
        raise RuntimeError(f"held-out graphs: {bad} of {len(graphs)} differ from the oracle")
    G = len(graphs)
    base = {"value": G / secs, "unit": "graphs/s", "cores": workers, "kind": "port",
            "sample": f"all {G} held-out graphs, each decomposed by the oracle's exact peel (faster than the "
                      "reference's chained single-k runs, so the ratio is conservative), one single-threaded "
                      f"process per graph at a time on {workers} host processes ({secs:.1f} s); the engine "
                      f"decomposes them in {learned_ms:.0f} ms of support + peel device time "
                      f"({G / (learned_ms * 1e-3):.0f} graphs/s)"}
    return base, f"all {G} graphs: per-edge truss numbers (sha256) and k_max equal the oracle's"



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
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    st = eng.stats()
    launches = st.kernel_launches - launches0
    if dist:
        ms = max_over_ranks(ms, td, "cuda")
    k_max = int(d_k.item())
    truss = d_out.cpu().numpy().view(np.uint32)

    # phase breakdown: the same step again, one at a time (stats read after each)
    phases = {"build": [], "support": [], "peel": [], "peel_kernel": []}
    for _ in range(min(args.steps, 5)):
        step()
        s_ = eng.stats()
        for key, val in (("build", s_.build_ms), ("support", s_.support_ms), ("peel", s_.peel_ms),
                         ("peel_kernel", s_.peel_kernel_ms)):
            phases[key].append(val)
    st = eng.stats()
    pm = {k_: statistics.mean(v_) for k_, v_ in phases.items()}

    # parity with the oracle fixture of this graph (hash of the per-edge truss numbers, k_max, and
    # the reference schedule's pass statistics)
    fx = fixture(args.workload)
    parity = None
    if fx:
        import hashlib

        got = hashlib.sha256(np.ascontiguousarray(truss[:m]).astype("<u4").tobytes()).hexdigest()
        if got != fx["truss_sha256"] or k_max != fx["k_max"] or not np.array_equal(truss[:m], truss[m:]):
            raise RuntimeError("decomposition differs from the oracle fixture")
        if st.plain_passes != fx["plain_passes"] or st.plain_alive_sum != fx["plain_alive_sum"]:
            raise RuntimeError(f"pass statistics {st.plain_passes}/{st.plain_alive_sum} differ from the fixture")
        parity = (f"per-edge truss numbers equal the oracle fixture {os.path.relpath(FIXTURES[args.workload], ROOT)} "
                  f"(sha256 {got[:16]}...), k_max {k_max}, {fx['plain_passes']} reference passes")

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

    # the reference's own unit on the same graph: single-k runs at k = 3 (kt_engine_ktruss)
    d_keep = torch.empty(N, dtype=torch.uint8, device="cuda")
    for _ in range(2):
        eng.ktruss(d_src.data_ptr(), d_dst.data_ptr(), N, n, 3, d_keep.data_ptr(), sync=False)
    torch.cuda.synchronize()
    ev4, ev5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev4.record(stream)
    for _ in range(args.steps):
        eng.ktruss(d_src.data_ptr(), d_dst.data_ptr(), N, n, 3, d_keep.data_ptr(), sync=False)
    ev5.record(stream)
    torch.cuda.synchronize()
    k3_ms = ev4.elapsed_time(ev5) / args.steps
    k3_kept = int(d_keep.sum().item()) // 2
    # the 3-truss is every edge whose truss number is at least 3
    if fx and k3_kept != sum(c for t, c in fx["histogram"].items() if int(t) >= 3):
        raise RuntimeError("k = 3 truss differs from the fixture")

    # the plain method's small configuration (Erdos-Renyi G(4096, 16/4095)), decomposed completely
    en, es, ed, et, ek = load_er4096()
    d_es = torch.from_numpy(es.view(np.int32)).cuda()
    d_ed = torch.from_numpy(ed.view(np.int32)).cuda()
    d_eo = torch.empty(len(es), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        eng.decompose(d_es.data_ptr(), d_ed.data_ptr(), len(es), en, d_eo.data_ptr(), d_k.data_ptr(), sync=False)
    torch.cuda.synchronize()
    ev6, ev7 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev6.record(stream)
    for _ in range(args.steps):
        eng.decompose(d_es.data_ptr(), d_ed.data_ptr(), len(es), en, d_eo.data_ptr(), d_k.data_ptr(), sync=False)
    ev7.record(stream)
    torch.cuda.synchronize()
    er_ms = ev6.elapsed_time(ev7) / args.steps
    if int(d_k.item()) != ek or not np.array_equal(d_eo.cpu().numpy().view(np.uint32)[: len(et)], et):
        raise RuntimeError("er4096 decomposition differs from its fixture")

    # end to end through the host-buffer C ABI (pinned host memory placed on the GPU's NUMA node:
    # allocated and first touched from its CPUs; the thread's CPU set is restored afterwards)
    cpus0 = os.sched_getaffinity(0)
    numa = bind_near_gpu(local)
    h_src = torch.from_numpy(src.view(np.int32)).pin_memory()
    h_dst = torch.from_numpy(dst.view(np.int32)).pin_memory()
    h_out = torch.empty(N, dtype=torch.int32).pin_memory()
    h_out.fill_(0)
    os.sched_setaffinity(0, cpus0)
    g = kt.COOGraph(n, h_src.numpy().view(np.uint32), h_dst.numpy().view(np.uint32))
    out_np = h_out.numpy().view(np.uint32)
    for _ in range(max(1, args.warmup)):  # the same warm-up as the device-buffer steps
        kt.decompose(g, out=out_np)
    if dist:
        td.barrier()
    # the interpreter's collector stays out of the timed calls; each call's wall time is kept too
    gc.disable()
    call_s, call_dev = [], []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        _, k2 = kt.decompose(g, out=out_np)
        call_s.append(time.perf_counter() - t1)
        s_ = kt.last_stats()  # a host read of the call's own events (the call has synchronized)
        call_dev.append((s_.copy_in_ms, s_.last_ms, s_.copy_out_ms))
    e2e_s = (time.perf_counter() - t0) / args.steps
    gc.enable()
    slow = max(range(len(call_s)), key=lambda i: call_s[i])
    ls = kt.last_stats()
    if dist:
        e2e_s = max_over_ranks(e2e_s, td, "cuda")
    assert k2 == k_max
    if not np.array_equal(out_np, truss):
        raise RuntimeError("host-buffer and device-buffer decompositions differ")

    hbm, hbm_kind = peaks()
    traffic = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(args.workload, {})
    except Exception:
        pass
    sup_ms = pm["support"]
    sup_bytes = 4 * (n + 1) + 12 * m
    sup_gbs = sup_bytes / (sup_ms * 1e-3) / 1e9
    pk_ms = pm["peel_kernel"]
    passes = fx["plain_passes"] if fx else st.plain_passes
    alive_sum = fx["plain_alive_sum"] if fx else st.plain_alive_sum
    plain_bytes = 4 * (n + 1) * passes + 12 * alive_sum
    pk_gbs = plain_bytes / (pk_ms * 1e-3) / 1e9
    traffic_note = traffic.get("source")
    line = {"metric": "k-truss edges/s", "value": replica_throughput(m, world, ms), "unit": "edges/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": workload_config(args.workload, n, m),
            "work": "one full truss decomposition (every k): device CSR build, support count, peel, per-entry "
                    "truss numbers",
            "detail": {"k_max": k_max, "triangles": st.triangles, "peel_rounds": st.num_rounds,
                       "peel_levels": st.num_levels, "parallelism": f"replicas{world}",
                       "phase_ms": {"build": pm["build"], "support": sup_ms, "peel": pm["peel"]},
                       "peel_phase_ms": st.as_dict()["peel_phase_ms"], "compactions": st.compactions,
                       "walk_entries": st.walk_entries, "parity": parity,
                       "replay": {"ms_per_step": replay_ms, "mode": replay_mode,
                                  "how": "kt_engine_replay: the same steps through a CUDA graph of the device "
                                         "pipeline (repeat runs on unchanged input, no host-side input checks)"},
                       "schedule": sched},
            "single_k3": {"ms": k3_ms, "edges_per_s": m / (k3_ms * 1e-3), "kept_edges": k3_kept,
                          "how": "kt_engine_ktruss at k = 3 on the same graph (device buffers): the unit the "
                                 "reference arm times"},
            "er4096_full_decomposition": {"ms": er_ms, "edges_per_s": len(et) / (er_ms * 1e-3), "m": len(et),
                                          "k_max": ek},
            "e2e": {"value": replica_throughput(m, world, e2e_s * 1e3), "unit": "edges/s", "h2d_bytes_per_step": 8 * N,
                    "d2h_bytes_per_step": 4 * N, "ms_per_step": e2e_s * 1e3,
                    "call_ms": {"median": statistics.median(call_s) * 1e3, "min": min(call_s) * 1e3,
                                "max": max(call_s) * 1e3,
                                "slowest_device_ms": dict(zip(("copy_in", "decompose", "copy_out"),
                                                              call_dev[slow]))},
                    "last_call_device_ms": {"copy_in": ls.copy_in_ms, "decompose": ls.last_ms,
                                            "copy_out": ls.copy_out_ms},
                    "h2d_gbs": 8 * N / (ls.copy_in_ms * 1e-3) / 1e9 if ls.copy_in_ms else None,
                    "d2h_gbs": 4 * N / (ls.copy_out_ms * 1e-3) / 1e9 if ls.copy_out_ms else None,
                    "host_buffers": numa},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": "k_peel", "achieved": pk_gbs, "peak": hbm,
                         "peak_kind": hbm_kind, "unit": "GB/s", "frac": pk_gbs / hbm,
                         "traffic": traffic.get("k_peel"), "traffic_source": traffic_note,
                         "algorithmic_bytes": plain_bytes, "kernel_ms": pk_ms, "passes": passes,
                         "alive_sum": alive_sum, "passes_source": "oracle fixture" if fx else "engine round log"},
            "roofline_support": {"bound": "hbm", "kernel": "k_support", "achieved": sup_gbs, "peak": hbm,
                                 "unit": "GB/s", "frac": sup_gbs / hbm, "traffic": traffic.get("k_support"),
                                 "traffic_source": traffic_note, "algorithmic_bytes": sup_bytes, "kernel_ms": sup_ms},
            "clocks": clk.summary()}
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = host_threads()
        secs, cpasses, kept = k3_runs_cpu(n, src, dst, 1, args.cpu_runs, threads)
        if kept != k3_kept:
            raise RuntimeError("CPU and GPU k = 3 truss sizes differ")
        cms = float(np.mean(secs)) * 1e3
        line["cpu_baseline"] = {"value": m / (cms * 1e-3), "unit": "edges/s", "cores": threads, "kind": "port",
                                "sample": (f"{args.cpu_runs} complete single-k runs at k = 3 on the whole graph "
                                           f"({cms:.0f} ms each; the GPU's time for the same unit is single_k3.ms): "
                                           "the oracle port of the reference loop, count and mark sweeps on "
                                           f"{threads} host threads; a complete CPU decomposition of this graph "
                                           "takes hours")}
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
    ap.add_argument("--cpu-runs", type=int, default=3,
                    help="cpu_baseline: complete single-k runs at k = 3 timed on the host cores")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--decomposition-estimate", type=int, default=0, metavar="STRATA",
                    help="reference arm: also estimate the complete CPU decomposition from STRATA complete level "
                         "runs (an extrapolation, reported apart from value)")
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
