"""The reference's own CUDA build on this GPU, beside the engine, on the same graphs.

    make -C oracle stage REF_DIR=<reference checkout>   # once, where the reference sources are
    python tests/compat/reference_sweep.py [--scale 20] [--sweep-scale 18] [--chain] [--out FILE]

Builds the reference's unmodified sources (the staged copy, baseline/_ref/src, or REF_DIR) with
oracle/Makefile for sm_103a, links tests/compat/ref_sweep_driver.cpp against their objects, and
drives the reference's own entry point ktruss() (kernel.h:12) through its own option parser:
  * every variant (-d x -f x -r) and block size (-b 128..1024) at k = 3 and k = k_max on R-MAT
    `--sweep-scale`, to find the fastest configuration at each k;
  * the default configuration and the fastest one at k = 3 and k = k_max on R-MAT `--scale`;
  * with --chain, the decomposition of R-MAT `--scale` by chaining the reference's single-k GPU
    runs k = 3, 4, ..., k_max (the default configuration); the last level of a complete chain,
    k_max + 1, whose truss is empty, cannot run on the reference's GPU path (it aborts when a
    k-truss has no edge left: a zero-block launch in removeCOOCSRDeletedEdgesOnDevice).
Times are the reference's own k-truss timer (kernel_ddc.cu:227-244, -w 1 -x 3, median of the timed
runs; its CSR build and copies are outside it, as in the reference).  Every reference result is
checked against the engine: the edge count and an order-free hash of the k-truss edge set.  The
engine's time for the same unit is kt_engine_ktruss (single k) or kt_engine_decompose (chain),
CUDA events on device-resident input.  Prints one JSON document.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ktruss-explorer_gb300"))

import ktruss_gb300 as kt  # noqa: E402

STAGED = os.path.join(ROOT, "baseline", "_ref", "src")
REF_OUT = os.path.join(ROOT, "oracle", "_ref")
LIB_OBJS = ["graph.o", "info.o", "kernel.o", "kernel_d.o", "kernel_ddc.o", "kernel_ddt.o", "kernel_duc.o",
            "kernel_dut.o", "kernel_h.o", "kernel_hdc.o", "kernel_hdt.o", "kernel_huc.o", "kernel_hut.o"]
VARIANTS = [(d, f, r) for d in ("undirected", "directed-by-index", "directed-by-degree")
            for f in ("coocsr", "tiled-coocsr") for r in ("all", "affected")]
BLOCKS = (128, 256, 512, 1024)
MASK = (1 << 64) - 1


def mix(z: np.ndarray) -> np.ndarray:
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def edge_set_summary(u: np.ndarray, v: np.ndarray) -> tuple[int, str]:
    """The driver's summary of an edge set given as canonical pairs u < v."""
    with np.errstate(over="ignore"):
        h = int(mix((u.astype(np.uint64) << np.uint64(32)) | v.astype(np.uint64)).sum(dtype=np.uint64))
    return len(u), f"{h & MASK:016x}"


def build(ref_dir: str) -> str:
    subprocess.run(["make", "-s", f"-j{os.cpu_count() or 8}", "-C", os.path.join(ROOT, "oracle"), "ref-objs",
                    f"REF_DIR={ref_dir}"], check=True)
    exe = os.path.join(REF_OUT, "ref_sweep_driver")
    subprocess.run(["nvcc", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-I", ref_dir, "-o", exe,
                    os.path.join(HERE, "ref_sweep_driver.cpp")] + [os.path.join(REF_OUT, o) for o in LIB_OBJS],
                   check=True)
    return exe


def write_graph(path: str, n: int, u: np.ndarray, v: np.ndarray, seed: int = 5) -> None:
    """The reference's TSV ("dst src 1", 1-based, both directions), entries in random order (the
    reference's host-side quicksort of each CSR row is quadratic on rows that arrive sorted)."""
    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    perm = np.random.default_rng(seed).permutation(len(src))
    kt.write_coo_graph_to_file(kt.COOGraph(n, src[perm], dst[perm]), path)


def run_driver(exe: str, graph: str, lines: list[str], timeout: float) -> list[dict]:
    """Runs configuration lines through the driver; returns one record per RESULT line with the
    reference's timed runs (ms) that preceded it."""
    r = subprocess.run([exe, graph], input="\n".join(lines) + "\n", capture_output=True, text=True,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference driver failed ({r.returncode}): {r.stderr[-2000:]}")
    out, times = [], []
    for ln in r.stdout.splitlines():
        if ln.startswith("RESULT"):
            f = dict(x.split("=") for x in ln.split()[1:])
            out.append({"k": int(f["k"]), "edges": int(f["edges"]), "hash": f["hash"], "ms": times})
            times = []
        elif ln.endswith(" ms") and "," in ln:
            times.append(float(ln.rsplit(",", 1)[1].split()[0]))
    return out


def engine_times(n, u, v, ks, reps=5):
    """Engine: single-k runs (kt_engine_ktruss) at each k and the decomposition, device buffers."""
    import torch

    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    N = len(src)
    eng = kt.Engine(0)
    eng.reserve(n, N)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_keep = torch.empty(N, dtype=torch.uint8, device="cuda")
    d_out = torch.empty(N, dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.ExternalStream(eng.stream)
    torch.cuda.synchronize()

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    res = {"decompose_ms": timed(lambda: eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), N, n, d_out.data_ptr(),
                                                       d_k.data_ptr(), sync=False))}
    truss = d_out.cpu().numpy().view(np.uint32)[: len(u)]
    res["k_max"] = int(d_k.item())
    for k in ks:
        res[f"ktruss_k{k}_ms"] = timed(lambda: eng.ktruss(d_src.data_ptr(), d_dst.data_ptr(), N, n, k,
                                                          d_keep.data_ptr(), sync=False))
    eng.close()
    return res, truss


def sweep_lines(k: int) -> list[str]:
    lines = []
    for d, f, r in VARIANTS:
        for b in BLOCKS:
            lines.append(f"-k {k} -p gpu -d {d} -f {f} -r {r} -b {b} -w 1 -x 3 -v 0")
    return lines


def check(records, truss, u, v):
    """Each reference record against the engine's k-truss edge set {t(e) >= k}."""
    bad = []
    for rec in records:
        sel = truss >= rec["k"]
        cnt, h = edge_set_summary(u[sel], v[sel])
        rec["matches_engine"] = rec["edges"] == cnt and rec["hash"] == h
        if not rec["matches_engine"]:
            bad.append(rec["k"])
    return bad


def parse_cfg(line: str) -> tuple:
    opts = line.split()
    get = lambda flag, default: opts[opts.index(flag) + 1] if flag in opts else default
    return (get("-d", "directed-by-degree"), get("-f", "coocsr"), get("-r", "all"), int(get("-b", "512")))


def run_graph(exe, tmp, scale, roles_lines):
    """Engine times and the reference's runs on R-MAT `scale`; roles_lines(k3, kmax) gives
    {role: [config lines]} for the roles "k3" and "kmax"."""
    n, u, v = kt.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 1)
    eng, truss = engine_times(n, u, v, [3])
    kmax = eng["k_max"]
    eng.update(engine_times(n, u, v, [kmax])[0])
    path = os.path.join(tmp, f"rmat{scale}.tsv")
    write_graph(path, n, u, v)
    g = {"n": n, "m": len(u), "k_max": kmax, "engine": eng, "runs": {}}
    for role, lines in roles_lines(3, kmax).items():
        t1 = time.time()
        recs = run_driver(exe, path, lines, timeout=3600)
        bad = check(recs, truss, u, v)
        if bad or len(recs) != len(lines):
            raise RuntimeError(f"rmat{scale}: reference k-truss differs from the engine at k = {bad}")
        g["runs"][role] = [{"config": parse_cfg(ln), "k": rec["k"], "ms_median": float(np.median(rec["ms"])),
                            "ms": rec["ms"], "edges": rec["edges"], "matches_engine": rec["matches_engine"]}
                           for ln, rec in zip(lines, recs)]
        g["runs"][role + "_wall_s"] = time.time() - t1
    return g, (n, u, v, truss, path)


def save(doc, path):
    if path:
        with open(path, "w") as f:
            f.write(json.dumps(doc, indent=1) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--sweep-scale", type=int, default=18)
    ap.add_argument("--chain", action="store_true")
    ap.add_argument("--ref-dir", default=os.environ.get("KT_REFERENCE_DIR") or STAGED)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    t0 = time.time()
    exe = build(args.ref_dir)
    doc = {"build_s": time.time() - t0, "graphs": {}}
    with tempfile.TemporaryDirectory() as tmp:
        sweep, _ = run_graph(exe, tmp, args.sweep_scale,
                             lambda k3, kmax: {"k3": sweep_lines(k3), "kmax": sweep_lines(kmax)})
        best = {role: min(sweep["runs"][role], key=lambda x: x["ms_median"])["config"] for role in ("k3", "kmax")}
        doc["graphs"][f"rmat{args.sweep_scale}"] = sweep
        doc["best_config"] = {role: list(c) for role, c in best.items()}
        save(doc, args.out)

        def large_lines(k3, kmax):
            out = {}
            for role, k in (("k3", k3), ("kmax", kmax)):
                d, f, r, b = best[role]
                out[role] = [f"-k {k} -p gpu -w 1 -x 3 -v 0",
                             f"-k {k} -p gpu -d {d} -f {f} -r {r} -b {b} -w 1 -x 3 -v 0"]
            return out

        large, (n, u, v, truss, path) = run_graph(exe, tmp, args.scale, large_lines)
        doc["graphs"][f"rmat{args.scale}"] = large
        save(doc, args.out)
        if args.chain:
            t1 = time.time()
            kmax = large["k_max"]
            recs = run_driver(exe, path, [f"chain {kmax} -p gpu -w 0 -x 1 -v 0"], timeout=5400)
            bad = check(recs, truss, u, v)
            if bad or [r["k"] for r in recs] != list(range(3, kmax + 1)):
                raise RuntimeError(f"chain: reference k-truss differs from the engine at k = {bad}")
            doc["chain"] = {"scale": args.scale, "levels_run": len(recs), "k_range": [3, kmax],
                            "ktruss_ms_total": float(sum(sum(r["ms"]) for r in recs)),
                            "ktruss_ms_per_level": [float(sum(r["ms"])) for r in recs],
                            "wall_s": time.time() - t1, "all_levels_match_engine": True,
                            "engine_decompose_ms": large["engine"]["decompose_ms"],
                            "note": "levels k = 3 .. k_max; the empty level k_max + 1 of a complete chain is not "
                                    "run (the reference's GPU path aborts on an empty k-truss)"}
            save(doc, args.out)
    print(json.dumps(doc, indent=1))


if __name__ == "__main__":
    main()
