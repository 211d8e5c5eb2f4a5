"""Pins the stress workload to the oracle: R-MAT scale 24, edge factor 32, (a, b, c, d) =
(0.57, 0.19, 0.19, 0.05), seed 1, symmetrized, deduplicated, self loops removed, plus 16 planted
cliques of 64-512 random vertices (seed 8).

    python tests/golden/make_stress_fixture.py [threads]   # writes tests/golden/rmat24_seed1.json

The edge list comes from the library's seeded host generators (kt_gen_rmat, kt_plant_cliques;
SplitMix64 counters, the same on x86-64 and AArch64; the oracle has no clique planter) and is
pinned by its hash.  Every truss number comes from the oracle's exact peel on host threads
(ko_decompose_peel_mt, the same rounds as its one-thread peel, which the R-MAT 20 fixture
cross-checks against the chained single-k algorithm of kernel_hdc.cu), with the pass statistics
of the reference's chained schedule per level.  512.7 M edges: about 27 GB of host memory and 55
minutes on eight x86-64 cores.  The fixture keeps hashes and counts only:
  edges_sha256   SHA-256 of the edge list in generator order (u, v pairs), uint32 little-endian
  truss_sha256   SHA-256 of the truss numbers in that order, uint32 little-endian
  histogram      truss number -> edge count
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "ktruss-explorer_gb300"))

import oracle  # noqa: E402

GRAPH = dict(scale=24, edge_factor=32, a=0.57, b=0.19, c=0.19, seed=1, cliques=[16, 64, 512], clique_seed=8)
OUT = os.path.join(HERE, "rmat24_seed1.json")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).astype("<u4").tobytes()).hexdigest()


def main():
    import ktruss_gb300 as kt  # host generators only; no device is used

    threads = int(sys.argv[1]) if len(sys.argv) > 1 else min(16, os.cpu_count() or 1)
    g = GRAPH
    t0 = time.time()
    n, u, v = kt.gen_rmat(g["scale"], g["edge_factor"], g["a"], g["b"], g["c"], g["seed"])
    count, lo, hi = g["cliques"]
    n, u, v = kt.plant_cliques(n, u, v, count, lo, hi, g["clique_seed"])
    m = len(u)
    edges_sha = sha(np.stack([u, v], 1))
    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    del u, v
    print(f"generated n={n} m={m} in {time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    r = oracle.decompose(n, src, dst, method="peel", levels=True, threads=threads)
    peel_s = time.time() - t0
    del src, dst
    t = r["truss"][:m]
    assert np.array_equal(r["truss"][m:], t)
    print(f"peel: k_max={r['k_max']} rounds={r['rounds']} passes={r['plain_passes']} in {peel_s:.0f} s", flush=True)
    lp, la = r["level_passes"], r["level_alive"]
    levels = [[int(k), int(lp[k]), int(la[k])] for k in range(len(lp)) if lp[k]]
    assert sum(x[1] for x in levels) == r["plain_passes"] and sum(x[2] for x in levels) == r["plain_alive_sum"]
    hist = np.bincount(t)
    fixture = {
        "graph": g, "num_nodes": int(n), "num_edges": int(m),
        "edges_sha256": edges_sha,
        "truss_sha256": sha(t),
        "k_max": int(r["k_max"]),
        "histogram": {str(i): int(c) for i, c in enumerate(hist) if c},
        "plain_passes": int(r["plain_passes"]), "plain_alive_sum": int(r["plain_alive_sum"]),
        "peel_rounds": int(r["rounds"]),
        "levels": levels,
        "oracle_seconds": round(peel_s), "oracle_threads": threads,
        "made_by": "tests/golden/make_stress_fixture.py (kt_gen_rmat + kt_plant_cliques host generators, "
                   "oracle.decompose peel on host threads)",
    }
    with open(OUT, "w") as f:
        json.dump(fixture, f, indent=1)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
