"""Pins the benchmarked single-graph workload to the oracle: R-MAT scale 20, edge factor 16,
(a, b, c, d) = (0.57, 0.19, 0.19, 0.05), seed 1, symmetrized, deduplicated, self loops removed.

    python tests/golden/make_headline_fixture.py      # writes tests/golden/rmat20_seed1.json

The graph is made by the oracle's own generator (oracle.gen_rmat, no product library).  The
oracle's exact peel (ko_decompose_peel_levels) gives every edge's truss number, k_max, and the
pass statistics of the reference's chained schedule - per level k the count-and-prune passes of
the single-k run at k and the sum of their alive oriented edges (kernel_hdc.cu:107-201 chained
over k).  The peel is cross-checked here against the chained single-k algorithm itself
(oracle.ktruss, the restatement of kernel_hdc.cu) at k = 3 on the whole graph and at k = k_max and
k_max + 1 on the (k-1)-truss: equal edge sets and equal pass counts.  The fixture keeps hashes and
counts only (the per-edge numbers are 63 MB):
  edges_sha256   SHA-256 of the canonical edge list (u < v, sorted), uint32 little-endian pairs
  truss_sha256   SHA-256 of the truss numbers in that edge order, uint32 little-endian
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

import oracle  # noqa: E402

GRAPH = dict(scale=20, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1)
OUT = os.path.join(HERE, "rmat20_seed1.json")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).astype("<u4").tobytes()).hexdigest()


def canon_keys(s, d):
    a, b = np.minimum(s, d).astype(np.uint64), np.maximum(s, d).astype(np.uint64)
    return np.unique((a << np.uint64(32)) | b)


def main():
    t0 = time.time()
    n, u, v = oracle.gen_rmat(GRAPH["scale"], GRAPH["edge_factor"], GRAPH["a"], GRAPH["b"], GRAPH["c"], GRAPH["seed"])
    m = len(u)
    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    print(f"generated n={n} m={m} in {time.time() - t0:.1f} s", flush=True)
    t0 = time.time()
    r = oracle.decompose(n, src, dst, method="peel", levels=True)
    peel_s = time.time() - t0
    t = r["truss"][:m]
    assert np.array_equal(r["truss"][m:], t)
    print(f"peel: k_max={r['k_max']} passes={r['plain_passes']} in {peel_s:.1f} s", flush=True)
    lp, la = r["level_passes"], r["level_alive"]
    levels = [[int(k), int(lp[k]), int(la[k])] for k in range(len(lp)) if lp[k]]
    assert sum(x[1] for x in levels) == r["plain_passes"] and sum(x[2] for x in levels) == r["plain_alive_sum"]
    keys = (u.astype(np.uint64) << np.uint64(32)) | v.astype(np.uint64)
    checks = []
    for k in (3, r["k_max"], r["k_max"] + 1):
        sel = t >= k - 1 if k > 3 else np.ones(m, bool)  # the chain's input at level k
        s_in = np.concatenate([u[sel], v[sel]])
        d_in = np.concatenate([v[sel], u[sel]])
        t1 = time.time()
        os_, od, alive = oracle.ktruss(n, s_in, d_in, k, pass_log=True)
        got = canon_keys(os_, od)
        want = keys[t >= k]
        assert np.array_equal(got, want), f"chained k={k} differs from the peel"
        assert len(alive) == int(lp[k]), f"k={k}: {len(alive)} passes vs {int(lp[k])}"
        assert int(alive.sum()) == int(la[k])
        checks.append({"k": int(k), "input_edges": int(sel.sum()), "truss_edges": int(len(want)),
                       "passes": int(len(alive)), "seconds": round(time.time() - t1, 1)})
        print(f"chained k={k}: {len(want)} edges, {len(alive)} passes ok", flush=True)
    hist = np.bincount(t)
    fixture = {
        "graph": GRAPH, "num_nodes": int(n), "num_edges": int(m),
        "edges_sha256": sha(np.stack([u, v], 1)),
        "truss_sha256": sha(t),
        "k_max": int(r["k_max"]),
        "histogram": {str(i): int(c) for i, c in enumerate(hist) if c},
        "plain_passes": int(r["plain_passes"]), "plain_alive_sum": int(r["plain_alive_sum"]),
        "peel_rounds": int(r["rounds"]),
        "levels": levels,
        "chained_checks": checks,
        "made_by": "tests/golden/make_headline_fixture.py (oracle.gen_rmat, oracle.decompose peel, "
                   "oracle.ktruss chained checks)",
    }
    with open(OUT, "w") as f:
        json.dump(fixture, f, indent=1)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
