"""Generates the golden fixtures in tests/golden/ from the reference's own executable.

    make -C oracle ref            # builds oracle/_ref/ktruss from the reference sources
    python tests/golden/make_golden.py

For every fixture graph this script
  * writes it in the reference's TSV format (graph.cu:96-104: "dst src 1", 1-based, both
    directions),
  * runs the reference CLI on the CPU path (`-p cpu`) for k = 3, 4, ... with each output as the
    next input (the (k+1)-truss of G is the (k+1)-truss of its k-truss) until the output is
    empty, giving every edge's truss number and k_max,
  * counts the reference's count-and-prune passes per run (`-v 2` prints one "Iteration" line
    per pass) and, with `-e` large enough to compact after every pass, the edges left after
    each pass, from which the alive-edge sum over all passes follows,
  * runs all 12 CPU variants (-d x -f x -r, plus -e 1) at several k and checks they agree.
Outputs: <name>.tsv.gz ("u v t" per undirected edge, 0-based, u < v) and manifest.json.
The reference cannot travel to the GPU machine; these files are the pinned parity anchor.
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "ktruss")
sys.path.insert(0, os.path.join(ROOT, "ktruss-explorer_gb300"))

import ktruss_gb300 as kt  # noqa: E402  (generators only)


def canon(u, v):
    u = np.asarray(u, np.uint64)
    v = np.asarray(v, np.uint64)
    a, b = np.minimum(u, v), np.maximum(u, v)
    keys = np.unique((a << np.uint64(32)) | b)
    return (keys >> np.uint64(32)).astype(np.uint32), (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def edge_sha(u, v) -> str:
    u, v = canon(u, v)
    return hashlib.sha256(np.stack([u, v], 1).astype("<u4").tobytes()).hexdigest()


def write_ref_tsv(path, u, v):
    with open(path, "w") as f:
        for a, b in zip(u.tolist(), v.tolist()):
            f.write(f"{b + 1}\t{a + 1}\t1\n{a + 1}\t{b + 1}\t1\n")


def read_ref_tsv(path):
    if os.path.getsize(path) == 0:
        return np.zeros(0, np.uint32), np.zeros(0, np.uint32)
    x = np.loadtxt(path, dtype=np.int64, ndmin=2)
    return (x[:, 1] - 1).astype(np.uint32), (x[:, 0] - 1).astype(np.uint32)


def run_ref(args, cwd):
    """Runs the reference CLI; verify may abort afterwards (its -c file is a dummy), which is
    fine because the -o output is written before verify (main.cu:35-43)."""
    r = subprocess.run(["stdbuf", "-oL", REF] + args, cwd=cwd, capture_output=True, text=True)
    return r.stdout


def chain(tsv, tmp, n_nodes):
    """Chained single-k reference runs; returns per-edge truss dict, k_max, passes, alive sum."""
    cur = tsv
    k = 3
    truss = {}
    u0, v0 = read_ref_tsv(tsv)
    cu, cv = canon(u0, v0)
    for a, b in zip(cu.tolist(), cv.tolist()):
        truss[(a, b)] = 2
    passes = 0
    alive_sum = 0
    kmax = 2 if len(cu) else 0
    while True:
        out = os.path.join(tmp, f"out{k}.tsv")
        # -e 1000000: compact after every pass so -v 2 reports the edges left after each pass
        txt = run_ref(["-p", "cpu", "-g", cur, "-k", str(k), "-o", out, "-c", cur, "-v", "2", "-e", "1000000"], tmp)
        iters = len(re.findall(r"^\s*Iteration \d+", txt, re.M))
        remaining = [int(x) for x in re.findall(r"# edges remaining = (\d+)", txt)]
        cin_u, cin_v = read_ref_tsv(cur)
        alive = len(canon(cin_u, cin_v)[0])
        passes += iters
        # pass i sees the edges alive at its start: the input, then what each compaction left
        seq = [alive] + remaining
        alive_sum += sum(seq[:iters])
        ou, ov = read_ref_tsv(out)
        if len(ou) == 0:
            break
        ou, ov = canon(ou, ov)
        for a, b in zip(ou.tolist(), ov.tolist()):
            truss[(a, b)] = k
        kmax = k
        cur = out
        k += 1
    return truss, kmax, passes, alive_sum


VARIANTS = [(d, f, r) for d in ("undirected", "directed-by-index", "directed-by-degree")
            for f in ("coocsr", "tiled-coocsr") for r in ("all", "affected")]


def variant_check(tsv, tmp, k, expect):
    """All 12 CPU variants (and -e 1) at this k must return the expected edge set."""
    results = {}
    for d, f, r in VARIANTS + [("directed-by-degree", "coocsr", "all-e1")]:
        out = os.path.join(tmp, "var.tsv")
        if os.path.exists(out):
            os.remove(out)
        rr = "all" if r == "all-e1" else r
        args = ["-p", "cpu", "-g", tsv, "-k", str(k), "-o", out, "-c", tsv, "-v", "0", "-d", d, "-f", f, "-r", rr,
                "-t", "4"]
        if r == "all-e1":
            args += ["-e", "1"]
        run_ref(args, tmp)
        ou, ov = read_ref_tsv(out)
        sha = edge_sha(ou, ov) if len(ou) else "empty"
        results[f"{d}/{f}/{r}"] = sha
        if sha != expect:
            raise SystemExit(f"reference variant {d}/{f}/{r} disagrees at k={k} on {tsv}")
    return results


def graphs():
    """(name, spec, num_nodes, u, v) for every fixture graph."""
    out = []

    def add(name, spec, n, u, v):
        u, v = canon(u, v)
        out.append((name, spec, n, u, v))

    # the 9-vertex graph: K5 on 1..5, triangle 6-7-8, bridge 5-6, pendant 9-1 (1-based)
    e = [(a, b) for a in range(5) for b in range(a + 1, 5)] + [(5, 6), (6, 7), (5, 7), (4, 5), (8, 0)]
    add("tiny9", {"kind": "hand"}, 9, *zip(*e))
    e = [(a, b) for a in range(6) for b in range(a + 1, 6)]
    add("k6", {"kind": "hand"}, 6, *zip(*e))
    e = [(i, (i + 1) % 8) for i in range(8)]
    add("cycle8", {"kind": "hand"}, 8, *zip(*e))
    e = [(0, i) for i in range(1, 6)] + [(5, 6), (6, 7), (7, 8)]
    add("tree9", {"kind": "hand"}, 9, *zip(*e))
    e = [(a, b) for a in range(4) for b in range(a + 1, 4)] + \
        [(a, b) for a in range(4, 9) for b in range(a + 1, 9)] + [(3, 4), (9, 10), (10, 11), (9, 11), (11, 0)]
    add("cliques_bridge", {"kind": "hand"}, 12, *zip(*e))
    add("one_edge", {"kind": "hand"}, 2, [0], [1])

    n, u, v = kt.gen_er(4096, 16 / 4095, 1)
    add("er4096", {"kind": "er", "n": 4096, "p": 16 / 4095, "seed": 1}, n, u, v)
    n, u, v = kt.gen_rmat(10, 16, 0.57, 0.19, 0.19, 1)
    add("rmat10", {"kind": "rmat", "scale": 10, "ef": 16, "seed": 1}, n, u, v)
    n, u, v = kt.gen_rmat(12, 8, 0.57, 0.19, 0.19, 2)
    add("rmat12", {"kind": "rmat", "scale": 12, "ef": 8, "seed": 2}, n, u, v)
    n, u, v = kt.gen_ba(2000, 4, 1)
    n, u, v = kt.plant_cliques(n, u, v, 2, 8, 16, 11)
    add("ba2000", {"kind": "ba", "n": 2000, "m": 4, "seed": 1, "cliques": [2, 8, 16, 11]}, n, u, v)
    n, u, v = kt.gen_ws(2000, 10, 0.1, 1)
    add("ws2000", {"kind": "ws", "n": 2000, "k": 10, "p": 0.1, "seed": 1}, n, u, v)
    r = float(np.sqrt(16 / (np.pi * 2000)))
    n, u, v = kt.gen_rgg(2000, r, 1)
    add("rgg2000", {"kind": "rgg", "n": 2000, "radius": r, "seed": 1}, n, u, v)
    n, u, v = kt.gen_er(1000, 0.01, 5)
    n, u, v = kt.plant_cliques(n, u, v, 3, 10, 30, 7)
    add("er1000_cliques", {"kind": "er", "n": 1000, "p": 0.01, "seed": 5, "cliques": [3, 10, 30, 7]}, n, u, v)
    return out


def main():
    if not os.path.exists(REF):
        raise SystemExit(f"{REF} missing: run `make -C oracle ref` first")
    manifest = {"reference": "ktruss -p cpu (built from the reference sources by oracle/Makefile)",
                "format": "u v t per undirected edge, 0-based, u < v; t = truss number", "graphs": {}}
    for name, spec, n, u, v in graphs():
        with tempfile.TemporaryDirectory() as tmp:
            tsv = os.path.join(tmp, "g.tsv")
            write_ref_tsv(tsv, u, v)
            truss, kmax, passes, alive_sum = chain(tsv, tmp, n)
            t = np.array([truss[(a, b)] for a, b in zip(u.tolist(), v.tolist())], np.uint32)
            ks = sorted({0, 1, 2, 3, 4, max(kmax, 2), kmax + 1} | ({(kmax + 3) // 2} if kmax > 4 else set()))
            checks = {}
            for k in ks:
                keep = t >= k if k >= 2 else np.zeros(len(t), bool)
                expect = edge_sha(u[keep], v[keep]) if keep.any() else "empty"
                checks[str(k)] = {"edges": int(keep.sum()), "sha": expect,
                                  "variants_agree": len(variant_check(tsv, tmp, k, expect))}
        with gzip.open(os.path.join(HERE, f"{name}.tsv.gz"), "wt") as f:
            for a, b, c in zip(u.tolist(), v.tolist(), t.tolist()):
                f.write(f"{a}\t{b}\t{c}\n")
        hist = np.bincount(t, minlength=kmax + 1).tolist() if len(t) else []
        manifest["graphs"][name] = {"spec": spec, "num_nodes": int(n), "num_edges": int(len(u)),
                                    "edge_sha": edge_sha(u, v), "k_max": int(kmax), "truss_hist": hist,
                                    "ref_passes": int(passes), "ref_alive_sum": int(alive_sum), "single_k": checks}
        print(f"{name}: n={n} m={len(u)} k_max={kmax} passes={passes} alive_sum={alive_sum}", flush=True)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
