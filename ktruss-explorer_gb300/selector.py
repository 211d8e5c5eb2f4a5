"""Training data, training and evaluation of the learned schedule selector (kt_selector).

    python ktruss-explorer_gb300/selector.py collect --count 2000 --seed 1 --out data/selector_train.npz
    python ktruss-explorer_gb300/selector.py collect --count 200 --seed 2 --out data/selector_heldout.npz
    python ktruss-explorer_gb300/selector.py collect --families batch --count 300 --seed 3 --out data/selector_batch.npz
    python ktruss-explorer_gb300/selector.py collect --families large --count 24 --seed 4 --out data/selector_large.npz
    python ktruss-explorer_gb300/selector.py evaluate

`collect` generates seeded graphs - Erdos-Renyi, R-MAT scale 12-18, Barabasi-Albert, random
geometric (unit square, radius for an average degree of 8-64) and graphs with planted cliques -
and for each records the selector's 16 features (computed by the library on the device) and the
device time of all 36 schedules of the autotuner's grid (kt_engine_autotune).  `evaluate` trains
the network with the library's CUDA kernels on the training set and reports, on the held-out
set, the time of its choices against the exhaustively tuned best and the default schedule.
The data in data/ were measured on a GB300.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import ktruss_gb300 as kt  # noqa: E402

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
FAMILIES = ("er", "rmat", "ba", "rgg", "cliques")
# Unions of 16-128 graphs of the batch distribution (kt_gen_batch), as kt_engine_decompose_batch
# sees them: a separate training set, so that the network also knows batches.
BATCH_FAMILIES = ("batch",)
# Large R-MAT graphs (scale 19-23, edge factor 16 or 32, half of them with planted cliques): a
# separate training set where the oriented rows meet hubs of hundreds of thousands of neighbours.
LARGE_FAMILIES = ("rmat_large",)


def graph_spec(index: int, seed: int, families=FAMILIES) -> dict:
    """Deterministic recipe of training graph `index` of the set with this seed."""
    rng = np.random.default_rng([seed, index])
    fam = families[index % len(families)]
    if fam == "batch":
        return dict(family=fam, graphs=int(round(2 ** rng.uniform(4, 7))), n_min=500, n_max=50000,
                    seed=int(rng.integers(1, 2**31)))
    gseed = int(rng.integers(1, 2**31))
    logn = lambda lo, hi: int(round(2 ** rng.uniform(lo, hi)))
    if fam == "rmat_large":
        return dict(family=fam, scale=int(rng.integers(19, 24)), ef=int(rng.choice([16, 32])),
                    cliques=int(rng.choice([0, 8])), seed=gseed)
    if fam == "er":
        return dict(family=fam, n=logn(11, 17), degree=float(rng.uniform(4, 32)), seed=gseed)
    if fam == "rmat":
        return dict(family=fam, scale=int(rng.integers(12, 19)), ef=int(rng.choice([8, 16])), seed=gseed)
    if fam == "ba":
        return dict(family=fam, n=logn(11, 17), m=int(rng.choice([2, 4, 8, 16])), seed=gseed)
    if fam == "rgg":
        return dict(family=fam, n=logn(11, 16), degree=float(rng.uniform(8, 64)), seed=gseed)
    base = str(rng.choice(["er", "ba"]))
    return dict(family=fam, base=base, n=logn(11, 16), degree=float(rng.uniform(4, 16)), m=int(rng.choice([2, 4, 8])),
                count=int(rng.integers(1, 9)), min_size=8, max_size=int(rng.integers(16, 129)), seed=gseed)


def make_graph(spec: dict):
    """(num_nodes, u, v) of a spec, u < v."""
    f = spec["family"]
    if f == "batch":
        n, u, v, _ = kt.gen_batch(spec["graphs"], spec["n_min"], spec["n_max"], spec["seed"])
        return n, u, v
    if f == "er":
        n = spec["n"]
        return kt.gen_er(n, spec["degree"] / (n - 1), spec["seed"])
    if f == "rmat":
        return kt.gen_rmat(spec["scale"], spec["ef"], 0.57, 0.19, 0.19, spec["seed"])
    if f == "rmat_large":
        g = kt.gen_rmat(spec["scale"], spec["ef"], 0.57, 0.19, 0.19, spec["seed"])
        return kt.plant_cliques(*g, spec["cliques"], 64, 256, spec["seed"] + 1) if spec["cliques"] else g
    if f == "ba":
        return kt.gen_ba(spec["n"], spec["m"], spec["seed"])
    if f == "rgg":
        n = spec["n"]
        return kt.gen_rgg(n, math.sqrt(spec["degree"] / (math.pi * n)), spec["seed"])
    n = spec["n"]
    if spec["base"] == "er":
        g = kt.gen_er(n, spec["degree"] / (n - 1), spec["seed"])
    else:
        g = kt.gen_ba(n, spec["m"], spec["seed"])
    return kt.plant_cliques(*g, spec["count"], spec["min_size"], min(spec["max_size"], n), spec["seed"] + 1)


def collect(count: int, seed: int, device: int = 0, repeats: int = 1, log=None, families=FAMILIES) -> dict:
    """Features and the times of all grid schedules for `count` seeded graphs."""
    import torch

    torch.cuda.set_device(device)
    eng = kt.Engine(device)
    grid = kt.schedule_grid()
    feats = np.zeros((count, kt.SELECTOR_FEATURES), np.float32)
    times = np.zeros((count, kt.SELECTOR_SCHEDULES), np.float32)
    specs, edges = [], np.zeros(count, np.int64)
    t0 = time.time()
    for i in range(count):
        spec = graph_spec(i, seed, families)
        n, u, v = make_graph(spec)
        src = torch.from_numpy(np.concatenate([u, v]).view(np.int32)).cuda()
        dst = torch.from_numpy(np.concatenate([v, u]).view(np.int32)).cuda()
        torch.cuda.synchronize()
        feats[i] = eng.features(src.data_ptr(), dst.data_ptr(), src.numel(), n)
        _, table = eng.autotune(src.data_ptr(), dst.data_ptr(), src.numel(), n, candidates=grid, repeats=repeats)
        times[i] = [ms for _, ms in table]
        specs.append(json.dumps(spec, sort_keys=True))
        edges[i] = len(u)
        if log and (i + 1) % 100 == 0:
            log(f"{i + 1}/{count} graphs, {time.time() - t0:.0f} s")
    eng.close()
    return dict(features=feats, times=times, specs=np.array(specs), edges=edges)


def save(path: str, data: dict) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, **data)


def load(path: str) -> dict:
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def load_training() -> dict:
    """The training data in data/: the 2000 single graphs, plus the batch unions and the large
    R-MAT graphs when present."""
    d = load(os.path.join(DATA, "selector_train.npz"))
    for name in ("selector_batch.npz", "selector_large.npz"):
        extra = os.path.join(DATA, name)
        if os.path.exists(extra):
            b = load(extra)
            d = {k: np.concatenate([d[k], b[k]]) for k in ("features", "times", "specs", "edges")}
    return d


def train(data: dict, epochs: int = 300, batch: int = 64, lr: float = 3e-3, seed: int = 1, device: int = 0):
    """A selector trained on `data` by the library's CUDA kernels; returns (selector, epoch losses)."""
    sel = kt.Selector(device, seed)
    losses = sel.train(data["features"], data["times"], epochs=epochs, batch=batch, lr=lr, seed=seed)
    return sel, losses


def evaluate(sel, data: dict) -> dict:
    """Time of the selector's choices on `data` against the per-graph best (exhaustive autotuning),
    the default schedule and the single schedule that is best over the whole set."""
    t = data["times"].astype(np.float64)
    choice = np.array([kt.schedule_index(s) for s in sel.predict(data["features"])])
    rows = np.arange(len(t))
    chosen = t[rows, choice].sum()
    best = t.min(axis=1).sum()
    default = t[:, kt.schedule_index(kt.schedule_default())].sum()
    fixed = t.sum(axis=0)
    return {"graphs": int(len(t)), "chosen_ms": float(chosen), "tuned_ms": float(best), "default_ms": float(default),
            "best_fixed_ms": float(fixed.min()), "best_fixed": kt.schedule_grid()[int(fixed.argmin())].as_tuple(),
            "regret": float(chosen / best - 1.0), "gain_vs_default": float(default / chosen),
            "exact_choice": float(np.mean(choice == t.argmin(axis=1)))}


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--count", type=int, default=2000)
    c.add_argument("--seed", type=int, default=1)
    c.add_argument("--repeats", type=int, default=1)
    c.add_argument("--out", required=True)
    c.add_argument("--families", default="graphs", choices=["graphs", "batch", "large"],
                   help="graphs: ER, R-MAT, BA, RGG, planted cliques; batch: unions of batch graphs; "
                        "large: R-MAT scale 19-23")
    e = sub.add_parser("evaluate")
    e.add_argument("--train", default=None, help="training set (default: data/, with the batch unions)")
    e.add_argument("--heldout", default=os.path.join(DATA, "selector_heldout.npz"))
    e.add_argument("--epochs", type=int, default=300)
    args = ap.parse_args()
    if args.cmd == "collect":
        fams = {"batch": BATCH_FAMILIES, "large": LARGE_FAMILIES}.get(args.families, FAMILIES)
        d = collect(args.count, args.seed, repeats=args.repeats, log=lambda s: print(s, flush=True), families=fams)
        save(args.out, d)
        print(f"wrote {args.out}: {args.count} graphs", flush=True)
    else:
        t0 = time.time()
        sel, losses = train(load(args.train) if args.train else load_training(), epochs=args.epochs)
        r = evaluate(sel, load(args.heldout))
        r["train_s"] = time.time() - t0
        r["loss_first_last"] = [float(losses[0]), float(losses[-1])]
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
