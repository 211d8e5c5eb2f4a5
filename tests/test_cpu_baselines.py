"""The CPU legs of the benchmark, on the CPU: the whole-batch run of the reference algorithm (one
process per graph over shared memory) agrees with the oracle graph by graph, the timed repeat runs
of the reference loop on host threads give the serial loop's k-truss, and the stratified estimate
of a complete CPU decomposition covers the whole chain once."""
import hashlib
import os
import sys

import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import ROOT, both_directions, edge_keys

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_batch_processes_match_the_oracle_per_graph():
    n, u, v, off = kt.gen_batch(24, 300, 6000, 9)
    res, secs, workers = oracle.decompose_batch_processes(u, v, off, workers=3)
    assert len(res) == 24 and secs > 0 and workers == 3
    lo, hi = np.searchsorted(u, off[:-1]), np.searchsorted(u, off[1:])
    for g, k_max, sha in sorted(res):
        lu, lv = u[lo[g]:hi[g]] - off[g], v[lo[g]:hi[g]] - off[g]
        s, d = both_directions(lu, lv)
        r = oracle.decompose(int(off[g + 1] - off[g]), s, d, method="peel", threads=1)
        assert k_max == r["k_max"], g
        assert sha == hashlib.sha256(r["truss"][: len(lu)].astype("<u4").tobytes()).hexdigest(), g


def test_peel_processes_on_graphs_in_generator_order():
    """The held-out set's CPU leg: graphs listed one after another with their edges in generator
    order (not canonical), decomposed by the exact peel, one process per graph; the same k_max and
    truss hashes as the chain."""
    parts = [kt.gen_rmat(9, 8, 0.57, 0.19, 0.19, 3), kt.gen_ba(700, 4, 5), kt.gen_ws(500, 10, 0.1, 6)]
    us, vs, off = [], [], [0]
    for n, u, v in parts:
        us.append(v.astype(np.uint64) + off[-1])  # (v, u): sources not sorted within a graph
        vs.append(u.astype(np.uint64) + off[-1])
        off.append(off[-1] + n)
    u, v, off = np.concatenate(us), np.concatenate(vs), np.array(off, np.uint32)
    peel, _, _ = oracle.decompose_batch_processes(u, v, off, workers=2, per_task=1, method="peel")
    chain, _, _ = oracle.decompose_batch_processes(u, v, off, workers=2, per_task=1, method="chain")
    assert sorted(peel) == sorted(chain) and len(peel) == 3


@pytest.mark.parametrize("k", [3, 5, 9])
def test_threaded_repeat_runs_equal_the_serial_loop(k):
    n, u, v = oracle.gen_rmat(12, 16, 0.57, 0.19, 0.19, 4)
    src, dst = both_directions(u, v)
    os_, od, secs, passes = oracle.ktruss_runs(n, src, dst, k, 3, 4)
    ref_s, ref_d, alive = oracle.ktruss(n, src, dst, k, pass_log=True)
    assert np.array_equal(edge_keys(os_, od), edge_keys(ref_s, ref_d))
    assert len(secs) == 3 and (passes == len(alive)).all()


def test_decomposition_estimate_covers_every_level_once():
    n, u, v = oracle.gen_rmat(11, 16, 0.57, 0.19, 0.19, 5)
    src, dst = both_directions(u, v)
    est = bench.decomposition_estimate(n, len(u), src, dst, threads=2, strata=3)
    rows = est["strata"]
    assert abs(sum(r["group_volume_share"] for r in rows) - 1.0) < 1e-9
    covered = [k for r in rows for k in range(r["levels"][0], r["levels"][1] + 1)]
    assert covered == sorted(set(covered)) and covered[0] == 3
    assert all(r["levels"][0] <= r["k"] <= r["levels"][1] for r in rows)
    assert est["chain_seconds_extrapolated"] > 0


def test_workload_config_is_the_same_for_both_arms():
    a = bench.workload_config("rmat20", 1 << 20, 15701019)
    assert a == bench.workload_config("rmat20", 1 << 20, 15701019)
    assert set(a) == {"workload", "n", "m", "l2"}
