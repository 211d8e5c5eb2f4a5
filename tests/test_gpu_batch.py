"""Batched decomposition: many graphs on disjoint vertex ranges in one call; every graph's truss
numbers and k_max must equal its own decomposition (checked against the oracle per graph)."""
import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import both_directions

pytestmark = pytest.mark.gpu


def _per_graph_oracle(n, u, v, off):
    truss = np.zeros(len(u), np.uint32)
    kmax = np.zeros(len(off) - 1, np.uint32)
    gid = np.searchsorted(off, u, side="right") - 1
    for g in range(len(off) - 1):
        sel = np.nonzero(gid == g)[0]
        if len(sel) == 0:
            continue
        lu, lv = u[sel] - off[g], v[sel] - off[g]
        s, d = both_directions(lu, lv)
        r = oracle.decompose(int(off[g + 1] - off[g]), s, d, method="peel")
        truss[sel] = r["truss"][: len(sel)]
        kmax[g] = r["k_max"]
    return truss, kmax


def test_benchmarked_batch_sample_matches_oracle():
    """The benchmarked batch itself (4096 graphs, n log-uniform in [500, 50000], half Barabasi-Albert,
    half Watts-Strogatz, 0-3 planted cliques of 8-64 vertices, seed 1), decomposed in one call; 96
    graphs spread over it (every 43rd) are checked against the oracle, which runs in a process pool
    started with spawn."""
    n, u, v, off = kt.gen_batch(4096, 500, 50000, 1)
    src, dst = both_directions(u, v)
    truss, kmax = kt.decompose_batch(src, dst, n, off)
    m = len(u)
    pick = np.arange(0, 4096, 43)
    lo = np.searchsorted(u, off[pick], side="left")
    hi = np.searchsorted(u, off[pick + 1], side="left")
    jobs = []
    for g, a, b in zip(pick, lo, hi):
        lu, lv = u[a:b] - off[g], v[a:b] - off[g]
        s, d = both_directions(lu, lv)
        jobs.append((int(off[g + 1] - off[g]), s, d))
    assert max(j[0] for j in jobs) > 25000 and sum(len(j[1]) for j in jobs) > 4_000_000
    results = oracle.decompose_many(jobs)
    for (g, a, b), (t_ref, k_ref) in zip(zip(pick, lo, hi), results):
        assert kmax[g] == k_ref, f"graph {g}: k_max {kmax[g]} != {k_ref}"
        assert np.array_equal(truss[a:b], t_ref[: b - a]), f"graph {g}: truss numbers differ"
        assert np.array_equal(truss[m + a:m + b], t_ref[: b - a]), f"graph {g}: reverse entries differ"


@pytest.mark.parametrize("seed", [5, 6])
def test_batch_matches_each_graph(seed):
    n, u, v, off = kt.gen_batch(48, 64, 2500, seed)
    src, dst = both_directions(u, v)
    truss, kmax = kt.decompose_batch(src, dst, n, off)
    ref_t, ref_k = _per_graph_oracle(n, u, v, off)
    assert np.array_equal(truss[: len(u)], ref_t) and np.array_equal(truss[len(u):], ref_t)
    assert np.array_equal(kmax, ref_k)


def test_batch_with_empty_graphs_and_device_api():
    torch = pytest.importorskip("torch")
    # three graphs: K5, no edges, a triangle
    u = np.array([0, 0, 0, 0, 1, 1, 1, 2, 2, 3, 7, 7, 8], np.uint32)
    v = np.array([1, 2, 3, 4, 2, 3, 4, 3, 4, 4, 8, 9, 9], np.uint32)
    off = np.array([0, 5, 7, 10], np.uint32)
    src, dst = both_directions(u, v)
    eng = kt.Engine(0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
    d_src, d_dst, d_off = t(src), t(dst), t(off)
    d_out = torch.zeros(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.full((3,), 99, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose_batch(d_src.data_ptr(), d_dst.data_ptr(), len(src), 10, d_off.data_ptr(), 3, d_out.data_ptr(),
                        d_k.data_ptr())
    assert d_k.cpu().tolist() == [5, 0, 3]
    assert set(d_out.cpu().tolist()) == {5, 3}
    eng.close()


def test_batch_rejects_cross_graph_entries():
    u = np.array([0, 1], np.uint32)
    v = np.array([1, 3], np.uint32)
    src, dst = both_directions(u, v)
    with pytest.raises(kt.KtrussError) as ei:
        kt.decompose_batch(src, dst, 4, np.array([0, 2, 4], np.uint32))
    assert ei.value.status == 1


def test_batch_autotuner_keeps_a_schedule_that_decomposes_the_batch():
    """kt_engine_autotune_batch times candidates as batch decompositions of a sample batch; the
    schedule it keeps decomposes another batch of the distribution exactly."""
    torch = pytest.importorskip("torch")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
    ns, us, vs, _ = kt.gen_batch(24, 300, 2000, 41)
    ss, sd = both_directions(us, vs)
    eng = kt.Engine(0)
    cands = [(4, 8, 0, 50, 0), (8, 16, 85, 0, 0), (16, 32, 0, 0, 0)]
    d_ss, d_sd = t(ss), t(sd)
    torch.cuda.synchronize()
    best, table = eng.autotune(d_ss.data_ptr(), d_sd.data_ptr(), len(ss), ns, candidates=cands, repeats=2, batch=True)
    assert best.as_tuple() in cands and len(table) == 3 and all(ms > 0 for _, ms in table)
    assert best.as_tuple() == min(table, key=lambda x: x[1])[0].as_tuple()
    assert eng.schedule().as_tuple() == best.as_tuple()
    n, u, v, off = kt.gen_batch(20, 300, 2000, 42)
    src, dst = both_directions(u, v)
    d_src, d_dst, d_off = t(src), t(dst), t(off)
    d_out = torch.zeros(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(len(off) - 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose_batch(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_off.data_ptr(), len(off) - 1,
                        d_out.data_ptr(), d_k.data_ptr())
    truss, kmax = _per_graph_oracle(n, u, v, off)
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32)[: len(u)], truss)
    assert np.array_equal(d_k.cpu().numpy().view(np.uint32), kmax)
    eng.close()


def test_batch_kmax_with_entries_in_any_order():
    """Per-graph k_max does not depend on the entries being listed graph by graph (a warp's entries
    then span many graphs), and a cross-graph entry among one graph's entries is still found."""
    n, u, v, off = kt.gen_batch(40, 64, 800, 9)
    src, dst = both_directions(u, v)
    truss, kmax = kt.decompose_batch(src, dst, n, off)
    perm = np.random.default_rng(3).permutation(len(src))
    truss_p, kmax_p = kt.decompose_batch(src[perm], dst[perm], n, off)
    assert np.array_equal(kmax_p, kmax)
    assert np.array_equal(truss_p, truss[perm])
    # two 12-cliques; one entry pair joins them, placed among the first clique's entries
    iu, iv = np.triu_indices(12, 1)
    cu = np.concatenate([iu, iu + 12]).astype(np.uint32)
    cv = np.concatenate([iv, iv + 12]).astype(np.uint32)
    s2, d2 = both_directions(cu, cv)
    s2 = np.insert(s2, 40, [3, 15]).astype(np.uint32)
    d2 = np.insert(d2, 40, [15, 3]).astype(np.uint32)
    with pytest.raises(kt.KtrussError) as ei:
        kt.decompose_batch(s2, d2, 24, np.array([0, 12, 24], np.uint32))
    assert ei.value.status == 1


def test_batch_kmax_of_many_tiny_graphs():
    """Hundreds of graphs of 6-30 entries each, so that every 32-entry step of a warp spans several
    graphs: each clique K_s is its own graph with k_max s (K_2 and K_1 give 2 and 0)."""
    rng = np.random.default_rng(12)
    sizes = rng.integers(1, 7, 400)
    us, vs, off = [], [], [0]
    for s in sizes:
        iu, iv = np.triu_indices(int(s), 1)
        us.append(iu + off[-1])
        vs.append(iv + off[-1])
        off.append(off[-1] + int(s))
    u = np.concatenate(us).astype(np.uint32)
    v = np.concatenate(vs).astype(np.uint32)
    off = np.array(off, np.uint32)
    src, dst = both_directions(u, v)
    truss, kmax = kt.decompose_batch(src, dst, int(off[-1]), off)
    want = np.where(sizes >= 2, sizes, 0)
    assert np.array_equal(kmax, want.astype(np.uint32))
    g = np.searchsorted(off, u, side="right") - 1
    assert np.array_equal(truss[: len(u)], sizes[g].astype(np.uint32))
