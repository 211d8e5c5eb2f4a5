"""The benchmarked single-graph workloads pinned to the oracle: the headline R-MAT 20 (edge factor
16, seed 1) and the stress R-MAT 24 (edge factor 32, seed 1, 16 planted cliques).

tests/golden/rmat20_seed1.json and rmat24_seed1.json hold the oracle's decompositions of the graphs
as hashes and counts (tests/golden/make_headline_fixture.py, make_stress_fixture.py).  On the CPU:
the oracle's generator makes exactly the engine generator's graphs, the R-MAT 20 fixture's edge
list is the one both make, and both fixtures are self-consistent.  On the GPU: the engine's
decomposition of each graph, through the C ABI, has the fixture's truss numbers (hash and
histogram), k_max, peel rounds and the reference schedule's pass statistics."""
import hashlib
import json
import os

import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import GOLDEN

FIXTURE = os.path.join(GOLDEN, "rmat20_seed1.json")
STRESS = os.path.join(GOLDEN, "rmat24_seed1.json")


def _fixture(path=FIXTURE):
    with open(path) as f:
        return json.load(f)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).astype("<u4").tobytes()).hexdigest()


@pytest.mark.parametrize("args", [(10, 16, 0.57, 0.19, 0.19, 1), (14, 8, 0.45, 0.15, 0.15, 7),
                                  (16, 16, 0.57, 0.19, 0.19, 3), (12, 32, 0.25, 0.25, 0.25, 11)])
def test_oracle_generator_equals_engine_generator(args):
    n1, u1, v1 = kt.gen_rmat(*args)
    n2, u2, v2 = oracle.gen_rmat(*args)
    assert n1 == n2 and np.array_equal(u1, u2) and np.array_equal(v1, v2)


def test_fixture_edge_list_is_the_generated_graph():
    fx = _fixture()
    g = fx["graph"]
    n, u, v = oracle.gen_rmat(g["scale"], g["edge_factor"], g["a"], g["b"], g["c"], g["seed"])
    assert n == fx["num_nodes"] and len(u) == fx["num_edges"]
    assert _sha(np.stack([u, v], 1)) == fx["edges_sha256"]


@pytest.mark.parametrize("path", [FIXTURE, STRESS])
def test_fixture_is_self_consistent(path):
    fx = _fixture(path)
    assert sum(fx["histogram"].values()) == fx["num_edges"]
    assert max(int(k) for k in fx["histogram"]) == fx["k_max"]
    assert sum(p for _, p, _ in fx["levels"]) == fx["plain_passes"]
    assert sum(a for _, _, a in fx["levels"]) == fx["plain_alive_sum"]
    assert fx["levels"][0][:2] == [3, 1] and fx["levels"][0][2] == fx["num_edges"]
    assert fx["levels"][-1][0] == fx["k_max"] + 1


@pytest.mark.gpu
def test_engine_decomposition_of_the_headline_graph_matches_the_oracle():
    torch = pytest.importorskip("torch")
    fx = _fixture()
    g = fx["graph"]
    n, u, v = kt.gen_rmat(g["scale"], g["edge_factor"], g["a"], g["b"], g["c"], g["seed"])
    m = len(u)
    assert _sha(np.stack([u, v], 1)) == fx["edges_sha256"]
    src = np.concatenate([u, v]).astype(np.uint32)
    dst = np.concatenate([v, u]).astype(np.uint32)
    eng = kt.Engine(0)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_out = torch.zeros(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
    s = eng.stats()
    truss = d_out.cpu().numpy().view(np.uint32)
    eng.close()
    assert int(d_k.item()) == fx["k_max"] == s.k_max
    assert np.array_equal(truss[:m], truss[m:])
    hist = np.bincount(truss[:m])
    assert {str(i): int(c) for i, c in enumerate(hist) if c} == fx["histogram"]
    assert _sha(truss[:m]) == fx["truss_sha256"]
    assert s.plain_passes == fx["plain_passes"] and s.plain_alive_sum == fx["plain_alive_sum"]
    assert s.num_rounds == fx["peel_rounds"]


@pytest.mark.gpu
def test_host_buffer_decomposition_of_the_headline_graph_matches_the_oracle():
    fx = _fixture()
    g = fx["graph"]
    n, u, v = kt.gen_rmat(g["scale"], g["edge_factor"], g["a"], g["b"], g["c"], g["seed"])
    truss, k_max = kt.decompose(kt.COOGraph.from_undirected(n, u, v))
    assert k_max == fx["k_max"]
    assert _sha(truss[: len(u)]) == fx["truss_sha256"]


@pytest.mark.gpu
def test_engine_decomposition_of_the_stress_graph_matches_the_oracle():
    """R-MAT 24 with cliques (512.7 M edges; about 12 GB of input and 80 GB of workspace on the
    device): its 8,930 peel rounds run in the two-blocks-per-SM build, with compactions and recount
    rounds, and every truss number equals the oracle's."""
    torch = pytest.importorskip("torch")
    fx = _fixture(STRESS)
    g = fx["graph"]
    n, u, v = kt.gen_rmat(g["scale"], g["edge_factor"], g["a"], g["b"], g["c"], g["seed"])
    count, lo, hi = g["cliques"]
    n, u, v = kt.plant_cliques(n, u, v, count, lo, hi, g["clique_seed"])
    m = len(u)
    assert n == fx["num_nodes"] and m == fx["num_edges"]
    assert _sha(np.stack([u, v], 1)) == fx["edges_sha256"]
    d_src = torch.from_numpy(np.concatenate([u, v]).view(np.int32)).cuda()
    d_dst = torch.from_numpy(np.concatenate([v, u]).view(np.int32)).cuda()
    del u, v
    d_out = torch.zeros(2 * m, dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    eng = kt.Engine(0)
    torch.cuda.synchronize()
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), 2 * m, n, d_out.data_ptr(), d_k.data_ptr())
    s = eng.stats()
    eng.close()
    del d_src, d_dst
    truss = d_out[:m].cpu().numpy().view(np.uint32)
    assert torch.equal(d_out[:m], d_out[m:])
    del d_out
    assert int(d_k.item()) == fx["k_max"] == s.k_max
    assert _sha(truss) == fx["truss_sha256"]
    hist = np.bincount(truss)
    assert {str(i): int(c) for i, c in enumerate(hist) if c} == fx["histogram"]
    assert s.plain_passes == fx["plain_passes"] and s.plain_alive_sum == fx["plain_alive_sum"]
    assert s.num_rounds == fx["peel_rounds"]
