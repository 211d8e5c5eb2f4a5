"""The reference's variant switches (-d, -f, -r, -b, -t, -y; config.h:51-161) select distinct kernel
paths for single-k truss calls, and every path gives the oracle's k-truss:
  directed-by-degree / directed-by-index   the engine's peel on the degree- or id-oriented CSR
                                           (recount all: recount rounds allowed; affected:
                                           support decrements only)
  undirected                               count-and-delete passes with counts capped at k-2
  tiled-coocsr                             count-and-delete passes over the column-tiled index
The count-and-delete paths take exactly the reference's passes (the oracle's pass log)."""
import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import both_directions, edge_keys

pytestmark = pytest.mark.gpu

GRAPHS = [
    ("rmat13", lambda: kt.gen_rmat(13, 16, 0.57, 0.19, 0.19, 31)),
    ("ba4000_cliques", lambda: kt.plant_cliques(*kt.gen_ba(4000, 6, 32), 3, 12, 40, 33)),
    ("ws6000", lambda: kt.gen_ws(6000, 10, 0.1, 34)),
]

VARIANTS = [("directed-by-degree", "coocsr", "all"), ("directed-by-degree", "coocsr", "affected"),
            ("directed-by-index", "coocsr", "all"), ("directed-by-index", "coocsr", "affected"),
            ("undirected", "coocsr", "all"), ("undirected", "coocsr", "affected"),
            ("directed-by-degree", "tiled-coocsr", "all"), ("undirected", "tiled-coocsr", "affected")]
DIRECTEDNESS = {"undirected": oracle.UNDIRECTED, "directed-by-index": oracle.DIRECTED_BY_INDEX,
                "directed-by-degree": oracle.DIRECTED_BY_DEGREE}


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("name,make", GRAPHS, ids=[g[0] for g in GRAPHS])
def test_every_variant_matches_oracle(name, make, torch):
    n, u, v = make()
    src, dst = both_directions(u, v)
    k_max = oracle.decompose(n, src, dst)["k_max"]
    eng = kt.Engine(0)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_keep = torch.zeros(len(src), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for k in sorted({1, 2, 3, 4, max(3, k_max // 2), k_max, k_max + 1}):
        os_, od, alive = oracle.ktruss(n, src, dst, k, pass_log=True)
        want = edge_keys(os_, od)
        for d, f, r in VARIANTS:
            eng.set_variant(d, f, r, block_size=256, num_tiles=4, num_parallel_tiles=2)
            d_keep.fill_(7)
            torch.cuda.synchronize()
            eng.ktruss(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, k, d_keep.data_ptr())
            keep = d_keep.cpu().numpy()
            assert set(np.unique(keep)) <= {0, 1}, (k, d, f, r)
            keep = keep.astype(bool)
            assert np.array_equal(edge_keys(src[keep], dst[keep]), want), (k, d, f, r)
            st = eng.stats()
            if k >= 3 and (d == "undirected" or f == "tiled-coocsr"):
                # the reference's own pass count for this variant (kernel_duc.cu / kernel_ddt.cu loops)
                ref_d = DIRECTEDNESS[d] if f == "coocsr" else oracle.DIRECTED_BY_DEGREE
                _, _, ref_alive = oracle.ktruss(n, src, dst, k, ref_d, oracle.RECOUNT_ALL, pass_log=True)
                assert st.num_rounds == len(ref_alive), (k, d, f, r, st.num_rounds, len(ref_alive))
    eng.close()


def test_variant_switches_are_validated_and_kept(torch):
    eng = kt.Engine(0)
    v = eng.variant()
    assert (v.directedness, v.input_format, v.recount, v.block_size, v.num_tiles, v.num_parallel_tiles) == \
        (2, 0, 0, 512, 8, 8)
    eng.set_variant("undirected", "tiled-coocsr", "affected", 128, 16, 4)
    v = eng.variant()
    assert (v.directedness, v.input_format, v.recount, v.block_size, v.num_tiles, v.num_parallel_tiles) == \
        (0, 1, 1, 128, 16, 4)
    for bad in (dict(block_size=0), dict(block_size=2048), dict(num_tiles=0), dict(num_parallel_tiles=0)):
        with pytest.raises(kt.KtrussError):
            eng.set_variant(**bad)
    eng.close()


def test_variant_repeat_runs_replay_directly(torch):
    """Count-and-delete passes read a flag per pass, so their repeat runs are launched directly
    (not captured as a CUDA graph) and give the same k-truss."""
    n, u, v = kt.gen_rmat(12, 16, 0.57, 0.19, 0.19, 35)
    src, dst = both_directions(u, v)
    eng = kt.Engine(0)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_keep = torch.zeros(len(src), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for d, f in (("undirected", "coocsr"), ("directed-by-degree", "tiled-coocsr"), ("directed-by-index", "coocsr")):
        eng.set_variant(d, f, "all")
        eng.ktruss(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, 5, d_keep.data_ptr())
        first = d_keep.clone()
        eng.replay()
        eng.replay()
        assert torch.equal(d_keep, first), (d, f)
        assert eng.replay_mode() == ("cuda graph" if d == "directed-by-index" else "direct launches"), (d, f)
    eng.close()


def test_tiled_calls_around_a_batch_that_grows_the_default_engine_staging():
    """The host-buffer calls share one engine: a tiled single-k call (its tile table), a batch call
    with more graphs than any before it (its staging grows), and the tiled call again, which must
    still find its own table and the same truss."""
    n, u, v = kt.gen_rmat(11, 12, 0.57, 0.19, 0.19, 41)
    g = kt.COOGraph.from_undirected(n, u, v)
    cfg = kt.Config(k=5, input_format="tiled-coocsr", num_tiles=4, num_parallel_tiles=2)
    first = kt.ktruss(g, cfg).canonical()
    # more graphs than any other test's batch, so that the staging grows whatever ran before
    bn, bu, bv, off = kt.gen_batch(5000, 64, 128, 43)
    bs, bd = both_directions(bu, bv)
    truss, kmax = kt.decompose_batch(bs, bd, bn, off)
    assert len(kmax) == 5000
    again = kt.ktruss(g, cfg).canonical()
    assert np.array_equal(first, again)
    os_, od = oracle.ktruss(n, g.src_idx, g.dst_idx, 5)
    assert np.array_equal(first, edge_keys(os_, od))
