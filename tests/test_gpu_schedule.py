"""Every kernel schedule (support group, chunk width, compaction threshold) gives the oracle's
truss numbers bit for bit; invalid schedules are rejected."""
import itertools

import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import both_directions

pytestmark = pytest.mark.gpu

GRAPHS = [
    ("rmat13", lambda: kt.gen_rmat(13, 16, 0.57, 0.19, 0.19, 11)),
    ("ba6000_cliques", lambda: kt.plant_cliques(*kt.gen_ba(6000, 4, 12), 3, 16, 48, 13)),
    ("ws8000", lambda: kt.gen_ws(8000, 10, 0.1, 14)),
]

SCHEDULES = list(itertools.product((0, 4, 8, 16, 32), (8, 16, 32), (0, 50, 85), (0, 1, 50), (0,))) + \
    list(itertools.product((0, 8), (8, 32), (0, 85), (0, 50), (1, 2)))


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("name,make", GRAPHS, ids=[g[0] for g in GRAPHS])
def test_every_schedule_matches_oracle(name, make, torch):
    n, u, v = make()
    src, dst = both_directions(u, v)
    ref = oracle.decompose(n, src, dst, method="peel")
    eng = kt.Engine(0)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    for sched in SCHEDULES:
        g, w, c, rc, pb = sched
        eng.set_schedule(*sched)
        assert eng.schedule().as_tuple() == sched
        d_out.fill_(-1)
        torch.cuda.synchronize()  # the engine runs on its own stream
        eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
        assert int(d_k.item()) == ref["k_max"], sched
        assert np.array_equal(d_out.cpu().numpy().view(np.uint32), ref["truss"]), sched
        st = eng.stats()
        assert st.compactions == 0 or c != 0


@pytest.mark.parametrize("w,rc,pb", [(8, 0, 0), (16, 0, 2), (32, 50, 2), (8, 1, 1)])
def test_single_k_with_narrow_chunks(w, rc, pb, torch):
    n, u, v = kt.plant_cliques(*kt.gen_ba(5000, 8, 21), 2, 20, 40, 22)
    src, dst = both_directions(u, v)
    ref = oracle.decompose(n, src, dst, method="peel")
    eng = kt.Engine(0)
    eng.set_schedule(16, w, 85, rc, pb)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    keep = torch.empty(len(src), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for k in (3, 5, ref["k_max"], ref["k_max"] + 1):
        eng.ktruss(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, k, keep.data_ptr())
        assert np.array_equal(keep.cpu().numpy().astype(bool), ref["truss"] >= k), k


def test_batch_with_narrow_chunks(torch):
    n, u, v, off = kt.gen_batch(24, 500, 4000, 31)
    src, dst = both_directions(u, v)
    eng = kt.Engine(0)
    eng.set_schedule(4, 8, 50, 25, 2)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_off = torch.from_numpy(off.view(np.int32)).cuda()
    d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(len(off) - 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose_batch(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_off.data_ptr(), len(off) - 1,
                        d_out.data_ptr(), d_k.data_ptr())
    ref = oracle.decompose(n, src, dst, method="peel")
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), ref["truss"])


@pytest.mark.parametrize("bad", [(2, 32, 85, 0, 0), (64, 32, 85, 0, 0), (8, 4, 85, 0, 0), (8, 64, 85, 0, 0),
                                 (8, 32, 100, 0, 0), (8, 32, 85, 101, 0), (8, 32, 85, 50, 3)])
def test_invalid_schedule_rejected(bad):
    eng = kt.Engine(0)
    before = eng.schedule().as_tuple()
    with pytest.raises(kt.KtrussError) as ei:
        eng.set_schedule(*bad)
    assert ei.value.status == 1  # KT_ERR_INVALID_ARG
    assert eng.schedule().as_tuple() == before


def _clique_union(sizes):
    us, vs, base = [], [], 0
    for s in sizes:
        iu, iv = np.triu_indices(s, 1)
        us.append(iu + base)
        vs.append(iv + base)
        base += s
    return base, np.concatenate(us).astype(np.uint32), np.concatenate(vs).astype(np.uint32)


@pytest.mark.parametrize("sizes", [[20] * 300, [100, 100, 64]], ids=["many_small", "few_large"])
@pytest.mark.parametrize("w,rc,pb", [(8, 0, 0), (32, 0, 2), (8, 50, 2)])
def test_chunk_buffer_overflow(sizes, w, rc, pb, torch):
    """A level whose whole frontier is every edge of many cliques needs more chunks than the
    buffer holds (m + 4096 on an engine sized for this graph): the rest is walked by warps (many
    edges) or blocks (few edges).  Every edge of a c-clique has truss number c."""
    n, u, v = _clique_union(sizes)
    m = len(u)
    chunks = sum((s * (s - 1) // 2) * -(-(s - 1) // w) for s in sizes)
    if w == 8:
        assert chunks > m + 4096  # the buffer overflows
    src, dst = both_directions(u, v)
    expect = np.concatenate([np.full(s * (s - 1) // 2, s, np.uint32) for s in sizes])
    eng = kt.Engine(0)
    eng.reserve(n, len(src))
    eng.set_schedule(8, w, 85, rc, pb)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
    out = d_out.cpu().numpy().view(np.uint32)
    assert int(d_k.item()) == max(sizes)
    assert np.array_equal(out[:m], expect) and np.array_equal(out[m:], expect)


def test_vertex_hash_count_on_rows_beyond_its_tables(torch):
    """The vertex-centric count (support group 0) on a 2,100-vertex clique with a pendant path: rows
    of up to 2,099 oriented entries exceed the 2,048 of a block table (searched in HBM instead), the
    top vertices have more in-edges than one block item takes (several items per vertex), and the
    path's vertices go to single warps.  Clique edges have truss number 2,100, path edges 2."""
    s_ = 2100
    iu, iv = np.triu_indices(s_, 1)
    path_u = np.arange(s_ - 1, s_ + 40, dtype=np.int64)
    u = np.concatenate([iu, path_u]).astype(np.uint32)
    v = np.concatenate([iv, path_u + 1]).astype(np.uint32)
    n = s_ + 41
    src, dst = both_directions(u, v)
    eng = kt.Engine(0)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    want = np.where(np.arange(len(u)) < len(iu), s_, 2).astype(np.uint32)
    for g in (0, 8):
        eng.set_schedule(g, 32, 85, 50, 0)
        d_out.fill_(-1)
        torch.cuda.synchronize()
        eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
        out = d_out.cpu().numpy().view(np.uint32)
        assert int(d_k.item()) == s_, g
        assert np.array_equal(out[: len(u)], want) and np.array_equal(out[len(u):], want), g
        assert eng.stats().triangles == s_ * (s_ - 1) * (s_ - 2) // 6, g
    eng.close()
