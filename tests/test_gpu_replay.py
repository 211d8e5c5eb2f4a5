"""kt_engine_replay: the last decomposition or single-k call repeated through a CUDA graph of its
device pipeline (the reference's -w/-x repeat runs, kernel_ddc.cu:227-244).  Every replay must give
the first call's results bit for bit, whatever was left in the outputs, and a new call, schedule
or reservation must replace what is replayed."""
import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import both_directions

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _device_graph(torch, make):
    n, u, v = make()
    src, dst = both_directions(u, v)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
    return n, src, dst, dev(src), dev(dst)


GRAPHS = [
    ("rmat13", lambda: kt.gen_rmat(13, 16, 0.57, 0.19, 0.19, 31)),
    ("ba5000_cliques", lambda: kt.plant_cliques(*kt.gen_ba(5000, 8, 32), 2, 20, 40, 33)),
]


@pytest.mark.parametrize("name,make", GRAPHS, ids=[g[0] for g in GRAPHS])
def test_replayed_decomposition_is_identical(name, make, torch):
    n, src, dst, d_src, d_dst = _device_graph(torch, make)
    ref = oracle.decompose(n, src, dst, method="peel")
    eng = kt.Engine(0)
    d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
    first = eng.stats()
    launches = first.kernel_launches
    for i in range(3):
        d_out.fill_(-1)
        d_k.fill_(0)
        torch.cuda.synchronize()
        eng.replay()
        assert int(d_k.item()) == ref["k_max"], i
        assert np.array_equal(d_out.cpu().numpy().view(np.uint32), ref["truss"]), i
        st = eng.stats()
        assert (st.k_max, st.num_rounds, st.num_levels, st.triangles, st.walk_entries) == \
            (first.k_max, first.num_rounds, first.num_levels, first.triangles, first.walk_entries)
        assert st.last_ms > 0 and st.build_ms == 0
        assert st.kernel_launches > launches  # the graph's kernels are counted
        launches = st.kernel_launches
    assert eng.replay_mode() in ("cuda graph", "direct launches")


def test_replayed_single_k_truss(torch):
    n, src, dst, d_src, d_dst = _device_graph(torch, GRAPHS[1][1])
    ref = oracle.decompose(n, src, dst, method="peel")
    eng = kt.Engine(0)
    d_keep = torch.empty(len(src), dtype=torch.uint8, device="cuda")
    for k in (2, 3, 7, ref["k_max"], ref["k_max"] + 1):
        torch.cuda.synchronize()
        eng.ktruss(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, k, d_keep.data_ptr())
        d_keep.fill_(7)
        torch.cuda.synchronize()
        eng.replay()
        eng.replay()
        assert np.array_equal(d_keep.cpu().numpy(), (ref["truss"] >= k).astype(np.uint8)), k


def test_replay_follows_the_last_call_and_schedule(torch):
    n1, src1, dst1, s1, t1 = _device_graph(torch, GRAPHS[0][1])
    n2, src2, dst2, s2, t2 = _device_graph(torch, lambda: kt.gen_ws(6000, 10, 0.1, 34))
    ref1 = oracle.decompose(n1, src1, dst1, method="peel")
    ref2 = oracle.decompose(n2, src2, dst2, method="peel")
    eng = kt.Engine(0)
    o1 = torch.empty(len(src1), dtype=torch.int32, device="cuda")
    o2 = torch.empty(len(src2), dtype=torch.int32, device="cuda")
    k = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose(s1.data_ptr(), t1.data_ptr(), len(src1), n1, o1.data_ptr(), k.data_ptr())
    eng.replay()
    eng.decompose(s2.data_ptr(), t2.data_ptr(), len(src2), n2, o2.data_ptr(), k.data_ptr())
    o2.fill_(-1)
    torch.cuda.synchronize()
    eng.replay()  # the second graph now
    assert np.array_equal(o2.cpu().numpy().view(np.uint32), ref2["truss"])
    for sched in ((16, 8, 0, 0, 0), (4, 16, 85, 1, 2)):
        eng.set_schedule(*sched)
        o2.fill_(-1)
        torch.cuda.synchronize()
        eng.replay()
        assert np.array_equal(o2.cpu().numpy().view(np.uint32), ref2["truss"]), sched
    eng.reserve(4 * n2, 4 * len(src2))  # a new workspace: the pipeline is captured again
    o2.fill_(-1)
    torch.cuda.synchronize()
    eng.replay()
    assert np.array_equal(o2.cpu().numpy().view(np.uint32), ref2["truss"])
    assert np.array_equal(o1.cpu().numpy().view(np.uint32), ref1["truss"])


def test_replay_after_other_work_on_the_engine(torch):
    """Features of another graph and a symmetrize call in between rebuild the workspace; the
    replay still repeats the remembered call exactly."""
    n1, src1, dst1, s1, t1 = _device_graph(torch, GRAPHS[1][1])
    n2, src2, dst2, s2, t2 = _device_graph(torch, lambda: kt.gen_rmat(12, 16, 0.57, 0.19, 0.19, 37))
    ref1 = oracle.decompose(n1, src1, dst1, method="peel")
    eng = kt.Engine(0)
    o1 = torch.empty(len(src1), dtype=torch.int32, device="cuda")
    k = torch.zeros(1, dtype=torch.int32, device="cuda")
    so = torch.empty(2 * len(src2), dtype=torch.int32, device="cuda")
    do = torch.empty(2 * len(src2), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose(s1.data_ptr(), t1.data_ptr(), len(src1), n1, o1.data_ptr(), k.data_ptr())
    eng.replay()
    eng.features(s2.data_ptr(), t2.data_ptr(), len(src2), n2)
    eng.symmetrize(s2.data_ptr(), t2.data_ptr(), len(src2), n2, so.data_ptr(), do.data_ptr(), 2 * len(src2))
    o1.fill_(-1)
    torch.cuda.synchronize()
    eng.replay()
    assert int(k.item()) == ref1["k_max"]
    assert np.array_equal(o1.cpu().numpy().view(np.uint32), ref1["truss"])


def test_replay_needs_a_successful_call(torch):
    eng = kt.Engine(0)
    with pytest.raises(kt.KtrussError) as ei:
        eng.replay()
    assert ei.value.status == 1  # KT_ERR_INVALID_ARG
    # a call rejected by its input checks is not repeated
    d = torch.tensor([0, 1, 1, 1], dtype=torch.int32, device="cuda")  # (1,1) is a self loop
    out = torch.empty(4, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(kt.KtrussError):
        eng.decompose(d.data_ptr(), d.flip(0).data_ptr(), 4, 2, out.data_ptr(), 0)
    with pytest.raises(kt.KtrussError) as ei:
        eng.replay()
    assert ei.value.status == 1


def test_cli_repeat_runs_replay(tmp_path):
    """-w 1 -x 3: four runs of the single-k truss, the last three through the replay."""
    n, u, v = kt.plant_cliques(*kt.gen_ba(3000, 6, 35), 2, 12, 30, 36)
    src, dst = both_directions(u, v)
    ref = oracle.decompose(n, src, dst, method="peel")
    g = kt.COOGraph(n, src, dst)
    cfg = kt.parse_args(["-k", "6", "-w", "1", "-x", "3", "-v", "0"])
    t = kt.ktruss(g, cfg)
    keep = ref["truss"] >= 6
    assert t.num_edges == int(keep.sum())
    got = set(zip(t.src_idx.tolist(), t.dst_idx.tolist()))
    want = {(int(s), int(d)) for s, d, kk in zip(src, dst, keep) if kk}
    assert got == want
