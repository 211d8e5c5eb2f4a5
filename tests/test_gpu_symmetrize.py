"""kt_engine_symmetrize: an arbitrary entry list (one or both directions, duplicates, self loops)
made into the symmetric simple graph on the device, against numpy's unique, and decomposed."""
import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def _expected(src, dst):
    s, d = src.astype(np.int64), dst.astype(np.int64)
    keep = s != d
    lo, hi = np.minimum(s, d)[keep], np.maximum(s, d)[keep]
    pairs = np.unique(lo << 32 | hi)
    lo, hi = (pairs >> 32).astype(np.uint32), (pairs & 0xffffffff).astype(np.uint32)
    return np.concatenate([lo, hi]), np.concatenate([hi, lo])


def _run(torch, eng, src, dst, n, capacity=None):
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
    cap = 2 * len(src) if capacity is None else capacity
    so = torch.full((max(cap, 1),), -1, dtype=torch.int32, device="cuda")
    do = torch.full((max(cap, 1),), -1, dtype=torch.int32, device="cuda")
    d_src, d_dst = dev(src), dev(dst)
    torch.cuda.synchronize()
    count = eng.symmetrize(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, so.data_ptr(), do.data_ptr(), cap)
    return count, so.cpu().numpy().view(np.uint32), do.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("seed,n,entries", [(1, 50, 400), (2, 3000, 40000), (3, 1 << 20, 300000)])
def test_matches_numpy_unique(seed, n, entries, torch):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, entries).astype(np.uint32)
    dst = rng.integers(0, n, entries).astype(np.uint32)
    dup = rng.integers(0, entries, entries // 4)  # repeated entries, some reversed
    src = np.concatenate([src, dst[dup[::2]], src[dup[1::2]]])
    dst = np.concatenate([dst, src[dup[::2]], dst[dup[1::2]]])
    src[:10] = dst[:10]  # self loops
    es, ed = _expected(src, dst)
    count, so, do = _run(torch, kt.Engine(0), src, dst, n)
    assert count == len(es)
    assert np.array_equal(so[:count], es) and np.array_equal(do[:count], ed)


def test_one_direction_graph_decomposes_like_the_oracle(torch):
    n, u, v = kt.plant_cliques(*kt.gen_ba(4000, 6, 41), 2, 15, 30, 42)
    rng = np.random.default_rng(43)
    flip = rng.random(len(u)) < 0.5
    src = np.where(flip, v, u).astype(np.uint32)  # each edge once, in a random direction
    dst = np.where(flip, u, v).astype(np.uint32)
    eng = kt.Engine(0)
    count, so, do = _run(torch, eng, src, dst, n)
    assert count == 2 * len(u)
    ref = oracle.decompose(n, so[:count], do[:count], method="peel")
    truss, k_max = kt.decompose(kt.COOGraph(n, so[:count], do[:count]))
    assert k_max == ref["k_max"] and np.array_equal(truss, ref["truss"])


def test_capacity_and_bad_ids(torch):
    eng = kt.Engine(0)
    src = np.array([0, 1, 2, 2], np.uint32)
    dst = np.array([1, 2, 0, 2], np.uint32)
    with pytest.raises(kt.KtrussError) as ei:
        _run(torch, eng, src, dst, 3, capacity=5)
    assert ei.value.status == 4  # KT_ERR_CAPACITY: 6 entries needed
    count, so, do = _run(torch, eng, src, dst, 3, capacity=6)
    assert count == 6 and list(so[:6]) == [0, 0, 1, 1, 2, 2] and list(do[:6]) == [1, 2, 2, 0, 0, 1]
    with pytest.raises(kt.KtrussError) as ei:
        _run(torch, eng, np.array([0, 7], np.uint32), np.array([7, 0], np.uint32), 3)
    assert ei.value.status == 1  # KT_ERR_INVALID_ARG
    assert _run(torch, eng, np.zeros(0, np.uint32), np.zeros(0, np.uint32), 0)[0] == 0
