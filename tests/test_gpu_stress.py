"""Stress: R-MAT with edge factor 32 plus 16 planted cliques of 64-512 vertices (deep peeling).

At this size the oracle is too slow, so the decomposition is checked through properties that do
not depend on size, against a second code path of the engine (the single-k peel, which has no
levels): for every tested k, the edges with truss number >= k are exactly the k-truss; k_max is
at least the smallest planted clique and the (k_max+1)-truss is empty; the host-buffer call
agrees with the device-buffer call.  The scale is KT_STRESS_SCALE (default 21; the R-MAT 24
stress workload is the same test with KT_STRESS_SCALE=24)."""
import os

import numpy as np
import pytest

import ktruss_gb300 as kt
from conftest import both_directions

pytestmark = pytest.mark.gpu

SCALE = int(os.environ.get("KT_STRESS_SCALE", "21"))


@pytest.fixture(scope="module")
def stress():
    torch = pytest.importorskip("torch")
    n, u, v = kt.gen_rmat(SCALE, 32, 0.57, 0.19, 0.19, 1)
    n, u, v = kt.plant_cliques(n, u, v, 16, 64, 512, 8)
    src, dst = both_directions(u, v)
    eng = kt.Engine(0)
    eng.reserve(n, len(src))
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
    st = eng.stats()
    truss = d_out[: len(u)].cpu().numpy().view(np.uint32).copy()
    yield dict(torch=torch, eng=eng, n=n, u=u, v=v, src=src, d_src=d_src, d_dst=d_dst, d_out=d_out,
               truss=truss, k_max=int(d_k.item()), stats=st)
    eng.close()


def test_both_directions_agree_and_k_max(stress):
    out = stress["d_out"].cpu().numpy().view(np.uint32)
    m = len(stress["u"])
    assert np.array_equal(out[:m], out[m:])
    assert stress["k_max"] == int(stress["truss"].max())
    assert stress["k_max"] >= 64  # a planted 64-clique alone is a 64-truss
    assert stress["truss"].min() >= 2
    st = stress["stats"]
    assert st.num_edges == m and st.triangles > 0 and st.num_levels > 0


def test_truss_sets_equal_single_k(stress):
    torch, eng = stress["torch"], stress["eng"]
    src = stress["src"]
    m = len(stress["u"])
    keep = torch.empty(len(src), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    k_max = stress["k_max"]
    for k in sorted({3, 4, 5, 8, k_max // 2, k_max - 1, k_max, k_max + 1}):
        eng.ktruss(stress["d_src"].data_ptr(), stress["d_dst"].data_ptr(), len(src), stress["n"], k,
                   keep.data_ptr())
        got = keep[:m].cpu().numpy().astype(bool)
        assert np.array_equal(got, stress["truss"] >= k), k
    assert not got.any()  # k_max + 1


def test_host_buffer_call_agrees(stress):
    if SCALE > 22:
        pytest.skip("host copy of the largest graph is covered by bench.py's e2e check")
    g = kt.COOGraph(stress["n"], stress["src"], np.concatenate([stress["v"], stress["u"]]))
    truss, k_max = kt.decompose(g)
    assert k_max == stress["k_max"]
    assert np.array_equal(truss[: len(stress["u"])], stress["truss"])
