"""kt_decompose_noalloc: the decomposition for callers that cannot let the library allocate
device memory (their memory manager owns every byte, or cudaMalloc/cudaFree are too costly in
their loop).  It must give exactly what the allocating engine API gives, call after call, although
every call reuses the same static scratch.  This file is collected last on purpose."""
import numpy as np
import pytest

import ktruss_gb300 as kt
from conftest import both_directions, load_golden

pytestmark = pytest.mark.gpu


def _graphs():
    n1, u1, v1 = kt.gen_rmat(14, 8, 0.57, 0.19, 0.19, 21)     # larger graph first ...
    n2, u2, v2, _ = load_golden("cliques_bridge")               # ... then a tiny one: stale scratch must not leak
    n3, u3, v3 = kt.plant_cliques(*kt.gen_ba(5000, 6, 3), 2, 20, 40, 4)
    return [(n1, u1, v1), (n2, u2, v2), (n3, u3, v3)]


def _device(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


def test_noalloc_matches_engine_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    eng = kt.Engine(0)
    for n, u, v in _graphs():
        src, dst = both_directions(u, v)
        d_src, d_dst = _device(torch, src), _device(torch, dst)
        ref = torch.zeros(len(src), dtype=torch.int32, device="cuda")
        ref_k = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, ref.data_ptr(), ref_k.data_ptr())
        for _ in range(2):  # two calls in a row on the shared scratch
            out = torch.full((len(src),), -1, dtype=torch.int32, device="cuda")
            out_k = torch.zeros(1, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            kt.decompose_noalloc(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, out.data_ptr(), out_k.data_ptr())
            assert int(out_k.item()) == int(ref_k.item())
            assert torch.equal(out, ref)
    eng.close()


def test_noalloc_calls_allocate_no_device_memory():
    """After a first round of calls (which backs the static array and loads every kernel the calls
    use), further calls on graphs of different sizes leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    bufs = []
    for n, u, v in _graphs():
        src, dst = both_directions(u, v)
        out = torch.zeros(len(src), dtype=torch.int32, device="cuda")
        out_k = torch.zeros(1, dtype=torch.int32, device="cuda")
        bufs.append((n, len(src), _device(torch, src), _device(torch, dst), out, out_k))
    torch.cuda.synchronize()

    def call(b):
        n, N, d_src, d_dst, out, out_k = b
        kt.decompose_noalloc(d_src.data_ptr(), d_dst.data_ptr(), N, n, out.data_ptr(), out_k.data_ptr())

    for b in bufs:
        call(b)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for b in bufs[::-1] + bufs:
        call(b)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"


def test_noalloc_rejects_graphs_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    d = torch.zeros(4, dtype=torch.int32, device="cuda")
    with pytest.raises(kt.KtrussError) as ei:
        kt.decompose_noalloc(d.data_ptr(), d.data_ptr(), (1 << 19) + 2, 8, d.data_ptr())
    assert ei.value.status == 13  # KT_ERR_TOO_LARGE, checked before any device work
    with pytest.raises(kt.KtrussError) as ei:
        kt.decompose_noalloc(d.data_ptr(), d.data_ptr(), 2, (1 << 17) + 1, d.data_ptr())
    assert ei.value.status == 13
