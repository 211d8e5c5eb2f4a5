"""The reference's tiled COO/CSR layout (coo2tiledcoocsr, graph.cu:641-706): the oracle's
restatement against the reference's own compiled builder (CPU, where its objects exist), and the
device builder kt_engine_tiled_coocsr against the oracle (GPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import ROOT, both_directions, load_golden

GRAPH_O = os.path.join(ROOT, "oracle", "_ref", "graph.o")
CASES = [("tiny9", 1), ("tiny9", 3), ("rmat10", 8), ("er1000_cliques", 5), ("ba2000", 16)]


def _entries(name):
    n, u, v, _ = load_golden(name)
    src, dst = both_directions(u, v)
    return n, src, dst


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not os.path.exists(GRAPH_O) or not shutil.which("nvcc"):
        pytest.skip("reference objects not built here")
    exe = str(tmp_path_factory.mktemp("tiled") / "tiled_driver")
    r = subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe,
                        os.path.join(ROOT, "tests", "compat", "tiled_driver.cpp"), GRAPH_O],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("name,T", CASES)
def test_oracle_matches_reference_builder(name, T, driver):
    n, src, dst = _entries(name)
    text = f"{n} {len(src)} {T}\n" + "".join(f"{s} {d}\n" for s, d in zip(src.tolist(), dst.tolist()))
    r = subprocess.run([driver], input=text, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    ts, rows = (int(x) for x in lines[0].split())
    ref_ptr = np.array(lines[1:rows + 2], np.int64)
    pairs = np.array([ln.split() for ln in lines[rows + 2:rows + 2 + len(src)]], np.int64)
    ptr, s, d = oracle.tiled_coocsr(n, src, dst, T)
    assert ts == (n + T - 1) // T and len(ptr) == rows + 1
    assert np.array_equal(ptr, ref_ptr)
    assert np.array_equal(s, pairs[:, 0]) and np.array_equal(d, pairs[:, 1])


@pytest.mark.gpu
@pytest.mark.parametrize("name,T", CASES + [("rmat12", 64), ("ws2000", 7)])
def test_device_builder_matches_oracle(name, T):
    torch = pytest.importorskip("torch")
    n, src, dst = _entries(name)
    ptr, s, d = oracle.tiled_coocsr(n, src, dst, T)
    eng = kt.Engine(0)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()
    d_src, d_dst = dev(src), dev(dst)
    d_ptr = torch.full((len(ptr),), -1, dtype=torch.int32, device="cuda")
    d_s = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_d = torch.empty(len(src), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.tiled_coocsr(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, T, d_ptr.data_ptr(), d_s.data_ptr(),
                     d_d.data_ptr())
    assert np.array_equal(d_ptr.cpu().numpy().view(np.uint32), ptr)
    assert np.array_equal(d_s.cpu().numpy().view(np.uint32), s)
    assert np.array_equal(d_d.cpu().numpy().view(np.uint32), d)


@pytest.mark.gpu
def test_device_builder_rejects_bad_input():
    torch = pytest.importorskip("torch")
    eng = kt.Engine(0)
    d = torch.tensor([0, 5], dtype=torch.int32, device="cuda")
    out = torch.empty(64, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(kt.KtrussError) as ei:  # vertex 5 >= num_nodes 4
        eng.tiled_coocsr(d.data_ptr(), d.flip(0).data_ptr(), 2, 4, 2, out.data_ptr(), out.data_ptr(), out.data_ptr())
    assert ei.value.status == 1  # KT_ERR_INVALID_ARG
    with pytest.raises(kt.KtrussError):
        eng.tiled_coocsr(d.data_ptr(), d.data_ptr(), 2, 8, 0, out.data_ptr(), out.data_ptr(), out.data_ptr())
