"""Device-side TSV ingest against the host reader (which restates createCOOFromFile,
graph.cu:37-79): same entries in the same order, same vertex count, same statuses."""
import os

import numpy as np
import pytest

import ktruss_gb300 as kt
from conftest import GOLDEN_NAMES, both_directions, load_golden

pytestmark = pytest.mark.gpu

KT_ERR_SELF_LOOP, KT_ERR_CAPACITY, KT_ERR_IO = 2, 4, 9


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.fixture(scope="module")
def eng():
    e = kt.Engine(0)
    yield e
    e.close()


def _device_read(torch, eng, path, capacity=None):
    size = os.path.getsize(path)
    cap = capacity if capacity is not None else size // 4 + 1
    d_src = torch.zeros(max(cap, 1), dtype=torch.int32, device="cuda")
    d_dst = torch.zeros(max(cap, 1), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    n_e, n_v = eng.read_tsv(path, d_src.data_ptr(), d_dst.data_ptr(), cap)
    return n_v, d_src[:n_e].cpu().numpy().view(np.uint32), d_dst[:n_e].cpu().numpy().view(np.uint32)


def _status(fn):
    try:
        fn()
        return 0
    except kt.KtrussError as e:
        return e.status


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_golden_files_match_host_reader(name, torch, eng, tmp_path):
    n, u, v, _ = load_golden(name)
    src, dst = both_directions(u, v)
    path = str(tmp_path / f"{name}.tsv")
    kt.write_coo_graph_to_file(kt.COOGraph(n, src, dst), path)
    h = kt.create_coo_from_file(path)
    nv, s, d = _device_read(torch, eng, path)
    assert nv == h.num_nodes
    assert np.array_equal(s, h.src_idx) and np.array_equal(d, h.dst_idx)


def test_whitespace_forms_and_tile_boundaries(torch, eng, tmp_path):
    rng = np.random.default_rng(3)
    n, u, v = kt.gen_rmat(12, 16, 0.57, 0.19, 0.19, 5)
    src, dst = both_directions(u, v)
    seps = [" ", "\t", "  ", "\t \t"]
    ends = ["\n", "\r\n", "\n\n", " \n"]
    parts = []
    for i in range(len(src)):
        a, b, x = int(dst[i]) + 1, int(src[i]) + 1, int(rng.integers(0, 10**9))
        parts.append(f"{a}{seps[i % 4]}{b}{seps[(i + 1) % 4]}{x}{ends[i % 4]}")
    text = "".join(parts).rstrip("\n")  # no trailing newline
    assert len(text) > 4 * 32768  # several tiles, numbers straddle tile edges
    path = str(tmp_path / "ws.tsv")
    with open(path, "w") as f:
        f.write(text)
    h = kt.create_coo_from_file(path)
    nv, s, d = _device_read(torch, eng, path)
    assert nv == h.num_nodes and len(s) == len(src)
    assert np.array_equal(s, h.src_idx) and np.array_equal(d, h.dst_idx)


@pytest.mark.parametrize("text,status", [
    ("", 0),
    ("   \n\n", 0),
    ("2 1 1\n1 2 1\n", 0),
    ("3 3 1\n", KT_ERR_SELF_LOOP),
    ("2 1 1\n1 1 7\n", KT_ERR_SELF_LOOP),
    ("0 1 1\n", KT_ERR_IO),
    ("2 1 1\n1 2\n", KT_ERR_IO),
    ("2 1 x\n", KT_ERR_IO),
    ("2 1 1\n1 2 1\n#\n", KT_ERR_IO),
    ("4294967296 1 1\n", KT_ERR_IO),
    ("4294967295 1 1\n1 4294967295 1\n", 0),
    ("12345678901 1 1\n", KT_ERR_IO),
])
def test_statuses_match_host_reader(text, status, torch, eng, tmp_path):
    path = str(tmp_path / "t.tsv")
    with open(path, "w") as f:
        f.write(text)
    host = _status(lambda: kt.create_coo_from_file(path))
    dev = _status(lambda: _device_read(torch, eng, path))
    assert host == status and dev == status, (host, dev)
    if status == 0:
        h = kt.create_coo_from_file(path)
        nv, s, d = _device_read(torch, eng, path)
        assert nv == h.num_nodes and np.array_equal(s, h.src_idx) and np.array_equal(d, h.dst_idx)


def test_capacity_and_unaligned_device_text(torch, eng, tmp_path):
    text = b"2 1 1\n1 2 1\n3 1 1\n1 3 1\n"
    path = str(tmp_path / "c.tsv")
    with open(path, "wb") as f:
        f.write(text)
    assert _status(lambda: _device_read(torch, eng, path, capacity=3)) == KT_ERR_CAPACITY
    # text already on the device, starting at an odd address
    buf = torch.zeros(len(text) + 8, dtype=torch.uint8, device="cuda")
    buf[3:3 + len(text)] = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda()
    d_src = torch.zeros(4, dtype=torch.int32, device="cuda")
    d_dst = torch.zeros(4, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    n_e, n_v = eng.parse_tsv(buf.data_ptr() + 3, len(text), d_src.data_ptr(), d_dst.data_ptr(), 4)
    assert (n_e, n_v) == (4, 3)
    assert d_src.cpu().tolist() == [0, 1, 0, 2] and d_dst.cpu().tolist() == [1, 0, 2, 0]


def test_read_then_decompose_on_device(torch, eng, tmp_path):
    n, u, v, t = load_golden("er4096")
    src, dst = both_directions(u, v)
    path = str(tmp_path / "er.tsv")
    kt.write_coo_graph_to_file(kt.COOGraph(n, src, dst), path)
    cap = len(src)
    d_src = torch.zeros(cap, dtype=torch.int32, device="cuda")
    d_dst = torch.zeros(cap, dtype=torch.int32, device="cuda")
    out = torch.zeros(cap, dtype=torch.int32, device="cuda")
    kk = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    n_e, n_v = eng.read_tsv(path, d_src.data_ptr(), d_dst.data_ptr(), cap)
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), n_e, n_v, out.data_ptr(), kk.data_ptr())
    got = out.cpu().numpy().view(np.uint32)
    assert np.array_equal(got[: len(u)], t) and np.array_equal(got[len(u):], t)
