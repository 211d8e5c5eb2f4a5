"""CPU tests of the host side: the C ABI library loads and exports its declared symbols, config
parsing and printing (config.h), TSV I/O (graph.cu), verify (verify.cu), generators, CLI."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import ktruss_gb300 as kt
from conftest import GOLDEN_NAMES, ROOT, edge_keys, load_golden

HEADER = os.path.join(ROOT, "include", "ktruss_gb300.h")


def declared_functions(path):
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(kt_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(kt.LIB_PATH)
    names = declared_functions(HEADER)
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    L = kt.lib()
    for code in range(14):
        assert L.kt_status_string(code)


def test_parse_args_defaults_and_flags():
    c = kt.parse_args([])
    assert (c.k, c.processor, c.directedness, c.input_format, c.recount) == (3, "gpu", "directed-by-degree",
                                                                           "coocsr", "all")
    assert (c.block_size, c.num_tiles, c.num_parallel_tiles, c.verbosity) == (512, 8, 8, 1)
    c = kt.parse_args(["-g", "a.tsv", "-k", "7", "-c", "b.tsv", "-o", "o.tsv", "-w", "2", "-x", "3", "-p", "cpu",
                       "-d", "undirected", "-f", "tiled-coocsr", "-e", "4", "-r", "affected", "-b", "128", "-t", "16",
                       "-y", "2", "-v", "0"])
    assert c == kt.Config("a.tsv", 7, "b.tsv", "o.tsv", 2, 3, "cpu", "undirected", "tiled-coocsr", 4, "affected",
                          128, 16, 2, 0, 0, 0)


@pytest.mark.parametrize("argv", [["-p", "tpu"], ["-d", "sideways"], ["-f", "csr"], ["-r", "some"], ["-q"]])
def test_parse_args_rejects_bad_values(argv):
    with pytest.raises(kt.KtrussError) as ei:
        kt.parse_args(argv)
    assert ei.value.status == 1


def test_k_wraps_like_atoi():
    assert kt.parse_args(["-k", "-1"]).k == 2**32 - 1


def test_tsv_roundtrip(tmp_path):
    n, u, v, t = load_golden("tiny9")
    g = kt.COOGraph.from_undirected(n, u, v)
    p = str(tmp_path / "g.tsv")
    kt.write_coo_graph_to_file(g, p)
    lines = open(p).read().splitlines()
    assert lines[0] == f"{v[0] + 1}\t{u[0] + 1}\t1"
    h = kt.create_coo_from_file(p)
    assert h.num_nodes == n and np.array_equal(h.src_idx, g.src_idx) and np.array_equal(h.dst_idx, g.dst_idx)
    kt.write_truss_to_file(g, np.concatenate([t, t]), str(tmp_path / "t.tsv"))
    third = [int(x.split("\t")[2]) for x in open(tmp_path / "t.tsv").read().splitlines()]
    assert third == list(np.concatenate([t, t]))


def test_tsv_writer_bytes(tmp_path):
    """Parallel formatting gives the same bytes as one formatted line per entry, across batch
    boundaries (2.5 M entries) and at the largest ids and third-column values."""
    rng = np.random.default_rng(12)
    m = 2_500_000
    src = rng.integers(0, 2**32 - 1, m, dtype=np.uint64).astype(np.uint32)
    dst = rng.integers(0, 2**32 - 1, m, dtype=np.uint64).astype(np.uint32)
    third = rng.integers(0, 2**32, m, dtype=np.uint64).astype(np.uint32)
    src[:3] = [0, 2**32 - 2, 7]
    third[:3] = [0, 2**32 - 1, 9]
    g = kt.COOGraph(2**32 - 1, src, dst)
    p = tmp_path / "w.tsv"
    kt.write_truss_to_file(g, third, str(p))
    d1, s1, t1 = dst.astype(np.int64) + 1, src.astype(np.int64) + 1, third.astype(np.int64)
    want = "".join(f"{a}\t{b}\t{c}\n" for a, b, c in zip(d1.tolist(), s1.tolist(), t1.tolist()))
    assert p.read_bytes() == want.encode()
    q = tmp_path / "g.tsv"
    kt.write_coo_graph_to_file(kt.COOGraph(2**32 - 1, src[:1000], dst[:1000]), str(q))
    assert q.read_text() == "".join(f"{a}\t{b}\t1\n" for a, b in zip(d1[:1000].tolist(), s1[:1000].tolist()))


def test_tsv_errors(tmp_path):
    with pytest.raises(kt.KtrussError) as ei:
        kt.create_coo_from_file(str(tmp_path / "missing.tsv"))
    assert ei.value.status == 9
    p = tmp_path / "loop.tsv"
    p.write_text("1\t2\t1\n2\t2\t1\n")
    with pytest.raises(kt.KtrussError) as ei:
        kt.create_coo_from_file(str(p))
    assert ei.value.status == 2
    p.write_text("1\t2\n")
    with pytest.raises(kt.KtrussError) as ei:
        kt.create_coo_from_file(str(p))
    assert ei.value.status == 9


def test_tsv_num_nodes_is_max_id(tmp_path):
    p = tmp_path / "g.tsv"
    p.write_text("7\t3\t1\n3\t7\t1\n")
    g = kt.create_coo_from_file(str(p))
    assert g.num_nodes == 7 and list(g.src_idx) == [2, 6] and list(g.dst_idx) == [6, 2]


def test_verify(tmp_path):
    n, u, v, t = load_golden("cliques_bridge")
    keep = t >= 4
    g = kt.COOGraph.from_undirected(n, u[keep], v[keep])
    ref = str(tmp_path / "ref.tsv")
    # the reference file in another order verifies
    kt.write_coo_graph_to_file(kt.COOGraph(n, g.src_idx[::-1], g.dst_idx[::-1]), ref)
    kt.verify(g, kt.Config(compare_file_name=ref, verbosity=0))
    bad = kt.COOGraph.from_undirected(n, u[keep][:-1], v[keep][:-1])
    with pytest.raises(kt.KtrussError) as ei:
        kt.verify(bad, kt.Config(compare_file_name=ref, verbosity=0))
    assert ei.value.status == 10
    swapped = kt.COOGraph(n, g.src_idx.copy(), g.dst_idx.copy())
    swapped.dst_idx[0] = (swapped.dst_idx[0] + 1) % n
    with pytest.raises(kt.KtrussError):
        kt.verify(swapped, kt.Config(compare_file_name=ref, verbosity=0))


def test_processor_cpu_is_unsupported():
    n, u, v, t = load_golden("k6")
    with pytest.raises(kt.KtrussError) as ei:
        kt.ktruss(kt.COOGraph.from_undirected(n, u, v), kt.Config(processor="cpu"))
    assert ei.value.status == 5


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_generators_are_deterministic(name, manifest):
    spec = manifest["graphs"][name]["spec"]
    if spec["kind"] == "hand":
        pytest.skip("hand-made graph")
    if spec["kind"] == "er":
        n, u, v = kt.gen_er(spec["n"], spec["p"], spec["seed"])
    elif spec["kind"] == "rmat":
        n, u, v = kt.gen_rmat(spec["scale"], spec["ef"], 0.57, 0.19, 0.19, spec["seed"])
    elif spec["kind"] == "ba":
        n, u, v = kt.gen_ba(spec["n"], spec["m"], spec["seed"])
    elif spec["kind"] == "ws":
        n, u, v = kt.gen_ws(spec["n"], spec["k"], spec["p"], spec["seed"])
    elif spec["kind"] == "rgg":
        n, u, v = kt.gen_rgg(spec["n"], spec["radius"], spec["seed"])
    if "cliques" in spec:
        n, u, v = kt.plant_cliques(n, u, v, *spec["cliques"])
    gn, gu, gv, _ = load_golden(name)
    assert n == gn and np.array_equal(u, gu) and np.array_equal(v, gv)


def test_generator_invariants():
    n, u, v = kt.gen_rmat(12, 8, 0.57, 0.19, 0.19, 3)
    assert (u < v).all() and len(edge_keys(u, v)) == len(u) and int(v.max()) < n
    n, u, v = kt.gen_ws(100, 6, 0.0, 1)
    assert len(u) == 300
    n, u, v = kt.plant_cliques(50, np.zeros(0, np.uint32), np.zeros(0, np.uint32), 1, 10, 10, 1)
    assert len(u) == 45


def test_cli_help_and_bad_option_exit_zero():
    if not os.path.exists(kt.CLI_PATH):
        pytest.skip("CLI not built")
    r = subprocess.run([kt.CLI_PATH, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage" in r.stderr
    r = subprocess.run([kt.CLI_PATH, "-p", "tpu"], capture_output=True, text=True)
    assert r.returncode == 0 and "Unrecognized -p option" in r.stderr


def test_cli_missing_graph_fails(tmp_path):
    if not os.path.exists(kt.CLI_PATH):
        pytest.skip("CLI not built")
    r = subprocess.run([kt.CLI_PATH, "-g", str(tmp_path / "nope.tsv"), "-v", "0"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


def test_default_schedule():
    assert kt.schedule_default().as_tuple() == (8, 32, 85, 50, 0)


def test_schedule_grid():
    grid = [s.as_tuple() for s in kt.schedule_grid()]
    assert len(grid) == 36 and len(set(grid)) == 36
    assert kt.schedule_default().as_tuple() in grid
