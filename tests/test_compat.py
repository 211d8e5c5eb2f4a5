"""The C++ link-compatible entry point `void ktruss(COOGraph*, COOGraph*, Config)` (kernel.h:12):
programs built against the reference's headers link against libktruss_compat.so unchanged."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import ktruss_gb300 as kt
from conftest import ROOT, both_directions, edge_keys, load_golden

LIBDIR = os.path.join(ROOT, "ktruss-explorer_gb300", "lib")
REF_OBJS = [os.path.join(ROOT, "oracle", "_ref", f) for f in ("main.o", "graph.o", "verify.o")]
# the reference sources: a checkout named by KT_REFERENCE_DIR, else the staged copy
# (make -C oracle stage), which travels with the repository to the GPU machine
REF_SRC = os.environ.get("KT_REFERENCE_DIR") or os.path.join(ROOT, "baseline", "_ref", "src")


def test_reference_main_links_against_the_shim(tmp_path):
    """Link the reference's own main/graph/verify objects (built by `make -C oracle ref` where the
    reference sources exist) with the shim instead of its kernel files, and run its help path."""
    if not all(os.path.exists(p) for p in REF_OBJS) or not shutil.which("nvcc"):
        pytest.skip("reference objects not built here")
    exe = str(tmp_path / "ktruss_ref_main")
    r = subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe] + REF_OBJS +
                       ["-L", LIBDIR, "-lktruss_compat", "-lktruss_gb300", f"-Xlinker=-rpath,{LIBDIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage" in r.stderr


def _driver(tmp_path):
    exe = str(tmp_path / "compat_driver")
    r = subprocess.run(["g++", "-O2", "-o", exe, os.path.join(ROOT, "tests", "compat", "compat_driver.cpp"),
                        "-I", os.path.join(ROOT, "include"), "-L", LIBDIR, "-lktruss_compat", "-lktruss_gb300",
                        f"-Wl,-rpath,{LIBDIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_driver_builds_against_compat_header(tmp_path):
    _driver(tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny9", "rmat10", "ba2000"])
def test_compat_entry_point_matches_golden(name, manifest, tmp_path):
    exe = _driver(tmp_path)
    n, u, v, t = load_golden(name)
    g = kt.COOGraph.from_undirected(n, u, v)
    path = str(tmp_path / "g.tsv")
    kt.write_coo_graph_to_file(g, path)
    for k_str, chk in manifest["graphs"][name]["single_k"].items():
        if int(k_str) < 2:
            continue
        r = subprocess.run([exe, path, k_str], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        lines = [ln.split() for ln in r.stdout.splitlines() if ln and ln[0].isdigit() and len(ln.split()) == 2]
        s = np.array([int(a) for a, b in lines], np.uint32)
        d = np.array([int(b) for a, b in lines], np.uint32)
        assert len(edge_keys(s, d)) == chk["edges"], k_str


def _write_ref_tsv(path, u, v):
    """Both directions in the reference's "dst src 1" format (graph.cu:96-104), 1-based."""
    with open(path, "w") as f:
        for a, b in zip(u.tolist(), v.tolist()):
            f.write(f"{b + 1}\t{a + 1}\t1\n{a + 1}\t{b + 1}\t1\n")


@pytest.mark.gpu
def test_reference_main_on_the_shim_passes_its_own_verify(manifest, tmp_path):
    """The reference's own main/graph/verify objects, compiled from its unmodified sources and linked
    against libktruss_compat.so instead of its kernel files, run k-truss queries on golden graphs
    (main.cu:13-53) and pass the reference's own verify (verify.cu:12-40) against the expected truss
    written as its -c file."""
    if not os.path.exists(os.path.join(REF_SRC, "main.cu")) or not shutil.which("nvcc"):
        pytest.skip("no reference sources here")
    subprocess.run(["make", "-s", "-j3", "-C", os.path.join(ROOT, "oracle"), "_ref/main.o", "_ref/graph.o",
                    "_ref/verify.o", f"REF_DIR={REF_SRC}"], check=True)
    exe = str(tmp_path / "ktruss_ref_main")
    r = subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-o", exe] + REF_OBJS +
                       ["-L", LIBDIR, "-lktruss_compat", "-lktruss_gb300", f"-Xlinker=-rpath,{LIBDIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    runs = 0
    for name in ("tiny9", "k6", "rmat10", "ba2000", "er1000_cliques"):
        n, u, v, t = load_golden(name)
        graph = str(tmp_path / f"{name}.tsv")
        _write_ref_tsv(graph, u, v)
        for k in sorted({3, 4, int(t.max()), int(t.max()) + 1}):
            sel = t >= k
            expected = str(tmp_path / f"{name}.{k}.tsv")
            _write_ref_tsv(expected, u[sel], v[sel])
            r = subprocess.run([exe, "-g", graph, "-k", str(k), "-c", expected, "-v", "1"], capture_output=True,
                               text=True, timeout=300)
            assert r.returncode == 0, (name, k, r.stdout[-2000:], r.stderr[-2000:])
            assert "PASSED" in r.stdout, (name, k)
            runs += 1
    assert runs >= 15
