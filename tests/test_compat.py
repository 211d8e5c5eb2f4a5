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
