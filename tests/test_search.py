"""The peel's row search (fenced_lower_bound: fences, then one 32-entry block) and the plain lower
bound, built for the host from csrc/kt_device.cuh and checked against numpy's searchsorted on
random sorted rows of every length class (at most 32 entries, around the fence stride, long)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "ktruss-explorer_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not shutil.which("nvcc"):
        pytest.skip("nvcc not found")
    exe = str(tmp_path_factory.mktemp("search") / "search_driver")
    r = subprocess.run(["nvcc", "-std=c++17", "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-o", exe,
                        os.path.join(ROOT, "tests", "compat", "search_driver.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fenced_search_matches_searchsorted(seed, driver):
    rng = np.random.default_rng(seed)
    rows, ptr = [], [0]
    for _ in range(300):
        L = int(rng.choice([0, 1, 7, 31, 32, 33, 63, 64, 65, 100, 1023, 1025, 3000]))
        rows.append(np.sort(rng.choice(10 * L + 10, L, replace=False)).astype(np.uint32))
        ptr.append(ptr[-1] + L)
    a = np.concatenate(rows)
    queries = []
    for r in range(len(rows)):
        lo, hi = ptr[r], ptr[r + 1]
        vals = rng.integers(0, 10 * (hi - lo) + 12, 6).tolist()
        if hi > lo:
            vals += [int(a[lo]), int(a[hi - 1]), int(a[rng.integers(lo, hi)])]
        queries += [(lo, hi, v) for v in vals]
    text = f"{len(a)}\n" + " ".join(map(str, a.tolist())) + f"\n{len(queries)}\n" + \
        "".join(f"{lo} {hi} {t}\n" for lo, hi, t in queries)
    r = subprocess.run([driver], input=text, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.array([ln.split() for ln in r.stdout.split("\n") if ln], np.int64)
    want = np.array([lo + np.searchsorted(a[lo:hi], t, side="left") for lo, hi, t in queries], np.int64)
    assert np.array_equal(got[:, 0], want)
    assert np.array_equal(got[:, 1], want)
