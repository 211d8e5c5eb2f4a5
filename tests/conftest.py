"""Shared test setup: import paths, the `gpu` marker and fixture loading."""
import gzip
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ktruss-explorer_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the compiled CUDA path")


def load_manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def load_golden(name):
    """Returns (num_nodes, u, v, t) of a fixture graph; u < v, t = truss number."""
    man = load_manifest()["graphs"][name]
    with gzip.open(os.path.join(GOLDEN, f"{name}.tsv.gz"), "rt") as f:
        data = np.loadtxt(f, dtype=np.int64, ndmin=2)
    if data.size == 0:
        z = np.zeros(0, np.uint32)
        return man["num_nodes"], z, z, z
    return (man["num_nodes"], data[:, 0].astype(np.uint32), data[:, 1].astype(np.uint32),
            data[:, 2].astype(np.uint32))


def both_directions(u, v):
    return np.concatenate([u, v]).astype(np.uint32), np.concatenate([v, u]).astype(np.uint32)


def edge_keys(src, dst):
    """Sorted unique canonical (min, max) keys of a COO edge list."""
    a = np.minimum(src, dst).astype(np.uint64)
    b = np.maximum(src, dst).astype(np.uint64)
    return np.unique((a << np.uint64(32)) | b)


GOLDEN_NAMES = sorted(load_manifest()["graphs"].keys()) if os.path.exists(os.path.join(GOLDEN, "manifest.json")) else []


@pytest.fixture(scope="session")
def manifest():
    return load_manifest()
