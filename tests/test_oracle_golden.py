"""The CPU oracle against the reference's own outputs (tests/golden, made by make_golden.py).

These pin the oracle before it is trusted as the checker of the GPU engine."""
import hashlib

import numpy as np
import pytest

import oracle
from conftest import GOLDEN_NAMES, both_directions, edge_keys, load_golden


def sha_of_keys(keys):
    if len(keys) == 0:
        return "empty"
    u = (keys >> np.uint64(32)).astype(np.uint32)
    v = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    return hashlib.sha256(np.stack([u, v], 1).astype("<u4").tobytes()).hexdigest()


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_fixture_integrity(name, manifest):
    n, u, v, t = load_golden(name)
    g = manifest["graphs"][name]
    assert len(u) == g["num_edges"]
    assert sha_of_keys(edge_keys(u, v)) == g["edge_sha"]
    assert (u < v).all()
    assert int(t.max(initial=0)) == g["k_max"] or g["num_edges"] == 0


@pytest.mark.parametrize("method", ["chain", "peel", "peel-threads"])
@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_decomposition_matches_reference(name, method, manifest):
    n, u, v, t = load_golden(name)
    src, dst = both_directions(u, v)
    if method == "peel-threads":
        r = oracle.decompose(n, src, dst, method="peel", threads=4)
    else:
        r = oracle.decompose(n, src, dst, method=method, threads=1)
    m = len(u)
    assert np.array_equal(r["truss"][:m], t)
    assert np.array_equal(r["truss"][m:], t)
    g = manifest["graphs"][name]
    assert r["k_max"] == g["k_max"]
    # pass statistics of the reference's count-and-prune loop (counted from its -v 2 output)
    assert r["plain_passes"] == g["ref_passes"]
    assert r["plain_alive_sum"] == g["ref_alive_sum"]


VARIANTS = [(d, rc, e) for d in (oracle.UNDIRECTED, oracle.DIRECTED_BY_INDEX, oracle.DIRECTED_BY_DEGREE)
            for rc in (oracle.RECOUNT_ALL, oracle.RECOUNT_AFFECTED) for e in (0, 1)]


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_single_k_variants_match_reference(name, manifest):
    n, u, v, t = load_golden(name)
    src, dst = both_directions(u, v)
    for k_str, chk in manifest["graphs"][name]["single_k"].items():
        k = int(k_str)
        for d, rc, e in VARIANTS:
            os_, od = oracle.ktruss(n, src, dst, k, d, rc, e)
            keys = edge_keys(os_, od)
            assert len(os_) == 2 * len(keys), "output must hold both directions"
            assert len(keys) == chk["edges"], (k, d, rc, e)
            assert sha_of_keys(keys) == chk["sha"], (k, d, rc, e)


@pytest.mark.parametrize("seed", [1, 2])
def test_threaded_peel_equals_serial_peel(seed):
    """The oracle's peel split over host threads computes exactly what the serial peel computes:
    truss numbers, k_max, rounds and the per-level pass statistics of the reference chain."""
    n, u, v = oracle.gen_rmat(13, 16, 0.57, 0.19, 0.19, seed)
    src, dst = both_directions(u, v)
    a = oracle.decompose(n, src, dst, levels=True, threads=1)
    for threads in (2, 7):
        b = oracle.decompose(n, src, dst, levels=True, threads=threads)
        for key in a:
            if isinstance(a[key], np.ndarray):
                assert np.array_equal(a[key], b[key]), key
            else:
                assert a[key] == b[key], key


def test_level_statistics_sum_to_the_pass_totals(manifest):
    for name in GOLDEN_NAMES:
        n, u, v, t = load_golden(name)
        if len(u) == 0:
            continue
        src, dst = both_directions(u, v)
        r = oracle.decompose(n, src, dst, levels=True)
        assert int(r["level_passes"].sum()) == manifest["graphs"][name]["ref_passes"]
        assert int(r["level_alive"].sum()) == manifest["graphs"][name]["ref_alive_sum"]
