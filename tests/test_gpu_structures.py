"""Structural edge cases against the oracle: graphs without triangles, cliques with pendants and
bridges, shared-vertex cliques, wheels, windmills, books, a triangulated grid, a sparse graph over a
large id range and a hub with 100 000 leaves beside a clique - one at a time and all in one batch."""
import itertools

import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
from conftest import both_directions

pytestmark = pytest.mark.gpu


def _canon(pairs):
    a = np.array(sorted({(min(x, y), max(x, y)) for x, y in pairs if x != y}), np.uint32).reshape(-1, 2)
    return a[:, 0].copy(), a[:, 1].copy()


def _clique(vs):
    return list(itertools.combinations(vs, 2))


def star(n=100001):
    return n, _canon([(0, i) for i in range(1, n)])


def grid(w=300, h=300):
    e = [(y * w + x, y * w + x + 1) for y in range(h) for x in range(w - 1)]
    e += [(y * w + x, (y + 1) * w + x) for y in range(h - 1) for x in range(w)]
    return w * h, _canon(e)


def triangulated_grid(w=200, h=200):
    n, (u, v) = grid(w, h)
    diag = [(y * w + x, (y + 1) * w + x + 1) for y in range(h - 1) for x in range(w - 1)]
    return n, _canon(list(zip(u.tolist(), v.tolist())) + diag)


def clique_pendants(c=200):
    return c + c, _canon(_clique(range(c)) + [(i, c + i) for i in range(c)])


def bridged_cliques():
    return 130, _canon(_clique(range(60)) + _clique(range(60, 130)) + [(0, 60), (1, 61)])


def shared_vertex_cliques():
    return 79, _canon(_clique(range(40)) + _clique([0] + list(range(40, 79))))


def wheel(n=5000):
    return n, _canon([(0, i) for i in range(1, n)] + [(i, i + 1) for i in range(1, n - 1)] + [(n - 1, 1)])


def windmill(blades=3000):
    return 2 * blades + 1, _canon([(0, 2 * i + 1) for i in range(blades)] + [(0, 2 * i + 2) for i in range(blades)]
                                  + [(2 * i + 1, 2 * i + 2) for i in range(blades)])


def book(pages=20000):
    return pages + 2, _canon([(0, 1)] + [(0, i) for i in range(2, pages + 2)] + [(1, i) for i in range(2, pages + 2)])


def sparse_ids():
    rng = np.random.default_rng(7)
    vs = rng.choice(1 << 20, 60, replace=False).tolist()
    return 1 << 20, _canon(_clique(vs[:12]) + list(zip(vs[12:], vs[13:])))


def hub_and_clique():
    leaves = 100000
    return leaves + 1, _canon([(0, i) for i in range(1, leaves + 1)] + _clique(range(1, 31)))


CASES = [star, grid, triangulated_grid, clique_pendants, bridged_cliques, shared_vertex_cliques, wheel, windmill,
         book, sparse_ids, hub_and_clique]


@pytest.mark.parametrize("make", CASES, ids=[c.__name__ for c in CASES])
def test_structure_matches_oracle(make):
    n, (u, v) = make()
    src, dst = both_directions(u, v)
    truss, k_max = kt.decompose(kt.COOGraph(n, src, dst))
    ref = oracle.decompose(n, src, dst, method="peel")
    assert k_max == ref["k_max"]
    assert np.array_equal(truss, ref["truss"])


def test_all_structures_in_one_batch():
    parts, off = [], [0]
    for make in CASES:
        n, (u, v) = make()
        parts.append((u + off[-1], v + off[-1], n, u, v))
        off.append(off[-1] + n)
    U = np.concatenate([p[0] for p in parts]).astype(np.uint32)
    V = np.concatenate([p[1] for p in parts]).astype(np.uint32)
    src, dst = both_directions(U, V)
    truss, kmax = kt.decompose_batch(src, dst, off[-1], np.array(off, np.uint32))
    pos = 0
    for g, (_, _, n, u, v) in enumerate(parts):
        s, d = both_directions(u, v)
        ref = oracle.decompose(n, s, d, method="peel")
        assert kmax[g] == ref["k_max"], g
        assert np.array_equal(truss[pos:pos + len(u)], ref["truss"][: len(u)]), g
        pos += len(u)
