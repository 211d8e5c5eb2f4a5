"""CPU checks of the selector oracle: its backpropagated gradient against central finite
differences, its labels, and the binding's grid mapping (no GPU needed)."""
import numpy as np

import ktruss_gb300 as kt
import selector_oracle as so


def _problem(seed, n=12):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.3, so.NPARAMS)
    mean = rng.normal(0, 1, so.F)
    scale = rng.uniform(0.5, 2.0, so.F)
    feats = rng.normal(0, 1.5, (n, so.F))
    times = rng.uniform(1, 10, (n, so.SCHEDULES))
    return p, mean, scale, feats, times


def test_gradient_matches_finite_differences():
    p, mean, scale, feats, times = _problem(3)
    _, g = so.loss_and_grad(p, mean, scale, feats, times)
    rng = np.random.default_rng(4)
    idx = np.concatenate([rng.choice(np.arange(a, b), 6, replace=False) for a, b in
                          [(so.W1, so.B1), (so.B1, so.W2), (so.W2, so.B2), (so.B2, so.W3), (so.W3, so.B3),
                           (so.B3, so.NPARAMS)]])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = so.loss_and_grad(q, mean, scale, feats, times)
        q[i] -= 2 * h
        lm, _ = so.loss_and_grad(q, mean, scale, feats, times)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_labels():
    t = np.full((1, so.SCHEDULES), 10.0)
    t[0, 2 * 5 + 1] = 3.0  # variant 5 with recount on is fastest
    t[0, 2 * 7 + 0] = 4.0  # best recount-off schedule
    yv, yr = so.labels(t)
    assert yv[0] == 5 and yr[0] == 1
    t[0, 2 * 7 + 0] = 2.0
    yv, yr = so.labels(t)
    assert yv[0] == 7 and yr[0] == 0


def test_grid_order_is_variant_then_recount():
    grid = [s.as_tuple() for s in kt.schedule_grid()]
    assert len(grid) == so.SCHEDULES
    for v in range(so.V):
        a, b = grid[2 * v], grid[2 * v + 1]
        assert a[:3] == b[:3] and a[3] == 0 and b[3] == 50 and a[4] == b[4] == 0
    assert kt.schedule_index(kt.schedule_default()) == 2 * 11 + 1  # variant (8, 32, 85), recount on
