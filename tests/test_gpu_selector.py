"""Learned schedule selector: its CUDA kernels against the float64 oracle (gradient, Adam step,
inference, graph features), exactness of decompositions that use it, and what the trained
network gains over the default schedule on held-out graphs (GB300 timings in data/)."""
import os

import numpy as np
import pytest

import ktruss_gb300 as kt
import oracle
import selector as sel_mod
import selector_oracle as so
from conftest import both_directions

pytestmark = pytest.mark.gpu


def _problem(seed, n):
    rng = np.random.default_rng(seed)
    feats = rng.normal(0, 2, (n, so.F)).astype(np.float32)
    times = rng.uniform(1, 10, (n, so.SCHEDULES)).astype(np.float32)
    return feats, times


def test_gradient_matches_oracle():
    s = kt.Selector(0, seed=7)
    feats, times = _problem(1, 96)
    rng = np.random.default_rng(2)
    mean = rng.normal(0, 1, so.F).astype(np.float32)
    scale = rng.uniform(0.5, 2, so.F).astype(np.float32)
    s.set_params(mean=mean, scale=scale)
    p, _, _ = s.params()
    loss, g = s.gradient(feats, times)
    ref_loss, ref_g = so.loss_and_grad(p, mean, scale, feats, times)
    assert abs(loss - ref_loss) <= 1e-5 * max(1.0, abs(ref_loss))
    tol = 1e-4 * np.abs(ref_g).max()
    assert np.max(np.abs(g - ref_g)) <= tol, np.max(np.abs(g - ref_g))


def test_adam_step_matches_oracle():
    s = kt.Selector(0, seed=8)
    feats, times = _problem(3, 48)
    p0, _, _ = s.params()
    lr = 1e-2
    s.train(feats, times, epochs=1, batch=64, lr=lr, seed=5)  # one step over the whole set
    p1, mean, scale = s.params()
    mu, sd = so.standardization(feats)
    assert np.allclose(mean, mu, rtol=1e-5, atol=1e-6) and np.allclose(scale, sd, rtol=1e-5)
    _, g = so.loss_and_grad(p0, mu, sd, feats, times)
    ref, _, _ = so.adam_step(p0.astype(np.float64), g, np.zeros_like(g), np.zeros_like(g), 1, lr)
    assert np.max(np.abs(p1 - ref)) <= 2e-3 * lr


def test_predict_matches_oracle():
    s = kt.Selector(0, seed=9)
    feats, _ = _problem(4, 200)
    rng = np.random.default_rng(5)
    s.set_params(mean=rng.normal(0, 1, so.F), scale=rng.uniform(0.5, 2, so.F))
    p, mean, scale = s.params()
    got = np.array([kt.schedule_index(x) for x in s.predict(feats)])
    o = so.forward(p, mean, scale, feats)[-1]
    ref = so.choose(p, mean, scale, feats)
    # ignore graphs whose top two logits (or the recount logit) sit within float rounding
    top2 = np.sort(o[:, :so.V], axis=1)[:, -2:]
    clear = (top2[:, 1] - top2[:, 0] > 1e-4) & (np.abs(o[:, so.V]) > 1e-4)
    assert clear.sum() > 150
    assert np.array_equal(got[clear], ref[clear])


def _features_numpy(n, u, v):
    """The 16 features from their definitions, in float64."""
    deg = np.bincount(u, minlength=n) + np.bincount(v, minlength=n)
    rank = np.lexsort((np.arange(n), deg))  # ascending (degree, id)
    pos = np.empty(n, np.int64)
    pos[rank] = np.arange(n)
    lo = np.where(pos[u] < pos[v], u, v)
    od = np.bincount(lo, minlength=n)
    m = len(u)
    mn = np.minimum(deg[u], deg[v]).astype(np.float64)
    avg = 2 * m / n
    f = np.array([
        np.log2(n), np.log2(m + 1), avg, np.log2(deg.max() + 1),
        np.sqrt(max((deg.astype(np.float64) ** 2).sum() / n - avg ** 2, 0)) / avg,
        np.log2((deg.astype(np.float64) ** 2).sum() / (2 * m) + 1), np.mean(deg <= 2), np.mean(deg >= 64),
        np.log2(od.max() + 1), np.sqrt((od.astype(np.float64) ** 2).sum() / n) / (m / n),
        np.log2(mn.sum() / m + 1), np.mean(mn <= 8), np.mean(mn >= 32),
        np.log2(2 * m / (n * (n - 1.0)) + 1e-12), np.log2(np.sqrt((mn ** 2).sum() / m) + 1),
        np.log2(deg.max() / avg + 1)])
    return f


@pytest.mark.parametrize("make", [lambda: kt.gen_rmat(12, 16, 0.57, 0.19, 0.19, 3),
                                  lambda: kt.plant_cliques(*kt.gen_ba(3000, 4, 4), 2, 30, 70, 5),
                                  # one statistics block; the most blocks, several items per thread
                                  lambda: kt.gen_er(60, 0.2, 7),
                                  lambda: kt.gen_rmat(18, 16, 0.57, 0.19, 0.19, 5)])
def test_features_match_definition(make):
    torch = pytest.importorskip("torch")
    n, u, v = make()
    src, dst = both_directions(u, v)
    eng = kt.Engine(0)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    torch.cuda.synchronize()
    f = eng.features(d_src.data_ptr(), d_dst.data_ptr(), len(src), n)
    ref = _features_numpy(n, u.astype(np.int64), v.astype(np.int64))
    assert np.allclose(f, ref, rtol=1e-5, atol=1e-5), np.abs(f - ref)


def test_decompositions_with_selector_are_exact():
    torch = pytest.importorskip("torch")
    s = kt.Selector(0, seed=11)
    rng = np.random.default_rng(6)
    s.set_params(params=rng.normal(0, 0.5, so.NPARAMS))  # arbitrary choices
    eng = kt.Engine(0)
    eng.set_selector(s)
    for make in (lambda: kt.gen_rmat(13, 16, 0.57, 0.19, 0.19, 7), lambda: kt.gen_ws(6000, 10, 0.1, 8),
                 lambda: kt.plant_cliques(*kt.gen_er(4000, 0.003, 9), 3, 20, 60, 10)):
        n, u, v = make()
        src, dst = both_directions(u, v)
        d_src = torch.from_numpy(src.view(np.int32)).cuda()
        d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
        d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
        d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
        ref = oracle.decompose(n, src, dst, method="peel")
        assert int(d_k.item()) == ref["k_max"]
        assert np.array_equal(d_out.cpu().numpy().view(np.uint32), ref["truss"])
        feats = eng.features(d_src.data_ptr(), d_dst.data_ptr(), len(src), n)
        assert eng.schedule().as_tuple() == s.predict(feats)[0].as_tuple()
    eng.set_selector(None)


def test_selector_choice_stays_on_the_device_and_replays_as_a_graph():
    """With a selector attached the schedule is chosen on the device: a decomposition enqueued
    without synchronizing gives the oracle's result, the engine reports the choice once the call has
    finished, and repeat runs capture the whole pipeline - features, inference, support count and
    peel - as one CUDA graph."""
    torch = pytest.importorskip("torch")
    s = kt.Selector(0, seed=12)
    rng = np.random.default_rng(8)
    s.set_params(params=rng.normal(0, 0.5, so.NPARAMS))
    eng = kt.Engine(0)
    eng.set_selector(s)
    n, u, v = kt.plant_cliques(*kt.gen_ba(8000, 6, 13), 2, 30, 50, 14)
    src, dst = both_directions(u, v)
    d_src = torch.from_numpy(src.view(np.int32)).cuda()
    d_dst = torch.from_numpy(dst.view(np.int32)).cuda()
    d_out = torch.empty(len(src), dtype=torch.int32, device="cuda")
    d_k = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr(), sync=False)
    st = eng.stats()  # waits for the call; the schedule it ran with is the device's choice
    ref = oracle.decompose(n, src, dst, method="peel")
    assert int(d_k.item()) == ref["k_max"] and np.array_equal(d_out.cpu().numpy().view(np.uint32), ref["truss"])
    feats = eng.features(d_src.data_ptr(), d_dst.data_ptr(), len(src), n)
    assert eng.schedule().as_tuple() == s.predict(feats)[0].as_tuple()
    assert st.k_max == ref["k_max"]
    first = d_out.clone()
    eng.decompose(d_src.data_ptr(), d_dst.data_ptr(), len(src), n, d_out.data_ptr(), d_k.data_ptr())
    eng.replay()
    eng.replay()
    assert eng.replay_mode() == "cuda graph"
    assert torch.equal(d_out, first)
    eng.set_selector(None)
    eng.close()


DATA = sel_mod.DATA
HAVE_DATA = all(os.path.exists(os.path.join(DATA, f)) for f in ("selector_train.npz", "selector_heldout.npz"))


@pytest.mark.skipif(not HAVE_DATA, reason="no selector timing data")
def test_trained_selector_gains_over_default_on_heldout_graphs():
    """Trained on the training graphs' timings, the network's choices on the held-out graphs take
    less total time than the default schedule; its regret against per-graph exhaustive tuning is
    reported in the assertion message."""
    train = sel_mod.load_training()
    held = sel_mod.load(os.path.join(DATA, "selector_heldout.npz"))
    s, losses = sel_mod.train(train, epochs=300)
    assert losses[-1] < 0.8 * losses[0]
    r = sel_mod.evaluate(s, held)
    assert r["gain_vs_default"] > 1.0, r
    assert r["chosen_ms"] <= r["best_fixed_ms"] * 1.02, r
