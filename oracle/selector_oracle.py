"""selector_oracle.py — TEST INFRASTRUCTURE ONLY (the checker, never the product).

Float64 numpy restatement of the learned schedule selector's math, used to check the library's
FP32 CUDA kernels (kt_selector.cu): the 16 -> 64 -> 64 -> 19 ReLU network, its labels from the
autotuner's timings, the loss (softmax cross-entropy over the 18 variants plus the logistic loss
of the recount switch, averaged over the graphs), its gradient by backpropagation, one Adam
step, and the argmax choice.  The gradient is pinned by central finite differences in
tests/test_selector_oracle.py.  There is no reference counterpart: the reference picks its
variants by command-line flags.
"""
from __future__ import annotations

import numpy as np

F, H, V = 16, 64, 18
O = V + 1
SCHEDULES = 2 * V
W1, B1 = 0, H * F
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + O * H
NPARAMS = B3 + O


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[W1:B1].reshape(H, F), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3], p[W3:B3].reshape(O, H),
            p[B3:NPARAMS])


def labels(times):
    """Best variant (by its better recount setting) and whether recount-on beats recount-off."""
    t = np.asarray(times, np.float64).reshape(-1, V, 2)
    yv = np.argmin(t.min(axis=2), axis=1)
    yr = (t[:, :, 1].min(axis=1) < t[:, :, 0].min(axis=1)).astype(np.int64)
    return yv, yr


def forward(p, mean, scale, features):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = (np.asarray(features, np.float64) - np.asarray(mean, np.float64)) / np.asarray(scale, np.float64)
    a1 = x @ w1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ w2.T + b2
    h2 = np.maximum(a2, 0)
    o = h2 @ w3.T + b3
    return x, a1, h1, a2, h2, o


def loss_and_grad(p, mean, scale, features, times):
    """Mean loss over the graphs and its gradient with respect to the flat parameters."""
    x, a1, h1, a2, h2, o = forward(p, mean, scale, features)
    n = x.shape[0]
    yv, yr = labels(times)
    logits, z = o[:, :V], o[:, V]
    mx = logits.max(axis=1, keepdims=True)
    e = np.exp(logits - mx)
    s = e.sum(axis=1, keepdims=True)
    prob = e / s
    ce = np.log(s[:, 0]) + mx[:, 0] - logits[np.arange(n), yv]
    bce = np.maximum(z, 0) - z * yr + np.log1p(np.exp(-np.abs(z)))
    loss = float(np.mean(ce + bce))
    d_o = np.zeros_like(o)
    d_o[:, :V] = prob
    d_o[np.arange(n), yv] -= 1.0
    d_o[:, V] = 1.0 / (1.0 + np.exp(-z)) - yr
    d_o /= n
    w1, b1, w2, b2, w3, b3 = unpack(p)
    d_a2 = (d_o @ w3) * (a2 > 0)
    d_a1 = (d_a2 @ w2) * (a1 > 0)
    g = np.zeros(NPARAMS)
    g[W1:B1] = (d_a1.T @ x).ravel()
    g[B1:W2] = d_a1.sum(axis=0)
    g[W2:B2] = (d_a2.T @ h1).ravel()
    g[B2:W3] = d_a2.sum(axis=0)
    g[W3:B3] = (d_o.T @ h2).ravel()
    g[B3:NPARAMS] = d_o.sum(axis=0)
    return loss, g


def standardization(features):
    """Mean and population standard deviation per feature (1 where it is below 1e-6)."""
    f = np.asarray(features, np.float64)
    mu = f.mean(axis=0)
    sd = np.sqrt(((f - mu) ** 2).mean(axis=0))
    sd[sd <= 1e-6] = 1.0
    return mu, sd


def adam_step(p, g, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    p = p - lr * (m / (1 - beta1 ** t)) / (np.sqrt(v / (1 - beta2 ** t)) + eps)
    return p, m, v


def choose(p, mean, scale, features):
    """Schedule index (variant * 2 + recount) in the autotuner's grid order."""
    o = forward(p, mean, scale, features)[-1]
    return np.argmax(o[:, :V], axis=1) * 2 + (o[:, V] > 0)
