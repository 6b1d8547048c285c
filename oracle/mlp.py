"""CPU oracle of the learned rank predictor (test infrastructure only).

The reference has no learned truncation; this module restates, in float64
numpy, exactly what the device kernels compute so their forward pass,
gradients and Adam step can be checked:

* features of one bond sector (64 scaled log10 singular values of the previous
  visit, the sector's QN offset from the dominant sector, log10 of the
  truncation cutoff, log2(1 + kept at the previous visit), log10 of the bond's
  smallest kept singular value at the previous visit, log2(Dmax / previous
  bond dimension));
* ``y = w2 . relu(W1 x + b1) + b2`` with parameters packed as
  ``W1 (hidden x in, row-major) | b1 | w2 | b2``;
* mean-squared-error loss and its gradient, the gradient checked here against
  central finite differences;
* one Adam step (Kingma & Ba 2015, bias-corrected moments).
"""
from __future__ import annotations

import numpy as np

N_SV = 64
N_IN = N_SV + 6
N_HIDDEN = 128
N_PARAMS = N_HIDDEN * N_IN + 2 * N_HIDDEN + 1


def features(svals, qn, top_qn, trunc_err, prev_kept, prev_cut, growth):
    """Feature vector of one sector (float32, like the device code)."""
    out = np.zeros(N_IN, np.float64)
    s = np.zeros(N_SV)
    sv = np.asarray(svals, np.float64)[:N_SV]
    s[: len(sv)] = sv
    out[:N_SV] = np.log10(np.maximum(s, 1e-20)) / 10.0
    out[N_SV] = (qn[0] - top_qn[0]) / 4.0
    out[N_SV + 1] = (qn[1] - top_qn[1]) / 4.0
    out[N_SV + 2] = np.log10(max(trunc_err, 1e-30)) / 10.0
    out[N_SV + 3] = np.log2(1.0 + prev_kept) / 10.0
    out[N_SV + 4] = np.log10(max(prev_cut, 1e-20)) / 10.0
    out[N_SV + 5] = growth
    return out.astype(np.float32)


def unpack(p):
    p = np.asarray(p, np.float64)
    H, I = N_HIDDEN, N_IN
    W1 = p[: H * I].reshape(H, I)
    b1 = p[H * I: H * I + H]
    w2 = p[H * I + H: H * I + 2 * H]
    b2 = p[H * I + 2 * H]
    return W1, b1, w2, b2


def forward(p, x):
    W1, b1, w2, b2 = unpack(p)
    pre = np.asarray(x, np.float64) @ W1.T + b1
    return np.maximum(pre, 0.0) @ w2 + b2, pre


def loss(p, x, t):
    y, _ = forward(p, x)
    return float(np.mean((y - np.asarray(t, np.float64)) ** 2))


def loss_grad(p, x, t):
    """(loss, gradient) of the mean squared error."""
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    W1, b1, w2, b2 = unpack(p)
    y, pre = forward(p, x)
    n = x.shape[0]
    dy = 2.0 * (y - t) / n
    act = np.maximum(pre, 0.0)
    gw2 = act.T @ dy
    gb2 = dy.sum()
    dpre = np.outer(dy, w2) * (pre > 0)
    gW1 = dpre.T @ x
    gb1 = dpre.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gw2, [gb2]])
    return float(np.mean((y - t) ** 2)), g


def finite_difference_grad(p, x, t, idx, h=1e-6):
    """Central differences of the loss for the parameters ``idx``."""
    p = np.asarray(p, np.float64).copy()
    out = np.zeros(len(idx))
    for j, i in enumerate(idx):
        old = p[i]
        p[i] = old + h
        lp = loss(p, x, t)
        p[i] = old - h
        lm = loss(p, x, t)
        p[i] = old
        out[j] = (lp - lm) / (2 * h)
    return out


def adam_step(p, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update; returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def predicted_sketch(y):
    """Kept count predicted from the network output y = log2(1 + kept)."""
    return np.maximum(0.0, np.ceil(np.exp2(np.asarray(y, np.float64)) - 1.0)).astype(np.int64)
