"""Learned rank predictor on the device against the CPU oracle, and what the
trained network gains in a sweep.

* forward pass, loss and gradient of the device kernels against the float64
  oracle (``oracle/mlp.py``, itself pinned by finite differences);
* one Adam step against the oracle's;
* device training fits a learnable target;
* recorded sweep samples: labels are the kept counts of the next visit;
* gain: a network trained on sweeps of two couplings predicts the kept ranks
  of a third coupling better than the rule without it (sketch = previous kept
  count), so the learned randomized SVD misses (regrows) less often, while
  the exact block SVD, run beside every randomized truncation on the same
  state, finds the same kept states and truncation error (within 1e-10).
"""
import numpy as np
import pytest

from oracle import mlp
from ultradmrg_gb300 import api, rank_training as RT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def _problem(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.1, mlp.N_PARAMS).astype(np.float32)
    x = rng.normal(0, 1, (n, mlp.N_IN)).astype(np.float32)
    t = rng.normal(0, 1, n).astype(np.float32)
    return p, x, t


def test_sizes(ctx):
    m = api.RankModel(ctx, 1)
    assert (m.n_in, m.n_hidden, m.n_params) == (mlp.N_IN, mlp.N_HIDDEN, mlp.N_PARAMS)
    p = m.params
    assert p.shape == (mlp.N_PARAMS,) and np.all(np.isfinite(p))


@pytest.mark.parametrize("n", [1, 37, 1000])
def test_forward_matches_oracle(ctx, n):
    p, x, _ = _problem(n, n)
    m = api.RankModel(ctx, 0)
    m.params = p
    assert np.array_equal(m.params, p)
    y = m.predict(x)
    ref, _ = mlp.forward(p, x)
    # FP32 fma chains of length 70 and 128: relative 1e-5 of the activations' scale
    scale = 1.0 + np.abs(ref)
    assert np.max(np.abs(y - ref) / scale) <= 1e-5


@pytest.mark.parametrize("n", [1, 64, 777])
def test_gradient_matches_oracle(ctx, n):
    p, x, t = _problem(n, 100 + n)
    m = api.RankModel(ctx, 0)
    m.params = p
    loss, g = m.loss_grad(x, t)
    lref, gref = mlp.loss_grad(p, x, t)
    assert abs(loss - lref) <= 1e-5 * max(1.0, lref)
    # float32 forward, float64 accumulation over samples: 1e-5 of the gradient norm
    err = np.linalg.norm(g - gref) / np.linalg.norm(gref)
    print(f"n={n}: |g - g_ref| / |g_ref| = {err:.2e}")
    assert err <= 1e-5
    # and directly against finite differences of the oracle loss on a few parameters
    idx = [0, 5, mlp.N_HIDDEN * mlp.N_IN + 3, mlp.N_PARAMS - 2, mlp.N_PARAMS - 1]
    fd = mlp.finite_difference_grad(p, x, t, idx)
    assert np.allclose(g[idx], fd, rtol=1e-4, atol=1e-6)


def test_adam_step_matches_oracle(ctx):
    n = 256
    p, x, t = _problem(n, 7)
    m = api.RankModel(ctx, 0)
    m.params = p
    _, g = m.loss_grad(x, t)
    m.train(x, t, epochs=1, batch=n, lr=1e-2, seed=0)  # one full-batch step
    got = m.params.astype(np.float64)
    ref, _, _ = mlp.adam_step(p.astype(np.float64), g.astype(np.float64), 0.0, 0.0, 1, lr=1e-2)
    # the first step is -lr * g / (|g| + eps): compare where |g| >> eps
    big = np.abs(g) > 1e-5
    assert np.max(np.abs(got - ref)[big]) <= 1e-6
    assert np.max(np.abs(got - ref)) <= 1e-2 + 1e-6


def test_training_fits_learnable_target(ctx):
    rng = np.random.default_rng(3)
    n = 4096
    x = rng.normal(0, 1, (n, mlp.N_IN)).astype(np.float32)
    w = rng.normal(0, 1, mlp.N_IN) / np.sqrt(mlp.N_IN)
    t = (np.maximum(x @ w, 0) * 3 + 1).astype(np.float32)
    m = api.RankModel(ctx, 5)
    l0, _ = m.loss_grad(x, t)
    loss = m.train(x, t, epochs=60, batch=128, lr=2e-3, seed=1)
    print(f"loss {l0:.3f} -> {loss:.4f}")
    assert loss < 0.02 * l0
    assert abs(loss - mlp.loss(m.params, x, t)) <= 1e-4 * max(loss, 1e-3) + 1e-6


SMALL = [RT.Stage(16, 1), RT.Stage(32, 1), RT.Stage(64, 2), RT.Stage(128, 2)]


def test_recorded_samples(ctx):
    chain = RT.Chain(4, 4, 8.0, 2)
    rec = api.RankModel(ctx, 0)
    e0, log, X, Y = RT.sweep_schedule(ctx, chain, SMALL[:3], model=rec, record=True, svd_mode=1)
    assert X.shape == (len(Y), mlp.N_IN) and len(Y) > 0
    kept = np.exp2(Y.astype(np.float64)) - 1
    assert np.allclose(kept, np.round(kept), atol=1e-3)  # labels log2(1 + integer)
    assert kept.max() >= 1 and np.all(kept >= 0)
    # previous-kept feature: log2(1 + k)/10 of an integer k
    pk = np.exp2(10 * X[:, mlp.N_SV + 3].astype(np.float64)) - 1
    assert np.allclose(pk, np.round(pk), atol=1e-2)


def _log_totals(log):
    return (sum(r["svd_grow_rounds"] for r in log), sum(r["svd_sketch_total"] for r in log),
            sum(r["svd_sec"] for r in log))


def test_learned_gain(ctx):
    """Trained on U = 4 and 12, evaluated on U = 8 (4x4 cylinder, 2 holes)."""
    train_chains = [RT.Chain(4, 4, U, 2) for U in (4.0, 12.0)]
    X, Y = RT.collect(ctx, train_chains, lambda c: SMALL, svd_mode=1)
    model, loss = RT.train(ctx, X, Y, epochs=300, batch=128, lr=2e-3)
    chain = RT.Chain(4, 4, 8.0, 2)
    # held-out samples of the evaluation chain: prediction error in log2(1 + kept)
    rec = api.RankModel(ctx, 0)
    _, _, Xe, Ye = RT.sweep_schedule(ctx, chain, SMALL, model=rec, record=True, svd_mode=0)
    base = 10 * Xe[:, mlp.N_SV + 3]  # the rule without the network: kept as last time
    mse_base = float(np.mean((base - Ye) ** 2))
    mse_net = float(np.mean((model.predict(Xe) - Ye) ** 2))
    # the same schedule with the randomized SVD sized by each rule, every
    # truncation judged by the exact block SVD on the same state (audit)
    _, log_prev, _, _ = RT.sweep_schedule(ctx, chain, SMALL, svd_mode=1, svd_audit=True)
    _, log_lrn, _, _ = RT.sweep_schedule(ctx, chain, SMALL, model=model, svd_mode=2,
                                         svd_audit=True)
    g_prev, s_prev, t_prev = _log_totals(log_prev)
    g_lrn, s_lrn, t_lrn = _log_totals(log_lrn)
    print(f"train loss {loss:.4f} on {len(Y)} samples; held-out mse: network {mse_net:.4f}, "
          f"previous-kept rule {mse_base:.4f}")
    print(f"grow rounds: previous-kept {g_prev}, learned {g_lrn}; "
          f"sketch columns {s_prev} vs {s_lrn}; svd s {t_prev:.3f} vs {t_lrn:.3f}")
    assert mse_net < mse_base
    assert g_lrn < g_prev
    # the truncation itself is unchanged: the exact SVD decides it
    for log in (log_prev, log_lrn):
        audited = [r for r in log if r["svd_audit_err"] >= 0]
        assert len(audited) >= len(log) // 2
        assert max(r["svd_audit_err"] for r in audited) <= 1e-10
        assert sum(r["svd_audit_kept_diff"] for r in audited) == 0
