"""The learned step-size proposer: the MLP's BF16 forward and backward kernels against the
float64 CPU oracle (oracle/mlp.py), training on the GPU, the device-side features and
step log, and the proposer inside the Dormand-Prince loop (every attempt still gated by
the embedded error estimate)."""
import math

import numpy as np
import pytest

from oracle import mlp as omlp
from simbuca_gb300 import configs, proposer
from simbuca_gb300.api import Batch

pytestmark = pytest.mark.gpu


def rand_weights(seed=0):
    return proposer.init_weights(seed) + np.random.default_rng(seed + 1).normal(
        0, 0.05, proposer.NP).astype(np.float32)


def test_param_count(ctx):
    assert ctx._L.sg_mlp_param_count() == omlp.NP == proposer.NP


def test_forward_matches_oracle(ctx):
    rng = np.random.default_rng(3)
    X = rng.normal(0, 1, (200, 16)).astype(np.float32)
    w = rand_weights(3)
    out = ctx.mlp_forward(X, w)
    ref = omlp.forward(X, w)
    assert np.abs(out - ref).max() <= 2e-5 * max(1.0, np.abs(ref).max())


def test_gradient_matches_oracle(ctx):
    rng = np.random.default_rng(4)
    X = rng.normal(0, 1, (300, 16)).astype(np.float32)
    Y = rng.normal(0, 1, 300).astype(np.float32)
    w = rand_weights(4)
    loss, g = ctx.mlp_grad(X, Y, w)
    rloss, rg = omlp.loss_and_grad(X, Y, w)
    assert loss == pytest.approx(rloss, rel=1e-5)
    assert np.abs(g - rg).max() <= 1e-4 * np.abs(rg).max()
    # and the oracle's gradient against central differences of its own loss
    k = [5, 1030, 2000, 5250, 5312]
    eps = 1e-3
    for i in k:
        wp, wm = w.astype(np.float64).copy(), w.astype(np.float64).copy()
        wp[i] += eps
        wm[i] -= eps
        fd = (omlp.loss_and_grad(X, Y, wp, bf16=False)[0] -
              omlp.loss_and_grad(X, Y, wm, bf16=False)[0]) / (2 * eps)
        an = omlp.loss_and_grad(X, Y, w, bf16=False)[1][i]
        assert fd == pytest.approx(an, rel=2e-3, abs=1e-6), i


def test_training_reduces_loss(ctx):
    rng = np.random.default_rng(5)
    X = rng.normal(0, 1, (4000, 16)).astype(np.float32)
    Y = (0.5 * np.tanh(X[:, 0]) - 0.3 * X[:, 9] + 0.1 * X[:, 12] * X[:, 13]).astype(np.float32)
    w, hist = ctx.mlp_train(X, Y, proposer.init_weights(0), iters=600, batch=256, lr=2e-3)
    assert hist[-20:].mean() < 0.1 * hist[:5].mean()
    pred = ctx.mlp_forward(X, w)
    assert np.mean((pred - Y) ** 2) < 0.1 * np.var(Y)


def test_features_and_log(ctx):
    """Device features of the logged steps against the state read back."""
    w = configs.penning_1k(n=400, seed=6)
    c = w.clouds[0]
    b = Batch(ctx, w.counts, w.fields, w.odes, 1)
    b.upload(c.pos, c.vel, c.mass, c.charge)
    b.set_log(16)
    info, _ = b.step()
    f, hp, h, e, t = b.read_log(0)
    assert len(f) == 1
    # features of the first step: the uploaded state
    L = np.sqrt(((c.pos - c.pos.mean(0)) ** 2).mean(0)).max()
    v0 = math.sqrt((c.vel ** 2).mean())
    np.testing.assert_allclose(f[0, 0:3], 0.0, atol=1e-6)
    np.testing.assert_allclose(f[0, 3:6], c.pos.std(0) / L - 1.0, atol=1e-5)
    np.testing.assert_allclose(f[0, 6:9], np.sqrt((c.vel ** 2).mean(0)) / v0 - 1.0, atol=1e-5)
    assert h[0] == pytest.approx(info[0]["h_last"]) and e[0] == pytest.approx(info[0]["err"])
    for _ in range(5):
        info, _ = b.step()
    f, hp, h, e, t = b.read_log(0)
    assert len(f) == 6
    np.testing.assert_allclose(hp[1:], h[:-1])           # h_prev chains
    np.testing.assert_allclose(f[1:, 9], np.log10(h[:-1]) + 8.0, rtol=1e-5)


def test_proposer_in_the_loop(ctx):
    """Train on a short history of one cloud, then run the same physics from another
    seed with the reference's controller and with the proposer: both runs finish, every
    accepted step met the tolerance, and the counters are reported."""
    wtrain = configs.learned_4k(n=512, seed=11, sim_time=1e-3)
    X, y = proposer.collect(ctx, wtrain, 400)
    assert len(y) > 300 and np.isfinite(X).all() and np.isfinite(y).all()
    wts, hist = ctx.mlp_train(X, y, proposer.init_weights(0), iters=800, batch=256, lr=2e-3)
    assert hist[-20:].mean() < hist[:5].mean()
    ev = configs.learned_4k(n=512, seed=12, sim_time=3e-6)
    ref = proposer.run_controller(ctx, ev, 3e-6)
    mlp = proposer.run_controller(ctx, ev, 3e-6, weights=wts, safety=0.9)
    print("reference controller", ref)
    print("proposer", mlp)
    for r in (ref, mlp):
        assert r["status"] == 0 and r["sim_us"] >= 3.0
    # the proposer is never far from the reference controller's step sizes
    assert 0.5 < mlp["mean_h"] / ref["mean_h"] < 2.0


def test_mlp_beats_the_controller_rule_on_held_out_steps(ctx):
    """What the trained network gains over the method without it, measured on steps it
    has not seen: the reference controller sets the next step from the last error ratio
    alone, h_k/h_{k-1} = err^-0.2 (up to its constant safety factor); the MLP predicts the
    same target, log(h_k err_k^-0.2 / h_{k-1}), from the cloud moments and step history.
    Its mean-squared error on held-out accepted steps must be lower."""
    X, y = [], []
    for w, n in ((configs.penning_1k(), 700), (configs.learned_4k(n=1024, seed=5), 700)):
        xi, yi = proposer.collect(ctx, w, n)
        X.append(xi)
        y.append(yi)
    X, y = np.concatenate(X), np.concatenate(y)
    assert len(y) > 1000
    test = np.random.default_rng(0).random(len(y)) < 0.2
    wts, hist = ctx.mlp_train(X[~test], y[~test], proposer.init_weights(0), iters=1500,
                              batch=256, lr=2e-3)
    pred = ctx.mlp_forward(X[test], wts)
    mse_mlp = float(np.mean((pred - y[test]) ** 2))
    # the controller rule: log ratio = -0.2 ln(err_{k-1}); feature 10 is log10 of that error
    rule = -0.2 * math.log(10.0) * X[test, 10]
    mse_rule = float(np.mean((rule - y[test]) ** 2))
    # and the best constant shift of that rule (its safety factor fitted to these data)
    shift = float(np.mean(y[~test] + 0.2 * math.log(10.0) * X[~test, 10]))
    mse_rule_fit = float(np.mean((rule + shift - y[test]) ** 2))
    print(f"held-out MSE: MLP {mse_mlp:.4g}, controller rule {mse_rule:.4g}, "
          f"rule with fitted safety {mse_rule_fit:.4g}")
    assert mse_mlp < min(mse_rule, mse_rule_fit)


def test_controller_safety_mode(ctx):
    """The ablation mode: the reference's rule with its own safety factor 0.9 reproduces
    the reference controller's run exactly; a smaller factor takes smaller steps."""
    ev = configs.learned_4k(n=512, seed=13, sim_time=1e-6)
    ctx.set_fused(False)  # the ablation runs through the proposer kernel: tiled path for both
    try:
        ref = proposer.run_controller(ctx, ev, 1e-6)
        same = proposer.run_controller(ctx, ev, 1e-6, controller_safety=0.9)
    finally:
        ctx.set_fused(True)
    for k in ("steps", "rejects", "force_evals", "sim_us"):
        assert same[k] == ref[k], k
    low = proposer.run_controller(ctx, ev, 1e-6, controller_safety=0.7)
    assert low["status"] == 0 and low["done"] == 1
    assert low["mean_h"] < ref["mean_h"]
