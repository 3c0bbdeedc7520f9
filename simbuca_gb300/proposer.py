"""The learned step-size proposer: collecting step histories, training, evaluation.

    python -m simbuca_gb300.proposer [--out DIR] [--quick] [--eval WORKLOAD --horizon S]

1. collect: run the Penning-trap workloads (1,000 ions; 65,536 ions with drive and
   friction; the 1M-ion spheroid) with the reference's controller and the device-side
   step log on; every accepted step gives (features at its start, target), the target
   being log(h_k err_k^-0.2 / h_{k-1}), the step-size ratio that would have met the
   tolerance exactly.
2. train: the MLP 16 -> 64 -> 64 -> 1 (BF16 weights, FP32 accumulation) on the GPU
   with the library's own forward, backward and Adam kernels (sg_mlp_train).
3. evaluate: by default the 4,096-ion cloud under a dipole drive at nu_minus then a
   quadrupole drive at nu_c (--eval names another workload of configs.WORKLOADS, e.g.
   penning_65k), once with the reference's controller and once with the proposer per
   safety factor, from the same state; every attempt is accepted or rejected by the
   Dormand-Prince error estimate in both.  Reported: rejected-attempt fraction, force
   evaluations per simulated microsecond and simulated microseconds per wall second.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from . import abi, configs
from .api import Batch, Context

NP = 64 * 16 + 64 + 64 * 64 + 64 + 64 + 1

# Weights trained by `python -m simbuca_gb300.proposer --eval penning_65k --horizon 4e-7
# --max-attempts 1000 --no-fp64-eval --safety 0.8,0.85,0.9` on a GB300 (2,303 accepted
# steps of the 1,000-ion, 65,536-ion and 1M-ion workloads, 4,000 Adam iterations).
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                               "proposer_weights.npy")
# The safety factor of the trained proposer on the 65,536-ion workload's study: fewest
# force evaluations per simulated microsecond of 0.8, 0.85 and 0.9.
DEFAULT_SAFETY = 0.85


def default_weights() -> np.ndarray:
    """The shipped trained weights (FP32 master copy, NP values)."""
    w = np.load(DEFAULT_WEIGHTS).astype(np.float32)
    if w.shape != (NP,) or not np.isfinite(w).all():
        raise RuntimeError(f"{DEFAULT_WEIGHTS}: not a trained proposer")
    return w


def init_weights(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, math.sqrt(1.0 / 16), 64 * 16), np.zeros(64),
             rng.normal(0, math.sqrt(1.0 / 64), 64 * 64), np.zeros(64),
             rng.normal(0, math.sqrt(1.0 / 64), 64) * 0.1, np.zeros(1)]
    return np.concatenate(parts).astype(np.float32)


def drop_features(w: np.ndarray, feats) -> np.ndarray:
    """Weights that ignore the given inputs: their first-layer columns set to zero
    (trained with those inputs zeroed, they then stay zero)."""
    w = np.array(w, np.float32, copy=True)
    w[:64 * 16].reshape(64, 16)[:, list(feats)] = 0.0
    return w


def targets(h_prev, h, err):
    err = np.maximum(err, 1e-12)
    y = np.log(h * err ** -0.2 / np.where(h_prev > 0, h_prev, h))
    return np.clip(y, math.log(0.2), math.log(10.0)).astype(np.float32)


def collect(ctx: Context, w: configs.Workload, n_steps: int, precision=abi.SG_PREC_FP32C,
            skip: int = 3):
    """Run n_steps accepted steps of the workload with the step log on; (X, y)."""
    allc = w.concat()
    b = Batch(ctx, w.counts, w.fields, w.odes, precision)
    b.upload(allc.pos, allc.vel, allc.mass, allc.charge)
    b.set_log(n_steps + 8)
    for _ in range(n_steps):
        info, st = b.step(raise_on_error=False)
        if st != 0 or all(s["done"] for s in info):
            break
    Xs, ys = [], []
    for c in range(len(w.counts)):
        f, hp, h, e, t = b.read_log(c)
        keep = slice(skip, None)  # the first steps grow from h0 = 1 ns
        Xs.append(f[keep])
        ys.append(targets(hp[keep], h[keep], e[keep]))
    return np.concatenate(Xs), np.concatenate(ys)


def run_controller(ctx: Context, w: configs.Workload, horizon: float, weights=None,
                   safety=0.9, precision=abi.SG_PREC_FP32C, state=None,
                   max_attempts: int = 100000, controller_safety=None, beta: float = 0.0,
                   log_cap: int = 0):
    """Advance one workload by `horizon` seconds (at most max_attempts attempts; `done`
    tells whether the horizon was reached); returns the controller's counters (and,
    with log_cap > 0, the step log of cloud 0 under "log")."""
    allc = w.concat()
    odes = [configs.ode(o.rtol, o.atol, o.h0, o.t0 + horizon, t0=o.t0, beta=beta)
            for o in w.odes]
    b = Batch(ctx, w.counts, w.fields, odes, precision)
    if state is None:
        b.upload(allc.pos, allc.vel, allc.mass, allc.charge)
    else:
        b.upload(state[0], state[1], allc.mass, allc.charge)
    if weights is not None:
        b.set_proposer(weights, safety)
    elif controller_safety is not None:
        b.set_controller_safety(controller_safety)
    if log_cap > 0:
        b.set_log(log_cap)
    t0 = time.perf_counter()
    info, st = b.run(max_attempts=max_attempts, raise_on_error=False)
    wall = time.perf_counter() - t0
    s = info[0]
    sim_us = (s["t"] - w.odes[0].t0) * 1e6
    attempts = s["steps"] + s["rejects"]
    out = {"steps": s["steps"], "rejects": s["rejects"], "attempts": attempts,
           "reject_fraction": s["rejects"] / max(attempts, 1),
           "force_evals": s["force_evals"], "coulomb_evals": s["coulomb_evals"],
           "force_evals_per_sim_us": s["force_evals"] / sim_us, "sim_us": sim_us,
           "wall_s": wall, "sim_us_per_wall_s": sim_us / wall, "status": s["status"],
           "done": s["done"],
           "mean_h": sim_us * 1e-6 / max(s["steps"], 1)}
    if log_cap > 0:
        out["log"] = b.read_log(0)
    return out


def compare(ctx: Context, w: configs.Workload, horizon: float, betas, weights=None,
            safety=DEFAULT_SAFETY, log_cap: int = 0, max_attempts: int = 1 << 40,
            on_result=None):
    """The same workload and horizon under the reference's I-controller and PI
    controllers (beta > 0), and with the learned proposer when weights are given."""
    res = {}
    for beta in betas:
        tag = "i_controller" if beta == 0 else f"pi_beta_{beta}"
        res[tag] = run_controller(ctx, w, horizon, beta=beta, log_cap=log_cap,
                                  max_attempts=max_attempts)
        if on_result:
            on_result(tag, res[tag])
    if weights is not None:
        tag = f"mlp_safety_{safety}"
        res[tag] = run_controller(ctx, w, horizon, weights=weights, safety=safety,
                                  log_cap=log_cap, max_attempts=max_attempts)
        if on_result:
            on_result(tag, res[tag])
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=".")
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--horizon", type=float, default=1e-3)
    ap.add_argument("--safety", default="0.75,0.8,0.85,0.9")
    ap.add_argument("--eval", default="learned_4k", choices=sorted(configs.WORKLOADS))
    ap.add_argument("--no-fp64-eval", action="store_true")
    ap.add_argument("--drop-features", default="",
                    help="comma-separated input indices the network ignores (e.g. 9, the "
                         "absolute log step size)")
    ap.add_argument("--max-attempts", type=int, default=100000,
                    help="attempt cap of each evaluation run")
    ap.add_argument("--compare", action="store_true",
                    help="no training: run the evaluation workload under the controllers "
                         "of --betas (and the shipped proposer with --with-mlp), write "
                         "compare.json and the step logs (compare_logs.npz) to --out")
    ap.add_argument("--betas", default="0,0.04,0.08")
    ap.add_argument("--with-mlp", action="store_true")
    ap.add_argument("--seed", type=int, default=None,
                    help="seed of the evaluation cloud (learned_4k only; default its own)")
    ap.add_argument("--log-cap", type=int, default=0)
    a = ap.parse_args()
    ctx = Context(0)
    t0 = time.perf_counter()
    if a.compare:
        kw = {} if a.seed is None else {"seed": a.seed}
        ev = (configs.learned_4k(sim_time=a.horizon, **kw) if a.eval == "learned_4k"
              else configs.WORKLOADS[a.eval]())
        def save(tag, r):
            with open(os.path.join(a.out, f"compare_{tag}.json"), "w") as f:
                json.dump({k: v for k, v in r.items() if k != "log"}, f, indent=1)
            print(tag, json.dumps({k: v for k, v in r.items() if k != "log"}), flush=True)

        res = compare(ctx, ev, a.horizon, [float(b) for b in a.betas.split(",")],
                      weights=default_weights() if a.with_mlp else None,
                      log_cap=a.log_cap, max_attempts=a.max_attempts, on_result=save)
        logs = {}
        for k, r in res.items():
            lg = r.pop("log", None)
            if lg is not None:
                for name, arr in zip(("feat", "h_prev", "h", "err", "t"), lg):
                    logs[f"{k}__{name}"] = arr
        res["workload"] = a.eval
        res["horizon_s"] = a.horizon
        res["seed"] = a.seed
        print(json.dumps(res, indent=1), flush=True)
        with open(os.path.join(a.out, "compare.json"), "w") as f:
            json.dump(res, f, indent=1)
        if logs:
            np.savez_compressed(os.path.join(a.out, "compare_logs.npz"), **logs)
        ctx.close()
        return
    X, y = [], []
    plan = [(configs.penning_1k(), 600 if a.quick else 2000),
            (configs.penning_65k(), 60 if a.quick else 300),
            (configs.spheroid_1m(), 0 if a.quick else 12)]
    for w, n in plan:
        if n == 0:
            continue
        xi, yi = collect(ctx, w, n)
        X.append(xi)
        y.append(yi)
        print(f"collected {len(yi)} steps from {w.name}", flush=True)
    X = np.concatenate(X)
    y = np.concatenate(y)
    dropped = [int(v) for v in a.drop_features.split(",") if v.strip()]
    if dropped:
        X[:, dropped] = 0.0
    # hold out every fifth sample to compare the MLP with the reference controller's rule
    rng = np.random.default_rng(0)
    test = rng.random(len(y)) < 0.2
    w0 = drop_features(init_weights(0), dropped)
    wts, hist = ctx.mlp_train(X[~test], y[~test], w0, iters=300 if a.quick else 4000,
                              batch=256, lr=2e-3)
    pred = ctx.mlp_forward(X[test], wts)
    mse_mlp = float(np.mean((pred - y[test]) ** 2))
    # the reference's I-controller predicts log(h*_k / h_{k-1}) as -0.2 ln(err_{k-1})
    ctrl_pred = -0.2 * math.log(10.0) * X[test, 10]
    mse_ctrl = float(np.mean((ctrl_pred - y[test]) ** 2))
    print(f"trained on {int((~test).sum())} samples: loss {hist[0]:.4g} -> {hist[-1]:.4g}; "
          f"held-out MSE mlp {mse_mlp:.4g} vs controller rule {mse_ctrl:.4g}", flush=True)
    # retrain on everything for the deployed weights
    wts, hist = ctx.mlp_train(X, y, w0, iters=300 if a.quick else 4000, batch=256, lr=2e-3)
    np.save(os.path.join(a.out, "proposer_weights.npy"), wts)
    ev = (configs.learned_4k(sim_time=a.horizon) if a.eval == "learned_4k"
          else configs.WORKLOADS[a.eval]())
    res = {"eval_workload": a.eval, "dropped_features": dropped, "train_samples": int(len(y)),
           "train_loss_first": float(hist[0]),
           "train_loss_last": float(hist[-1]), "heldout_mse_mlp": mse_mlp,
           "heldout_mse_controller_rule": mse_ctrl, "horizon_s": a.horizon,
           "reference_controller": run_controller(ctx, ev, a.horizon,
                                                 max_attempts=a.max_attempts)}
    if not a.quick and not a.no_fp64_eval:
        res["reference_controller_fp64"] = run_controller(ctx, ev, a.horizon,
                                                          precision=abi.SG_PREC_FP64)
    for s in [float(v) for v in a.safety.split(",")]:
        res[f"mlp_safety_{s}"] = run_controller(ctx, ev, a.horizon, weights=wts, safety=s,
                                                max_attempts=a.max_attempts)
        # the same safety in the reference's own rule: what learning adds beyond it
        res[f"controller_safety_{s}"] = run_controller(ctx, ev, a.horizon, controller_safety=s,
                                                       max_attempts=a.max_attempts)
    res["collect_and_train_s"] = time.perf_counter() - t0
    print(json.dumps(res, indent=1))
    with open(os.path.join(a.out, "proposer_eval.json"), "w") as f:
        json.dump(res, f, indent=1)
    ctx.close()


if __name__ == "__main__":
    main()
