"""Many independent clouds of uneven size in one batch: every cloud matches its own
oracle run; per-cloud controllers, statuses and end times stay independent."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from simbuca_gb300.api import Batch
from helpers import replay_error, run_recording

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)


def small_scan(n_clouds=6, sim_time=0.3e-6):
    w = configs.scan_512(n_clouds=n_clouds, sim_time=sim_time)
    # keep the clouds small for the oracle: 33..700 ions
    counts = [33, 700, 64, 257, 128, 511][:n_clouds]
    rng = configs.rng_for(77)
    w.clouds = [configs.gaussian_cloud(rng, n, 0.5e-3, 300.0, np.full(n, 132.905)) for n in counts]
    return w


@pytest.mark.parametrize("prec,variant", [(SG_PREC_FP64, -1), (SG_PREC_FP32C, -1),
                                          (SG_PREC_FP32C, 9), (SG_PREC_FP32C, 14)])
def test_batch_matches_single_runs(ctx, prec, variant):
    """Each cloud of the batch against the oracle replaying that cloud's accepted steps,
    and against the oracle's own adaptive run for the step count; also with every cloud
    in k-d order (the launch shapes large scans take)."""
    w = small_scan()
    allc = w.concat()
    ctx.set_coulomb_variant(variant)
    try:
        b = Batch(ctx, w.counts, w.fields, w.odes, prec)
        b.upload(allc.pos, allc.vel, allc.mass, allc.charge)
        ts, hs, info = run_recording(b)
        p, v = b.download()
    finally:
        ctx.set_coulomb_variant(-1)
    off = 0
    tol = 1e-12 if prec == SG_PREC_FP64 else 1e-9
    for k, c in enumerate(w.clouds):
        n = len(c.mass)
        o = w.odes[k]
        assert info[k]["done"] == 1 and info[k]["status"] == 0
        ep, ev = replay_error(c, w.fields[k], ts[k], hs[k], p[off:off + n], v[off:off + n])
        assert ep <= tol and ev <= tol, (k, ep, ev)
        _, _, cr, _, _ = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, w.fields[k],
                                         rtol=o.rtol, atol=o.atol, h0=o.h0, t0=0.0,
                                         t_end=o.t_end)
        if prec == SG_PREC_FP64:
            assert abs(info[k]["steps"] - cr.steps) <= 1, k
        else:  # FP32c force noise moves the step sizes (see test_dp45_gpu)
            assert abs(info[k]["steps"] - cr.steps) <= max(2, cr.steps // 5), k
        off += n


def test_batch_run_equals_stepwise(ctx):
    """sg_batch_run (graph replays, no per-step sync) lands on the same state as
    sg_dp45_step called step by step."""
    w = small_scan(4)
    allc = w.concat()
    out = []
    for mode in ("run", "step"):
        b = Batch(ctx, w.counts, w.fields, w.odes, SG_PREC_FP32C)
        b.upload(allc.pos, allc.vel, allc.mass, allc.charge)
        if mode == "run":
            b.run()
        else:
            run_recording(b)
        out.append(b.download())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_one_step_each(ctx):
    w = small_scan()
    allc = w.concat()
    b = Batch(ctx, w.counts, w.fields, w.odes, SG_PREC_FP64)
    b.upload(allc.pos, allc.vel, allc.mass, allc.charge)
    for k in range(1, 3):
        info, st = b.step()
        assert all(s["steps"] == k for s in info)


def test_independent_end_times(ctx):
    w = small_scan(4)
    allc = w.concat()
    b = Batch(ctx, w.counts, w.fields, w.odes, SG_PREC_FP64)
    b.upload(allc.pos, allc.vel, allc.mass, allc.charge)
    b.set_t_end(1, 0.1e-6)
    info, _ = b.run()
    assert info[1]["t"] < info[0]["t"]
    assert 0.1e-6 <= info[1]["t"] < 0.2e-6
    assert all(s["done"] for s in info)


def test_moments(ctx):
    w = small_scan(3)
    allc = w.concat()
    b = Batch(ctx, w.counts, w.fields, w.odes, SG_PREC_FP64)
    b.upload(allc.pos, allc.vel, allc.mass, allc.charge)
    m = b.moments()
    off = 0
    for k, c in enumerate(w.clouds):
        ref = oracle.moments(c.pos, c.vel, c.mass)
        np.testing.assert_allclose(m[k], ref, rtol=1e-9, atol=1e-15)
        off += len(c.mass)


def test_sorted_order_round_trip(ctx):
    """A batch in k-d tree order: download returns the caller's order, and the
    integration matches the oracle replaying the accepted steps."""
    w = configs.penning_1k(n=3000, seed=21)
    c = w.clouds[0]
    fp = configs.penning_field(quad=(0.5, configs.nu_c(132.905), 0.0, 0.0, 1.0), delta=1e3)
    ctx.set_coulomb_variant(4)
    try:
        b = Batch(ctx, [3000], [fp], [configs.ode(1e-9, 1e-15, 1e-9, 1.0)], SG_PREC_FP32C)
        b.upload(c.pos, c.vel, c.mass, c.charge)
        p0, v0 = b.download()
        assert np.array_equal(p0, c.pos) and np.array_equal(v0, c.vel)
        ts, hs = [], []
        for _ in range(6):
            i0 = b.info()[0]
            info, st = b.step()
            ts.append(i0["t"])
            hs.append(info[0]["h_last"])
        p, v = b.download()
    finally:
        ctx.set_coulomb_variant(-1)
    ep, ev = replay_error(c, fp, np.array(ts), np.array(hs), p, v)
    assert ep <= 1e-9 and ev <= 1e-9, (ep, ev)


@pytest.mark.parametrize("variant", [4, 7])
def test_sorted_set_state_keeps_order(ctx, variant):
    """set_state on a k-d ordered batch keeps the ion order (only the tile bounds move):
    the caller's order comes back and the next steps still match the oracle."""
    w = configs.penning_1k(n=4000, seed=22)
    c = w.clouds[0]
    fp = configs.penning_field(delta=1e3)
    ctx.set_coulomb_variant(variant)
    try:
        b = Batch(ctx, [4000], [fp], [configs.ode(1e-9, 1e-15, 1e-9, 1.0)], SG_PREC_FP32C)
        b.upload(c.pos, c.vel, c.mass, c.charge)
        rng = np.random.default_rng(5)
        p1 = c.pos + rng.normal(0, 2e-5, c.pos.shape)  # every ion moved
        v1 = c.vel * 0.9
        b.set_state(p1, v1)
        p, v = b.download()
        assert np.array_equal(p, p1) and np.array_equal(v, v1)
        t0 = b.info()[0]["t"]
        ts, hs = [], []
        for _ in range(4):
            i0 = b.info()[0]
            info, _ = b.step()
            ts.append(i0["t"])
            hs.append(info[0]["h_last"])
        p, v = b.download()
    finally:
        ctx.set_coulomb_variant(-1)
    from simbuca_gb300.configs import Cloud
    ep, ev = replay_error(Cloud(p1, v1, c.mass, c.charge), fp, np.array(ts), np.array(hs), p, v)
    assert ep <= 1e-9 and ev <= 1e-9, (ep, ev)


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_ragged_edges(ctx, prec):
    """One-, two- and three-ion clouds, a cloud without the Coulomb term and a larger
    cloud in one batch, each with its own end time: every cloud matches the oracle
    replaying its accepted steps."""
    rng = configs.rng_for(88)
    counts = [1, 2, 3, 700, 40]
    clouds = [configs.gaussian_cloud(rng, n, 0.4e-3, 300.0, np.full(n, 132.905)) for n in counts]
    fields = [configs.penning_field(delta=1e3) for _ in counts]
    fields[4] = configs.penning_field(coulomb=False, delta=1e3)
    odes = [configs.ode(1e-9, 1e-15, 1e-9, t) for t in (2e-7, 3e-7, 1e-7, 2.5e-7, 4e-7)]
    allp = np.concatenate([c.pos for c in clouds])
    allv = np.concatenate([c.vel for c in clouds])
    allm = np.concatenate([c.mass for c in clouds])
    allq = np.concatenate([c.charge for c in clouds])
    b = Batch(ctx, counts, fields, odes, prec)
    b.upload(allp, allv, allm, allq)
    ts, hs, info = run_recording(b)
    p, v = b.download()
    off = 0
    tol = 1e-12 if prec == SG_PREC_FP64 else 1e-9
    for k, c in enumerate(clouds):
        n = counts[k]
        assert info[k]["done"] == 1 and info[k]["status"] == 0
        assert info[k]["t"] >= odes[k].t_end
        ep, ev = replay_error(c, fields[k], ts[k], hs[k], p[off:off + n], v[off:off + n])
        assert ep <= tol and ev <= tol, (k, ep, ev)
        off += n
