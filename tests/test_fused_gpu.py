"""The fused small-cloud path: whole Dormand-Prince attempts of FP32c clouds of up to
2,048 ions in one thread-block-cluster launch per cloud.

The default takes clouds of up to 512 ions (where it beats the tiled kernels); these
tests force it up to 2,048.  It must integrate exactly what the reference's step() loop integrates
(bin/ode.cpp:61-218, 426-494) with the FP32c force of the tiled path: the oracle
replays its accepted schedule to FP32c rounding, its step counts follow the oracle's
own adaptive run, a fixed-step run agrees with the tiled kernels' and with the FP64
form, clouds of a ragged batch advance exactly as they do alone, and the controller's
statuses (underflow, reject budget) come on the same attempt as in the oracle."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import abi, configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from simbuca_gb300.api import Batch
from helpers import TRAPP, paul_fp, replay_error, run_recording

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle(ctx):
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)
    ctx.set_fused(2)  # up to 2,048 ions (the default takes clouds of up to 512)
    yield
    ctx.set_fused(1)


def drive_field():
    return configs.penning_field(quad=(0.5, configs.nu_c(132.905), 0.0, 0.0, 1.0),
                                 dipole=(0.1, 1138.4, 0.0, 0.0, 1.0), delta=1e3)


def batch_of(ctx, clouds, fp, t_end, prec=SG_PREC_FP32C, adaptive=True, h0=1e-9,
             max_rejects=0, beta=0.0):
    op = configs.ode(1e-9, 1e-15, h0, t_end, adaptive=adaptive, max_rejects=max_rejects,
                     beta=beta)
    b = Batch(ctx, [len(c.mass) for c in clouds], [fp] * len(clouds), [op] * len(clouds), prec)
    cat = configs.Workload("b", clouds, [fp] * len(clouds), [op] * len(clouds), t_end).concat()
    b.upload(cat.pos, cat.vel, cat.mass, cat.charge)
    return b


@pytest.mark.parametrize("n", [300, 1000, 2048])
def test_fused_path_against_oracle(ctx, n):
    c = configs.penning_1k(n=n, seed=40 + n).clouds[0]
    fp = drive_field()
    t_end = 0.3e-6 if n < 2048 else 0.1e-6
    b = batch_of(ctx, [c], fp, t_end)
    assert b.fused() > 0
    ts, hs, last = run_recording(b)
    assert last[0]["status"] == 0 and last[0]["done"] == 1
    p, v = b.download()
    ep, ev = replay_error(c, fp, ts[0], hs[0], p, v)
    print(n, "steps", last[0]["steps"], "rejects", last[0]["rejects"], "replay", ep, ev)
    assert ep <= 1e-9 and ev <= 1e-9, (ep, ev)
    _, _, cr, _, _ = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fp, rtol=1e-9,
                                     atol=1e-15, h0=1e-9, t0=0.0, t_end=t_end)
    assert abs(last[0]["steps"] - cr.steps) <= max(2, cr.steps // 10)
    # the in-run check ran on the fused sums
    rec = b.force_check()[0]
    assert rec["breaches"] == 0 and rec["max_err"] <= 1e-6


def test_fused_matches_tiled_and_fp64_on_fixed_steps(ctx):
    """40 fixed 4 ns steps of a 1,000-ion cloud: the fused path, the tiled FP32c kernels
    and the FP64 form agree to the FP32c force error carried through the steps."""
    c = configs.penning_1k(n=1000, seed=3).clouds[0]
    fp = drive_field()
    out = {}
    for tag, prec, fused in (("fused", SG_PREC_FP32C, True), ("tiled", SG_PREC_FP32C, False),
                             ("fp64", SG_PREC_FP64, False)):
        ctx.set_fused(2 if fused else 0)
        try:
            b = batch_of(ctx, [c], fp, 1.0, prec=prec, adaptive=False, h0=4e-9)
            assert (b.fused() > 0) == fused
            info, _ = b.run(max_attempts=40)
            assert info[0]["steps"] == 40
            out[tag] = b.download()
        finally:
            ctx.set_fused(2)
    for tag in ("fused", "tiled"):
        ep = np.abs(out[tag][0] - out["fp64"][0]).max() / np.abs(out["fp64"][0]).max()
        ev = np.abs(out[tag][1] - out["fp64"][1]).max() / np.abs(out["fp64"][1]).max()
        print(tag, "vs fp64", ep, ev)
        assert ep <= 1e-9 and ev <= 1e-9


def test_ragged_batch(ctx):
    """Each cloud of a batch has its own cluster: in a ragged batch (1 to 2,048 ions, one
    of them a single ion) every cloud's state is the oracle's replay of its own accepted
    schedule, and it takes the steps it takes alone.  (Bit-for-bit equality with the
    single run is not expected: the stage-1 Coulomb sum of an upload is taken by the
    tiled kernels, whose work split depends on the whole batch.)"""
    counts = [1, 2, 31, 33, 517, 2048]
    clouds = [configs.penning_1k(n=n, seed=60 + k).clouds[0] for k, n in enumerate(counts)]
    fp = drive_field()
    t_end = 0.05e-6
    b = batch_of(ctx, clouds, fp, t_end)
    R = b.fused()
    assert R > 0
    ts, hs, last = run_recording(b)
    assert all(i["done"] and i["status"] == 0 for i in last)
    p, v = b.download()
    off = 0
    for k, c in enumerate(clouds):
        n = len(c.mass)
        pk, vk = p[off:off + n], v[off:off + n]
        ep, ev = replay_error(c, fp, ts[k], hs[k], pk, vk)
        assert ep <= 1e-9 and ev <= 1e-9, (k, ep, ev)
        b1 = batch_of(ctx, [c], fp, t_end)
        _, _, l1 = run_recording(b1)
        print(n, "cluster", R, b1.fused(), "replay", ep, ev, "steps", last[k]["steps"],
              l1[0]["steps"])
        assert abs(l1[0]["steps"] - last[k]["steps"]) <= 1
        off += n


def test_one_step_per_call(ctx):
    """sg_dp45_step on the fused path: every call takes exactly one accepted step of every
    cloud, its rejected attempts included in the same launch."""
    clouds = [configs.penning_1k(n=n, seed=70 + n).clouds[0] for n in (200, 900)]
    b = batch_of(ctx, clouds, drive_field(), 1.0)
    prev = b.info()
    for _ in range(25):
        cur, st = b.step()
        assert st == 0
        for a, p0 in zip(cur, prev):
            assert a["steps"] == p0["steps"] + 1
        prev = cur


def test_underflow_and_reject_budget(ctx):
    """A nearly coincident pair keeps every attempt rejected at the 0.2 floor: underflow
    at the oracle's attempt (|h| <= |pos[0][0]| eps, bin/ode.cpp:482), and a reject budget
    of 3 stops the cloud at its third reject."""
    c = configs.penning_1k(n=256, seed=21).clouds[0]
    pos = c.pos.copy()
    pos[2] = pos[1] + 1e-13
    fp = paul_fp(TRAPP)
    _, _, cr, _, _ = oracle.dp45_run(pos, c.vel, c.mass, c.charge, fp, rtol=1e-15, atol=1e-30,
                                     h0=1e-9, t0=0.0, t_end=1e-6, max_steps=2, hist_cap=10)
    assert cr.status == abi.SG_H_UNDERFLOW
    from simbuca_gb300.configs import Cloud
    cl = Cloud(pos, c.vel, c.mass, c.charge)
    op = configs.ode(1e-15, 1e-30, 1e-9, 1e-6)
    b = Batch(ctx, [len(c.mass)], [fp], [op], SG_PREC_FP32C)
    b.upload(cl.pos, cl.vel, cl.mass, cl.charge)
    assert b.fused() > 0
    info, _ = b.run(max_attempts=200, raise_on_error=False)
    assert info[0]["status"] == abi.SG_H_UNDERFLOW and info[0]["rejects"] == cr.rejects
    op = configs.ode(1e-15, 1e-30, 1e-9, 1e-6, max_rejects=3)
    b = Batch(ctx, [len(c.mass)], [fp], [op], SG_PREC_FP32C)
    b.upload(cl.pos, cl.vel, cl.mass, cl.charge)
    info, st = b.step(raise_on_error=False)
    assert st == abi.SG_TOO_MANY_REJECTS and info[0]["rejects"] == 3


def test_pi_controller_on_the_fused_path(ctx):
    """beta of the PI controller reaches the fused path's controller: FP32c steps follow
    the oracle's PI history to the FP32c noise of the error norm."""
    c = configs.penning_1k(n=500, seed=81).clouds[0]
    fp = drive_field()
    t_end = 0.2e-6
    _, _, cr, oh, _ = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fp, rtol=1e-9,
                                      atol=1e-15, h0=1e-9, t0=0.0, t_end=t_end,
                                      hist_cap=100000, beta=0.08)
    b = batch_of(ctx, [c], fp, t_end, beta=0.08)
    ts, hs, last = run_recording(b)
    p, v = b.download()
    ep, ev = replay_error(c, fp, ts[0], hs[0], p, v)
    assert ep <= 1e-9 and ev <= 1e-9
    assert abs(last[0]["steps"] - cr.steps) <= max(2, cr.steps // 10)
    # FP32c force noise reaches the error norm through its atol-scaled components, so
    # the step sizes follow the oracle's on average (as in the tiled path's test)
    ho = oh[oh[:, 3] == 1][:, 1]
    np.testing.assert_allclose(np.mean(hs[0][3:]), np.mean(ho[3:]), rtol=0.05)
