"""Dormand-Prince integration on the device against the reference's goldens and the
oracle: attempt histories (h, err, accept), fixed-step trajectories, Penning runs
with stage times t + c_s h, and the failure statuses.

Trajectory parity is checked by replay: the oracle re-runs the exact step sequence
(t_k, h_k) the device accepted.  Comparing two independently controlled adaptive runs
at their end time is ill-conditioned at rtol 1e-9, atol 1e-15: components near zero
have scale atol, so the error norm carries ~1e-8 relative rounding noise, which moves
the step sizes and hence the end time; a 1e-15 perturbation of the initial state of
the oracle alone changes its final velocities by ~5e-8 this way."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import abi, configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from simbuca_gb300.api import Batch
from helpers import TRAPP, paul_fp, replay_error, run_recording

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)


def one_cloud(ctx, pos, vel, mass, charge, fp, rtol, atol, h0, t_end, prec, adaptive=True,
              max_rejects=0, method=5, beta=0.0):
    op = configs.ode(rtol, atol, h0, t_end, adaptive=adaptive, max_rejects=max_rejects,
                     method=method, beta=beta)
    b = Batch(ctx, [len(mass)], [fp], [op], prec)
    b.upload(pos, vel, mass, charge)
    return b


def attempt_history(b, max_attempts=100000):
    """Run attempt by attempt, recording (t_start, h, err, accepted) like the golden."""
    hist = []
    prev = b.info()[0]
    for _ in range(max_attempts):
        if prev["done"]:
            break
        b.attempts(1)
        cur = b.info()[0]
        acc = cur["steps"] > prev["steps"]
        hist.append((prev["t"], prev["h"], cur["err"], 1.0 if acc else 0.0))
        prev = cur
    return np.array(hist), prev


@pytest.mark.parametrize("tag", ["tight", "default"])
def test_golden_adaptive_fp64(ctx, tag):
    g = np.load(os.path.join(GOLD, "dp45_adaptive.npz"))
    rtol, atol, t_end, h0 = g[f"{tag}_cfg"]
    fp = paul_fp(TRAPP)
    b = one_cloud(ctx, g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"], g[f"{tag}_charge"],
                  fp, rtol, atol, h0, t_end, SG_PREC_FP64)
    hist, last = attempt_history(b)
    gh = g[f"{tag}_hist"]
    assert hist.shape == gh.shape
    assert np.array_equal(hist[:, 3], gh[:, 3])          # same accept/reject sequence
    np.testing.assert_allclose(hist[:, :2], gh[:, :2], rtol=1e-8)    # t, h
    # error norms; tiny norms of the first steps sit on the rounding floor
    np.testing.assert_allclose(hist[:, 2], gh[:, 2], rtol=1e-5, atol=1e-9)
    assert last["steps"] == int(g[f"{tag}_ctrl"][5])
    p, v = b.download()
    # same schedule through the oracle: state to rounding
    acc = hist[hist[:, 3] == 1]
    from simbuca_gb300.configs import Cloud
    c0 = Cloud(g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"], g[f"{tag}_charge"])
    ep, ev = replay_error(c0, fp, acc[:, 0], acc[:, 1], p, v)
    assert ep <= 1e-12 and ev <= 1e-12, (ep, ev)
    # and the reference's own end state, within the schedule sensitivity
    np.testing.assert_allclose(p, g[f"{tag}_pos"], rtol=1e-6, atol=1e-12)


def test_golden_adaptive_fp32c(ctx):
    g = np.load(os.path.join(GOLD, "dp45_adaptive.npz"))
    tag = "tight"
    rtol, atol, t_end, h0 = g[f"{tag}_cfg"]
    fp = paul_fp(TRAPP)
    b = one_cloud(ctx, g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"], g[f"{tag}_charge"],
                  fp, rtol, atol, h0, t_end, SG_PREC_FP32C)
    ts, hs, last = run_recording(b)
    assert last[0]["status"] == 0 and last[0]["done"] == 1
    p, v = b.download()
    from simbuca_gb300.configs import Cloud
    c0 = Cloud(g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"], g[f"{tag}_charge"])
    ep, ev = replay_error(c0, fp, ts[0], hs[0], p, v)
    assert ep <= 1e-9 and ev <= 1e-9, (ep, ev)
    # accepted/rejected counts of the FP64 reference run
    assert abs(last[0]["steps"] - int(g[f"{tag}_ctrl"][5])) <= 1


@pytest.mark.parametrize("beta", [0.04, 0.08])
def test_pi_controller_vs_oracle(ctx, beta):
    """The PI controller (beta of bin/ode.cpp:431-439) on the device against the oracle's
    restatement, FP64: the golden's Paul-trap cloud at its tight tolerances (the whole
    attempt history), and a Penning cloud with drive and friction (the accepted step
    sizes, which follow the last bits of the first steps' error norms: see the test of
    the reference controller below)."""
    g = np.load(os.path.join(GOLD, "dp45_adaptive.npz"))
    tag = "tight"
    rtol, atol, t_end, h0 = g[f"{tag}_cfg"]
    fp = paul_fp(TRAPP)
    args = (g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"], g[f"{tag}_charge"], fp)
    _, _, cr, oh, nh = oracle.dp45_run(*args, rtol=rtol, atol=atol, h0=h0, t0=0.0,
                                       t_end=t_end, hist_cap=100000, beta=beta)
    assert cr.status == 0
    b = one_cloud(ctx, *args, rtol, atol, h0, t_end, SG_PREC_FP64, beta=beta)
    hist, last = attempt_history(b)
    assert hist.shape == oh.shape
    assert np.array_equal(hist[:, 3], oh[:, 3])          # same accept/reject sequence
    # The first step's error norm sits on the rounding floor (~1e-6 relative between
    # the device's and the oracle's summation orders).  The I-controller clamps the
    # growth after it at 10x, so its step sizes never see that noise; the PI factor
    # errold^beta lowers the scale below the clamp, and the noise, times alpha, stays
    # in every later step size.
    np.testing.assert_allclose(hist[:, :2], oh[:, :2], rtol=1e-5)
    np.testing.assert_allclose(hist[:, 2], oh[:, 2], rtol=1e-5, atol=1e-9)
    assert last["steps"] == cr.steps and last["rejects"] == cr.rejects

    c = configs.penning_1k(n=300, seed=11).clouds[0]
    fpn = configs.penning_field(quad=(0.5, configs.nu_c(132.905), 0.0, 0.0, 1.0), delta=1e3)
    te = 0.3e-6
    _, _, cr, oh, nh = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fpn, rtol=1e-9,
                                       atol=1e-15, h0=1e-9, t0=0.0, t_end=te,
                                       hist_cap=100000, beta=beta)
    assert cr.status == 0
    b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, fpn, 1e-9, 1e-15, 1e-9, te,
                  SG_PREC_FP64, beta=beta)
    ts, hs, last = run_recording(b)
    ho = oh[oh[:, 3] == 1][:, 1]
    assert last[0]["steps"] == cr.steps
    np.testing.assert_allclose(hs[0][:2], ho[:2], rtol=1e-5)
    np.testing.assert_allclose(hs[0][2:20], ho[2:20], rtol=1e-6)


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_golden_cash_karp(ctx, prec):
    """Cash-Karp (the reference's RungaKutta4, bin/ode.cpp:220-345) with the error sum
    that the reference carries from one attempt to the next."""
    g = np.load(os.path.join(GOLD, "ck45_adaptive.npz"))
    fp = paul_fp(TRAPP)
    b = one_cloud(ctx, g["pos0"], g["vel0"], g["mass"], g["charge"], fp, 1e-9, 1e-15, 1e-9,
                  4e-7, prec, method=4)
    hist, last = attempt_history(b)
    gh = g["hist"]
    p, v = b.download()
    acc = hist[hist[:, 3] == 1]
    from simbuca_gb300.configs import Cloud
    c0 = Cloud(g["pos0"], g["vel0"], g["mass"], g["charge"])
    ep, ev = replay_error(c0, fp, acc[:, 0], acc[:, 1], p, v, method=4)
    if prec == SG_PREC_FP64:
        assert hist.shape == gh.shape
        assert np.array_equal(hist[:, 3], gh[:, 3])
        np.testing.assert_allclose(hist[:, :2], gh[:, :2], rtol=1e-8)
        np.testing.assert_allclose(hist[:, 2], gh[:, 2], rtol=1e-5, atol=1e-9)
        assert ep <= 1e-12 and ev <= 1e-12, (ep, ev)
    else:
        assert last["status"] == 0 and last["done"] == 1
        assert abs(len(acc) - int((gh[:, 3] == 1).sum())) <= 1
        assert ep <= 1e-9 and ev <= 1e-9, (ep, ev)
    # a Cash-Karp attempt takes six force evaluations
    assert last["force_evals"] == 6 * len(hist)


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_golden_gear(ctx, prec):
    """Gear predictor-corrector (bin/ode.cpp:347-424): 300 fixed steps of 2 ns against the
    reference's own step() run, one force evaluation per step."""
    g = np.load(os.path.join(GOLD, "gear_fixed.npz"))
    b = one_cloud(ctx, g["pos0"], g["vel0"], g["mass"], g["charge"], paul_fp(TRAPP), 1e-9,
                  1e-15, 2e-9, 1.0, prec, method=1)
    info, _ = b.run(max_attempts=300)
    s = info[0]
    assert s["steps"] == 300 and s["rejects"] == 0 and s["status"] == 0
    assert s["force_evals"] == 300 and s["h"] == 2e-9
    p, v = b.download()
    ep = np.abs(p - g["pos"]).max() / np.abs(g["pos"]).max()
    ev = np.abs(v - g["vel"]).max() / np.abs(g["vel"]).max()
    print(prec, ep, ev)
    tol = 1e-11 if prec == SG_PREC_FP64 else 1e-7
    assert ep <= tol and ev <= tol, (ep, ev)


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_gear_penning_vs_oracle(ctx, prec):
    """Gear with the Penning trap, a quadrupole drive and friction: velocity-dependent
    forces at the predicted state and stage time t + h."""
    w = configs.penning_1k(n=300, seed=7)
    c = w.clouds[0]
    fp = configs.penning_field(quad=(0.5, configs.nu_c(configs.M_CS), 0.0, 0.0, 1.0), delta=1e3)
    b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, fp, 1e-9, 1e-15, 1e-9, 1.0, prec,
                  method=1)
    b.run(max_attempts=200)
    p, v = b.download()
    pr, vr, cr, _, _ = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fp, rtol=1e-9,
                                       atol=1e-15, h0=1e-9, t0=0.0, t_end=1.0, adaptive=False,
                                       max_steps=200, method=1)
    ep = np.abs(p - pr).max() / np.abs(pr).max()
    ev = np.abs(v - vr).max() / np.abs(vr).max()
    print(prec, ep, ev)
    tol = 1e-11 if prec == SG_PREC_FP64 else 1e-7
    assert ep <= tol and ev <= tol, (ep, ev)
    assert b.info()[0]["t"] == pytest.approx(cr.t, rel=1e-14)


def test_method_mix_rejected(ctx):
    fp = paul_fp(TRAPP)
    ops = [configs.ode(1e-9, 1e-15, 1e-9, 1e-7, method=m) for m in (5, 4)]
    with pytest.raises(abi.SimGBError):
        Batch(ctx, [8, 8], [fp, fp], ops, SG_PREC_FP64)
    with pytest.raises(abi.SimGBError):
        Batch(ctx, [8], [fp], [configs.ode(1e-9, 1e-15, 1e-9, 1e-7, method=3)], SG_PREC_FP64)


def test_golden_fixed_step(ctx):
    g = np.load(os.path.join(GOLD, "dp45_fixed.npz"))
    for prec, tol in ((SG_PREC_FP64, 1e-12), (SG_PREC_FP32C, 1e-9)):
        b = one_cloud(ctx, g["pos0"], g["vel0"], g["mass"], g["charge"], paul_fp(TRAPP), 1e-7,
                      1e-7, 2e-9, 1.0, prec, adaptive=False)
        info, _ = b.run(max_attempts=40)
        assert info[0]["steps"] == 40 and info[0]["rejects"] == 0
        p, v = b.download()
        ep = np.abs(p - g["pos"]).max() / np.abs(g["pos"]).max()
        ev = np.abs(v - g["vel"]).max() / np.abs(g["vel"]).max()
        assert ep <= tol and ev <= tol, (prec, ep, ev)


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_penning_drive_vs_oracle(ctx, prec):
    """Penning trap + quadrupole + dipole drive + friction, stage times t + c_s h."""
    w = configs.penning_1k(n=300, seed=9)
    c = w.clouds[0]
    fp = configs.penning_field(quad=(0.5, configs.nu_c(132.905), 0.0, 0.0, 1.0),
                               dipole=(0.1, 1138.4, 0.0, 0.0, 1.0), delta=1e3)
    t_end = 0.5e-6
    _, _, cr, hist, nh = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fp, rtol=1e-9,
                                         atol=1e-15, h0=1e-9, t0=0.0, t_end=t_end,
                                         hist_cap=100000)
    assert cr.status == 0
    b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, fp, 1e-9, 1e-15, 1e-9, t_end, prec)
    ts, hs, last = run_recording(b)
    p, v = b.download()
    ep, ev = replay_error(c, fp, ts[0], hs[0], p, v)
    tol = 1e-12 if prec == SG_PREC_FP64 else 1e-9
    assert ep <= tol and ev <= tol, (ep, ev)
    # the oracle's own adaptive run: same step count and sizes (FP64); FP32c force noise
    # reaches the error norm through components whose scale is atol (first steps)
    ho = hist[hist[:, 3] == 1][:, 1]
    if prec == SG_PREC_FP64:
        assert last[0]["steps"] == cr.steps
        # The first step (h0 = 1 ns) has an embedded error near the rounding level of
        # the stage derivatives, so the second step size follows the last bits of the
        # Coulomb sums, which the device adds in another order: 1e-5 there, 1e-6 after.
        np.testing.assert_allclose(hs[0][:2], ho[:2], rtol=1e-5)
        np.testing.assert_allclose(hs[0][2:20], ho[2:20], rtol=1e-6)
    else:
        assert abs(last[0]["steps"] - cr.steps) <= max(2, cr.steps // 10)
        np.testing.assert_allclose(np.mean(hs[0][3:]), np.mean(ho[3:]), rtol=0.05)


def test_graph_and_direct_identical(ctx):
    w = configs.penning_1k(n=500, seed=3)
    c = w.clouds[0]
    fp = configs.penning_field()
    out = []
    for graph in (True, False):
        ctx.set_use_graph(graph)
        b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, fp, 1e-9, 1e-15, 1e-9, 1e-6,
                      SG_PREC_FP32C)
        b.run()
        out.append(b.download())
    ctx.set_use_graph(True)
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_step_takes_one_step(ctx):
    w = configs.penning_1k(n=200, seed=4)
    c = w.clouds[0]
    b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, configs.penning_field(), 1e-9, 1e-15,
                  1e-9, 1.0, SG_PREC_FP64)
    for k in range(1, 4):
        info, st = b.step()
        assert st == 0 and info[0]["steps"] == k


def test_underflow_status(ctx):
    g = np.load(os.path.join(GOLD, "force_edges.npz"))
    pos = g["pos2"].copy()
    pos[1] = pos[0] + 1e-13
    b = one_cloud(ctx, pos, g["vel2"], g["mass2"], g["charge2"], paul_fp(TRAPP), 1e-15, 1e-30,
                  1e-9, 1e-6, SG_PREC_FP64)
    info, st = b.run(raise_on_error=False)
    assert st == 0 and info[0]["status"] == abi.SG_H_UNDERFLOW and info[0]["done"] == 1
    # the mirror of step() raises what the reference throws
    from simbuca_gb300 import ode
    cl = ode.IonCloud(pos, g["vel2"], g["mass2"], g["charge2"])
    od = ode.OdeVars()
    od.Init_ode(5, 1e-9, True)
    od.rk_rtol, od.rk_atol = 1e-15, 1e-30
    od.forcev.coulomb_interaction = True
    od.forcev.trap_param.E_kick = 0.0
    with pytest.raises(RuntimeError, match="stepsize underflow created"):
        for _ in range(100000):
            ode.step(cl, od)


def test_underflow_reads_callers_first_ion_in_kd_order(ctx):
    """The underflow test |h| <= |pos[0][0]| eps (bin/ode.cpp:482) reads the caller's
    first ion also when the device holds the cloud in k-d order.  That ion sits at
    x = 0.1 m, so the k-d order puts it in the last leaf and the first leaf's first ion
    is ~1 mm out.  A nearly coincident pair keeps every attempt rejected at the 0.2
    floor, so h = 1e-9 0.2^k: the caller's ion gives underflow at k = 11, the first
    sorted ion would give it ~3 rejects later.  Both runs are bounded."""
    c = configs.penning_1k(n=512, seed=21).clouds[0]
    pos = c.pos.copy()
    pos[0] = [0.1, 2e-4, -1e-4]           # the caller's first ion: |x| = 0.1 m
    pos[2] = pos[1] + 1e-13               # a nearly coincident pair: err explodes
    fp = paul_fp(TRAPP)
    _, _, cr, oh, nh = oracle.dp45_run(pos, c.vel, c.mass, c.charge, fp, rtol=1e-15,
                                       atol=1e-30, h0=1e-9, t0=0.0, t_end=1e-6,
                                       max_steps=2, hist_cap=1000)
    assert cr.status == abi.SG_H_UNDERFLOW and cr.steps == 0
    k = int(np.ceil(np.log(1e-9 / (0.1 * np.finfo(float).eps)) / np.log(5.0)))
    assert cr.rejects == k == 11
    ctx.set_coulomb_variant(9)            # a k-d ordered launch shape
    try:
        b = one_cloud(ctx, pos, c.vel, c.mass, c.charge, fp, 1e-15, 1e-30, 1e-9, 1e-6,
                      SG_PREC_FP32C)
        info, st = b.run(max_attempts=100, raise_on_error=False)
    finally:
        ctx.set_coulomb_variant(-1)
    s = info[0]
    assert s["status"] == abi.SG_H_UNDERFLOW and s["done"] == 1
    assert s["rejects"] == cr.rejects and s["steps"] == 0, (s, cr.rejects)
    assert s["h"] == pytest.approx(cr.h, rel=1e-12)


def test_nonfinite_status(ctx):
    """Two ions at exactly the same place: the FP64 sum is 0/0 as in the reference, and
    the controller stops the cloud with SG_NONFINITE instead of looping."""
    g = np.load(os.path.join(GOLD, "force_edges.npz"))
    pos = g["pos3"].copy()
    pos[2] = pos[1]
    b = one_cloud(ctx, pos, g["vel3"], g["mass3"], g["charge3"], paul_fp(TRAPP), 1e-9, 1e-15,
                  1e-9, 1e-6, SG_PREC_FP64)
    info, st = b.run(max_attempts=5, raise_on_error=False)
    assert info[0]["status"] == abi.SG_NONFINITE


def test_too_many_rejects(ctx):
    w = configs.penning_1k(n=100, seed=5)
    c = w.clouds[0]
    # h0 far too large for rtol 1e-12: the first step needs several rejects
    b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, configs.penning_field(), 1e-12, 1e-18,
                  1e-6, 1.0, SG_PREC_FP64, max_rejects=2)
    info, st = b.run(max_attempts=10, raise_on_error=False)
    assert info[0]["status"] == abi.SG_TOO_MANY_REJECTS


def test_reference_mirror_step_and_force(ctx):
    """The IonCloud/_ode_vars/step()/force() mirror drives the same device path."""
    from simbuca_gb300 import ode
    g = np.load(os.path.join(GOLD, "dp45_adaptive.npz"))
    tag = "tight"
    rtol, atol, t_end, h0 = g[f"{tag}_cfg"]
    cl = ode.IonCloud(g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"], g[f"{tag}_charge"])
    od = ode.OdeVars()
    od.Init_ode(5, h0, True)
    od.rk_rtol, od.rk_atol = rtol, atol
    od.forcev.coulomb_interaction = True
    od.forcev.trap_param.E_kick = 0.0
    acc = ode.force(cl, od)
    ref = oracle.force(cl.pos2, cl.vel2, cl.mass, cl.charge, 0.0, paul_fp(TRAPP))
    np.testing.assert_allclose(acc, ref, rtol=1e-12)
    while cl.lifetime < t_end:
        ode.step(cl, od)
    np.testing.assert_allclose(cl.pos, g[f"{tag}_pos"], rtol=1e-9, atol=1e-15)


def test_kernel_timing_in_graph_and_direct(ctx):
    """Coulomb launches of the tiled path are timed with CUDA events both inside the
    attempt graph and with direct launches; both count 6 Coulomb sums per attempt."""
    w = configs.penning_1k(n=700, seed=8)
    c = w.clouds[0]
    ctx.set_fused(False)
    for graph in (True, False):
        ctx.set_use_graph(graph)
        b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, configs.penning_field(), 1e-9, 1e-15,
                      1e-9, 1.0, SG_PREC_FP32C)
        ctx.set_kernel_timing(True)
        i0 = b.info()[0]
        for _ in range(3):
            b.step()
        i1 = b.info()[0]
        kt = ctx.kernel_timing()
        ctx.set_kernel_timing(False)
        attempts = (i1["steps"] + i1["rejects"]) - (i0["steps"] + i0["rejects"])
        assert kt["coulomb_launches"] == 6 * attempts
        assert kt["coulomb_ms"] > 0 and kt["interactions"] == 6 * attempts * 700 * 699
    ctx.set_use_graph(True)
    ctx.set_fused(True)


@pytest.mark.parametrize("method,coul,stages", [(5, 6, 9), (4, 6, 9), (1, 1, 4)])
def test_kernel_timing_counts(ctx, method, coul, stages):
    """Kernel timing of graph-replayed attempts: one event pair per Coulomb launch and per
    O(N) launch (stages, control, commit) for each integrator, all with positive times."""
    w = configs.penning_1k(n=600, seed=31)
    c = w.clouds[0]
    fp = configs.penning_field(delta=1e3)
    ctx.set_fused(False)  # the tiled path's launches
    try:
        b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, fp, 1e-9, 1e-15, 2e-9, 1.0,
                      SG_PREC_FP32C, adaptive=(method != 1), method=method)
        b.attempts(2)
        ctx.set_kernel_timing(True)
        try:
            b.attempts(5)
            kt = ctx.kernel_timing()
            st = ctx.stage_timing()
        finally:
            ctx.set_kernel_timing(False)
    finally:
        ctx.set_fused(True)
    assert kt["coulomb_launches"] == 5 * coul and kt["coulomb_ms"] > 0
    assert kt["interactions"] == pytest.approx(5 * coul * 600 * 599)
    assert st["stage_launches"] == 5 * stages and st["stage_ms"] > 0
    assert b.info()[0]["status"] == 0


@pytest.mark.parametrize("variant", [9, 14])
@pytest.mark.parametrize("method", [4, 1])
def test_integrators_in_kd_order(ctx, variant, method):
    """Cash-Karp and Gear with the ions in k-d order (the launch shapes large clouds take;
    the far tiles' conditioning estimate comes from the first Coulomb sum of each
    attempt): the end state matches the oracle -- Cash-Karp replaying the accepted
    schedule, Gear over the same fixed steps."""
    w = configs.penning_1k(n=3000, seed=41)
    c = w.clouds[0]
    fp = configs.penning_field(quad=(0.5, configs.nu_c(configs.M_CS), 0.0, 0.0, 1.0), delta=1e3)
    ctx.set_coulomb_variant(variant)
    try:
        if method == 4:
            b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, fp, 1e-9, 1e-15, 1e-9, 0.15e-6,
                          SG_PREC_FP32C, method=4)
            ts, hs, last = run_recording(b)
            assert last[0]["status"] == 0 and last[0]["done"] == 1
        else:
            b = one_cloud(ctx, c.pos, c.vel, c.mass, c.charge, fp, 1e-9, 1e-15, 2e-9, 1.0,
                          SG_PREC_FP32C, adaptive=False, method=1)
            info, _ = b.run(max_attempts=60)
            assert info[0]["steps"] == 60 and info[0]["status"] == 0
        p, v = b.download()
    finally:
        ctx.set_coulomb_variant(-1)
    if method == 4:
        ep, ev = replay_error(c, fp, ts[0], hs[0], p, v, method=4)
        assert ep <= 1e-9 and ev <= 1e-9, (ep, ev)
    else:
        pr, vr, _, _, _ = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fp, rtol=1e-9,
                                          atol=1e-15, h0=2e-9, t0=0.0, t_end=1.0,
                                          adaptive=False, max_steps=60, method=1)
        ep = np.abs(p - pr).max() / np.abs(pr).max()
        ev = np.abs(v - vr).max() / np.abs(vr).max()
        assert ep <= 1e-7 and ev <= 1e-7, (ep, ev)
