"""The CPU oracle (C restatement) against golden vectors made by the compiled reference
(tests/golden/make_golden.py), and -- where the reference checkout exists -- against
the reference harness live.  CPU only."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300.abi import (SG_F_COULOMB, SG_F_FROZEN_T, SG_F_PAUL, SG_F_TOF, SG_OK,
                               SG_H_UNDERFLOW, FieldParams)

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def paul_fp(trapp, coulomb=True, tof=False, scale=1.0):
    fp = FieldParams()
    fp.flags = SG_F_PAUL | SG_F_FROZEN_T | (SG_F_COULOMB if coulomb else 0) | (SG_F_TOF if tof else 0)
    fp.coulomb_scale = scale
    fp.Vrf, fp.Vdc, fp.kappa, fp.r0, fp.z0, fp.freq_rf, fp.E_kick = [float(x) for x in trapp]
    return fp


@pytest.fixture(scope="module", autouse=True)
def built():
    oracle.build()
    oracle.set_threads(4)


def test_force_1k_bitexact():
    g = np.load(os.path.join(GOLD, "force_1k.npz"))
    fp = paul_fp(g["trapp"], coulomb=True, tof=True)
    f = oracle.force(g["pos"], g["vel"], g["mass"], g["charge"], float(g["t"]), fp)
    assert np.array_equal(f, g["f_all"])
    fpc = FieldParams()
    fpc.flags = SG_F_COULOMB
    fpc.coulomb_scale = 1.0
    fc = oracle.force(g["pos"], g["vel"], g["mass"], g["charge"], float(g["t"]), fpc)
    assert np.array_equal(fc, g["f_coulomb"])


def test_force_mixed_bitexact():
    g = np.load(os.path.join(GOLD, "force_mixed.npz"))
    fp = paul_fp(g["trapp"], coulomb=True, scale=float(g["coulomb_scale"]))
    f = oracle.force(g["pos"], g["vel"], g["mass"], g["charge"], float(g["t"]), fp)
    assert np.array_equal(f, g["f"])


def test_force_edges():
    g = np.load(os.path.join(GOLD, "force_edges.npz"))
    fp = paul_fp(np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0]))
    for n in (1, 2, 3):
        f = oracle.force(g[f"pos{n}"], g[f"vel{n}"], g[f"mass{n}"], g[f"charge{n}"], 2e-8, fp)
        assert np.array_equal(f, g[f"f{n}"]), n


def test_coulomb_kq_matches_reference_loop():
    g = np.load(os.path.join(GOLD, "force_1k.npz"))
    kq = 1.0 * oracle.KE * oracle.EL_CHARGE * g["charge"] * oracle.EL_CHARGE / g["mass"]
    a = oracle.coulomb_kq(g["pos"], g["charge"].astype(np.float64), kq)
    assert np.array_equal(a, g["f_coulomb"])
    rows = oracle.coulomb_kq_rows(g["pos"], g["charge"].astype(np.float64), kq, 100, 137)
    assert np.array_equal(rows, g["f_coulomb"][100:137])


@pytest.mark.parametrize("tag", ["tight", "default"])
def test_dp45_adaptive_history(tag):
    g = np.load(os.path.join(GOLD, "dp45_adaptive.npz"))
    rtol, atol, t_end, h0 = g[f"{tag}_cfg"]
    fp = paul_fp(np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0]))
    fp.flags &= ~SG_F_TOF
    p, v, c, hist, nh = oracle.dp45_run(g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"],
                                        g[f"{tag}_charge"], fp, rtol=rtol, atol=atol, h0=h0,
                                        t0=0.0, t_end=t_end, hist_cap=100000)
    assert c.status == SG_OK
    gh = g[f"{tag}_hist"]
    assert hist.shape == gh.shape
    # accept/reject sequence identical; every number of the history to rounding
    assert np.array_equal(hist[:, 3], gh[:, 3])
    np.testing.assert_allclose(hist, gh, rtol=1e-13, atol=0)
    np.testing.assert_allclose(p, g[f"{tag}_pos"], rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(v, g[f"{tag}_vel"], rtol=1e-12, atol=1e-12)
    ctrl = g[f"{tag}_ctrl"]
    assert c.t == pytest.approx(ctrl[0], rel=1e-13)
    assert c.h == pytest.approx(ctrl[1], rel=1e-12)
    assert c.steps == int(ctrl[5])


def test_ck45_adaptive_history():
    """Cash-Karp (bin/ode.cpp:220-345), including the error sum that the reference never
    resets between attempts."""
    g = np.load(os.path.join(GOLD, "ck45_adaptive.npz"))
    fp = paul_fp(np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0]))
    fp.flags &= ~SG_F_TOF
    p, v, c, hist, nh = oracle.dp45_run(g["pos0"], g["vel0"], g["mass"], g["charge"], fp,
                                        rtol=1e-9, atol=1e-15, h0=1e-9, t0=0.0, t_end=4e-7,
                                        hist_cap=100000, method=4)
    assert np.array_equal(hist, g["hist"])
    assert np.array_equal(p, g["pos"]) and np.array_equal(v, g["vel"])


def test_gear_fixed_steps():
    """GearMethod (bin/ode.cpp:347-424) through step(): 300 fixed steps, bit for bit."""
    g = np.load(os.path.join(GOLD, "gear_fixed.npz"))
    fp = paul_fp(np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0]))
    fp.flags &= ~SG_F_TOF
    p, v, c, hist, nh = oracle.dp45_run(g["pos0"], g["vel0"], g["mass"], g["charge"], fp,
                                        rtol=1e-9, atol=1e-15, h0=2e-9, t0=0.0, t_end=1.0,
                                        adaptive=False, max_steps=300, hist_cap=400, method=1)
    assert nh == 300 and c.steps == int(g["ctrl"][5])
    assert np.array_equal(p, g["pos"]) and np.array_equal(v, g["vel"])
    assert c.t == g["ctrl"][0]


def test_dp45_fixed_steps():
    g = np.load(os.path.join(GOLD, "dp45_fixed.npz"))
    fp = paul_fp(np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0]))
    fp.flags &= ~SG_F_TOF
    p, v, c, hist, nh = oracle.dp45_run(g["pos0"], g["vel0"], g["mass"], g["charge"], fp,
                                        rtol=1e-7, atol=1e-7, h0=2e-9, t0=0.0, t_end=1.0,
                                        adaptive=False, max_steps=40, hist_cap=100)
    assert nh == 40 and np.all(hist[:, 3] == 1)
    np.testing.assert_allclose(p, g["pos"], rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(v, g["vel"], rtol=1e-12, atol=1e-12)


def test_controller_table():
    """error_succes (bin/ode.cpp:426-457) on a table of errors."""
    c = oracle.OrcCtrl()
    c.h, c.errold, c.reject = 1.0, 1e-4, 0
    assert oracle.lib().orc_error_succes(0.0, c) == 1 and c.hnext == 10.0
    c.h, c.reject = 1.0, 0
    assert oracle.lib().orc_error_succes(1e-12, c) == 1 and c.hnext == 10.0  # clamped
    c.h, c.reject = 1.0, 0
    assert oracle.lib().orc_error_succes(0.5, c) == 1
    assert c.hnext == pytest.approx(0.9 * 0.5 ** -0.2)
    assert oracle.lib().orc_error_succes(2.0, c) == 0 and c.h == pytest.approx(0.9 * 2 ** -0.2)
    assert c.reject == 1
    h = c.h
    assert oracle.lib().orc_error_succes(0.01, c) == 1 and c.hnext == h  # no growth after reject
    c.h = 1.0
    assert oracle.lib().orc_error_succes(1e9, c) == 0 and c.h == pytest.approx(0.2)


@pytest.mark.parametrize("beta", [0.04, 0.08])
def test_pi_controller_table(beta):
    """The PI form of error_succes (bin/ode.cpp:431-439): alpha = 0.2 - 0.75 beta and the
    factor errold^beta on accepted steps; rejects use err^-alpha alone."""
    alpha = 0.2 - 0.75 * beta
    c = oracle.OrcCtrl()
    c.beta = beta
    c.h, c.errold, c.reject = 1.0, 0.3, 0
    assert oracle.lib().orc_error_succes(0.5, c) == 1
    assert c.hnext == pytest.approx(0.9 * 0.5 ** -alpha * 0.3 ** beta, rel=1e-15)
    assert c.errold == 0.5
    assert oracle.lib().orc_error_succes(2.0, c) == 0
    assert c.h == pytest.approx(0.9 * 2.0 ** -alpha, rel=1e-15) and c.reject == 1
    c.h, c.reject, c.errold = 1.0, 0, 1e-4
    assert oracle.lib().orc_error_succes(1e-3, c) == 1
    # 0.9 * 1e-3^-alpha * 1e-4^beta, clamped to [0.2, 10]
    assert c.hnext == pytest.approx(min(10.0, 0.9 * 1e-3 ** -alpha * 1e-4 ** beta), rel=1e-15)


def test_beta_zero_is_the_reference_controller():
    """beta = 0 multiplies by errold^0 = 1 exactly: the history against the reference's
    golden is the one of the test above."""
    g = np.load(os.path.join(GOLD, "dp45_adaptive.npz"))
    tag = "default"
    rtol, atol, t_end, h0 = g[f"{tag}_cfg"]
    fp = paul_fp(np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0]))
    fp.flags &= ~SG_F_TOF
    _, _, c, hist, _ = oracle.dp45_run(g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"],
                                       g[f"{tag}_charge"], fp, rtol=rtol, atol=atol, h0=h0,
                                       t0=0.0, t_end=t_end, hist_cap=100000, beta=0.0)
    gh = g[f"{tag}_hist"]
    assert np.array_equal(hist[:, 3], gh[:, 3])
    np.testing.assert_allclose(hist, gh, rtol=1e-13, atol=0)
    # PI control changes the sequence (and needs no more attempts here)
    _, _, c8, hist8, _ = oracle.dp45_run(g[f"{tag}_pos0"], g[f"{tag}_vel0"], g[f"{tag}_mass"],
                                         g[f"{tag}_charge"], fp, rtol=rtol, atol=atol, h0=h0,
                                         t0=0.0, t_end=t_end, hist_cap=100000, beta=0.08)
    assert c8.status == SG_OK and not np.array_equal(hist8[:, 1], gh[: len(hist8), 1])


def test_underflow_status():
    """A step size driven to zero gives the reference's underflow (ode.cpp:482-483)."""
    g = np.load(os.path.join(GOLD, "force_edges.npz"))
    fp = paul_fp(np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 0.0]), coulomb=True)
    pos = g["pos2"].copy()
    pos[1] = pos[0] + 1e-13  # nearly coincident pair: error norm explodes
    _, _, c, _, nh = oracle.dp45_run(pos, g["vel2"], g["mass2"], g["charge2"], fp, rtol=1e-15,
                                     atol=1e-30, h0=1e-9, t0=0.0, t_end=1e-6, hist_cap=10)
    assert c.status == SG_H_UNDERFLOW and nh == -SG_H_UNDERFLOW


@pytest.mark.skipif(not oracle.ref_available(), reason="reference harness not built here")
def test_live_reference_random():
    rng = np.random.default_rng(123)
    n = 257
    pos = rng.normal(0, 7e-4, (n, 3))
    vel = rng.normal(0, 50, (n, 3))
    mass = rng.uniform(40, 200, n) * oracle.AMU
    charge = rng.integers(1, 4, n).astype(np.int32)
    trapp = np.array([30.0, 2.0, 0.01, 0.005, 0.006, 1.1e6, 20.0])
    ref = oracle.ref_force(pos, vel, mass, charge, 3.3e-7, trap=1, tof=1, coulomb=1,
                           coulomb_scale=1.5, trapp=trapp)
    f = oracle.force(pos, vel, mass, charge, 3.3e-7, paul_fp(trapp, True, True, 1.5))
    assert np.array_equal(f, ref)


def _num(lines):
    return np.array([[float(x) for x in ln.split()[2:]] for ln in lines])


def test_cloud_stats_match_reference_text():
    """PrintCloud statistics (bin/ioncloud.cpp:148-183) of the oracle against the
    reference's own output lines (6 significant digits)."""
    g = np.load(os.path.join(GOLD, "print_state.npz"))
    st = oracle.cloud_stats(g["pos"], g["vel"], g["mass"], g["species"], 2)
    for s in range(2):
        ln = str(g[f"cloud{s}"][0]).split()
        assert int(ln[0]) == s and ln[1] == str(g["names"][s]) and int(ln[2]) == len(g["mass"])
        ref = np.array([float(x) for x in ln[3:]])
        mine = np.concatenate([[float(g["t"]) * 1e3], st[s, :6] * 1e3, st[s, 6:7]])
        np.testing.assert_allclose(mine, ref, rtol=1.5e-6)
