"""Device-side observables (the recorder) against the oracle and the reference's own
text output: PrintCloud statistics per species, the kept ion states, the print rule of
move_particles (bin/ion_fly.cpp:103-108), ring overflow, and the text writer."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from simbuca_gb300.api import Batch
from helpers import TRAPP, paul_fp

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    oracle.build()


def two_species(n, seed):
    rng = np.random.default_rng(seed)
    species = (rng.random(n) < 0.4).astype(np.int32)
    mass = np.where(species == 0, 132.905, 86.909) * oracle.AMU
    pos = rng.normal(0.0, 5e-4, (n, 3))
    vel = rng.normal(0.0, 100.0, (n, 3))
    return pos, vel, mass, np.ones(n, np.int32), species


@pytest.mark.parametrize("n,prec", [(2000, SG_PREC_FP64), (10000, SG_PREC_FP32C)])
def test_record_now_vs_oracle(ctx, n, prec):
    """n = 10000 in FP32c runs the k-d ordered kernel: records come back in the
    caller's order."""
    pos, vel, mass, charge, species = two_species(n, n)
    fp = paul_fp(TRAPP)
    op = configs.ode(1e-9, 1e-15, 1e-9, 1e-6, t0=2.5e-7)
    b = Batch(ctx, [n], [fp], [op], prec)
    b.upload(pos, vel, mass, charge)
    b.set_recorder(0.0, stride=3, capacity=4, species=species, n_species=2)
    b.record_now()
    r = b.records(0)
    assert r["t"].tolist() == [2.5e-7]
    ref = oracle.cloud_stats(pos, vel, mass, species, 2)
    np.testing.assert_allclose(r["stats"][0], ref, rtol=1e-12, atol=1e-20)
    ions = r["ions"][0]
    assert np.array_equal(ions[:, :6], np.hstack([pos, vel])[::3])
    assert np.array_equal(ions[:, 7], species[::3])
    e = mass * (vel ** 2).sum(1) * 0.5 * 6.24150e18  # PrintParticle's energy
    np.testing.assert_allclose(ions[:, 6], e[::3], rtol=1e-13)
    assert b.records(0)["t"].size == 0  # consumed


def test_print_rule_and_states(ctx):
    """Records land after the steps where (t - t0) > interval * prints, with the state
    of that step: the same run stepped one step at a time gives the expected list."""
    g = np.load(os.path.join(GOLD, "dp45_adaptive.npz"))
    pos, vel, mass, charge = g["tight_pos0"], g["tight_vel0"], g["tight_mass"], g["tight_charge"]
    fp = paul_fp(TRAPP)
    interval = 3e-8
    a = Batch(ctx, [len(mass)], [fp], [configs.ode(1e-9, 1e-15, 1e-9, 4e-7)], SG_PREC_FP64)
    a.upload(pos, vel, mass, charge)
    a.set_recorder(interval, stride=1, capacity=64)
    a.run()
    rec = a.records(0)
    from simbuca_gb300.api import Context
    cx = Context(0)
    try:
        b = Batch(cx, [len(mass)], [fp], [configs.ode(1e-9, 1e-15, 1e-9, 4e-7)], SG_PREC_FP64)
        b.upload(pos, vel, mass, charge)
        exp_t, exp_y, n_print = [], [], 0
        while True:
            info, _ = b.step()
            t = info[0]["t"]
            if t > interval * n_print:
                n_print += 1
                p, v = b.download()
                exp_t.append(t)
                exp_y.append(np.hstack([p, v]))
            if info[0]["done"]:
                break
    finally:
        cx.close()
    assert rec["t"].tolist() == exp_t
    for got, exp in zip(rec["ions"], exp_y):
        assert np.array_equal(got[:, :6], exp)


def test_ring_full_holds_then_resumes(ctx):
    """A ring of 2 records with a print after every step: the cloud waits for the host
    and no record is lost."""
    pos, vel, mass, charge, species = two_species(256, 5)
    fp = paul_fp(TRAPP)
    b = Batch(ctx, [256], [fp], [configs.ode(1e-9, 1e-15, 1e-9, 2e-7)], SG_PREC_FP64)
    b.upload(pos, vel, mass, charge)
    b.set_recorder(1e-30, stride=64, capacity=2, species=species, n_species=2)
    b.attempts(12)  # no host sync inside: the cloud holds after two records
    info = b.info()[0]  # syncs and drains
    assert info["steps"] == 2
    info, _ = b.run()
    rec = b.records(0)
    assert len(rec["t"]) == info[0]["steps"]
    assert np.all(np.diff(rec["t"]) > 0)


def test_write_text_matches_reference(ctx, tmp_path):
    """The text writer against the reference's own PrintParticles/PrintCloud lines for
    the same state (tests/golden/make_golden.py): same fields, numbers to the printed
    6 digits."""
    g = np.load(os.path.join(GOLD, "print_state.npz"))
    n = len(g["mass"])
    names = [str(x) for x in g["names"]]
    op = configs.ode(1e-9, 1e-15, 1e-9, 1.0, t0=float(g["t"]))
    b = Batch(ctx, [n], [paul_fp(TRAPP)], [op], SG_PREC_FP64)
    b.upload(g["pos"], g["vel"], g["mass"], np.ones(n, np.int32))
    b.set_recorder(0.0, stride=1, capacity=2, species=g["species"], n_species=2)
    b.record_now()
    prefix = str(tmp_path / "run")
    b.write_text(0, prefix, names)

    def data(name):
        with open(prefix + name) as f:
            return [ln.rstrip("\n") for ln in f if not ln.startswith("#")]

    for name, ref in (("_pAll.txt", g["pall"]), ("_cloud0.txt", g["cloud0"]),
                      ("_cloud1.txt", g["cloud1"])):
        got = data(name)
        assert len(got) == len(ref), name
        nfix = 3 if name.startswith("_cloud") else 2
        for a, r in zip(got, ref):
            fa, fr = a.split(), str(r).split()
            assert fa[:nfix] == fr[:nfix] and len(fa) == len(fr)
            va = np.array([float(x) for x in fa[nfix:]])
            vr = np.array([float(x) for x in fr[nfix:]])
            np.testing.assert_allclose(va, vr, rtol=1.5e-6, atol=1e-300)


def test_restart_from_written_text(ctx, tmp_path):
    """Run, record, write the reference's text output, restart a new batch from its last
    print time (sg_particles_text_last) and from a binary state file: both restarts hold
    the recorded state (text: to the 7 printed digits; binary: exactly)."""
    from simbuca_gb300.api import load_state, read_particles_text, save_state
    n = 500
    pos, vel, mass, charge, species = two_species(n, 12)
    op = configs.ode(1e-9, 1e-15, 1e-9, 0.4e-6)
    b = Batch(ctx, [n], [configs.penning_field(delta=1e3)], [op], SG_PREC_FP64)
    b.upload(pos, vel, mass, charge)
    b.set_recorder(0.1e-6, stride=1, capacity=16, species=species, n_species=2)
    info, _ = b.run()
    b.record_now()
    p_end, v_end = b.download()
    prefix = str(tmp_path / "run")
    names = ["Cs133", "Rb87"]
    b.write_text(0, prefix, names)
    s = read_particles_text(prefix + "_pAll.txt", names,
                            [132.905 * oracle.AMU, 86.909 * oracle.AMU], [1, 1])
    assert len(s["ids"]) == n and np.array_equal(s["species"], species)
    assert s["t"] == pytest.approx(info[0]["t"], rel=1e-6)
    np.testing.assert_allclose(s["pos"], p_end, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(s["vel"], v_end, rtol=1e-6, atol=1e-9)
    f = str(tmp_path / "state.bin")
    save_state(f, p_end, v_end, mass, charge, t=info[0]["t"], species=species)
    st = load_state(f)
    b2 = Batch(ctx, [n], [configs.penning_field(delta=1e3)],
               [configs.ode(1e-9, 1e-15, 1e-9, 1.0, t0=st["t"])], SG_PREC_FP64)
    b2.upload(st["pos"], st["vel"], st["mass"], st["charge"])
    p2, v2 = b2.download()
    assert np.array_equal(p2, p_end) and np.array_equal(v2, v_end)
    assert b2.info()[0]["t"] == info[0]["t"]
