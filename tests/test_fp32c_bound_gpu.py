"""The FP32-compensated form's per-ion bound (relative force error <= 1e-6 against the
FP64 direct sum of bin/force.cpp:147-174) beyond the two clouds its far fix-up threshold
was first calibrated on, and the in-run check that measures the error while a cloud
evolves.

Sampled rows (random ions, the ions nearest the centre -- where the net force is small
next to the far terms -- and both ions of the closest pairs) are compared with the
oracle's FP64 rows on a 262,144-ion uniform spheroid, a 1,048,576-ion Gaussian cloud,
the 65,536-ion Gaussian cloud at 1 K, and a 65,536-ion cloud 125 times denser than
that one."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import configs
from simbuca_gb300.abi import SG_PREC_FP32C
from simbuca_gb300.api import Batch
from helpers import kq_of, rel_err_per_ion, summary

pytestmark = pytest.mark.gpu
BOUND = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)


def sampled_rows(pos, n_random=40, n_central=16, n_close=16, seed=1):
    n = len(pos)
    rng = np.random.default_rng(seed)
    c = pos.mean(0)
    r2 = ((pos - c) ** 2).sum(1)
    # closest pairs: neighbours in a lexicographic order of a fine grid
    order = np.lexsort(np.floor((pos - pos.min(0)) / 2e-6).T)
    d = np.linalg.norm(np.diff(pos[order], axis=0), axis=1)
    close = np.argsort(d)[:n_close]
    rows = np.concatenate([rng.choice(n, n_random, replace=False), np.argsort(r2)[:n_central],
                           order[close], order[close + 1]])
    return np.unique(rows)


def check_rows(ctx, pos, q, mass, label):
    kq = kq_of(mass, q)
    a = ctx.coulomb_accel(pos, q, kq, SG_PREC_FP32C)
    assert np.isfinite(a).all()
    rows = sampled_rows(pos)
    ref = np.stack([oracle.coulomb_kq_rows(pos, q, kq, int(i), int(i) + 1)[0] for i in rows])
    e = rel_err_per_ion(a[rows], ref)
    print(label, summary(e))
    assert e.max() <= BOUND, (label, summary(e))


def test_spheroid_262k(ctx):
    c = configs.spheroid_cloud(configs.rng_for(12), 1 << 18, 2e-3, 4e-3, 1.0, configs.M_CS)
    check_rows(ctx, c.pos, c.charge.astype(np.float64), c.mass, "spheroid 262k")


def test_gaussian_1m(ctx):
    n = 1 << 20
    c = configs.gaussian_cloud(configs.rng_for(13), n, 1e-3, 300.0, np.full(n, configs.M_CS))
    check_rows(ctx, c.pos, c.charge.astype(np.float64), c.mass, "gaussian 1M")


def test_gaussian_65k_cold(ctx):
    n = 65536
    c = configs.gaussian_cloud(configs.rng_for(14), n, 1e-3, 1.0, np.full(n, configs.M_CS))
    check_rows(ctx, c.pos, c.charge.astype(np.float64), c.mass, "65k at 1 K")


def test_gaussian_65k_dense(ctx):
    n = 65536
    c = configs.gaussian_cloud(configs.rng_for(15), n, 0.2e-3, 1.0, np.full(n, configs.M_CS))
    check_rows(ctx, c.pos, c.charge.astype(np.float64), c.mass, "65k, sigma 0.2 mm")


def test_in_run_check_on_the_65k_workload(ctx):
    """The check runs inside the attempt loop at its default interval: on the 65,536-ion
    workload it finds no probe above the bound and keeps the density prior."""
    w = configs.penning_65k()
    c = w.clouds[0]
    b = Batch(ctx, [len(c.mass)], w.fields, w.odes, SG_PREC_FP32C)
    b.set_force_check(2)
    b.upload(c.pos, c.vel, c.mass, c.charge)
    for _ in range(12):
        b.step()
    rec = b.force_check()[0]
    print(rec)
    assert rec["checks"] >= 6 and rec["probes"] == 8 * rec["checks"]
    assert rec["breaches"] == 0 and 0.0 < rec["max_err"] <= BOUND
    assert rec["kfar"] <= rec["kfar_prior"]


def test_in_run_check_repairs_a_far_threshold_set_too_high(ctx):
    """With the far fix-up switched off (prior kfar = 1e6) the central ions of the
    1,048,576-ion spheroid carry the hi-only far error (~1.1e-6 before the fix-up
    existed).  The first check measures c on them and lowers kfar to 5e-7 / c; the
    attempts after it are checked within the bound."""
    w = configs.spheroid_1m()
    c = w.clouds[0]
    b = Batch(ctx, [len(c.mass)], w.fields, w.odes, SG_PREC_FP32C)
    b.set_far_threshold(1e6)
    b.set_force_check(1)
    b.upload(c.pos, c.vel, c.mass, c.charge)
    b.attempts(1)
    first = b.force_check()[0]
    print("first", first)
    assert first["checks"] == 1 and first["kfar_prior"] == pytest.approx(1e6)
    assert first["c_far"] > 2e-7                      # the hi-only far error is measured
    assert first["kfar"] == pytest.approx(max(5e-7 / first["c_far"], 0.05), rel=1e-5)
    b.attempts(2)
    rec = b.force_check()[0]
    print("after", rec)
    assert rec["checks"] == 3
    assert rec["last_err"] <= BOUND and rec["kfar"] <= first["kfar"] * (1 + 1e-6)
