"""Host logic without a GPU: workload generators and trap frequencies."""
import math

import numpy as np
import pytest

from simbuca_gb300 import configs
from simbuca_gb300.abi import SG_F_COULOMB, SG_F_FRICTION, SG_F_PENNING, SG_F_QUAD
from simbuca_gb300.constants import AMU, KB


def test_penning_frequencies():
    nc, npl, nm, nz = configs.penning_freqs(132.905)
    assert nc == pytest.approx(808794.2, abs=1.0)
    assert npl == pytest.approx(807655.8, abs=1.0)
    assert nm == pytest.approx(1138.42, abs=0.05)
    assert nz == pytest.approx(42882.5, abs=0.5)
    assert npl + nm == pytest.approx(nc, rel=1e-12)
    assert npl ** 2 + nm ** 2 + nz ** 2 == pytest.approx(nc ** 2, rel=1e-12)  # invariance theorem
    assert configs.nu_c(132.905) - configs.nu_c(132.906) == pytest.approx(6.1, abs=0.05)


def test_small_workload():
    w = configs.penning_1k()
    c = w.clouds[0]
    assert c.pos.shape == (1000, 3) and c.vel.shape == (1000, 3)
    assert np.all(c.mass == 132.905 * AMU) and np.all(c.charge == 1)
    assert abs(c.pos.std() - 0.5e-3) < 0.03e-3
    sv = math.sqrt(KB * 300 / (132.905 * AMU))
    assert sv == pytest.approx(137.0, abs=0.5)
    assert abs(c.vel.std() - sv) < 0.05 * sv
    assert w.fields[0].flags == SG_F_PENNING | SG_F_COULOMB
    assert w.odes[0].rtol == 1e-9 and w.odes[0].atol == 1e-15
    # seeded: identical twice
    assert np.array_equal(configs.penning_1k().clouds[0].pos, c.pos)


def test_65k_workload():
    w = configs.penning_65k()
    c = w.clouds[0]
    assert c.pos.shape == (65536, 3)
    m = np.unique(c.mass / AMU)
    assert np.allclose(m, [132.905, 132.906])
    fp = w.fields[0]
    assert fp.flags & SG_F_QUAD and fp.flags & SG_F_FRICTION
    assert fp.nu_q == pytest.approx((configs.nu_c(132.905) + configs.nu_c(132.906)) / 2)
    assert fp.Uq == 0.5 and fp.delta == 1e3 and fp.tq_off == 200e-6
    assert w.interactions_per_force() == 65536 * 65535


def test_scan_counts():
    n = configs.scan_counts()
    assert len(n) == 512 and n.min() >= 64 and n.max() <= 8192
    # log-uniform: median near sqrt(64 * 8192) = 724
    assert 500 < np.median(n) < 1000
    w = configs.scan_512(n_clouds=8)
    d = [f.nu_q - configs.nu_c(132.905) for f in w.fields]
    assert d[0] == pytest.approx(-5.0) and d[-1] == pytest.approx(5.0)


def test_spheroid_inside():
    rng = configs.rng_for(2)
    c = configs.spheroid_cloud(rng, 5000, 2e-3, 4e-3, 1.0, 132.905)
    r = (c.pos[:, 0] / 2e-3) ** 2 + (c.pos[:, 1] / 2e-3) ** 2 + (c.pos[:, 2] / 4e-3) ** 2
    assert r.max() <= 1.0 and r.mean() == pytest.approx(0.6, abs=0.03)  # E[r^2] = 3/5 in a ball
