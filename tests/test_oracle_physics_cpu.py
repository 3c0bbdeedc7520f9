"""The oracle's Penning-trap terms have no reference code to be compared with (the
reference simulates Paul traps); they are pinned by physics instead: the three
eigenmotions of one ion return after their analytic periods, energy is conserved with
the electrostatic and magnetic terms alone, and buffer-gas friction decays velocities
as exp(-delta t).  CPU only."""
import math

import numpy as np
import pytest

import oracle
from simbuca_gb300 import configs
from simbuca_gb300.abi import SG_F_FRICTION, FieldParams

M = 132.905
MASS = np.array([M * oracle.AMU])
Q = np.array([1], np.int32)


@pytest.fixture(scope="module", autouse=True)
def built():
    oracle.build()


def fixed_run(pos, vel, fp, period, n_steps):
    p, v, c, _, _ = oracle.dp45_run(np.array([pos]), np.array([vel]), MASS, Q, fp, rtol=1e-9,
                                    atol=1e-15, h0=period / n_steps, t0=0.0, t_end=1.0,
                                    adaptive=False, max_steps=n_steps)
    assert c.steps == n_steps
    return p[0], v[0]


def test_axial_period():
    nc, npl, nm, nz = configs.penning_freqs(M)
    z0 = 1e-4
    p, v = fixed_run([0.0, 0.0, z0], [0.0, 0.0, 0.0], configs.penning_field(coulomb=False),
                     1.0 / nz, 4000)
    assert abs(p[2] - z0) / z0 < 1e-8
    assert abs(v[2]) / (2 * math.pi * nz * z0) < 1e-8
    assert np.abs(p[:2]).max() == 0.0 and np.abs(v[:2]).max() == 0.0


@pytest.mark.parametrize("mode", ["plus", "minus"])
def test_radial_eigenmodes(mode):
    """Circular orbit at the modified cyclotron or magnetron frequency: velocity
    (0, -omega r0, 0) at (r0, 0, 0) solves the radial equation exactly (the ion turns in
    the sense of its cyclotron motion)."""
    nc, npl, nm, nz = configs.penning_freqs(M)
    nu = npl if mode == "plus" else nm
    r0 = 2e-4
    w = 2 * math.pi * nu
    # the magnetron period spans ~700 cyclotron periods: steps of ~1/25 of the latter
    n = 2000 if mode == "plus" else 20000
    p, v = fixed_run([r0, 0.0, 0.0], [0.0, -w * r0, 0.0], configs.penning_field(coulomb=False),
                     1.0 / nu, n)
    tol = 1e-8 if mode == "plus" else 1e-6
    assert np.abs(p - [r0, 0.0, 0.0]).max() / r0 < tol, p
    assert np.abs(v - [0.0, -w * r0, 0.0]).max() / (w * r0) < tol, v


def test_energy_conserved_with_fields_only():
    fp = configs.penning_field(coulomb=False)
    kp = fp.V0 / (2 * fp.d0 ** 2)
    rng = np.random.default_rng(3)
    pos = rng.normal(0, 3e-4, 3)
    vel = rng.normal(0, 100.0, 3)

    def energy(p, v):
        return 0.5 * MASS[0] * (v ** 2).sum() + oracle.EL_CHARGE * kp * (p[2] ** 2 - 0.5 * (p[0] ** 2 + p[1] ** 2))

    p, v, c, _, _ = oracle.dp45_run(np.array([pos]), np.array([vel]), MASS, Q, fp, rtol=1e-11,
                                    atol=1e-18, h0=1e-10, t0=0.0, t_end=20e-6)
    e0, e1 = energy(pos, vel), energy(p[0], v[0])
    assert abs(e1 - e0) / abs(e0) < 1e-8, (e0, e1)


def test_friction_decay():
    fp = FieldParams()
    fp.flags = SG_F_FRICTION
    fp.delta = 1e3
    x0 = np.array([1e-4, -2e-4, 5e-5])
    v0 = np.array([120.0, -80.0, 30.0])
    t = 1e-3
    p, v = fixed_run(x0, v0, fp, t, 2000)
    np.testing.assert_allclose(v, v0 * math.exp(-fp.delta * t), rtol=1e-12)
    np.testing.assert_allclose(p, x0 + v0 * (1 - math.exp(-fp.delta * t)) / fp.delta, rtol=1e-12)
