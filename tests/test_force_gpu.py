"""Complete force() replacement on the GPU (sg_force) against the reference's goldens
and the oracle: Paul trap + TOF + Coulomb, and the Penning, excitation and friction
terms."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import configs
from simbuca_gb300.abi import (SG_F_COULOMB, SG_F_DIPOLE, SG_F_FRICTION, SG_F_PENNING,
                               SG_F_QUAD, SG_PREC_FP32C, SG_PREC_FP64, FieldParams)
from helpers import TRAPP, paul_fp, rel_err_per_ion, summary

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)


def test_golden_paul_tof_coulomb(ctx):
    g = np.load(os.path.join(GOLD, "force_1k.npz"))
    fp = paul_fp(g["trapp"], coulomb=True, tof=True)
    a = ctx.force(g["pos"], g["vel"], g["mass"], g["charge"], float(g["t"]), fp, SG_PREC_FP64)
    e = rel_err_per_ion(a, g["f_all"])
    assert e.max() <= 1e-12, summary(e)
    a32 = ctx.force(g["pos"], g["vel"], g["mass"], g["charge"], float(g["t"]), fp, SG_PREC_FP32C)
    assert rel_err_per_ion(a32, g["f_all"]).max() <= 1e-6


def test_golden_mixed(ctx):
    g = np.load(os.path.join(GOLD, "force_mixed.npz"))
    fp = paul_fp(g["trapp"], coulomb=True, scale=float(g["coulomb_scale"]))
    a = ctx.force(g["pos"], g["vel"], g["mass"], g["charge"], 0.0, fp, SG_PREC_FP64)
    assert rel_err_per_ion(a, g["f"]).max() <= 1e-12


def test_golden_edges(ctx):
    g = np.load(os.path.join(GOLD, "force_edges.npz"))
    fp = paul_fp(TRAPP)
    for n in (1, 2, 3):
        a = ctx.force(g[f"pos{n}"], g[f"vel{n}"], g[f"mass{n}"], g[f"charge{n}"], 2e-8, fp)
        assert rel_err_per_ion(a, g[f"f{n}"]).max() <= 1e-12, n


def penning_all(t_on=0.0):
    fp = configs.penning_field(quad=(0.5, configs.nu_c(132.905), 0.3, t_on, 1.0),
                               dipole=(0.1, 1138.0, 0.2, t_on, 1.0), delta=1e3)
    return fp


@pytest.mark.parametrize("t", [0.0, 3.7e-7, 1.23e-5])
def test_penning_terms(ctx, t):
    w = configs.penning_1k(n=777)
    c = w.clouds[0]
    fp = penning_all()
    ref = oracle.force(c.pos, c.vel, c.mass, c.charge, t, fp)
    a = ctx.force(c.pos, c.vel, c.mass, c.charge, t, fp, SG_PREC_FP64)
    e = rel_err_per_ion(a, ref)
    assert e.max() <= 1e-12, summary(e)
    a32 = ctx.force(c.pos, c.vel, c.mass, c.charge, t, fp, SG_PREC_FP32C)
    assert rel_err_per_ion(a32, ref).max() <= 1e-6


def test_field_only_matches_formula(ctx):
    """Without Coulomb the Penning acceleration is exactly the formula of simgb.h."""
    w = configs.penning_1k(n=50)
    c = w.clouds[0]
    fp = configs.penning_field(coulomb=False)
    a = ctx.force(c.pos, c.vel, c.mass, c.charge, 0.0, fp)
    qm = c.charge * oracle.EL_CHARGE / c.mass
    kp = fp.V0 / (2 * fp.d0 ** 2)
    ex = kp * c.pos[:, 0] + fp.B * c.vel[:, 1]
    ey = kp * c.pos[:, 1] - fp.B * c.vel[:, 0]
    ez = -2 * kp * c.pos[:, 2]
    np.testing.assert_allclose(a, qm[:, None] * np.stack([ex, ey, ez], 1), rtol=1e-14)


def test_drive_window(ctx):
    """Excitations act only inside [t_on, t_off)."""
    w = configs.penning_1k(n=40)
    c = w.clouds[0]
    fp = configs.penning_field(coulomb=False, quad=(0.5, 8e5, 0.0, 1e-6, 2e-6))
    base = configs.penning_field(coulomb=False)
    for t, on in ((0.5e-6, False), (1.5e-6, True), (2.0e-6, False)):
        a = ctx.force(c.pos, c.vel, c.mass, c.charge, t, fp)
        b = ctx.force(c.pos, c.vel, c.mass, c.charge, t, base)
        assert (not np.array_equal(a, b)) == on
