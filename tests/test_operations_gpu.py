"""The operation sequence on the device (sg_batch_set_operations) against the reference's
own operations::launch (bin/operation.cpp:33-124) run on the same cloud
(tests/golden/ops_sequence.npz): normal, trap ramp, TOF, free flight, normal with fixed
2 ns steps.  Also the print after each operation and a dissociation."""
import os

import numpy as np
import pytest

from simbuca_gb300 import abi, configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from simbuca_gb300.api import Batch
from helpers import TRAPP, paul_fp

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def golden_ops(g, print_after=0):
    ops = []
    for k in range(len(g["kinds"])):
        ops.append(dict(kind=int(g["kinds"][k]), duration=float(g["durations"][k]),
                        new_vrf=float(g["new_vrf"][k]), new_vdc=float(g["new_vdc"][k]),
                        e_kick=float(g["e_kick"][k]), print_after=print_after))
    return ops


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_sequence_matches_reference(ctx, prec):
    g = np.load(os.path.join(GOLD, "ops_sequence.npz"))
    n = len(g["mass"])
    fp = paul_fp(TRAPP)  # Paul trap and Coulomb; the operations switch trap and TOF
    b = Batch(ctx, [n], [fp], [configs.ode(1e-7, 1e-7, float(g["h0"]), 1.0, adaptive=False)],
              prec)
    b.upload(g["pos0"], g["vel0"], g["mass"], g["charge"])
    b.set_operations(golden_ops(g))
    info, _ = b.run()
    s = info[0]
    assert s["status"] == 0 and s["done"] == 1
    assert s["t"] == g["t"][0]  # same step count per operation, same rounding of t
    assert b.operation_index() == [len(g["kinds"])]
    p, v = b.download()
    ep = np.abs(p - g["pos"]).max() / np.abs(g["pos"]).max()
    ev = np.abs(v - g["vel"]).max() / np.abs(g["vel"]).max()
    print(prec, ep, ev)
    tol = 1e-11 if prec == SG_PREC_FP64 else 1e-7
    assert ep <= tol and ev <= tol, (ep, ev)


def test_print_after_each_operation(ctx):
    g = np.load(os.path.join(GOLD, "ops_sequence.npz"))
    n = len(g["mass"])
    b = Batch(ctx, [n], [paul_fp(TRAPP)],
              [configs.ode(1e-7, 1e-7, float(g["h0"]), 1.0, adaptive=False)], SG_PREC_FP64)
    b.upload(g["pos0"], g["vel0"], g["mass"], g["charge"])
    b.set_recorder(0.0, stride=8, capacity=16)
    b.set_operations(golden_ops(g, print_after=1))
    b.run()
    t = b.records(0)["t"]
    # one record when each operation ends: the first step at or past its end
    ends, t0, h = [], 0.0, float(g["h0"])
    cur = 0.0
    for d in g["durations"]:
        end = cur + d
        while cur < end:
            cur = cur + h
        ends.append(cur)
    assert t.tolist() == ends


def mt19937_uniform(seed, k):
    """The reference's MTRand doubles (32-bit output / 2^32) from numpy's MT19937 with
    the classic 32-bit seeding."""
    bg = np.random.MT19937()
    bg._legacy_seeding(seed)
    return bg.random_raw(k).astype(np.float64) / 4294967296.0


def test_dissociation(ctx):
    rng = np.random.default_rng(3)
    n = 500
    species = (rng.random(n) < 0.5).astype(np.int32)
    mass = np.where(species == 0, 132.905, 86.909) * 1.6605402e-27
    pos = rng.normal(0, 5e-4, (n, 3))
    vel = rng.normal(0, 100, (n, 3))
    b = Batch(ctx, [n], [paul_fp(TRAPP)], [configs.ode(1e-7, 1e-7, 2e-9, 1.0, adaptive=False)],
              SG_PREC_FP64)
    b.upload(pos, vel, mass, np.ones(n, np.int32))
    b.set_recorder(0.0, stride=1, capacity=8, species=species, n_species=3)
    pm = 40.0 * 1.6605402e-27
    b.set_operations([dict(kind=abi.SG_OP_NORMAL, duration=1e-8, print_after=1),
                      dict(kind=abi.SG_OP_DISSOCIATION, reactant=0, product=2, fraction=0.3,
                           product_mass=pm),
                      dict(kind=abi.SG_OP_NORMAL, duration=1e-8, print_after=1)])
    b.run()
    r = b.records(0)
    assert len(r["t"]) == 2
    before, after = r["ions"][0][:, 7], r["ions"][1][:, 7]
    assert np.array_equal(before, species)
    # expected: one draw per species-0 ion in order, seed 0
    u = mt19937_uniform(0, int((species == 0).sum()))
    exp = species.copy()
    idx = np.nonzero(species == 0)[0]
    exp[idx[u < 0.3]] = 2
    assert np.array_equal(after, exp)
    # the print mass changed, the dynamics mass did not: energies of product ions
    # use pm with the state's velocities
    v = r["ions"][1][:, 3:6]
    e = np.where(exp == 2, pm, mass) * (v ** 2).sum(1) * 0.5 * 6.24150e18
    np.testing.assert_allclose(r["ions"][1][:, 6], e, rtol=1e-13)
    assert r["stats"][1][2][7] == (exp == 2).sum()


def test_reference_mirror_operations():
    """The same sequence through the reference-shaped Python mirror (operation /
    operations with trap_param.newVrf/newVdc/E_kick as the INI parser leaves them)."""
    from simbuca_gb300 import ode
    g = np.load(os.path.join(GOLD, "ops_sequence.npz"))
    cloud = ode.IonCloud(g["pos0"], g["vel0"], g["mass"], g["charge"])
    odev = ode.OdeVars(precision=SG_PREC_FP64)
    odev.Init_ode(5, float(g["h0"]), False)
    fv = odev.forcev
    fv.coulomb_interaction, fv.coulomb_scale = True, 1.0
    tp = fv.trap_param
    tp.Vrf, tp.Vdc, tp.kappa, tp.r0, tp.z0, tp.freq_rf, tp.E_kick = [float(x) for x in TRAPP]
    tp.newVrf, tp.newVdc, tp.E_kick = 80.0, 2.0, 50.0
    ops = ode.Operations()
    for name, d in zip(["normal", "trap_ramp", "tof", "nop", "normal"], g["durations"]):
        ops.add(ode.Operation(name=name, time=float(d)))
    assert ops.total_time() == pytest.approx(1.7e-7)
    ops.launch(cloud, odev)
    assert cloud.lifetime == g["t"][0]
    ep = np.abs(cloud.pos - g["pos"]).max() / np.abs(g["pos"]).max()
    assert ep <= 1e-11, ep
