"""The batched frequency scan's observable: a cyclotron resonance.  One cloud per
detuning (the same 200-ion, 10 K cloud each time), driven by a dipole field at
nu_plus + Delta for 10 us, all in one batch; integrated with the FP32-compensated
Coulomb sum, with the FP64 form, and -- for three of the detunings -- by the CPU oracle
(the reference's FP64 direct sum and RK45).  The radial kinetic temperature after the
drive must trace the same resonance curve with the same peak in all three."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from simbuca_gb300.api import Batch, Context

pytestmark = pytest.mark.gpu
N_ION, T_DRIVE = 200, 10e-6
DETUNE = np.linspace(-300e3, 300e3, 13)


def scan_workload():
    cloud = configs.gaussian_cloud(configs.rng_for(77), N_ION, 0.1e-3, 10.0,
                                   np.full(N_ION, configs.M_CS))
    nu_plus = configs.penning_freqs(configs.M_CS)[1]
    clouds, fields, odes = [], [], []
    for d in DETUNE:
        clouds.append(cloud)
        fields.append(configs.penning_field(dipole=(0.1, nu_plus + d, 0.0, 0.0, T_DRIVE)))
        odes.append(configs.ode(1e-9, 1e-15, configs.H0, T_DRIVE))
    return clouds, fields, odes


@pytest.fixture(scope="module")
def curves():
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)
    clouds, fields, odes = scan_workload()
    pos = np.concatenate([c.pos for c in clouds])
    vel = np.concatenate([c.vel for c in clouds])
    mass = np.concatenate([c.mass for c in clouds])
    charge = np.concatenate([c.charge for c in clouds])
    out = {}
    for prec in (SG_PREC_FP64, SG_PREC_FP32C):
        cx = Context(0)
        try:
            b = Batch(cx, [N_ION] * len(clouds), fields, odes, prec)
            b.upload(pos, vel, mass, charge)
            info, _ = b.run()
            assert all(s["status"] == 0 and s["done"] for s in info)
            out[prec] = b.moments()[:, 9]  # T_radial per cloud
        finally:
            cx.close()
    ref = {}
    for k in (0, len(DETUNE) // 2, len(DETUNE) - 3):
        c = clouds[k]
        p, v, _, _, _ = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fields[k], rtol=1e-9,
                                        atol=1e-15, h0=configs.H0, t0=0.0, t_end=T_DRIVE)
        ref[k] = oracle.moments(p, v, c.mass)[9]
    out["oracle"] = ref
    return out


def test_resonance_curve(curves):
    t64, t32 = curves[SG_PREC_FP64], curves[SG_PREC_FP32C]
    print("T_r FP64 ", np.array2string(t64, precision=4))
    print("T_r FP32c", np.array2string(t32, precision=4))
    # a resonance: the drive heats the cloud most at nu_plus
    peak = int(np.argmax(t64))
    assert abs(DETUNE[peak]) <= 50e3
    assert t64[peak] > 2 * max(t64[0], t64[-1])
    # FP32c traces the same curve
    assert int(np.argmax(t32)) == peak
    np.testing.assert_allclose(t32, t64, rtol=1e-4)
    # and both agree with the reference's own arithmetic where the oracle ran
    for k, tr in curves["oracle"].items():
        assert t64[k] == pytest.approx(tr, rel=1e-8)
        assert t32[k] == pytest.approx(tr, rel=1e-4)
