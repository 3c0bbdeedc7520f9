"""Cloud observables over a long horizon: the 1,000-ion Penning cloud integrated for
10 us (about 1,100 adaptive Dormand-Prince steps, eight cyclotron periods) by the CPU
oracle (the reference's FP64 direct sum and RK45, restated bit for bit), by the device in
FP64 and by the device with the FP32-compensated Coulomb sum.  Individual trajectories
of an N-body cloud separate over such a horizon; the cloud's centroid, RMS size and
temperatures must agree."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from simbuca_gb300.api import Batch, Context

pytestmark = pytest.mark.gpu
T_END = 10e-6


@pytest.fixture(scope="module")
def runs():
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)
    w = configs.penning_1k()
    c, fp, op = w.clouds[0], w.fields[0], w.odes[0]
    p, v, ctrl, _, _ = oracle.dp45_run(c.pos, c.vel, c.mass, c.charge, fp, rtol=op.rtol,
                                       atol=op.atol, h0=op.h0, t0=0.0, t_end=T_END)
    out = {"oracle": (oracle.moments(p, v, c.mass), ctrl.t, ctrl.steps)}
    for prec in (SG_PREC_FP64, SG_PREC_FP32C):
        cx = Context(0)
        try:
            o = configs.ode(op.rtol, op.atol, op.h0, T_END)
            b = Batch(cx, [len(c.mass)], [fp], [o], prec)
            b.upload(c.pos, c.vel, c.mass, c.charge)
            info, _ = b.run()
            out[prec] = (b.moments()[0], info[0]["t"], info[0]["steps"])
        finally:
            cx.close()
    return out


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_observables_match_oracle(runs, prec):
    ref, t_ref, steps_ref = runs["oracle"]
    got, t, steps = runs[prec]
    print(prec, "steps", steps, "vs", steps_ref, "t", t, t_ref)
    print("  rms size rel", rel(got[3:6], ref[3:6]), "T_r/T_z rel", rel(got[9:11], ref[9:11]))
    # same end time to within a step, similar step counts
    assert abs(steps - steps_ref) <= max(3, steps_ref // 20)
    # RMS radius per axis and radial/axial temperatures (IonCloud::Temperature)
    tol = 1e-9 if prec == SG_PREC_FP64 else 1e-5
    assert np.all(rel(got[3:6], ref[3:6]) <= tol)
    assert np.all(rel(got[9:11], ref[9:11]) <= 10 * tol)
    # the centroid stays at the trap centre within a small fraction of the cloud size
    assert np.all(np.abs(got[0:3] - ref[0:3]) <= 1e-3 * ref[3:6])
