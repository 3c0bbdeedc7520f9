"""Shared helpers of the parity tests."""
import numpy as np

import oracle
from simbuca_gb300.abi import (SG_F_COULOMB, SG_F_FROZEN_T, SG_F_PAUL, SG_F_TOF, FieldParams)

TRAPP = np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0])


def paul_fp(trapp=TRAPP, coulomb=True, tof=False, scale=1.0, frozen=True):
    fp = FieldParams()
    fp.flags = SG_F_PAUL | (SG_F_FROZEN_T if frozen else 0) | (SG_F_COULOMB if coulomb else 0) \
        | (SG_F_TOF if tof else 0)
    fp.coulomb_scale = scale
    fp.Vrf, fp.Vdc, fp.kappa, fp.r0, fp.z0, fp.freq_rf, fp.E_kick = [float(x) for x in trapp]
    return fp


def kq_of(mass, charge, scale=1.0):
    """coulomb_scale*ke*e*q*e/m in the order of bin/force.cpp:153."""
    return scale * oracle.KE * oracle.EL_CHARGE * np.asarray(charge, np.float64) * \
        oracle.EL_CHARGE / np.asarray(mass, np.float64)


def rel_err_per_ion(a, ref):
    num = np.linalg.norm(a - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    return num / np.where(den > 0, den, 1.0)


def summary(e):
    return {"max": float(e.max()), "p99": float(np.percentile(e, 99)),
            "median": float(np.median(e))}


def run_recording(batch, max_calls=100000):
    """Advance a Batch one accepted step per cloud at a time (sg_dp45_step) until every
    cloud is done; returns per-cloud arrays of accepted (t_start, h) and the last info."""
    n = batch.n_clouds
    ts = [[] for _ in range(n)]
    hs = [[] for _ in range(n)]
    prev = batch.info()
    for _ in range(max_calls):
        if all(s["done"] for s in prev):
            break
        cur, st = batch.step(raise_on_error=False)
        for c in range(n):
            if cur[c]["steps"] > prev[c]["steps"]:
                ts[c].append(prev[c]["t"])
                hs[c].append(cur[c]["h_last"])
        prev = cur
        if st != 0:
            break
    return [np.array(x) for x in ts], [np.array(x) for x in hs], prev


def replay_error(cloud, fp, ts, hs, pos, vel, method=5):
    """Relative max difference of (pos, vel) against the oracle replaying (ts, hs)."""
    pr, vr = oracle.dp45_replay(cloud.pos, cloud.vel, cloud.mass, cloud.charge, fp, ts, hs,
                                method=method)
    ep = np.abs(pos - pr).max() / np.abs(pr).max()
    ev = np.abs(vel - vr).max() / np.abs(vr).max()
    return ep, ev
