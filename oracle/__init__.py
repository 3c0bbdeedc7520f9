"""CPU oracle for the Simbuca hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
may import this package; it is the checker, never the thing measured or shipped.

Two libraries are wrapped with ctypes:

* ``liboracle.so`` -- the C restatement (oracle.c), built with ``make`` in this
  directory on every machine;
* ``_ref/libsimbuca_ref.so`` -- the reference's own CPU path compiled from its
  sources plus ``ref_harness.cpp`` (``make ref``); only where the reference
  checkout exists.  Used to pin the restatement (golden vectors).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libsimbuca_ref.so")
ORC_SO = os.path.join(HERE, "liboracle.so")

# reference constants, bin/globals.h:4-16
PI = 3.14159265358979323
EL_CHARGE = 1.60217733e-19
AMU = 1.6605402e-27
KE = 8.987551787e9
KB = 1.3806504e-23

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference harness when asked)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


class OrcCtrl(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double),
                ("h", ctypes.c_double), ("hnext", ctypes.c_double),
                ("errold", ctypes.c_double), ("err", ctypes.c_double),
                ("t", ctypes.c_double), ("t_end", ctypes.c_double),
                ("reject", ctypes.c_int32), ("adaptive", ctypes.c_int32),
                ("max_rejects", ctypes.c_int32), ("status", ctypes.c_int32),
                ("steps", ctypes.c_int64), ("rejects", ctypes.c_int64),
                ("force_evals", ctypes.c_int64), ("attempts", ctypes.c_int64),
                ("beta", ctypes.c_double)]


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


_orc = None


def lib():
    global _orc
    if _orc is None:
        if not os.path.exists(ORC_SO):
            build()
        L = ctypes.CDLL(ORC_SO)
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_coulomb_kq.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_coulomb_kq_rows.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int,
                                          ctypes.c_int, _dp]
        L.orc_coulomb_sub.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_double, _dp]
        L.orc_field.argtypes = [ctypes.c_int, _dp, _dp, _dp, _ip, ctypes.c_double,
                                ctypes.c_void_p, _dp]
        L.orc_force.argtypes = L.orc_field.argtypes
        L.orc_dp45_run.argtypes = [ctypes.c_int, _dp, _dp, _dp, _ip, ctypes.c_void_p,
                                   ctypes.POINTER(OrcCtrl), ctypes.c_int64, _dp,
                                   ctypes.c_int64]
        L.orc_dp45_run.restype = ctypes.c_int64
        L.orc_rk_run.argtypes = [ctypes.c_int] + L.orc_dp45_run.argtypes
        L.orc_rk_run.restype = ctypes.c_int64
        L.orc_error_succes.argtypes = [ctypes.c_double, ctypes.POINTER(OrcCtrl)]
        L.orc_moments.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_dp45_replay.argtypes = [ctypes.c_int, _dp, _dp, _dp, _ip, ctypes.c_void_p, _dp,
                                      _dp, ctypes.c_int]
        L.orc_rk_replay.argtypes = [ctypes.c_int] + L.orc_dp45_replay.argtypes
        L.orc_cloud_stats.argtypes = [ctypes.c_int, _dp, _dp, _dp, _ip, ctypes.c_int, _dp]
        _orc = L
    return _orc


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def coulomb_kq(pos, q, kq):
    pos = np.ascontiguousarray(pos, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    kq = np.ascontiguousarray(kq, np.float64)
    out = np.zeros_like(pos)
    lib().orc_coulomb_kq(len(q), _d(pos), _d(q), _d(kq), _d(out))
    return out


def coulomb_kq_rows(pos, q, kq, i0, i1):
    pos = np.ascontiguousarray(pos, np.float64)
    q = np.ascontiguousarray(q, np.float64)
    kq = np.ascontiguousarray(kq, np.float64)
    out = np.zeros((i1 - i0, 3))
    lib().orc_coulomb_kq_rows(len(q), _d(pos), _d(q), _d(kq), int(i0), int(i1), _d(out))
    return out


def force(pos, vel, mass, charge, t, fp):
    """orc_force: field terms of fp (an sg_field_params ctypes struct) + Coulomb."""
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    out = np.zeros_like(pos)
    lib().orc_force(len(mass), _d(pos), _d(vel), _d(mass), _i(charge), float(t),
                    ctypes.byref(fp), _d(out))
    return out


def field(pos, vel, mass, charge, t, fp):
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    out = np.zeros_like(pos)
    lib().orc_field(len(mass), _d(pos), _d(vel), _d(mass), _i(charge), float(t),
                    ctypes.byref(fp), _d(out))
    return out


def dp45_run(pos, vel, mass, charge, fp, *, rtol, atol, h0, t0, t_end, adaptive=True,
             max_steps=1 << 62, hist_cap=0, max_rejects=0, method=5, beta=0.0):
    """Run the restated step loop (method 5 Dormand-Prince, 4 Cash-Karp); returns
    (pos, vel, ctrl, hist[attempts, 4], n_attempts)."""
    pos = np.array(pos, np.float64, order="C")
    vel = np.array(vel, np.float64, order="C")
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    c = OrcCtrl()
    c.rtol, c.atol, c.h, c.hnext, c.errold = rtol, atol, h0, h0, 1e-4
    c.t, c.t_end, c.adaptive, c.max_rejects = t0, t_end, int(adaptive), int(max_rejects)
    c.beta = float(beta)
    hist = np.zeros((max(hist_cap, 1), 4))
    nh = lib().orc_rk_run(int(method), len(mass), _d(pos), _d(vel), _d(mass), _i(charge),
                          ctypes.byref(fp), ctypes.byref(c), int(max_steps), _d(hist),
                          int(hist_cap))
    n_rec = min(max(nh, 0), hist_cap)
    return pos, vel, c, hist[:n_rec], nh


def dp45_replay(pos, vel, mass, charge, fp, ts, hs, method=5):
    """Fixed steps with the schedule (ts[k], hs[k]); returns (pos, vel).
    method 5 = Dormand-Prince, 4 = Cash-Karp."""
    pos = np.array(pos, np.float64, order="C")
    vel = np.array(vel, np.float64, order="C")
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    ts = np.ascontiguousarray(ts, np.float64)
    hs = np.ascontiguousarray(hs, np.float64)
    st = lib().orc_rk_replay(int(method), len(mass), _d(pos), _d(vel), _d(mass), _i(charge),
                             ctypes.byref(fp), _d(ts), _d(hs), len(ts))
    assert st == 0
    return pos, vel


def moments(pos, vel, mass):
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    out = np.zeros(12)
    lib().orc_moments(len(mass), _d(pos), _d(vel), _d(mass), _d(out))
    return out


# ---------------------------------------------------------------------------
# the compiled reference (only where its sources exist)
# ---------------------------------------------------------------------------
_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_SO)
        L.ref_force.argtypes = [ctypes.c_int, _dp, _dp, _dp, _ip, ctypes.c_double,
                                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                _dp, _dp]
        L.ref_dp45_run.argtypes = [ctypes.c_int, _dp, _dp, _dp, _ip, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_longlong, ctypes.c_int, _dp, ctypes.c_longlong,
                                   _dp, ctypes.c_int]
        L.ref_dp45_run.restype = ctypes.c_longlong
        L.ref_print.argtypes = [ctypes.c_int, _dp, _dp, _dp, _ip, _ip,
                                ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.c_double,
                                ctypes.c_char_p, ctypes.c_longlong]
        L.ref_print.restype = ctypes.c_longlong
        _ref = L
    return _ref


def ref_force(pos, vel, mass, charge, t, *, trap, tof, coulomb, coulomb_scale, trapp):
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    trapp = np.ascontiguousarray(trapp, np.float64)
    out = np.zeros_like(pos)
    ref_lib().ref_force(len(mass), _d(pos), _d(vel), _d(mass), _i(charge), float(t),
                        int(trap), int(tof), int(coulomb), float(coulomb_scale), _d(trapp),
                        _d(out))
    return out


def ref_dp45_run(pos, vel, mass, charge, *, trap, tof, coulomb, coulomb_scale, trapp, t0,
                 t_end, h0, adaptive, rtol, atol, max_steps, mode, hist_cap=0, method=5):
    pos = np.array(pos, np.float64, order="C")
    vel = np.array(vel, np.float64, order="C")
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    trapp = np.ascontiguousarray(trapp, np.float64)
    hist = np.zeros((max(hist_cap, 1), 4))
    ctrl = np.zeros(7)
    nh = ref_lib().ref_dp45_run(len(mass), _d(pos), _d(vel), _d(mass), _i(charge), int(trap),
                                int(tof), int(coulomb), float(coulomb_scale), _d(trapp),
                                float(t0), float(t_end), float(h0), int(adaptive), float(rtol),
                                float(atol), int(max_steps), int(mode), _d(hist), int(hist_cap),
                                _d(ctrl), int(method))
    return pos, vel, ctrl, hist[:min(max(nh, 0), hist_cap)], nh


def cloud_stats(pos, vel, mass, species, n_species):
    """PrintCloud statistics per species: [n_species, 9] (x0 y0 z0 x1 y1 z1 m, energy eV,
    ions of the species, ions of the cloud)."""
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    species = np.ascontiguousarray(species, np.int32)
    out = np.zeros((n_species, 9))
    lib().orc_cloud_stats(len(mass), _d(pos), _d(vel), _d(mass), _i(species), int(n_species),
                          _d(out))
    return out


def ref_print(pos, vel, mass, charge, species, names, t):
    """The reference's PrintParticles + PrintCloud text for a state: {file suffix: text}."""
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    species = np.ascontiguousarray(species, np.int32)
    arr = (ctypes.c_char_p * len(names))(*[x.encode() for x in names])
    cap = 200 * len(mass) + 4096
    buf = ctypes.create_string_buffer(cap)
    ln = ref_lib().ref_print(len(mass), _d(pos), _d(vel), _d(mass), _i(charge), _i(species), arr,
                             len(names), float(t), buf, cap)
    text = buf.raw[:ln].decode()
    out, cur = {}, None
    for line in text.splitlines(keepends=True):
        if line.startswith("@@"):
            cur = line[2:].strip()
            out[cur] = ""
        elif cur is not None:
            out[cur] += line
    return out
