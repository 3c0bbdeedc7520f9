"""Python host API over the libsimgb C ABI (include/simgb.h).

``Context`` owns a CUDA stream and device buffers; ``Batch`` is a set of resident
clouds integrated on the device.  Arrays are numpy, host memory, in the reference's
layouts (positions/velocities ``[n, 3]`` float64, masses in kg, integer charges).
There is no CPU fallback: every call goes through libsimgb.so.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import abi
from .abi import FieldParams, OdeParams, StepInfo, check, dptr, iptr


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


class Context:
    def __init__(self, device: int = 0):
        self._L = abi.load()
        h = ctypes.c_void_p()
        check(self._L.sg_create(int(device), ctypes.byref(h)), "sg_create")
        self._h = h
        self._batch_gen = 0  # a context holds one batch; older Batch objects go stale

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._L.sg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- stand-alone force calls ---------------------------------------------
    def coulomb_accel(self, pos, q, kq, precision=abi.SG_PREC_FP64):
        pos = _f64(pos)
        n = pos.shape[0]
        q = _f64(q)
        kq = _f64(kq)
        out = np.empty((n, 3))
        check(self._L.sg_coulomb_accel(self._h, int(precision), n, dptr(pos), dptr(q), dptr(kq),
                                       dptr(out)), "sg_coulomb_accel")
        return out

    def force(self, pos, vel, mass, charge, t, fp: FieldParams, precision=abi.SG_PREC_FP64):
        pos = _f64(pos)
        vel = _f64(vel)
        mass = _f64(mass)
        charge = np.ascontiguousarray(charge, dtype=np.int32)
        n = pos.shape[0]
        out = np.empty((n, 3))
        check(self._L.sg_force(self._h, int(precision), n, dptr(pos), dptr(vel), dptr(mass),
                               iptr(charge), float(t), ctypes.byref(fp), dptr(out)), "sg_force")
        return out

    def probe_peaks(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(self._L.sg_probe_peaks(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
              "sg_probe_peaks")
        return {"fp32_gflops": a.value, "fp32x2_gflops": b.value, "fp64_gflops": c.value}

    def timer_start(self):
        check(self._L.sg_timer_start(self._h), "sg_timer_start")

    def timer_stop(self) -> float:
        ms = ctypes.c_double()
        check(self._L.sg_timer_stop(self._h, ctypes.byref(ms)), "sg_timer_stop")
        return ms.value

    def sync(self):
        check(self._L.sg_sync(self._h), "sg_sync")

    def set_kernel_timing(self, on: bool):
        check(self._L.sg_set_kernel_timing(self._h, int(bool(on))), "sg_set_kernel_timing")

    def kernel_timing(self):
        ms, n, inter = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
        check(self._L.sg_kernel_timing(self._h, ctypes.byref(ms), ctypes.byref(n),
                                       ctypes.byref(inter)), "sg_kernel_timing")
        return {"coulomb_ms": ms.value, "coulomb_launches": n.value, "interactions": inter.value}

    def stage_timing(self):
        """Milliseconds and launches of the O(N) kernels timed since kernel timing was
        switched on (graph-replayed attempts)."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(self._L.sg_stage_timing(self._h, ctypes.byref(ms), ctypes.byref(n)),
              "sg_stage_timing")
        return {"stage_ms": ms.value, "stage_launches": n.value}

    def fixup_count(self) -> int:
        c = ctypes.c_int64()
        check(self._L.sg_fixup_count(self._h, ctypes.byref(c)), "sg_fixup_count")
        return c.value

    def set_coulomb_variant(self, v: int):
        check(self._L.sg_set_coulomb_variant(self._h, int(v)), "sg_set_coulomb_variant")

    # ---- step-size proposer MLP (BF16 weights, FP32 accumulation) ------------------
    def mlp_forward(self, X, w):
        X = np.ascontiguousarray(X, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        out = np.empty(len(X), np.float32)
        check(self._L.sg_mlp_forward(self._h, len(X), abi.fptr(X), abi.fptr(w), abi.fptr(out)),
              "sg_mlp_forward")
        return out

    def mlp_grad(self, X, Y, w):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        g = np.empty(self._L.sg_mlp_param_count(), np.float32)
        loss = np.zeros(1, np.float32)
        check(self._L.sg_mlp_grad(self._h, len(Y), abi.fptr(X), abi.fptr(Y), abi.fptr(w),
                                  abi.fptr(g), abi.fptr(loss)), "sg_mlp_grad")
        return float(loss[0]), g

    def mlp_train(self, X, Y, w0, iters=2000, batch=256, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        w = np.array(w0, np.float32, order="C")
        hist = np.zeros(max(iters, 1), np.float32)
        check(self._L.sg_mlp_train(self._h, len(Y), abi.fptr(X), abi.fptr(Y), int(iters),
                                   int(batch), float(lr), int(seed), abi.fptr(w), abi.fptr(hist)),
              "sg_mlp_train")
        return w, hist[:iters]

    def set_use_graph(self, on: bool):
        check(self._L.sg_set_use_graph(self._h, int(bool(on))), "sg_set_use_graph")

    def set_fused(self, mode):
        """Whole attempts of small clouds in one cluster launch: 1 (default, True) for
        clouds of up to 512 ions, 2 up to 2,048 ions, 0 (False) never."""
        check(self._L.sg_set_fused(self._h, int(mode)), "sg_set_fused")

    def fused_timing(self):
        """(ms, launches) of the fused launches timed while kernel timing is on."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        check(self._L.sg_fused_timing(self._h, ctypes.byref(ms), ctypes.byref(n)),
              "sg_fused_timing")
        return {"ms": ms.value, "launches": n.value}

    def set_wait_test(self, tile: int, limit_us: int = 1000):
        """Make the FP32c Coulomb kernels of the current batch give up a bounded wait at
        j-tile `tile` after limit_us (tile < 0: off); see sg_set_wait_test."""
        check(self._L.sg_set_wait_test(self._h, int(tile), int(limit_us)), "sg_set_wait_test")


class Batch:
    """Resident clouds advanced on the device by the Dormand-Prince loop.

    A Context holds one batch at a time: creating a new Batch on the same Context
    releases the previous one, whose methods then raise.  Use one Context per batch
    to keep several alive."""

    def __init__(self, ctx: Context, counts, fields, odes, precision=abi.SG_PREC_FP64):
        self.ctx = ctx
        self._L = ctx._L
        ctx._batch_gen += 1
        self._gen = ctx._batch_gen
        self.counts = np.ascontiguousarray(counts, dtype=np.int32)
        self.n_clouds = len(self.counts)
        self.n = int(self.counts.sum())
        self.precision = int(precision)
        fa = (FieldParams * self.n_clouds)(*[f.copy() for f in fields])
        oa = (OdeParams * self.n_clouds)(*odes)
        self._fields = fa
        check(self._L.sg_batch_create(ctx.handle, self.n_clouds, iptr(self.counts), fa, oa,
                                      self.precision), "sg_batch_create")
        self._info = (StepInfo * self.n_clouds)()

    def _live(self):
        if self.ctx._batch_gen != self._gen:
            raise RuntimeError("this Batch was replaced by a newer Batch on the same Context")

    def upload(self, pos, vel, mass, charge):
        self._live()
        pos, vel, mass = _f64(pos), _f64(vel), _f64(mass)
        charge = np.ascontiguousarray(charge, dtype=np.int32)
        assert pos.shape == (self.n, 3) and vel.shape == (self.n, 3)
        check(self._L.sg_batch_upload(self.ctx.handle, dptr(pos), dptr(vel), dptr(mass),
                                      iptr(charge)), "sg_batch_upload")

    def set_state(self, pos, vel):
        self._live()
        pos, vel = _f64(pos), _f64(vel)
        check(self._L.sg_batch_set_state(self.ctx.handle, dptr(pos), dptr(vel)),
              "sg_batch_set_state")

    def download(self, pos=None, vel=None):
        self._live()
        pos = np.empty((self.n, 3)) if pos is None else pos
        vel = np.empty((self.n, 3)) if vel is None else vel
        check(self._L.sg_batch_download(self.ctx.handle, dptr(pos), dptr(vel)),
              "sg_batch_download")
        return pos, vel

    def attempts(self, n: int):
        self._live()
        check(self._L.sg_batch_attempts(self.ctx.handle, int(n)), "sg_batch_attempts")

    def fused(self) -> int:
        """Cluster size of the fused small-cloud path this batch runs with (0: tiled)."""
        self._live()
        v = ctypes.c_int()
        check(self._L.sg_batch_fused(self.ctx.handle, ctypes.byref(v)), "sg_batch_fused")
        return v.value

    def set_force_check(self, every_attempts: int):
        """In-run check of the FP32c sums every `every_attempts` attempts (0: off)."""
        self._live()
        check(self._L.sg_batch_set_force_check(self.ctx.handle, int(every_attempts)),
              "sg_batch_set_force_check")

    def force_check(self):
        """Per cloud: the in-run check's record (sg_check_info as a dict)."""
        self._live()
        out = (abi.CheckInfo * self.n_clouds)()
        check(self._L.sg_batch_force_check(self.ctx.handle, out), "sg_batch_force_check")
        return [o.as_dict() for o in out]

    def set_far_threshold(self, kfar: float):
        """Prior of the far fix-up threshold of every cloud (0: from each cloud's density);
        applies from the next upload or set_state."""
        self._live()
        check(self._L.sg_batch_set_far_threshold(self.ctx.handle, float(kfar)),
              "sg_batch_set_far_threshold")

    def step(self, raise_on_error=True):
        self._live()
        st = self._L.sg_dp45_step(self.ctx.handle, self._info)
        if raise_on_error:
            check(st, "sg_dp45_step")
        return [s.as_dict() for s in self._info], st

    def run(self, max_attempts: int = 1 << 62, raise_on_error=True):
        self._live()
        st = self._L.sg_batch_run(self.ctx.handle, int(max_attempts), self._info)
        if raise_on_error:
            check(st, "sg_batch_run")
        return [s.as_dict() for s in self._info], st

    def variant(self) -> int:
        """FP32c Coulomb launch shape this batch was planned with."""
        self._live()
        v = ctypes.c_int(0)
        check(self._L.sg_batch_variant(self.ctx.handle, ctypes.byref(v)), "sg_batch_variant")
        return v.value

    def set_recorder(self, print_interval: float, stride: int = 1, capacity: int = 64,
                     species=None, n_species: int = 1):
        """Device-side observables every print_interval of simulated time (the
        reference's print rule); species per ion in the caller's order."""
        self._live()
        sp = None
        if species is not None:
            self._species = np.ascontiguousarray(species, np.int32)
            sp = iptr(self._species)
        check(self._L.sg_batch_set_recorder(self.ctx.handle, float(print_interval), int(stride),
                                            int(capacity), sp, int(n_species)),
              "sg_batch_set_recorder")
        self._n_species = int(n_species)

    def record_now(self):
        self._live()
        check(self._L.sg_batch_record_now(self.ctx.handle), "sg_batch_record_now")

    def records(self, cloud: int = 0):
        """Drained records of a cloud: dict(t [R], stats [R, species, 9],
        ions [R, kept, 8] = x y z vx vy vz, energy (eV), species)."""
        self._live()
        n, ln, kept = ctypes.c_int64(0), ctypes.c_int(0), ctypes.c_int(0)
        check(self._L.sg_batch_records(self.ctx.handle, int(cloud), ctypes.byref(n),
                                       ctypes.byref(ln), ctypes.byref(kept)), "sg_batch_records")
        out = np.empty((n.value, max(ln.value, 1)))
        got = ctypes.c_int64(0)
        check(self._L.sg_batch_read_records(self.ctx.handle, int(cloud), n.value, dptr(out),
                                            ctypes.byref(got)), "sg_batch_read_records")
        out = out[:got.value]
        S = getattr(self, "_n_species", 1)
        return {"t": out[:, 0].copy(),
                "stats": out[:, 1:1 + 9 * S].reshape(len(out), S, 9),
                "ions": out[:, 1 + 9 * S:].reshape(len(out), kept.value, 8)}

    def write_text(self, cloud: int, prefix: str, names):
        """The reference's _pAll.txt / _cloud<s>.txt lines of the drained records."""
        self._live()
        arr = (ctypes.c_char_p * len(names))(*[x.encode() for x in names])
        check(self._L.sg_batch_write_text(self.ctx.handle, int(cloud), prefix.encode(), arr,
                                          len(names)), "sg_batch_write_text")

    def set_operations(self, ops):
        """The operation sequence (list of abi.Operation or dicts of its fields), run on
        the device; replaces the batch's end time."""
        self._live()
        arr = (abi.Operation * max(len(ops), 1))()
        for k, o in enumerate(ops):
            if isinstance(o, dict):
                for key, v in o.items():
                    setattr(arr[k], key, v)
            else:
                arr[k] = o
        check(self._L.sg_batch_set_operations(self.ctx.handle, arr, len(ops)),
              "sg_batch_set_operations")

    def operation_index(self):
        self._live()
        out = (ctypes.c_int * self.n_clouds)()
        check(self._L.sg_batch_operation_index(self.ctx.handle, out), "sg_batch_operation_index")
        return list(out)

    def info(self):
        self._live()
        check(self._L.sg_batch_info(self.ctx.handle, self._info), "sg_batch_info")
        return [s.as_dict() for s in self._info]

    def moments(self):
        self._live()
        out = np.empty((self.n_clouds, 12))
        check(self._L.sg_batch_moments(self.ctx.handle, dptr(out)), "sg_batch_moments")
        return out

    def set_field(self, cloud: int, fp: FieldParams):
        self._live()
        check(self._L.sg_batch_set_field(self.ctx.handle, int(cloud), ctypes.byref(fp)),
              "sg_batch_set_field")

    def set_proposer(self, w=None, safety: float = 0.9):
        """Learned step-size proposer (weights w) or, with w None, the reference's
        controller."""
        self._live()
        if w is None:
            check(self._L.sg_batch_set_proposer(self.ctx.handle, None, float(safety)),
                  "sg_batch_set_proposer")
        else:
            w = np.ascontiguousarray(w, np.float32)
            self._w = w
            check(self._L.sg_batch_set_proposer(self.ctx.handle, abi.fptr(w), float(safety)),
                  "sg_batch_set_proposer")

    def set_controller_safety(self, safety: float):
        """The reference's controller with its accepted-step safety factor 0.9 replaced
        by `safety` (the ablation of the learned proposer)."""
        self._live()
        check(self._L.sg_batch_set_controller_safety(self.ctx.handle, float(safety)),
              "sg_batch_set_controller_safety")

    def set_log(self, capacity: int):
        self._live()
        check(self._L.sg_batch_set_log(self.ctx.handle, int(capacity)), "sg_batch_set_log")
        self._log_cap = int(capacity)

    def read_log(self, cloud: int = 0):
        """(features [m,16] float32, h_prev, h, err, t) of the logged accepted steps."""
        self._live()
        cap = getattr(self, "_log_cap", 0)
        feat = np.zeros((max(cap, 1), 16), np.float32)
        num = np.zeros((max(cap, 1), 4))
        cnt = ctypes.c_int()
        check(self._L.sg_batch_read_log(self.ctx.handle, int(cloud), abi.fptr(feat), dptr(num),
                                        cap, ctypes.byref(cnt)), "sg_batch_read_log")
        m = cnt.value
        return feat[:m], num[:m, 0], num[:m, 1], num[:m, 2], num[:m, 3]

    def set_t_end(self, cloud: int, t_end: float):
        self._live()
        check(self._L.sg_batch_set_t_end(self.ctx.handle, int(cloud), float(t_end)),
              "sg_batch_set_t_end")


def init_cloud(n: int, ev_max, seed: int, semiaxis, offset, mass):
    """InitCloud (bin/initialization.cpp:117-206) through sg_init_cloud: n ions in the
    ellipsoid offset + semiaxis * (unit ball), Maxwell-Boltzmann speeds around ev_max
    (eV; one value, or radial and axial), MT19937 stream seeded with `seed`.  mass in kg
    (scalar or per ion).  Returns (pos [n,3] m, vel [n,3] m/s)."""
    L = abi.load()
    ev = np.ascontiguousarray(np.atleast_1d(np.asarray(ev_max, np.float64)))
    semi = np.ascontiguousarray(semiaxis, np.float64)
    off = np.ascontiguousarray(offset, np.float64)
    m = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, np.float64), (n,)))
    pos = np.empty((n, 3))
    vel = np.empty((n, 3))
    check(L.sg_init_cloud(int(n), dptr(ev), len(ev), int(seed) & 0xFFFFFFFF, dptr(semi),
                          dptr(off), dptr(m), dptr(pos), dptr(vel)), "sg_init_cloud")
    return pos, vel


def save_state(path: str, pos, vel, mass, charge, t: float = 0.0, species=None):
    """Binary restart file through sg_state_save (layout in include/simgb.h)."""
    L = abi.load()
    pos, vel = _f64(pos), _f64(vel)
    mass = np.ascontiguousarray(mass, np.float64)
    charge = np.ascontiguousarray(charge, np.int32)
    sp = None if species is None else np.ascontiguousarray(species, np.int32)
    check(L.sg_state_save(os.fsencode(path), len(mass), float(t), dptr(pos), dptr(vel),
                          dptr(mass), iptr(charge), iptr(sp) if sp is not None else None),
          "sg_state_save")


def load_state(path: str) -> dict:
    """A state written by save_state: pos, vel (m, m/s, [n,3]), mass (kg), charge,
    species, t (s)."""
    L = abi.load()
    n, t = ctypes.c_int(0), ctypes.c_double(0.0)
    check(L.sg_state_info(os.fsencode(path), ctypes.byref(n), ctypes.byref(t)), "sg_state_info")
    k = n.value
    pos, vel = np.empty((k, 3)), np.empty((k, 3))
    mass = np.empty(k)
    charge, species = np.empty(k, np.int32), np.empty(k, np.int32)
    check(L.sg_state_load(os.fsencode(path), k, ctypes.byref(t), dptr(pos), dptr(vel),
                          dptr(mass), iptr(charge), iptr(species)), "sg_state_load")
    return {"pos": pos, "vel": vel, "mass": mass, "charge": charge, "species": species,
            "t": t.value}


def read_particles_text(path: str, names, masses, charges, cap: int | None = None) -> dict:
    """The ions of the last print time of the reference's particle output
    (PrintParticles: "ID name t[ms] x y z[mm] vx vy vz E[eV]"), in file order, through
    sg_particles_text_last.  names/masses (kg)/charges describe the species."""
    L = abi.load()
    enc = [str(x).encode() for x in names]
    arr = (ctypes.c_char_p * len(enc))(*enc)
    m = np.ascontiguousarray(masses, np.float64)
    q = np.ascontiguousarray(charges, np.int32)
    if cap is None:
        with open(path, "rb") as f:
            cap = sum(1 for _ in f)
    ids = np.empty(cap, np.int32)
    pos, vel = np.empty((cap, 3)), np.empty((cap, 3))
    mass, charge, species = np.empty(cap), np.empty(cap, np.int32), np.empty(cap, np.int32)
    n, t = ctypes.c_int(0), ctypes.c_double(0.0)
    check(L.sg_particles_text_last(os.fsencode(path), arr, dptr(m), iptr(q), len(enc), int(cap),
                                   ctypes.byref(n), ctypes.byref(t), iptr(ids), dptr(pos),
                                   dptr(vel), dptr(mass), iptr(charge), iptr(species)),
          "sg_particles_text_last")
    k = n.value
    return {"ids": ids[:k], "pos": pos[:k], "vel": vel[:k], "mass": mass[:k],
            "charge": charge[:k], "species": species[:k], "t": t.value}
