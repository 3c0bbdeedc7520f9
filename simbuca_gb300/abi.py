"""ctypes mirror of include/simgb.h and the loader of libsimgb.so.

The shared library is built in-tree by ``simbuca_gb300.build`` (nvcc, sm_103a).
Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsimgb.so")

# status codes
SG_OK, SG_BAD_ARG, SG_CUDA_ERR, SG_H_UNDERFLOW, SG_NONFINITE, SG_TIMEOUT, SG_NO_DEVICE, \
    SG_TOO_MANY_REJECTS, SG_NOT_READY, SG_TOO_LARGE, SG_IO_ERR = range(11)
SG_PREC_FP64, SG_PREC_FP32C = 0, 1

# field flags
SG_F_COULOMB = 1 << 0
SG_F_PAUL = 1 << 1
SG_F_TOF = 1 << 2
SG_F_PENNING = 1 << 3
SG_F_QUAD = 1 << 4
SG_F_DIPOLE = 1 << 5
SG_F_FRICTION = 1 << 6
SG_F_FROZEN_T = 1 << 7


class FieldParams(ctypes.Structure):
    """sg_field_params (include/simgb.h)."""
    _fields_ = [("flags", ctypes.c_uint32), ("pad0", ctypes.c_uint32),
                ("coulomb_scale", ctypes.c_double),
                ("Vrf", ctypes.c_double), ("Vdc", ctypes.c_double), ("kappa", ctypes.c_double),
                ("r0", ctypes.c_double), ("z0", ctypes.c_double), ("freq_rf", ctypes.c_double),
                ("E_kick", ctypes.c_double),
                ("B", ctypes.c_double), ("V0", ctypes.c_double), ("d0", ctypes.c_double),
                ("r_el", ctypes.c_double),
                ("Uq", ctypes.c_double), ("nu_q", ctypes.c_double), ("phi_q", ctypes.c_double),
                ("tq_on", ctypes.c_double), ("tq_off", ctypes.c_double),
                ("Ud", ctypes.c_double), ("nu_d", ctypes.c_double), ("phi_d", ctypes.c_double),
                ("td_on", ctypes.c_double), ("td_off", ctypes.c_double),
                ("delta", ctypes.c_double)]

    def copy(self) -> "FieldParams":
        c = FieldParams()
        ctypes.memmove(ctypes.byref(c), ctypes.byref(self), ctypes.sizeof(FieldParams))
        return c


class OdeParams(ctypes.Structure):
    """sg_ode_params (include/simgb.h)."""
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double), ("h0", ctypes.c_double),
                ("t0", ctypes.c_double), ("t_end", ctypes.c_double),
                ("adaptive", ctypes.c_int32), ("max_rejects", ctypes.c_int32),
                ("method", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("beta", ctypes.c_double)]


class StepInfo(ctypes.Structure):
    """sg_step_info (include/simgb.h)."""
    _fields_ = [("t", ctypes.c_double), ("h", ctypes.c_double), ("h_last", ctypes.c_double),
                ("err", ctypes.c_double), ("errold", ctypes.c_double),
                ("steps", ctypes.c_int64), ("rejects", ctypes.c_int64),
                ("force_evals", ctypes.c_int64), ("coulomb_evals", ctypes.c_int64),
                ("status", ctypes.c_int32), ("done", ctypes.c_int32),
                ("reject", ctypes.c_int32), ("pad", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class CheckInfo(ctypes.Structure):
    """sg_check_info (include/simgb.h)."""
    _fields_ = [("max_err", ctypes.c_double), ("last_err", ctypes.c_double),
                ("c_far", ctypes.c_double), ("kfar", ctypes.c_double),
                ("kfar_prior", ctypes.c_double), ("checks", ctypes.c_int64),
                ("probes", ctypes.c_int64), ("breaches", ctypes.c_int64),
                ("max_err_far", ctypes.c_double), ("max_err_near", ctypes.c_double),
                ("max_err_random", ctypes.c_double), ("worst_err", ctypes.c_double),
                ("worst_rf", ctypes.c_double), ("worst_rn", ctypes.c_double),
                ("worst_ion", ctypes.c_int32), ("worst_kind", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


SG_OP_NORMAL, SG_OP_TOF, SG_OP_TRAP_RAMP, SG_OP_FREE, SG_OP_DISSOCIATION = 0, 1, 2, 3, 4


class Operation(ctypes.Structure):
    """sg_operation (include/simgb.h)."""
    _fields_ = [("kind", ctypes.c_int32), ("print_after", ctypes.c_int32),
                ("duration", ctypes.c_double), ("print_time", ctypes.c_double),
                ("timestep", ctypes.c_double), ("new_vrf", ctypes.c_double),
                ("new_vdc", ctypes.c_double), ("e_kick", ctypes.c_double),
                ("reactant", ctypes.c_int32), ("product", ctypes.c_int32),
                ("fraction", ctypes.c_double), ("product_mass", ctypes.c_double)]


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

# every extern "C" symbol declared in include/simgb.h
EXPORTED = [
    "sg_create", "sg_destroy", "sg_status_string", "sg_last_cuda_error", "sg_sync",
    "sg_version", "sg_coulomb_accel", "sg_force", "sg_coulomb_accel_noalloc", "sg_set_wait_test",
    "sg_batch_set_force_check", "sg_batch_force_check", "sg_batch_set_far_threshold",
    "sg_set_fused", "sg_batch_fused", "sg_fused_timing",
    "sg_batch_create", "sg_batch_upload",
    "sg_batch_set_state", "sg_batch_download", "sg_batch_attempts", "sg_dp45_step",
    "sg_batch_run", "sg_batch_info", "sg_batch_set_field", "sg_batch_set_t_end",
    "sg_set_kernel_timing", "sg_kernel_timing", "sg_stage_timing", "sg_fixup_count",
    "sg_set_coulomb_variant",
    "sg_batch_variant", "sg_init_cloud", "sg_state_save", "sg_state_info", "sg_state_load",
    "sg_particles_text_last", "sg_batch_set_recorder", "sg_batch_record_now",
    "sg_batch_records", "sg_batch_read_records", "sg_batch_write_text",
    "sg_batch_set_operations", "sg_batch_operation_index",
    "sg_set_use_graph",
    "sg_timer_start",
    "sg_timer_stop", "sg_batch_moments", "sg_probe_peaks",
    "sg_mlp_param_count", "sg_mlp_forward", "sg_mlp_grad", "sg_mlp_train",
    "sg_batch_set_proposer", "sg_batch_set_controller_safety", "sg_batch_set_log",
    "sg_batch_read_log",
    "cunbody1_force", "cunbody1_force_begin", "cunbody1_force_end",
]

_lib = None


class SimGBError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = load().sg_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{where}: {msg} (status {status})")


def _declare(L):
    L.sg_create.argtypes = [ctypes.c_int, ctypes.POINTER(_vp)]
    L.sg_destroy.argtypes = [_vp]
    L.sg_status_string.argtypes = [ctypes.c_int]
    L.sg_status_string.restype = ctypes.c_char_p
    L.sg_last_cuda_error.argtypes = [_vp]
    L.sg_sync.argtypes = [_vp]
    L.sg_coulomb_accel.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp]
    L.sg_force.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _ip,
                           ctypes.c_double, ctypes.POINTER(FieldParams), _dp]
    L.sg_coulomb_accel_noalloc.argtypes = [ctypes.c_int, _vp, _vp, _vp, _vp, _vp]
    L.sg_set_wait_test.argtypes = [_vp, ctypes.c_int, ctypes.c_int]
    L.sg_batch_set_force_check.argtypes = [_vp, ctypes.c_int]
    L.sg_batch_force_check.argtypes = [_vp, ctypes.POINTER(CheckInfo)]
    L.sg_batch_set_far_threshold.argtypes = [_vp, ctypes.c_double]
    L.sg_set_fused.argtypes = [_vp, ctypes.c_int]
    L.sg_batch_fused.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
    L.sg_fused_timing.argtypes = [_vp, _dp, ctypes.POINTER(ctypes.c_int64)]
    L.sg_batch_create.argtypes = [_vp, ctypes.c_int, _ip, ctypes.POINTER(FieldParams),
                                  ctypes.POINTER(OdeParams), ctypes.c_int]
    L.sg_batch_upload.argtypes = [_vp, _dp, _dp, _dp, _ip]
    L.sg_batch_set_state.argtypes = [_vp, _dp, _dp]
    L.sg_batch_download.argtypes = [_vp, _dp, _dp]
    L.sg_batch_attempts.argtypes = [_vp, ctypes.c_int]
    L.sg_dp45_step.argtypes = [_vp, ctypes.POINTER(StepInfo)]
    L.sg_batch_run.argtypes = [_vp, ctypes.c_int64, ctypes.POINTER(StepInfo)]
    L.sg_batch_info.argtypes = [_vp, ctypes.POINTER(StepInfo)]
    L.sg_batch_set_field.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(FieldParams)]
    L.sg_batch_set_t_end.argtypes = [_vp, ctypes.c_int, ctypes.c_double]
    L.sg_set_kernel_timing.argtypes = [_vp, ctypes.c_int]
    L.sg_kernel_timing.argtypes = [_vp, _dp, ctypes.POINTER(ctypes.c_int64), _dp]
    L.sg_stage_timing.argtypes = [_vp, _dp, ctypes.POINTER(ctypes.c_int64)]
    L.sg_set_use_graph.argtypes = [_vp, ctypes.c_int]
    L.sg_fixup_count.argtypes = [_vp, ctypes.POINTER(ctypes.c_int64)]
    L.sg_set_coulomb_variant.argtypes = [_vp, ctypes.c_int]
    L.sg_batch_variant.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
    L.sg_batch_set_recorder.argtypes = [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, _ip,
                                        ctypes.c_int]
    L.sg_batch_record_now.argtypes = [_vp]
    L.sg_batch_records.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    L.sg_batch_read_records.argtypes = [_vp, ctypes.c_int, ctypes.c_int64, _dp,
                                        ctypes.POINTER(ctypes.c_int64)]
    L.sg_batch_write_text.argtypes = [_vp, ctypes.c_int, ctypes.c_char_p,
                                      ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]
    L.sg_batch_set_operations.argtypes = [_vp, ctypes.POINTER(Operation), ctypes.c_int]
    L.sg_batch_operation_index.argtypes = [_vp, ctypes.POINTER(ctypes.c_int)]
    L.sg_init_cloud.argtypes = [ctypes.c_int, _dp, ctypes.c_int, ctypes.c_uint32, _dp, _dp, _dp,
                                _dp, _dp]
    L.sg_state_save.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, _dp, _dp, _dp,
                                _ip, _ip]
    L.sg_state_info.argtypes = [ctypes.c_char_p, _ip, _dp]
    L.sg_state_load.argtypes = [ctypes.c_char_p, ctypes.c_int, _dp, _dp, _dp, _dp, _ip, _ip]
    L.sg_particles_text_last.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p), _dp,
                                         _ip, ctypes.c_int, ctypes.c_int, _ip, _dp, _ip, _dp,
                                         _dp, _dp, _ip, _ip]
    L.sg_timer_start.argtypes = [_vp]
    L.sg_timer_stop.argtypes = [_vp, _dp]
    L.sg_batch_moments.argtypes = [_vp, _dp]
    L.sg_probe_peaks.argtypes = [_vp, _dp, _dp, _dp]
    _fp = ctypes.POINTER(ctypes.c_float)
    L.sg_mlp_forward.argtypes = [_vp, ctypes.c_int, _fp, _fp, _fp]
    L.sg_mlp_grad.argtypes = [_vp, ctypes.c_int, _fp, _fp, _fp, _fp, _fp]
    L.sg_mlp_train.argtypes = [_vp, ctypes.c_int, _fp, _fp, ctypes.c_int, ctypes.c_int,
                               ctypes.c_float, ctypes.c_uint64, _fp, _fp]
    L.sg_batch_set_proposer.argtypes = [_vp, _fp, ctypes.c_double]
    L.sg_batch_set_controller_safety.argtypes = [_vp, ctypes.c_double]
    L.sg_batch_set_log.argtypes = [_vp, ctypes.c_int]
    L.sg_batch_read_log.argtypes = [_vp, ctypes.c_int, _fp, _dp, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_int)]
    for name in ("cunbody1_force", "cunbody1_force_begin", "cunbody1_force_end"):
        f = getattr(L, name)
        f.argtypes = [_dp, _dp, _dp, ctypes.c_double, _dp, ctypes.c_int, ctypes.c_int]
        f.restype = None


def load():
    """Load libsimgb.so from the package directory; raise if it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libsimgb.so not found at {LIB_PATH}: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != SG_OK:
        raise SimGBError(status, where)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)
