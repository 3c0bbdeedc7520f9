"""Host-side mirror of the reference's integration interface, backed by libsimgb.

Names and argument meaning follow the reference:

* ``IonCloud``  -- bin/ioncloud.h:17-71 (pos, vel, pos2, vel2 ``[n][3]``, mass in kg,
  integer charge, lifetime, nrparticles);
* ``ForceVars`` -- _force_vars, bin/ode.h:42-56 (derivs, coulomb_scale,
  coulomb_interaction, trap, tof, trap_param);
* ``OdeVars``   -- _ode_vars, bin/ode.h:58-133 (h, hnext, rk_rtol, rk_atol, errold,
  reject, EPS, Init_ode);
* ``force(cloud, odev)`` -- bin/force.h:6: writes accelerations of pos2/vel2 at the
  cloud lifetime into ``odev.forcev.derivs``;
* ``step(cloud, odev)``  -- bin/ode.h:135: one accepted Dormand-Prince step; raises
  ``RuntimeError("stepsize underflow created")`` where the reference throws
  (bin/ode.cpp:482-483).

Besides the reference's Paul trap (``TrapParam``), ``ForceVars.extra`` may carry an
``FieldParams`` with Penning-trap, excitation and friction terms.  With
``frozen_time`` (the default, as in bin/force.cpp:36) every stage sees the step-start
time; otherwise stage s sees t + c_s h.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import abi
from .abi import FieldParams, OdeParams
from .api import Batch, Context


@dataclasses.dataclass
class TrapParam:
    """_trap_param, bin/trapparameters.h:6-27 (defaults bin/trapparameters.cpp:2-10)."""
    Vrf: float = 50.0
    Vdc: float = 5.0
    kappa: float = 0.001
    r0: float = 0.04
    z0: float = 0.04
    freq_rf: float = 50e5
    trap_type: int = 0
    E_kick: float = 0.0
    newVrf: float = 0.0
    newVdc: float = 0.0


@dataclasses.dataclass
class ForceVars:
    """_force_vars, bin/ode.h:42-56 (defaults bin/ode.cpp:646-653)."""
    coulomb_scale: float = 1.0
    coulomb_interaction: bool = False
    trap: bool = True
    tof: bool = False
    trap_ramp: bool = False
    trap_param: TrapParam = dataclasses.field(default_factory=TrapParam)
    extra: FieldParams | None = None      # Penning / excitation / friction terms
    frozen_time: bool = True
    derivs: np.ndarray | None = None

    def field_params(self) -> FieldParams:
        fp = self.extra.copy() if self.extra is not None else FieldParams()
        fp.flags &= ~(abi.SG_F_PAUL | abi.SG_F_TOF | abi.SG_F_COULOMB | abi.SG_F_FROZEN_T)
        tp = self.trap_param
        fp.Vrf, fp.Vdc, fp.kappa, fp.r0, fp.z0 = tp.Vrf, tp.Vdc, tp.kappa, tp.r0, tp.z0
        fp.freq_rf, fp.E_kick = tp.freq_rf, tp.E_kick
        fp.coulomb_scale = self.coulomb_scale
        if self.trap:
            fp.flags |= abi.SG_F_PAUL
        if self.tof:
            fp.flags |= abi.SG_F_TOF
        if self.coulomb_interaction:
            fp.flags |= abi.SG_F_COULOMB
        if self.frozen_time:
            fp.flags |= abi.SG_F_FROZEN_T
        return fp


class IonCloud:
    """IonCloud, bin/ioncloud.h:17-71 (the state arrays only)."""

    def __init__(self, pos=None, vel=None, mass=None, charge=None, lifetime: float = 0.0):
        self.pos = np.zeros((0, 3)) if pos is None else np.array(pos, np.float64, order="C")
        self.vel = np.zeros_like(self.pos) if vel is None else np.array(vel, np.float64, order="C")
        self.pos2 = self.pos.copy()
        self.vel2 = self.vel.copy()
        n = len(self.pos)
        self.mass = np.zeros(n) if mass is None else np.array(mass, np.float64)
        self.charge = np.ones(n, np.int32) if charge is None else np.array(charge, np.int32)
        self.lifetime = float(lifetime)

    @property
    def nrparticles(self) -> int:
        return len(self.pos)

    def AddParticle(self, x, y, z, vx, vy, vz, mass_kg, charge=1):
        self.pos = np.vstack([self.pos, [[x, y, z]]])
        self.vel = np.vstack([self.vel, [[vx, vy, vz]]])
        self.pos2, self.vel2 = self.pos.copy(), self.vel.copy()
        self.mass = np.append(self.mass, mass_kg)
        self.charge = np.append(self.charge, np.int32(charge)).astype(np.int32)

    def Temperature(self):
        """(T_radial, T_axial) as bin/ioncloud.cpp:316-335."""
        from .constants import KB
        n = self.nrparticles
        if n == 0:
            return (0.0, 0.0)
        er = float(np.sum(self.mass * (self.vel[:, 0] ** 2 + self.vel[:, 1] ** 2))) * (0.5 / n)
        ez = float(np.sum(self.mass * self.vel[:, 2] ** 2)) * (0.5 / n)
        return (er * 2.0 / (3.0 * KB), ez * 2.0 / (3.0 * KB))


class OdeVars:
    """_ode_vars, bin/ode.h:58-133: integrator settings and controller state."""

    def __init__(self, precision=abi.SG_PREC_FP64, device: int = 0):
        self.h = 1e-9            # httry default (bin/ode.cpp:509)
        self.hnext = 1e-9
        self.rk_atol = 1e-7      # bin/ode.cpp:515-516
        self.rk_rtol = 1e-7
        self.errold = 1.0e-4
        self.beta = 0.0          # PI term of error_succes (bin/ode.cpp:431); 0 as built
        self.reject = False
        self.EPS = float(np.finfo(np.float64).eps)
        self.change_stepsize = True
        self.DP5 = True
        self.method = 5          # Init_ode order
        self.forcev = ForceVars()
        self.precision = precision
        self.device = device
        self.countstep = 0
        self._ctx: Context | None = None
        self._batch: Batch | None = None
        self._batch_key = None

    def Init_ode(self, ode_order: int, timestep: float, adaptive_stepsize: bool):
        """bin/ode.cpp:539-587: order 5 Dormand-Prince, 4 Cash-Karp (the reference's
        RungaKutta4), 1 Gear; the reference falls back to order 4 for any other."""
        self.method = ode_order if ode_order in (1, 4, 5) else 4
        self.errold = 1.0e-4
        self.reject = False
        self.h = self.hnext = float(timestep)
        self.countstep = 0
        self.change_stepsize = bool(adaptive_stepsize)
        self._batch = None

    def context(self) -> Context:
        if self._ctx is None:
            self._ctx = Context(self.device)
        return self._ctx


def force(cloud: IonCloud, odev: OdeVars) -> np.ndarray:
    """force(), bin/force.cpp:34-178: accelerations of (pos2, vel2) at cloud.lifetime."""
    fv = odev.forcev
    acc = odev.context().force(cloud.pos2, cloud.vel2, cloud.mass, cloud.charge,
                               cloud.lifetime, fv.field_params(), odev.precision)
    fv.derivs = acc
    return acc


def step(cloud: IonCloud, odev: OdeVars) -> None:
    """step(), bin/ode.cpp:459-494: one accepted step of the whole cloud on the device."""
    fp = odev.forcev.field_params()
    key = (cloud.nrparticles, odev.precision, bytes(fp), odev.rk_rtol, odev.rk_atol,
           odev.change_stepsize, odev.method, odev.beta)
    if odev._batch is None or odev._batch_key != key:
        op = OdeParams()
        op.rtol, op.atol, op.h0 = odev.rk_rtol, odev.rk_atol, odev.h
        op.t0, op.t_end = cloud.lifetime, float("inf")
        op.adaptive, op.max_rejects = int(odev.change_stepsize), 0
        op.method = odev.method
        op.beta = odev.beta
        odev._batch = Batch(odev.context(), [cloud.nrparticles], [fp], [op], odev.precision)
        odev._batch.upload(cloud.pos, cloud.vel, cloud.mass, cloud.charge)
        odev._batch_key = key
    info, st = odev._batch.step(raise_on_error=False)
    if st == abi.SG_H_UNDERFLOW:
        raise RuntimeError("stepsize underflow created")
    abi.check(st, "step")
    cloud.pos, cloud.vel = odev._batch.download()
    cloud.pos2, cloud.vel2 = cloud.pos.copy(), cloud.vel.copy()
    s = info[0]
    cloud.lifetime = s["t"]
    odev.h = odev.hnext = s["h"]
    odev.errold = s["errold"]
    odev.reject = bool(s["reject"])
    odev.countstep = s["steps"] + s["rejects"]


def GetTimeStep(odev: OdeVars) -> float:
    """bin/ode.cpp:496-498."""
    return odev.h


@dataclasses.dataclass
class Operation:
    """operation, bin/operation.h:17-33: one step of the run's sequence."""
    name: str = "normal"       # normal | tof | trap_ramp | dissociation | anything else
    time: float = 1e-9         # duration (s)
    print_time: float = 0.0
    timestep: float = 0.0
    dissociation_fraction: float = 1.0
    dissociation_reactant: int = 0   # species index (the reference uses ion names)
    dissociation_product: int = 0
    product_mass: float = 0.0        # kg


class Operations:
    """operations, bin/operation.h:35-44: add(), total_time(), launch().  launch runs
    the whole sequence on the device (sg_batch_set_operations): the trap switches, the
    trap ramp to trap_param.newVrf/newVdc and the TOF kick trap_param.E_kick are the
    reference's, taken from odev.forcev as its INI parser leaves them."""

    _KINDS = {"normal": abi.SG_OP_NORMAL, "tof": abi.SG_OP_TOF,
              "trap_ramp": abi.SG_OP_TRAP_RAMP, "dissociation": abi.SG_OP_DISSOCIATION}

    def __init__(self):
        self.ops: list[Operation] = []

    def add(self, op: Operation) -> None:
        self.ops.append(op)

    def total_time(self) -> float:
        return float(sum(op.time for op in self.ops))

    def launch(self, cloud: IonCloud, odev: OdeVars, print_after_operation: bool = False,
               recorder=None):
        """Runs every operation; cloud.pos/vel/lifetime are updated.  recorder, if given,
        is (print_interval, stride, capacity) for the device recorder; the batch is
        returned so that its records can be read."""
        if not self.ops:
            raise RuntimeError("No operation loaded")
        fv = odev.forcev
        trap0 = fv.trap
        fv.trap = True  # the trap terms the operations switch
        fp = fv.field_params()
        fv.trap = trap0
        tp = fv.trap_param
        seq = []
        for o in self.ops:
            kind = self._KINDS.get(o.name, abi.SG_OP_FREE)
            q = abi.Operation()
            q.kind, q.print_after = kind, int(print_after_operation)
            q.duration, q.print_time, q.timestep = o.time, o.print_time, o.timestep
            q.new_vrf, q.new_vdc, q.e_kick = tp.newVrf, tp.newVdc, tp.E_kick
            q.reactant, q.product = o.dissociation_reactant, o.dissociation_product
            q.fraction, q.product_mass = o.dissociation_fraction, o.product_mass
            seq.append(q)
        op = OdeParams()
        op.rtol, op.atol, op.h0 = odev.rk_rtol, odev.rk_atol, odev.h
        op.t0, op.t_end = cloud.lifetime, float("inf")
        op.adaptive, op.max_rejects, op.method = int(odev.change_stepsize), 0, odev.method
        op.beta = odev.beta
        b = Batch(odev.context(), [cloud.nrparticles], [fp], [op], odev.precision)
        b.upload(cloud.pos, cloud.vel, cloud.mass, cloud.charge)
        if recorder is not None:
            b.set_recorder(*recorder)
        b.set_operations(seq)
        info, st = b.run(raise_on_error=False)
        if st == abi.SG_H_UNDERFLOW:
            raise RuntimeError("stepsize underflow created")
        abi.check(st, "operations")
        cloud.pos, cloud.vel = b.download()
        cloud.pos2, cloud.vel2 = cloud.pos.copy(), cloud.vel.copy()
        cloud.lifetime = info[0]["t"]
        odev.h = odev.hnext = info[0]["h"]
        odev._batch = None  # the next step() starts from the new state
        return b
