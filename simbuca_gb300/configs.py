"""Seeded synthetic ion clouds and trap settings for the benchmark workloads.

There is no public dataset for this path: every workload is a seeded synthetic
cloud.  Positions are Gaussian per axis (or uniform in a spheroid, drawn by
rejection as the reference's InitCloud does, bin/initialization.cpp:157-173);
velocities are Maxwell-Boltzmann, i.e. Gaussian per component with
sigma_v = sqrt(k_B T / m).  The generator is numpy's Philox bit generator seeded
with the workload seed; the arrays it returns are what both the GPU path and the
CPU oracle read, so parity never depends on cross-platform RNG streams.

Workloads (SI units):
  penning_1k     1,000 ions 132.905 u, sigma 0.5 mm, 300 K, seed 0; B 7 T,
                 V0 10 V, d0 1 cm; rtol 1e-9, atol 1e-15; 20 us; no drive, no gas.
  penning_65k    65,536 ions, 50/50 132.905 / 132.906 u, sigma 1 mm, 300 K, seed 1;
                 quadrupole drive at the mass-weighted nu_c, 0.5 V, 200 us;
                 friction delta 1e3 /s; rtol 1e-9.
  spheroid_1m    1,048,576 ions 132.905 u, uniform spheroid 2 mm radial x 4 mm axial,
                 1 K, seed 2; B 7 T, V0 10 V; 50 Dormand-Prince steps.
  scan_512       512 clouds, n_c = floor(exp(U[ln 64, ln 8192])) (seed 3), sigma
                 0.5 mm, 300 K, 132.905 u; quadrupole drive at nu_c + Delta_k,
                 Delta_k = -5 + 10 k/511 Hz, 0.2 V, 100 us; delta 5e2 /s.
  learned_4k     4,096 ions 132.905 u, 300 K, seed 4; dipole 0.1 V at nu_minus, then
                 quadrupole 0.5 V at nu_c, over 1 ms; delta 1e3 /s.
The electrode radius of the excitation terms is not given by the workloads; it
is r_el = 10 mm (= d0) throughout.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .abi import (FieldParams, OdeParams, SG_F_COULOMB, SG_F_DIPOLE, SG_F_FRICTION,
                  SG_F_PENNING, SG_F_QUAD)
from .constants import AMU, EL_CHARGE, KB, PI

B_TESLA = 7.0
V0 = 10.0
D0 = 0.01
R_EL = 0.01
M_CS = 132.905
M_CS2 = 132.906


@dataclasses.dataclass
class Cloud:
    pos: np.ndarray      # [n,3] m
    vel: np.ndarray      # [n,3] m/s
    mass: np.ndarray     # [n] kg
    charge: np.ndarray   # [n] int32


@dataclasses.dataclass
class Workload:
    name: str
    clouds: list            # list[Cloud]
    fields: list            # list[FieldParams], one per cloud
    odes: list              # list[OdeParams], one per cloud
    sim_time: float         # s of simulated time per cloud
    max_steps: int | None = None

    @property
    def counts(self):
        return [len(c.mass) for c in self.clouds]

    @property
    def n_total(self):
        return int(sum(self.counts))

    def concat(self) -> Cloud:
        return Cloud(np.concatenate([c.pos for c in self.clouds]),
                     np.concatenate([c.vel for c in self.clouds]),
                     np.concatenate([c.mass for c in self.clouds]),
                     np.concatenate([c.charge for c in self.clouds]).astype(np.int32))

    def interactions_per_force(self) -> float:
        return float(sum(n * (n - 1) for n in self.counts))


def nu_c(m_amu: float, q: int = 1, B: float = B_TESLA) -> float:
    return q * EL_CHARGE * B / (m_amu * AMU) / (2 * PI)


def penning_freqs(m_amu: float, q: int = 1, B: float = B_TESLA, V0_: float = V0,
                  d0: float = D0):
    """(nu_c, nu_plus, nu_minus, nu_z) of the ideal Penning trap, Hz."""
    m = m_amu * AMU
    wc = q * EL_CHARGE * B / m
    wz = math.sqrt(q * EL_CHARGE * V0_ / (m * d0 * d0))
    root = math.sqrt(wc * wc - 2 * wz * wz)
    wp, wm = (wc + root) / 2, (wc - root) / 2
    return tuple(w / (2 * PI) for w in (wc, wp, wm, wz))


def rng_for(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(seed))


def gaussian_cloud(rng, n, sigma, temp_K, masses_amu, charge=1) -> Cloud:
    masses = np.asarray(masses_amu, np.float64) * AMU
    pos = rng.normal(0.0, sigma, size=(n, 3))
    sv = np.sqrt(KB * temp_K / masses)
    vel = rng.normal(0.0, 1.0, size=(n, 3)) * sv[:, None]
    return Cloud(np.ascontiguousarray(pos), np.ascontiguousarray(vel), masses,
                 np.full(n, charge, np.int32))


def spheroid_cloud(rng, n, a_r, a_z, temp_K, m_amu) -> Cloud:
    out = np.empty((n, 3))
    k = 0
    while k < n:
        m = max(1024, int(1.3 * (n - k)) + 16)
        u = rng.uniform(-1.0, 1.0, size=(m, 3))
        u = u[(u * u).sum(1) <= 1.0]
        take = min(len(u), n - k)
        out[k:k + take] = u[:take]
        k += take
    out *= np.array([a_r, a_r, a_z])
    masses = np.full(n, m_amu * AMU)
    sv = math.sqrt(KB * temp_K / (m_amu * AMU))
    vel = rng.normal(0.0, sv, size=(n, 3))
    return Cloud(np.ascontiguousarray(out), vel, masses, np.ones(n, np.int32))


def penning_field(coulomb=True, quad=None, dipole=None, delta=0.0) -> FieldParams:
    fp = FieldParams()
    fp.flags = SG_F_PENNING | (SG_F_COULOMB if coulomb else 0)
    fp.coulomb_scale = 1.0
    fp.B, fp.V0, fp.d0, fp.r_el = B_TESLA, V0, D0, R_EL
    if quad is not None:
        fp.flags |= SG_F_QUAD
        fp.Uq, fp.nu_q, fp.phi_q, fp.tq_on, fp.tq_off = quad
    if dipole is not None:
        fp.flags |= SG_F_DIPOLE
        fp.Ud, fp.nu_d, fp.phi_d, fp.td_on, fp.td_off = dipole
    if delta:
        fp.flags |= SG_F_FRICTION
        fp.delta = delta
    return fp


def ode(rtol, atol, h0, t_end, t0=0.0, adaptive=True, max_rejects=0, method=5,
        beta=0.0) -> OdeParams:
    """Controller settings; method 5 = Dormand-Prince, 4 = Cash-Karp, 1 = Gear; beta
    is the PI term of the step-size controller (0: the reference's I-controller)."""
    o = OdeParams()
    o.rtol, o.atol, o.h0, o.t0, o.t_end = rtol, atol, h0, t0, t_end
    o.adaptive, o.max_rejects, o.method = int(adaptive), int(max_rejects), int(method)
    o.beta = float(beta)
    return o


H0 = 1e-9  # first trial step (the reference's default httry, bin/ode.cpp:509)


def penning_1k(n: int = 1000, seed: int = 0) -> Workload:
    rng = rng_for(seed)
    c = gaussian_cloud(rng, n, 0.5e-3, 300.0, np.full(n, M_CS))
    T = 20e-6
    return Workload("penning_1k", [c], [penning_field()], [ode(1e-9, 1e-15, H0, T)], T)


def penning_65k(n: int = 65536, seed: int = 1) -> Workload:
    rng = rng_for(seed)
    masses = np.where(np.arange(n) % 2 == 0, M_CS, M_CS2)
    c = gaussian_cloud(rng, n, 1e-3, 300.0, masses)
    nu = float(np.mean([nu_c(m) for m in masses[:2]]))  # 50/50 mix: mass-weighted mean
    T = 200e-6
    fp = penning_field(quad=(0.5, nu, 0.0, 0.0, T), delta=1e3)
    return Workload("penning_65k", [c], [fp], [ode(1e-9, 1e-15, H0, T)], T)


def spheroid_1m(n: int = 1 << 20, seed: int = 2) -> Workload:
    rng = rng_for(seed)
    c = spheroid_cloud(rng, n, 2e-3, 4e-3, 1.0, M_CS)
    return Workload("spheroid_1m", [c], [penning_field()], [ode(1e-9, 1e-15, H0, 1.0)],
                    1.0, max_steps=50)


def scan_counts(n_clouds: int = 512, seed: int = 3, lo: int = 64, hi: int = 8192):
    rng = rng_for(seed)
    u = rng.uniform(math.log(lo), math.log(hi), size=n_clouds)
    return np.floor(np.exp(u)).astype(np.int64).clip(lo, hi)


def scan_512(n_clouds: int = 512, seed: int = 3, sim_time: float = 100e-6) -> Workload:
    counts = scan_counts(n_clouds, seed)
    rng = rng_for(seed + 1000)
    base = nu_c(M_CS)
    clouds, fields, odes = [], [], []
    for k, n in enumerate(counts):
        clouds.append(gaussian_cloud(rng, int(n), 0.5e-3, 300.0, np.full(int(n), M_CS)))
        d = -5.0 + 10.0 * k / max(n_clouds - 1, 1)
        fields.append(penning_field(quad=(0.2, base + d, 0.0, 0.0, sim_time), delta=5e2))
        odes.append(ode(1e-9, 1e-15, H0, sim_time))
    return Workload("scan_512", clouds, fields, odes, sim_time)


def learned_4k(n: int = 4096, seed: int = 4, sim_time: float = 1e-3) -> Workload:
    rng = rng_for(seed)
    c = gaussian_cloud(rng, n, 0.5e-3, 300.0, np.full(n, M_CS))
    nc, _, nm, _ = penning_freqs(M_CS)
    half = sim_time / 2
    fp = penning_field(dipole=(0.1, nm, 0.0, 0.0, half), quad=(0.5, nc, 0.0, half, sim_time),
                       delta=1e3)
    return Workload("learned_4k", [c], [fp], [ode(1e-9, 1e-15, H0, sim_time)], sim_time)


WORKLOADS = {"penning_1k": penning_1k, "penning_65k": penning_65k,
             "spheroid_1m": spheroid_1m, "scan_512": scan_512, "learned_4k": learned_4k}
