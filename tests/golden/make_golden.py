"""Generates the golden vectors in this directory by running the reference Simbuca
CPU path itself, compiled from its own sources (oracle/Makefile `make ref`).

    python tests/golden/make_golden.py

Needs the reference checkout, its root directory named by the environment variable
SIMBUCA_REF_DIR (the `ref` make targets read its sources); the committed .npz files
are what the tests use everywhere else.  Inputs are seeded
synthetic clouds (numpy Philox), stored next to the outputs.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from simbuca_gb300 import configs  # noqa: E402

AMU = oracle.AMU
REF_BIN = os.path.join(os.environ.get("SIMBUCA_REF_DIR", ""), "bin")  # read only
# Paul trap of the reference (_trap_param defaults, bin/trapparameters.cpp:2-10) with a
# TOF kick: Vrf, Vdc, kappa, r0, z0, freq_rf, E_kick
TRAPP = np.array([50.0, 5.0, 0.001, 0.04, 0.04, 50e5, 100.0])


def cloud(n, seed, sigma=0.5e-3, temp=300.0, mixed=False):
    rng = configs.rng_for(seed)
    m = np.full(n, 132.905)
    c = configs.gaussian_cloud(rng, n, sigma, temp, m)
    if mixed:
        c.charge = np.where(np.arange(n) % 3 == 0, 2, 1).astype(np.int32)
        c.mass = np.where(np.arange(n) % 2 == 0, 132.905, 86.909) * AMU
    return c


def init_library():
    """The reference's InitCloud harness (oracle/Makefile `make ref-init`).  Its
    initialization.cpp reads ../libraries/ mass tables when loaded, so it is loaded
    from the reference's bin/ directory."""
    odir = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-C", odir, "-s", "ref-init", f"REF_SRC={REF_BIN}"], check=True)
    cwd = os.getcwd()
    os.chdir(REF_BIN)
    try:
        lib = ctypes.CDLL(os.path.join(odir, "_ref", "libsimbuca_ref_init.so"))
    finally:
        os.chdir(cwd)
    return lib


OPS = dict(kinds=[0, 2, 1, 3, 0], durations=[4e-8, 6e-8, 2e-8, 2e-8, 3e-8],
           new_vrf=[0, 80.0, 0, 0, 0], new_vdc=[0, 2.0, 0, 0, 0], e_kick=[0, 0, 50.0, 0, 0])


def ops_scenario(path):
    """One operation sequence through the reference's operations::launch, in a process
    of its own (the reference keeps the run's state in globals)."""
    lib = init_library()
    c = cloud(64, 41)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    arrs = {k: np.ascontiguousarray(v, np.float64) for k, v in OPS.items() if k != "kinds"}
    kinds = np.ascontiguousarray(OPS["kinds"], np.int32)
    pos, vel, t = np.zeros((64, 3)), np.zeros((64, 3)), np.zeros(3)
    lib.ref_ops_run(64, c.pos.ctypes.data_as(dp), c.vel.ctypes.data_as(dp),
                    c.mass.ctypes.data_as(dp), c.charge.ctypes.data_as(ip),
                    TRAPP.ctypes.data_as(dp), 1, ctypes.c_double(2e-9), 5, len(kinds),
                    kinds.ctypes.data_as(ip), arrs["durations"].ctypes.data_as(dp),
                    arrs["new_vrf"].ctypes.data_as(dp), arrs["new_vdc"].ctypes.data_as(dp),
                    arrs["e_kick"].ctypes.data_as(dp), pos.ctypes.data_as(dp),
                    vel.ctypes.data_as(dp), t.ctypes.data_as(dp))
    np.savez_compressed(path, pos0=c.pos, vel0=c.vel, mass=c.mass, charge=c.charge, pos=pos,
                        vel=vel, t=t, h0=2e-9, **{k: np.asarray(v) for k, v in OPS.items()})


def main():
    if len(sys.argv) > 2 and sys.argv[1] == "--ops":
        ops_scenario(sys.argv[2])
        return
    oracle.build(ref=True)
    assert oracle.ref_available(), "reference harness did not build"
    out = {}

    # 1. force() on the 1,000-ion cloud of the small workload: Coulomb only, and
    #    Paul trap + TOF + Coulomb at a stage time.
    c = configs.penning_1k().clouds[0]
    t = 1.3e-7
    f_coul = oracle.ref_force(c.pos, c.vel, c.mass, c.charge, t, trap=0, tof=0, coulomb=1,
                              coulomb_scale=1.0, trapp=TRAPP)
    f_all = oracle.ref_force(c.pos, c.vel, c.mass, c.charge, t, trap=1, tof=1, coulomb=1,
                             coulomb_scale=1.0, trapp=TRAPP)
    np.savez_compressed(os.path.join(HERE, "force_1k.npz"), pos=c.pos, vel=c.vel, mass=c.mass,
                        charge=c.charge, t=t, trapp=TRAPP, f_coulomb=f_coul, f_all=f_all)
    out["force_1k"] = f_all.shape

    # 2. mixed charges and masses, scaled Coulomb
    c = cloud(300, 11, mixed=True)
    f = oracle.ref_force(c.pos, c.vel, c.mass, c.charge, 0.0, trap=1, tof=0, coulomb=1,
                         coulomb_scale=0.75, trapp=TRAPP)
    np.savez_compressed(os.path.join(HERE, "force_mixed.npz"), pos=c.pos, vel=c.vel, mass=c.mass,
                        charge=c.charge, t=0.0, trapp=TRAPP, coulomb_scale=0.75, f=f)

    # 3. edge sizes: one ion (no partner), two ions
    edges = {}
    for n in (1, 2, 3):
        c = cloud(n, 20 + n)
        edges[f"pos{n}"], edges[f"vel{n}"] = c.pos, c.vel
        edges[f"mass{n}"], edges[f"charge{n}"] = c.mass, c.charge
        edges[f"f{n}"] = oracle.ref_force(c.pos, c.vel, c.mass, c.charge, 2e-8, trap=1, tof=0,
                                          coulomb=1, coulomb_scale=1.0, trapp=TRAPP)
    np.savez_compressed(os.path.join(HERE, "force_edges.npz"), **edges)

    # 4. adaptive Dormand-Prince: Paul trap + Coulomb, attempt history (t, h, err, accepted)
    runs = {}
    for tag, n, seed, rtol, atol, t_end in (("tight", 128, 5, 1e-9, 1e-15, 4e-7),
                                            ("default", 200, 6, 1e-7, 1e-7, 2e-6)):
        c = cloud(n, seed)
        p, v, ctrl, hist, nh = oracle.ref_dp45_run(
            c.pos, c.vel, c.mass, c.charge, trap=1, tof=0, coulomb=1, coulomb_scale=1.0,
            trapp=TRAPP, t0=0.0, t_end=t_end, h0=1e-9, adaptive=1, rtol=rtol, atol=atol,
            max_steps=1 << 40, mode=1, hist_cap=200000)
        assert nh > 0
        # the same run through the reference's own step() must land on the same state
        p0, v0, ctrl0, _, _ = oracle.ref_dp45_run(
            c.pos, c.vel, c.mass, c.charge, trap=1, tof=0, coulomb=1, coulomb_scale=1.0,
            trapp=TRAPP, t0=0.0, t_end=t_end, h0=1e-9, adaptive=1, rtol=rtol, atol=atol,
            max_steps=1 << 40, mode=0)
        assert np.array_equal(p0, p) and np.array_equal(v0, v) and np.array_equal(ctrl0, ctrl)
        runs.update({f"{tag}_pos0": c.pos, f"{tag}_vel0": c.vel, f"{tag}_mass": c.mass,
                     f"{tag}_charge": c.charge, f"{tag}_pos": p, f"{tag}_vel": v,
                     f"{tag}_ctrl": ctrl, f"{tag}_hist": hist,
                     f"{tag}_cfg": np.array([rtol, atol, t_end, 1e-9])})
        out[f"dp45_{tag}"] = (len(hist), int((hist[:, 3] == 0).sum()))
    np.savez_compressed(os.path.join(HERE, "dp45_adaptive.npz"), **runs)

    # 5. Cash-Karp (the reference's "RungaKutta4", Init_ode order 4), adaptive, with the
    #    reference's error sum carried over from the previous attempt
    c = cloud(150, 8)
    p, v, ctrl, hist, nh = oracle.ref_dp45_run(
        c.pos, c.vel, c.mass, c.charge, trap=1, tof=0, coulomb=1, coulomb_scale=1.0, trapp=TRAPP,
        t0=0.0, t_end=4e-7, h0=1e-9, adaptive=1, rtol=1e-9, atol=1e-15, max_steps=1 << 40,
        mode=1, hist_cap=100000, method=4)
    p0, v0, ctrl0, _, _ = oracle.ref_dp45_run(
        c.pos, c.vel, c.mass, c.charge, trap=1, tof=0, coulomb=1, coulomb_scale=1.0, trapp=TRAPP,
        t0=0.0, t_end=4e-7, h0=1e-9, adaptive=1, rtol=1e-9, atol=1e-15, max_steps=1 << 40,
        mode=0, method=4)
    assert np.array_equal(p0, p) and np.array_equal(ctrl0, ctrl)
    np.savez_compressed(os.path.join(HERE, "ck45_adaptive.npz"), pos0=c.pos, vel0=c.vel,
                        mass=c.mass, charge=c.charge, pos=p, vel=v, ctrl=ctrl, hist=hist)
    out["ck45"] = (len(hist), int((hist[:, 3] == 0).sum()))

    # 6. Gear predictor-corrector (Init_ode order 1): fixed 2 ns steps through step()
    c = cloud(150, 9)
    p, v, ctrl, hist, nh = oracle.ref_dp45_run(
        c.pos, c.vel, c.mass, c.charge, trap=1, tof=0, coulomb=1, coulomb_scale=1.0, trapp=TRAPP,
        t0=0.0, t_end=1.0, h0=2e-9, adaptive=0, rtol=1e-9, atol=1e-15, max_steps=300, mode=0,
        method=1)
    np.savez_compressed(os.path.join(HERE, "gear_fixed.npz"), pos0=c.pos, vel0=c.vel,
                        mass=c.mass, charge=c.charge, pos=p, vel=v, ctrl=ctrl)
    out["gear"] = int(ctrl[5])

    # 7. InitCloud (bin/initialization.cpp:117-206): the reference's generator itself,
    #    one and two Maxwell-Boltzmann energies, mixed masses
    init = {}
    lib = init_library()
    for tag, n, ev, seed, semi, off in (("a", 1000, [0.5], 7, [1e-3, 1e-3, 2e-3], [0, 0, 1e-4]),
                                        ("b", 2500, [0.2, 0.05], 12345, [2e-3, 2e-3, 4e-3],
                                         [1e-4, -2e-4, 0.0])):
        mass = np.where(np.arange(n) % 2 == 0, 132.905, 86.909) * AMU
        ev, semi, off = (np.array(x, np.float64) for x in (ev, semi, off))
        pos, vel = np.zeros((n, 3)), np.zeros((n, 3))
        ch = np.ones(n, np.int32)
        dp = ctypes.POINTER(ctypes.c_double)
        got = lib.ref_init_cloud(n, ev.ctypes.data_as(dp), len(ev), seed, semi.ctypes.data_as(dp),
                                 off.ctypes.data_as(dp), mass.ctypes.data_as(dp),
                                 ch.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 pos.ctypes.data_as(dp), vel.ctypes.data_as(dp))
        assert got == n
        init.update({f"{tag}_n": n, f"{tag}_ev": ev, f"{tag}_seed": seed, f"{tag}_semi": semi,
                     f"{tag}_off": off, f"{tag}_mass": mass, f"{tag}_pos": pos, f"{tag}_vel": vel})
    np.savez_compressed(os.path.join(HERE, "init_cloud.npz"), **init)
    out["init_cloud"] = 2

    # 8. the reference's text output (PrintParticles + PrintCloud) of a two-species state
    rng = configs.rng_for(31)
    n = 300
    species = (rng.random(n) < 0.3).astype(np.int32)  # 0 = Cs133, 1 = Rb87
    mass = np.where(species == 0, 132.905, 86.909) * AMU
    pos = rng.normal(0.0, 6e-4, (n, 3)) + np.array([1e-5, -2e-5, 3e-5])
    vel = rng.normal(0.0, 120.0, (n, 3))
    names = ["Cs133", "Rb87"]
    text = oracle.ref_print(pos, vel, mass, np.ones(n, np.int32), species, names, 3.7e-6)
    data = {k: [ln for ln in v.splitlines() if ln and not ln.startswith("#")]
            for k, v in text.items()}
    np.savez_compressed(os.path.join(HERE, "print_state.npz"), pos=pos, vel=vel, mass=mass,
                        species=species, names=np.array(names), t=3.7e-6,
                        pall=np.array(data["_pAll.txt"]), cloud0=np.array(data["_cloud0.txt"]),
                        cloud1=np.array(data["_cloud1.txt"]))
    out["print_state"] = len(data["_pAll.txt"])

    # 9. an operation sequence (normal, trap ramp, TOF, free flight, normal) with fixed
    #    2 ns Dormand-Prince steps through the reference's operations::launch
    subprocess.run([sys.executable, os.path.abspath(__file__), "--ops",
                    os.path.join(HERE, "ops_sequence.npz")], check=True)
    out["ops_sequence"] = float(np.load(os.path.join(HERE, "ops_sequence.npz"))["t"][0])

    # 10. fixed step, 40 steps of 2 ns
    c = cloud(64, 7)
    p, v, ctrl, hist, nh = oracle.ref_dp45_run(
        c.pos, c.vel, c.mass, c.charge, trap=1, tof=0, coulomb=1, coulomb_scale=1.0, trapp=TRAPP,
        t0=0.0, t_end=1.0, h0=2e-9, adaptive=0, rtol=1e-7, atol=1e-7, max_steps=40, mode=1,
        hist_cap=100)
    np.savez_compressed(os.path.join(HERE, "dp45_fixed.npz"), pos0=c.pos, vel0=c.vel,
                        mass=c.mass, charge=c.charge, pos=p, vel=v, ctrl=ctrl, hist=hist)
    out["dp45_fixed"] = len(hist)
    print(out)


if __name__ == "__main__":
    main()
