"""State files (no GPU): the binary restart file round trip and its failure statuses, and
the restart from the reference's own particle output (PrintParticles lines made by the
compiled reference, tests/golden/print_state.npz)."""
import os

import numpy as np
import pytest

from simbuca_gb300 import abi
from simbuca_gb300.abi import SG_BAD_ARG, SG_IO_ERR, SG_TOO_LARGE
from simbuca_gb300.api import load_state, read_particles_text, save_state

GOLD = os.path.join(os.path.dirname(__file__), "golden")
AMU = 1.66053873e-27


def status_of(fn, *a):
    with pytest.raises(RuntimeError) as e:
        fn(*a)
    return str(e.value)


def test_binary_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    n = 1001
    pos = rng.normal(0, 1e-3, (n, 3))
    vel = rng.normal(0, 100, (n, 3))
    mass = rng.uniform(40, 200, n) * AMU
    charge = rng.integers(-2, 4, n).astype(np.int32)
    species = rng.integers(0, 3, n).astype(np.int32)
    p = str(tmp_path / "s.bin")
    save_state(p, pos, vel, mass, charge, t=3.25e-6, species=species)
    assert os.path.getsize(p) == 24 + n * (24 + 24 + 8 + 4 + 4)
    s = load_state(p)
    assert s["t"] == 3.25e-6
    for k, v in (("pos", pos), ("vel", vel), ("mass", mass), ("charge", charge),
                 ("species", species)):
        assert np.array_equal(s[k], v), k
    save_state(p, pos, vel, mass, charge)  # no species: zeros, t = 0
    s = load_state(p)
    assert s["t"] == 0.0 and not s["species"].any() and np.array_equal(s["pos"], pos)


def test_empty_state(tmp_path):
    p = str(tmp_path / "e.bin")
    save_state(p, np.empty((0, 3)), np.empty((0, 3)), np.empty(0), np.empty(0, np.int32), 1.0)
    s = load_state(p)
    assert s["pos"].shape == (0, 3) and s["t"] == 1.0


def test_binary_failures(tmp_path):
    L = abi.load()
    import ctypes
    n, t = ctypes.c_int(0), ctypes.c_double(0.0)
    missing = str(tmp_path / "none.bin").encode()
    assert L.sg_state_info(missing, ctypes.byref(n), ctypes.byref(t)) == SG_IO_ERR
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"NOTSTATE" + bytes(16))
    assert L.sg_state_info(str(bad).encode(), ctypes.byref(n), ctypes.byref(t)) == SG_IO_ERR
    # truncated: header says 10 ions, arrays cut short
    p = str(tmp_path / "cut.bin")
    z = np.zeros((10, 3))
    save_state(p, z, z, np.ones(10), np.ones(10, np.int32))
    data = open(p, "rb").read()
    open(p, "wb").write(data[:100])
    buf = np.empty(30)
    q = np.empty(10, np.int32)
    assert L.sg_state_load(p.encode(), 10, ctypes.byref(t), abi.dptr(buf), abi.dptr(buf),
                           abi.dptr(np.empty(10)), abi.iptr(q), None) == SG_IO_ERR
    # capacity below n
    open(p, "wb").write(data)
    assert L.sg_state_load(p.encode(), 5, ctypes.byref(t), abi.dptr(buf), abi.dptr(buf),
                           abi.dptr(np.empty(10)), abi.iptr(q), None) == SG_TOO_LARGE
    assert L.sg_state_save(None, 1, 0.0, None, None, None, None, None) == SG_BAD_ARG


def write_lines(path, lines):
    with open(path, "w") as f:
        for ln in lines:
            f.write(str(ln) + "\n")


def test_restart_from_reference_output(tmp_path):
    """The reference's PrintParticles lines (300 ions, two species) read back: ids, species,
    masses from the table, positions and velocities to the 7 printed digits."""
    g = np.load(os.path.join(GOLD, "print_state.npz"))
    names = [str(x) for x in g["names"]]
    masses = [g["mass"][g["species"] == s][0] for s in range(len(names))]
    p = str(tmp_path / "run_pAll.txt")
    write_lines(p, g["pall"])
    s = read_particles_text(p, names, masses, [1, 1])
    n = len(g["mass"])
    assert len(s["ids"]) == n and np.array_equal(s["ids"], np.arange(n))
    assert s["t"] == pytest.approx(float(g["t"]), rel=1e-12)
    assert np.array_equal(s["species"], g["species"])
    assert np.array_equal(s["mass"], g["mass"])
    np.testing.assert_allclose(s["pos"], g["pos"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(s["vel"], g["vel"], rtol=1e-6, atol=1e-9)


def test_text_last_snapshot_and_errors(tmp_path):
    g = np.load(os.path.join(GOLD, "print_state.npz"))
    names = [str(x) for x in g["names"]]
    masses = [g["mass"][g["species"] == s][0] for s in range(len(names))]
    early = [ln.replace("3.700000e-03", "1.000000e-03", 1) for ln in g["pall"][:50]]
    p = str(tmp_path / "two.txt")
    write_lines(p, list(early) + list(g["pall"]))
    s = read_particles_text(p, names, masses, [1, 1])
    assert len(s["ids"]) == len(g["pall"]) and s["t"] == pytest.approx(3.7e-6, rel=1e-12)
    # the same print written twice at the same time: the last one only
    p2 = str(tmp_path / "dup.txt")
    write_lines(p2, list(g["pall"]) + list(g["pall"]))
    s2 = read_particles_text(p2, names, masses, [1, 1])
    assert len(s2["ids"]) == len(g["pall"]) and np.array_equal(s2["ids"], s["ids"])
    # capacity below the snapshot
    assert "status 9)" in status_of(read_particles_text, p, names, masses, [1, 1], 10)
    # a name missing from the table
    assert "status 1)" in status_of(read_particles_text, p, names[:1], masses[:1], [1])
    # malformed line
    bad = str(tmp_path / "bad.txt")
    write_lines(bad, list(g["pall"][:3]) + ["0 Rb87 oops"])
    assert "status 10)" in status_of(read_particles_text, bad, names, masses, [1, 1])
