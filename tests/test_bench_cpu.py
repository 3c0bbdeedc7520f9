"""bench.py's reference arm on the host: the oracle's Dormand-Prince steps of the
workload's cloud (the reference's FP64 force() and step() loop, bin/force.cpp:34-178 and
bin/ode.cpp:459-494), settled by the same rule as the device arm, printing the same
metric and config keys; --beta runs the controller's PI form (bin/ode.cpp:428-439) in it.
The device arm fails loudly without a GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def bench(*argv, check=True):
    r = subprocess.run([sys.executable, "bench.py", *argv], cwd=ROOT, capture_output=True,
                       text=True, timeout=300)
    if check:
        assert r.returncode == 0, r.stderr[-2000:]
    return r


def reference_line(*extra):
    r = bench("--impl", "reference", "--workload", "penning_1k", "--steps", "3", "--warmup",
              "1", "--settle", "4", *extra)
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.fixture(scope="module")
def lines():
    return {b: reference_line("--beta", str(b)) for b in (0.0, 0.04)}


def test_reference_line_contract(lines):
    d = lines[0.0]
    assert d["impl"] == "reference" and d["unit"] == "sim-us/wall-s"
    assert d["metric"].startswith("sim-us/wall-s") and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] >= 1 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    cfg = d["config"]
    assert cfg["workload"] == "penning_1k" and cfg["ions"] == 1000
    assert cfg["step_control"].startswith("reference I-controller")
    assert 1 <= cfg["settle_steps"] <= 4 and cfg["h_settled"] > 0


def test_reference_arm_runs_the_pi_controller(lines):
    a, b = lines[0.0], lines[0.04]
    assert b["config"]["step_control"].startswith("PI controller, beta 0.04")
    # the same settled start, a different step-size rule: a different schedule
    assert a["mean_h"] != b["mean_h"]


def test_device_arm_fails_loudly_without_a_gpu():
    pytest.importorskip("torch")
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = bench("--workload", "penning_1k", "--steps", "1", "--warmup", "0", check=False)
    assert r.returncode != 0
    assert "{" not in r.stdout  # no bench line
