"""Drop-in at link level (CPU only): the reference's complete program, built from its
own sources with the CUNBODY backend selected, links against libsimgb.so in place of
the closed libcunbody1.a, with no source change; and the __GB300_ON__ backend of
force() compiles against the reference's headers and links with its objects.  Needs
the reference checkout, named by the environment variable SIMBUCA_REF_DIR (its root
directory); without it these tests skip."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.environ.get("SIMBUCA_REF_DIR", "")
REF = os.path.join(REF_DIR, "bin") if REF_DIR else ""
BIN = os.path.join(ROOT, "oracle", "_ref", "cunbody", "simbuca_gb300")
GBF = os.path.join(ROOT, "oracle", "_ref", "gb300_force", "gb300_force_check")
needs_ref = pytest.mark.skipif(not (REF and os.path.isdir(REF)),
                               reason="reference checkout not given (SIMBUCA_REF_DIR)")


def make(target):
    from simbuca_gb300 import build
    build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), target,
                    f"REF_SRC={REF}"], check=True)


@needs_ref
def test_reference_links_against_libsimgb():
    make("cunbody-link")
    assert os.path.exists(BIN)
    und = subprocess.run(["nm", "-D", "--undefined-only", BIN], capture_output=True, text=True,
                         check=True).stdout
    assert "cunbody1_force_begin" in und and "cunbody1_force_end" in und
    deps = subprocess.run(["ldd", BIN], capture_output=True, text=True).stdout
    assert "libsimgb.so" in deps and "not found" not in deps.split("libsimgb.so")[1].split("\n")[0]


@needs_ref
def test_gb300_force_backend_builds_against_reference_headers():
    make("gb300-force-link")
    assert os.path.exists(GBF)
    und = subprocess.run(["nm", "-D", "--undefined-only", GBF], capture_output=True,
                         text=True, check=True).stdout
    assert "sg_coulomb_accel" in und and "sg_create" in und
    r = subprocess.run([GBF], capture_output=True, text=True, timeout=120)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        # against the reference's own CPU loop, within the FP32-compensated bound
        assert r.returncode == 0, r.stdout + r.stderr
    else:
        assert r.returncode == 3 and "no usable CUDA device" in r.stdout, r.stdout + r.stderr
