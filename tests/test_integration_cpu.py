"""Drop-in at link level (CPU only): the reference's complete program, built from its
own sources with the CUNBODY backend selected, links against libsimgb.so in place of
the closed libcunbody1.a, with no source change.  Needs the reference checkout."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference/bin"
BIN = os.path.join(ROOT, "oracle", "_ref", "cunbody", "simbuca_gb300")


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_reference_links_against_libsimgb():
    from simbuca_gb300 import build
    build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "cunbody-link"],
                   check=True)
    assert os.path.exists(BIN)
    und = subprocess.run(["nm", "-D", "--undefined-only", BIN], capture_output=True, text=True,
                         check=True).stdout
    assert "cunbody1_force_begin" in und and "cunbody1_force_end" in und
    deps = subprocess.run(["ldd", BIN], capture_output=True, text=True).stdout
    assert "libsimgb.so" in deps and "not found" not in deps.split("libsimgb.so")[1].split("\n")[0]
