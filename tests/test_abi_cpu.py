"""The C ABI without a GPU: libsimgb.so loads and exports every function that
include/simgb.h declares, and the ctypes mirrors have the C layouts.  No compute calls."""
import ctypes
import os
import re
import subprocess

import pytest

from simbuca_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "simgb.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(\w+)\s*\(", src, flags=re.M)
    return sorted({n for n in names if n.startswith(("sg_", "cunbody1_"))})


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(abi.LIB_PATH):
        from simbuca_gb300 import build
        build.build()
    return abi.load()


def test_header_and_binding_agree():
    assert declared_functions() == sorted(abi.EXPORTED)


def test_library_exports_all_symbols(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_status_strings(lib):
    assert lib.sg_status_string(abi.SG_H_UNDERFLOW) == b"stepsize underflow created"
    assert lib.sg_status_string(999) == b"unknown status"
    assert lib.sg_version() >= 100


def test_null_context_is_rejected(lib):
    # argument checks happen before any CUDA call
    assert lib.sg_destroy(None) == abi.SG_BAD_ARG
    assert lib.sg_sync(None) == abi.SG_BAD_ARG
    assert lib.sg_batch_attempts(None, 1) == abi.SG_BAD_ARG
    assert lib.sg_create(0, None) == abi.SG_BAD_ARG
    assert lib.sg_stage_timing(None, None, None) == abi.SG_BAD_ARG
    assert lib.sg_kernel_timing(None, None, None, None) == abi.SG_BAD_ARG
    assert lib.sg_batch_set_controller_safety(None, 0.9) == abi.SG_BAD_ARG
    assert lib.sg_batch_set_proposer(None, None, 0.9) == abi.SG_BAD_ARG
    assert lib.sg_dp45_step(None, None) == abi.SG_BAD_ARG
    assert lib.sg_batch_run(None, 1, None) == abi.SG_BAD_ARG


def test_status_string_io(lib):
    assert lib.sg_status_string(abi.SG_IO_ERR) == b"file could not be read or written"


STRUCTS = {
    "sg_field_params": abi.FieldParams,
    "sg_ode_params": abi.OdeParams,
    "sg_step_info": abi.StepInfo,
    "sg_check_info": abi.CheckInfo,
}


def test_struct_layouts(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, cls in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            a, b, c = line.split()
            got[(a, b)] = int(c)
    for cname, cls in STRUCTS.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
