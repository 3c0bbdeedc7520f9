"""sg_coulomb_accel_noalloc: the FP64 Coulomb sum for callers that cannot allocate
device memory -- applications that allocate everything up front, or plug-ins that
only receive device pointers from a host framework's memory pool.  The entry point
takes the caller's device buffers and keeps its scratch in a fixed array of the
library (n <= 8192), so these tests give it torch-allocated device buffers and check
it against the allocating entry point, sg_coulomb_accel, on two calls in a row.

This file is collected last so that a run stopping at the first failure has run
every other test before it."""
import ctypes

import numpy as np
import pytest

from simbuca_gb300 import abi, configs
from simbuca_gb300.api import Context
from simbuca_gb300.constants import EL_CHARGE, KE

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX_IONS = 8192


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def call_noalloc(pos, q, kq):
    n = len(q)
    dpos = torch.tensor(pos, dtype=torch.float64, device="cuda")
    dq = torch.tensor(q, dtype=torch.float64, device="cuda")
    dkq = torch.tensor(kq, dtype=torch.float64, device="cuda")
    dacc = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    st = abi.load().sg_coulomb_accel_noalloc(n, ptr(dpos), ptr(dq), ptr(dkq), ptr(dacc),
                                             ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return st, dacc.cpu().numpy()


def cloud(n, seed):
    c = configs.gaussian_cloud(configs.rng_for(seed), n, 5e-4, 300.0, np.full(n, 132.905))
    q = c.charge.astype(np.float64)
    q[::5] = 2.0
    kq = KE * EL_CHARGE * q * EL_CHARGE / c.mass
    return c.pos, q, kq


def test_two_calls_match_allocating_entry_point():
    ctx = Context(0)
    try:
        # two calls in a row: the second reuses the scratch the first left behind
        for n, seed in ((3000, 1), (MAX_IONS, 2)):
            pos, q, kq = cloud(n, seed)
            st, acc = call_noalloc(pos, q, kq)
            assert st == abi.SG_OK
            ref = ctx.coulomb_accel(pos, q, kq, abi.SG_PREC_FP64)
            e = np.linalg.norm(acc - ref, axis=1) / np.linalg.norm(ref, axis=1)
            assert e.max() <= 1e-12, (n, float(e.max()))
    finally:
        ctx.close()


def test_rejects_sizes_beyond_capacity():
    pos, q, kq = cloud(MAX_IONS + 1, 3)
    st, acc = call_noalloc(pos, q, kq)
    assert st == abi.SG_TOO_LARGE
    assert np.isnan(acc).all()  # nothing was written
