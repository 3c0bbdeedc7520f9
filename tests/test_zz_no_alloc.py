"""sg_coulomb_accel_noalloc: the FP64 Coulomb sum for callers that cannot allocate
device memory -- applications that allocate everything up front, or plug-ins that
only receive device pointers from a host framework's memory pool.  The entry point
takes the caller's device buffers and keeps its scratch in a fixed array of the
library (n <= 8192), so these tests give it torch-allocated device buffers and check
it against the allocating entry point, sg_coulomb_accel, on two calls in a row and on
the sizes where its block layout changes (one ion, fewer than a 32-ion pad, one
j-chunk to two, a partial last i-block).

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
TOL = 1e-12  # the FP64 form's per-ion relative tolerance


def ptr(t):
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


def call_noalloc(pos, q, kq, null=None):
    n = len(q)
    dev = dict(
        pos=torch.tensor(pos, dtype=torch.float64, device="cuda"),
        q=torch.tensor(q, dtype=torch.float64, device="cuda"),
        kq=torch.tensor(kq, dtype=torch.float64, device="cuda"),
        acc=torch.full((max(n, 1), 3), float("nan"), dtype=torch.float64, device="cuda"),
    )
    args = {k: (None if k == null else v) for k, v in dev.items()}
    stream = torch.cuda.current_stream()
    st = abi.load().sg_coulomb_accel_noalloc(n, ptr(args["pos"]), ptr(args["q"]),
                                             ptr(args["kq"]), ptr(args["acc"]),
                                             ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return st, dev["acc"].cpu().numpy()[:n]


def cloud(n, seed):
    c = configs.gaussian_cloud(configs.rng_for(seed), n, 5e-4, 300.0, np.full(n, 132.905))
    q = c.charge.astype(np.float64)
    q[::5] = 2.0
    kq = KE * EL_CHARGE * q * EL_CHARGE / c.mass
    return c.pos, q, kq


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def check_against_allocating(ctx, n, seed):
    pos, q, kq = cloud(n, seed)
    st, acc = call_noalloc(pos, q, kq)
    assert st == abi.SG_OK
    if n == 1:
        assert np.all(acc == 0.0)  # the self pair is excluded: no force at all
        return
    ref = ctx.coulomb_accel(pos, q, kq, abi.SG_PREC_FP64)
    e = np.linalg.norm(acc - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert e.max() <= TOL, (n, float(e.max()))


def test_two_calls_match_allocating_entry_point(ctx):
    # two calls in a row: the second reuses the scratch the first left behind
    for n, seed in ((3000, 1), (MAX_IONS, 2)):
        check_against_allocating(ctx, n, seed)


@pytest.mark.parametrize("n", [1, 2, 31, 33, 257, 511, 513])
def test_edge_sizes_match_allocating_entry_point(ctx, n):
    check_against_allocating(ctx, n, 10 + n)


def test_rejects_sizes_beyond_capacity():
    pos, q, kq = cloud(MAX_IONS + 1, 3)
    st, acc = call_noalloc(pos, q, kq)
    assert st == abi.SG_TOO_LARGE
    assert np.isnan(acc).all()  # nothing was written


def test_zero_ions_and_null_pointers():
    pos, q, kq = cloud(64, 4)
    st, _ = call_noalloc(pos[:0], q[:0], kq[:0])
    assert st == abi.SG_OK
    for name in ("pos", "q", "kq", "acc"):
        st, acc = call_noalloc(pos, q, kq, null=name)
        assert st == abi.SG_BAD_ARG, name
        assert np.isnan(acc).all(), name  # nothing was queued
