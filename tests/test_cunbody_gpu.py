"""The CUNBODY-compatible slot (bin/cunbody.h:11-33) exported by libsimgb:
ai = sum_j mj (xj - xi) / (|xj - xi|^2 + eps2)^{3/2}, driven as the reference's
_cunbody wrapper does (bin/cunbody.cpp:43-90: xj = xi = pos2, mj = 1, eps2 = 1e-23)."""
import ctypes

import numpy as np
import pytest

from simbuca_gb300 import abi

pytestmark = pytest.mark.gpu


def reference_sum(xj, mj, xi, eps2):
    d = xj[None, :, :] - xi[:, None, :]
    r2 = (d * d).sum(-1) + eps2
    w = np.where(r2 > 0, mj[None, :] / np.where(r2 > 0, r2, 1.0) ** 1.5, 0.0)
    return (d * w[:, :, None]).sum(1)


def call(fn, xj, mj, xi, eps2):
    L = abi.load()
    ai = np.zeros((len(xi), 3))
    getattr(L, fn)(abi.dptr(xj), abi.dptr(mj), abi.dptr(xi), eps2, abi.dptr(ai), len(xi), len(xj))
    return ai


def test_wrapper_usage():
    rng = np.random.default_rng(1)
    n = 700
    x = rng.normal(0, 5e-4, (n, 3))
    m = np.ones(n)
    eps2 = float(np.float32(1e-23))  # the wrapper keeps eps in a float (bin/cunbody.h:49)
    ai = call("cunbody1_force", x, m, x.copy(), eps2)
    ref = reference_sum(x, m, x, eps2)
    np.testing.assert_allclose(ai, ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())


def test_begin_end_distinct_sets():
    rng = np.random.default_rng(2)
    xj = rng.normal(0, 1e-3, (300, 3))
    mj = rng.uniform(0.5, 2.0, 300)
    xi = rng.normal(0, 1e-3, (129, 3))
    L = abi.load()
    ai = np.zeros((129, 3))
    args = (abi.dptr(xj), abi.dptr(mj), abi.dptr(xi), 1e-12, abi.dptr(ai), 129, 300)
    L.cunbody1_force_begin(*args)
    L.cunbody1_force_end(*args)
    ref = reference_sum(xj, mj, xi, 1e-12)
    np.testing.assert_allclose(ai, ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())
