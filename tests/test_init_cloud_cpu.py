"""Initial-cloud generator (sg_init_cloud, host side of libsimgb) against golden vectors
made by the reference's own InitCloud (bin/initialization.cpp:117-206), compiled from its
sources (tests/golden/make_golden.py).  Bit for bit on the machine the goldens were made
on (x86-64 glibc); elsewhere libm's last-bit differences in log/acos/sin/cos may show,
so other machines compare to 1e-14."""
import os
import platform

import numpy as np
import pytest

from simbuca_gb300 import abi
from simbuca_gb300.api import init_cloud

GOLD = os.path.join(os.path.dirname(__file__), "golden")
EXACT = platform.machine() in ("x86_64", "AMD64")


@pytest.mark.parametrize("tag", ["a", "b"])
def test_init_cloud_matches_reference(tag):
    g = np.load(os.path.join(GOLD, "init_cloud.npz"))
    n = int(g[f"{tag}_n"])
    pos, vel = init_cloud(n, g[f"{tag}_ev"], int(g[f"{tag}_seed"]), g[f"{tag}_semi"],
                          g[f"{tag}_off"], g[f"{tag}_mass"])
    if EXACT:
        assert np.array_equal(pos, g[f"{tag}_pos"])
        assert np.array_equal(vel, g[f"{tag}_vel"])
    else:
        np.testing.assert_allclose(pos, g[f"{tag}_pos"], rtol=1e-14, atol=1e-20)
        np.testing.assert_allclose(vel, g[f"{tag}_vel"], rtol=1e-14, atol=1e-12)


def test_init_cloud_geometry():
    """Every ion inside its ellipsoid; the draw is uniform (mean radius^2 = 3/5)."""
    semi = np.array([1e-3, 2e-3, 3e-3])
    off = np.array([1e-4, 0.0, -2e-4])
    pos, vel = init_cloud(20000, [0.3], 99, semi, off, 132.905 * 1.6605402e-27)
    r2 = (((pos - off) / semi) ** 2).sum(1)
    assert r2.max() <= 1.0 + 1e-12
    assert abs(r2.mean() - 0.6) < 0.01
    assert np.isfinite(vel).all()


def test_init_cloud_bad_arguments():
    L = abi.load()
    assert L.sg_init_cloud(-1, None, 1, 0, None, None, None, None, None) == abi.SG_BAD_ARG
    e = np.ones(3)
    assert L.sg_init_cloud(1, abi.dptr(e), 3, 0, abi.dptr(e), abi.dptr(e), abi.dptr(e),
                           abi.dptr(e), abi.dptr(e)) == abi.SG_BAD_ARG
