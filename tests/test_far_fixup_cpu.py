"""The far-field fix-up's arithmetic on the CPU (no GPU): for ions near the centre of the
1M-ion uniform spheroid, summing far pairs from the high FP32 parts of the frame
coordinates leaves a relative error above 1e-6 (their net force is small next to the far
terms), and the first-order correction the fix-up kernel adds,
    delta = y3 (D - 3 y^2 (u.D) u),  D = (lo_j - lo_i) + (hi_j - hi_i - fl(hi_j - hi_i)),
with the error-free two-sum, brings it back far below.  numpy float32 emulates the
kernel's FP32 operations; "far" is the pair distance beyond 0.45 frame units here (the
kernel decides per 128-ion tile)."""
import numpy as np
import pytest

from simbuca_gb300 import configs

f32 = np.float32


def two_diff_err(a, b, s):
    bv = (s - a).astype(f32)
    av = (s - bv).astype(f32)
    return ((a - av).astype(f32) + (-b - bv).astype(f32)).astype(f32)


@pytest.fixture(scope="module")
def spheroid():
    pos = configs.spheroid_1m().clouds[0].pos
    cen = pos.mean(0)
    L = np.sqrt(((pos - cen) ** 2).mean(0)).max()
    u = (pos - cen) / L
    hi = u.astype(f32)
    lo = (u - hi.astype(np.float64)).astype(f32)
    return u, hi, lo


def test_far_correction_restores_central_ions(spheroid):
    u, hi, lo = spheroid
    worst_before, worst_after = 0.0, 0.0
    for i in np.argsort((u ** 2).sum(1))[2:6]:
        d = u - u[i]
        rr = np.sqrt((d ** 2).sum(1))
        rr[i] = np.inf
        exact = (d / rr[:, None] ** 3).sum(0)
        far = rr > 0.45
        U = (hi - hi[i]).astype(f32)
        r2 = ((U.astype(np.float64) ** 2).sum(1) + 1e-24).astype(f32)
        y = (1.0 / np.sqrt(r2.astype(np.float64))).astype(f32)
        y3 = (y * y * y).astype(f32)
        main = np.where(far[:, None], y3[:, None].astype(np.float64) * U, d / rr[:, None] ** 3).sum(0)
        D = ((lo - lo[i]).astype(f32) + two_diff_err(hi, hi[i], U)).astype(f32)
        ud = (U * D).sum(1).astype(f32)
        s3 = (f32(3) * y * y * ud).astype(f32)
        delta = (y3[:, None] * (D - s3[:, None] * U)).astype(f32)
        corr = np.where(far[:, None], delta.astype(np.float64), 0.0).sum(0)
        n = np.linalg.norm(exact)
        worst_before = max(worst_before, np.linalg.norm(main - exact) / n)
        worst_after = max(worst_after, np.linalg.norm(main + corr - exact) / n)
    print("before", worst_before, "after", worst_after)
    assert worst_before > 1e-6      # the case the fix-up exists for
    assert worst_after < 5e-8
