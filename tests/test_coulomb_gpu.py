"""Coulomb sum on the GPU (sg_coulomb_accel) against the CPU oracle and the reference's
golden vectors.  Per-ion relative error |a - a_ref| / |a_ref|:
FP64 plain form <= 1e-12, FP32-compensated form <= 1e-6."""
import os

import numpy as np
import pytest

import oracle
from simbuca_gb300 import abi, configs
from simbuca_gb300.abi import SG_PREC_FP32C, SG_PREC_FP64
from helpers import kq_of, rel_err_per_ion, summary

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = {SG_PREC_FP64: 1e-12, SG_PREC_FP32C: 1e-6}


@pytest.fixture(scope="module", autouse=True)
def _oracle():
    oracle.build()
    oracle.set_threads(os.cpu_count() or 4)


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_golden_1k(ctx, prec):
    g = np.load(os.path.join(GOLD, "force_1k.npz"))
    kq = kq_of(g["mass"], g["charge"])
    a = ctx.coulomb_accel(g["pos"], g["charge"].astype(np.float64), kq, prec)
    e = rel_err_per_ion(a, g["f_coulomb"])
    print(prec, summary(e))
    assert e.max() <= TOL[prec]


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
@pytest.mark.parametrize("n", [2, 3, 31, 32, 33, 127, 129, 511, 513, 1000, 4097])
def test_sizes(ctx, prec, n):
    rng = np.random.default_rng(n)
    pos = rng.normal(0, 4e-4, (n, 3)) + np.array([1e-4, -2e-4, 3e-5])
    q = np.ones(n)
    kq = kq_of(np.full(n, 132.905 * oracle.AMU), q)
    ref = oracle.coulomb_kq(pos, q, kq)
    a = ctx.coulomb_accel(pos, q, kq, prec)
    e = rel_err_per_ion(a, ref)
    assert e.max() <= TOL[prec], (n, summary(e))


@pytest.mark.parametrize("prec", [SG_PREC_FP64, SG_PREC_FP32C])
def test_mixed_charges_and_offset(ctx, prec):
    g = np.load(os.path.join(GOLD, "force_mixed.npz"))
    pos = g["pos"] + np.array([5e-3, -3e-3, 1e-2])  # cloud far from the origin
    q = g["charge"].astype(np.float64)
    q[5::7] = -1.0
    kq = kq_of(g["mass"], q, 0.75)
    ref = oracle.coulomb_kq(pos, q, kq)
    a = ctx.coulomb_accel(pos, q, kq, prec)
    e = rel_err_per_ion(a, ref)
    assert e.max() <= TOL[prec], summary(e)


def test_single_ion_is_zero(ctx):
    for prec in (SG_PREC_FP64, SG_PREC_FP32C):
        a = ctx.coulomb_accel(np.array([[1e-3, 2e-3, 3e-3]]), np.ones(1), np.ones(1), prec)
        assert np.all(a == 0.0)


def test_deterministic(ctx):
    w = configs.penning_1k(n=3000)
    c = w.clouds[0]
    kq = kq_of(c.mass, c.charge)
    for prec in (SG_PREC_FP64, SG_PREC_FP32C):
        a = ctx.coulomb_accel(c.pos, c.charge.astype(np.float64), kq, prec)
        b = ctx.coulomb_accel(c.pos, c.charge.astype(np.float64), kq, prec)
        assert np.array_equal(a, b)


def test_65k_sampled_rows(ctx):
    """The 65,536-ion cloud: oracle rows for random ions, the ions with the closest
    neighbours and the ions nearest the centre (where the relative error is worst)."""
    c = configs.penning_65k().clouds[0]
    n = len(c.mass)
    q = c.charge.astype(np.float64)
    kq = kq_of(c.mass, q)
    r2 = (c.pos ** 2).sum(1)
    rng = np.random.default_rng(0)
    # closest pairs through a coarse grid sort (no scipy on every machine)
    order = np.lexsort(np.floor(c.pos / 2e-5).T)
    d = np.linalg.norm(np.diff(c.pos[order], axis=0), axis=1)
    close = order[np.argsort(d)[:150]]
    rows = np.unique(np.concatenate([rng.choice(n, 300, replace=False), np.argsort(r2)[:150],
                                     close]))
    ref = np.stack([oracle.coulomb_kq_rows(c.pos, q, kq, int(i), int(i) + 1)[0] for i in rows])
    for prec in (SG_PREC_FP64, SG_PREC_FP32C):
        a = ctx.coulomb_accel(c.pos, q, kq, prec)[rows]
        e = rel_err_per_ion(a, ref)
        print(prec, summary(e))
        assert e.max() <= TOL[prec], summary(e)


def test_bad_arguments(ctx):
    L = abi.load()
    assert L.sg_coulomb_accel(ctx.handle, 7, 3, None, None, None, None) == abi.SG_BAD_ARG
    assert L.sg_coulomb_accel(ctx.handle, 0, -1, None, None, None, None) == abi.SG_BAD_ARG


@pytest.mark.parametrize("variant", [4, 7, 8, 9, 12, 13, 14, 15, 16])
@pytest.mark.parametrize("n", [100, 1000, 5000, 20000])
def test_sorted_variant(ctx, n, variant):
    """Ions in k-d tree order, far tile pairs from the high parts only: same accuracy,
    results returned in the caller's order."""
    rng = np.random.default_rng(100 + n)
    pos = rng.normal(0, 6e-4, (n, 3)) + np.array([2e-4, 0.0, -1e-4])
    q = np.ones(n)
    q[::11] = 2.0
    kq = kq_of(np.full(n, 132.905 * oracle.AMU), q)
    rows = np.unique(rng.choice(n, min(n, 600), replace=False))
    ref = np.stack([oracle.coulomb_kq_rows(pos, q, kq, int(i), int(i) + 1)[0] for i in rows])
    ctx.set_coulomb_variant(variant)
    try:
        a = ctx.coulomb_accel(pos, q, kq, SG_PREC_FP32C)[rows]
    finally:
        ctx.set_coulomb_variant(-1)
    e = rel_err_per_ion(a, ref)
    assert e.max() <= 1e-6, summary(e)


@pytest.mark.parametrize("variant", list(range(17)))
@pytest.mark.parametrize("n", [33, 1000, 3000])
def test_every_launch_shape(ctx, variant, n):
    """Every FP32c launch shape (sg_set_coulomb_variant) on small and mid-size clouds."""
    rng = np.random.default_rng(7 * n + variant)
    pos = rng.normal(0, 5e-4, (n, 3))
    q = np.ones(n)
    kq = kq_of(np.full(n, 132.905 * oracle.AMU), q)
    ref = oracle.coulomb_kq(pos, q, kq)
    ctx.set_coulomb_variant(variant)
    try:
        a = ctx.coulomb_accel(pos, q, kq, SG_PREC_FP32C)
    finally:
        ctx.set_coulomb_variant(-1)
    e = rel_err_per_ion(a, ref)
    assert e.max() <= 1e-6, (variant, n, summary(e))


@pytest.mark.parametrize("variant", [5, 9, 13])
@pytest.mark.parametrize("qval", [1.0, 2.0, -1.0, 3.0])
def test_uniform_charge(ctx, qval, variant):
    """Clouds whose ions share one charge hold normalized charges and skip the charge
    product away from the padding tile; 3,001 ions leave padding in the last tile."""
    n = 3001
    rng = np.random.default_rng(int(10 * qval) + variant + 50)
    pos = rng.normal(0, 5e-4, (n, 3))
    q = np.full(n, qval)
    kq = kq_of(np.full(n, 132.905 * oracle.AMU), q)
    ref = oracle.coulomb_kq(pos, q, kq)
    ctx.set_coulomb_variant(variant)
    try:
        a = ctx.coulomb_accel(pos, q, kq, SG_PREC_FP32C)
    finally:
        ctx.set_coulomb_variant(-1)
    e = rel_err_per_ion(a, ref)
    assert e.max() <= 1e-6, (qval, variant, summary(e))


def test_1m_spheroid_rows_and_momentum(ctx):
    """The 1,048,576-ion spheroid at full size (automatic k-d ordered shape): sampled
    oracle rows (random, nearest the centre, closest pairs) to 1e-6, and the pair sum's
    size-independent property -- internal forces cancel: |sum_i m_i a_i| is at the
    rounding level of sum_i |m_i a_i|."""
    w = configs.spheroid_1m()
    c = w.clouds[0]
    n = len(c.mass)
    q = c.charge.astype(np.float64)
    kq = kq_of(c.mass, q)
    a = ctx.coulomb_accel(c.pos, q, kq, SG_PREC_FP32C)
    assert np.isfinite(a).all()
    f = a * c.mass[:, None]
    bal = np.linalg.norm(f.sum(0)) / np.linalg.norm(f, axis=1).sum()
    print("momentum balance", bal)
    assert bal < 1e-7
    rng = np.random.default_rng(1)
    r2 = (c.pos ** 2).sum(1)
    order = np.lexsort(np.floor(c.pos / 2e-6).T)
    d = np.linalg.norm(np.diff(c.pos[order], axis=0), axis=1)
    rows = np.unique(np.concatenate([rng.choice(n, 40, replace=False), np.argsort(r2)[:12],
                                     order[np.argsort(d)[:12]]]))
    ref = np.stack([oracle.coulomb_kq_rows(c.pos, q, kq, int(i), int(i) + 1)[0] for i in rows])
    e = rel_err_per_ion(a[rows], ref)
    print(summary(e))
    assert e.max() <= 1e-6, summary(e)
