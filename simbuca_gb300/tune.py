"""Launch-shape autotuner of the FP32c Coulomb kernel.

    python -m simbuca_gb300.tune [--sizes 1024,8192,65536] [--out table.json]

For every cloud size it times sg_coulomb_accel once per launch shape
(sg_set_coulomb_variant) with CUDA events around the Coulomb kernel and keeps the
fastest; the table maps a cloud size to the variant to use, the GB300 counterpart of
the reference's per-GPU NBODY launch tables (libraries/NBODY/*.dat).
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np

from . import abi, configs
from .api import Context
from .constants import EL_CHARGE, KE

VARIANTS = {0: "128x4", 1: "128x2", 2: "256x2", 3: "64x4", 4: "sorted128x4", 5: "64x2",
            6: "32x4", 7: "sorted32x4", 8: "sorted64x2", 9: "sorted128x1", 10: "32x2",
            11: "32x1", 12: "sorted128x1t256", 13: "sorted64x2t256", 14: "sorted64x2t256u4",
            15: "sorted32x4t256", 16: "sorted64x2t256s4"}
TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")


def time_variant(ctx: Context, pos, q, kq, variant: int, reps: int = 3) -> float:
    ctx.set_coulomb_variant(variant)
    ctx.coulomb_accel(pos, q, kq, abi.SG_PREC_FP32C)  # plan + warm-up
    ctx.set_kernel_timing(True)
    for _ in range(reps):
        ctx.coulomb_accel(pos, q, kq, abi.SG_PREC_FP32C)
    kt = ctx.kernel_timing()
    ctx.set_kernel_timing(False)
    return kt["coulomb_ms"] / max(kt["coulomb_launches"], 1)


def tune(sizes, device: int = 0):
    ctx = Context(device)
    rows = []
    for n in sizes:
        c = configs.gaussian_cloud(configs.rng_for(n), n, 1e-3, 300.0, np.full(n, configs.M_CS))
        q = np.ones(n)
        kq = KE * EL_CHARGE * q * EL_CHARGE / c.mass
        t = {v: time_variant(ctx, c.pos, q, kq, v) for v in VARIANTS}
        best = min(t, key=t.get)
        inter = n * (n - 1)
        rows.append({"n": n, "best": best, "shape": VARIANTS[best],
                     "ms": {VARIANTS[v]: t[v] for v in t},
                     "interactions_per_s": inter / (t[best] * 1e-3)})
    ctx.close()
    return rows


def choose(table, n: int) -> int:
    """Variant for a cloud of n ions: the entry of the nearest tuned size."""
    if not table:
        return 0
    best = min(table, key=lambda r: abs(np.log(r["n"]) - np.log(max(n, 1))))
    return int(best["best"])


def load_table(path: str = TABLE):
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="256,1024,4096,16384,65536,262144")
    ap.add_argument("--out", default=TABLE)
    a = ap.parse_args()
    rows = tune([int(x) for x in a.sizes.split(",")])
    for r in rows:
        print(json.dumps(r))
    with open(a.out, "w") as f:
        json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
