"""Benchmark of the Simbuca hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload penning_65k] [--precision fp32c|fp64]

Workload (default): 65,536 singly charged ions, 50/50 132.905/132.906 u, Gaussian
sigma 1 mm, 300 K, seed 1, ideal Penning trap (7 T, 10 V, d0 1 cm), quadrupole drive
0.5 V at the mass-weighted nu_c, friction delta 1e3 /s, Dormand-Prince rtol 1e-9.
A step is one accepted Dormand-Prince step of the whole cloud (all its attempts).
Metric: simulated microseconds per wall second (higher is better).

Our arm (FP32-compensated Coulomb, device-resident state, CUDA-graph attempts):
value = device-timed rate with the state resident in HBM; e2e = the same through the
public C ABI with the state uploaded from pinned host memory and read back every
step.  Kernel times (roofline: the Coulomb kernel; stage_roofline: the O(N) kernels)
come from a second pass of as many steps with CUDA events around those launches.  The
plain FP64 GPU form is timed on the same cloud for comparison.  Rank 0 also times the
CPU oracle on a bounded row sample (cpu_baseline).  Step control is the reference's
I-controller; --proposer on runs the learned step-size proposer instead.

Reference arm (--impl reference): the CPU oracle (the reference's FP64 direct sum and
Dormand-Prince loop restated in C, oracle/) on all host cores, full attempts of the
same workload.  N > 1 runs independent replicas (one cloud per GPU).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_PER_INTERACTION = 20  # convention of bin/nbody_kernel.cu:186-211


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="penning_65k")
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sequential", action="store_true",
                    help="batched workloads: skip the one-cloud-at-a-time comparison pass")
    ap.add_argument("--variant", type=int, default=-1,
                    help="FP32c Coulomb launch shape (-1 automatic, 0..16 fixed: sg_set_coulomb_variant)")
    ap.add_argument("--method", type=int, default=5, choices=[4, 5],
                    help="5 Dormand-Prince, 4 Cash-Karp")
    ap.add_argument("--proposer", default="off", choices=["on", "off"],
                    help="the reference's controller (default) or the learned step-size "
                         "proposer with the shipped weights")
    ap.add_argument("--beta", type=float, default=0.0,
                    help="beta of the controller's PI form (bin/ode.cpp:428-439) in both arms; "
                         "0 is the reference's compiled I-controller")
    ap.add_argument("--proposer-safety", type=float, default=None,
                    help="safety factor of the proposer (default: the trained one's)")
    ap.add_argument("--fused", default="auto", choices=["auto", "on", "off"],
                    help="fused small-cloud path: automatic (clouds of up to 512 ions), on "
                         "(up to 2,048: sg_set_fused 2) or off")
    ap.add_argument("--settle", type=int, default=60,
                    help="at most this many steps to let the step size settle before warm-up")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only: no data-path collective)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self, n_gpus):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def l2_flush():
    """Write a buffer larger than the 129 MB L2 between timed steps."""
    import torch
    if not hasattr(l2_flush, "buf"):
        l2_flush.buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    l2_flush.buf.zero_()
    torch.cuda.synchronize()


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def coulomb_kernel_name(prec, variant):
    from simbuca_gb300 import abi
    if prec != abi.SG_PREC_FP32C:
        return "coulomb_fp64_kernel"
    sorted_shapes = (4, 7, 8, 9, 12, 13, 14, 15, 16)
    return "coulomb_fp32c_sorted_kernel" if variant in sorted_shapes else "coulomb_fp32c_kernel"


# Algorithmic HBM traffic of one Dormand-Prince attempt per ion in the O(N) kernels:
# stage s = 1..6 combines read y and k_1..k_s and write y_s (48(s+2) B), the final
# combine with the error norm moves 384 B (FP64 SoA, 48 B per 6-vector).
STAGE_BYTES_PER_ION = 48 * sum(s + 2 for s in range(1, 7)) + 384  # 1968


def stage_roofline(args, w, st, attempts):
    """The O(N) kernels of the kernel-timing pass (7 stage combines, control, commit):
    algorithmic bytes / event-timed duration against the measured HBM copy rate."""
    if args.method != 5 or not st["stage_ms"] or not attempts:
        return None
    peak = None
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        src = "MEASURED_PEAKS.json hbm_gbs (measured copy)"
    except (OSError, ValueError, KeyError):
        peak, src = 6800.0, "fallback 6.8 TB/s"
    byts = STAGE_BYTES_PER_ION * w.n_total * attempts
    achieved = byts / (st["stage_ms"] * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "bytes_per_ion_attempt": STAGE_BYTES_PER_ION,
            "launches": st["stage_launches"], "ms": st["stage_ms"], "peak_source": src,
            "note": ("per-attempt working set below the 129 MB L2: reads partly from L2"
                     if STAGE_BYTES_PER_ION * w.n_total < 129e6 else
                     "per-attempt working set above the 129 MB L2")
            + "; these kernels are bound by the FP64 pipe first (~80 FP64 operations "
              "per ion and stage)"}


def settled(hist_h) -> bool:
    """The step size has settled once three successive accepted steps changed it by
    less than 10 % each (the controller starts at h0 = 1 ns and grows h by up to 10x)."""
    return len(hist_h) >= 4 and all(abs(hist_h[-k] / hist_h[-k - 1] - 1) < 0.1
                                    for k in (1, 2, 3))


def check_summary(records, every):
    """The in-run FP32c force check (sg_batch_force_check) over every cloud."""
    if not records or not any(r["checks"] for r in records):
        return None
    return {"every_attempts": every,
            "checks": int(sum(r["checks"] for r in records)),
            "probes": int(sum(r["probes"] for r in records)),
            "breaches_above_1e-6": int(sum(r["breaches"] for r in records)),
            "max_err": max(r["max_err"] for r in records),
            "max_err_far_near_random": [max(r["max_err_far"] for r in records),
                                        max(r["max_err_near"] for r in records),
                                        max(r["max_err_random"] for r in records)],
            "c_far_max": max(r["c_far"] for r in records),
            "kfar_min": min(r["kfar"] for r in records),
            "kfar_prior_min": min(r["kfar_prior"] for r in records),
            "what": "per-ion relative Coulomb error of 8 probe ions per cloud (largest far and "
                    "near conditioning ratios without fix-up, and 4 random) against their FP64 "
                    "rows, every few attempts of the whole run"}


CHECK_EVERY = 16  # the library's default interval of the in-run force check


def controller_name(args) -> str:
    if args.beta > 0.0:
        return f"PI controller, beta {args.beta:g} (bin/ode.cpp:428-439)"
    return "reference I-controller (bin/ode.cpp:426-457)"


def apply_step_control(args, batch) -> str:
    """The learned proposer with the shipped weights (every attempt still accepted or
    rejected by the Dormand-Prince error estimate), or the reference's I-controller."""
    if args.proposer == "off":
        return controller_name(args)
    from simbuca_gb300 import proposer
    s = args.proposer_safety if args.proposer_safety is not None else proposer.DEFAULT_SAFETY
    batch.set_proposer(proposer.default_weights(), s)
    return f"learned proposer, safety {s}"


def run_ours(args, dist: Dist):
    import torch
    from simbuca_gb300 import abi, configs
    from simbuca_gb300.api import Batch, Context

    torch.cuda.set_device(dist.local)
    w = configs.WORKLOADS[args.workload]()
    allc = w.concat()
    prec = abi.SG_PREC_FP32C if args.precision == "fp32c" else abi.SG_PREC_FP64
    for o in w.odes:
        o.method = args.method
        o.beta = args.beta
    ctx = Context(dist.local)
    if args.variant >= 0:
        ctx.set_coulomb_variant(args.variant)
    ctx.set_fused({"auto": 1, "on": 2, "off": 0}[args.fused])
    peaks = ctx.probe_peaks()
    batch = Batch(ctx, w.counts, w.fields, w.odes, prec)
    batch.upload(allc.pos, allc.vel, allc.mass, allc.charge)
    step_control = apply_step_control(args, batch)

    def info0():
        return batch.info()

    # Settle: the controller starts from h0 = 1 ns and grows h by up to 10x per step;
    # the workload's rate is quoted at the step size it settles at (at most 60 steps).
    hist_h = []
    for _ in range(args.settle):
        info, _ = batch.step()
        hist_h.append(info[0]["h_last"])
        if settled(hist_h):
            break
    snap_pos, snap_vel = batch.download()
    snap = info0()
    settle_steps = len(hist_h)
    for _ in range(args.warmup):
        batch.step()
    # the kernel-timing pass and the end-to-end pass restart from this state, so that
    # all three passes integrate the same stretch of the trajectory
    seg_pos, seg_vel = batch.download()
    s_before = info0()

    # ---- device-resident timed region -------------------------------------
    ctx.fixup_count()  # reset the FP32c conditioning fix-up counter
    ctx.set_kernel_timing(False)
    clocks = ClockSampler(dist.local)
    dist.barrier()
    torch.cuda.synchronize()
    ctx.sync()
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        l2_flush()
        ctx.timer_start()
        batch.step()
        step_ms.append(ctx.timer_stop())
    ctx.sync()
    clk = clocks.stop()
    dist.barrier()
    s_after = info0()
    fixups = ctx.fixup_count()
    total_ms = sum(step_ms)
    checks = check_summary(batch.force_check(), CHECK_EVERY) if prec == abi.SG_PREC_FP32C else None

    # ---- Coulomb kernel timing: a second pass of as many steps with CUDA events
    # around every Coulomb launch (the events and their host reads stay out of the
    # timed region above)
    batch.set_state(seg_pos, seg_vel)
    ctx.set_kernel_timing(True)
    kt_ms = []
    k_before = info0()
    for _ in range(args.steps):
        l2_flush()
        ctx.timer_start()
        batch.step()
        kt_ms.append(ctx.timer_stop())
    ctx.sync()
    kt = ctx.kernel_timing()
    st = ctx.stage_timing()
    ft = ctx.fused_timing()
    ctx.set_kernel_timing(False)
    fused_cluster = batch.fused()
    kt_total_ms = sum(kt_ms)
    kt_attempts = sum((a["steps"] + a["rejects"]) - (b["steps"] + b["rejects"])
                      for a, b in zip(info0(), k_before))
    sim_us = sum(a["t"] - b["t"] for a, b in zip(s_after, s_before)) * 1e6
    attempts = sum((a["steps"] + a["rejects"]) - (b["steps"] + b["rejects"])
                   for a, b in zip(s_after, s_before))
    max_ms = dist.max(total_ms)
    sim_us_all = dist.sum(sim_us)
    value = sim_us_all / (max_ms * 1e-3)

    # ---- end to end through the C ABI with pinned host buffers -----------
    pos_h = torch.empty((w.n_total, 3), dtype=torch.float64, pin_memory=True).numpy()
    vel_h = torch.empty((w.n_total, 3), dtype=torch.float64, pin_memory=True).numpy()
    pos_h[:] = seg_pos
    vel_h[:] = seg_vel
    e2e_ms = []
    parts = np.zeros(3)
    e_before = info0()
    dist.barrier()
    for _ in range(args.steps):
        l2_flush()
        t0 = time.perf_counter()
        batch.set_state(pos_h, vel_h)      # H2D of the step's input state
        t1 = time.perf_counter()
        batch.step()
        t2 = time.perf_counter()
        batch.download(pos_h, vel_h)       # D2H of the step's result
        t3 = time.perf_counter()
        e2e_ms.append((t3 - t0) * 1e3)
        parts += np.array([t1 - t0, t2 - t1, t3 - t2]) * 1e3
    e_after = info0()
    e2e_sim = dist.sum(sum(a["t"] - b["t"] for a, b in zip(e_after, e_before)) * 1e6)
    e2e_val = e2e_sim / (dist.max(sum(e2e_ms)) * 1e-3)
    bytes_state = 2 * w.n_total * 3 * 8

    # ---- roofline of the Coulomb kernel -----------------------------------
    if fused_cluster:
        # the fused small-cloud kernel: whole attempts (Coulomb sums and stages) per
        # launch; achieved counts the Coulomb flops of the timing pass's attempts only
        inter_pass = 6.0 * kt_attempts * sum(float(n) * (n - 1) for n in w.counts)
        kt = {"coulomb_ms": ft["ms"], "coulomb_launches": ft["launches"],
              "interactions": inter_pass}
    per_launch_inter = kt["interactions"] / max(kt["coulomb_launches"], 1)
    avg_launch_s = kt["coulomb_ms"] * 1e-3 / max(kt["coulomb_launches"], 1)
    achieved = FLOPS_PER_INTERACTION * per_launch_inter / avg_launch_s / 1e12
    if prec == abi.SG_PREC_FP32C:
        peak = max(peaks["fp32_gflops"], peaks["fp32x2_gflops"]) / 1e3
    else:
        peak = peaks["fp64_gflops"] / 1e3
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            for key in (f"{args.workload}:{args.precision}:{batch.variant()}",
                        f"{args.workload}:{args.precision}"):
                if key in tj:
                    traffic = tj[key]["dram_bytes_per_launch"]
                    break
        except (ValueError, KeyError):
            traffic = None

    out = {
        "metric": "sim-us/wall-s (Coulomb + Penning field + Dormand-Prince, one cloud per GPU)",
        "value": value,
        "unit": "sim-us/wall-s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": max_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32c+fp64" if prec == abi.SG_PREC_FP32C else "fp64",
        "data": "synthetic (seeded Gaussian cloud, Maxwell-Boltzmann velocities)",
        "config": {"workload": args.workload, "ions": w.n_total, "clouds": len(w.counts),
                   "precision": args.precision, "rtol": 1e-9, "atol": 1e-15,
                   "parallelism": f"replicas x{dist.world}",
                   "l2": "flushed (256 MB write) between timed steps",
                   "settle_steps": settle_steps, "h_settled": snap[0]["h"],
                   "method": "dormand-prince" if args.method == 5 else "cash-karp",
                   "step_control": step_control,
                   "coulomb_variant": batch.variant(),
                   "fused_cluster": fused_cluster},
        "e2e": {"value": e2e_val, "unit": "sim-us/wall-s", "h2d_bytes_per_step": bytes_state,
                "d2h_bytes_per_step": bytes_state, "ms_per_step": sum(e2e_ms) / args.steps,
                "ms_upload_step_download": (parts / args.steps).tolist(),
                "mean_h": sum(a["t"] - b["t"] for a, b in zip(e_after, e_before)) /
                max(1, sum(a["steps"] - b["steps"] for a, b in zip(e_after, e_before)))},
        "mean_h": sim_us * 1e-6 / max(1, sum(a["steps"] - b["steps"] for a, b in zip(s_after, s_before))),
        # per attempt: 7 stages, 6 Coulomb sums, 6 reductions, control, commit, and with
        # FP32c on batches over 8,192 ions the 6 fix-up launches of the conditioning work
        # list (smaller batches fix up inside the reduction); per step one hold reset
        # (+2 per attempt with the proposer: cloud moments and the MLP)
        # fused small-cloud path: one launch per step (its attempts inside it)
        "gpu_launches": int((args.steps if fused_cluster else
                             attempts * ((27 if prec == abi.SG_PREC_FP32C and w.n_total > 8192
                                          else 21) + (2 if args.proposer == "on" else 0)))
                            + args.steps
                            + (3 * (attempts // CHECK_EVERY) if prec == abi.SG_PREC_FP32C else 0)),
        "fixup_ions_per_coulomb_call": fixups / max(1, 6 * attempts),
        "force_check": checks,
        "attempts": int(attempts),
        "interactions_per_s": kt["interactions"] / (kt["coulomb_ms"] * 1e-3) if kt["coulomb_ms"] else None,
        "roofline": {"bound": "fp32" if prec == abi.SG_PREC_FP32C else "fp64",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "kernel": ("fused_attempts_kernel (cluster of %d CTAs per cloud; whole "
                                "attempts, Coulomb flops counted)" % fused_cluster
                                if fused_cluster else coulomb_kernel_name(prec, batch.variant())),
                     "flops_per_interaction": FLOPS_PER_INTERACTION,
                     "peak_source": "measured in-run by FMA issue probes (sg_probe_peaks)",
                     "coulomb_share_of_step": kt["coulomb_ms"] / kt_total_ms if kt_total_ms else None,
                     "timing_pass": {"steps": args.steps, "attempts": int(kt_attempts),
                                     "ms": kt_total_ms}},
        "stage_roofline": stage_roofline(args, w, st, kt_attempts),
        "peaks_measured": {k: v / 1e3 for k, v in peaks.items()},
        "clocks": clk,
    }

    # ---- accuracy of this run against the FP64 form, and the plain FP64 rate ----
    if not args.no_fp64_compare and prec == abi.SG_PREC_FP32C:
        q = allc.charge.astype(np.float64)
        from simbuca_gb300.constants import EL_CHARGE, KE
        kq = KE * EL_CHARGE * q * EL_CHARGE / allc.mass
        a32 = ctx.coulomb_accel(allc.pos, q, kq, abi.SG_PREC_FP32C)
        a64 = ctx.coulomb_accel(allc.pos, q, kq, abi.SG_PREC_FP64)
        e = np.linalg.norm(a32 - a64, axis=1) / np.linalg.norm(a64, axis=1)
        tot64 = ctx.force(allc.pos, allc.vel, allc.mass, allc.charge, 0.0, w.fields[0],
                          abi.SG_PREC_FP64) if len(w.counts) == 1 else None
        out["force_err_vs_fp64"] = {"coulomb_max": float(e.max()),
                                    "coulomb_p99": float(np.percentile(e, 99)),
                                    "coulomb_median": float(np.median(e))}
        if tot64 is not None:
            tot32 = ctx.force(allc.pos, allc.vel, allc.mass, allc.charge, 0.0, w.fields[0],
                              abi.SG_PREC_FP32C)
            et = np.linalg.norm(tot32 - tot64, axis=1) / np.linalg.norm(tot64, axis=1)
            out["force_err_vs_fp64"]["total_max"] = float(et.max())
        # plain FP64 GPU form and a second FP32c run, both from the settled snapshot
        # (same state, time and step size), each on its own context
        from simbuca_gb300.configs import ode as mk_ode
        odes = [mk_ode(o.rtol, o.atol, s["h"], o.t_end, t0=s["t"], beta=args.beta)
                for o, s in zip(w.odes, snap)]
        n64 = max(2, min(args.steps, 4))
        runs = {}
        for tag, pr in (("fp64", abi.SG_PREC_FP64), ("fp32c", abi.SG_PREC_FP32C)):
            cx = Context(dist.local)
            cx.set_fused({"auto": 1, "on": 2, "off": 0}[args.fused])
            bb = Batch(cx, w.counts, w.fields, odes, pr)
            bb.upload(snap_pos, snap_vel, allc.mass, allc.charge)
            bb.step()  # untimed: captures and instantiates the attempt graph
            i0 = bb.info()
            cx.timer_start()
            for _ in range(n64):
                bb.step()
            ms = cx.timer_stop()
            i1 = bb.info()
            pp, vv = bb.download()
            sim = sum(a["t"] - b["t"] for a, b in zip(i1, i0)) * 1e6
            runs[tag] = (sim / (ms * 1e-3), ms / n64, pp, vv, i1)
            cx.close()
        out["plain_fp64"] = {"value": runs["fp64"][0], "unit": "sim-us/wall-s", "steps": n64,
                             "ms_per_step": runs["fp64"][1]}
        out["speedup_vs_plain_fp64"] = value / runs["fp64"][0]
        p32, v32, p64, v64 = runs["fp32c"][2], runs["fp32c"][3], runs["fp64"][2], runs["fp64"][3]
        out["state_err_vs_fp64"] = {
            "steps": n64,
            "t_fp32c": runs["fp32c"][4][0]["t"], "t_fp64": runs["fp64"][4][0]["t"],
            "pos_max_rel": float(np.abs(p32 - p64).max() / np.abs(p64).max()),
            "vel_max_rel": float(np.abs(v32 - v64).max() / np.abs(v64).max())}

    # ---- CPU baseline: the oracle on a bounded row sample ----------------
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_sample(w, allc, s_before, s_after)
    ctx.close()
    return out


# ---------------------------------------------------------------------------
# our arm, many clouds: one batch advanced by graph-replayed attempts
# ---------------------------------------------------------------------------
def run_batched(args, dist: Dist):
    import torch
    from simbuca_gb300 import abi, configs
    from simbuca_gb300.api import Batch, Context
    from simbuca_gb300.configs import ode as mk_ode

    torch.cuda.set_device(dist.local)
    w = configs.WORKLOADS[args.workload]()
    allc = w.concat()
    prec = abi.SG_PREC_FP32C if args.precision == "fp32c" else abi.SG_PREC_FP64
    for o in w.odes:
        o.beta = args.beta
    ctx = Context(dist.local)
    if args.variant >= 0:
        ctx.set_coulomb_variant(args.variant)
    ctx.set_fused({"auto": 1, "on": 2, "off": 0}[args.fused])
    batch = Batch(ctx, w.counts, w.fields, w.odes, prec)
    batch.upload(allc.pos, allc.vel, allc.mass, allc.charge)
    step_control = apply_step_control(args, batch)
    per_step = 10  # attempts of every cloud per bench step (one graph replay each)

    def tsum(info):
        return sum(x["t"] for x in info)

    # settle: the step sizes start at 1 ns and grow by <= 10x per accepted step
    for _ in range(max(1, args.settle // 10)):
        batch.attempts(per_step)
    batch.info()
    snap_pos, snap_vel = batch.download()
    snap = batch.info()
    for _ in range(args.warmup):
        batch.attempts(per_step)
    s_before = batch.info()
    ctx.set_kernel_timing(False)
    clocks = ClockSampler(dist.local)
    dist.barrier()
    ctx.sync()
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        l2_flush()
        ctx.timer_start()
        batch.attempts(per_step)
        step_ms.append(ctx.timer_stop())
    clk = clocks.stop()
    s_after = batch.info()
    total_ms = sum(step_ms)
    checks = check_summary(batch.force_check(), CHECK_EVERY) if prec == abi.SG_PREC_FP32C else None
    sim_us = (tsum(s_after) - tsum(s_before)) * 1e6
    attempts = sum((a["steps"] + a["rejects"]) - (b["steps"] + b["rejects"])
                   for a, b in zip(s_after, s_before))
    value = dist.sum(sim_us) / (dist.max(total_ms) * 1e-3)

    # the same clouds one at a time, from the same settled state and step sizes
    seq_ms, seq_sim = 0.0, 0.0
    off = 0
    for k, n in enumerate([] if args.no_sequential else w.counts):
        o = w.odes[k]
        op = mk_ode(o.rtol, o.atol, snap[k]["h"], o.t_end, t0=snap[k]["t"], beta=args.beta)
        b1 = Batch(ctx, [n], [w.fields[k]], [op], prec)
        sl = slice(off, off + n)
        b1.upload(snap_pos[sl], snap_vel[sl], allc.mass[sl], allc.charge[sl])
        apply_step_control(args, b1)
        b1.attempts(1)  # untimed: captures and instantiates the attempt graph
        i0 = b1.info()
        ctx.timer_start()
        b1.attempts(per_step * args.steps)
        seq_ms += ctx.timer_stop()
        seq_sim += (b1.info()[0]["t"] - i0[0]["t"]) * 1e6
        off += n
    seq_value = seq_sim / (seq_ms * 1e-3) if seq_ms else None
    out = {
        "metric": "summed sim-us/wall-s over the clouds of a batched frequency scan",
        "value": value, "unit": "sim-us/wall-s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dist.max(total_ms) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32c+fp64" if prec == abi.SG_PREC_FP32C else "fp64",
        "data": "synthetic (seeded Gaussian clouds, Maxwell-Boltzmann velocities)",
        "config": {"workload": args.workload, "ions": w.n_total, "clouds": len(w.counts),
                   "precision": args.precision, "attempts_per_step": per_step,
                   "step_control": step_control,
                   "parallelism": f"replicas x{dist.world}",
                   "l2": "flushed (256 MB write) between timed steps"},
        "gpu_launches": int(((27 if args.precision == "fp32c" else 21)
                             + (2 if args.proposer == "on" else 0)) * per_step * args.steps
                            + (3 * (per_step * args.steps // CHECK_EVERY)
                               if args.precision == "fp32c" else 0)),
        "attempts": int(attempts),
        "force_check": checks,
        "coulomb_interactions_per_s": sum(
            6.0 * n * (n - 1) * ((a["steps"] + a["rejects"]) - (b["steps"] + b["rejects"]))
            for n, a, b in zip(w.counts, s_after, s_before)) / (total_ms * 1e-3),
        "one_at_a_time": {"value": seq_value, "unit": "sim-us/wall-s",
                          "ms_total": seq_ms, "sim_us_total": seq_sim},
        "speedup_vs_one_at_a_time": value / seq_value if seq_value else None,
        "coulomb_variant": batch.variant(),
        "clocks": clk,
    }
    ctx.close()
    return out



def cpu_baseline_sample(w, allc, s_before, s_after, target_s=15.0):
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    n = w.n_total
    q = allc.charge.astype(np.float64)
    from simbuca_gb300.constants import EL_CHARGE, KE
    kq = KE * EL_CHARGE * q * EL_CHARGE / allc.mass
    rows = min(n, 256)
    t0 = time.perf_counter()
    oracle.coulomb_kq_rows(allc.pos, q, kq, 0, rows)
    dt = time.perf_counter() - t0
    # grow the sample to ~target_s of CPU work
    rows = int(min(n, max(rows, rows * target_s / max(dt, 1e-3))))
    rows = max(cores, rows // cores * cores)
    t0 = time.perf_counter()
    oracle.coulomb_kq_rows(allc.pos, q, kq, 0, rows)
    dt = time.perf_counter() - t0
    rate = rows * (n - 1) / dt  # interactions/s
    steps = sum(a["steps"] - b["steps"] for a, b in zip(s_after, s_before))
    attempts = sum((a["steps"] + a["rejects"]) - (b["steps"] + b["rejects"])
                   for a, b in zip(s_after, s_before))
    sim_s = sum(a["t"] - b["t"] for a, b in zip(s_after, s_before))
    inter_per_attempt = 7 * w.interactions_per_force()
    cpu_s = attempts * inter_per_attempt / rate
    return {"value": sim_s * 1e6 / cpu_s, "unit": "sim-us/wall-s", "cores": cores, "kind": "port",
            "interactions_per_s": rate,
            "sample": (f"oracle FP64 Coulomb rows 0..{rows} of {n} ({dt:.1f} s on {cores} threads); "
                       f"extrapolated to this run's {attempts} attempts ({steps} steps, "
                       f"7 force calls each, the reference count)")}


# ---------------------------------------------------------------------------
# reference arm: the CPU oracle on all host cores
# ---------------------------------------------------------------------------
REF_TIME_CAP_S = 60.0  # the reference arm's timed steps stop once this much time has passed


def run_reference(args, dist: Dist):
    """The CPU oracle's full Dormand-Prince steps of the workload's (first) cloud on all
    host threads.  Like our arm it first lets the step size settle by the same rule and
    takes the same warm-up steps, so both arms time the same stretch of trajectory;
    it times the first of its `steps` steps, stopping early once REF_TIME_CAP_S have
    passed (at least one step; ~8 s each at 65,536 ions on 16 Arm threads)."""
    if dist.rank != 0:
        return None
    import oracle
    from simbuca_gb300 import configs
    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    w = configs.WORKLOADS[args.workload]()
    # one cloud at a time, as the reference runs them
    cl0 = w.clouds[0]
    fp, op = w.fields[0], w.odes[0]
    pos, vel = cl0.pos.copy(), cl0.vel.copy()
    h = op.h0
    t = op.t0

    def one_step():
        """One accepted step (all its attempts) with the state carried over; returns
        (accepted step size, attempts)."""
        nonlocal pos, vel, t, h
        p2, v2, cc, hist, nh = oracle.dp45_run(pos, vel, cl0.mass, cl0.charge, fp,
                                               rtol=op.rtol, atol=op.atol, h0=h, t0=t,
                                               t_end=float("inf"), max_steps=1, hist_cap=64,
                                               beta=args.beta)
        dsim = cc.t - t
        pos, vel, t, h = p2, v2, cc.t, cc.h
        return dsim, max(nh, 1)

    t_start = time.perf_counter()
    hist_h = []
    for _ in range(args.settle):
        hist_h.append(one_step()[0])
        if settled(hist_h):
            break
    h_settled = h
    for _ in range(args.warmup):
        one_step()
    prep_s = time.perf_counter() - t_start
    t0 = time.perf_counter()
    sim = 0.0
    att = 0
    steps = 0
    while steps < max(1, args.steps):
        d, a = one_step()
        sim += d
        att += a
        steps += 1
        if time.perf_counter() - t0 >= REF_TIME_CAP_S:
            break
    dt = time.perf_counter() - t0
    value = sim * 1e6 / dt
    return {
        "impl": "reference",
        "metric": "sim-us/wall-s (Coulomb + Penning field + Dormand-Prince, one cloud per GPU)",
        "value": value, "unit": "sim-us/wall-s", "n_gpus": dist.world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded Gaussian cloud, Maxwell-Boltzmann velocities)",
        "config": {"workload": args.workload, "ions": len(cl0.mass), "clouds": 1,
                   "precision": "fp64", "rtol": op.rtol, "atol": op.atol,
                   "parallelism": f"CPU threads x{cores}",
                   "l2": "not applicable (CPU)",
                   "settle_steps": len(hist_h), "h_settled": h_settled,
                   "method": "dormand-prince",
                   "step_control": controller_name(args),
                   "coulomb_variant": "CPU FP64 direct sum",
                   "timed_steps": f"{steps} of {args.steps} (timing stops after "
                                  f"{REF_TIME_CAP_S:.0f} s)",
                   "settle_and_warmup_s": prep_s},
        "mean_h": sim / steps,
        "attempts": att,
        "cpu_baseline": {"value": value, "unit": "sim-us/wall-s", "cores": cores, "kind": "port",
                         "sample": f"{steps} accepted Dormand-Prince steps ({att} attempts) of "
                                   f"the full cloud after {len(hist_h)} settle and "
                                   f"{args.warmup} warm-up steps, FP64 oracle on {cores} threads"},
        "e2e": {"value": value, "unit": "sim-us/wall-s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    dist = Dist(args.gpus)
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        else:
            from simbuca_gb300 import configs
            multi = args.workload in ("scan_512",)
            out = run_batched(args, dist) if multi else run_ours(args, dist)
        if dist.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
