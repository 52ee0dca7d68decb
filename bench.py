#!/usr/bin/env python3
"""Benchmark: 3D zone-updates/s per SSP-RK3 step on GB300.

Workload: 3D periodic box [0,1]^3 at 256^3 interior cells (+4 ghost cells per
side), MLAU flux + WCNS4 characteristic reconstruction + CT + SSP-RK3,
gamma=5/3, seeded random-phase ICs at rms Mach 1e-2 (beta=1, 1% density
perturbation, B = B0 + curl A).  A zone-update is one interior cell advanced
by one full RK3 step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|split]
  python bench.py --impl reference ...   # CPU implementation on the host cores

Prints one JSON line (rank 0).  Device timing: CUDA events on the library's
stream around exactly K steps, barrier + synchronize on both sides, max over
ranks.  `e2e` repeats the K steps through the reference-named C ABI driver
(mhd_fd_ct_3d) with pinned host arrays: every step copies the 8 state arrays
host->device and back.  The state (1.18 GB) is far larger than L2 (129 MB),
so no explicit L2 flush is needed between steps.
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

METRIC = "3D zone-updates/s per RK3 step"
UNIT = "zone-updates/s"
VARS = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")
KIND_NAMES = ("prim", "aux", "rec", "flux", "emf", "update", "copy", "cfl", "split_sweep",
              "split_prep", "split_update")


def workload_desc(n, mach, precision):
    return {
        "workload": f"3D periodic box {n}^3, MLAU + WCNS4 (char.) + CT + SSP-RK3, gamma=5/3, "
                    f"rms Mach {mach:g}, beta=1",
        "grid": [n, n, n], "ghosts": 4, "flux": "MLAU", "order": 4, "rk": 3,
        "precision": precision,
        "l2": "state (8 x float64 x 264^3 = 1.18 GB) >> 129 MB L2; no flush needed",
    }


# --- clocks ------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --- distributed plumbing (replicas only; no data-path collective) --------------
class Ranks:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = False
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = True

    def barrier(self):
        if self.pg:
            import torch.distributed as dist
            dist.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            import torch.distributed as dist
            dist.destroy_process_group()


# --- roofline -----------------------------------------------------------------
def load_opcounts():
    with open(os.path.join(ROOT, "mlau_gb300", "opcounts.json")) as fh:
        return json.load(fh)


def launch_flops(kind, n, off, opc, precision):
    """Algorithmic FP64 flops (reference algorithm, oracle/opcount.py) of one
    launch of a kernel kind at interior size n^3."""
    N = n + 2 * off
    c = opc["mlau_wcns4_lowmach"]
    if kind == "rec":
        return c["rec_per_cell"] * (N - 4) * N * N
    if kind == "flux":
        return c["flux_per_face"] * (N - 5) * N * N
    if kind == "split_sweep":
        return (c["rec_per_cell"] * (N - 4) + c["flux_per_face"] * (N - 5)) * N * N
    return None


def traffic_for(kind):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as fh:
            t = json.load(fh)
        return t.get(kind)
    return None


def roofline(timing, n, off, peaks, precision):
    opc = load_opcounts()
    dom = max(timing, key=lambda k: timing[k][1]) if timing else None
    if dom is None:
        return None
    cnt, tot = timing[dom]
    avg_s = tot / cnt * 1e-3
    fl = launch_flops(dom, n, off, opc, precision)
    p64, p32 = peaks
    peak = p64 if precision == "fp64" else p32
    out = {"kernel": dom, "bound": "fp64" if precision == "fp64" else "fp32",
           "unit": "TFLOP/s", "avg_launch_ms": avg_s * 1e3, "launches": cnt,
           "share_of_step": tot / sum(v[1] for v in timing.values()),
           "peak": peak / 1e12,
           "peak_source": "live FMA-throughput probe on this GPU (2 flop/FMA); "
                          "MEASURED_PEAKS.json has no FP64/FP32 figure",
           "traffic": traffic_for(dom)}
    if fl is not None:
        out["achieved"] = fl / avg_s / 1e12
        out["frac"] = out["achieved"] / out["peak"]
        out["algorithmic_flops_per_launch"] = fl
        out["flops_source"] = "reference algorithm op count (oracle/opcount.py, " \
                              "mlau_gb300/opcounts.json)"
    return out


# --- our arm -----------------------------------------------------------------
def run_ours(args, R: Ranks):
    import mlau_gb300 as M
    from mlau_gb300 import ics

    M.set_device(R.local)
    n, off = args.n, 4
    st, meta = ics.turbulence_3d(n=n, mach=args.mach, seed=1000 + R.rank)
    prec = M.FP32_SPLIT if args.precision == "split" else M.FP64
    sim = M.Sim(3, st["ro"].shape, off=off, dx=meta["dx"], dy=meta["dy"], dz=meta["dz"],
                gamma=meta["gamma"], odr=4, flux="mlau", nrk=3, precision=prec)
    sim.upload(st)
    dt, vmax = sim.cfl(0.4, meta["dx"], 0.0, 0.0)
    peaks = M.measure_fma_peaks()
    for _ in range(args.warmup):
        sim.step(dt, 1)
    sim.sync()
    sim.set_timing(True)
    R.barrier()
    sim.sync()
    with ClockSampler(R.local) as clk:
        ms = sim.time_steps(dt, args.steps)
    sim.sync()
    R.barrier()
    timing = sim.timing()
    sim.set_timing(False)
    ms_max = R.max(ms)
    zones = n ** 3
    value = zones * args.steps * R.world / (ms_max * 1e-3)
    launches = sim.launches_per_step * args.steps
    result = {"ms_per_step": ms_max / args.steps, "value": value, "timing": timing,
              "clocks": clk.summary(), "dt": dt, "launches": launches, "peaks": peaks,
              "device_bytes": sim.device_bytes}
    # end to end through the C ABI drop-in driver with pinned host buffers
    result["e2e"] = run_e2e(args, R, st, meta, dt, M, prec)
    sim.close()
    return result


def run_e2e(args, R, st, meta, dt, M, prec):
    n = args.n
    host = {k: np.ascontiguousarray(st[k].copy()) for k in VARS}
    for a in host.values():
        M.pin(a)
    nz, ny, nx = host["ro"].shape
    M.set_scheme(3, 4, "mlau", 3)
    M.set_precision(3, prec)
    args_c = [host[k] for k in VARS]
    M.mhd_fd_ct_3d(*args_c, dt, meta["dx"], meta["dy"], meta["dz"], nx, ny, nz, 4, 4, 4,
                   meta["gamma"])  # warm-up: builds the cached device context
    R.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        M.mhd_fd_ct_3d(*args_c, dt, meta["dx"], meta["dy"], meta["dz"], nx, ny, nz, 4, 4, 4,
                       meta["gamma"])
    t1 = time.perf_counter()
    R.barrier()
    el = R.max(t1 - t0)
    for a in host.values():
        M.unpin(a)
    M.release_dropin()
    bytes_per_step = sum(a.nbytes for a in host.values())
    return {"value": n ** 3 * args.steps * R.world / el, "unit": UNIT,
            "h2d_bytes_per_step": bytes_per_step, "d2h_bytes_per_step": bytes_per_step,
            "path": "C ABI mhd_fd_ct_3d (reference signature), pinned host arrays"}


def cpu_baseline(threads=None, n=96, steps=1):
    """The CPU restatement of the reference driver (oracle/, bit-identical to
    the reference and within ~20% of its speed) on this host's cores."""
    os.environ["OMP_NUM_THREADS"] = str(threads or os.cpu_count())
    from mlau_gb300 import ics
    from oracle import Port

    st, meta = ics.turbulence_3d(n=n, mach=1e-2, seed=7)
    dt = 0.4 * meta["dx"] / meta["vfast"]
    Port.step3d(st, dt, meta["dx"], meta["dy"], meta["dz"], odr=4, flux="mlau")  # warm
    t0 = time.perf_counter()
    for _ in range(steps):
        Port.step3d(st, dt, meta["dx"], meta["dy"], meta["dz"], odr=4, flux="mlau")
    el = time.perf_counter() - t0
    return {"value": n ** 3 * steps / el, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
            "kind": "port",
            "sample": f"{n}^3 interior x {steps} RK3 step(s) of the same MLAU+WCNS4 workload, "
                      f"OpenMP, after one warm-up step"}


def run_reference(args, R: Ranks):
    """--impl reference: the reference's CPU implementation of the path (its C
    restatement; the reference's own object files do not travel to this host)
    with all host threads; each step is a bounded 128^3 sample of the workload."""
    if R.rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    from mlau_gb300 import ics
    from oracle import Port
    n = args.ref_n
    st, meta = ics.turbulence_3d(n=n, mach=args.mach, seed=7)
    dt = 0.4 * meta["dx"] / meta["vfast"]
    for _ in range(args.warmup):
        Port.step3d(st, dt, meta["dx"], meta["dy"], meta["dz"], odr=4, flux="mlau")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        Port.step3d(st, dt, meta["dx"], meta["dy"], meta["dz"], odr=4, flux="mlau")
    el = time.perf_counter() - t0
    v = n ** 3 * args.steps / el
    cores = int(os.environ["OMP_NUM_THREADS"])
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-phase ICs)",
            "config": workload_desc(args.n, args.mach, "fp64-plain") | {
                "sample": f"{n}^3 interior per step (bounded sample of the {args.n}^3 workload)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{n}^3 interior x {args.steps} steps"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--mach", type=float, default=1e-2)
    ap.add_argument("--precision", choices=("fp64", "split"), default="fp64")
    ap.add_argument("--ref-n", type=int, default=128)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    R = Ranks()
    try:
        if args.impl == "reference":
            run_reference(args, R)
            return
        res = run_ours(args, R)
        if R.rank != 0:
            return
        prec_name = "fp64" if args.precision == "fp64" else "fp32-split"
        line = {
            "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": R.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic (seeded random-phase ICs; no dataset in the reference)",
            "config": workload_desc(args.n, args.mach, prec_name) | {
                "parallelism": f"replicas x{R.world}" if R.world > 1 else "single GPU",
                "dt": res["dt"]},
            "roofline": roofline(res["timing"], args.n, 4, res["peaks"], args.precision),
            "e2e": res["e2e"],
            "gpu_launches": res["launches"],
            "clocks": res["clocks"],
            "kernel_ms": {k: {"launches": c, "total_ms": t} for k, (c, t) in res["timing"].items()},
            "peaks_measured": {"fp64_tflops": res["peaks"][0] / 1e12,
                               "fp32_tflops": res["peaks"][1] / 1e12},
            "device_bytes": res["device_bytes"],
        }
        if not args.no_cpu_baseline and R.world == 1:
            line["cpu_baseline"] = cpu_baseline()
        print(json.dumps(line), flush=True)
    finally:
        R.close()


if __name__ == "__main__":
    main()
