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
        "l2": f"state (8 x float64 x {n + 8}^3 = {8 * 8 * (n + 8) ** 3 / 1e9:.2f} GB) >> 129 MB L2; "
              "no flush needed",
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
        sm, mx, reasons, pw = [], None, set(), []
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
            try:
                pw.append(float(p[3]))
            except ValueError:
                pass
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "power_w": statistics.median(pw) if pw else None}


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
    if kind == "split_sweep":  # one timed launch = the three direction sweeps of a stage
        return 3 * (c["rec_per_cell"] * (N - 4) + c["flux_per_face"] * (N - 5)) * N * N
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
PRECISIONS = {"fp64": "FP64", "split": "FP32_SPLIT", "split_f64": "FP32_SPLIT_F64"}


def run_ours(args, R: Ranks, precision, st, meta, e2e=True):
    import mlau_gb300 as M

    M.set_device(R.local)
    n, off = args.n, 4
    prec = getattr(M, PRECISIONS[precision])
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
    if e2e:
        result["e2e"] = run_e2e(args, R, st, meta, dt, M, prec)
    sim.close()
    return result


def run_accuracy(n, mach, steps, seed=8):
    """The 3D configuration's accuracy record: `steps` RK3 steps at a fixed dt
    (CFL 0.4 of the initial state) from one seeded state, in plain FP64 and in
    both FP32-split forms; per-variable relative L1 of each split result
    against the FP64 one, and max |div B| * dx / max |B| of every result."""
    import mlau_gb300 as M
    from mlau_gb300 import ics
    st, m = ics.turbulence_3d(n=n, mach=mach, seed=seed)
    dt = 0.4 * m["dx"] / m["vfast"]
    out, ms = {}, {}
    for name in ("fp64", "split", "split_f64"):
        with M.Sim(3, st["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], gamma=m["gamma"],
                   odr=4, flux="mlau", nrk=3, precision=getattr(M, PRECISIONS[name])) as s:
            s.upload(st)
            ms[name] = s.time_steps(dt, steps)
            out[name] = s.download()
    rec = {"grid": [n, n, n], "rms_mach": mach, "steps": steps, "dt": dt, "seed": seed,
           "tolerance_ro": 1e-6,
           "div_b": {k: ics.div_b_3d(v, m["dx"], m["dy"], m["dz"]) for k, v in out.items()},
           "ms_per_step": {k: v / steps for k, v in ms.items()}}
    for name in ("split", "split_f64"):
        rec[f"l1_{name}_vs_fp64"] = rel_l1(out[name], out["fp64"])
    return rec


def rel_l1(a, b, off=4):
    """Relative L1 difference of a against b over the interior, per variable."""
    core = (slice(off, -off),) * 3
    return {k: float(np.abs(a[k][core] - b[k][core]).sum() / np.abs(b[k][core]).sum())
            for k in VARS}


def host_array(like):
    """An empty host array shaped like `like`, on 2 MB transparent huge pages
    where the kernel offers them (anonymous mapping + MADV_HUGEPAGE, before the
    first touch).  Pinned 4 KB pages cost the host-to-device copy some 15 %
    (172 against 201 GB/s for the 8 arrays of the 256^3 state, measured);
    device-to-host is the same on both."""
    import mmap
    nbytes = like.nbytes
    try:
        m = mmap.mmap(-1, nbytes, flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
        m.madvise(mmap.MADV_HUGEPAGE)
    except (AttributeError, OSError, ValueError):
        return np.empty_like(like), False
    return np.frombuffer(m, dtype=like.dtype).reshape(like.shape), True


def run_e2e(args, R, st, meta, dt, M, prec):
    """The same K steps through the reference-named driver with host arrays.
    The host arrays are first touched, pinned and driven from the CPUs next to
    this rank's GPU (its PCI root's local CPU list), so that on a multi-socket
    host they sit on the GPU's own memory node, as a production caller would
    place them; the affinity is restored afterwards.  They sit on huge pages
    where the kernel offers them (host_array)."""
    n = args.n
    cpus = M.local_cpus(R.local)
    old_aff = os.sched_getaffinity(0) if cpus else None
    if cpus:
        try:
            os.sched_setaffinity(0, cpus)
        except OSError:
            cpus = None
    host, huge = {}, True
    for k in VARS:
        host[k], h = host_array(st[k])
        huge = huge and h
        host[k][...] = st[k]  # first touch from the local CPUs
    for a in host.values():
        M.pin(a)
    nz, ny, nx = host["ro"].shape
    M.set_scheme(3, 4, "mlau", 3)
    M.set_precision(3, prec)
    args_c = [host[k] for k in VARS]
    M.mhd_fd_ct_3d(*args_c, dt, meta["dx"], meta["dy"], meta["dz"], nx, ny, nz, 4, 4, 4,
                   meta["gamma"])  # warm-up: builds the cached device context
    R.barrier()
    calls = []
    with ClockSampler(R.local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            tc = time.perf_counter()
            M.mhd_fd_ct_3d(*args_c, dt, meta["dx"], meta["dy"], meta["dz"], nx, ny, nz, 4, 4, 4,
                           meta["gamma"])
            calls.append(time.perf_counter() - tc)
        t1 = time.perf_counter()
    R.barrier()
    el = R.max(t1 - t0)
    for a in host.values():
        M.unpin(a)
    M.release_dropin()
    if old_aff:
        os.sched_setaffinity(0, old_aff)
    bytes_per_step = sum(a.nbytes for a in host.values())
    place = (f"host arrays on the GPU's local CPUs {min(cpus)}-{max(cpus)}" if cpus
             else "host arrays where the process runs (GPU-local CPUs unknown)")
    place += ", huge pages requested (madvise)" if huge else ", 4 KB pages"
    return {"value": n ** 3 * args.steps * R.world / el, "unit": UNIT,
            "h2d_bytes_per_step": bytes_per_step, "d2h_bytes_per_step": bytes_per_step,
            "path": "C ABI mhd_fd_ct_3d (reference signature), pinned host arrays",
            "placement": place,
            # per-call spread: the host link is shared with the machine's other
            # GPUs, and its throughput moves between runs
            "call_ms": {"min": 1e3 * min(calls), "median": 1e3 * float(np.median(calls)),
                        "max": 1e3 * max(calls), "each": [round(1e3 * c, 1) for c in calls]},
            "clocks": clk.summary()}


def cpu_baseline(threads=None, n=256, steps=2, mach=1e-2):
    """The CPU restatement of the reference driver (oracle/, bit-identical to
    the reference and within ~20% of its speed) on this host's cores."""
    os.environ["OMP_NUM_THREADS"] = str(threads or os.cpu_count())
    from mlau_gb300 import ics
    from oracle import Port

    st, meta = ics.turbulence_3d(n=n, mach=mach, seed=7)
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
    restatement, bit-identical to the reference; the reference's own object
    files do not travel to this host) with all host threads, on the
    benchmark's own workload (--ref-n defaults to --n)."""
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
                "sample": f"{n}^3 interior per step" + (
                    " (the benchmark's own workload)" if n == args.n
                    else f" (bounded sample of the {args.n}^3 workload)"),
                "same_config": n == args.n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{n}^3 interior x {args.steps} steps"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --- 2D and 1D single-problem workloads ------------------------------------------
def run_step2d(args):
    """Config C1: 2D periodic box 512^2, LHLLD + WCNS4 + CT + SSP-RK3, FP64 plain
    (bit-exact to the reference), gamma=5/3, random-phase ICs (v_rms 0.5,
    beta 1); K steps at a fixed dt, device-resident, plus the CPU
    restatement of the reference timed on a bounded sample beside it."""
    import mlau_gb300 as M
    from mlau_gb300 import ics
    n = args.n2d
    st, m = ics.turbulence_2d(n=n, seed=3, vrms=0.5)
    dt = 0.4 * m["dx"] / m["vfast"]
    peaks = M.measure_fma_peaks()
    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=4,
               flux="lhlld", nrk=3) as s:
        s.upload(st)
        s.step(dt, args.warmup)
        s.sync()
        s.set_timing(True)
        with ClockSampler(0) as clk:
            ms = s.time_steps(dt, args.steps)
        timing = s.timing()
        launches = s.launches_per_step * args.steps
    v = n * n * args.steps / (ms * 1e-3)
    opc = load_opcounts()["lhlld_wcns4_2d"]
    N = n + 8
    dom = max(timing, key=lambda k: timing[k][1])
    cnt, tot = timing[dom]
    fl = {"rec": opc["rec_per_cell"] * (N - 4) * N, "flux": opc["flux_per_face"] * (N - 5) * N}
    roof = {"kernel": dom, "bound": "fp64", "unit": "TFLOP/s", "peak": peaks[0] / 1e12,
            "peak_source": "live FMA-throughput probe (2 flop/FMA)", "traffic": None,
            "avg_launch_ms": tot / cnt, "share_of_step": tot / sum(x[1] for x in timing.values())}
    if dom in fl:
        roof["achieved"] = fl[dom] / (tot / cnt * 1e-3) / 1e12
        roof["frac"] = roof["achieved"] / roof["peak"]
    # CPU restatement of the reference on a bounded sample (same problem)
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    from oracle import Port
    cst = ics.copy_state(st)
    Port.step2d(cst, dt, m["dx"], m["dy"], odr=4, flux="lhlld")
    t0 = time.perf_counter()
    for _ in range(args.cpu_steps):
        Port.step2d(cst, dt, m["dx"], m["dy"], odr=4, flux="lhlld")
    cv = n * n * args.cpu_steps / (time.perf_counter() - t0)
    return {"metric": "2D zone-updates/s per RK3 step", "value": v, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded random-phase ICs)",
            "config": {"workload": f"2D periodic box {n}^2, LHLLD + WCNS4 + CT + SSP-RK3, "
                                   "gamma=5/3, v_rms 0.5, beta 1, FP64 plain (bit-exact)",
                       "l2": f"state 8 x {N * N * 8 / 1e6:.1f} MB fits in L2: steady-state "
                             "throughput of a resident problem, no flush"},
            "roofline": roof, "gpu_launches": launches, "clocks": clk.summary(),
            "kernel_ms": {k: {"launches": c, "total_ms": t} for k, (c, t) in timing.items()},
            "cpu_baseline": {"value": cv, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port", "sample": f"{n}^2 x {args.cpu_steps} steps"}}


def run_mrx2d(args):
    """The MRX problem's main loop (2D/MPI/MRX/main.cpp:48-68) at its size,
    2048 x 256 cells: hyperbolic step (MC-limited MUSCL, LHLLD, CT, RK3),
    resistive diffusion of B with its energy flux, viscosity, and the CFL dt
    read back every loop, as the reference does.  FP64 plain (bit-exact);
    the CPU restatement of the same loop timed beside it."""
    import mlau_gb300 as M
    from mlau_gb300 import ics
    st, m = ics.mrx_2d(seed=1)
    ny, nx = st["ro"].shape
    cells = (nx - 8) * (ny - 8)

    def loop(s, dt, n):
        for _ in range(n):
            s.step(dt, 1)
            s.resistive(m["eta0"], dt)
            s.viscous(m["nu0"], dt)
            dt, _ = s.cfl(m["cfl"], m["dr"], m["vfast"], dt)
        return dt

    with M.Sim(2, st["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=5,
               flux="lhlld", nrk=3) as s:
        s.set_bc2d(*m["tables"])
        s.upload(st)
        dt = loop(s, m["dt"], args.warmup)
        s.sync()
        with ClockSampler(0) as clk:
            t0 = time.perf_counter()
            dt = loop(s, dt, args.steps)
            s.sync()
            sec = time.perf_counter() - t0
        # the operators alone, CUDA-event timed on the library's stream
        s.set_timing(False)
        op_ms = {}
        for op, coef in (("resistive", m["eta0"]), ("viscous", m["nu0"])):
            fn = getattr(s, op)
            for _ in range(3):
                fn(coef, dt)
            s.sync()
            t1 = time.perf_counter()
            for _ in range(args.steps):
                fn(coef, dt)
            s.sync()
            op_ms[op] = (time.perf_counter() - t1) * 1e3 / args.steps
        # heat conduction along B (off in the reference's MRX setup: kk0 = 0)
        # at kk0 = eta0, with its Gauss-Seidel sweep count
        sweeps = s.conduction(m["eta0"], dt)
        s.sync()
        t1 = time.perf_counter()
        for _ in range(10):
            sweeps = s.conduction(m["eta0"], dt)
        op_ms["conduction"] = (time.perf_counter() - t1) * 1e3 / 10
        op_ms["conduction_sweeps"] = sweeps
        launches = (s.launches_per_step + 3 * 4 + 1 + 3 * 3 + 3 + 1) * args.steps
    v = cells * args.steps / sec
    from oracle import Port
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    cst = ics.copy_state(st)
    kw = dict(gamma=m["gamma"], odr=5, nrk=3, dnx=m["tables"][0], dny=m["tables"][1])
    t0 = time.perf_counter()
    for _ in range(args.cpu_steps):
        Port.step2d(cst, m["dt"], m["dx"], m["dy"], flux="lhlld", **kw)
        Port.resistive2d(cst, m["eta0"], m["dt"], m["dx"], m["dy"], **kw)
        Port.viscous2d(cst, m["nu0"], m["dt"], m["dx"], m["dy"], **kw)
    cv = cells * args.cpu_steps / (time.perf_counter() - t0)
    return {"metric": "MRX loop zone-updates/s (step + resistive + viscous + CFL)", "value": v,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (Harris sheet with seeded Vy noise; the reference seeds from the clock)",
            "config": {"workload": "MRX 2048 x 256, x periodic / y walls, MUSCL-MC + LHLLD + CT + "
                                   "RK3, eta0 = nu0 = 2e-3, CFL 0.2 dt read back per loop",
                       "l2": "state 8 x 4.3 MB fits in L2: steady-state throughput, no flush"},
            "operator_ms": op_ms, "gpu_launches": launches, "clocks": clk.summary(),
            "cpu_baseline": {"value": cv, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port", "sample": f"MRX 2048 x 256 x {args.cpu_steps} loops"}}


def run_step1d(args):
    """Config C0: 1D Riemann problem, 2048 cells, MLAU + MUSCL (minmod) + RK3,
    gamma=2, CFL 0.4, open boundaries, dt fixed from the initial state, run to
    t_end=0.1 as the 1D driver does; the whole run is timed (one problem is
    latency bound: 11 launches per step, the open boundary beside the first stage)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    import mlau_gb300 as M
    from mlau_gb300 import ics
    from oracle import Port
    st, m = ics.riemann_1d(n=2048, seed=0)
    with M.Sim(1, st["ro"].shape, dx=m["dx"], gamma=m["gamma"], odr=2, flux="mlau", nrk=3) as s:
        s.set_bx(m["bx"])
        s.set_bc("open")
        s.upload(st)
        dt, _ = s.cfl(0.4, m["dx"], 1.0, 0.0)
        t, nsteps = 0.0, 0
        while t < 0.1:
            t += dt
            nsteps += 1
        s.step(dt, args.warmup)
        s.sync()
        with ClockSampler(0) as clk:
            ms = s.time_steps(dt, nsteps)
        launches = s.launches_per_step * nsteps
    v = 2048 * nsteps / (ms * 1e-3)
    cst = ics.copy_state(st)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        Port.step1d(cst, m["bx"], dt, m["dx"], gamma=m["gamma"], odr=2, flux="mlau", nrk=3)
    cv = 2048 * nsteps / (time.perf_counter() - t0)
    return {"metric": "1D zone-updates/s per RK3 step (whole run to t_end)", "value": v,
            "unit": UNIT, "n_gpus": 1, "steps": nsteps, "warmup": args.warmup,
            "ms_per_step": ms / nsteps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Riemann states)",
            "config": {"workload": "1D Riemann problem, 2048 cells, MLAU + MUSCL-minmod + RK3, "
                                   "gamma=2, CFL 0.4, open boundaries, t_end 0.1",
                       "time_to_solution_ms": ms, "l2": "fits in L2 (one resident problem)"},
            "roofline": None,
            "roofline_note": "latency bound: each warp's FP64 chain (a warp FP64 instruction holds "
                             "its sub-partition's pipe 64 cycles) and 11 launches per step",
            "gpu_launches": launches, "clocks": clk.summary(),
            "cpu_baseline": {"value": cv, "unit": UNIT,
                             "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                             "sample": f"the whole run, {nsteps} steps, OpenMP"}}


# --- batched 2D and serving workloads ------------------------------------------
def batch2d_requests(n_inst, seed, n2d=(64, 1024), t_end=(0.05, 0.5)):
    """256 uneven periodic 2D instances: sizes log-uniform per axis, solver and
    gamma uniform, rms Mach U[1e-3, 2], beta log-uniform in [0.1, 10]."""
    from mlau_gb300 import serve
    return serve.make_requests(n_inst, rate=1.0, seed=seed, mix=(0.0, 1.0, 0.0), n2d=n2d,
                               t_end_2d=t_end, split_frac=1.0)


def run_batch2d(args, n_inst=None, steps=None, warmup=None):
    """Batched 2D engine, FP32-split: all instances in one persistent
    cooperative launch per step, tile shape from the autotuner, steps replayed
    from captured graphs; zone-updates/s over the instances still running."""
    import mlau_gb300 as M
    n_inst = n_inst or args.batch_n
    steps = steps or args.steps
    warmup = warmup or args.warmup
    reqs = batch2d_requests(n_inst, seed=5)
    cells = sum(r.state["ro"].size for r in reqs)
    b = M.Batch.open(cells, len(reqs), precision=M.FP32_SPLIT, odr=4)
    slots = [b.add(r.state, r.meta["dx"], r.meta["dy"], r.meta["gamma"], r.meta["flux"],
                   r.meta["cfl"], r.meta["t_end"]) for r in reqs]
    tw, th, tune_ms = b.autotune(steps=2)
    b.run(warmup, steps_per_graph=warmup)
    before = [b.info(s)[1] for s in slots]
    active = sum(b.info(s)[2] for s in slots)
    with ClockSampler(0) as clk:
        left, ms = b.run(steps, steps_per_graph=steps)
    # zone-updates actually done: instances that retire mid-run stop counting
    zones = sum(r.interior * (b.info(s)[1] - n0) for r, s, n0 in zip(reqs, slots, before))
    failed = sum(b.failed(s) for s in slots)
    v = zones / (ms * 1e-3)
    b.close()
    return {"metric": "batched 2D zone-updates/s (uneven instances, one persistent launch per "
                      "step, FP32-split)",
            "value": v, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warmup,
            "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
            "config": {"workload": f"{len(reqs)} periodic 2D instances, sizes log-uniform "
                                   f"64..1024 per axis, solver/gamma uniform, Mach U[1e-3,2], "
                                   f"beta logU[0.1,10], WCNS4 + CT + RK3, own CFL dt",
                       "zone_updates": zones, "instances_active_at_start": active,
                       "instances_active_at_end": left,
                       "tile": [tw, th], "autotune_ms": tune_ms,
                       "graph_steps": steps, "failed_instances": failed,
                       "l2": "working set >> 129 MB L2"},
            "gpu_launches": steps, "clocks": clk.summary()}


def run_serve(args):
    """Serving (continuous batching under an HBM budget) against solving the
    same requests one at a time with the plain FP64 path, at several arrival
    rates; time-to-solution counts from each request's arrival."""
    import mlau_gb300 as M
    from mlau_gb300 import serve
    rates = [float(x) for x in args.rates.split(",")]
    kw = dict(seed=11, n1d=(256, args.serve_n1d_max), n2d=(64, args.serve_n2d_max),
              n3d=(64, args.serve_n3d_max), t_end_2d=(0.05, args.serve_t_end_max))
    base = serve.make_requests(args.serve_n, rate=rates[0], **kw)
    # one-at-a-time FP64 baseline: execution time of each request, measured once
    execs, zu_serial = [], 0
    for r in base:
        _, steps, sec = serve.solve_alone_fp64(r)
        execs.append(sec)
        zu_serial += r.interior * steps
    out = {"metric": "serving time-to-solution p50/p99 and zone-updates/s",
           "unit": "s", "n_gpus": 1, "higher_is_better": False, "dtype": "f64 | f32+f64",
           "data": "synthetic seeded Poisson request stream",
           "config": {"workload": f"{args.serve_n} requests: 50% 1D Riemann N "
                                  f"logU[256,{args.serve_n1d_max}], 40% 2D periodic (sizes logU "
                                  f"64..{args.serve_n2d_max}, t_end U[0.05,{args.serve_t_end_max:g}]), "
                                  f"10% 3D periodic 64^3..{args.serve_n3d_max}^3 x 200 steps; FP64 "
                                  f"or FP32-split per request (1D in FP64)",
                      "budget_gb": args.budget_gb,
                      "ranges": {k: list(v) for k, v in kw.items() if k != "seed"}},
           "rates": {}}
    for rate in rates:
        reqs = serve.make_requests(args.serve_n, rate=rate, **kw)
        lat_s, end_s = serve.serial_schedule(reqs, execs)
        with serve.Server(budget_bytes=args.budget_gb * 1e9) as srv:
            done = srv.run(reqs, realtime=True)
            makespan = max(r.t_done for r in done)
        zu = sum(r.zone_updates for r in done)
        out["rates"][str(rate)] = {
            "served": serve.summary([r.latency for r in done], zu, makespan),
            "one_at_a_time_fp64": serve.summary(lat_s, zu_serial, end_s),
            "failed": sum(r.failed for r in done),
            "by_kind_p50_s": {k: float(np.percentile([r.latency for r in done if r.kind == k], 50))
                              for k in ("1d", "2d", "3d") if any(r.kind == k for r in done)},
        }
    head = out["rates"][str(rates[-1])]["served"]
    out["value"] = head["p99_s"]
    out["p50_s"], out["p99_s"] = head["p50_s"], head["p99_s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--mach", type=float, default=1e-2)
    ap.add_argument("--precision", choices=("both", "fp64", "split"), default="both",
                    help="both: FP32-split is the headline value, FP64 beside it")
    ap.add_argument("--workload", choices=("step3d", "step2d", "step1d", "batch2d", "serve",
                                           "mrx2d", "accuracy3d"),
                    default="step3d")
    ap.add_argument("--n2d", type=int, default=512)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--ref-n", type=int, default=None,
                    help="interior size of the reference arm's steps (default: --n, the "
                         "benchmark's own workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the end-to-end drop-in measurement (profiling runs)")
    ap.add_argument("--no-config-samples", dest="config_samples", action="store_false",
                    help="skip the 1D / 2D / MRX samples of the default line")
    ap.add_argument("--batch-sample", type=int, default=64,
                    help="instances of the batched-engine sample in the default line (0: skip)")
    ap.add_argument("--accuracy-steps", type=int, default=200,
                    help="steps of the split-vs-FP64 accuracy record (0: skip it)")
    ap.add_argument("--batch-n", type=int, default=256)
    ap.add_argument("--serve-n", type=int, default=24)
    ap.add_argument("--rates", default="5,50,200")
    ap.add_argument("--budget-gb", type=float, default=120.0)
    ap.add_argument("--serve-n1d-max", type=int, default=16384)
    ap.add_argument("--serve-n2d-max", type=int, default=1024)
    ap.add_argument("--serve-n3d-max", type=int, default=128)
    ap.add_argument("--serve-t-end-max", type=float, default=0.5)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.ref_n is None:
        args.ref_n = args.n
    R = Ranks()
    try:
        if args.impl == "reference":
            run_reference(args, R)
            return
        if args.workload in ("step2d", "step1d"):
            if R.rank == 0:
                fn = run_step2d if args.workload == "step2d" else run_step1d
                print(json.dumps(fn(args)), flush=True)
            return
        if args.workload == "mrx2d":
            if R.rank == 0:
                print(json.dumps(run_mrx2d(args)), flush=True)
            return
        if args.workload == "accuracy3d":
            if R.rank == 0:
                recs = [run_accuracy(args.n, mach, args.accuracy_steps)
                        for mach in sorted({args.mach, 1e-4}, reverse=True)]
                zu = args.n ** 3 * 1e3  # zone-updates per step, per ms -> per s
                print(json.dumps({
                    "metric": "3D split-vs-FP64 relative L1 after the configuration's steps",
                    "value": max(r["l1_split_vs_fp64"]["ro"] for r in recs),
                    "unit": "relative L1 of density", "higher_is_better": False, "n_gpus": 1,
                    "steps": args.accuracy_steps, "dtype": "f32+f64 vs f64",
                    "data": "synthetic (seeded random-phase ICs)",
                    "config": workload_desc(args.n, args.mach, "fp64 and both FP32-split forms"),
                    "zone_updates_per_s": {
                        r["rms_mach"]: {k: zu / v for k, v in r["ms_per_step"].items()}
                        for r in recs},
                    "accuracy": recs}), flush=True)
            return
        if args.workload == "batch2d":
            if R.rank == 0:
                print(json.dumps(run_batch2d(args)), flush=True)
            return
        if args.workload == "serve":
            if R.rank == 0:
                print(json.dumps(run_serve(args)), flush=True)
            return
        from mlau_gb300 import ics
        st, meta = ics.turbulence_3d(n=args.n, mach=args.mach, seed=1000 + R.rank)
        precs = ("split", "fp64") if args.precision == "both" else (args.precision,)
        res = {p: run_ours(args, R, p, st, meta, e2e=not args.no_e2e) for p in precs}
        if args.precision == "both":
            # the split form with FP64 state arithmetic, device-timed beside it
            res["split_f64"] = run_ours(args, R, "split_f64", st, meta, e2e=False)
        if R.rank != 0:
            return
        head = precs[0]
        r = res[head]
        prec_name = {"fp64": "fp64", "split": "fp32-split", "split_f64": "fp32-split-f64"}[head]
        line = {
            "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": R.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if head == "fp64" else "f32+f64",
            "data": "synthetic (seeded random-phase ICs; no dataset in the reference)",
            "config": workload_desc(args.n, args.mach, prec_name) | {
                "parallelism": f"replicas x{R.world}" if R.world > 1 else "single GPU",
                "dt": r["dt"]},
            "roofline": roofline(r["timing"], args.n, 4, r["peaks"], head),
            "e2e": r.get("e2e"),
            "gpu_launches": r["launches"],
            "clocks": r["clocks"],
            "kernel_ms": {k: {"launches": c, "total_ms": t} for k, (c, t) in r["timing"].items()},
            "peaks_measured": {"fp64_tflops": r["peaks"][0] / 1e12,
                               "fp32_tflops": r["peaks"][1] / 1e12},
            "device_bytes": r["device_bytes"],
        }
        if "fp64" in res and head != "fp64":
            f = res["fp64"]
            line["fp64"] = {
                "value": f["value"], "ms_per_step": f["ms_per_step"], "e2e": f.get("e2e"),
                "roofline": roofline(f["timing"], args.n, 4, f["peaks"], "fp64"),
                "gpu_launches": f["launches"], "clocks": f["clocks"],
                "kernel_ms": {k: {"launches": c, "total_ms": t}
                              for k, (c, t) in f["timing"].items()}}
            line["split_over_fp64"] = r["value"] / f["value"]
        if "split_f64" in res:
            q = res["split_f64"]
            line["split_f64"] = {
                "what": "FP32 reconstruction / Riemann solver / EMFs, with pressure recovery, "
                        "RK accumulation and CT curl in FP64 arithmetic (float-float in the "
                        "headline form)",
                "value": q["value"], "ms_per_step": q["ms_per_step"],
                "over_fp64": q["value"] / res["fp64"]["value"] if "fp64" in res else None,
                "gpu_launches": q["launches"],
                "kernel_ms": {k: {"launches": c, "total_ms": t}
                              for k, (c, t) in q["timing"].items()}}
        if args.batch_sample > 0 and R.world == 1 and args.precision == "both":
            # a bounded sample of the batched engine (uneven 2D instances)
            bl = run_batch2d(args, n_inst=args.batch_sample, steps=5, warmup=3)
            line["batch2d_sample"] = {k: bl[k] for k in ("metric", "value", "unit", "ms_per_step",
                                                         "steps", "config", "clocks")}
        if args.config_samples and R.world == 1 and args.precision == "both":
            # bounded samples of the other configurations, so that the default
            # run records them too: 1D Riemann problem to t_end, 2D 512^2, the
            # MRX loop (each with its CPU restatement beside it)
            a2 = argparse.Namespace(**vars(args))
            a2.steps, a2.warmup, a2.cpu_steps = 20, 3, 1
            samples = {}
            for name, fn in (("step1d", run_step1d), ("step2d", run_step2d), ("mrx2d", run_mrx2d)):
                r2 = fn(a2)
                samples[name] = {k: r2.get(k) for k in ("metric", "value", "unit", "ms_per_step",
                                                        "steps", "config", "cpu_baseline",
                                                        "roofline")}
            # and the serving loop on a bounded request stream (12 requests at
            # 50 req/s, reduced sizes), against one-at-a-time FP64
            a3 = argparse.Namespace(**vars(args))
            a3.serve_n, a3.rates = 12, "50"
            a3.serve_n1d_max, a3.serve_n2d_max, a3.serve_n3d_max = 4096, 256, 64
            a3.serve_t_end_max = 0.2
            try:
                sv = run_serve(a3)
                samples["serve"] = {k: sv.get(k) for k in ("metric", "unit", "p50_s", "p99_s",
                                                           "config", "rates")}
            except Exception as e:  # the headline line must not depend on the sample
                samples["serve"] = {"error": f"{type(e).__name__}: {e}"}
            line["config_samples"] = samples
        if args.accuracy_steps > 0 and R.world == 1 and args.precision == "both":
            # the configuration's 200-step accuracy record at both Mach numbers
            line["accuracy"] = [run_accuracy(args.n, mach, args.accuracy_steps)
                                for mach in sorted({args.mach, 1e-4}, reverse=True)]
        if not args.no_cpu_baseline and R.world == 1:
            line["cpu_baseline"] = cpu_baseline(n=args.n, mach=args.mach)
        print(json.dumps(line), flush=True)
    finally:
        R.close()


if __name__ == "__main__":
    main()
