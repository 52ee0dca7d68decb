"""Request serving on one GPU: a stream of independent MHD problems (1D
Riemann problems, 2D periodic boxes, 3D periodic boxes), each with its own
size, solver, gamma, end time and arithmetic, admitted under an HBM budget
and advanced with continuous batching.

The reference runs one problem per process (1D/SERIAL/shock/main.cpp,
2D/SERIAL/OTvortex/main.cpp, 3D/MPI/OTvortex/main.cpp); this module has no
counterpart there.  Each request is stepped with the same scheme as those
drivers, so its result does not depend on what else is being served:

  lane "1d"    one FP64 1D engine (Batch.open1d): every 1D request, stepped
               like mhd_fd4c_1d with the 1D driver's one-off dt
  lane "2d64"  one FP64 2D engine (Batch.open, MLAU_FP64): each instance bit
               for bit like mhd_fd_ct_2d with a CFL dt every step
  lane "2d32"  one FP32-split 2D engine
  lane "3d"    one device-resident simulation (Sim) per request, FP64 or
               FP32-split, CFL dt every step

Each lane runs in its own host thread and owns its engine: admission,
stepping (captured graphs of `steps_per_tick` steps) and retirement happen
there, between engine runs.  The HBM budget is divided between the lanes
when the server starts; a request waits (FIFO per lane) until its lane has a
slot and room for its cells.  The 1D and 2D lanes share the SMs through a
block allocator: the 1D lane (the smallest requests in work) takes the
blocks it can use first, the 2D lanes split the rest in proportion to their
live cells, and the grids together never exceed what is co-resident, so the
lanes' persistent kernels run side by side.  1D requests always run in FP64 (the 1D problem
is small; its FP64 step is cheap).
"""
from __future__ import annotations

import collections
import dataclasses
import math
import queue
import threading
import time

import numpy as np

from . import FP32_SPLIT, FP64, Batch, MlauError, Sim, ics

KINDS = ("1d", "2d", "3d")
FLUXES = ("mlau", "lhlld", "hlld", "roe")


@dataclasses.dataclass
class Request:
    rid: int
    kind: str                  # "1d" | "2d" | "3d"
    precision: int             # FP64 | FP32_SPLIT (1D is served in FP64)
    arrival: float             # seconds after the start of the stream
    state: dict
    meta: dict                 # dx, dy, dz, gamma, bx, flux, cfl, t_end, steps, ...
    interior: int              # interior cells
    # filled in by the server
    t_admit: float = math.nan
    t_done: float = math.nan
    steps: int = 0
    failed: bool = False
    result: dict | None = None
    lane: str = ""

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival

    @property
    def zone_updates(self) -> int:
        return self.interior * self.steps


# --- the request stream ------------------------------------------------------
def make_requests(n, rate, seed=0, mix=(0.5, 0.4, 0.1), n1d=(256, 16384), n2d=(64, 1024),
                  n3d=(64, 128), t_end_2d=(0.05, 0.5), steps_3d=200, split_frac=0.5, off=4,
                  mach_2d=(1e-3, 2.0), beta_2d=(0.1, 10.0)):
    """Seeded Poisson stream of n requests at `rate` per second.

    1D: Riemann problems on [0,1] (states drawn as in ics.riemann_1d), N
        log-uniform in n1d, gamma 2, MLAU, MUSCL (odr 2), RK3, CFL 0.4,
        t_end 0.1, open boundaries.
    2D: periodic boxes of the random-phase recipe (ics.turbulence_2d), nx and
        ny log-uniform in n2d, solver and gamma (1.4, 5/3, 2) uniform, rms
        Mach uniform in mach_2d (default [1e-3, 2]), beta log-uniform in
        beta_2d (default [0.1, 10]), t_end uniform in t_end_2d, CFL 0.4,
        WCNS4.  (The strongest of these - Mach 2 with beta 0.1 on a coarse
        grid - can drive the pressure negative; such a request retires with
        `failed` set.)
    3D: periodic boxes (ics.turbulence_3d), n log-uniform in n3d, rms Mach
        1e-2 or 1e-4, MLAU + WCNS4, steps_3d steps with a CFL dt.
    Precision FP32-split with probability split_frac."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n)
    arrivals = np.cumsum(gaps) - gaps[0]
    out = []
    for k in range(n):
        kind = KINDS[int(rng.choice(3, p=mix))]
        prec = FP32_SPLIT if rng.uniform() < split_frac else FP64
        s = int(rng.integers(0, 2 ** 31))
        logu = lambda lo, hi: int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        if kind == "1d":
            st, m = ics.riemann_1d(n=logu(*n1d), seed=s, off=off)
            meta = dict(dx=m["dx"], bx=m["bx"], gamma=m["gamma"], flux="mlau", odr=2, nrk=3,
                        bc="open", cfl=0.4, t_end=0.1)
            interior = st["ro"].size - 2 * off
            prec = FP64
        elif kind == "2d":
            gamma = float(rng.choice([1.4, 5.0 / 3.0, 2.0]))
            mach = float(rng.uniform(*mach_2d))
            beta = float(math.exp(rng.uniform(math.log(beta_2d[0]), math.log(beta_2d[1]))))
            nx, ny = logu(*n2d), logu(*n2d)
            st, m = ics.turbulence_2d(n=nx, ny=ny, seed=s, off=off, gamma=gamma, vrms=mach,
                                      beta=beta)
            meta = dict(dx=m["dx"], dy=m["dy"], gamma=gamma, flux=FLUXES[int(rng.integers(4))],
                        cfl=0.4, t_end=float(rng.uniform(*t_end_2d)), mach=mach, beta=beta)
            interior = nx * ny
        else:
            nn = logu(*n3d)
            mach = float(rng.choice([1e-2, 1e-4]))
            st, m = ics.turbulence_3d(n=nn, mach=mach, seed=s, off=off)
            meta = dict(dx=m["dx"], dy=m["dy"], dz=m["dz"], gamma=m["gamma"], flux="mlau",
                        cfl=0.4, steps=steps_3d, vfast=m["vfast"], mach=mach)
            interior = nn ** 3
        out.append(Request(k, kind, prec, float(arrivals[k]), st, meta, interior))
    return out


# --- shared SM blocks ---------------------------------------------------------
class _Blocks:
    """Co-resident blocks shared by the lanes' persistent kernels.  A lane
    takes a grant before a run and gives it back after, so the grids running
    at one time never add up to more than fit together.

    Priority lanes (the 1D lane: its requests are the smallest in work,
    cells x steps, so serving them first is shortest-remaining-work-first)
    are granted the blocks they can use - one per tile of their live
    instances - first; the other lanes share the rest in proportion to their
    live cells (their work per step)."""

    def __init__(self, total):
        self.total = total
        self.free = total
        self.load = {}
        self.useful = {}
        self.prio = set()
        self.cv = threading.Condition()

    def set_load(self, lane, cells, useful=None, prio=False):
        with self.cv:
            self.load[lane] = cells
            self.useful[lane] = useful
            if prio:
                self.prio.add(lane)

    def _want(self, lane, floor):
        if lane in self.prio:
            u = self.useful.get(lane) or self.total
            return min(max(floor, u), self.total // 2)
        held = sum(min(max(floor, self.useful.get(p) or 0), self.total // 2)
                   for p in self.prio if self.load.get(p, 0) > 0)
        rest = max(self.total - held, floor)
        busy = sum(v for k, v in self.load.items() if v > 0 and k not in self.prio)
        share = rest * self.load.get(lane, 0) / max(busy, 1)
        return min(max(floor, int(share) // floor * floor), self.total)

    def acquire(self, lane, floor=8):
        with self.cv:
            want = self._want(lane, floor)
            while self.free < min(want, floor):
                self.cv.wait(0.05)
            got = min(want, self.free)
            self.free -= got
            return got

    def release(self, n):
        with self.cv:
            self.free += n
            self.cv.notify_all()


# --- lanes -------------------------------------------------------------------
class _Lane(threading.Thread):
    def __init__(self, server, name):
        super().__init__(name=f"mlau-lane-{name}", daemon=True)
        self.server, self.lane = server, name
        self.inbox: queue.Queue = queue.Queue()
        self.waiting: collections.deque = collections.deque()
        self.error: BaseException | None = None

    def _drain(self, block):
        try:
            r = self.inbox.get(timeout=0.002) if block else self.inbox.get_nowait()
            while True:
                self.waiting.append(r)
                r = self.inbox.get_nowait()
        except queue.Empty:
            pass

    def run(self):
        try:
            self.loop()
        except BaseException as e:  # reported by Server.run
            self.error = e
            self.server._wake.set()


class _BatchLane(_Lane):
    def __init__(self, server, name, batch, steps_per_tick, prio=False, tile=None):
        super().__init__(server, name)
        self.batch, self.k = batch, steps_per_tick
        self.live: dict[int, Request] = {}
        self.prio, self.tile = prio, tile

    def _admit(self):
        while self.waiting:
            r = self.waiting[0]
            m = r.meta
            if r.kind == "1d":
                slot = self.batch.add1d(r.state, m["dx"], m["bx"], m["gamma"], m["flux"],
                                        m["nrk"], m["bc"], m["cfl"], m["t_end"])
            else:
                slot = self.batch.add(r.state, m["dx"], m["dy"], m["gamma"], m["flux"], m["cfl"],
                                      m["t_end"])
            if slot is None:
                if not self.live:  # larger than the lane's whole pool
                    self.waiting.popleft()
                    r.failed, r.lane = True, self.lane
                    self.server._finish(r)
                    continue
                return
            self.waiting.popleft()
            r.t_admit = self.server.now()
            r.lane = self.lane
            self.live[slot] = r

    def loop(self):
        srv, b = self.server, self.batch
        while not srv.abort.is_set():
            self._drain(block=not self.live)
            self._admit()
            cells = sum(r.interior for r in self.live.values())
            useful = (sum(-(-r.interior // self.tile) for r in self.live.values())
                      if self.tile else None)
            srv.blocks.set_load(self.lane, cells, useful, self.prio)
            if not self.live:
                if srv.closing.is_set() and not self.waiting and self.inbox.empty():
                    return
                continue
            grant = srv.blocks.acquire(self.lane)
            try:
                b.set_grid(grant)
                b.run(self.k, steps_per_graph=self.k)
            finally:
                srv.blocks.release(grant)
            for slot, r in list(self.live.items()):
                _, steps, active = b.info(slot)
                if active:
                    continue
                r.result = b.download(slot)
                r.steps, r.failed = steps, b.failed(slot)
                b.remove(slot)
                del self.live[slot]
                srv._finish(r)


class _Lane3D(_Lane):
    """Per-request 3D simulations, stepped round-robin: each step takes the
    CFL dt of its simulation (3D/MPI/OTvortex/cflcheck.hpp), on that
    simulation's own stream."""

    def __init__(self, server, budget_bytes):
        super().__init__(server, "3d")
        self.budget = budget_bytes
        self.used = 0
        self.live: list[list] = []
        # device bytes per padded cell of a 3D simulation, from small ones
        self.per_cell = {}
        for prec in (FP64, FP32_SPLIT):
            with Sim(3, (16, 16, 16), precision=prec) as s:
                self.per_cell[prec] = s.device_bytes / 16 ** 3

    def bytes_for(self, r):
        return int(r.state["ro"].size * self.per_cell[r.precision] * 1.02) + (1 << 20)

    def _admit(self):
        while self.waiting:
            r = self.waiting[0]
            need = self.bytes_for(r)
            if need > self.budget:  # can never fit
                self.waiting.popleft()
                r.failed, r.lane = True, "3d"
                self.server._finish(r)
                continue
            if self.used + need > self.budget:
                return
            self.waiting.popleft()
            m = r.meta
            s = Sim(3, r.state["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], gamma=m["gamma"],
                    odr=4, flux=m["flux"], nrk=3, precision=r.precision)
            s.upload(r.state)
            r.t_admit = self.server.now()
            r.lane = "3d"
            self.used += need
            self.live.append([r, s, need, 0.0])

    def loop(self):
        srv = self.server
        try:
            while not srv.abort.is_set():
                self._drain(block=not self.live)
                self._admit()
                if not self.live:
                    if srv.closing.is_set() and not self.waiting and self.inbox.empty():
                        return
                    continue
                self.round()
        finally:
            for item in self.live:
                item[1].close()

    def round(self):
        """One step of every live simulation, each on its own stream."""
        for item in list(self.live):
            r, s, need, dt = item
            m = r.meta
            dt, vmax = s.cfl(m["cfl"], min(m["dx"], m["dy"], m["dz"]), m["vfast"], dt)
            if not (math.isfinite(vmax) and dt > 0):
                r.failed = True
            else:
                s.step(dt, 1)
                r.steps += 1
            item[3] = dt
            if r.failed or r.steps >= m["steps"]:
                r.result = s.download()
                s.close()
                self.used -= need
                self.live.remove(item)
                self.server._finish(r)


# --- the server --------------------------------------------------------------
class Server:
    """Serve requests on the current GPU within `budget_bytes` of HBM.

    shares: fraction of the budget for each lane's pool ("1d", "2d64",
    "2d32", "3d").  max_inst: slots per batched lane."""

    BYTES_PER_CELL = {"1d": 312, "2d64": 472, "2d32": 352}

    def __init__(self, budget_bytes=120e9, shares=None, max_inst=256, steps_per_tick=None,
                 odr_2d=4, odr_1d=2):
        shares = shares or {"1d": 0.04, "2d64": 0.36, "2d32": 0.30, "3d": 0.30}
        spt = {"1d": 32, "2d64": 8, "2d32": 8}
        spt.update(steps_per_tick or {})
        self.budget = budget_bytes
        cap = {k: int(budget_bytes * shares[k] / self.BYTES_PER_CELL[k])
               for k in ("1d", "2d64", "2d32")}
        self.batches = {
            "1d": Batch.open1d(cap["1d"], max_inst, odr=odr_1d),
            "2d64": Batch.open(cap["2d64"], max_inst, precision=FP64, odr=odr_2d),
            "2d32": Batch.open(cap["2d32"], max_inst, precision=FP32_SPLIT, odr=odr_2d),
        }
        total = min(b.max_grid for b in self.batches.values())
        self.blocks = _Blocks(total)
        self.closing = threading.Event()
        self.abort = threading.Event()
        self._wake = threading.Event()
        self._lock = threading.Lock()
        self.done: list[Request] = []
        # the 1D lane is served first (see _Blocks); a block per 64-cell tile
        self.lanes = {k: _BatchLane(self, k, b, spt[k], prio=(k == "1d"),
                                    tile=64 if k == "1d" else None)
                      for k, b in self.batches.items()}
        self.lanes["3d"] = _Lane3D(self, budget_bytes * shares["3d"])
        self.t0 = None

    def device_bytes(self):
        return sum(b.device_bytes for b in self.batches.values())

    def now(self):
        return time.perf_counter() - self.t0

    def _finish(self, r):
        r.t_done = self.now()
        with self._lock:
            self.done.append(r)
        self._wake.set()

    @staticmethod
    def lane_of(r):
        if r.kind == "1d":
            return "1d"
        if r.kind == "2d":
            return "2d64" if r.precision == FP64 else "2d32"
        return "3d"

    def run(self, requests, realtime=True):
        """Feed the requests at their arrival times (realtime) or all at once,
        and return them completed, in completion order."""
        pending = sorted(requests, key=lambda r: r.arrival)
        self.t0 = time.perf_counter()
        for lane in self.lanes.values():
            lane.start()
        i = 0
        ok = False
        try:
            while i < len(pending):
                now = self.now()
                while i < len(pending) and (not realtime or pending[i].arrival <= now):
                    self.lanes[self.lane_of(pending[i])].inbox.put(pending[i])
                    i += 1
                if i < len(pending):
                    self._wake.wait(min(0.01, max(0.0, pending[i].arrival - now)))
                    self._wake.clear()
                self._raise_lane_errors()
            self.closing.set()
            for lane in self.lanes.values():
                while lane.is_alive():
                    lane.join(0.05)
                    self._raise_lane_errors()
            ok = True
        finally:
            self.closing.set()
            if not ok:  # stop every lane before the engines go away
                self.abort.set()
                for lane in self.lanes.values():
                    if lane.is_alive():
                        lane.join()
        self._raise_lane_errors()
        if len(self.done) != len(requests):
            raise MlauError(f"served {len(self.done)} of {len(requests)} requests")
        return list(self.done)

    def _raise_lane_errors(self):
        for lane in self.lanes.values():
            if lane.error is not None:
                raise MlauError(f"lane {lane.lane}: {lane.error}") from lane.error

    def close(self):
        self.closing.set()
        for b in self.batches.values():
            b.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# --- the one-at-a-time FP64 baseline ----------------------------------------
def solve_alone_fp64(r: Request):
    """Solve one request by itself with the plain FP64 single-problem path (the
    reference's scheme and time loop); returns (state, steps, seconds)."""
    m = r.meta
    t0 = time.perf_counter()
    steps = 0
    if r.kind == "1d":
        with Sim(1, r.state["ro"].shape, dx=m["dx"], gamma=m["gamma"], odr=m["odr"],
                 flux=m["flux"], nrk=m["nrk"]) as s:
            s.set_bx(m["bx"])
            s.set_bc(m["bc"])
            s.upload(r.state)
            dt, _ = s.cfl(m["cfl"], m["dx"], 1.0, 0.0)
            t = 0.0
            chunk = 64
            # t += dt until t >= t_end, exactly as the 1D driver's loop
            while True:
                n = 0
                while n < chunk:
                    t += dt
                    n += 1
                    if t >= m["t_end"]:
                        break
                s.step(dt, n)
                steps += n
                if t >= m["t_end"]:
                    break
            out = s.download()
    elif r.kind == "2d":
        with Sim(2, r.state["ro"].shape, dx=m["dx"], dy=m["dy"], gamma=m["gamma"], odr=4,
                 flux=m["flux"], nrk=3) as s:
            s.upload(r.state)
            t = 0.0
            while True:
                dt, vm = s.cfl(m["cfl"], min(m["dx"], m["dy"]), 0.0, 0.0)
                if not (vm > 0.0) or not math.isfinite(vm):
                    break
                if t + dt > m["t_end"]:
                    dt = m["t_end"] - t
                s.step(dt, 1)
                t += dt
                steps += 1
                if t >= m["t_end"] * (1.0 - 1e-12) or not (dt > 0.0):
                    break
            out = s.download()
    else:
        with Sim(3, r.state["ro"].shape, dx=m["dx"], dy=m["dy"], dz=m["dz"], gamma=m["gamma"],
                 odr=4, flux=m["flux"], nrk=3) as s:
            s.upload(r.state)
            dt = 0.0
            for _ in range(m["steps"]):
                dt, vm = s.cfl(m["cfl"], min(m["dx"], m["dy"], m["dz"]), m["vfast"], dt)
                s.step(dt, 1)
                steps += 1
            out = s.download()
    return out, steps, time.perf_counter() - t0


def serial_schedule(requests, exec_seconds):
    """Latencies of a one-at-a-time server: request i starts when it has
    arrived and request i-1 has finished."""
    order = sorted(range(len(requests)), key=lambda k: requests[k].arrival)
    free = 0.0
    lat = [0.0] * len(requests)
    for k in order:
        start = max(free, requests[k].arrival)
        free = start + exec_seconds[k]
        lat[k] = free - requests[k].arrival
    return lat, free


def summary(latencies, zone_updates, makespan):
    lat = np.asarray(latencies)
    return dict(p50_s=float(np.percentile(lat, 50)), p99_s=float(np.percentile(lat, 99)),
                mean_s=float(lat.mean()), zone_updates=int(zone_updates),
                makespan_s=float(makespan), zone_updates_per_s=float(zone_updates / makespan))
