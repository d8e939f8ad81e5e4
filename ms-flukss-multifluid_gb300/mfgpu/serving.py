"""Serving loop: independent MHD runs with continuous batching.

Requests arrive as a seeded Poisson stream.  Each request is one run, either

* 2D on n^2 cells (n in 64..512): the Orszag-Tang problem of the small
  configuration (periodic single-fluid ideal MHD, Roe 8-wave, minmod, 8-wave
  source) with the vortex velocity scaled by the request's speed, or
* 3D on n^3 cells (n in 48..128) over [-1, 1]^3: the multi-fluid heliosphere
  (plasma MHD + 3 neutral H fluids, GLM, charge exchange, inner solar-wind
  sphere, far-field inflow) with the request's inflow speed, magnetic-field
  angle and neutral/plasma density ratio,

run for a fixed number of steps.  3D grids start at 48^3: at 32^3 the inner
sphere (radius 0.1) is 1.6 cells wide and the run degenerates within tens of
steps in FP64 as well (dt falling by orders of magnitude).

The device side is native (mf_server_*): runs are admitted while a server's
HBM arena has room, stay resident, and every admitted run of a server
advances in the same launches each iteration; runs join and leave between
iterations.  This module only generates requests, builds initial states and
drives the loop.
"""
from __future__ import annotations

import ctypes
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import (BC_FARFIELD, MfParams, Context, Server, check, helio_params, load, make_box,
               MfFab, num_cons, orszag_params, run_spec, HELIO_T_INFLOW)

N2D = tuple(range(64, 513, 32))     # 2D grid sizes (cells per side)
N3D = tuple(range(48, 129, 16))     # 3D grid sizes
PATCH = {2: 32, 3: 16}


def physics_params(space_dim: int, precision: int, seed: int = 20240601) -> MfParams:
    """Physics shared by every run of one server: Orszag-Tang settings in 2D
    (periodic unit square), the heliosphere parameters of helio_params
    (seeded cross-section) in 3D; grid spacing, domain and far-field state
    are per run."""
    if space_dim == 2:
        return orszag_params(64, precision=precision)
    return helio_params(64, seed=seed, precision=precision)


def inflow(speed: float, angle_deg: float, ratio: float):
    """Far-field primitive states of a request: plasma rho 0.1, v = (-speed,
    0, 0), temperature 0.5, |B| = 0.05 at angle_deg to the flow in the x-y
    plane; the three neutral populations hold ratio * 0.1 in total (split
    1/2, 1/4, 1/4) with the plasma's velocity and temperature."""
    T = HELIO_T_INFLOW
    b = 0.05
    a = np.deg2rad(angle_deg)
    rp = 0.1
    wp = np.array([rp, -speed, 0.0, 0.0, rp * T, -b * np.cos(a), b * np.sin(a), 0.0])
    rn = ratio * rp
    wn = np.concatenate([[r, -speed, 0.0, 0.0, r * T] for r in (0.5 * rn, 0.25 * rn, 0.25 * rn)])
    return wp, wn


def run_physics(p: MfParams, n: int, wp=None, wn=None) -> MfParams:
    """The full parameter set of one run (what the server applies per run):
    2D on [0,1]^2 (periodic), 3D on [-1,1]^3 with the far-field state."""
    q = MfParams()
    ctypes.memmove(ctypes.addressof(q), ctypes.addressof(p), ctypes.sizeof(p))
    q.dx = (1.0 if p.space_dim == 2 else 2.0) / n
    for d in range(3):
        q.domain_lo[d] = 0
        q.domain_hi[d] = n - 1 if d < p.space_dim else 0
    if p.space_dim == 3:
        q.bc_kind = BC_FARFIELD
        for k in range(8):
            q.bc_plasma[k] = float(wp[k])
        for k in range(5):
            q.bc_neutral1[k] = float(wn[k])
    return q


def orszag_state(q: MfParams, speed: float) -> np.ndarray:
    """Orszag-Tang state (nc, 1, n, n) of the reference (problems/OrszagF.ChF:
    rho = gamma^2/4pi, p = gamma/4pi, v = speed (-sin 2pi y, sin 2pi x),
    B = (-sin 2pi y, sin 4pi x), Gaussian units)."""
    g = q.gamma
    n = q.domain_hi[0] + 1
    c = (np.arange(n) + 0.5) * q.dx
    Y, X = np.meshgrid(c, c, indexing="ij")
    tp = 2.0 * np.pi
    r0, p0 = g * g / (4.0 * np.pi), g / (4.0 * np.pi)
    ux, uy = -speed * np.sin(tp * Y), speed * np.sin(tp * X)
    bx, by = -np.sin(tp * Y), np.sin(2.0 * tp * X)
    U = np.zeros((num_cons(q), 1, n, n))
    U[0, 0] = r0
    U[1, 0] = r0 * ux
    U[2, 0] = r0 * uy
    U[4, 0] = p0 / (g - 1.0) + 0.5 * (r0 * (ux * ux + uy * uy) + (bx * bx + by * by) / (4.0 * np.pi))
    U[5, 0] = bx
    U[6, 0] = by
    return U


def initial_state(q: MfParams, wp, wn) -> np.ndarray:
    """Conserved state (nc, nz, ny, nx) of a 3D run: uniform inflow plus the
    inner solar-wind sphere (mf_init_helio_host)."""
    lib = load()
    nc = num_cons(q)
    hi = [q.domain_hi[0], q.domain_hi[1], q.domain_hi[2]]
    arr = np.zeros((nc, hi[2] + 1, hi[1] + 1, hi[0] + 1))
    box = make_box([0, 0, 0], hi)
    fab = MfFab(arr.ctypes.data, box, nc)
    wn = np.ascontiguousarray(wn[:5 * (q.n_fluids - 1)], dtype=np.float64)
    wp = np.ascontiguousarray(wp, dtype=np.float64)
    check(lib.mf_init_helio_host(ctypes.byref(q),
                                 wp.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                 wn.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                 ctypes.byref(fab), ctypes.byref(box)), "mf_init_helio_host")
    return arr


@dataclass
class Request:
    rid: int
    arrival: float           # seconds after the start of the stream
    space_dim: int
    n: int
    speed: float
    angle: float
    ratio: float
    steps: int
    t_admit: float = -1.0
    t_done: float = -1.0
    status: int = 0
    steps_done: int = 0
    result: np.ndarray | None = field(default=None, repr=False)

    def cells(self) -> int:
        return self.n ** self.space_dim


def make_requests(count: int, rate: float, steps: int, seed: int = 7, dims=(2, 3)):
    """A seeded Poisson stream: exponential inter-arrival times of mean
    1/rate; dimension uniform over dims; n uniform over N2D / N3D; speed
    U[0.5, 2], B angle U[0, 90] degrees, density ratio U[0.5, 4] (the last
    two used by 3D runs)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate))
        sd = int(rng.choice(dims))
        n = int(rng.choice(N2D if sd == 2 else N3D))
        out.append(Request(i, t, sd, n, float(rng.uniform(0.5, 2.0)),
                           float(rng.uniform(0.0, 90.0)), float(rng.uniform(0.5, 4.0)), steps))
    return out


def request_setup(p: MfParams, r: "Request", cfl: float):
    """(mf_run_spec, initial state) of a request on a server with physics p."""
    if r.space_dim == 2:
        q = run_physics(p, r.n)
        spec = run_spec([r.n, r.n], PATCH[2], q.dx, cfl)
        return spec, orszag_state(q, r.speed)
    wp, wn = inflow(r.speed, r.angle, r.ratio)
    q = run_physics(p, r.n, wp, wn)
    spec = run_spec([r.n] * 3, PATCH[3], q.dx, cfl, wp, wn)
    return spec, initial_state(q, wp, wn)


def lane_of(r) -> str:
    """Lane of a request: 2D runs, 3D runs up to 64^3, larger 3D runs."""
    if r.space_dim == 2:
        return "2d"
    return "3d-small" if r.n <= 64 else "3d-large"


LANE_SHARE = {"2d": 0.2, "3d-small": 0.2, "3d-large": 0.6}
# CUDA stream priority per lane (lower = more urgent): short runs first
LANE_PRIORITY = {"2d": -5, "3d-small": -5, "3d-large": 0}


class Engine:
    """Lanes of runs, each one server (one space dimension, one size class)
    with its own CUDA stream and host thread.

    serve() replays a request stream in real time: a request waits in its
    lane's FIFO queue from its arrival until the lane's server has a slot and
    arena room; each lane thread steps its server (one graph launch over all
    of the lane's runs), waits for it, retires finished runs (state copied
    back) and admits from its queue.  Lanes step independently, so a small
    run is not held to the pace of the largest one, and their launches
    overlap on the GPU (the library releases the GIL in every call)."""

    def __init__(self, precision: int, hbm_budget_bytes: float, max_runs: int = 64,
                 cfl: float = 0.4, lanes=("2d", "3d-small", "3d-large"),
                 keep_results: bool = False):
        import torch
        self.torch = torch
        self.cfl = cfl
        self.keep = keep_results
        self.ctx, self.srv, self.stream, self.phys = {}, {}, {}, {}
        share = sum(LANE_SHARE[k] for k in lanes)
        for k in lanes:
            sd = 2 if k == "2d" else 3
            p = physics_params(sd, precision)
            self.phys[k] = p
            self.ctx[k] = Context(p)
            self.srv[k] = Server(self.ctx[k], hbm_budget_bytes * LANE_SHARE[k] / share, max_runs)
            self.srv[k].set_priority(LANE_PRIORITY[k])
            self.stream[k] = torch.cuda.Stream()

    def close(self):
        for s in self.srv.values():
            s.close()
        for c in self.ctx.values():
            c.close()

    def spec_state(self, r: Request):
        return request_setup(self.phys[lane_of(r)], r, self.cfl)

    def _lane(self, k, queue, lock, t0, done_flag, prepared, stats, errors):
        srv, stream = self.srv[k], self.stream[k].cuda_stream
        active = {}
        iters = 0
        try:
            while True:
                with lock:
                    waiting = list(queue)
                for r in waiting:  # FIFO, skipping requests that do not fit yet
                    spec, state = prepared[r.rid]
                    rid = srv.admit(spec, state)
                    if rid is None:
                        if not active:
                            raise RuntimeError(f"request {r.rid} does not fit an empty lane")
                        continue
                    r.t_admit = time.perf_counter() - t0
                    active[rid] = r
                    with lock:
                        queue.remove(r)
                if not active:
                    with lock:
                        finished = done_flag[0] and not queue
                    if finished:
                        break
                    time.sleep(0.002)
                    continue
                srv.step(stream)
                srv.sync(stream)
                iters += 1
                for rid, r in list(active.items()):
                    steps, _, st = srv.info(rid)
                    if steps >= r.steps or st != 0:
                        r.status = st
                        r.steps_done = steps
                        out = srv.retire(rid, want_state=self.keep, stream=stream)
                        r.t_done = time.perf_counter() - t0
                        if self.keep:
                            r.result = out
                        del active[rid]
        except Exception as e:  # reported by serve()
            errors.append((k, repr(e)))
        stats[k] = iters

    def serve(self, requests, prepared=None):
        """Run the stream in real time; fills t_admit / t_done (seconds from
        the start), status, steps_done and (keep_results) the final states.
        prepared: optional {rid: (spec, state)} built ahead so that host
        set-up is not timed (built here otherwise, before the clock starts)."""
        import threading
        reqs = sorted(requests, key=lambda r: r.arrival)
        prepared = dict(prepared or {})
        for r in reqs:
            if r.rid not in prepared:
                prepared[r.rid] = self.spec_state(r)
        queues = {k: deque() for k in self.srv}
        lock = threading.Lock()
        done_flag = [False]
        stats, errors = {}, []
        t0 = time.perf_counter()
        threads = [threading.Thread(target=self._lane,
                                    args=(k, queues[k], lock, t0, done_flag, prepared, stats,
                                          errors), daemon=True) for k in self.srv]
        for th in threads:
            th.start()
        for r in reqs:  # arrivals
            wait = r.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            with lock:
                queues[lane_of(r)].append(r)
        with lock:
            done_flag[0] = True
        for th in threads:
            th.join()
        if errors:
            raise RuntimeError(f"serving lanes failed: {errors}")
        return {"wall_s": time.perf_counter() - t0, "iterations": stats}


def summarize(requests, wall_s: float) -> dict:
    """p50 / p99 time to solution (completion - arrival) overall and per
    lane, aggregate zone-updates/s (cells x steps taken, over the makespan)
    and the runs that stopped with an error status."""
    tts = np.array([r.t_done - r.arrival for r in requests])
    zones = float(sum(r.cells() * r.steps_done for r in requests))
    out = {"requests": len(requests), "p50_s": float(np.percentile(tts, 50)),
           "p99_s": float(np.percentile(tts, 99)), "mean_s": float(tts.mean()),
           "zone_updates": zones, "value": zones / wall_s, "makespan_s": wall_s,
           "failed": int(sum(1 for r in requests if r.status != 0))}
    lanes = {}
    for r in requests:
        lanes.setdefault(lane_of(r), []).append(r.t_done - r.arrival)
    out["lanes"] = {k: {"requests": len(v), "p50_s": float(np.percentile(v, 50)),
                        "p99_s": float(np.percentile(v, 99))} for k, v in lanes.items()}
    out["failures"] = [{"rid": r.rid, "dim": r.space_dim, "n": r.n, "status": r.status,
                        "steps": r.steps_done} for r in requests if r.status != 0]
    return out
