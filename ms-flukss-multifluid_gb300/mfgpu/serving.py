"""Serving loop: independent heliosphere runs with continuous batching.

Requests arrive as a seeded Poisson stream.  Each request is one run of the
multi-fluid heliosphere physics (plasma MHD + 3 neutral H fluids, GLM, charge
exchange, inner solar-wind sphere, far-field inflow) in 2D on n^2 cells or in
3D on n^3 cells over [-1, 1]^d, with its own inflow speed, magnetic-field
angle and neutral/plasma density ratio, run for a fixed number of steps.

The device side is native (mf_server_*): runs are admitted while the
server's HBM arena has room, stay resident, and every admitted run of a
server advances in the same launches each iteration; runs join and leave
between iterations.  2D and 3D runs live in two servers (one space dimension
per launch) that step on separate CUDA streams, so their work overlaps.
This module only generates requests, builds initial states and drives the
loop.
"""
from __future__ import annotations

import ctypes
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import (BC_FARFIELD, MfParams, Context, Server, check, helio_params, load, make_box,
               MfFab, num_cons, run_spec, HELIO_T_INFLOW)

N2D = tuple(range(64, 513, 32))     # 2D grid sizes (cells per side)
N3D = tuple(range(32, 129, 16))     # 3D grid sizes
PATCH = {2: 32, 3: 16}


def physics_params(space_dim: int, precision: int, seed: int = 20240601) -> MfParams:
    """Physics shared by every run of one server: the heliosphere parameters
    of helio_params (seeded cross-section) in 2 or 3 dimensions; grid
    spacing, domain and far-field state are per run."""
    p = helio_params(64, seed=seed, precision=precision)
    p.space_dim = space_dim
    if space_dim == 2:
        p.domain_lo[2] = p.domain_hi[2] = 0
        p.sun_center[2] = 0.0
    return p


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


def run_physics(p: MfParams, n: int, wp, wn) -> MfParams:
    """The full parameter set of one run (what the server applies per run)."""
    q = MfParams()
    ctypes.memmove(ctypes.addressof(q), ctypes.addressof(p), ctypes.sizeof(p))
    q.dx = 2.0 / n
    for d in range(3):
        q.domain_lo[d] = 0
        q.domain_hi[d] = n - 1 if d < p.space_dim else 0
    q.bc_kind = BC_FARFIELD
    for k in range(8):
        q.bc_plasma[k] = float(wp[k])
    for k in range(5):
        q.bc_neutral1[k] = float(wn[k])
    return q


def initial_state(q: MfParams, wp, wn) -> np.ndarray:
    """Conserved state (nc, nz, ny, nx) of a run: uniform inflow plus the
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
    result: np.ndarray | None = field(default=None, repr=False)

    def cells(self) -> int:
        return self.n ** self.space_dim


def make_requests(count: int, rate: float, steps: int, seed: int = 7, dims=(2, 3)):
    """A seeded Poisson stream: exponential inter-arrival times of mean
    1/rate; dimension uniform over dims; n uniform over N2D / N3D; inflow
    speed U[0.5, 2], B angle U[0, 90] degrees, density ratio U[0.5, 4]."""
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


class Engine:
    """One server per space dimension, each on its own CUDA stream.

    serve() replays a request stream in real time: a request waits in a FIFO
    queue from its arrival until its server has a slot and arena room; every
    iteration steps each non-empty server once (one graph launch over all of
    its runs) and then waits for both; a run that has taken its steps is
    retired (state copied back) and its memory is reused by the queue."""

    def __init__(self, precision: int, hbm_budget_bytes: float, max_runs: int = 64,
                 cfl: float = 0.4, dims=(2, 3), keep_results: bool = False):
        import torch
        self.torch = torch
        self.cfl = cfl
        self.keep = keep_results
        self.ctx, self.srv, self.stream, self.phys = {}, {}, {}, {}
        per = hbm_budget_bytes / len(dims)
        for sd in dims:
            p = physics_params(sd, precision)
            self.phys[sd] = p
            self.ctx[sd] = Context(p)
            self.srv[sd] = Server(self.ctx[sd], per, max_runs)
            self.stream[sd] = torch.cuda.Stream()

    def close(self):
        for s in self.srv.values():
            s.close()
        for c in self.ctx.values():
            c.close()

    def spec_state(self, r: Request):
        wp, wn = inflow(r.speed, r.angle, r.ratio)
        q = run_physics(self.phys[r.space_dim], r.n, wp, wn)
        spec = run_spec([r.n] * r.space_dim, PATCH[r.space_dim], q.dx, self.cfl, wp, wn)
        return spec, initial_state(q, wp, wn)

    def serve(self, requests, realtime: bool = True, prepared=None):
        """Run the stream; fills t_admit / t_done (seconds from the start),
        status and (keep_results) the final states.  prepared: optional
        {rid: (spec, state)} built ahead so host set-up is not timed."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        queue = deque()
        active = {}
        prepared = dict(prepared or {})
        t0 = time.perf_counter()
        iters = 0
        while pending or queue or active:
            now = time.perf_counter() - t0
            while pending and (pending[0].arrival <= now or not realtime):
                queue.append(pending.popleft())
            for r in list(queue):  # FIFO per server, skipping requests that do not fit
                if r.rid not in prepared:
                    prepared[r.rid] = self.spec_state(r)
                spec, state = prepared[r.rid]
                rid = self.srv[r.space_dim].admit(spec, state)
                if rid is None:
                    if self.srv[r.space_dim].active() == 0:
                        raise RuntimeError(f"request {r.rid} does not fit an empty server")
                    continue
                del prepared[r.rid]
                r.t_admit = time.perf_counter() - t0
                active[(r.space_dim, rid)] = r
                queue.remove(r)
            if not active:
                if pending:
                    time.sleep(max(0.0, min(0.01, pending[0].arrival - now)))
                continue
            stepping = [sd for sd in self.srv if self.srv[sd].active() > 0]
            for sd in stepping:
                self.srv[sd].step(self.stream[sd].cuda_stream)
            for sd in stepping:
                self.srv[sd].sync(self.stream[sd].cuda_stream)
            iters += 1
            for (sd, rid), r in list(active.items()):
                steps, _, st = self.srv[sd].info(rid)
                if steps >= r.steps or st != 0:
                    r.status = st
                    out = self.srv[sd].retire(rid, want_state=self.keep,
                                              stream=self.stream[sd].cuda_stream)
                    r.t_done = time.perf_counter() - t0
                    if self.keep:
                        r.result = out
                    del active[(sd, rid)]
        return {"wall_s": time.perf_counter() - t0, "iterations": iters}


def summarize(requests, wall_s: float) -> dict:
    """p50 / p99 time to solution (completion - arrival) and aggregate
    zone-updates/s (sum of cells x steps over the makespan)."""
    tts = np.array([r.t_done - r.arrival for r in requests])
    zones = float(sum(r.cells() * r.steps for r in requests))
    return {"requests": len(requests), "p50_s": float(np.percentile(tts, 50)),
            "p99_s": float(np.percentile(tts, 99)), "mean_s": float(tts.mean()),
            "zone_updates": zones, "value": zones / wall_s, "makespan_s": wall_s,
            "failed": int(sum(1 for r in requests if r.status != 0))}
