#!/usr/bin/env python
"""Zone-updates/s of the multi-fluid MHD level step on one GB300.

Workload (the single-GPU configuration the metric is quoted on): 3D
multi-fluid heliosphere on a 128^3 box over [-1,1]^3 split into 512 patches of
16^3 (4 ghost layers each), plasma MHD + 3 neutral H fluids (24 conserved
components), GLM cleaning, charge exchange with a seeded cross-section, an
inner solar-wind sphere, RK2, CFL 0.4.  A step advances every patch of the
level by one time step; zone-updates per step = 128^3.

Arms:
  default            this repository's CUDA path (FP64 headline, FP32-mixed beside it)
  --impl reference   the CPU restatement of the reference patch update on the
                     host cores (a bounded sample of the same workload)

Timing: warm-up steps, then exactly K steps bracketed by a barrier and
torch.cuda.synchronize(); device time from CUDA events recorded on the stream
the steps are launched on; max over ranks.  The state (>1.3 GB per array) is
larger than L2, so no flush is needed between steps.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ms-flukss-multifluid_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

METRIC = "zone-updates/s on 1 GB300 (FP64 vs FP32-mixed), % HBM peak, p50/p99 latency"
UNIT = "zone-updates/s"
N_DEFAULT = 128
PATCH_DEFAULT = 16
CFL = 0.4


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--patch", type=int, default=PATCH_DEFAULT)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-amr", action="store_true")
    ap.add_argument("--no-config1", action="store_true")
    ap.add_argument("--config1-steps", type=int, default=200)
    ap.add_argument("--amr-n0", type=int, default=48)
    ap.add_argument("--amr-steps", type=int, default=3)
    ap.add_argument("--l1-steps", type=int, default=500)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=16)
    ap.add_argument("--serve-steps", type=int, default=200)
    ap.add_argument("--serve-budget-gb", type=float, default=60.0)
    return ap.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, mx, pw = [], [], []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                pw.append(float(r[3]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        loaded = [s for s, p in zip(sm, pw) if p > 200.0] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(pw) if pw else None}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_table():
    """Per-launch DRAM bytes of each kernel kind from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic_helio.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def _build_level(mfgpu, p, boxes, torch):
    ctx = mfgpu.Context(p)
    lev = mfgpu.Level(ctx, boxes)
    host = torch.empty(lev.ndoubles, dtype=torch.float64, pin_memory=True)
    flat = host.numpy()
    flat[:] = 0.0
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, "helio")
    lev.upload(host.data_ptr())
    dt0, _, _ = lev.compute_dt()
    ch = p.factor_ch * p.dx / dt0
    cp = (ch * p.dx / p.factor_cp) ** 0.5
    ctx.set_dedner(ch, cp)
    return ctx, lev, host, dt0


def _algorithmic_bytes(kind, p, boxes, nc, rsize):
    """Minimum bytes one launch of a kernel kind must move (each value once)."""
    sd = p.space_dim
    cells = sum((hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) for lo, hi in boxes)
    faces = 0
    wline = 0
    for lo, hi in boxes:
        n = [hi[d] - lo[d] + 1 for d in range(3)]
        faces += (n[0] + 1) * n[1] * n[2]  # one direction
        wline += (n[0] + 4) * n[1] * n[2]  # primitive cells one direction's faces need
    wcells = sum((hi[0] - lo[0] + 5) * (hi[1] - lo[1] + 5) * (hi[2] - lo[2] + 5) for lo, hi in boxes)
    if kind == "flux":
        # read W once on the face stencil, write the fluxes and Bn of every face
        return wline * 8 * nc + faces * (nc + 1) * rsize
    if kind == "update":
        # read U, W and (stage 2) Uold once, read the fluxes of every face, write U
        return cells * 8 * nc * 3.5 + sd * faces * (nc + 1) * rsize
    if kind == "prim":
        return wcells * 8 * nc * 2
    if kind == "exchange":
        ghost = sum(((hi[0] - lo[0] + 9) * (hi[1] - lo[1] + 9) * (hi[2] - lo[2] + 9))
                    - (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1)
                    for lo, hi in boxes)
        return ghost * nc * 16
    return 0


def _progress(what):
    """Section marker on stderr (the JSON line on stdout is printed last)."""
    print(f"[bench] {what}", file=sys.stderr, flush=True)


def _time_steps(lev, torch, stream, steps):
    """K asynchronous level steps between CUDA events on the launching
    stream, inside an NVTX range "timed" (ncu --nvtx-include "timed/" then
    captures the timed launches only)."""
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")
    ev0.record(stream)
    for _ in range(steps):
        lev.step_async(stream.cuda_stream)
    ev1.record(stream)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


def run_ours(a):
    import numpy as np
    import torch

    import build as mfbuild
    mfbuild.build()
    import mfgpu

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    n, patch = a.n, a.patch
    boxes = mfgpu.tile_boxes(n, patch, 3)
    zones = n ** 3
    stream = torch.cuda.Stream()
    p64 = mfgpu.helio_params(n, precision=mfgpu.PREC_FP64)
    ctx, lev, host, dt0 = _build_level(mfgpu, p64, boxes, torch)
    # the project's autotuner: threads per block of each kernel kind and the
    # stage schedule (split kernels or a fused tile shape), picked by timing
    tuned = {"threads": list(lev.autotune(3)), "schedule": list(lev.schedule()),
             "flux_form": "lines" if lev.flux_form() == mfgpu.FLUX_LINES else "faces"}
    lev.seed_dt(CFL * dt0, CFL, stream.cuda_stream)
    for _ in range(a.warmup):
        lev.step_async(stream.cuda_stream)
    torch.cuda.synchronize()
    st, _, _, _ = lev.result(stream.cuda_stream)
    mfgpu.check(st, "warm-up steps")

    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    ms = _time_steps(lev, torch, stream, a.steps)
    barrier()
    clocks = sampler.stop()
    st, dt_min, _, _ = lev.result(stream.cuda_stream)
    mfgpu.check(st, "timed steps")
    ms_all = ms
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_all = float(t.item())
    value = ws * zones * a.steps / (ms_all * 1e-3)
    launches = lev.launches_per_step()

    # per-launch device times of one step (CUDA events on the launching stream)
    prof = lev.profile_step(CFL * dt_min)
    by_kind = {}
    for kind, t in prof:
        tot, cnt = by_kind.get(kind, (0.0, 0))
        by_kind[kind] = (tot + t, cnt + 1)
    step_ms_prof = sum(t for _, t in prof)
    dom = max(by_kind, key=lambda k: by_kind[k][0])
    dom_avg_ms = by_kind[dom][0] / by_kind[dom][1]
    nc = ctx.nc
    alg = _algorithmic_bytes(dom, p64, boxes, nc, 8)
    peak, peak_kind = _peaks()
    achieved = alg / (dom_avg_ms * 1e-3) / 1e9
    traffic = _traffic_table().get(f"fp64_{dom}") if n == N_DEFAULT else None

    # end to end through the C ABI with host buffers: H2D of the level's valid
    # state (pinned, packed without ghosts), one step (mf_level_step fills the
    # ghosts by its exchange and returns the new dt on the host), D2H of the
    # valid state
    e2e_steps = max(1, a.e2e_steps)
    vhost = torch.empty(lev.valid_doubles(), dtype=torch.float64, pin_memory=True)
    nbytes = vhost.numel() * 8
    dt_e = CFL * dt_min
    lev.upload(host.data_ptr(), stream.cuda_stream)
    lev.download_valid(vhost.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(e2e_steps):
        lev.upload_valid(vhost.data_ptr(), stream.cuda_stream)
        st, ndt, _, _ = lev.step(dt_e, stream.cuda_stream)
        mfgpu.check(st, "e2e step")
        lev.download_valid(vhost.data_ptr(), stream.cuda_stream)
        dt_e = CFL * ndt
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    e2e_ms = e0.elapsed_time(e1)
    e2e_value = ws * zones * e2e_steps / (max(e2e_ms * 1e-3, wall))

    fast = None
    if not a.no_mixed:
        pf = mfgpu.helio_params(n, precision=mfgpu.PREC_FP64_FAST)
        ctxf, levf, hostf, dtf = _build_level(mfgpu, pf, boxes, torch)
        tunedf = {"threads": list(levf.autotune(3)), "schedule": list(levf.schedule()),
                  "flux_form": "lines" if levf.flux_form() == mfgpu.FLUX_LINES else "faces"}
        levf.seed_dt(CFL * dtf, CFL, stream.cuda_stream)
        for _ in range(a.warmup):
            levf.step_async(stream.cuda_stream)
        torch.cuda.synchronize()
        barrier()
        msf = _time_steps(levf, torch, stream, a.steps)
        barrier()
        stf, _, _, _ = levf.result(stream.cuda_stream)
        mfgpu.check(stf, "fast fp64 steps")
        proff = levf.profile_step(CFL * dtf)
        fast = {"value": ws * zones * a.steps / (msf * 1e-3), "ms_per_step": msf / a.steps,
                "speedup_vs_fp64": (ws * zones * a.steps / (msf * 1e-3)) / value,
                "per_kind_ms": {}, "autotuned": tunedf,
                "dtype": "f64 with fused multiply-adds and reused reciprocals"}
        for kind, t in proff:
            fast["per_kind_ms"][kind] = fast["per_kind_ms"].get(kind, 0.0) + t
        levf.close()
        ctxf.close()
        del hostf

    mixed_forms = {}
    if not a.no_mixed:
        # the mixed-precision forms: "mixed" keeps the charge-exchange rates in
        # FP64 (MF_PREC_MIXED); "mixed_ce32" computes them in FP32 as well
        forms = (("mixed", mfgpu.PREC_MIXED,
                  "f32 reconstruction, Riemann fluxes and CFL wave speeds; f64 conserved state, "
                  "flux-divergence accumulation, pressure recovery (also in the CFL wave "
                  "speeds), positivity fix and charge-exchange rates"),
                 ("mixed_ce32", mfgpu.PREC_MIXED_CE32,
                  "f32 reconstruction, Riemann fluxes, CFL wave speeds and charge-exchange "
                  "rates; f64 conserved state, flux-divergence accumulation, pressure recovery "
                  "(also in the CFL wave speeds) and positivity fix"))
        built = {}
        for name, prec, dtype in forms:
            pm = mfgpu.helio_params(n, precision=prec)
            ctxm, levm, hostm, dtm = _build_level(mfgpu, pm, boxes, torch)
            tunedm = {"threads": list(levm.autotune(3)), "schedule": list(levm.schedule()),
                      "overlap_chunks": levm.overlap()}
            levm.seed_dt(CFL * dtm, CFL, stream.cuda_stream)
            for _ in range(a.warmup):
                levm.step_async(stream.cuda_stream)
            torch.cuda.synchronize()
            barrier()
            msm = _time_steps(levm, torch, stream, a.steps)
            barrier()
            stm, _, _, _ = levm.result(stream.cuda_stream)
            mfgpu.check(stm, f"{name} steps")
            vm = ws * zones * a.steps / (msm * 1e-3)
            profm = levm.profile_step(CFL * dtm)
            per_kind = {}
            for kind, t in profm:
                per_kind[kind] = per_kind.get(kind, 0.0) + t
            mixed_forms[name] = {
                "value": vm, "ms_per_step": msm / a.steps, "speedup_vs_fp64": vm / value,
                "step_hbm_frac": (vm * 16 * nc / 1e9) / peak, "per_kind_ms": per_kind,
                "launches_per_step": levm.launches_per_step(), "autotuned": tunedm,
                "dtype": dtype}
            built[name] = (ctxm, levm, hostm)
        # accuracy: same initial state, same dt sequence, FP64 and both forms
        nsteps_acc = max(1, a.l1_steps)
        flat0 = np.zeros(lev.ndoubles)
        for i in range(len(boxes)):
            flo, fhi = lev.fab_box(i)
            lev.patch_view(flat0, i)[:] = mfgpu.init_host_fab(p64, flo, fhi, "helio")
        lev.upload(flat0.ctypes.data)
        lev.set_time(0.0)
        for ctxm, levm, _ in built.values():
            levm.upload(flat0.ctypes.data)
            levm.set_time(0.0)
        ch = p64.factor_ch * p64.dx / dt0
        cp = (ch * p64.dx / p64.factor_cp) ** 0.5
        dt = CFL * dt0
        _progress("mixed accuracy")
        acc_done, acc_error = 0, None
        for _ in range(nsteps_acc):
            ctx.set_dedner(ch, cp)
            sts = {}
            for name, (ctxm, levm, _) in built.items():
                ctxm.set_dedner(ch, cp)
                sts[name] = levm.step(dt, allow_error=True)[0]
            st, ndt, _, _ = lev.step(dt, allow_error=True)
            if st != 0 or any(v != 0 for v in sts.values()):
                acc_error = {"step": acc_done + 1, "fp64_status": int(st),
                             **{f"{k}_status": int(v) for k, v in sts.items()}}
                break
            acc_done += 1
            ch = p64.factor_ch * p64.dx / ndt
            cp = (ch * p64.dx / p64.factor_cp) ** 0.5
            dt = CFL * ndt
        a64 = np.zeros(lev.ndoubles)
        lev.download(a64.ctypes.data)
        ng = ctx.ng
        for name, (ctxm, levm, _) in built.items():
            amx = np.zeros(lev.ndoubles)
            levm.download(amx.ctypes.data)
            num, den = {}, {}
            for i in range(len(boxes)):
                g64 = lev.patch_view(a64, i)[:, ng:-ng, ng:-ng, ng:-ng]
                gmx = lev.patch_view(amx, i)[:, ng:-ng, ng:-ng, ng:-ng]
                qs = {"rho": (g64[0], gmx[0]),
                      "rho_n1": (g64[9], gmx[9]), "rho_n2": (g64[14], gmx[14]),
                      "rho_n3": (g64[19], gmx[19]),
                      "absB": (np.sqrt(g64[5] ** 2 + g64[6] ** 2 + g64[7] ** 2),
                               np.sqrt(gmx[5] ** 2 + gmx[6] ** 2 + gmx[7] ** 2))}
                ke64 = 0.5 * (g64[1] ** 2 + g64[2] ** 2 + g64[3] ** 2) / g64[0]
                kemx = 0.5 * (gmx[1] ** 2 + gmx[2] ** 2 + gmx[3] ** 2) / gmx[0]
                b64 = (g64[5] ** 2 + g64[6] ** 2 + g64[7] ** 2) / (8 * np.pi)
                bmx = (gmx[5] ** 2 + gmx[6] ** 2 + gmx[7] ** 2) / (8 * np.pi)
                qs["p"] = ((2.0 / 3.0) * (g64[4] - ke64 - b64),
                           (2.0 / 3.0) * (gmx[4] - kemx - bmx))
                for k, (x, y) in qs.items():
                    num[k] = num.get(k, 0.0) + float(np.sum(np.abs(y - x)))
                    den[k] = den.get(k, 0.0) + float(np.sum(np.abs(x)))
            mixed_forms[name]["l1_rel_vs_fp64"] = {k: num[k] / den[k] for k in num}
            mixed_forms[name]["l1_steps"] = acc_done
            mixed_forms[name]["l1_error"] = acc_error
            levm.close()
            ctxm.close()

    _progress("config 1")
    c1_res = None if a.no_config1 else run_config1(mfgpu, torch, stream, a)
    _progress("amr")
    amr_res = None if a.no_amr else run_amr(mfgpu, torch, stream, a)
    _progress("serving")
    serve_res = None if a.no_serve else run_serving(mfgpu, torch, a)
    _progress("cpu baseline")

    cpu = None
    if not a.no_cpu_baseline and rank == 0 and ws == 1:
        cpu = cpu_baseline(n, patch, min_seconds=10.0, max_steps=30)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_all / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {**_workload_config(n, patch, len(boxes)),
                   "l2": "inputs larger than L2 (state arrays > 1.3 GB); no flush",
                   "parallelism": f"{ws} independent replica(s), one per GPU"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "steps": e2e_steps,
                "path": "mf_level_upload_valid (pinned host, valid cells) + mf_level_step + "
                        "mf_level_download_valid"},
        "gpu_launches": launches * a.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg, "avg_launch_ms": dom_avg_ms,
                     "step_hbm_frac": (value * 16 * nc / 1e9) / peak,
                     "per_kind_ms": {k: v[0] for k, v in by_kind.items()},
                     "profiled_step_ms": step_ms_prof,
                     # the bound that binds: the FP64 pipe (2 FP64 instructions per SM per
                     # clock on GB300), measured by ncu on this kernel (committed profile)
                     "fp64_pipe_active": _traffic_table().get(f"fp64_pipe_active_{dom}")
                     if n == N_DEFAULT else None,
                     "fp64_pipe_source": "ncu sm__pipe_fp64_cycles_active of this kernel on "
                                         "the 64-patch case of this workload"},
        "clocks": clocks,
        "autotuned": tuned,
    }
    if fast is not None:
        line["fp64_fast"] = fast
    for name, res in mixed_forms.items():
        line[name] = res
    if c1_res is not None:
        line["config1"] = c1_res
    if amr_res is not None:
        line["amr"] = amr_res
    if serve_res is not None:
        line["serving"] = serve_res
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line))
    lev.close()
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


AMR_TAG_STEPS = 60      # base-grid steps before tagging (t ~ 0.19: shocks have formed)
AMR_THRESHOLD = 0.3     # undivided relative density gradient
AMR_SEED = 20240601


def run_config1(mfgpu, torch, stream, a):
    """Config 1: 2D single-fluid ideal MHD on one 256^2 periodic patch over
    [0,1]^2 with 4 ghost layers (Orszag-Tang, problems/OrszagF.ChF), Roe
    8-wave, minmod, 8-wave source, RK2, CFL 0.4: the patch as a one-patch
    level (its periodic images through the level's exchange), autotuned,
    K steps between CUDA events after 3 warm-up steps, FP64 and mixed.  Beside
    it the oracle on the same patch for a bounded sample of steps (one patch:
    one host thread does the work)."""
    import numpy as np
    n, steps = 256, max(1, a.config1_steps)
    boxes = [((0, 0, 0), (n - 1, n - 1, 0))]
    res = {"config": "Orszag-Tang 256^2 periodic, 1 patch + 4 ghosts, single-fluid ideal MHD, "
                     "Roe 8-wave, minmod, 8-wave source, RK2, CFL 0.4",
           "zones_per_step": n * n, "steps": steps}
    p64 = None
    for name, prec in (("fp64", mfgpu.PREC_FP64), ("mixed", mfgpu.PREC_MIXED)):
        p = mfgpu.orszag_params(n, mfgpu.TA_RK2, prec)
        if prec == mfgpu.PREC_FP64:
            p64 = p
        ctx = mfgpu.Context(p)
        lev = mfgpu.Level(ctx, boxes)
        flat = np.zeros(lev.ndoubles)
        flo, fhi = lev.fab_box(0)
        lev.patch_view(flat, 0)[:] = mfgpu.init_host_fab(p, flo, fhi, "orszag")
        lev.upload(flat.ctypes.data)
        lev.autotune(3)
        lev.upload(flat.ctypes.data)
        dt0 = lev.compute_dt()[0]
        lev.seed_dt(CFL * dt0, CFL, stream.cuda_stream)
        for _ in range(3):
            lev.step_async(stream.cuda_stream)
        torch.cuda.synchronize()
        ms = _time_steps(lev, torch, stream, steps)
        st = lev.result(stream.cuda_stream)[0]
        mfgpu.check(st, f"config 1 {name} steps")
        res[name] = {"value": n * n * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                     "launches_per_step": lev.launches_per_step()}
        lev.close()
        ctx.close()
    res["mixed"]["speedup_vs_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    res["value"] = res["fp64"]["value"]
    # the oracle on the same patch: a bounded sample of level steps
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    ng = pyoracle.num_ghost(p64)
    flo, fhi = pyoracle.grow(boxes[0][0], boxes[0][1], ng, 2)
    U = np.zeros(pyoracle.fab_shape(flo, fhi, pyoracle.num_cons(p64)))
    pyoracle.init_orszag(p64, U, flo, fhi, boxes[0][0], boxes[0][1])
    dt = CFL * pyoracle.compute_dt(p64, U, flo, fhi, boxes[0][0], boxes[0][1])[1]
    nst = 20
    t0 = time.perf_counter()
    for _ in range(nst):
        st, ndt, _, _ = pyoracle.level_step(p64, [U], [(flo, fhi)], boxes, dt, 1)
        assert st == 0, st
        dt = CFL * ndt
    el = time.perf_counter() - t0
    res["cpu_oracle"] = {"value": n * n * nst / el, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{nst} steps of the patch, {el:.1f} s"}
    return res


def run_amr(mfgpu, torch, stream, a):
    """Batched AMR hierarchy: a three-dimensional Orszag-Tang vortex on an
    n0^3 base grid, 3 levels with refinement ratios 2 then 4, patches of
    8/16/24/32 cells on a side drawn from a seeded distribution where the
    undivided relative density gradient is >= 0.3, properly nested.  The
    levels are coupled by mf_hier_step: a hierarchy step is 1, 2 and 8 steps
    of levels 0, 1, 2 (subcycling) with the coarse-fine ghosts interpolated
    in space and time before every fine step, the flux registers fed by every
    level step, and reflux plus average down when a finer level catches up.
    Every level steps in batched launches replayed from a CUDA graph with
    autotuned block shapes.  Beside it: the patches of level 1 stepped one
    mf_patch_update call each (the per-patch form of the reference's level
    loop)."""
    import numpy as np
    from mfgpu import amr

    n0 = a.amr_n0
    p0 = amr.orszag3d_params(n0)
    base = mfgpu.tile_boxes(n0, 16, 3)
    ctx0 = mfgpu.Context(p0)
    lev0 = mfgpu.Level(ctx0, base)
    g0 = amr.orszag3d_state(p0, (0, 0, 0), (n0 - 1,) * 3)
    buf0 = amr.fill_level_buffer(lev0, g0, 1)  # held while the library reads it
    lev0.upload(buf0.ctypes.data)
    dt0 = lev0.compute_dt()[0]
    lev0.seed_dt(CFL * dt0, CFL, stream.cuda_stream)
    for _ in range(AMR_TAG_STEPS):
        lev0.step_async(stream.cuda_stream)
    torch.cuda.synchronize()
    mfgpu.check(lev0.result(stream.cuda_stream)[0], "base-grid steps")
    out = np.zeros(lev0.ndoubles)
    lev0.download(out.ctypes.data)
    ng = ctx0.ng
    U0 = np.zeros((ctx0.nc, n0, n0, n0))
    for i, (lo, hi) in enumerate(base):
        U0[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = \
            lev0.patch_view(out, i)[:, ng:-ng, ng:-ng, ng:-ng]
    lev0.close()
    ctx0.close()
    tags = amr.relgrad_tags(U0[0], AMR_THRESHOLD)
    hier = amr.build_hierarchy(tags, ratios=(2, 4), seed=AMR_SEED)
    ratios = [2, 4]

    def make(prec):
        pb = amr.orszag3d_params(n0, precision=prec)
        params = [amr.level_params(pb, R) for (R, n, boxes) in hier]
        refine = {id(p): R for p, (R, n, boxes) in zip(params, hier)}

        def init(p, lo, hi):
            return amr.prolong_fab(U0, refine[id(p)], lo, hi)

        dh = amr.DeviceHierarchy(mfgpu, params, [b for (R, n, b) in hier], ratios, init)
        shapes = [lev.autotune(3) for lev in dh.levels]
        return dh, shapes

    res = {}
    zones = 0
    for name in ("fp64", "mixed"):
        dh, shapes = make(mfgpu.PREC_FP64 if name == "fp64" else mfgpu.PREC_MIXED)
        zones = dh.cells_per_step()
        dt = CFL * dh.compute_dt()
        for _ in range(max(1, min(a.warmup, 2))):
            dt = CFL * dh.step(dt, stream.cuda_stream)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.amr_steps):
            dt = CFL * dh.step(dt, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.amr_steps
        res[name] = {"value": zones / (ms * 1e-3), "ms_per_hierarchy_step": ms,
                     "gpu_launches_per_hierarchy_step": dh.hier.launches_per_step()}
        if name == "fp64":
            info = []
            for lv, ((R, n, boxes), lev) in enumerate(zip(hier, dh.levels)):
                sizes = {}
                for lo, hi in boxes:
                    s_ = hi[0] - lo[0] + 1
                    sizes[str(s_)] = sizes.get(str(s_), 0) + 1
                e = {"refinement": R, "domain": n, "patches": len(boxes),
                     "cells": lev.ncells, "patch_sizes": sizes,
                     "threads_prim_flux_update": list(shapes[lv])}
                if lv > 0:
                    e["coupling_to_coarser"] = dh.hier.info(lv - 1)
                info.append(e)
            res["levels"] = info
            # per-patch calls: every patch of level 1 once (mf_patch_update
            # returns the patch's dt to the host, as updateState does)
            ctx1, lev1 = dh.ctxs[1], dh.levels[1]
            boxes1 = hier[1][2]
            t0 = time.perf_counter()
            for i, (lo, hi) in enumerate(boxes1):
                flo, fhi = lev1.fab_box(i)
                ctx1.patch_update(lev1.patch_fab_ptr(i), flo, fhi, lo, hi, 1e-9)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            lev1.seed_dt(1e-9, CFL, stream.cuda_stream)
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(3):
                lev1.step_async(stream.cuda_stream)
            ev1.record(stream)
            torch.cuda.synchronize()
            lev_ms = ev0.elapsed_time(ev1) / 3
            res["per_patch_calls"] = {
                "level": 1, "patches": len(boxes1), "value": lev1.ncells / wall,
                "batched_level_value": lev1.ncells / (lev_ms * 1e-3),
                "batched_speedup": (lev1.ncells / (lev_ms * 1e-3)) / (lev1.ncells / wall),
                "path": "one mf_patch_update per patch (host-synchronous, as the reference's "
                        "per-patch loop) vs the batched level step"}
        dh.close()
    res["value"] = res["fp64"]["value"]
    res["zone_updates_per_hierarchy_step"] = zones
    res["mixed_speedup"] = res["mixed"]["value"] / res["fp64"]["value"]
    res["config"] = (f"3D Orszag-Tang (single-fluid ideal MHD, Roe 8-wave, minmod, 8-wave "
                     f"source, RK2), base {n0}^3, ratios 2,4, tags |relgrad rho| >= "
                     f"{AMR_THRESHOLD} after {AMR_TAG_STEPS} base steps, patch sizes "
                     f"{list(amr.SIZES)} seeded, properly nested; levels coupled by "
                     f"mf_hier_step (subcycled 1/2/8, coarse-fine ghosts interpolated in "
                     f"space and time, reflux, average down)")
    return res


SERVE_RATE = 20.0      # requests per second (Poisson)
SERVE_SEED = 7


def run_serving(mfgpu, torch, a):
    """Serving: a seeded Poisson stream (mean 20 requests/s) of independent
    heliosphere runs, each 2D on n^2 (n in 64..512) or 3D on n^3 (n in
    32..128) over [-1,1]^d with inflow speed U[0.5,2], B angle U[0,90] deg and
    neutral/plasma density ratio U[0.5,4], each for the same number of steps.
    Runs are admitted by HBM footprint into one server per dimension, stay
    resident, and every admitted run of a server advances in the same launches
    each iteration (continuous batching).  Time to solution = completion -
    arrival, in real time; initial states are built before the clock starts."""
    from mfgpu import serving
    out = {}
    for name, prec in (("fp64", mfgpu.PREC_FP64), ("mixed", mfgpu.PREC_MIXED)):
        reqs = serving.make_requests(a.serve_requests, SERVE_RATE, a.serve_steps,
                                     seed=SERVE_SEED)
        eng = serving.Engine(prec, a.serve_budget_gb * 1e9, max_runs=64)
        prepared = {r.rid: eng.spec_state(r) for r in reqs}
        torch.cuda.synchronize()
        info = eng.serve(reqs, prepared=prepared)
        torch.cuda.synchronize()
        summ = serving.summarize(reqs, info["wall_s"])
        summ["iterations"] = info["iterations"]
        summ["mean_queue_s"] = float(sum(r.t_admit - r.arrival for r in reqs) / len(reqs))
        out[name] = summ
        eng.close()
    out["value"] = out["fp64"]["value"]
    out["unit"] = UNIT
    out["config"] = (f"{a.serve_requests} requests, Poisson {SERVE_RATE}/s (seed {SERVE_SEED}), "
                     f"{a.serve_steps} steps each; 2D requests: periodic Orszag-Tang (single-fluid "
                     "ideal MHD, 8-wave source) on n^2, n in 64..512 (patches 32^2), the vortex "
                     "velocity scaled by the request's inflow speed; 3D requests: the heliosphere "
                     "(plasma + 3 neutral fluids, GLM, charge exchange) on n^3, n in 48..128 "
                     "(patches 16^3) with the request's inflow speed, B angle and density ratio; "
                     "HBM budget "
                     f"{a.serve_budget_gb:g} GB per precision, lanes (one server, stream and "
                     "host thread each): 2D, 3D n<=64, 3D n>64")
    return out


def _workload_config(n, patch, npatch):
    """The workload as both arms name it."""
    return {"workload": f"3D multi-fluid heliosphere {n}^3 on [-1,1]^3, {npatch} patches of "
                        f"{patch}^3 + 4 ghosts, plasma MHD + 3 neutral H fluids (24 comps), GLM, "
                        "charge exchange, bipolar inner sphere, RK2, CFL 0.4",
            "zones_per_step": n ** 3, "patches": npatch, "patch": patch}


def cpu_baseline(n, patch, min_seconds=10.0, max_steps=30, warmup=1, fixed_steps=None):
    """The oracle (C restatement of the reference patch update, OpenMP over
    patches as AMRLevelIdealMHD::stepOMP) on the whole workload: every patch
    of the level, initial state from the oracle's own set-up, the level's dt
    chain (cfl * dt_min capped at max_dt_growth times the previous dt) and
    GLM speeds from each step's dt_min.  Loads only the oracle library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    p = pyoracle.helio_params(n)
    boxes = pyoracle.tile_boxes(n, patch, 3)
    ng = pyoracle.num_ghost(p)
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = pyoracle.grow(lo, hi, ng, 3)
        arrays.append(pyoracle.helio_fab(p, flo, fhi))
        fboxes.append((flo, fhi))
    threads = os.cpu_count() or 1
    dmin = min(pyoracle.compute_dt(p, a, fb[0], fb[1], b[0], b[1])[1]
               for a, fb, b in zip(arrays, fboxes, boxes))
    dt = CFL * dmin

    def step(dt, dmin, t):
        ch = p.factor_ch * p.dx / dmin
        p.dedner_ch, p.dedner_cp = ch, (ch * p.dx / p.factor_cp) ** 0.5
        st, ndt, _, _ = pyoracle.level_step(p, arrays, fboxes, boxes, dt, threads, time=t)
        assert st == 0, st
        return min(CFL * ndt, p.max_dt_growth * dt), ndt, t + dt

    t = 0.0
    for _ in range(warmup):
        dt, dmin, t = step(dt, dmin, t)
    steps = 0
    t0 = time.perf_counter()
    while True:
        dt, dmin, t = step(dt, dmin, t)
        steps += 1
        el = time.perf_counter() - t0
        if fixed_steps is not None:
            if steps >= fixed_steps:
                break
        elif el >= min_seconds or steps >= max_steps:
            break
    el = time.perf_counter() - t0
    zones = n ** 3
    return {"value": zones * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the whole workload ({len(boxes)} patches, {zones} zones), {steps} level "
                      f"steps after {warmup} warm-up, {el:.1f} s",
            "threads": pyoracle.max_threads()}


def run_reference(a):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    cb = cpu_baseline(a.n, a.patch, warmup=max(1, a.warmup), fixed_steps=max(1, a.steps))
    npatch = (a.n // a.patch) ** 3
    line = {
        "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": _workload_config(a.n, a.patch, npatch),
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    a = _args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
