"""Serving: independent runs stepped together in shared launches.

GPU tests: a run inside a server matches the oracle's level step; a run's
result is bitwise the same alone and in a mix of other runs that join and
leave while it runs; the engine drains a small request stream.  CPU tests:
request generation and per-run parameters.
"""
import numpy as np
import pytest

import mfgpu
from mfgpu import serving
from helpers import rel_err

RTOL = 1e-12


def test_requests_are_seeded_and_in_range():
    a = serving.make_requests(50, 20.0, 200, seed=3)
    b = serving.make_requests(50, 20.0, 200, seed=3)
    assert [(r.arrival, r.n, r.speed) for r in a] == [(r.arrival, r.n, r.speed) for r in b]
    assert all(0.5 <= r.speed <= 2.0 and 0.0 <= r.angle <= 90.0 and 0.5 <= r.ratio <= 4.0
               for r in a)
    assert all((r.n in serving.N2D) if r.space_dim == 2 else (r.n in serving.N3D) for r in a)
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert np.all(gaps > 0) and 0.02 < gaps.mean() < 0.1


def test_inflow_state():
    wp, wn = serving.inflow(1.5, 90.0, 2.0)
    assert wp[1] == -1.5 and abs(wp[5]) < 1e-15 and wp[6] == pytest.approx(0.05)
    assert sum(wn[0::5]) == pytest.approx(2.0 * wp[0])
    p = serving.physics_params(3, mfgpu.PREC_FP64)
    q = serving.run_physics(p, 48, wp, wn)
    U = serving.initial_state(q, wp, wn)
    assert U.shape == (mfgpu.num_cons(p), 48, 48, 48)
    assert np.allclose(U[0, 0, 0, 0], wp[0])


def test_orszag_request_state():
    """The 2D request state is the reference's Orszag-Tang set-up with the
    velocity scaled by the request's speed."""
    p = serving.physics_params(2, mfgpu.PREC_FP64)
    q = serving.run_physics(p, 32)
    U = serving.orszag_state(q, 1.0)
    ref = mfgpu.init_host_fab(q, [0, 0, 0], [31, 31, 0], "orszag")
    assert np.allclose(U, ref, rtol=1e-13, atol=1e-14)
    U2 = serving.orszag_state(q, 2.0)
    assert np.allclose(U2[1:3], 2.0 * U[1:3])


def _run(sd, n, speed=1.0, angle=30.0, ratio=2.0, prec=mfgpu.PREC_FP64, cfl=0.4):
    p = serving.physics_params(sd, prec)
    r = serving.Request(0, 0.0, sd, n, speed, angle, ratio, 1)
    spec, U0 = serving.request_setup(p, r, cfl)
    q = serving.run_physics(p, n, *(serving.inflow(speed, angle, ratio) if sd == 3 else ()))
    return p, q, spec, U0


@pytest.mark.gpu
@pytest.mark.parametrize("sd,n,patch", [(2, 48, 16), (3, 32, 16)])
def test_server_run_matches_oracle(gpulib, oracle, sd, n, patch):
    """Two steps, each from the oracle's state: the run is admitted, takes
    one step in the server and is compared with the oracle's level step at
    the per-step tolerance."""
    p, q, spec, U0 = _run(sd, n)
    spec.patch = patch
    ctx = mfgpu.Context(p)
    srv = mfgpu.Server(ctx, 2e9, 4)
    boxes = mfgpu.tile_boxes(n, patch, sd)
    ng = ctx.ng

    def valid(a):
        return a[:, :, ng:-ng, ng:-ng] if sd == 2 else a[:, ng:-ng, ng:-ng, ng:-ng]

    def window(U, lo, hi):
        if sd == 2:
            return U[:, :, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
        return U[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]

    state = U0
    for step in range(2):
        # oracle: the run's patches with zero ghosts, as the server holds them
        arrays, fboxes = [], []
        for lo, hi in boxes:
            flo, fhi = mfgpu.grow(lo, hi, ng, sd)
            a = np.zeros(mfgpu.fab_shape(flo, fhi, ctx.nc))
            valid(a)[...] = window(state, lo, hi)
            arrays.append(a)
            fboxes.append((flo, fhi))
        dmin = min(oracle.compute_dt(q, a, fb[0], fb[1], b[0], b[1])[1]
                   for a, fb, b in zip(arrays, fboxes, boxes))
        ch = q.factor_ch * q.dx / dmin
        q.dedner_ch, q.dedner_cp = ch, float(np.sqrt(ch * q.dx / q.factor_cp))
        st, ndt_o, _, _ = oracle.level_step(q, arrays, fboxes, boxes, spec.cfl * dmin)
        assert st == 0
        rid = srv.admit(spec, state)
        srv.step()
        srv.sync()
        steps, ndt_g, st_g = srv.info(rid)
        assert steps == 1 and st_g == 0
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        out = srv.retire(rid)
        nxt = np.zeros_like(state)
        for (lo, hi), a in zip(boxes, arrays):
            assert np.all(rel_err(window(out, lo, hi), valid(a)) <= RTOL), (step, lo)
            window(nxt, lo, hi)[...] = valid(a)
        state = nxt
    assert srv.active() == 0
    srv.close()
    ctx.close()


def _alone(sd, spec, U0, steps, prec):
    p = serving.physics_params(sd, prec)
    ctx = mfgpu.Context(p)
    srv = mfgpu.Server(ctx, 2e9, 4)
    rid = srv.admit(spec, U0)
    for _ in range(steps):
        srv.step()
    srv.sync()
    assert srv.info(rid)[2] == 0
    out = srv.retire(rid)
    srv.close()
    ctx.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("sd,prec", [(2, mfgpu.PREC_FP64), (2, mfgpu.PREC_MIXED),
                                     (3, mfgpu.PREC_MIXED)])
def test_alone_equals_mix(gpulib, sd, prec):
    """Run a takes 12 steps alone, then 12 steps in a server where run b
    is admitted with it, run c joins after 4 steps and b leaves after 8:
    a's final state is bitwise the same."""
    n0, n1, n2 = (64, 96, 48) if sd == 2 else (32, 48, 32)
    _, _, sa, Ua = _run(sd, n0, 1.0, 30.0, 2.0, prec)
    _, _, sb, Ub = _run(sd, n1, 1.7, 80.0, 0.7, prec)
    _, _, sc, Uc = _run(sd, n2, 0.6, 10.0, 3.5, prec)
    ref = _alone(sd, sa, Ua, 12, prec)
    p = serving.physics_params(sd, prec)
    ctx = mfgpu.Context(p)
    srv = mfgpu.Server(ctx, 4e9, 8)
    rb = srv.admit(sb, Ub)
    ra = srv.admit(sa, Ua)
    for k in range(12):
        if k == 4:
            rc = srv.admit(sc, Uc)
        if k == 8:
            srv.sync()
            srv.retire(rb, want_state=False)
        srv.step()
    srv.sync()
    assert srv.info(ra)[0] == 12 and srv.info(rc)[0] == 8
    out = srv.retire(ra)
    assert np.array_equal(out, ref)
    srv.close()
    ctx.close()


@pytest.mark.gpu
def test_admission_by_footprint(gpulib):
    """A budget that holds one 3D run: the second waits (MF_ERR_NO_ROOM)
    until the first retires."""
    _, _, s1, U1 = _run(3, 48)
    p = serving.physics_params(3, mfgpu.PREC_FP64)
    ctx = mfgpu.Context(p)
    probe = mfgpu.Server(ctx, 1e8, 2)
    need = probe.run_bytes(s1)
    probe.close()
    srv = mfgpu.Server(ctx, 1.6 * need * 1.2, 4)
    r1 = srv.admit(s1, U1)
    assert r1 is not None
    assert srv.admit(s1, U1) is None
    srv.step()
    srv.sync()
    srv.retire(r1, want_state=False)
    assert srv.admit(s1, U1) is not None
    srv.close()
    ctx.close()


@pytest.mark.gpu
def test_engine_drains_stream(gpulib):
    reqs = serving.make_requests(6, 50.0, 6, seed=5)
    for r in reqs:
        r.n = 64 if r.space_dim == 2 else 32
    eng = serving.Engine(mfgpu.PREC_MIXED, 6e9, max_runs=8, keep_results=True)
    info = eng.serve(reqs)
    assert sum(info["iterations"].values()) >= 6
    for r in reqs:
        assert r.status == 0 and r.t_done >= r.t_admit >= 0.0
        assert np.all(np.isfinite(r.result))
    # the first request alone gives the same state
    r = reqs[0]
    spec, U0 = eng.spec_state(r)
    ref = _alone(r.space_dim, spec, U0, r.steps, mfgpu.PREC_MIXED)
    assert all(q.steps_done == q.steps for q in reqs)
    assert np.array_equal(ref, r.result)
    s = serving.summarize(reqs, info["wall_s"])
    assert s["failed"] == 0 and s["p99_s"] >= s["p50_s"] > 0
    eng.close()
