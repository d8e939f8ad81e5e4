"""The inner-sphere reset with the reference's default bipolar field, the level
time it depends on, and the growth cap of chained time steps.

* HELIOREINIT_DEFAULT (swlism/HeliosphericPlasmaBCF.ChF:1435-1566) with
  sunBmonopolar != 1 (the reference default, swlism/HeliosphericProblem.cpp:
  106,156): B keeps its sign where the colatitude theta is below the current
  sheet's thetaS(r, phi, t) and flips elsewhere; the current-sheet surface
  iHCS (the first tracking surface) takes +1 / -1.
* AMR_MHDAM::assignDt (srcIdeal/AMR_MHDAM.cpp:1570-1706): the next dt is
  cfl * dt_min, at most max_dt_growth times the current dt.

CPU: the oracle's bipolar reset against the monopolar one (flat sheet: the
southern field flips) and against a numpy restatement of thetaS (tilted sheet
at a later time).  GPU: patch and level steps with the bipolar field, a tilted
sheet and a non-zero time against the oracle at the per-step tolerance; the
device time of async level steps and the capped dt chain (bitwise against
synchronous steps with the capped dt sequence); mf_hier_assign_dt.
"""
import numpy as np
import pytest

import mfgpu
from helpers import rel_err, valid_view

RTOL = 1e-12


def _helio(n, monopolar=0, tilt=0.0, surfaces=0, ta=mfgpu.TA_RK2):
    p = mfgpu.helio_params(n, time_approximation=ta)
    p.sun_b_monopolar = monopolar
    p.sun_tilt = tilt
    if surfaces:
        p.num_tracking_surfaces = surfaces
        p.limiter_ls = mfgpu.LIM_MINMOD
    return p


def _centres(p, lo, hi):
    """Cell-centre coordinates relative to the sun on the fab [lo, hi]
    (arrays shaped like one component of the fab)."""
    k, j, i = np.meshgrid(*[np.arange(lo[d], hi[d] + 1) for d in (2, 1, 0)], indexing="ij")
    return ((i + 0.5) * p.dx - p.sun_center[0], (j + 0.5) * p.dx - p.sun_center[1],
            (k + 0.5) * p.dx - p.sun_center[2])


def _thetas(p, x, y, z, t):
    """Colatitude and current-sheet colatitude of HELIOREINIT_DEFAULT."""
    r = np.sqrt(x * x + y * y + z * z)
    xy = np.sqrt(x * x + y * y)
    cosT = z / r
    cosF, sinF = x / xy, y / xy
    ph = p.sun_beta * (r - p.sun_v * t)
    sinB = sinF * np.cos(ph) + cosF * np.sin(ph)
    cosB = cosF * np.cos(ph) - sinF * np.sin(ph)
    tl = np.deg2rad(p.sun_tilt)
    thS = np.arcsin(np.sin(tl) * sinB / np.sqrt((np.cos(tl) * cosB) ** 2 + sinB ** 2)) + np.pi / 2
    return np.arccos(cosT), thS


def test_oracle_flat_sheet_flips_the_southern_field(oracle):
    n = 48
    res = {}
    for mono in (1, 0):
        p = _helio(n, monopolar=mono, surfaces=1)
        ng = mfgpu.num_ghost(p)
        lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ng, 3)
        U = mfgpu.init_host_fab(p, lo, hi, "helio")
        dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1] * 3)[1]
        assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1] * 3, dt)[0] == 0
        res[mono] = U
    p = _helio(n)
    x, y, z = _centres(p, lo, hi)
    sphere = (x * x + y * y + z * z <= p.reinit_r0 ** 2)
    assert sphere.sum() >= 50
    south = sphere & (z < 0)
    m, b = res[1], res[0]
    for q in (5, 6, 7):
        assert np.array_equal(b[q][south], -m[q][south])
        assert np.array_equal(b[q][sphere & (z > 0)], m[q][sphere & (z > 0)])
    for q in (0, 1, 2, 3, 4):
        assert np.array_equal(b[q][sphere], m[q][sphere])
    ils = mfgpu.num_fluid_cons(p)
    assert np.array_equal(b[ils][sphere], np.where(z[sphere] > 0, 1.0, -1.0))


def test_oracle_tilted_sheet_at_a_later_time(oracle):
    """First-order step (one stage: the reset at time t + dt) with a sheet
    tilted by 30 degrees: the sign of B and the current-sheet surface follow
    theta < thetaS(r, phi, t + dt) cell by cell."""
    n = 48
    p = _helio(n, tilt=30.0, surfaces=1, ta=mfgpu.TA_FIRST_ORDER)
    pm = _helio(n, monopolar=1, tilt=30.0, surfaces=1, ta=mfgpu.TA_FIRST_ORDER)
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ng, 3)
    U0 = mfgpu.init_host_fab(p, lo, hi, "helio")
    t, dt = 0.37, 2e-4
    Ub, Um = U0.copy(), U0.copy()
    assert oracle.patch_update(p, Ub, lo, hi, [0, 0, 0], [n - 1] * 3, dt, time=t)[0] == 0
    assert oracle.patch_update(pm, Um, lo, hi, [0, 0, 0], [n - 1] * 3, dt, time=t)[0] == 0
    x, y, z = _centres(p, lo, hi)
    sphere = (x * x + y * y + z * z <= p.reinit_r0 ** 2)
    th, ths = _thetas(p, x[sphere], y[sphere], z[sphere], t + dt)
    assert np.min(np.abs(th - ths)) > 1e-9  # no cell on the sheet itself
    keep = th < ths
    assert 0 < keep.sum() < keep.size
    sign = np.where(keep, 1.0, -1.0)
    for q in (5, 6, 7):
        assert np.array_equal(Ub[q][sphere], sign * Um[q][sphere])
    ils = mfgpu.num_fluid_cons(p)
    assert np.array_equal(Ub[ils][sphere], sign)


def test_params_default_is_bipolar_with_growth_cap():
    p = mfgpu._base_params(3, 4)
    assert p.sun_b_monopolar == 0 and p.max_dt_growth == 1.1 and p.sun_tilt == 0.0


@pytest.mark.gpu
def test_library_default_is_bipolar_with_growth_cap(gpulib):
    p = mfgpu.default_params(3, 4)
    assert p.sun_b_monopolar == 0 and p.max_dt_growth == 1.1 and p.sun_tilt == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("tilt,surfaces,tracer", [(0.0, 0, False), (30.0, 1, False),
                                                  (30.0, 2, True)])
def test_gpu_bipolar_patch_vs_oracle(gpulib, oracle, tilt, surfaces, tracer):
    n = 32
    p = mfgpu.helio_params(n, region_tracer=tracer)
    p.sun_tilt = tilt
    if surfaces:
        p.num_tracking_surfaces = surfaces
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ng, 3)
    U = mfgpu.init_host_fab(p, lo, hi, "helio")
    vlo, vhi = [0, 0, 0], [n - 1] * 3
    t = 0.21
    ctx.set_current_time(t)
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    for step in range(2):
        Uo = U.copy()
        st, ndt_o, _ = oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt, time=t)
        assert st == 0
        import torch
        tg = torch.from_numpy(U.copy()).cuda()
        _, ndt_g, _ = ctx.patch_update(tg.data_ptr(), lo, hi, vlo, vhi, dt)
        Ug = tg.cpu().numpy()
        e = rel_err(valid_view(Ug, ng, 3), valid_view(Uo, ng, 3), nls=p.num_tracking_surfaces)
        assert np.all(e <= RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        U = Uo
        t += dt
        ctx.set_current_time(t)
        dt = 0.4 * ndt_o
    ctx.close()


def _level(p, n, patch):
    ctx = mfgpu.Context(p)
    boxes = mfgpu.tile_boxes(n, patch, 3)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    arrays, fboxes = [], []
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        a = mfgpu.init_host_fab(p, flo, fhi, "helio")
        lev.patch_view(flat, i)[:] = a
        arrays.append(a)
        fboxes.append((flo, fhi))
    lev.upload(flat.ctypes.data)
    return ctx, lev, boxes, arrays, fboxes, flat


@pytest.mark.gpu
def test_gpu_bipolar_level_time_vs_oracle(gpulib, oracle):
    """Level steps of a tilted sheet from a non-zero level time: the level
    passes its time to the reset and advances it by each step's dt."""
    n, patch = 32, 16
    p = mfgpu.helio_params(n)
    p.sun_tilt = 25.0
    ctx, lev, boxes, arrays, fboxes, flat = _level(p, n, patch)
    ng = ctx.ng
    t = 0.13
    lev.set_time(t)
    dt = 0.4 * lev.compute_dt()[0]
    for step in range(2):
        st, ndt_o, _, _ = oracle.level_step(p, arrays, fboxes, boxes, dt, time=t)
        assert st == 0
        st, ndt_g, _, _ = lev.step(dt)
        assert lev.time() == t + dt
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(out, i), ng, 3), valid_view(arrays[i], ng, 3))
            assert np.all(e <= RTOL), (step, i, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        t = t + dt
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()


@pytest.mark.gpu
def test_gpu_async_growth_cap_and_time(gpulib):
    """Seeded with a dt far below the CFL limit, async steps grow it by
    max_dt_growth per step (1.1 by default); the device time is the sum of
    the steps' dts, and the state equals that of synchronous steps with the
    same capped dt sequence bitwise."""
    n, patch = 32, 16
    p = mfgpu.helio_params(n)
    ctx, lev, boxes, arrays, fboxes, flat = _level(p, n, patch)
    dt0 = 0.01 * 0.4 * lev.compute_dt()[0]
    t0 = 0.5
    lev.set_time(t0)
    lev.seed_dt(dt0, 0.4)
    for _ in range(3):
        lev.step_async()
    assert lev.result()[0] == 0
    a = np.zeros(lev.ndoubles)
    lev.download(a.ctypes.data)
    dts = [dt0, dt0 * 1.1, dt0 * 1.1 * 1.1]
    assert lev.time() == pytest.approx(t0 + sum(dts), rel=1e-15)
    lev.upload(flat.ctypes.data)
    lev.set_time(t0)
    # the async steps take the GLM speeds of the previous step's dt_min
    # (AMRLevelIdealMHD.cpp:1531-1548); the synchronous ones get them set
    for d in dts:
        st, nd, _, _ = lev.step(d)
        assert st == 0
        ch = p.factor_ch * p.dx / nd
        ctx.set_dedner(ch, float(np.sqrt(ch * p.dx / p.factor_cp)))
    b = np.zeros(lev.ndoubles)
    lev.download(b.ctypes.data)
    assert np.array_equal(a, b)
    lev.close()
    ctx.close()


@pytest.mark.gpu
def test_gpu_no_growth_cap(gpulib):
    """max_dt_growth <= 0 disables the cap: the seeded dt is replaced by
    cfl * dt_min after the first step."""
    n, patch = 32, 16
    p = mfgpu.helio_params(n)
    p.max_dt_growth = 0.0
    ctx, lev, boxes, arrays, fboxes, flat = _level(p, n, patch)
    dt0 = 0.01 * 0.4 * lev.compute_dt()[0]
    lev.seed_dt(dt0, 0.4)
    lev.step_async()
    lev.step_async()
    st, ndt1, _, _ = lev.result()
    assert st == 0
    # the second step ran with 0.4 * dt_min of the first: far above 1.1 dt0
    assert lev.time() > 0.0 + dt0 + 10 * 1.1 * dt0
    lev.close()
    ctx.close()


@pytest.mark.gpu
def test_gpu_hier_assign_dt(gpulib):
    from mfgpu import amr
    p0 = amr.orszag3d_params(16)
    params = [p0, amr.level_params(p0, 2)]
    boxes = [mfgpu.tile_boxes(16, 8, 3), [((8, 8, 8), (23, 23, 23))]]

    def init(p, lo, hi):
        return amr.orszag3d_state(p, lo, hi)

    dh = amr.DeviceHierarchy(mfgpu, params, boxes, [2], init)
    with pytest.raises(mfgpu.MfError):
        dh.hier.assign_dt(0.4)
    dt = 0.4 * dh.compute_dt()
    small = 0.01 * dt
    nd = dh.step(small)
    assert dh.hier.assign_dt(0.4) == min(0.4 * nd, small * 1.1)
    nd = dh.step(dt)
    assert dh.hier.assign_dt(0.4) == min(0.4 * nd, dt * 1.1)
    dh.close()
