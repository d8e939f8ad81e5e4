"""GPU parity: the CUDA path through the C ABI against the CPU restatement on
identical inputs.

Tolerance (FP64 path): 1e-12 relative per step in every conserved variable
(rel_err: pointwise relative error, components that pass through zero measured
against 1e-3 of their largest magnitude).  The new dt: 1e-12 relative.
"""
import ctypes

import numpy as np
import pytest

import mfgpu
from helpers import orszag_patch, periodic_fill, rel_err, to_device, to_host, valid_view

RTOL = 1e-12

pytestmark = pytest.mark.gpu


def _assert_argmin(oracle, p, U, lo, hi, cell, dt_min):
    """The reported cell attains the minimum dt (ties between cells whose dt
    agree to round-off may resolve either way)."""
    st, dtc, _ = oracle.compute_dt(p, U, lo, hi, list(cell), list(cell))
    assert st == 0
    assert dtc <= dt_min * (1.0 + RTOL), (cell, dtc, dt_min)


def _gpu_patch_step(ctx, U, lo, hi, vlo, vhi, dt, F=None, divB=None):
    t = to_device(U)
    tF = None
    if F is not None:
        tF = [(to_device(a), flo, fhi) for a, flo, fhi in F]
        Fspec = [(x.data_ptr(), flo, fhi) for x, flo, fhi in tF]
    tD = None
    if divB is not None:
        a, dlo, dhi = divB
        tD = to_device(a)
    st, ndt, cell = ctx.patch_update(t.data_ptr(), lo, hi, vlo, vhi, dt,
                                     F=Fspec if F is not None else None,
                                     divB=(tD.data_ptr(), divB[1], divB[2]) if divB is not None
                                     else None)
    out = to_host(t)
    Fo = [to_host(x) for x, _, _ in tF] if tF is not None else None
    Do = to_host(tD) if tD is not None else None
    return out, ndt, cell, Fo, Do


def _orszag_case(n, ta, prec=mfgpu.PREC_FP64, **kw):
    p = mfgpu.orszag_params(n, ta, prec)
    for k, v in kw.items():
        if k == "limiter":
            for q in range(8):
                p.limiter[q] = v
        else:
            setattr(p, k, v)
    return p


@pytest.mark.parametrize("ta", [mfgpu.TA_RK2, mfgpu.TA_FIRST_ORDER])
def test_orszag_single_patch_steps(gpulib, oracle, ta):
    n = 64
    p = _orszag_case(n, ta)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    st, dt0, _ = oracle.compute_dt(p, U, lo, hi, vlo, vhi)
    assert st == 0
    dt = 0.4 * dt0
    for step in range(4):
        Uo = U.copy()
        st, ndt_o, cell_o = oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt)
        assert st == 0
        Ug, ndt_g, cell_g, _, _ = _gpu_patch_step(ctx, U, lo, hi, vlo, vhi, dt)
        e = rel_err(valid_view(Ug, ng, 2), valid_view(Uo, ng, 2))
        assert np.all(e <= RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        _assert_argmin(oracle, p, Uo, lo, hi, cell_g, ndt_o)
        # next step from the oracle's state, ghosts refilled
        U = periodic_fill(Uo.copy(), ng, 2)
        dt = 0.4 * ndt_o
    ctx.close()


@pytest.mark.parametrize("lim", [lim for lim in mfgpu.LIMITERS if lim != mfgpu.LIM_MINMOD])
def test_limiters(gpulib, oracle, lim):
    n = 32
    p = _orszag_case(n, mfgpu.TA_RK2, limiter=lim)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    Uo = U.copy()
    assert oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt)[0] == 0
    Ug = _gpu_patch_step(ctx, U, lo, hi, vlo, vhi, dt)[0]
    e = rel_err(valid_view(Ug, ng, 2), valid_view(Uo, ng, 2))
    assert np.all(e <= RTOL), e


@pytest.mark.parametrize("flux,chk", [(3, 0), (2, 0), (4, 0), (11, 0), (13, 0), (1, 1)])
def test_solvers(gpulib, oracle, flux, chk):
    n = 32
    p = _orszag_case(n, mfgpu.TA_RK2, flux=flux, check_positivity=chk)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    Uo = U.copy()
    assert oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt)[0] == 0
    Ug = _gpu_patch_step(ctx, U, lo, hi, vlo, vhi, dt)[0]
    e = rel_err(valid_view(Ug, ng, 2), valid_view(Uo, ng, 2))
    assert np.all(e <= RTOL), e


def test_flux_and_divb_outputs(gpulib, oracle):
    n = 32
    p = _orszag_case(n, mfgpu.TA_RK2)
    ctx = mfgpu.Context(p)
    ng, nc = ctx.ng, ctx.nc
    U = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    F, Fg = [], []
    for d in range(2):
        fhi = list(vhi)
        fhi[d] += 1
        F.append((np.zeros(mfgpu.fab_shape(vlo, fhi, nc)), vlo, fhi))
        Fg.append((np.zeros(mfgpu.fab_shape(vlo, fhi, nc)), vlo, fhi))
    D = (np.zeros(mfgpu.fab_shape(vlo, vhi, 1)), vlo, vhi)
    Uo = U.copy()
    assert oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt, F=F, divB=D)[0] == 0
    Ug, _, _, Fo, Do = _gpu_patch_step(ctx, U, lo, hi, vlo, vhi, dt, F=Fg,
                                       divB=(np.zeros(mfgpu.fab_shape(vlo, vhi, 1)), vlo, vhi))
    for d in range(2):
        e = rel_err(Fo[d], F[d][0])
        assert np.all(e <= 1e-11), (d, e)
    scale = np.max(np.abs(D[0]))
    assert np.max(np.abs(Do - D[0])) <= 1e-11 * max(scale, 1e-300)


def _helio_single(n):
    p = mfgpu.helio_params(n)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ng, 3)
    U = mfgpu.init_host_fab(p, lo, hi, "helio")
    return p, ctx, U, lo, hi


def test_helio_single_patch_steps(gpulib, oracle):
    n = 24
    p, ctx, U, lo, hi = _helio_single(n)
    ng = ctx.ng
    vlo, vhi = [0, 0, 0], [n - 1] * 3
    dt0 = oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    ch = p.factor_ch * p.dx / dt0
    cp = np.sqrt(ch * p.dx / p.factor_cp)
    p.dedner_ch, p.dedner_cp = ch, cp
    ctx.set_dedner(ch, cp)
    dt = 0.4 * dt0
    for step in range(3):
        Uo = U.copy()
        st, ndt_o, cell_o = oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt)
        assert st == 0
        Ug, ndt_g, cell_g, _, _ = _gpu_patch_step(ctx, U, lo, hi, vlo, vhi, dt)
        e = rel_err(valid_view(Ug, ng, 3), valid_view(Uo, ng, 3))
        assert np.all(e <= RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        _assert_argmin(oracle, p, Uo, lo, hi, cell_g, ndt_o)
        U = Uo
        dt = 0.4 * ndt_o
    ctx.close()


def test_helio_level_vs_oracle(gpulib, oracle):
    n, patch = 32, 16
    p = mfgpu.helio_params(n)
    ctx = mfgpu.Context(p)
    ng, nc = ctx.ng, ctx.nc
    boxes = mfgpu.tile_boxes(n, patch, 3)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    arrays, fboxes = [], []
    for i, (blo, bhi) in enumerate(boxes):
        flo, fhi = lev.fab_box(i)
        a = mfgpu.init_host_fab(p, flo, fhi, "helio")
        lev.patch_view(flat, i)[:] = a
        arrays.append(a)
        fboxes.append((flo, fhi))
    lev.upload(flat.ctypes.data)
    dt0, _, _ = lev.compute_dt()
    odt = min(oracle.compute_dt(p, a, fb[0], fb[1], b[0], b[1])[1]
              for a, fb, b in zip(arrays, fboxes, boxes))
    assert abs(dt0 - odt) <= RTOL * odt
    ch = p.factor_ch * p.dx / dt0
    cp = float(np.sqrt(ch * p.dx / p.factor_cp))
    p.dedner_ch, p.dedner_cp = ch, cp
    ctx.set_dedner(ch, cp)
    dt = 0.4 * dt0
    for step in range(2):
        st, ndt_o, ip_o, cell_o = oracle.level_step(p, arrays, fboxes, boxes, dt)
        assert st == 0
        st, ndt_g, ip_g, cell_g = lev.step(dt)
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        for i in range(len(boxes)):
            g = valid_view(lev.patch_view(out, i), ng, 3)
            o = valid_view(arrays[i], ng, 3)
            e = rel_err(g, o)
            assert np.all(e <= RTOL), (step, i, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        _assert_argmin(oracle, p, arrays[ip_g], fboxes[ip_g][0], fboxes[ip_g][1], cell_g, ndt_o)
        # continue both from the oracle's state
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()


def test_orszag_level_equals_patch(gpulib, oracle):
    """Batched level (device exchange between the RK2 stages) gives the same
    numbers as the single-patch path (redundant stage-1 ghosts) and as the
    oracle."""
    n, patch = 64, 16
    p = mfgpu.orszag_params(n)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    boxes = mfgpu.tile_boxes(n, patch, 2)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, "orszag")
    lev.upload(flat.ctypes.data)
    dt = 0.4 * lev.compute_dt()[0]
    st, ndt, ip, cell = lev.step(dt)
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    # single patch covering the whole domain
    U = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    Ug, ndt1, cell1, _, _ = _gpu_patch_step(ctx, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
    whole = valid_view(Ug, ng, 2)
    for i, (blo, bhi) in enumerate(boxes):
        g = valid_view(lev.patch_view(out, i), ng, 2)
        ref = whole[:, :, blo[1]:bhi[1] + 1, blo[0]:bhi[0] + 1]
        assert np.array_equal(g, ref), i
    assert ndt == ndt1
    lev.close()
    ctx.close()


# MF_PREC_FP64_FAST rounds differently from the reference.  Where the Roe
# eigen-decomposition is near its triple point (fast ~ Alfven ~ slow speed),
# h = sqrt(szb^2 - 4 cc bb) turns a rounding-level difference of its argument
# into a sqrt(epsilon) ~ 1e-8 relative difference of the flux, so the fast path
# is held to 1e-7 per step (the parity path above is held to 1e-12).
FAST_RTOL = 1e-7


@pytest.mark.parametrize("case", ["orszag", "helio"])
def test_fast_fp64_per_step(gpulib, oracle, case):
    """MF_PREC_FP64_FAST (fused multiply-adds, reused reciprocals) stays within
    FAST_RTOL relative per step of the CPU restatement."""
    if case == "orszag":
        n, sd = 64, 2
        p = mfgpu.orszag_params(n, mfgpu.TA_RK2, mfgpu.PREC_FP64_FAST)
        ctx = mfgpu.Context(p)
        ng = ctx.ng
        U = orszag_patch(n, ng, p)
        lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
        vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    else:
        n, sd = 24, 3
        p = mfgpu.helio_params(n, precision=mfgpu.PREC_FP64_FAST)
        ctx = mfgpu.Context(p)
        ng = ctx.ng
        lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ng, 3)
        U = mfgpu.init_host_fab(p, lo, hi, "helio")
        vlo, vhi = [0, 0, 0], [n - 1] * 3
    dt0 = oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    if p.divb_cleaning == 5:
        ch = p.factor_ch * p.dx / dt0
        cp = float(np.sqrt(ch * p.dx / p.factor_cp))
        p.dedner_ch, p.dedner_cp = ch, cp
        ctx.set_dedner(ch, cp)
    dt = 0.4 * dt0
    for step in range(2):
        Uo = U.copy()
        st, ndt_o, _ = oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt)
        assert st == 0
        Ug, ndt_g, cell_g, _, _ = _gpu_patch_step(ctx, U, lo, hi, vlo, vhi, dt)
        e = rel_err(valid_view(Ug, ng, sd), valid_view(Uo, ng, sd))
        assert np.all(e <= FAST_RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= FAST_RTOL * ndt_o
        U = periodic_fill(Uo.copy(), ng, 2) if sd == 2 else Uo
        dt = 0.4 * ndt_o
    ctx.close()


def test_mixed_precision_error(gpulib, oracle):
    n = 64
    res = {}
    for prec in (mfgpu.PREC_FP64, mfgpu.PREC_MIXED):
        p = mfgpu.orszag_params(n, mfgpu.TA_RK2, prec)
        ctx = mfgpu.Context(p)
        ng = ctx.ng
        U = orszag_patch(n, ng, p)
        lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
        dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
        for _ in range(10):
            U, ndt, _, _, _ = _gpu_patch_step(ctx, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
            U = periodic_fill(U, ng, 2)
            dt = 0.4 * ndt
        res[prec] = valid_view(U, ng, 2)
        ctx.close()
    a, b = res[mfgpu.PREC_MIXED], res[mfgpu.PREC_FP64]
    l1 = np.sum(np.abs(a[0] - b[0])) / np.sum(np.abs(b[0]))
    assert l1 <= 1e-5, l1
    assert l1 > 0.0


def test_bad_arguments(gpulib):
    p = mfgpu.orszag_params(16)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U = orszag_patch(16, ng, p)
    t = to_device(U)
    lo, hi = mfgpu.grow([0, 0, 0], [15, 15, 0], ng, 2)
    # fab too small for the ghost width
    st, _, _ = ctx.patch_update(t.data_ptr(), [lo[0] + 1, lo[1], 0], hi, [0, 0, 0], [15, 15, 0],
                                1e-3, allow_error=True)
    assert st == mfgpu.MF_ERR_BAD_ARG
    st, _, _ = ctx.patch_update(t.data_ptr(), lo, hi, [0, 0, 0], [15, 15, 0], -1.0,
                                allow_error=True)
    assert st == mfgpu.MF_ERR_BAD_ARG
    q = mfgpu.helio_params(16)
    q.flux = 5  # VFRoe with GLM cleaning (main/MHDAM.cpp:1045)
    with pytest.raises(mfgpu.MfError) as ei:
        mfgpu.Context(q)
    assert ei.value.code == mfgpu.MF_ERR_UNSUPPORTED


def test_nonfinite_input_reported(gpulib):
    p = mfgpu.orszag_params(16)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U = orszag_patch(16, ng, p)
    U[4, 0, ng + 3, ng + 5] = np.nan
    t = to_device(U)
    lo, hi = mfgpu.grow([0, 0, 0], [15, 15, 0], ng, 2)
    st, _, _ = ctx.patch_update(t.data_ptr(), lo, hi, [0, 0, 0], [15, 15, 0], 1e-4,
                                allow_error=True)
    assert st == mfgpu.MF_ERR_NONFINITE
    # the context stays usable
    U = orszag_patch(16, ng, p)
    t = to_device(U)
    st, ndt, _ = ctx.patch_update(t.data_ptr(), lo, hi, [0, 0, 0], [15, 15, 0], 1e-4)
    assert st == 0 and ndt > 0


def _uniform_helio_patch(n, prec):
    """Single heliosphere patch holding the uniform inflow state (no inner
    sphere): away from the domain boundary (where the far-field ghosts hold
    the exact inflow primitives and the cells their round trip through the
    conserved form) every face flux difference is exactly zero, so one step
    changes the state there by the charge-exchange source alone."""
    p = mfgpu.helio_params(n, precision=prec)
    p.reinit_sphere = 0
    p.neutral_sun_bc = 0
    ctx = mfgpu.Context(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ctx.ng, 3)
    U = mfgpu.init_host_fab(p, lo, hi, "helio")
    return p, ctx, U, lo, hi


def test_mixed_charge_exchange_rates_are_fp64(gpulib):
    """MF_PREC_MIXED computes the charge-exchange rates in FP64: on a state
    whose fluxes cancel exactly, its step equals the fast FP64 path's
    bitwise.  MF_PREC_MIXED_CE32 (FP32 rates) differs at FP32 rounding of the
    source."""
    n, m = 24, 6  # interior: 6 cells from the domain boundary (two stages of stencils)
    out = {}
    for prec in (mfgpu.PREC_FP64_FAST, mfgpu.PREC_MIXED, mfgpu.PREC_MIXED_CE32):
        p, ctx, U, lo, hi = _uniform_helio_patch(n, prec)
        Ug = _gpu_patch_step(ctx, U, lo, hi, [0, 0, 0], [n - 1] * 3, 2e-3)[0]
        g = ctx.ng + m
        out[prec] = Ug[:, g:-g, g:-g, g:-g]
        src = np.max(np.abs(out[prec] - U[:, g:-g, g:-g, g:-g]))
        assert src > 1e-6, (prec, src)  # the source acts
        ctx.close()
    assert np.array_equal(out[mfgpu.PREC_MIXED], out[mfgpu.PREC_FP64_FAST])
    d = np.max(np.abs(out[mfgpu.PREC_MIXED_CE32] - out[mfgpu.PREC_FP64_FAST]))
    assert 0.0 < d <= 1e-6 * np.max(np.abs(out[mfgpu.PREC_FP64_FAST])), d


@pytest.mark.parametrize("prec", [mfgpu.PREC_MIXED, mfgpu.PREC_MIXED_CE32])
def test_mixed_modes_l1_vs_fp64(gpulib, prec):
    """Both mixed-precision forms against the FP64 GPU path on the 48^3
    heliosphere level (27 patches of 16^3, the inner sphere, GLM, charge
    exchange) after 20 steps with the same dt sequence: L1 relative error of
    rho, p, |B| and each neutral density <= 1e-5."""
    n, patch = 48, 16
    boxes = mfgpu.tile_boxes(n, patch, 3)
    levs = {}
    for pr in (mfgpu.PREC_FP64, prec):
        p = mfgpu.helio_params(n, precision=pr)
        ctx = mfgpu.Context(p)
        lev = mfgpu.Level(ctx, boxes)
        flat = np.zeros(lev.ndoubles)
        for i in range(len(boxes)):
            flo, fhi = lev.fab_box(i)
            lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, "helio")
        lev.upload(flat.ctypes.data)
        levs[pr] = (p, ctx, lev)
    p64, c64, l64 = levs[mfgpu.PREC_FP64]
    dt0 = l64.compute_dt()[0]
    dt = 0.4 * dt0
    nd = dt0
    for _ in range(20):
        ch = p64.factor_ch * p64.dx / nd
        cp = float(np.sqrt(ch * p64.dx / p64.factor_cp))
        for p, ctx, lev in levs.values():
            ctx.set_dedner(ch, cp)
        st, nd, _, _ = l64.step(dt)
        assert st == 0
        assert levs[prec][2].step(dt)[0] == 0
        dt = 0.4 * nd
    a = np.zeros(l64.ndoubles)
    b = np.zeros(l64.ndoubles)
    l64.download(a.ctypes.data)
    levs[prec][2].download(b.ctypes.data)
    ng = c64.ng
    num, den = {}, {}
    for i in range(len(boxes)):
        x = valid_view(l64.patch_view(a, i), ng, 3)
        y = valid_view(l64.patch_view(b, i), ng, 3)
        q = {"rho": (x[0], y[0]), "rho_n1": (x[9], y[9]), "rho_n2": (x[14], y[14]),
             "rho_n3": (x[19], y[19]),
             "absB": (np.sqrt((x[5:8] ** 2).sum(0)), np.sqrt((y[5:8] ** 2).sum(0)))}
        pr = []
        for z in (x, y):
            ke = 0.5 * (z[1] ** 2 + z[2] ** 2 + z[3] ** 2) / z[0]
            pr.append((2.0 / 3.0) * (z[4] - ke - (z[5:8] ** 2).sum(0) / (8 * np.pi)))
        q["p"] = tuple(pr)
        for k, (u, v) in q.items():
            num[k] = num.get(k, 0.0) + float(np.abs(v - u).sum())
            den[k] = den.get(k, 0.0) + float(np.abs(u).sum())
    l1 = {k: num[k] / den[k] for k in num}
    assert all(v <= 1e-5 for v in l1.values()), l1
    assert l1["rho"] > 0.0
    for p, ctx, lev in levs.values():
        lev.close()
        ctx.close()
