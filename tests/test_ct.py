"""Constrained transport (mf_params.divb_cleaning 1-3: the edge field of
Balsara-Spicer or, in 2D, Gardiner-Stone 1 / 2, srcIdeal/DivCleaningF.ChF:
75-854; recalculateB :4-72; per stage in EulerStep and the Hancock corrector,
src/PatchMHDAM.cpp:684-698, 1150-1160; the RK2 average of the edge field,
:1266-1275; the level's recalculation from UOld after the step,
srcIdeal/AMRLevelIdealMHD.cpp:1649-1688).

CPU: the oracle keeps the corner-centred divergence of the cell field (the
quantity this flux-CT form conserves) at round-off over several steps, for
every method and time scheme, where the unconstrained update lets it grow;
recalculating a stage's field from its own edge field and stage-start state
changes nothing; unsupported combinations are refused.  GPU: the CUDA path
against the oracle on identical inputs at the FP64 per-step tolerance
(single patch with the edge-field output, batched levels with the level
recalculation, the stand-alone recalculation bitwise), the fast and mixed
modes within theirs.
"""
import numpy as np
import pytest

import mfgpu
from mfgpu import amr
from helpers import orszag_patch, periodic_fill, rel_err, to_device, to_host, valid_view

RTOL = 1e-12
TAS = [mfgpu.TA_RK2, mfgpu.TA_HANCOCK, mfgpu.TA_FIRST_ORDER]


def _p2(n, ta, ct, prec=mfgpu.PREC_FP64, use8=0):
    p = mfgpu.orszag_params(n, ta, prec)
    p.divb_cleaning = ct
    p.use_8wave = use8
    return p


def _p3(n, ta, prec=mfgpu.PREC_FP64):
    p = amr.orszag3d_params(n, ta, prec)
    p.divb_cleaning = 1
    p.use_8wave = 0
    return p


def _patch3(p, n):
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ng, 3)
    U = np.ascontiguousarray(amr.orszag3d_state(p, lo, hi))
    return periodic_fill(U, ng, 3), lo, hi, ng


def _corner_div(U, dx, sd):
    """Divergence of the cell field at the cell corners: the mean over the
    2^(D-1) cell pairs across each direction of the differences, / dx."""
    if sd == 2:
        bx, by = U[5, 0], U[6, 0]
        dbx = (bx[1:, 1:] + bx[:-1, 1:] - bx[1:, :-1] - bx[:-1, :-1]) / (2 * dx)
        dby = (by[1:, 1:] + by[1:, :-1] - by[:-1, 1:] - by[:-1, :-1]) / (2 * dx)
        return dbx + dby
    out = 0.0
    for d, B in ((0, U[5]), (1, U[6]), (2, U[7])):
        ax = 2 - d                      # array axis of direction d (z, y, x order)
        hi = np.take(B, np.arange(1, B.shape[ax]), axis=ax)
        lo = np.take(B, np.arange(0, B.shape[ax] - 1), axis=ax)
        diff = hi - lo
        for a in range(3):
            if a != ax:
                diff = diff[tuple(slice(1, None) if b == a else slice(None) for b in range(3))] \
                    + diff[tuple(slice(None, -1) if b == a else slice(None) for b in range(3))]
        sl = tuple(slice(None) if b == ax else slice(None) for b in range(3))
        out = out + diff[sl] / (4 * dx)
    return out


def _edges(lo, hi, sd):
    from pyoracle import edge_boxes
    return [(np.zeros(mfgpu.fab_shape(a, b, 1)), a, b) for a, b in edge_boxes(lo, hi, sd)]


# ---------------------------------------------------------------------------
# CPU: the oracle
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("ta", TAS)
@pytest.mark.parametrize("ct", [0, 1, 2, 3])
def test_oracle_2d_keeps_corner_divergence(oracle, ta, ct):
    n = 32
    p = _p2(n, ta, ct)
    ng = mfgpu.num_ghost(p)
    U = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for _ in range(5):
        assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)[0] == 0
        U = periodic_fill(U, ng, 2)
    d = np.abs(_corner_div(U, p.dx, 2)[ng:-ng, ng:-ng]).max()
    scale = np.abs(U[5:7]).max() / p.dx
    if ct:
        assert d <= 1e-13 * scale, d / scale
    else:                               # without constrained transport it grows
        assert d > 1e-6 * scale


@pytest.mark.parametrize("ta", TAS)
def test_oracle_3d_bs_keeps_corner_divergence(oracle, ta):
    n = 12
    p = _p3(n, ta)
    U, lo, hi, ng = _patch3(p, n)
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1] * 3)[1]
    d0 = np.abs(_corner_div(U, p.dx, 3)[ng:-ng, ng:-ng, ng:-ng]).max()
    for _ in range(3):
        assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1] * 3, dt)[0] == 0
        U = periodic_fill(U, ng, 3)
    d = np.abs(_corner_div(U, p.dx, 3)[ng:-ng, ng:-ng, ng:-ng]).max()
    scale = np.abs(U[5:8]).max() / p.dx
    assert d <= d0 + 1e-13 * scale, (d0, d, scale)


@pytest.mark.parametrize("ct", [1, 2, 3])
def test_oracle_recalculation_of_a_stage_is_idempotent(oracle, ct):
    """First order: the step's field is Uold's minus the curl of the step's
    edge field, so recalculating it from Uold and that field again returns
    the same B (bitwise) and the same energy (to rounding)."""
    n = 24
    p = _p2(n, mfgpu.TA_FIRST_ORDER, ct)
    ng = mfgpu.num_ghost(p)
    U0 = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p, U0, lo, hi, vlo, vhi)[1]
    U = U0.copy()
    E = _edges(vlo, vhi, 2)
    assert oracle.patch_update(p, U, lo, hi, vlo, vhi, dt, E=E)[0] == 0
    assert np.abs(E[0][0]).max() > 0.0
    V = U.copy()
    assert oracle.recalculate_b(p, V, U0, lo, hi, E, dt, vlo, vhi) == 0
    assert np.array_equal(valid_view(V, ng, 2)[5:8], valid_view(U, ng, 2)[5:8])
    np.testing.assert_allclose(valid_view(V, ng, 2)[4], valid_view(U, ng, 2)[4], rtol=1e-15)


def test_oracle_refusals(oracle):
    n = 8
    p = _p3(n, mfgpu.TA_RK2)
    p.divb_cleaning = 2                 # Gardiner-Stone in 3D: undefined in the reference
    U, lo, hi, ng = _patch3(p, n)
    assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1] * 3, 1e-3)[0] == \
        mfgpu.MF_ERR_UNSUPPORTED
    p.divb_cleaning = 4                 # projection: needs an elliptic solver
    assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1] * 3, 1e-3)[0] == \
        mfgpu.MF_ERR_UNSUPPORTED


def test_device_refusals(gpulib):
    p = _p3(8, mfgpu.TA_RK2)
    p.divb_cleaning = 3
    with pytest.raises(mfgpu.MfError):
        mfgpu.Context(p)
    p.divb_cleaning = 4
    with pytest.raises(mfgpu.MfError):
        mfgpu.Context(p)


# ---------------------------------------------------------------------------
# GPU: the CUDA path against the oracle
# ---------------------------------------------------------------------------
def _gpu_patch(ctx, U, lo, hi, vlo, vhi, dt, sd):
    t = to_device(U)
    E = _edges(vlo, vhi, sd)
    tE = [(to_device(a), elo, ehi) for a, elo, ehi in E]
    st, ndt, _ = ctx.patch_update(t.data_ptr(), lo, hi, vlo, vhi, dt,
                                  E=[(x.data_ptr(), elo, ehi) for x, elo, ehi in tE])
    assert st == 0
    return to_host(t), ndt, [to_host(x) for x, _, _ in tE]


@pytest.mark.gpu
@pytest.mark.parametrize("ta", TAS)
@pytest.mark.parametrize("ct", [1, 2, 3])
def test_gpu_2d_patch_vs_oracle(gpulib, oracle, ta, ct):
    n = 48
    p = _p2(n, ta, ct)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U = orszag_patch(n, ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    for step in range(3):
        Uo = U.copy()
        Eo = _edges(vlo, vhi, 2)
        st, ndt_o, _ = oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt, E=Eo)
        assert st == 0
        Ug, ndt_g, Eg = _gpu_patch(ctx, U, lo, hi, vlo, vhi, dt, 2)
        e = rel_err(valid_view(Ug, ng, 2), valid_view(Uo, ng, 2))
        assert np.all(e <= RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        sc = np.abs(Eo[0][0]).max()
        assert np.abs(Eg[0] - Eo[0][0]).max() <= RTOL * sc, step
        U = periodic_fill(Uo.copy(), ng, 2)
        dt = 0.4 * ndt_o
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ta", TAS)
def test_gpu_3d_bs_patch_vs_oracle(gpulib, oracle, ta):
    n = 16
    p = _p3(n, ta)
    ctx = mfgpu.Context(p)
    U, lo, hi, ng = _patch3(p, n)
    vlo, vhi = [0, 0, 0], [n - 1] * 3
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    for step in range(2):
        Uo = U.copy()
        Eo = _edges(vlo, vhi, 3)
        assert oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt, E=Eo)[0] == 0
        Ug, _, Eg = _gpu_patch(ctx, U, lo, hi, vlo, vhi, dt, 3)
        e = rel_err(valid_view(Ug, ng, 3), valid_view(Uo, ng, 3))
        assert np.all(e <= RTOL), (step, e)
        for d in range(3):
            sc = np.abs(Eo[d][0]).max()
            assert np.abs(Eg[d] - Eo[d][0]).max() <= RTOL * sc, (step, d)
        U = periodic_fill(Uo.copy(), ng, 3)
    ctx.close()


@pytest.mark.gpu
def test_gpu_recalculate_magnetic_field_bitwise(gpulib, oracle):
    """mf_recalculate_magnetic_field on caller fabs (the level's UOld and a
    patch's edge field) against the oracle's recalculateB: bitwise."""
    n = 16
    p = _p3(n, mfgpu.TA_RK2)
    ctx = mfgpu.Context(p)
    U0, lo, hi, ng = _patch3(p, n)
    vlo, vhi = [0, 0, 0], [n - 1] * 3
    dt = 0.4 * oracle.compute_dt(p, U0, lo, hi, vlo, vhi)[1]
    U = U0.copy()
    E = _edges(vlo, vhi, 3)
    assert oracle.patch_update(p, U, lo, hi, vlo, vhi, dt, E=E)[0] == 0
    V = U.copy()
    assert oracle.recalculate_b(p, V, U0, lo, hi, E, dt, vlo, vhi) == 0
    tU, tU0 = to_device(U), to_device(U0)
    tE = [(to_device(a), elo, ehi) for a, elo, ehi in E]
    ctx.recalculate_magnetic_field(tU.data_ptr(), tU0.data_ptr(), lo, hi,
                                   [(x.data_ptr(), elo, ehi) for x, elo, ehi in tE], dt, vlo, vhi)
    assert np.array_equal(to_host(tU), V)
    ctx.close()


def _level_case(p, n, sd, patch):
    boxes = mfgpu.tile_boxes(n, patch, sd)
    ng = mfgpu.num_ghost(p)
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = mfgpu.grow(lo, hi, ng, sd)
        if sd == 2:
            a = mfgpu.init_host_fab(p, flo, fhi, "orszag")
        else:
            a = amr.orszag3d_state(p, flo, fhi)
        arrays.append(np.ascontiguousarray(a))
        fboxes.append((flo, fhi))
    return boxes, arrays, fboxes, ng


@pytest.mark.gpu
@pytest.mark.parametrize("sd,ct,ta", [(2, 1, mfgpu.TA_RK2), (2, 2, mfgpu.TA_FIRST_ORDER),
                                      (2, 3, mfgpu.TA_HANCOCK), (3, 1, mfgpu.TA_RK2),
                                      (3, 1, mfgpu.TA_HANCOCK)])
def test_gpu_level_vs_oracle(gpulib, oracle, sd, ct, ta):
    """Batched level steps (several patches, the exchange, each patch's edge
    field at its own boundary, then the level's recalculation of B from
    UOld and the step's edge field) against the oracle's level step."""
    n, patch = (48, 16) if sd == 2 else (16, 8)
    p = _p2(n, ta, ct) if sd == 2 else _p3(n, ta)
    boxes, arrays, fboxes, ng = _level_case(p, n, sd, patch)
    ctx = mfgpu.Context(p)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i, a in enumerate(arrays):
        lev.patch_view(flat, i)[:] = a
    lev.upload(flat.ctypes.data)
    dt = 0.4 * lev.compute_dt()[0]
    for step in range(2):
        st, ndt_o, _, _ = oracle.level_step(p, arrays, fboxes, boxes, dt)
        assert st == 0
        st, ndt_g, _, _ = lev.step(dt)
        assert st == 0
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(out, i), ng, sd), valid_view(arrays[i], ng, sd))
            assert np.all(e <= RTOL), (step, i, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(mfgpu.PREC_FP64_FAST, 1e-7), (mfgpu.PREC_MIXED, 1e-4)])
def test_gpu_fast_and_mixed(gpulib, oracle, prec, tol):
    """64^2, 3 RK2 steps with the Balsara-Spicer field: fast FP64 pointwise
    within tol of the oracle, mixed within tol in the L1 norm of B."""
    n = 64
    p = _p2(n, mfgpu.TA_RK2, 1, prec)
    p64 = _p2(n, mfgpu.TA_RK2, 1)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U = orszag_patch(n, ng, p64)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p64, U, lo, hi, vlo, vhi)[1]
    Ug, Uo = U.copy(), U.copy()
    for _ in range(3):
        assert oracle.patch_update(p64, Uo, lo, hi, vlo, vhi, dt)[0] == 0
        Uo = periodic_fill(Uo, ng, 2)
        Ug = periodic_fill(_gpu_patch(ctx, Ug, lo, hi, vlo, vhi, dt, 2)[0], ng, 2)
    g, o = valid_view(Ug, ng, 2), valid_view(Uo, ng, 2)
    if prec == mfgpu.PREC_FP64_FAST:
        assert np.all(rel_err(g, o) <= tol)
    else:
        l1 = np.abs(g[5:7] - o[5:7]).sum() / np.abs(o[5:7]).sum()
        assert l1 <= tol, l1
        # the mixed path keeps the corner divergence at rounding too (FP32 fluxes)
        d = np.abs(_corner_div(Ug, p.dx, 2)[ng:-ng, ng:-ng]).max()
        assert d <= 1e-10 * np.abs(g[5:7]).max() / p.dx
    ctx.close()


def test_ct_refused_where_not_built(gpulib):
    """The serving engine, the allocation-free call and coupled hierarchies
    do not take constrained transport (no GPU work: the checks come first)."""
    import ctypes
    p = _p2(16, mfgpu.TA_RK2, 1)
    ctx = mfgpu.Context(p)
    srv = ctypes.c_void_p()
    assert ctx.lib.mf_server_create(ctx.h, 1e9, 4, ctypes.byref(srv)) == mfgpu.MF_ERR_UNSUPPORTED
    ng = ctx.ng
    lo, hi = mfgpu.grow([0, 0, 0], [15, 15, 0], ng, 2)
    fab = mfgpu.MfFab(1024, mfgpu.make_box(lo, hi), ctx.nc)       # never dereferenced
    valid = mfgpu.make_box([0, 0, 0], [15, 15, 0])
    ndt = ctypes.c_double()
    cell = mfgpu.c_int3()
    assert ctx.lib.mf_patch_update_noalloc(ctx.h, ctypes.byref(fab), ctypes.byref(valid), 1e-3,
                                           None, None, ctypes.byref(ndt), cell, None) == \
        mfgpu.MF_ERR_UNSUPPORTED
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ta,hbc,use8", [(mfgpu.TA_RK2, 0, 0), (mfgpu.TA_HANCOCK, 0, 0),
                                         (mfgpu.TA_RK2, 1, 0), (mfgpu.TA_FIRST_ORDER, 0, 1)])
def test_gpu_helio_ct_with_region_tracer_vs_oracle(gpulib, oracle, ta, hbc, use8):
    """Constrained transport in the full heliosphere problem: far-field ghosts,
    three neutral fluids with charge exchange, the inner-sphere reset, the
    neutral pass-through at the sun and the region tracer, with the
    heliosphere boundary fluxes (HELIOBC, whose B fluxes enter the boundary
    edges) or the 8-wave source; level steps of 32^3 in 8 patches against the
    oracle (each step from the oracle's state)."""
    n = 32
    p = mfgpu.helio_params(n, time_approximation=ta, region_tracer=True)
    p.divb_cleaning = 1
    p.use_8wave = use8
    p.helio_bc = hbc
    boxes = mfgpu.tile_boxes(n, 16, 3)
    ng = mfgpu.num_ghost(p)
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = mfgpu.grow(lo, hi, ng, 3)
        arrays.append(np.ascontiguousarray(mfgpu.init_host_fab(p, flo, fhi, "helio")))
        fboxes.append((flo, fhi))
    ctx = mfgpu.Context(p)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i, a in enumerate(arrays):
        lev.patch_view(flat, i)[:] = a
    lev.upload(flat.ctypes.data)
    dt = 0.4 * lev.compute_dt()[0]
    for step in range(2):
        st, ndt_o, _, _ = oracle.level_step(p, arrays, fboxes, boxes, dt)
        assert st == 0
        st, ndt_g, _, _ = lev.step(dt)
        assert st == 0
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(out, i), ng, 3), valid_view(arrays[i], ng, 3),
                        nls=1)
            assert np.all(e <= RTOL), (step, i, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()


def test_ct_entry_points_reject_bad_arguments(gpulib):
    """Argument checks of mf_patch_update_e and mf_recalculate_magnetic_field
    (they come before any device work: the pointers are never dereferenced)."""
    import ctypes
    n = 16
    p = _p2(n, mfgpu.TA_RK2, 1)
    ctx = mfgpu.Context(p)
    lib, ng, nc = ctx.lib, ctx.ng, ctx.nc
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    fab = mfgpu.MfFab(4096, mfgpu.make_box(lo, hi), nc)
    valid = mfgpu.make_box([0, 0, 0], [n - 1, n - 1, 0])
    ndt = ctypes.c_double()
    cell = mfgpu.c_int3()
    small = (mfgpu.MfFab * 3)()
    small[0] = mfgpu.MfFab(8192, mfgpu.make_box([0, 0, 0], [n - 1, n - 1, 0]), 1)  # not nodal
    assert lib.mf_patch_update_e(ctx.h, ctypes.byref(fab), ctypes.byref(valid), 1e-3, None, None,
                                 ctypes.cast(small, ctypes.c_void_p), ctypes.byref(ndt), cell,
                                 None) == mfgpu.MF_ERR_BAD_ARG
    uold = mfgpu.MfFab(4096, mfgpu.make_box(lo, hi), nc)
    assert lib.mf_recalculate_magnetic_field(ctx.h, ctypes.byref(fab), ctypes.byref(uold),
                                             ctypes.cast(small, ctypes.c_void_p), 1e-3,
                                             ctypes.byref(valid), None) == mfgpu.MF_ERR_BAD_ARG
    ctx.close()
    q = _p2(n, mfgpu.TA_RK2, 0)         # no constrained transport: nothing to recalculate
    ctx = mfgpu.Context(q)
    good = (mfgpu.MfFab * 3)()
    good[0] = mfgpu.MfFab(8192, mfgpu.make_box([0, 0, 0], [n, n, 0]), 1)
    assert ctx.lib.mf_recalculate_magnetic_field(ctx.h, ctypes.byref(fab), ctypes.byref(uold),
                                                 ctypes.cast(good, ctypes.c_void_p), 1e-3,
                                                 ctypes.byref(valid), None) == \
        mfgpu.MF_ERR_BAD_ARG
    ctx.close()
