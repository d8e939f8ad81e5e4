"""mf_patch_update_noalloc: the patch update for callers that cannot allocate
device memory (processes whose device memory belongs to a pool allocator that
must not be bypassed, serving or real-time loops that forbid allocation after
start-up).  Its scratch lives in one static device array shared by all calls,
so the tests make two calls in a row and check each against the regular
mf_patch_update on the same input, within the parity tolerance of the GPU
tests: the updated state, the time step and its cell, and the flux and divB
outputs.  The file name sorts last so that a run stopping at the first failure
has already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import mfgpu
from helpers import orszag_patch, periodic_fill, rel_err, to_device, to_host, valid_view

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _call(fn, ctx, t, lo, hi, vlo, vhi, dt, F=None, divB=None):
    fab = mfgpu.MfFab(t.data_ptr(), mfgpu.make_box(lo, hi), ctx.nc)
    valid = mfgpu.make_box(vlo, vhi)
    ndt = ctypes.c_double()
    cell = mfgpu.c_int3()
    st = fn(ctx.h, ctypes.byref(fab), ctypes.byref(valid), dt,
            ctypes.byref(F) if F is not None else None,
            ctypes.byref(divB) if divB is not None else None, ctypes.byref(ndt), cell, None)
    return st, ndt.value, tuple(cell)


def _face_outputs(ctx, sd, vlo, vhi):
    """Device tensors and mf_fab descriptors of the flux outputs (faces of the
    valid box per direction) and of divB (the valid box)."""
    import torch
    fabs = (mfgpu.MfFab * 3)()
    ts = []
    for d in range(sd):
        hi = list(vhi)
        hi[d] += 1
        n = [hi[e] - vlo[e] + 1 for e in range(3)]
        t = torch.full((ctx.nc, n[2], n[1], n[0]), float("nan"), dtype=torch.float64,
                       device="cuda")
        ts.append(t)
        fabs[d] = mfgpu.MfFab(t.data_ptr(), mfgpu.make_box(vlo, hi), ctx.nc)
    n = [vhi[e] - vlo[e] + 1 for e in range(3)]
    tdb = torch.full((1, n[2], n[1], n[0]), float("nan"), dtype=torch.float64, device="cuda")
    dfab = mfgpu.MfFab(tdb.data_ptr(), mfgpu.make_box(vlo, vhi), 1)
    return fabs, ts, dfab, tdb


def _case(case):
    if case == "orszag":
        n, sd = 48, 2
        p = mfgpu.orszag_params(n)
        ctx = mfgpu.Context(p)
        U = orszag_patch(n, ctx.ng, p)
        lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ctx.ng, 2)
        vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
        dt = 2e-3
    else:
        n, sd = 16, 3
        p = mfgpu.helio_params(n, region_tracer=(case == "helio_tracer"))
        ctx = mfgpu.Context(p)
        lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ctx.ng, 3)
        U = mfgpu.init_host_fab(p, lo, hi, "helio")
        vlo, vhi = [0, 0, 0], [n - 1] * 3
        dt = 4e-3
    return p, ctx, U, lo, hi, vlo, vhi, sd, dt


@pytest.mark.parametrize("case", ["orszag", "helio", "helio_tracer"])
def test_noalloc_matches_patch_update(gpulib, case):
    p, ctx, U, lo, hi, vlo, vhi, sd, dt = _case(case)
    lib = ctx.lib
    ng = ctx.ng
    for call in range(2):
        ta = to_device(U)
        tb = to_device(U)
        sa, dta, ca = _call(lib.mf_patch_update, ctx, ta, lo, hi, vlo, vhi, dt)
        sb, dtb, cb = _call(lib.mf_patch_update_noalloc, ctx, tb, lo, hi, vlo, vhi, dt)
        assert sa == mfgpu.MF_OK and sb == mfgpu.MF_OK, (call, sa, sb)
        ua, ub = to_host(ta), to_host(tb)
        e = rel_err(valid_view(ub, ng, sd), valid_view(ua, ng, sd), nls=p.num_tracking_surfaces)
        assert np.all(e <= RTOL), (call, e)
        assert abs(dtb - dta) <= RTOL * dta, (call, dta, dtb)
        assert ca == cb, (call, ca, cb)
        U = periodic_fill(ua, ng, 2) if sd == 2 else ua
        dt = 0.4 * dta
    ctx.close()


def test_mixed_fp32_primitive_copy_matches_conversion(gpulib):
    """Mixed precision: mf_patch_update's FP32 flux kernels read the FP32
    copy of W that the primitive kernel writes; the no-allocation call has no
    room for that copy and converts W face by face.  Both roundings are
    round-to-nearest of the same FP64 values, so the states, the time step
    and its cell agree bitwise."""
    n = 16
    p = mfgpu.helio_params(n)
    p.precision = mfgpu.PREC_MIXED
    ctx = mfgpu.Context(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ctx.ng, 3)
    U = mfgpu.init_host_fab(p, lo, hi, "helio")
    vlo, vhi = [0, 0, 0], [n - 1] * 3
    ta, tb = to_device(U), to_device(U)
    sa, dta, ca = _call(ctx.lib.mf_patch_update, ctx, ta, lo, hi, vlo, vhi, 4e-3)
    sb, dtb, cb = _call(ctx.lib.mf_patch_update_noalloc, ctx, tb, lo, hi, vlo, vhi, 4e-3)
    assert sa == mfgpu.MF_OK and sb == mfgpu.MF_OK, (sa, sb)
    assert np.array_equal(to_host(ta), to_host(tb))
    assert dta == dtb and ca == cb, (dta, dtb, ca, cb)
    ctx.close()


def test_noalloc_rejects_patch_beyond_scratch(gpulib):
    n = 48
    p = mfgpu.helio_params(n)
    ctx = mfgpu.Context(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, ctx.ng, 3)
    U = mfgpu.init_host_fab(p, lo, hi, "helio")
    t = to_device(U)
    st, _, _ = _call(ctx.lib.mf_patch_update_noalloc, ctx, t, lo, hi, [0, 0, 0], [n - 1] * 3,
                     1e-3)
    assert st == mfgpu.MF_ERR_SCRATCH_LIMIT
    assert np.array_equal(to_host(t), U)
    ctx.close()


def test_noalloc_flux_and_divb_outputs(gpulib):
    """The flux output (the RK2 average of both stages' face fluxes, from the
    static array) and the divB output of two calls in a row equal those of
    mf_patch_update (Orszag-Tang with the 8-wave source, which fills divB)."""
    p, ctx, U, lo, hi, vlo, vhi, sd, dt = _case("orszag")
    lib = ctx.lib
    ng = ctx.ng
    for call in range(2):
        ta, tb = to_device(U), to_device(U)
        Fa, fa, Da, da = _face_outputs(ctx, sd, vlo, vhi)
        Fb, fb, Db, db = _face_outputs(ctx, sd, vlo, vhi)
        sa, dta, _ = _call(lib.mf_patch_update, ctx, ta, lo, hi, vlo, vhi, dt, Fa, Da)
        sb, dtb, _ = _call(lib.mf_patch_update_noalloc, ctx, tb, lo, hi, vlo, vhi, dt, Fb, Db)
        assert sa == mfgpu.MF_OK and sb == mfgpu.MF_OK, (call, sa, sb)
        for d in range(sd):
            x, y = to_host(fa[d]), to_host(fb[d])
            assert np.all(np.isfinite(x)) and np.all(np.isfinite(y)), (call, d)
            assert np.all(rel_err(y, x) <= RTOL), (call, d)
        x, y = to_host(da), to_host(db)
        assert np.all(np.isfinite(x))
        assert np.all(np.abs(y - x) <= RTOL * (np.max(np.abs(x)) + 1e-300)), call
        U = periodic_fill(to_host(ta), ng, 2)
        dt = 0.4 * dta
    ctx.close()


@pytest.mark.parametrize("what", ["hancock", "ct"])
def test_noalloc_unsupported_options(gpulib, what):
    """Hancock and constrained transport are refused before any device work."""
    n = 16
    p = mfgpu.orszag_params(n)
    if what == "hancock":
        p.time_approximation = mfgpu.TA_HANCOCK
    else:
        p.divb_cleaning = 1
        p.use_8wave = 0
    ctx = mfgpu.Context(p)
    U = orszag_patch(n, ctx.ng, p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ctx.ng, 2)
    t = to_device(U)
    st, _, _ = _call(ctx.lib.mf_patch_update_noalloc, ctx, t, lo, hi, [0, 0, 0], [n - 1, n - 1, 0],
                     1e-3)
    assert st == mfgpu.MF_ERR_UNSUPPORTED
    assert np.array_equal(to_host(t), U)
    ctx.close()


def test_noalloc_bad_arguments(gpulib):
    """Argument checks: a fab without the ghost layers, a valid box outside a
    non-periodic domain, a wrong flux box, a non-positive dt."""
    p, ctx, U, lo, hi, vlo, vhi, sd, dt = _case("helio")
    lib = ctx.lib
    t = to_device(U)
    f = lib.mf_patch_update_noalloc
    assert _call(f, ctx, t, lo, hi, [-1, 0, 0], vhi, dt)[0] == mfgpu.MF_ERR_BAD_ARG
    assert _call(f, ctx, t, lo, hi, vlo, [vhi[0] + 1] + vhi[1:], dt)[0] == mfgpu.MF_ERR_BAD_ARG
    assert _call(f, ctx, t, lo, hi, vlo, vhi, 0.0)[0] == mfgpu.MF_ERR_BAD_ARG
    assert _call(f, ctx, t, lo, hi, vlo, vhi, float("nan"))[0] == mfgpu.MF_ERR_BAD_ARG
    F, _, _, _ = _face_outputs(ctx, sd, vlo, [vhi[0] - 1] + vhi[1:])
    assert _call(f, ctx, t, lo, hi, vlo, vhi, dt, F)[0] == mfgpu.MF_ERR_BAD_ARG
    assert np.array_equal(to_host(t), U)
    ctx.close()
