"""mf_patch_update_noalloc: the patch update for callers that cannot allocate
device memory (code inside another framework's stream capture, processes whose
device memory belongs to a pool allocator, loops that forbid allocation after
start-up).  Its scratch lives in one static device array shared by all calls,
so the test makes two calls in a row and checks each against the regular
mf_patch_update on the same input, within the parity tolerance of the GPU
tests.  The file name sorts last so that a run stopping at the first failure
has already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import mfgpu
from helpers import orszag_patch, periodic_fill, rel_err, to_device, to_host, valid_view

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _call(fn, ctx, t, lo, hi, vlo, vhi, dt):
    fab = mfgpu.MfFab(t.data_ptr(), mfgpu.make_box(lo, hi), ctx.nc)
    valid = mfgpu.make_box(vlo, vhi)
    ndt = ctypes.c_double()
    cell = mfgpu.c_int3()
    st = fn(ctx.h, ctypes.byref(fab), ctypes.byref(valid), dt, None, None, ctypes.byref(ndt),
            cell, None)
    return st, ndt.value, tuple(cell)


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
