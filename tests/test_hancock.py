"""Hancock time integration (predictorHancock + correctorHancock,
src/PatchMHDAM.cpp:836-1189, 1287-1301).

CPU: properties of the oracle's restatement (mass conservation on a periodic
box, a uniform state stays uniform).  GPU: the CUDA path against the oracle at
the per-step tolerance (single patch and level, FP64), the level against
per-patch calls (bitwise), the fast and mixed modes within their tolerances.
"""
import numpy as np
import pytest

import mfgpu
from helpers import orszag_patch, periodic_fill, rel_err, to_device, to_host, valid_view

RTOL = 1e-12
TA = mfgpu.TA_HANCOCK


def _orszag(n, prec=mfgpu.PREC_FP64):
    p = mfgpu.orszag_params(n, TA, prec)
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    return p, ng, lo, hi, orszag_patch(n, ng, p)


def test_hancock_conserves_mass_on_periodic_box(oracle):
    n = 32
    p, ng, lo, hi, U = _orszag(n)
    m0 = U[0, :, ng:-ng, ng:-ng].sum()
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for _ in range(10):
        st, ndt, _ = oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        assert st == 0
        periodic_fill(U, ng, 2)
        dt = 0.4 * ndt
    assert abs(U[0, :, ng:-ng, ng:-ng].sum() - m0) <= 1e-13 * m0
    assert np.all(np.isfinite(U))


def test_hancock_keeps_uniform_state(oracle):
    n = 16
    p, ng, lo, hi, U = _orszag(n)
    U[:] = U[:, :, ng:ng + 1, ng:ng + 1]  # the state of one cell everywhere
    U0 = U.copy()
    st, ndt, _ = oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], 1e-3)
    assert st == 0
    np.testing.assert_allclose(valid_view(U, ng, 2), valid_view(U0, ng, 2), rtol=1e-14, atol=1e-15)


def _gpu_step(ctx, U, lo, hi, vlo, vhi, dt):
    t = to_device(U)
    st, ndt, cell = ctx.patch_update(t.data_ptr(), lo, hi, vlo, vhi, dt)
    return to_host(t), ndt


@pytest.mark.gpu
@pytest.mark.parametrize("lim", [mfgpu.LIM_MINMOD, mfgpu.LIM_VANLEER, mfgpu.LIM_KOREN,
                                 mfgpu.LIM_WENO3YC])
def test_gpu_hancock_orszag_vs_oracle(gpulib, oracle, lim):
    n = 64
    p, ng, lo, hi, U = _orszag(n)
    for q in range(8):
        p.limiter[q] = lim
    ctx = mfgpu.Context(p)
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for step in range(3):
        Ug, ndt_g = _gpu_step(ctx, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        st, ndt_o, _ = oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        assert st == 0
        e = rel_err(valid_view(Ug, ng, 2), valid_view(U, ng, 2))
        assert np.all(e <= RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        periodic_fill(U, ng, 2)
        dt = 0.4 * ndt_o
    ctx.close()


@pytest.mark.gpu
def test_gpu_hancock_helio_level_vs_oracle(gpulib, oracle):
    n, patch = 32, 16
    p = mfgpu.helio_params(n, time_approximation=TA)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
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
    dt0 = lev.compute_dt()[0]
    ch = p.factor_ch * p.dx / dt0
    p.dedner_ch, p.dedner_cp = ch, float(np.sqrt(ch * p.dx / p.factor_cp))
    ctx.set_dedner(p.dedner_ch, p.dedner_cp)
    dt = 0.4 * dt0
    for step in range(2):
        st, ndt_o, _, _ = oracle.level_step(p, arrays, fboxes, boxes, dt)
        assert st == 0
        st, ndt_g, _, _ = lev.step(dt)
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(out, i), ng, 3), valid_view(arrays[i], ng, 3))
            assert np.all(e <= RTOL), (step, i, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [mfgpu.PREC_FP64, mfgpu.PREC_MIXED])
def test_gpu_hancock_level_equals_patches(gpulib, prec):
    n, patch = 64, 16
    p, ng, lo, hi, U = _orszag(n, prec)
    ctx = mfgpu.Context(p)
    boxes = mfgpu.tile_boxes(n, patch, 2)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, "orszag")
    lev.upload(flat.ctypes.data)
    dt = 0.4 * lev.compute_dt()[0]
    st, ndt, _, _ = lev.step(dt)
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    Ug, ndt1 = _gpu_step(ctx, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
    whole = valid_view(Ug, ng, 2)
    for i, (blo, bhi) in enumerate(boxes):
        g = valid_view(lev.patch_view(out, i), ng, 2)
        assert np.array_equal(g, whole[:, :, blo[1]:bhi[1] + 1, blo[0]:bhi[0] + 1]), i
    assert ndt == ndt1
    lev.close()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(mfgpu.PREC_FP64_FAST, 1e-9), (mfgpu.PREC_MIXED, 1e-5)])
def test_gpu_hancock_fast_and_mixed(gpulib, oracle, prec, tol):
    """Orszag-Tang, 5 steps: fast FP64 pointwise within tol of the oracle,
    mixed precision within tol in L1 of density."""
    n = 64
    p, ng, lo, hi, U = _orszag(n, prec)
    p64, _, _, _, Uo = _orszag(n)
    ctx = mfgpu.Context(p)
    dt = 0.4 * oracle.compute_dt(p64, Uo, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for _ in range(5):
        U, _ = _gpu_step(ctx, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        periodic_fill(U, ng, 2)
        st, ndt, _ = oracle.patch_update(p64, Uo, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        periodic_fill(Uo, ng, 2)
        dt = 0.4 * ndt
    g, o = valid_view(U, ng, 2), valid_view(Uo, ng, 2)
    if prec == mfgpu.PREC_FP64_FAST:
        assert np.all(rel_err(g, o) <= tol)
    else:
        assert np.abs(g[0] - o[0]).sum() / np.abs(o[0]).sum() <= tol
    ctx.close()
