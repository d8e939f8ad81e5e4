"""Characteristic reconstruction (mhdam.char_reconstruction, Reconstruction::
faceValues src/Reconstruction.cpp:178-203: INITIALSLOPES, CHARANALYSISF, the
*FACESLOPES limiters, CHARSYNTHESISF, FROMSLOPESTOVALUES, CHECKTVD).

CPU: the oracle's characteristic path is active (results differ from the
primitive-variable path), conserves mass on a periodic box and keeps a uniform
state.  GPU: the CUDA path matches the oracle at the per-step tolerance for
every limiter, each TVD mode, RK2 and Hancock, and the GLM heliosphere level.
"""
import numpy as np
import pytest

import mfgpu
from helpers import orszag_patch, periodic_fill, rel_err, to_device, to_host, valid_view

RTOL = 1e-12
LIMS = list(mfgpu.LIMITERS)


def _case(n, ta=mfgpu.TA_RK2, lim=mfgpu.LIM_MINMOD, tvd=0, prec=mfgpu.PREC_FP64):
    p = mfgpu.orszag_params(n, ta, prec)
    p.char_reconstruction = 1
    p.check_tvd = tvd
    for q in range(8):
        p.limiter[q] = lim
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    return p, ng, lo, hi, orszag_patch(n, ng, p)


def test_char_path_active_and_conservative(oracle):
    n = 32
    p, ng, lo, hi, U = _case(n, tvd=1)
    q, _, _, _, V = _case(n)
    q.char_reconstruction = 0
    m0 = U[0, :, ng:-ng, ng:-ng].sum()
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for _ in range(5):
        assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)[0] == 0
        assert oracle.patch_update(q, V, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)[0] == 0
        periodic_fill(U, ng, 2)
        periodic_fill(V, ng, 2)
    assert np.all(np.isfinite(U))
    assert abs(U[0, :, ng:-ng, ng:-ng].sum() - m0) <= 1e-13 * m0
    assert np.max(np.abs(U - V)) > 1e-6  # the characteristic limiter changes the result


def test_char_path_keeps_uniform_state(oracle):
    n = 16
    p, ng, lo, hi, U = _case(n, tvd=1)
    U[:] = U[:, :, ng:ng + 1, ng:ng + 1]
    U0 = U.copy()
    assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], 1e-3)[0] == 0
    np.testing.assert_allclose(valid_view(U, ng, 2), valid_view(U0, ng, 2), rtol=1e-14, atol=1e-15)


def _gpu_vs_oracle(oracle, p, ng, lo, hi, U, n, steps=2):
    ctx = mfgpu.Context(p)
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for step in range(steps):
        t = to_device(U)
        _, ndt_g, _ = ctx.patch_update(t.data_ptr(), lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        Ug = to_host(t)
        st, ndt_o, _ = oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        assert st == 0
        e = rel_err(valid_view(Ug, ng, 2), valid_view(U, ng, 2))
        assert np.all(e <= RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        periodic_fill(U, ng, 2)
        dt = 0.4 * ndt_o
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("lim", LIMS)
def test_gpu_char_limiters_vs_oracle(gpulib, oracle, lim):
    n = 64
    p, ng, lo, hi, U = _case(n, lim=lim)
    _gpu_vs_oracle(oracle, p, ng, lo, hi, U, n)


@pytest.mark.gpu
@pytest.mark.parametrize("tvd", [1, 2])
@pytest.mark.parametrize("ta", [mfgpu.TA_RK2, mfgpu.TA_HANCOCK])
def test_gpu_char_tvd_and_time_vs_oracle(gpulib, oracle, tvd, ta):
    n = 64
    p, ng, lo, hi, U = _case(n, ta=ta, lim=mfgpu.LIM_VANLEER, tvd=tvd)
    _gpu_vs_oracle(oracle, p, ng, lo, hi, U, n)


@pytest.mark.gpu
def test_gpu_char_helio_level_vs_oracle(gpulib, oracle):
    n, patch = 32, 16
    p = mfgpu.helio_params(n)
    p.char_reconstruction, p.check_tvd = 1, 1
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
    st, ndt_o, _, _ = oracle.level_step(p, arrays, fboxes, boxes, 0.4 * dt0)
    assert st == 0
    st, ndt_g, _, _ = lev.step(0.4 * dt0)
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    for i in range(len(boxes)):
        e = rel_err(valid_view(lev.patch_view(out, i), ng, 3), valid_view(arrays[i], ng, 3))
        assert np.all(e <= RTOL), (i, e)
    assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
    lev.close()
    ctx.close()


@pytest.mark.gpu
def test_gpu_char_mixed_close(gpulib, oracle):
    """Mixed precision with characteristic limiting (projections in FP64):
    L1 of density within 1e-5 of the oracle after 5 steps."""
    n = 64
    p, ng, lo, hi, U = _case(n, prec=mfgpu.PREC_MIXED, tvd=1)
    p64, _, _, _, Uo = _case(n, tvd=1)
    ctx = mfgpu.Context(p)
    dt = 0.4 * oracle.compute_dt(p64, Uo, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for _ in range(5):
        t = to_device(U)
        ctx.patch_update(t.data_ptr(), lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        U = to_host(t)
        periodic_fill(U, ng, 2)
        st, ndt, _ = oracle.patch_update(p64, Uo, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        periodic_fill(Uo, ng, 2)
        dt = 0.4 * ndt
    g, o = valid_view(U, ng, 2), valid_view(Uo, ng, 2)
    assert np.abs(g[0] - o[0]).sum() / np.abs(o[0]).sum() <= 1e-5
    ctx.close()
