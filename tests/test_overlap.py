"""Chunked overlap of the split flux and update kernels of mixed-precision
stages (mf_level_set_overlap): launch k of a stage computes the FP32 fluxes
of chunk k and the update of chunk k - 1 in one grid of alternating blocks.
The same per-face and per-cell code on the same data in a different launch
order: the states, dts and argmin cells equal the unchunked ones bit for
bit."""
import numpy as np
import pytest

import mfgpu

pytestmark = pytest.mark.gpu


def _level(p, n, patch, sd, init):
    ctx = mfgpu.Context(p)
    boxes = mfgpu.tile_boxes(n, patch, sd)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, init)
    return ctx, lev, flat


def _run(lev, flat, chunks, nsteps, dt0, use_async):
    lev.upload(flat.ctypes.data)
    lev.set_time(0.0)
    lev.set_overlap(chunks)
    out_dt = []
    if use_async:
        lev.seed_dt(dt0, 0.4)
        for _ in range(nsteps):
            lev.step_async()
        st, nd, ip, cell = lev.result()
        assert st == 0
        out_dt.append((nd, ip, cell))
    else:
        dt = dt0
        for _ in range(nsteps):
            st, nd, ip, cell = lev.step(dt)
            assert st == 0
            out_dt.append((nd, ip, cell))
            dt = 0.4 * nd
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    return out, out_dt


CASES = [("helio_rk2", mfgpu.PREC_MIXED), ("helio_rk2_ce32", mfgpu.PREC_MIXED_CE32),
         ("helio_first_order", mfgpu.PREC_MIXED), ("orszag2d", mfgpu.PREC_MIXED)]


@pytest.mark.parametrize("name,prec", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("use_async", [False, True], ids=["sync", "graph"])
def test_overlap_equals_unchunked(gpulib, name, prec, use_async):
    if name.startswith("orszag2d"):
        p = mfgpu.orszag_params(64, mfgpu.TA_RK2, prec)
        n, patch, sd, init = 64, 16, 2, "orszag"
    else:
        ta = mfgpu.TA_FIRST_ORDER if "first_order" in name else mfgpu.TA_RK2
        p = mfgpu.helio_params(48, time_approximation=ta, precision=prec)
        n, patch, sd, init = 48, 16, 3, "helio"
    ctx, lev, flat = _level(p, n, patch, sd, init)
    lev.upload(flat.ctypes.data)
    dt0 = 0.4 * lev.compute_dt()[0]
    base_launches = lev.launches_per_step()
    ref, rdt = _run(lev, flat, 1, 3, dt0, use_async)
    for chunks in (2, 4, 8):
        got, gdt = _run(lev, flat, chunks, 3, dt0, use_async)
        k = lev.overlap()
        assert 2 <= k <= chunks
        per = 1 if "first_order" in name else 2
        assert lev.launches_per_step() == base_launches + per * (k - sd)
        assert np.array_equal(ref, got), chunks
        assert rdt == gdt, chunks
    lev.close()
    ctx.close()


def test_overlap_arguments(gpulib):
    p = mfgpu.helio_params(32)  # FP64: the overlap covers mixed precision only
    ctx, lev, flat = _level(p, 32, 16, 3, "helio")
    assert lev.overlap() == 1
    lev.set_overlap(1)
    with pytest.raises(mfgpu.MfError) as ei:
        lev.set_overlap(2)
    assert ei.value.code == mfgpu.MF_ERR_UNSUPPORTED
    lev.close()
    ctx.close()
    q = mfgpu.helio_params(32, precision=mfgpu.PREC_MIXED)
    ctx, lev, flat = _level(q, 32, 16, 3, "helio")
    for bad in (0, -1, 9):
        with pytest.raises(mfgpu.MfError) as ei:
            lev.set_overlap(bad)
        assert ei.value.code == mfgpu.MF_ERR_BAD_ARG
    lev.close()
    ctx.close()


@pytest.mark.parametrize("chunks", [2, 4, 8])
def test_overlap_profile_step(gpulib, chunks):
    """mf_level_profile_step times the overlapped launches one by one: chunks
    + 1 flux-and-update launches per RK2 stage, no separate flux or update
    launch, as many launches as mf_level_launches_per_step counts."""
    p = mfgpu.helio_params(48, precision=mfgpu.PREC_MIXED)
    ctx, lev, flat = _level(p, 48, 16, 3, "helio")
    lev.upload(flat.ctypes.data)
    lev.set_overlap(chunks)
    k = lev.overlap()
    dt0 = 0.4 * lev.compute_dt()[0]
    prof = lev.profile_step(dt0)
    kinds = [kd for kd, _ in prof]
    assert kinds.count("flux+update") == 2 * (k + 1)
    assert kinds.count("flux") == 0 and kinds.count("update") == 0
    assert len(prof) == lev.launches_per_step()
    lev.close()
    ctx.close()
