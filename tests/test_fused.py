"""The fused flux + update stage kernel of the mixed-precision level step
(mf_level_set_schedule with a tile shape) against the split kernels (face
fluxes of each direction in HBM, then the update): the same face fluxes, the
same FP32 sums of the directions' differences in the same order, the same
update code; and the tile shape does not change the result (each face and
each cell is computed once per stage in every shape, and every cell sums its
differences in the same order)."""
import numpy as np
import pytest

import mfgpu
from helpers import rel_err, valid_view

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _level(p, n, patch, sd, init="helio"):
    ctx = mfgpu.Context(p)
    boxes = mfgpu.tile_boxes(n, patch, sd)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, init)
    lev.upload(flat.ctypes.data)
    return ctx, lev, boxes, flat


def _steps(lev, flat, schedule, nsteps, dt0):
    lev.upload(flat.ctypes.data)
    lev.set_time(0.0)
    lev.set_schedule(schedule)
    out_dt = []
    dt = dt0
    for _ in range(nsteps):
        st, nd, ip, cell = lev.step(dt)
        assert st == 0
        out_dt.append((nd, ip, cell))
        dt = 0.4 * nd
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    return out, out_dt


CASES = ["helio", "helio_ce32", "helio_heliobc_checkpos", "helio_first_order", "orszag2d",
         "orszag2d_first_order"]


def _params(name):
    if name.startswith("orszag2d"):
        ta = mfgpu.TA_FIRST_ORDER if name.endswith("first_order") else mfgpu.TA_RK2
        return mfgpu.orszag_params(64, ta, mfgpu.PREC_MIXED), 64, 16, 2, "orszag"
    prec = mfgpu.PREC_MIXED_CE32 if name.endswith("ce32") else mfgpu.PREC_MIXED
    ta = mfgpu.TA_FIRST_ORDER if name.endswith("first_order") else mfgpu.TA_RK2
    p = mfgpu.helio_params(48, time_approximation=ta, precision=prec)
    if "heliobc" in name:
        p.helio_bc = 1
        p.check_positivity = 1
    return p, 48, 16, 3, "helio"


@pytest.mark.parametrize("name", CASES)
def test_fused_matches_split(gpulib, name):
    """MF_PREC_MIXED: the fused and the split kernels give the same states,
    dts and argmin cells bitwise over 3 steps.  MF_PREC_MIXED_CE32: the FP32
    charge-exchange code is compiled into the two kernels with different
    fused multiply-adds, so one step agrees to FP32 rounding of the source
    (the discontinuous solver branches near the inner sphere amplify such
    differences over later steps, as between any two FP32 evaluations)."""
    p, n, patch, sd, init = _params(name)
    ctx, lev, boxes, flat = _level(p, n, patch, sd, init)
    assert lev.schedule() == (0, 0, 0)  # levels start with the split kernels
    dt0 = 0.4 * lev.compute_dt()[0]
    ce32 = name.endswith("ce32")
    nsteps = 1 if ce32 else 3
    a, da = _steps(lev, flat, (0, 0, 0), nsteps, dt0)
    launches_split = lev.launches_per_step()
    tile = (8, 8, 4) if sd == 3 else (16, 16, 1)
    b, db = _steps(lev, flat, tile, nsteps, dt0)
    assert lev.launches_per_step() < launches_split
    if not ce32:
        assert np.array_equal(a, b)
        assert da == db
    else:
        ng = ctx.ng
        worst = 0.0
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(b, i), ng, sd),
                        valid_view(lev.patch_view(a, i), ng, sd))
            worst = max(worst, float(e.max()))
        assert worst <= TOL, worst
        assert abs(da[0][0] - db[0][0]) <= TOL * da[0][0]
    lev.close()
    ctx.close()


@pytest.mark.parametrize("tile", [(4, 4, 4), (16, 8, 1), (5, 6, 3), (16, 4, 4), (8, 8, 2)])
def test_tile_shape_does_not_change_results(gpulib, tile):
    """Every tile shape (including shapes that do not divide the patches)
    gives the default shape's state, dt and argmin bitwise."""
    p = mfgpu.helio_params(32, precision=mfgpu.PREC_MIXED)
    ctx, lev, boxes, flat = _level(p, 32, 16, 3)
    dt0 = 0.4 * lev.compute_dt()[0]
    a, da = _steps(lev, flat, (8, 8, 4), 2, dt0)
    b, db = _steps(lev, flat, tile, 2, dt0)
    assert lev.schedule() == tile
    assert np.array_equal(a, b) and da == db
    lev.close()
    ctx.close()


def test_schedule_arguments(gpulib):
    p = mfgpu.helio_params(32)  # FP64: the fused kernel covers mixed precision only
    ctx, lev, boxes, flat = _level(p, 32, 16, 3)
    assert lev.schedule() == (0, 0, 0)
    with pytest.raises(mfgpu.MfError) as ei:
        lev.set_schedule((8, 8, 4))
    assert ei.value.code == mfgpu.MF_ERR_UNSUPPORTED
    lev.close()
    ctx.close()
    q = mfgpu.helio_params(32, precision=mfgpu.PREC_MIXED)
    ctx, lev, boxes, flat = _level(q, 32, 16, 3)
    for bad in ((32, 32, 1), (-1, 8, 8), (16, 16, 8)):
        with pytest.raises(mfgpu.MfError) as ei:
            lev.set_schedule(bad)
        assert ei.value.code == mfgpu.MF_ERR_BAD_ARG
    lev.close()
    ctx.close()


@pytest.mark.parametrize("prec", [mfgpu.PREC_MIXED, mfgpu.PREC_FP64])
def test_autotune_picks_a_schedule(gpulib, prec):
    """The autotuner leaves the level on a schedule it can run (split, or a
    tile shape for mixed precision; split for FP64), and the level's steps
    give the split kernels' results bitwise."""
    p = mfgpu.helio_params(32, precision=prec)
    ctx, lev, boxes, flat = _level(p, 32, 16, 3)
    dt0 = 0.4 * lev.compute_dt()[0]
    a, da = _steps(lev, flat, (0, 0, 0), 2, dt0)
    lev.upload(flat.ctypes.data)
    shapes = lev.autotune(2)
    assert all(s in (64, 128, 256) for s in shapes)
    sch = lev.schedule()
    if prec == mfgpu.PREC_FP64:
        assert sch == (0, 0, 0)
    b, db = _steps(lev, flat, sch, 2, dt0)
    assert lev.schedule() == sch
    assert np.array_equal(a, b) and da == db
    lev.close()
    ctx.close()
