"""Edge cases of the level entry points: boxes the level refuses (none,
empty, outside the domain, overlapping, a 2D box off the z = 0 plane), and a
periodic 2D level of tiny ragged patches (one-cell-wide strips, 3-wide and
uneven blocks) whose ghosts come from several siblings and periodic images:
its FP64 steps equal the oracle's level steps bit for bit (the parity path
keeps the reference's rounding), for RK2 and first order."""
import numpy as np
import pytest

import mfgpu
from helpers import valid_view

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("boxes", [
    [],
    [((3, 0, 0), (2, 15, 0))],                                # empty (hi < lo)
    [((0, 0, 0), (16, 15, 0))],                               # outside the 16^2 domain
    [((0, 0, 0), (7, 15, 0)), ((7, 0, 0), (15, 15, 0))],      # overlapping
    [((0, 0, 0), (15, 15, 1))],                               # 2D box off the z = 0 plane
], ids=["none", "empty", "outside", "overlap", "not_2d"])
def test_level_rejects_bad_boxes(gpulib, boxes):
    p = mfgpu.orszag_params(16)
    ctx = mfgpu.Context(p)
    with pytest.raises(mfgpu.MfError) as ei:
        mfgpu.Level(ctx, boxes)
    assert ei.value.code == mfgpu.MF_ERR_BAD_ARG
    ctx.close()


# a periodic 16^2 domain cut into ragged pieces: one-cell-wide strips, a
# 3-wide strip, uneven blocks and a single cell
RAGGED = [((0, 0, 0), (0, 15, 0)), ((1, 0, 0), (3, 15, 0)), ((4, 0, 0), (15, 6, 0)),
          ((4, 7, 0), (4, 7, 0)), ((5, 7, 0), (15, 7, 0)), ((4, 8, 0), (9, 15, 0)),
          ((10, 8, 0), (15, 15, 0))]


@pytest.mark.parametrize("ta", [mfgpu.TA_RK2, mfgpu.TA_FIRST_ORDER], ids=["rk2", "first_order"])
def test_tiny_ragged_patches_equal_oracle_bitwise(gpulib, oracle, ta):
    p = mfgpu.orszag_params(16, ta, mfgpu.PREC_FP64)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    assert sum((hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) for lo, hi in RAGGED) == 256
    lev = mfgpu.Level(ctx, RAGGED)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(RAGGED)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, "orszag")
    lev.upload(flat.ctypes.data)
    arrays = [lev.patch_view(flat, i).copy() for i in range(len(RAGGED))]
    fboxes = [lev.fab_box(i) for i in range(len(RAGGED))]
    dt = 0.4 * lev.compute_dt()[0]
    for step in range(3):
        st, ndt_o, ip_o, cell_o = oracle.level_step(p, arrays, fboxes, RAGGED, dt)
        assert st == 0
        st, ndt_g, ip_g, cell_g = lev.step(dt)
        assert st == 0
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        for i in range(len(RAGGED)):
            assert np.array_equal(valid_view(lev.patch_view(out, i), ng, 2),
                                  valid_view(arrays[i], ng, 2)), (step, i)
        assert ndt_g == ndt_o and ip_g == ip_o and tuple(cell_g) == tuple(cell_o), step
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()
