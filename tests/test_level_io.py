"""Valid-cell transfers of a level (mf_level_upload_valid / _download_valid):
the packed host layout holds each patch's valid box at
mf_level_valid_offset(p); an upload writes exactly the valid cells of every
fab and leaves the ghosts alone; a download returns them; a level step from
valid-only uploads equals the step from a full upload (the step fills the
ghosts by its exchange)."""
import numpy as np
import pytest

import mfgpu
from helpers import valid_view

pytestmark = pytest.mark.gpu


def _level(n=32, patch=16):
    p = mfgpu.orszag_params(n)
    ctx = mfgpu.Context(p)
    boxes = mfgpu.tile_boxes(n, patch, 2)
    lev = mfgpu.Level(ctx, boxes)
    return p, ctx, boxes, lev


def test_valid_transfers_round_trip(gpulib):
    p, ctx, boxes, lev = _level()
    ng, nc = ctx.ng, ctx.nc
    assert lev.valid_doubles() == nc * sum(
        (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) for lo, hi in boxes)
    rng = np.random.default_rng(3)
    full = rng.standard_normal(lev.ndoubles)
    lev.upload(full.ctypes.data)
    packed = rng.standard_normal(lev.valid_doubles())
    lev.upload_valid(packed.ctypes.data)
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    for i in range(len(boxes)):
        g, f = lev.patch_view(out, i), lev.patch_view(full, i)
        assert np.array_equal(valid_view(g, ng, 2), lev.valid_view(packed, i))
        mask = np.ones(g.shape, bool)
        mask[:, :, ng:-ng, ng:-ng] = False
        assert np.array_equal(g[mask], f[mask])          # ghosts untouched
    back = np.zeros(lev.valid_doubles())
    lev.download_valid(back.ctypes.data)
    assert np.array_equal(back, packed)
    lev.close()
    ctx.close()


def test_step_from_valid_upload_equals_full_upload(gpulib):
    p, ctx, boxes, lev = _level()
    ng = ctx.ng
    flat = np.zeros(lev.ndoubles)
    for i, (lo, hi) in enumerate(boxes):
        flo, fhi = mfgpu.grow(lo, hi, ng, 2)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, "orszag")
    lev.upload(flat.ctypes.data)
    dt = 0.4 * lev.compute_dt()[0]
    assert lev.step(dt)[0] == 0
    ref = np.zeros(lev.ndoubles)
    lev.download(ref.ctypes.data)
    # the same step from the valid cells only, on a level whose ghosts are zero
    lev2 = mfgpu.Level(ctx, boxes)
    packed = np.zeros(lev2.valid_doubles())
    for i in range(len(boxes)):
        lev2.valid_view(packed, i)[:] = valid_view(lev.patch_view(flat, i), ng, 2)
    lev2.upload_valid(packed.ctypes.data)
    assert lev2.step(dt)[0] == 0
    out = np.zeros(lev2.valid_doubles())
    lev2.download_valid(out.ctypes.data)
    for i in range(len(boxes)):
        assert np.array_equal(lev2.valid_view(out, i), valid_view(lev.patch_view(ref, i), ng, 2))
    lev2.close()
    lev.close()
    ctx.close()
