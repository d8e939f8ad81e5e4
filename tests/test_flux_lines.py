"""Face fluxes of the FP64 paths by lines (mf_level_set_flux_form with
MF_FLUX_LINES): blocks over whole lines of faces along a direction compute
each cell's limited face values once in shared memory, then the Riemann
fluxes.  The same face_values calls on the same inputs and the same Riemann
code as the per-face kernel: in the parity path (MF_PREC_FP64, no
contraction) the level's states, dts and argmin cells are bitwise those of
MF_FLUX_FACES; in MF_PREC_FP64_FAST the two kernels may contract different
products into multiply-adds, so they agree to rounding."""
import numpy as np
import pytest

import mfgpu
from helpers import rel_err, valid_view
from mfgpu import amr

pytestmark = pytest.mark.gpu


def _helio(n, prec=mfgpu.PREC_FP64, ta=mfgpu.TA_RK2, **kw):
    p = mfgpu.helio_params(n, time_approximation=ta, precision=prec,
                           region_tracer=kw.pop("region_tracer", False))
    for k, v in kw.items():
        if k == "limiter":
            for q in range(8):
                p.limiter[q] = v
        else:
            setattr(p, k, v)
    return p


CASES = {
    "helio": lambda prec: (_helio(48, prec), 48, 16, 3, "helio"),
    "helio_checkpos_char_vanalbada": lambda prec: (
        _helio(32, prec, check_positivity=1, char_reconstruction=1,
               limiter=mfgpu.LIM_VANALBADA), 32, 16, 3, "helio"),
    "helio_tracer_heliobc": lambda prec: (
        _helio(32, prec, region_tracer=True, helio_bc=1), 32, 16, 3, "helio"),
    "helio_first_order": lambda prec: (
        _helio(32, prec, ta=mfgpu.TA_FIRST_ORDER), 32, 8, 3, "helio"),
    "orszag2d": lambda prec: (mfgpu.orszag_params(64, mfgpu.TA_RK2, prec), 64, 16, 2, "orszag"),
}


def _level(p, n, patch, sd, init):
    ctx = mfgpu.Context(p)
    boxes = mfgpu.tile_boxes(n, patch, sd)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, init)
    return ctx, lev, flat, boxes


def _steps(lev, flat, form, nsteps, dt0, ctx):
    lev.upload(flat.ctypes.data)
    lev.set_time(0.0)
    lev.set_flux_form(form)
    assert lev.flux_form() == form
    out_dt, dt = [], dt0
    for _ in range(nsteps):
        st, nd, ip, cell = lev.step(dt)
        assert st == 0
        out_dt.append((nd, ip, cell))
        dt = 0.4 * nd
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    return out, out_dt


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("prec", [mfgpu.PREC_FP64, mfgpu.PREC_FP64_FAST], ids=["fp64", "fast"])
def test_lines_equal_faces(gpulib, name, prec):
    p, n, patch, sd, init = CASES[name](prec)
    ctx, lev, flat, boxes = _level(p, n, patch, sd, init)
    lev.upload(flat.ctypes.data)
    dt0 = 0.4 * lev.compute_dt()[0]
    a, da = _steps(lev, flat, mfgpu.FLUX_FACES, 2, dt0, ctx)
    b, db = _steps(lev, flat, mfgpu.FLUX_LINES, 2, dt0, ctx)
    if prec == mfgpu.PREC_FP64:
        assert np.array_equal(a, b)
        assert da == db
    else:
        ng = ctx.ng
        worst = 0.0
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(b, i), ng, sd),
                        valid_view(lev.patch_view(a, i), ng, sd))
            worst = max(worst, float(e.max()))
        assert worst <= 1e-12, worst
    lev.close()
    ctx.close()


def test_lines_equal_faces_uneven_partial_level(gpulib):
    """Uneven patches (8^3 and 16^3) covering part of a periodic domain."""
    boxes = [((0, 0, 0), (15, 15, 15)), ((16, 0, 0), (23, 7, 7)), ((24, 0, 0), (31, 7, 7)),
             ((16, 8, 0), (23, 15, 7)), ((0, 16, 0), (7, 23, 7)), ((16, 0, 8), (31, 15, 23)),
             ((0, 0, 16), (7, 7, 23))]
    p = amr.orszag3d_params(32)
    ctx = mfgpu.Context(p)
    lev = mfgpu.Level(ctx, boxes)
    g = amr.orszag3d_state(p, (0, 0, 0), (31, 31, 31))
    buf = amr.fill_level_buffer(lev, g, 1)
    res = []
    for form in (mfgpu.FLUX_FACES, mfgpu.FLUX_LINES):
        lev.upload(buf.ctypes.data)
        lev.set_flux_form(form)
        dt = 0.4 * lev.compute_dt()[0]
        steps = []
        for _ in range(2):
            st, nd, ip, cell = lev.step(dt)
            assert st == 0
            steps.append((nd, ip, cell))
            dt = 0.4 * nd
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        res.append((out, steps))
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1]
    lev.close()
    ctx.close()


def test_flux_form_arguments(gpulib):
    p = mfgpu.helio_params(32, precision=mfgpu.PREC_MIXED)
    ctx, lev, flat, _ = _level(p, 32, 16, 3, "helio")
    assert lev.flux_form() == mfgpu.FLUX_FACES
    with pytest.raises(mfgpu.MfError) as ei:
        lev.set_flux_form(mfgpu.FLUX_LINES)
    assert ei.value.code == mfgpu.MF_ERR_UNSUPPORTED
    lev.close()
    ctx.close()
    q = mfgpu.helio_params(32)
    ctx, lev, flat, _ = _level(q, 32, 16, 3, "helio")
    for bad in (-1, 2):
        with pytest.raises(mfgpu.MfError) as ei:
            lev.set_flux_form(bad)
        assert ei.value.code == mfgpu.MF_ERR_BAD_ARG
    lev.set_flux_form(mfgpu.FLUX_LINES)
    shapes = lev.autotune(2)
    assert lev.flux_form() in (mfgpu.FLUX_FACES, mfgpu.FLUX_LINES)
    assert all(s in (64, 128, 256) for s in shapes)
    lev.close()
    ctx.close()


def test_flux_lines_refuse_long_patches(gpulib):
    """A patch longer than 254 cells along a direction does not fit one
    block's shared memory in the line form: MF_ERR_UNSUPPORTED, and the level
    keeps stepping per face."""
    p = mfgpu.orszag_params(512, mfgpu.TA_RK2, mfgpu.PREC_FP64)
    ctx = mfgpu.Context(p)
    lev = mfgpu.Level(ctx, [((0, 0, 0), (511, 63, 0))] + [((0, y, 0), (511, y + 63, 0))
                                                         for y in range(64, 512, 64)])
    with pytest.raises(mfgpu.MfError) as ei:
        lev.set_flux_form(mfgpu.FLUX_LINES)
    assert ei.value.code == mfgpu.MF_ERR_UNSUPPORTED
    assert lev.flux_form() == mfgpu.FLUX_FACES
    lev.close()
    ctx.close()
