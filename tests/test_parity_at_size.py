"""Parity at the benchmark configurations' full sizes.

* Orszag-Tang, 2D single-fluid ideal MHD on one 256 x 256 periodic patch with
  4 ghost layers, Roe 8-wave, minmod, 8-wave source, RK2, CFL 0.4, 200 steps
  (problems/OrszagF.ChF): the GPU patch update and the oracle each advance
  their own state; after every step the two states, the new dt and its cell
  are bitwise equal (the FP64 path keeps the reference's rounding: no fused
  multiply-adds, the Fortran's order of operations).
* The 128^3 heliosphere level (512 patches of 16^3, plasma + 3 neutral fluids,
  GLM, charge exchange, the inner sphere): two level steps against the
  oracle's level step at the per-step tolerance of 1e-12 relative in every
  conserved variable.
"""
import numpy as np
import pytest

import mfgpu
from helpers import periodic_fill, rel_err, to_device, to_host, valid_view

pytestmark = pytest.mark.gpu


def test_orszag_256_200_steps_bitwise(gpulib, oracle):
    n, steps = 256, 200
    p = mfgpu.orszag_params(n)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    Uo = periodic_fill(oracle_init(oracle, p, lo, hi), ng, 2)
    Ug = Uo.copy()
    st, dto, _ = oracle.compute_dt(p, Uo, lo, hi, vlo, vhi)
    assert st == 0
    dtg = dto
    for step in range(steps):
        st, ndt_o, cell_o = oracle.patch_update(p, Uo, lo, hi, vlo, vhi, 0.4 * dto)
        assert st == 0
        t = to_device(Ug)
        _, ndt_g, cell_g = ctx.patch_update(t.data_ptr(), lo, hi, vlo, vhi, 0.4 * dtg)
        Ug = to_host(t)
        assert np.array_equal(valid_view(Ug, ng, 2), valid_view(Uo, ng, 2)), step
        assert ndt_g == ndt_o and tuple(cell_g) == tuple(cell_o), (step, ndt_g, ndt_o)
        periodic_fill(Uo, ng, 2)
        periodic_fill(Ug, ng, 2)
        dto, dtg = ndt_o, ndt_g
    ctx.close()


def oracle_init(oracle, p, lo, hi):
    U = np.zeros(mfgpu.fab_shape(lo, hi, mfgpu.num_cons(p)))
    assert oracle.init_orszag(p, U, lo, hi, lo, hi) == 0
    return U


def test_helio_128_level_two_steps(gpulib, oracle):
    n, patch = 128, 16
    p = oracle.helio_params(n)
    q = mfgpu.helio_params(n)
    assert bytes(p) == bytes(q)
    ctx = mfgpu.Context(q)
    ng = ctx.ng
    boxes = mfgpu.tile_boxes(n, patch, 3)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    arrays, fboxes = [], []
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        a = oracle.helio_fab(p, flo, fhi)
        lev.patch_view(flat, i)[:] = a
        arrays.append(a)
        fboxes.append((flo, fhi))
    lev.upload(flat.ctypes.data)
    dt0, _, _ = lev.compute_dt()
    odt = min(oracle.compute_dt(p, a, fb[0], fb[1], b[0], b[1])[1]
              for a, fb, b in zip(arrays, fboxes, boxes))
    assert abs(dt0 - odt) <= 1e-12 * odt
    dmin, dt = dt0, 0.4 * dt0
    out = np.zeros(lev.ndoubles)
    for step in range(2):
        ch = p.factor_ch * p.dx / dmin
        cp = float(np.sqrt(ch * p.dx / p.factor_cp))
        p.dedner_ch, p.dedner_cp = ch, cp
        ctx.set_dedner(ch, cp)
        st, ndt_o, _, _ = oracle.level_step(p, arrays, fboxes, boxes, dt, time=lev.time())
        assert st == 0
        st, ndt_g, _, _ = lev.step(dt)
        assert st == 0
        lev.download(out.ctypes.data)
        worst = 0.0
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(out, i), ng, 3), valid_view(arrays[i], ng, 3))
            worst = max(worst, float(e.max()))
        assert worst <= 1e-12, (step, worst)
        assert abs(ndt_g - ndt_o) <= 1e-12 * ndt_o
        # continue both from the oracle's state
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dmin, dt = ndt_o, min(0.4 * ndt_o, 1.1 * dt)
    lev.close()
    ctx.close()
