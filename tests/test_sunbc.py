"""Neutral pass-through at the sun (mf_params.neutral_sun_bc:
HeliosphericProblem::postTimeStep -> NEUTRALS_SUNBC, swlism/SWLISMF.ChF:
1555-1598, strips of HeliosphericProblem::define,
swlism/HeliosphericProblem.cpp:476-527).

After a level step every cell of the sphere of radius sun_r downstream of
the sun holds neutral fluid 1 of the cell mirrored across the sun's x plane
with the y and z momenta reversed: in the oracle's level step (CPU) and in
the device level step, which also matches the oracle at the per-step
tolerance (GPU).  A single-patch update does not apply it (a level
post-processing in the reference).
"""
import numpy as np
import pytest

import mfgpu
from helpers import rel_err, valid_view

N = 32


def _global(arrays, boxes, ng, nc):
    G = np.zeros((nc, N, N, N))
    for a, (lo, hi) in zip(arrays, boxes):
        G[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = a[:, ng:-ng, ng:-ng, ng:-ng]
    return G


def _mirror_pairs(p):
    dx = p.dx
    sun = [int(np.floor(p.sun_center[d] / dx + 0.5)) for d in range(3)]
    iR0 = 1 + int(np.floor(p.reinit_r0 / dx + 0.5))
    pairs = []
    for a in range(iR0):
        for k in range(sun[2] - iR0 - 1, sun[2] + iR0 + 1):
            for j in range(sun[1] - iR0 - 1, sun[1] + iR0 + 1):
                i = sun[0] + a
                x = (i + 0.5) * dx - p.sun_center[0]
                y = (j + 0.5) * dx - p.sun_center[1]
                z = (k + 0.5) * dx - p.sun_center[2]
                if x * x + y * y + z * z <= p.sun_r * p.sun_r:
                    pairs.append(((i, j, k), (sun[0] - (i - sun[0] + 1), j, k)))
    return pairs


def _check_mirror(G, p):
    pairs = _mirror_pairs(p)
    assert len(pairs) > 0
    s0 = 9  # neutral fluid 1 (GLM: psi at 8)
    for (i, j, k), (f, _, _) in pairs:
        to, src = G[s0:s0 + 5, k, j, i], G[s0:s0 + 5, k, j, f]
        assert np.array_equal(to, src * np.array([1, 1, -1, -1, 1])), (i, j, k)


def _setup(p):
    boxes = mfgpu.tile_boxes(N, 16, 3)
    ng = mfgpu.num_ghost(p)
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = mfgpu.grow(lo, hi, ng, 3)
        arrays.append(np.ascontiguousarray(mfgpu.init_host_fab(p, flo, fhi, "helio")))
        fboxes.append((flo, fhi))
    return boxes, ng, arrays, fboxes


def test_oracle_level_step_passes_neutrals_through_the_sun(oracle):
    p = mfgpu.helio_params(N)
    assert p.neutral_sun_bc == 1
    boxes, ng, arrays, fboxes = _setup(p)
    st, _, _, _ = oracle.level_step(p, arrays, fboxes, boxes, 1e-4)
    assert st == 0
    _check_mirror(_global(arrays, boxes, ng, mfgpu.num_cons(p)), p)
    # off: the relation does not hold after the step
    q = mfgpu.helio_params(N)
    q.neutral_sun_bc = 0
    boxes, ng, arrays, fboxes = _setup(q)
    oracle.level_step(q, arrays, fboxes, boxes, 1e-4)
    with pytest.raises(AssertionError):
        _check_mirror(_global(arrays, boxes, ng, mfgpu.num_cons(q)), q)


def test_sun_bc_needs_neutrals_3d(gpulib):
    p = mfgpu.orszag_params(16)
    p.neutral_sun_bc = 1
    with pytest.raises(mfgpu.MfError):
        mfgpu.Context(p)


@pytest.mark.gpu
def test_gpu_level_sun_bc_vs_oracle(gpulib, oracle):
    p = mfgpu.helio_params(N)
    boxes, ng, arrays, fboxes = _setup(p)
    ctx = mfgpu.Context(p)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i, a in enumerate(arrays):
        lev.patch_view(flat, i)[:] = a
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
    outs = [lev.patch_view(out, i).copy() for i in range(len(boxes))]
    _check_mirror(_global(outs, boxes, ng, ctx.nc), p)
    for i in range(len(boxes)):
        e = rel_err(valid_view(outs[i], ng, 3), valid_view(arrays[i], ng, 3))
        assert np.all(e <= 1e-12), (i, e)
    assert abs(ndt_g - ndt_o) <= 1e-12 * ndt_o
    lev.close()
    ctx.close()
