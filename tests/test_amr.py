"""Batched levels of uneven patches (the AMR hierarchy form).

CPU: the hierarchy builder (GETRELGRAD tagging restated, the seeded patch
cover and its nesting).  GPU: a level whose patches have uneven sizes and
leave coarse-fine edges inside the domain steps exactly like the per-patch
calls and like the oracle; the autotuner changes launch shapes, not results.
"""
import numpy as np
import pytest

import mfgpu
from mfgpu import amr
from helpers import rel_err, to_device, to_host, valid_view

RTOL = 1e-12


def _relgrad_loop(u, axis, periodic):
    """GETRELGRAD (src/PatchMHDAMF.ChF:318-415) as explicit loops."""
    out = np.zeros_like(u)
    n = u.shape[axis]
    it = np.nditer(u, flags=["multi_index"])
    for _ in it:
        idx = list(it.multi_index)
        i = idx[axis]

        def at(k):
            j = list(idx)
            j[axis] = k % n
            return u[tuple(j)]

        if periodic or 0 < i < n - 1:
            diff = 0.5 * (at(i + 1) - at(i - 1))
            aver = 0.5 * (at(i + 1) + at(i - 1))
            out[tuple(idx)] = 0.0 if abs(aver) < 1e-32 else diff / aver
        elif i == 0:
            diff = at(1) - at(0)
            aver = 0.5 * (at(1) + at(0))
            out[tuple(idx)] = 0.0 if abs(aver) < 1e-32 else diff / aver
        else:
            out[tuple(idx)] = (at(i) - at(i - 1)) / (0.5 * (at(i) + at(i - 1)))
    return out


@pytest.mark.parametrize("periodic", [True, False])
def test_relgrad_matches_loops(periodic):
    rng = np.random.default_rng(3)
    u = 1.0 + rng.random((5, 6, 7))
    for axis in range(3):
        np.testing.assert_allclose(amr.relgrad(u, axis, periodic),
                                   _relgrad_loop(u, axis, periodic), rtol=0, atol=1e-15)


def test_hierarchy_cover_and_nesting():
    rng = np.random.default_rng(7)
    n0 = 32
    tags = np.zeros((n0,) * 3, bool)
    tags[rng.random((n0,) * 3) < 0.01] = True
    tags[10:14, 5:25, 8:20] = True
    levels = amr.build_hierarchy(tags, ratios=(2, 4), seed=11)
    assert [lv[0] for lv in levels] == [1, 2, 8]
    prev = None
    for R, n, boxes in levels:
        cov = np.zeros((n,) * 3, np.int32)
        for lo, hi in boxes:
            e = [h - l + 1 for l, h in zip(lo, hi)]
            assert e[0] == e[1] == e[2] and e[0] in amr.SIZES
            assert all(0 <= l and h < n for l, h in zip(lo, hi))
            cov[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] += 1
        assert cov.max() == 1  # no overlap
        if R == 1:
            assert cov.min() == 1  # the base level covers the domain
        else:
            # every cell of level l lies inside level l-1's patches
            pR, pn, pcov = prev
            r = R // pR
            under = pcov[::1, ::1, ::1].repeat(r, 0).repeat(r, 1).repeat(r, 2)
            assert not np.any((cov > 0) & (under == 0))
            # every tagged base cell under the allowed granules is covered; a
            # granule is allowed when it and its 26 neighbours (periodic) lie
            # inside level l-1 (proper nesting)
            t = tags.repeat(R, 0).repeat(R, 1).repeat(R, 2) if R > 1 else tags
            inside = amr._block_all(under > 0, amr.GRANULE)
            allowed = inside.copy()
            for sh in np.ndindex(3, 3, 3):
                allowed &= np.roll(inside, tuple(x - 1 for x in sh), axis=(0, 1, 2))
            allowed_cells = allowed.repeat(amr.GRANULE, 0).repeat(amr.GRANULE, 1).repeat(
                amr.GRANULE, 2)
            assert not np.any(t & allowed_cells & (cov == 0))
        prev = (R, n, cov)


def _partial_level_boxes():
    """Uneven patches (8^3 and 16^3) covering part of a periodic 32^3 domain:
    coarse-fine edges inside the domain, periodic neighbours across x."""
    return [((0, 0, 0), (15, 15, 15)), ((16, 0, 0), (23, 7, 7)), ((24, 0, 0), (31, 7, 7)),
            ((16, 8, 0), (23, 15, 7)), ((0, 16, 0), (7, 23, 7)), ((16, 0, 8), (31, 15, 23)),
            ((0, 0, 16), (7, 7, 23))]


def _global(p, n=32):
    """Periodic state on the whole domain; fabs index it with wrap-around so
    that ghost cells are bitwise the cells they image."""
    return amr.orszag3d_state(p, (0, 0, 0), (n - 1,) * 3)


def _fill(lev, p):
    g = _global(p)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(lev.boxes)):
        lo, hi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = amr.prolong_fab(g, 1, lo, hi)
    return flat


def test_partial_level_oracle_exchange_consistent(oracle):
    """The wrap-around fill gives sibling ghosts equal to the sibling's cells,
    so an exchange changes nothing (the precondition of the GPU comparison)."""
    p = amr.orszag3d_params(32)
    boxes = _partial_level_boxes()
    g = _global(p)
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = mfgpu.grow(lo, hi, 4, 3)
        arrays.append(np.ascontiguousarray(amr.prolong_fab(g, 1, flo, fhi)))
        fboxes.append((flo, fhi))
    before = [a.copy() for a in arrays]
    oracle.level_exchange(p, arrays, fboxes, boxes)
    for a, b in zip(arrays, before):
        assert np.array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [mfgpu.PREC_FP64, mfgpu.PREC_MIXED])
def test_partial_uneven_level_equals_patches(gpulib, prec):
    """Level step over uneven patches with coarse-fine edges == one
    mf_patch_update per patch on the same fabs (bitwise)."""
    p = amr.orszag3d_params(32, precision=prec)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    boxes = _partial_level_boxes()
    lev = mfgpu.Level(ctx, boxes)
    flat = _fill(lev, p)
    lev.upload(flat.ctypes.data)
    dt = 0.4 * lev.compute_dt()[0]
    st, ndt, ip, cell = lev.step(dt)
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    dmin = np.inf
    for i, (lo, hi) in enumerate(boxes):
        flo, fhi = lev.fab_box(i)
        t = to_device(lev.patch_view(flat, i))
        _, pdt, _ = ctx.patch_update(t.data_ptr(), flo, fhi, lo, hi, dt)
        U = to_host(t)
        assert np.array_equal(valid_view(lev.patch_view(out, i), ng, 3), valid_view(U, ng, 3)), i
        dmin = min(dmin, pdt)
    assert ndt == dmin
    lev.close()
    ctx.close()


@pytest.mark.gpu
def test_partial_uneven_level_vs_oracle(gpulib, oracle):
    p = amr.orszag3d_params(32)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    boxes = _partial_level_boxes()
    lev = mfgpu.Level(ctx, boxes)
    flat = _fill(lev, p)
    lev.upload(flat.ctypes.data)
    arrays = [lev.patch_view(flat, i).copy() for i in range(len(boxes))]
    fboxes = [lev.fab_box(i) for i in range(len(boxes))]
    dt = 0.4 * lev.compute_dt()[0]
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
        # the coarse-fine ghosts are held; continue from the oracle's valid cells
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()


@pytest.mark.gpu
def test_autotune_keeps_results(gpulib):
    p = amr.orszag3d_params(32)
    ctx = mfgpu.Context(p)
    boxes = _partial_level_boxes()
    res = []
    for tune in (False, True):
        lev = mfgpu.Level(ctx, boxes)
        flat = _fill(lev, p)
        lev.upload(flat.ctypes.data)
        if tune:
            shapes = lev.autotune(2)
            assert all(s in (64, 128, 256) for s in shapes)
        dt = 0.4 * lev.compute_dt()[0]
        lev.seed_dt(dt, 0.4)
        for _ in range(3):
            lev.step_async()
        st, ndt, ip, cell = lev.result()
        assert st == 0
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        res.append((out, ndt, ip, cell))
        lev.close()
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1:] == res[1][1:]
    ctx.close()
