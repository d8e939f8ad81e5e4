"""Heliosphere boundary fluxes (mf_params.helio_bc: HeliosphericProblem::fluxBC
-> HELIOBC, swlism/HeliosphericProblem.cpp:1994-2188, swlism/HeliosphericF.ChF:
221-910, with BFLUX :1363-1560 and BFLUXR :1562-1768).

CPU: known answers of the oracle's restatement on single faces (the high-x
face carries the exact far-field flux; a face whose domain-side state leaves
faster than the fast speed carries that state's flux, one entered faster
than it the ghost state's; equal subsonic states give the exact flux; the
low faces of y and z mirror the high faces; neutral populations 2 and 3 only
leave).  GPU: level steps of the 32^3 heliosphere (boundary faces on all six
sides) against the oracle at the per-step tolerance (RK2, Hancock, first
order), the fast and mixed modes within theirs.
"""
import numpy as np
import pytest

import mfgpu
from helpers import rel_err, valid_view

RTOL = 1e-12


def _params():
    p = mfgpu.helio_params(16)
    p.helio_bc = 1
    return p


def _physical_flux(w, d):
    rho, u, p, B = w[0], np.array(w[1:4]), w[4], np.array(w[5:8])
    g = 5.0 / 3.0
    un, bn = u[d], B[d]
    bb = B @ B
    P = p + bb / (8 * np.pi)
    E = p / (g - 1) + 0.5 * rho * (u @ u) + bb / (8 * np.pi)
    f = np.zeros(8)
    f[0] = rho * un
    f[1:4] = rho * un * u - bn * B / (4 * np.pi)
    f[1 + d] += P
    f[4] = un * (E + P) - bn * (u @ B) / (4 * np.pi)
    f[5:8] = un * B - u * bn
    f[5 + d] = 0.0
    return f


def _state(rng, nc):
    w = np.zeros(nc)
    w[0] = rng.uniform(0.2, 2.0)
    w[1:4] = rng.uniform(-0.8, 0.8, 3)
    w[4] = rng.uniform(0.2, 2.0)
    w[5:8] = rng.uniform(-0.6, 0.6, 3)
    w[8] = rng.uniform(-0.05, 0.05)
    for s in range(9, nc, 5):
        w[s] = rng.uniform(0.05, 1.0)
        w[s + 1:s + 4] = rng.uniform(-1.0, 1.0, 3)
        w[s + 4] = rng.uniform(0.01, 1.0)
    return w


def test_inflow_face_is_far_field_flux(oracle):
    p = _params()
    rng = np.random.default_rng(1)
    nc = mfgpu.num_cons(p)
    b = np.array(p.bc_plasma[:])
    for _ in range(5):
        f, bn = oracle.helio_bc_face(p, 0, 1, _state(rng, nc), _state(rng, nc))
        np.testing.assert_allclose(f[:8], _physical_flux(b, 0), rtol=1e-13, atol=1e-15)
        assert bn == b[5]


@pytest.mark.parametrize("d", [1, 2])
def test_supersonic_faces_take_one_side(oracle, d):
    p = _params()
    rng = np.random.default_rng(2 + d)
    nc = mfgpu.num_cons(p)
    for _ in range(5):
        win, wout = _state(rng, nc), _state(rng, nc)
        win[1 + d] = 8.0                        # leaves faster than the fast speed
        f, bn = oracle.helio_bc_face(p, d, 1, win, wout)
        np.testing.assert_allclose(f[:8], _physical_flux(win, d), rtol=1e-12, atol=1e-14)
        assert bn == win[5 + d]
        win[1 + d] = -8.0                       # entered faster than the fast speed
        f, bn = oracle.helio_bc_face(p, d, 1, win, wout)
        np.testing.assert_allclose(f[:8], _physical_flux(wout, d), rtol=1e-12, atol=1e-14)
        assert bn == wout[5 + d]


def test_equal_subsonic_states_give_exact_flux(oracle):
    p = _params()
    rng = np.random.default_rng(7)
    nc = mfgpu.num_cons(p)
    for _ in range(5):
        w = _state(rng, nc)
        w[2] = abs(w[2]) * 0.1                  # 0 <= u_y < fast speed: the Roe branch
        f, bn = oracle.helio_bc_face(p, 1, 1, w, w)
        np.testing.assert_allclose(f[:8], _physical_flux(w, 1), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("d", [1, 2])
def test_low_face_mirrors_high_face(oracle, d):
    """A low face is the high face of the problem with every velocity and
    field vector reversed (a reflection across the face composed with a half
    turn about its normal, a symmetry of ideal MHD and of the Euler
    equations): the mass and energy fluxes and Bn change sign, the momentum
    and tangential-field fluxes do not; the same for the neutral
    populations."""
    p = _params()
    nc = mfgpu.num_cons(p)
    rng = np.random.default_rng(11 + d)

    def invert(w):
        m = w.copy()
        m[1:4], m[5:8] = -m[1:4], -m[5:8]
        for s in range(9, nc, 5):
            m[s + 1:s + 4] = -m[s + 1:s + 4]
        return m

    sign = np.ones(nc)
    sign[0] = sign[4] = -1.0
    sign[8] = np.nan                           # the GLM psi flux is not HELIOBC's
    for s in range(9, nc, 5):
        sign[s] = sign[s + 4] = -1.0
    keep = ~np.isnan(sign)
    for _ in range(8):
        ghost, inner = _state(rng, nc), _state(rng, nc)
        flo, bnlo = oracle.helio_bc_face(p, d, 0, ghost, inner)
        fhi, bnhi = oracle.helio_bc_face(p, d, 1, invert(inner), invert(ghost))
        np.testing.assert_allclose(flo[keep], (sign * fhi)[keep], rtol=1e-12, atol=1e-14)
        assert bnlo == pytest.approx(-bnhi, rel=1e-14, abs=1e-15)


def test_neutral_populations_2_3_only_leave(oracle):
    p = _params()
    nc = mfgpu.num_cons(p)
    rng = np.random.default_rng(5)
    for d in range(3):
        w = _state(rng, nc)
        for f_ in (2, 3):
            w[9 + (f_ - 1) * 5 + 1 + d] = -0.5    # moving into the domain at a high face
        f, _ = oracle.helio_bc_face(p, d, 1, w, _state(rng, nc))
        assert f[14] == 0.0 and f[19] == 0.0


def test_heliobc_needs_farfield_3d(gpulib):
    p = mfgpu.orszag_params(16)
    p.helio_bc = 1
    with pytest.raises(mfgpu.MfError):
        mfgpu.Context(p)


def _level_case(ta, prec=mfgpu.PREC_FP64, n=32):
    p = mfgpu.helio_params(n, time_approximation=ta, precision=prec)
    p.helio_bc = 1
    return p, mfgpu.tile_boxes(n, 16, 3)


def _host_level(p, boxes):
    ng = mfgpu.num_ghost(p)
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = mfgpu.grow(lo, hi, ng, 3)
        arrays.append(np.ascontiguousarray(mfgpu.init_host_fab(p, flo, fhi, "helio")))
        fboxes.append((flo, fhi))
    return arrays, fboxes


def _device_level(p, boxes, arrays):
    """A device level holding the host arrays; GLM speeds from its dt."""
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
    return ctx, lev, flat, dt0


@pytest.mark.gpu
@pytest.mark.parametrize("ta", [mfgpu.TA_RK2, mfgpu.TA_HANCOCK, mfgpu.TA_FIRST_ORDER])
def test_gpu_heliobc_level_vs_oracle(gpulib, oracle, ta):
    p, boxes = _level_case(ta)
    arrays, fboxes = _host_level(p, boxes)
    ctx, lev, flat, dt0 = _device_level(p, boxes, arrays)
    ng = ctx.ng
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
        # next step from the oracle's state (as the other level tests do)
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dt = 0.4 * ndt_o
    lev.close()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(mfgpu.PREC_FP64_FAST, 1e-7), (mfgpu.PREC_MIXED, 1e-5)])
def test_gpu_heliobc_fast_and_mixed(gpulib, oracle, prec, tol):
    """64^3, 3 steps: fast FP64 pointwise within tol of the oracle, mixed
    within tol in L1 of density.  (On 32^3 the r = 0.1 sphere is 1.6 cells
    wide and the mixed form differs by 1e-3 next to it, with or without the
    boundary fluxes.)"""
    p, boxes = _level_case(mfgpu.TA_RK2, prec, 64)
    p64, _ = _level_case(mfgpu.TA_RK2, n=64)
    arrays, fboxes = _host_level(p64, boxes)
    ctx, lev, flat, dt0 = _device_level(p, boxes, arrays)
    p64.dedner_ch, p64.dedner_cp = p.dedner_ch, p.dedner_cp
    ng = ctx.ng
    dt = 0.4 * dt0
    for _ in range(3):
        lev.step(dt)
        st, ndt, _, _ = oracle.level_step(p64, arrays, fboxes, boxes, dt)
        dt = 0.4 * ndt
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    num = den = 0.0
    for i in range(len(boxes)):
        g = valid_view(lev.patch_view(out, i), ng, 3)
        o = valid_view(arrays[i], ng, 3)
        if prec == mfgpu.PREC_FP64_FAST:
            # psi starts at zero and stays near round-off (1e-12): checked
            # against the field's scale instead of pointwise relative
            e = rel_err(g, o)
            assert np.all(np.delete(e, 8) <= tol), (i, e)
            assert np.max(np.abs(g[8] - o[8])) <= tol * np.max(np.abs(o[5:8])), i
        num += np.abs(g[0] - o[0]).sum()
        den += np.abs(o[0]).sum()
    if prec == mfgpu.PREC_MIXED:
        assert num / den <= tol
    lev.close()
    ctx.close()
