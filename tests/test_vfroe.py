"""VFRoe MHD flux (flux 5: VFRoeRS, VFROE_FLUXES src/VFRoeF.ChF:327-658,
arithmetic averaging as RiemannSolver::make builds it, src/RiemannSolver.cpp:69-74).

CPU: the oracle's restatement is consistent (equal states give the exact
MHD flux), mirror-symmetric (reflecting the normal direction reverses the
normal fluxes) and GLM with VFRoe is refused as in the reference.  GPU: whole
patch steps with flux 5 against the oracle at the per-step tolerance, and
the fast / mixed modes within theirs.  (Face fluxes of every precision
against the committed fixtures: tests/test_golden.py.)
"""
import numpy as np
import pytest

import mfgpu
from helpers import orszag_patch, periodic_fill, rel_err, to_device, to_host, valid_view

RTOL = 1e-12


def _params():
    p = mfgpu.helio_params(16)
    p.flux, p.divb_cleaning, p.use_8wave = 5, 0, 1
    return p


def _physical_flux(w, d):
    """Exact MHD flux of one state (Gaussian units) in direction d."""
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


def _states(rng, n, nc):
    w = np.zeros((n, nc))
    w[:, 0] = rng.uniform(0.2, 2.0, n)
    w[:, 1:4] = rng.uniform(-1.5, 1.5, (n, 3))
    w[:, 4] = rng.uniform(0.1, 2.0, n)
    w[:, 5:8] = rng.uniform(-1.0, 1.0, (n, 3))
    for s in range(8, nc, 5):
        w[:, s] = rng.uniform(0.05, 1.0, n)
        w[:, s + 1:s + 4] = rng.uniform(-1.5, 1.5, (n, 3))
        w[:, s + 4] = rng.uniform(0.01, 1.0, n)
    return w


def test_vfroe_consistent(oracle):
    p = _params()
    w = _states(np.random.default_rng(5), 20, mfgpu.num_cons(p))
    for q in range(len(w)):
        for d in range(3):
            f = oracle.face_flux(p, d, w[q], w[q])[:8]
            np.testing.assert_allclose(f, _physical_flux(w[q], d), rtol=1e-12, atol=1e-13)


def test_vfroe_mirror_symmetric(oracle):
    """Reflecting x (u_x, B_x change sign; left and right swap) reverses the
    mass, tangential-momentum, energy and tangential-B fluxes and keeps the
    normal-momentum flux."""
    p = _params()
    rng = np.random.default_rng(9)
    wl, wr = _states(rng, 20, mfgpu.num_cons(p)), _states(rng, 20, mfgpu.num_cons(p))
    sign = np.array([-1, 1, -1, -1, -1, 0, -1, -1])
    for q in range(len(wl)):
        f = oracle.face_flux(p, 0, wl[q], wr[q])[:8]
        ml, mr = wr[q].copy(), wl[q].copy()
        for m in (ml, mr):
            m[1], m[5] = -m[1], -m[5]
        g = oracle.face_flux(p, 0, ml, mr)[:8]
        np.testing.assert_allclose(g, sign * f, rtol=1e-12, atol=1e-13)


def test_vfroe_with_glm_is_refused(gpulib):
    p = _params()
    p.divb_cleaning, p.use_8wave = 5, 0
    with pytest.raises(mfgpu.MfError):
        mfgpu.Context(p)


def _orszag(n, prec=mfgpu.PREC_FP64):
    p = mfgpu.orszag_params(n, mfgpu.TA_RK2, prec)
    p.flux = 5
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    return p, ng, lo, hi, orszag_patch(n, ng, p)


@pytest.mark.gpu
def test_gpu_vfroe_orszag_vs_oracle(gpulib, oracle):
    n = 64
    p, ng, lo, hi, U = _orszag(n)
    ctx = mfgpu.Context(p)
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for step in range(3):
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
@pytest.mark.parametrize("prec,tol", [(mfgpu.PREC_FP64_FAST, 1e-9), (mfgpu.PREC_MIXED, 1e-5)])
def test_gpu_vfroe_fast_and_mixed(gpulib, oracle, prec, tol):
    """5 steps: fast FP64 pointwise within tol of the oracle, mixed within
    tol in L1 of density."""
    n = 64
    p, ng, lo, hi, U = _orszag(n, prec)
    p64, _, _, _, Uo = _orszag(n)
    ctx = mfgpu.Context(p)
    dt = 0.4 * oracle.compute_dt(p64, Uo, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])[1]
    for _ in range(5):
        t = to_device(U)
        ctx.patch_update(t.data_ptr(), lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        U = periodic_fill(to_host(t), ng, 2)
        st, ndt, _ = oracle.patch_update(p64, Uo, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
        periodic_fill(Uo, ng, 2)
        dt = 0.4 * ndt
    g, o = valid_view(U, ng, 2), valid_view(Uo, ng, 2)
    if prec == mfgpu.PREC_FP64_FAST:
        assert np.all(rel_err(g, o) <= tol)
    else:
        assert np.abs(g[0] - o[0]).sum() / np.abs(o[0]).sum() <= tol
    ctx.close()
