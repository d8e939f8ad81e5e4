"""Committed golden fixtures (tests/golden/, made by make_golden.py from the
CPU restatement on seeded inputs): the restatement must reproduce them, and
the GPU FP64 path must match them within the parity tolerance."""
import os

import numpy as np
import pytest

import mfgpu
from helpers import rel_err, to_device, to_host

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SOLVERS = [(1, 0), (3, 0), (2, 0), (4, 0), (11, 0), (13, 0), (1, 5), (3, 5), (5, 0)]
RTOL_CPU = 1e-13
RTOL_GPU = 1e-12


def _load(name):
    return np.load(os.path.join(HERE, name))


def _solver_params(flux, cleaning):
    p = mfgpu.helio_params(16)
    p.flux, p.divb_cleaning = flux, cleaning
    p.use_8wave = 0 if cleaning == 5 else 1
    p.dedner_ch = 2.5
    return p


def test_face_fluxes_reproduce(oracle):
    g = _load("face_fluxes.npz")
    for flux, cleaning in SOLVERS:
        key = f"{flux}_{cleaning}"
        p = _solver_params(flux, cleaning)
        wl, wr, f = g[f"wl_{key}"], g[f"wr_{key}"], g[f"f_{key}"]
        for q in range(wl.shape[0]):
            for d in range(3):
                np.testing.assert_allclose(oracle.face_flux(p, d, wl[q], wr[q]), f[q, d],
                                           rtol=RTOL_CPU, atol=1e-15)


def test_orszag_step_reproduces(oracle):
    g = _load("orszag16_rk2.npz")
    p = mfgpu.orszag_params(16)
    U = g["u0"].copy()
    lo, hi = mfgpu.grow([0, 0, 0], [15, 15, 0], 4, 2)
    st, ndt, cell = oracle.patch_update(p, U, lo, hi, [0, 0, 0], [15, 15, 0], g["dt"][0])
    assert st == 0
    assert np.all(rel_err(U[:, :, 4:-4, 4:-4], g["u1"]) <= RTOL_CPU)
    assert ndt == pytest.approx(g["dt"][1], rel=RTOL_CPU)


def test_helio_step_reproduces(oracle):
    g = _load("helio12_rk2.npz")
    p = mfgpu.helio_params(12)
    p.dedner_ch, p.dedner_cp = g["dt"][2], g["dt"][3]
    U = g["u0"].copy()
    lo, hi = mfgpu.grow([0, 0, 0], [11] * 3, 4, 3)
    st, ndt, _ = oracle.patch_update(p, U, lo, hi, [0, 0, 0], [11] * 3, g["dt"][0])
    assert st == 0
    assert np.all(rel_err(U[:, 4:-4, 4:-4, 4:-4], g["u1"]) <= RTOL_CPU)
    assert ndt == pytest.approx(g["dt"][1], rel=RTOL_CPU)


def test_charge_exchange_reproduces(oracle):
    g = _load("charge_exchange.npz")
    p = mfgpu.helio_params(16)
    for q in range(g["w"].shape[0]):
        np.testing.assert_allclose(oracle.charge_exchange(p, g["w"][q], int(g["reg"][q]), 0.01),
                                   g["s"][q], rtol=RTOL_CPU, atol=1e-16)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["orszag16_rk2.npz", "helio12_rk2.npz"])
def test_gpu_matches_golden(gpulib, case):
    g = _load(case)
    if case.startswith("orszag"):
        p = mfgpu.orszag_params(16)
        sd, n = 2, 16
    else:
        p = mfgpu.helio_params(12)
        p.dedner_ch, p.dedner_cp = g["dt"][2], g["dt"][3]
        sd, n = 3, 12
    ctx = mfgpu.Context(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, n - 1 if sd == 3 else 0], 4, sd)
    t = to_device(g["u0"])
    _, ndt, _ = ctx.patch_update(t.data_ptr(), lo, hi, [0, 0, 0],
                                 [n - 1, n - 1, n - 1 if sd == 3 else 0], g["dt"][0])
    U = to_host(t)
    v = U[:, :, 4:-4, 4:-4] if sd == 2 else U[:, 4:-4, 4:-4, 4:-4]
    assert np.all(rel_err(v, g["u1"]) <= RTOL_GPU)
    assert ndt == pytest.approx(g["dt"][1], rel=RTOL_GPU)
    ctx.close()


def _face_err(g, f):
    """|g - f| / max(|f|, 1e-3 * largest flux of the face), per value."""
    s = np.max(np.abs(f), axis=1, keepdims=True)
    return np.abs(g - f) / np.maximum(np.abs(f), 1e-3 * s)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(mfgpu.PREC_FP64, RTOL_GPU), (mfgpu.PREC_FP64_FAST, 1e-7)])
def test_gpu_face_fluxes_match_golden(gpulib, prec, tol):
    """mf_face_fluxes (every solver, GLM and van Leer) against the fixtures."""
    g = _load("face_fluxes.npz")
    for flux, cleaning in SOLVERS:
        key = f"{flux}_{cleaning}"
        p = _solver_params(flux, cleaning)
        p.precision = prec
        ctx = mfgpu.Context(p)
        wl, wr, f = g[f"wl_{key}"], g[f"wr_{key}"], g[f"f_{key}"]
        for d in range(3):
            out = mfgpu.face_fluxes(ctx, d, wl, wr)
            assert np.all(_face_err(out, f[:, d]) <= tol), (key, d)
        ctx.close()


# A face between two cells at the pressure floor expanding away from each
# other (cold, magnetically dominated plasma next to the inner sphere):
# rho, u, v, w, p, bx, by, bz of the left and right states.
COLD_WL = [1.2397, -6.13836, -6.11161, -5.8306, 1e-10, -0.0621729, -0.0367102, -0.027216]
COLD_WR = [1.24407, 6.05228, -6.09729, -5.81983, 1e-10, 0.0122034, -0.0436705, -0.025546]


@pytest.mark.gpu
def test_mixed_cold_face_takes_rusanov(gpulib, oracle):
    """FP32 Roe eigenvectors are ill-conditioned at c^2 << b^2; the mixed
    path takes the Rusanov flux there (checked against the oracle's FP64
    Rusanov flux), and keeps the Roe flux on ordinary faces."""
    p = mfgpu.helio_params(16)
    p.divb_cleaning, p.use_8wave, p.flux = 0, 1, 1
    nc = mfgpu.num_cons(p)
    wl = np.zeros((1, nc))
    wr = np.zeros((1, nc))
    wl[0, :8], wr[0, :8] = COLD_WL, COLD_WR
    for f in range(3):  # ordinary neutral states
        s = 8 + 5 * f
        wl[0, s:s + 5] = wr[0, s:s + 5] = [0.1, -1.0, 0.0, 0.0, 0.05]
    p.precision = mfgpu.PREC_MIXED
    ctx = mfgpu.Context(p)
    got = mfgpu.face_fluxes(ctx, 0, wl, wr)[0]
    ctx.close()
    q = mfgpu.helio_params(16)
    q.divb_cleaning, q.use_8wave, q.flux = 0, 1, 2
    ref = oracle.face_flux(q, 0, wl[0], wr[0])
    assert np.all(np.isfinite(got))
    assert np.all(_face_err(got[None, :8], ref[None, :8]) <= 1e-4)
    # ordinary (warm) states: the mixed Roe flux stays within FP32 of the oracle's Roe flux
    wl[0, 4] = wr[0, 4] = 1.0
    ctx = mfgpu.Context(p)
    got = mfgpu.face_fluxes(ctx, 0, wl, wr)[0]
    ctx.close()
    q.flux = 1
    ref = oracle.face_flux(q, 0, wl[0], wr[0])
    assert np.all(_face_err(got[None, :8], ref[None, :8]) <= 1e-4)
