"""Committed golden fixtures (tests/golden/, made by make_golden.py from the
CPU restatement on seeded inputs): the restatement must reproduce them, and
the GPU FP64 path must match them within the parity tolerance."""
import os

import numpy as np
import pytest

import mfgpu
from helpers import rel_err, to_device, to_host

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SOLVERS = [(1, 0), (3, 0), (2, 0), (4, 0), (11, 0), (13, 0), (1, 5), (3, 5)]
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
