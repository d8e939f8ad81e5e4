"""Regenerate the committed golden fixtures of the CPU restatement.

    python tests/golden/make_golden.py

The reference publishes no test vectors and cannot be built here, so these
fixtures are outputs of the restatement itself (oracle/mf_oracle.c) on seeded
inputs.  They pin the restatement against drift; the restatement is pinned to
the reference's algorithm by tests/test_oracle_kats.py."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "ms-flukss-multifluid_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import mfgpu  # noqa: E402
import pyoracle  # noqa: E402
from helpers import periodic_fill  # noqa: E402

SOLVERS = [(1, 0), (3, 0), (2, 0), (4, 0), (11, 0), (13, 0), (1, 5), (3, 5), (5, 0)]


def solver_params(flux, cleaning):
    p = mfgpu.helio_params(16)
    p.flux, p.divb_cleaning = flux, cleaning
    p.use_8wave = 0 if cleaning == 5 else 1
    p.dedner_ch = 2.5
    return p


def random_states(rng, nc, glm, n):
    w = np.zeros((n, nc))
    w[:, 0] = rng.uniform(0.2, 2.0, n)
    w[:, 1:4] = rng.uniform(-1.5, 1.5, (n, 3))
    w[:, 4] = rng.uniform(0.1, 2.0, n)
    w[:, 5:8] = rng.uniform(-1.0, 1.0, (n, 3))
    if glm:
        w[:, 8] = rng.uniform(-0.1, 0.1, n)
    s = 8 + glm
    while s + 5 <= nc:
        w[:, s] = rng.uniform(0.05, 1.0, n)
        w[:, s + 1:s + 4] = rng.uniform(-1.5, 1.5, (n, 3))
        w[:, s + 4] = rng.uniform(0.01, 1.0, n)
        s += 5
    return w


def face_fluxes():
    out = {}
    for flux, cleaning in SOLVERS:
        p = solver_params(flux, cleaning)
        nc = mfgpu.num_cons(p)
        rng = np.random.default_rng(100 + flux + 7 * cleaning)
        wl = random_states(rng, nc, cleaning == 5, 16)
        wr = random_states(rng, nc, cleaning == 5, 16)
        f = np.array([[pyoracle.face_flux(p, d, wl[q], wr[q]) for d in range(3)]
                      for q in range(16)])
        key = f"{flux}_{cleaning}"
        out[f"wl_{key}"], out[f"wr_{key}"], out[f"f_{key}"] = wl, wr, f
    return out


def orszag_step():
    n = 16
    p = mfgpu.orszag_params(n)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], 4, 2)
    U0 = periodic_fill(mfgpu.init_host_fab(p, lo, hi, "orszag"), 4, 2)
    U = U0.copy()
    st, dt0, _ = pyoracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0])
    st, ndt, cell = pyoracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], 0.4 * dt0)
    assert st == 0
    return {"u0": U0, "u1": U[:, :, 4:-4, 4:-4].copy(), "dt": np.array([0.4 * dt0, ndt]),
            "cell": np.array(cell)}


def helio_step():
    n = 12
    p = mfgpu.helio_params(n)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1] * 3, 4, 3)
    U0 = mfgpu.init_host_fab(p, lo, hi, "helio")
    U = U0.copy()
    st, dt0, _ = pyoracle.compute_dt(p, U, lo, hi, [0, 0, 0], [n - 1] * 3)
    ch = p.factor_ch * p.dx / dt0
    cp = np.sqrt(ch * p.dx / p.factor_cp)
    p.dedner_ch, p.dedner_cp = ch, cp
    st, ndt, cell = pyoracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1] * 3, 0.4 * dt0)
    assert st == 0
    return {"u0": U0, "u1": U[:, 4:-4, 4:-4, 4:-4].copy(),
            "dt": np.array([0.4 * dt0, ndt, ch, cp]), "cell": np.array(cell)}


def charge_exchange():
    p = mfgpu.helio_params(16)
    nc = mfgpu.num_cons(p)
    rng = np.random.default_rng(5)
    w = random_states(rng, nc, True, 32)
    reg = rng.integers(1, 5, 32)
    s = np.array([pyoracle.charge_exchange(p, w[q], int(reg[q]), 0.01) for q in range(32)])
    return {"w": w, "reg": reg, "s": s}


def main():
    np.savez_compressed(os.path.join(HERE, "face_fluxes.npz"), **face_fluxes())
    np.savez_compressed(os.path.join(HERE, "orszag16_rk2.npz"), **orszag_step())
    np.savez_compressed(os.path.join(HERE, "helio12_rk2.npz"), **helio_step())
    np.savez_compressed(os.path.join(HERE, "charge_exchange.npz"), **charge_exchange())


if __name__ == "__main__":
    main()
