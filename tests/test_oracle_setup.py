"""The oracle's own problem set-up, which the CPU legs of the benchmark use so
that they load nothing of the product library: its struct layouts, its
heliosphere workload preset and its heliosphere initial state equal the
product's (bitwise), so both sides start every comparison and every timing
from the same state."""
import ctypes

import numpy as np
import pytest

import mfgpu


def _layout(cls):
    return [(name, getattr(cls, name).offset, getattr(cls, name).size)
            for name, _ in cls._fields_]


def test_struct_layouts_match(oracle):
    for a, b in ((oracle.MfParams, mfgpu.MfParams), (oracle.MfFab, mfgpu.MfFab),
                 (oracle.MfBox, mfgpu.MfBox)):
        assert _layout(a) == _layout(b)
        assert ctypes.sizeof(a) == ctypes.sizeof(b)


@pytest.mark.parametrize("n", [32, 128])
def test_workload_preset_matches(oracle, n):
    a = oracle.helio_params(n)
    b = mfgpu.helio_params(n)
    assert bytes(a) == bytes(b)


def _variants():
    out = []
    for name in ("default", "tracer", "surface", "tilt", "monopolar", "first_order"):
        p = mfgpu.helio_params(32, region_tracer=(name == "tracer"),
                               time_approximation=(mfgpu.TA_FIRST_ORDER
                                                   if name == "first_order" else mfgpu.TA_RK2))
        if name == "surface":
            p.num_tracking_surfaces = 1
        if name == "tilt":
            p.sun_tilt = 30.0
            p.num_tracking_surfaces = 2
            p.region_tracer = 1
        if name == "monopolar":
            p.sun_b_monopolar = 1
        out.append((name, p))
    return out


@pytest.mark.parametrize("name,p", _variants(), ids=[v[0] for v in _variants()])
def test_oracle_helio_init_equals_product(gpulib, oracle, name, p):
    """mf_init_helio_host (host code of the product library) and the oracle's
    restatement agree bitwise on a fab that contains the inner sphere."""
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([12, 12, 12], [19, 19, 19], ng, 3)
    a = mfgpu.init_host_fab(p, lo, hi, "helio")
    b = oracle.helio_fab(p, lo, hi)
    assert np.array_equal(a, b)
    if p.reinit_sphere:
        assert np.any(a[0] > 0.5)  # the sphere's dense wind is in the fab
