"""The C ABI without a GPU: the library loads, exports every function the
public headers declare, the ctypes structs match the C layout, parameter
validation and the host-side problem set-up work.  No compute call here needs
a device."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import mfgpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mf_patch.h")


def _declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:mf_status|void|int|long long|const char\*)\s+(mf_\w+)\s*\(",
                       src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_function(gpulib):
    names = _declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(gpulib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", mfgpu.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (mf_\w+)", out))
    assert set(names) <= exported, set(names) - exported


def test_binding_covers_header():
    assert set(_declared_functions()) == set(mfgpu.header_symbols())


def test_params_layout_matches_c():
    """sizeof / offsetof of mf_params, mf_fab, mf_box as compiled by gcc."""
    fields = [f[0] for f in mfgpu.MfParams._fields_]
    prog = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"',
            "int main(void) {",
            'printf("%zu %zu %zu\\n", sizeof(mf_params), sizeof(mf_fab), sizeof(mf_box));']
    for f in fields:
        prog.append(f'printf("%zu\\n", offsetof(mf_params, {f}));')
    prog.append("return 0; }")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write("\n".join(prog))
        subprocess.run(["gcc", "-std=c99", c, "-o", exe], check=True)
        lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sizes = [int(x) for x in lines[:3]]
    assert sizes == [ctypes.sizeof(mfgpu.MfParams), ctypes.sizeof(mfgpu.MfFab),
                     ctypes.sizeof(mfgpu.MfBox)]
    offs = [int(x) for x in lines[3:]]
    assert offs == [getattr(mfgpu.MfParams, f).offset for f in fields]


def test_params_default_and_validation(gpulib):
    p = mfgpu.default_params(3, 4)
    assert p.flux == 1 and p.use_8wave == 1 and p.divb_method == 1
    assert list(p.limiter) == [mfgpu.LIM_MINMOD] * 8
    assert p.entropy_fix == pytest.approx(0.3) and p.small_b == pytest.approx(1e-9)
    assert gpulib.mf_params_num_cons(ctypes.byref(p)) == 23
    # context creation is host-only
    ctx = mfgpu.Context(mfgpu.helio_params(32))
    assert ctx.nc == 24 and ctx.ng == 4
    ctx.close()
    bad = [("space_dim", 4, mfgpu.MF_ERR_BAD_ARG), ("divb_method", 3, mfgpu.MF_ERR_BAD_ARG),
           ("time_approximation", 7, mfgpu.MF_ERR_UNSUPPORTED),
           ("precision", 9, mfgpu.MF_ERR_BAD_ARG)]
    for field, val, code in bad:
        q = mfgpu.orszag_params(16)
        setattr(q, field, val)
        h = ctypes.c_void_p()
        assert gpulib.mf_create(ctypes.byref(q), ctypes.byref(h)) == code, field
    q = mfgpu.helio_params(16)
    q.use_8wave = 1            # GLM with the 8-wave source (main/MHDAM.cpp:1042-1046)
    h = ctypes.c_void_p()
    assert gpulib.mf_create(ctypes.byref(q), ctypes.byref(h)) == mfgpu.MF_ERR_UNSUPPORTED
    q = mfgpu.helio_params(16)
    q.flux = 5                 # GLM with VFRoe (main/MHDAM.cpp:1045)
    assert gpulib.mf_create(ctypes.byref(q), ctypes.byref(h)) == mfgpu.MF_ERR_UNSUPPORTED
    for code in range(10):
        assert mfgpu.status_string(code) != "unknown status"


def test_orszag_setup_matches_restatement(gpulib, oracle):
    p = mfgpu.orszag_params(32)
    lo, hi = mfgpu.grow([0, 0, 0], [31, 31, 0], 4, 2)
    a = mfgpu.init_host_fab(p, lo, hi, "orszag")
    b = np.zeros_like(a)
    assert oracle.init_orszag(p, b, lo, hi, lo, hi) == 0
    assert np.array_equal(a, b)


def test_helio_setup(gpulib):
    n = 32
    p = mfgpu.helio_params(n)
    lo, hi = [0, 0, 0], [n - 1] * 3
    U = mfgpu.init_host_fab(p, lo, hi, "helio")
    wp, wn = mfgpu.helio_inflow()
    c = (np.arange(n) + 0.5) * p.dx - 1.0
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    r = np.sqrt(x * x + y * y + z * z)
    inside = r <= p.reinit_r0
    assert inside.any()
    assert np.allclose(U[0][~inside], wp[0])
    assert np.allclose(U[9][~inside], wn[0])
    rr = r[inside] / p.sun_int_bc_radius
    assert np.allclose(U[0][inside], p.sun_rho / rr ** 2)
    vr = (U[1] * x + U[2] * y + U[3] * z) / (U[0] * r)
    assert np.allclose(vr[inside], p.sun_v)
