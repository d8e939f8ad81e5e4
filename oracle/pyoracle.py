"""ctypes binding of the CPU restatement (oracle/libmforacle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; the product never imports it.
Parity status: unpinned by reference outputs (see mf_oracle.c).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libmforacle.so")
_PKG = os.path.join(os.path.dirname(HERE), "ms-flukss-multifluid_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
import mfgpu  # noqa: E402  (struct layouts of include/mf_patch.h only)
from mfgpu import MfBox, MfFab, MfParams, make_box  # noqa: E402

_lib = None
_P = ctypes.POINTER
_DP = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("mf_oracle.c", "mf_oracle.h", "Makefile")]
    hdr = os.path.join(os.path.dirname(HERE), "include", "mf_patch.h")
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs + [hdr])):
        return LIB
    r = subprocess.run(["make", "-B" if force else "-s", "-C", HERE], capture_output=True,
                       text=True)
    if r.returncode != 0 or not os.path.exists(LIB):
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(LIB)
    sig = {
        "mf_oracle_patch_update": (ctypes.c_int, [_P(MfParams), ctypes.c_double, _P(MfFab),
                                                  _P(MfBox), ctypes.c_double, ctypes.c_void_p,
                                                  ctypes.c_void_p, _DP, ctypes.c_int * 3]),
        "mf_oracle_patch_update_e": (ctypes.c_int, [_P(MfParams), ctypes.c_double, _P(MfFab),
                                                    _P(MfBox), ctypes.c_double, ctypes.c_void_p,
                                                    ctypes.c_void_p, ctypes.c_void_p, _DP,
                                                    ctypes.c_int * 3]),
        "mf_oracle_recalculate_b": (ctypes.c_int, [_P(MfParams), _P(MfFab), _P(MfFab),
                                                   ctypes.c_void_p, ctypes.c_double, _P(MfBox)]),
        "mf_oracle_compute_dt": (ctypes.c_int, [_P(MfParams), _P(MfFab), _P(MfBox), _DP,
                                                ctypes.c_int * 3]),
        "mf_oracle_level_exchange": (ctypes.c_int, [_P(MfParams), ctypes.c_int, _P(MfFab),
                                                    _P(MfBox)]),
        "mf_oracle_level_step": (ctypes.c_int, [_P(MfParams), ctypes.c_double, ctypes.c_int,
                                                _P(MfFab), _P(MfBox), ctypes.c_double,
                                                ctypes.c_int, _DP, _P(ctypes.c_int),
                                                ctypes.c_int * 3]),
        "mf_oracle_face_flux": (ctypes.c_int, [_P(MfParams), ctypes.c_int, _DP, _DP, _DP]),
        "mf_oracle_cons_to_prim": (ctypes.c_int, [_P(MfParams), _DP, _DP]),
        "mf_oracle_face_values": (ctypes.c_int, [ctypes.c_int, ctypes.c_double,
                                                 ctypes.c_double, ctypes.c_double, _DP, _DP]),
        "mf_oracle_face_slopes": (ctypes.c_int, [ctypes.c_int, _DP, _DP]),
        "mf_oracle_helio_bc_face": (ctypes.c_int, [_P(MfParams), ctypes.c_int, ctypes.c_int, _DP,
                                                   _DP, _DP, _DP]),
        "mf_oracle_charge_exchange": (ctypes.c_int, [_P(MfParams), _DP, ctypes.c_int,
                                                     ctypes.c_double, _DP]),
        "mf_oracle_region": (ctypes.c_int, [_P(MfParams), ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, _DP]),
        "mf_oracle_init_orszag": (ctypes.c_int, [_P(MfParams), _P(MfFab), _P(MfBox)]),
        "mf_oracle_max_threads": (ctypes.c_int, []),
        "mf_oracle_hier_step": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, _P(ctypes.c_int),
                                               _DP, ctypes.c_double, ctypes.c_int, _DP, _DP]),
        "mf_oracle_cf_fill": (ctypes.c_int, [_P(MfParams), _P(MfParams), ctypes.c_int,
                                             ctypes.c_int, _P(MfFab), _P(MfFab), _P(MfBox),
                                             ctypes.c_int, _P(MfFab), _P(MfBox),
                                             ctypes.c_double]),
        "mf_oracle_average_down": (ctypes.c_int, [_P(MfParams), _P(MfParams), ctypes.c_int,
                                                  ctypes.c_int, _P(MfFab), _P(MfBox),
                                                  ctypes.c_int, _P(MfFab), _P(MfBox)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def _edge_fabs(E, keep):
    """E: list of (array, lo, hi), one per edge direction (1 in 2D)."""
    if E is None:
        return None
    arr = (MfFab * 3)()
    for d in range(3):
        a, lo, hi = E[min(d, len(E) - 1)]
        arr[d] = MfFab(a.ctypes.data, make_box(lo, hi), 1)
    keep.append(arr)
    return ctypes.cast(arr, ctypes.c_void_p)


def edge_boxes(lo, hi, sd):
    """Boxes of the EdgeBox on the cell box [lo, hi]: in 3D the nodal box made
    cell-centred along each direction, in 2D the nodal box."""
    nlo, nhi = list(lo), list(hi)
    for d in range(sd):
        nhi[d] += 1
    if sd == 2:
        return [(nlo, nhi)]
    out = []
    for d in range(3):
        h = list(nhi)
        h[d] -= 1
        out.append((list(nlo), h))
    return out


def recalculate_b(p: MfParams, U, Uold, fab_lo, fab_hi, E, dt, lo, hi):
    """PatchMHDMF::recalculateMagneticField on host fabs (U in place)."""
    lib = load()
    keep = []
    fu = MfFab(U.ctypes.data, make_box(fab_lo, fab_hi), U.shape[0])
    fo = MfFab(Uold.ctypes.data, make_box(fab_lo, fab_hi), Uold.shape[0])
    ep = _edge_fabs(E, keep)
    box = make_box(lo, hi)
    return lib.mf_oracle_recalculate_b(ctypes.byref(p), ctypes.byref(fu), ctypes.byref(fo), ep,
                                       dt, ctypes.byref(box))


def patch_update(p: MfParams, U: np.ndarray, fab_lo, fab_hi, valid_lo, valid_hi, dt,
                 F=None, divB=None, time=0.0, E=None):
    """updateState on a host fab (modified in place). F: list of
    (array, lo, hi) per direction; divB: (array, lo, hi); E: the edge field
    of constrained transport, list of (array, lo, hi) on edge_boxes(valid)."""
    lib = load()
    assert U.dtype == np.float64 and U.flags.c_contiguous
    nc = U.shape[0]
    fab = MfFab(U.ctypes.data, make_box(fab_lo, fab_hi), nc)
    valid = make_box(valid_lo, valid_hi)
    fptr = None
    keep = []
    if F is not None:
        arr = (MfFab * 3)()
        for d, (a, lo, hi) in enumerate(F):
            arr[d] = MfFab(a.ctypes.data, make_box(lo, hi), nc)
        keep.append(arr)
        fptr = ctypes.cast(arr, ctypes.c_void_p)
    dptr = None
    if divB is not None:
        a, lo, hi = divB
        dfab = MfFab(a.ctypes.data, make_box(lo, hi), 1)
        keep.append(dfab)
        dptr = ctypes.cast(ctypes.pointer(dfab), ctypes.c_void_p)
    ndt = ctypes.c_double()
    cell = (ctypes.c_int * 3)()
    eptr = _edge_fabs(E, keep)
    st = lib.mf_oracle_patch_update_e(ctypes.byref(p), time, ctypes.byref(fab),
                                      ctypes.byref(valid), dt, fptr, dptr, eptr,
                                      ctypes.byref(ndt), cell)
    return st, ndt.value, tuple(cell)


def compute_dt(p: MfParams, U: np.ndarray, fab_lo, fab_hi, lo, hi):
    lib = load()
    fab = MfFab(U.ctypes.data, make_box(fab_lo, fab_hi), U.shape[0])
    box = make_box(lo, hi)
    dt = ctypes.c_double()
    cell = (ctypes.c_int * 3)()
    st = lib.mf_oracle_compute_dt(ctypes.byref(p), ctypes.byref(fab), ctypes.byref(box),
                                  ctypes.byref(dt), cell)
    return st, dt.value, tuple(cell)


def _fab_array(arrays, fab_boxes):
    n = len(arrays)
    fabs = (MfFab * n)()
    for i, (a, (lo, hi)) in enumerate(zip(arrays, fab_boxes)):
        fabs[i] = MfFab(a.ctypes.data, make_box(lo, hi), a.shape[0])
    return fabs


def level_exchange(p: MfParams, arrays, fab_boxes, valid_boxes):
    lib = load()
    fabs = _fab_array(arrays, fab_boxes)
    vb = (MfBox * len(valid_boxes))(*[make_box(lo, hi) for lo, hi in valid_boxes])
    return lib.mf_oracle_level_exchange(ctypes.byref(p), len(arrays), fabs, vb)


def level_step(p: MfParams, arrays, fab_boxes, valid_boxes, dt, nthreads=0, time=0.0):
    """exchange + updateState on every patch (arrays modified in place)."""
    lib = load()
    fabs = _fab_array(arrays, fab_boxes)
    vb = (MfBox * len(valid_boxes))(*[make_box(lo, hi) for lo, hi in valid_boxes])
    ndt = ctypes.c_double()
    ip = ctypes.c_int()
    cell = (ctypes.c_int * 3)()
    st = lib.mf_oracle_level_step(ctypes.byref(p), time, len(arrays), fabs, vb, dt, nthreads,
                                  ctypes.byref(ndt), ctypes.byref(ip), cell)
    return st, ndt.value, ip.value, tuple(cell)


def face_flux(p: MfParams, direction: int, wl, wr):
    lib = load()
    nc = mfgpu.num_cons(p)
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    wr = np.ascontiguousarray(wr, dtype=np.float64)
    f = np.full(nc, np.nan)
    st = lib.mf_oracle_face_flux(ctypes.byref(p), direction, _dp(wl), _dp(wr), _dp(f))
    assert st == 0, st
    return f


def face_values(lim: int, wm1: float, wp: float, wp1: float):
    """(lo, hi): the limiter's values on the low and high face of the cell."""
    lo, hi = ctypes.c_double(), ctypes.c_double()
    st = load().mf_oracle_face_values(lim, wm1, wp, wp1, ctypes.byref(lo), ctypes.byref(hi))
    assert st == 0
    return lo.value, hi.value


def face_slopes(lim: int, sleft: float, sright: float):
    """(left, right) limited slopes from the left and right differences."""
    a, b = ctypes.c_double(sleft), ctypes.c_double(sright)
    st = load().mf_oracle_face_slopes(lim, ctypes.byref(a), ctypes.byref(b))
    assert st == 0
    return a.value, b.value


def cons_to_prim(p: MfParams, u):
    lib = load()
    u = np.ascontiguousarray(u, dtype=np.float64)
    w = np.full(mfgpu.num_cons(p), np.nan)
    st = lib.mf_oracle_cons_to_prim(ctypes.byref(p), _dp(u), _dp(w))
    assert st == 0, st
    return w


def charge_exchange(p: MfParams, w, reg, dt):
    lib = load()
    w = np.ascontiguousarray(w, dtype=np.float64)
    s = np.full(mfgpu.num_cons(p), np.nan)
    st = lib.mf_oracle_charge_exchange(ctypes.byref(p), _dp(w), reg, dt, _dp(s))
    assert st == 0, st
    return s


def region(p: MfParams, i, j, k, w):
    lib = load()
    w = np.ascontiguousarray(w, dtype=np.float64)
    return lib.mf_oracle_region(ctypes.byref(p), i, j, k, _dp(w))


def init_orszag(p: MfParams, U: np.ndarray, fab_lo, fab_hi, lo, hi):
    lib = load()
    fab = MfFab(U.ctypes.data, make_box(fab_lo, fab_hi), U.shape[0])
    box = make_box(lo, hi)
    return lib.mf_oracle_init_orszag(ctypes.byref(p), ctypes.byref(fab), ctypes.byref(box))


def max_threads() -> int:
    return load().mf_oracle_max_threads()


class _Level(ctypes.Structure):
    _fields_ = [("p", _P(MfParams)), ("npatch", ctypes.c_int), ("U", _P(MfFab)),
                ("valid", _P(MfBox))]


def _boxes(valid_boxes):
    return (MfBox * len(valid_boxes))(*[make_box(lo, hi) for lo, hi in valid_boxes])


def hier_step(levels, ratios, times, dt0, nthreads=0):
    """One step of the coarsest level of a subcycled hierarchy.  levels: list
    of (params, arrays, fab_boxes, valid_boxes) from coarse to fine (arrays
    modified in place); times: list of level times (updated in place).
    Returns (status, new_dt, (Ch, Cp))."""
    lib = load()
    n = len(levels)
    keep = []
    arr = (_Level * n)()
    for lev, (p, arrays, fboxes, vboxes) in enumerate(levels):
        fabs = _fab_array(arrays, fboxes)
        vb = _boxes(vboxes)
        keep += [fabs, vb]
        arr[lev] = _Level(ctypes.pointer(p), len(arrays), fabs, vb)
    rl = list(ratios)[:n - 1] or [1]
    rat = (ctypes.c_int * len(rl))(*rl)
    t = (ctypes.c_double * n)(*times)
    ndt = ctypes.c_double()
    ded = (ctypes.c_double * 2)()
    st = lib.mf_oracle_hier_step(n, ctypes.cast(arr, ctypes.c_void_p), rat, t, dt0, nthreads,
                                 ctypes.byref(ndt), ded)
    for lev in range(n):
        times[lev] = t[lev]
    return st, ndt.value, (ded[0], ded[1])


def cf_fill(pc, pf, ratio, coarse_old, coarse_new, coarse_fboxes, coarse_valid, fine_arrays,
            fine_fboxes, fine_valid, alpha):
    """Interpolate the fine ghost cells over uncovered coarse cells (in place)."""
    lib = load()
    fo = _fab_array(coarse_old, coarse_fboxes)
    fn = _fab_array(coarse_new, coarse_fboxes)
    ff = _fab_array(fine_arrays, fine_fboxes)
    return lib.mf_oracle_cf_fill(ctypes.byref(pc), ctypes.byref(pf), ratio, len(coarse_new), fo,
                                 fn, _boxes(coarse_valid), len(fine_arrays), ff,
                                 _boxes(fine_valid), alpha)


def average_down(pc, pf, ratio, coarse, coarse_fboxes, coarse_valid, fine_arrays, fine_fboxes,
                 fine_valid):
    """Average the fine level onto the coarse cells it covers (in place)."""
    lib = load()
    fc = _fab_array(coarse, coarse_fboxes)
    ff = _fab_array(fine_arrays, fine_fboxes)
    return lib.mf_oracle_average_down(ctypes.byref(pc), ctypes.byref(pf), ratio, len(coarse), fc,
                                      _boxes(coarse_valid), len(fine_arrays), ff,
                                      _boxes(fine_valid))


def helio_bc_face(p: MfParams, direction: int, side: int, wl, wr):
    """Fluxes and face-normal B of a face on the domain boundary with HELIOBC."""
    lib = load()
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    wr = np.ascontiguousarray(wr, dtype=np.float64)
    f = np.full(mfgpu.num_cons(p), np.nan)
    bn = ctypes.c_double()
    st = lib.mf_oracle_helio_bc_face(ctypes.byref(p), direction, side, _dp(wl), _dp(wr), _dp(f),
                                     ctypes.byref(bn))
    assert st == 0, st
    return f, bn.value
