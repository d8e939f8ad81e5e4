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

# Struct layouts of include/mf_patch.h, declared here so that the oracle and
# the CPU legs of the benchmark need nothing of the product package.  The
# entry points take any ctypes structure of the same layout (the product's
# binding declares the same structs; a test compares the two layouts).
c_int3 = ctypes.c_int * 3
c_double3 = ctypes.c_double * 3

TA_FIRST_ORDER, TA_HANCOCK, TA_RK2 = 0, 1, 2
PREC_FP64 = 0
BC_FARFIELD = 1
LIM_MINMOD = 1


class MfBox(ctypes.Structure):
    _fields_ = [("lo", c_int3), ("hi", c_int3)]


class MfFab(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("box", MfBox), ("ncomp", ctypes.c_int)]


class MfParams(ctypes.Structure):
    _fields_ = [
        ("space_dim", ctypes.c_int), ("n_fluids", ctypes.c_int),
        ("time_approximation", ctypes.c_int), ("flux", ctypes.c_int),
        ("divb_cleaning", ctypes.c_int), ("use_8wave", ctypes.c_int),
        ("divb_method", ctypes.c_int), ("limiter", ctypes.c_int * 8),
        ("check_positivity", ctypes.c_int), ("precision", ctypes.c_int),
        ("gamma", ctypes.c_double), ("smallr", ctypes.c_double), ("smallp", ctypes.c_double),
        ("entropy_fix", ctypes.c_double), ("small_b", ctypes.c_double), ("dx", ctypes.c_double),
        ("dedner_ch", ctypes.c_double), ("dedner_cp", ctypes.c_double),
        ("factor_ch", ctypes.c_double), ("factor_cp", ctypes.c_double),
        ("charge_exchange", ctypes.c_int), ("ce_scale_vel", ctypes.c_double),
        ("ce_sigma_scale", ctypes.c_double), ("ce_sigma_a", ctypes.c_double),
        ("ce_sigma_b", ctypes.c_double), ("ce_damp_c", ctypes.c_double),
        ("ce_damp_pow", ctypes.c_double), ("sun_center", c_double3), ("sun_r", ctypes.c_double),
        ("sun_v", ctypes.c_double), ("region_t_coeff", ctypes.c_double),
        ("region_tmlim", ctypes.c_double), ("region_zbot", ctypes.c_double),
        ("region_ztop", ctypes.c_double), ("reinit_sphere", ctypes.c_int),
        ("reinit_r0", ctypes.c_double), ("sun_int_bc_radius", ctypes.c_double),
        ("sun_rho", ctypes.c_double), ("sun_p", ctypes.c_double), ("sun_b", ctypes.c_double),
        ("sun_beta", ctypes.c_double), ("dir_br", ctypes.c_double), ("domain_lo", c_int3),
        ("domain_hi", c_int3), ("periodic", c_int3), ("bc_kind", ctypes.c_int),
        ("bc_plasma", ctypes.c_double * 8), ("bc_neutral1", ctypes.c_double * 5),
        ("char_reconstruction", ctypes.c_int), ("check_tvd", ctypes.c_int),
        ("helio_bc", ctypes.c_int), ("neutral_sun_bc", ctypes.c_int),
        ("num_tracking_surfaces", ctypes.c_int), ("limiter_ls", ctypes.c_int),
        ("region_tracer", ctypes.c_int), ("lism_u", ctypes.c_double * 3),
        ("max_dt_growth", ctypes.c_double), ("sun_b_monopolar", ctypes.c_int),
        ("sun_tilt", ctypes.c_double),
    ]


def make_box(lo, hi) -> MfBox:
    b = MfBox()
    for d in range(3):
        b.lo[d] = int(lo[d]) if d < len(lo) else 0
        b.hi[d] = int(hi[d]) if d < len(hi) else 0
    return b


def _pp(p):
    """A parameter struct of the layout of mf_params, by reference."""
    if ctypes.sizeof(p) != ctypes.sizeof(MfParams):
        raise TypeError("parameter struct does not have the layout of mf_params")
    return ctypes.byref(p)


def num_fluid_cons(p) -> int:
    """plasma, psi with GLM, 5 per neutral fluid (srcIdeal/EqSysMHDMF.cpp:11-48)"""
    return 8 + (1 if p.divb_cleaning == 5 else 0) + (p.n_fluids - 1) * 5


def num_cons(p) -> int:
    return num_fluid_cons(p) + p.num_tracking_surfaces


def num_ghost(p) -> int:
    """PatchMHDAM::numGhostCells (src/PatchMHDAM.cpp:280-286)"""
    return {TA_RK2: 4, TA_HANCOCK: 3}.get(p.time_approximation, 2)


def grow(lo, hi, n, sd):
    lo = list(lo) + [0] * (3 - len(lo))
    hi = list(hi) + [0] * (3 - len(hi))
    return ([lo[d] - n if d < sd else 0 for d in range(3)],
            [hi[d] + n if d < sd else 0 for d in range(3)])


def fab_shape(lo, hi, nc):
    return (nc, hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)


def tile_boxes(n, patch, space_dim):
    """Valid boxes of patch^d tiles covering 0..n-1 per direction (x fastest)."""
    boxes = []
    nz = n // patch if space_dim == 3 else 1
    for kb in range(nz):
        for jb in range(n // patch):
            for ib in range(n // patch):
                lo = [ib * patch, jb * patch, kb * patch if space_dim == 3 else 0]
                hi = [lo[0] + patch - 1, lo[1] + patch - 1,
                      lo[2] + patch - 1 if space_dim == 3 else 0]
                boxes.append((lo, hi))
    return boxes


_lib = None
_P = ctypes.POINTER
_DP = ctypes.POINTER(ctypes.c_double)
_PP = ctypes.c_void_p  # mf_params* (any struct of its layout)


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
        "mf_oracle_patch_update": (ctypes.c_int, [_PP, ctypes.c_double, _P(MfFab),
                                                  _P(MfBox), ctypes.c_double, ctypes.c_void_p,
                                                  ctypes.c_void_p, _DP, ctypes.c_int * 3]),
        "mf_oracle_patch_update_e": (ctypes.c_int, [_PP, ctypes.c_double, _P(MfFab),
                                                    _P(MfBox), ctypes.c_double, ctypes.c_void_p,
                                                    ctypes.c_void_p, ctypes.c_void_p, _DP,
                                                    ctypes.c_int * 3]),
        "mf_oracle_recalculate_b": (ctypes.c_int, [_PP, _P(MfFab), _P(MfFab),
                                                   ctypes.c_void_p, ctypes.c_double, _P(MfBox)]),
        "mf_oracle_compute_dt": (ctypes.c_int, [_PP, _P(MfFab), _P(MfBox), _DP,
                                                ctypes.c_int * 3]),
        "mf_oracle_level_exchange": (ctypes.c_int, [_PP, ctypes.c_int, _P(MfFab),
                                                    _P(MfBox)]),
        "mf_oracle_level_step": (ctypes.c_int, [_PP, ctypes.c_double, ctypes.c_int,
                                                _P(MfFab), _P(MfBox), ctypes.c_double,
                                                ctypes.c_int, _DP, _P(ctypes.c_int),
                                                ctypes.c_int * 3]),
        "mf_oracle_face_flux": (ctypes.c_int, [_PP, ctypes.c_int, _DP, _DP, _DP]),
        "mf_oracle_cons_to_prim": (ctypes.c_int, [_PP, _DP, _DP]),
        "mf_oracle_face_values": (ctypes.c_int, [ctypes.c_int, ctypes.c_double,
                                                 ctypes.c_double, ctypes.c_double, _DP, _DP]),
        "mf_oracle_face_slopes": (ctypes.c_int, [ctypes.c_int, _DP, _DP]),
        "mf_oracle_helio_bc_face": (ctypes.c_int, [_PP, ctypes.c_int, ctypes.c_int, _DP,
                                                   _DP, _DP, _DP]),
        "mf_oracle_charge_exchange": (ctypes.c_int, [_PP, _DP, ctypes.c_int,
                                                     ctypes.c_double, _DP]),
        "mf_oracle_region": (ctypes.c_int, [_PP, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, _DP]),
        "mf_oracle_init_orszag": (ctypes.c_int, [_PP, _P(MfFab), _P(MfBox)]),
        "mf_oracle_init_helio": (ctypes.c_int, [_PP, _DP, _DP, _P(MfFab), _P(MfBox)]),
        "mf_oracle_max_threads": (ctypes.c_int, []),
        "mf_oracle_hier_step": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, _P(ctypes.c_int),
                                               _DP, ctypes.c_double, ctypes.c_int, _DP, _DP]),
        "mf_oracle_cf_fill": (ctypes.c_int, [_PP, _PP, ctypes.c_int,
                                             ctypes.c_int, _P(MfFab), _P(MfFab), _P(MfBox),
                                             ctypes.c_int, _P(MfFab), _P(MfBox),
                                             ctypes.c_double]),
        "mf_oracle_average_down": (ctypes.c_int, [_PP, _PP, ctypes.c_int,
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
    return lib.mf_oracle_recalculate_b(_pp(p), ctypes.byref(fu), ctypes.byref(fo), ep,
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
    st = lib.mf_oracle_patch_update_e(_pp(p), time, ctypes.byref(fab),
                                      ctypes.byref(valid), dt, fptr, dptr, eptr,
                                      ctypes.byref(ndt), cell)
    return st, ndt.value, tuple(cell)


def compute_dt(p: MfParams, U: np.ndarray, fab_lo, fab_hi, lo, hi):
    lib = load()
    fab = MfFab(U.ctypes.data, make_box(fab_lo, fab_hi), U.shape[0])
    box = make_box(lo, hi)
    dt = ctypes.c_double()
    cell = (ctypes.c_int * 3)()
    st = lib.mf_oracle_compute_dt(_pp(p), ctypes.byref(fab), ctypes.byref(box),
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
    return lib.mf_oracle_level_exchange(_pp(p), len(arrays), fabs, vb)


def level_step(p: MfParams, arrays, fab_boxes, valid_boxes, dt, nthreads=0, time=0.0):
    """exchange + updateState on every patch (arrays modified in place)."""
    lib = load()
    fabs = _fab_array(arrays, fab_boxes)
    vb = (MfBox * len(valid_boxes))(*[make_box(lo, hi) for lo, hi in valid_boxes])
    ndt = ctypes.c_double()
    ip = ctypes.c_int()
    cell = (ctypes.c_int * 3)()
    st = lib.mf_oracle_level_step(_pp(p), time, len(arrays), fabs, vb, dt, nthreads,
                                  ctypes.byref(ndt), ctypes.byref(ip), cell)
    return st, ndt.value, ip.value, tuple(cell)


def face_flux(p: MfParams, direction: int, wl, wr):
    lib = load()
    nc = num_cons(p)
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    wr = np.ascontiguousarray(wr, dtype=np.float64)
    f = np.full(nc, np.nan)
    st = lib.mf_oracle_face_flux(_pp(p), direction, _dp(wl), _dp(wr), _dp(f))
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
    w = np.full(num_cons(p), np.nan)
    st = lib.mf_oracle_cons_to_prim(_pp(p), _dp(u), _dp(w))
    assert st == 0, st
    return w


def charge_exchange(p: MfParams, w, reg, dt):
    lib = load()
    w = np.ascontiguousarray(w, dtype=np.float64)
    s = np.full(num_cons(p), np.nan)
    st = lib.mf_oracle_charge_exchange(_pp(p), _dp(w), reg, dt, _dp(s))
    assert st == 0, st
    return s


def region(p: MfParams, i, j, k, w):
    lib = load()
    w = np.ascontiguousarray(w, dtype=np.float64)
    return lib.mf_oracle_region(_pp(p), i, j, k, _dp(w))


def init_orszag(p: MfParams, U: np.ndarray, fab_lo, fab_hi, lo, hi):
    lib = load()
    fab = MfFab(U.ctypes.data, make_box(fab_lo, fab_hi), U.shape[0])
    box = make_box(lo, hi)
    return lib.mf_oracle_init_orszag(_pp(p), ctypes.byref(fab), ctypes.byref(box))


def init_helio(p, U: np.ndarray, fab_lo, fab_hi, lo, hi, wp=None, wn=None):
    """The synthetic heliosphere's initial state on [lo, hi] of the host fab U
    (in place): the uniform inflow (helio_inflow() unless given), the
    tracking surfaces, the inner sphere at time 0."""
    lib = load()
    if wp is None:
        wp, wn = helio_inflow()
    wp = np.ascontiguousarray(wp, dtype=np.float64)
    wn = np.ascontiguousarray(wn if wn is not None else np.zeros(5), dtype=np.float64)
    if p.n_fluids > 1:
        wn = np.ascontiguousarray(wn[:5 * (p.n_fluids - 1)])
    fab = MfFab(U.ctypes.data, make_box(fab_lo, fab_hi), U.shape[0])
    box = make_box(lo, hi)
    return lib.mf_oracle_init_helio(_pp(p), _dp(wp), _dp(wn), ctypes.byref(fab),
                                    ctypes.byref(box))


def helio_fab(p, lo, hi) -> np.ndarray:
    """A host fab on [lo, hi] holding the heliosphere's initial state."""
    U = np.zeros(fab_shape(lo, hi, num_cons(p)))
    st = init_helio(p, U, lo, hi, lo, hi)
    assert st == 0, st
    return U


HELIO_T_INFLOW = 0.5


def helio_inflow():
    """Inflow primitive states of the synthetic heliosphere: plasma rho 0.1,
    v = (-1,0,0), p = rho T (T = 0.5), |B| = 0.05 at 60 degrees to the flow in
    the x-y plane; neutral fluids rho 0.1 / 0.05 / 0.05, same velocity and
    temperature."""
    T = HELIO_T_INFLOW
    b = 0.05
    ang = np.deg2rad(60.0)
    wp = np.array([0.1, -1.0, 0.0, 0.0, 0.1 * T, -b * np.cos(ang), b * np.sin(ang), 0.0],
                  dtype=np.float64)
    rhos = [0.1, 0.05, 0.05]
    wn = np.concatenate([[r, -1.0, 0.0, 0.0, r * T] for r in rhos]).astype(np.float64)
    return wp, wn


def helio_params(n: int = 128, seed: int = 20240601) -> MfParams:
    """The 3D multi-fluid heliosphere workload on [-1,1]^3 with n^3 cells,
    FP64, RK2: plasma MHD + 3 neutral H fluids, GLM cleaning (factor_ch 0.5),
    charge exchange with sigma(v) = 0.1 (a - b ln v)^2, (a, b) uniform in
    [1.5, 2.5] x [0.05, 0.15] from the seed, regions after
    DEFINE_REGIONS_2F, the inner solar-wind sphere of radius 0.1 (bipolar
    field, flat current sheet), far-field boundaries holding the inflow,
    the neutral pass-through at the sun, assignDt's growth cap 1.1."""
    p = MfParams()
    p.space_dim, p.n_fluids = 3, 4
    p.time_approximation = TA_RK2
    p.flux = 1
    p.divb_cleaning = 5
    p.use_8wave = 0
    p.divb_method = 1
    for v in range(8):
        p.limiter[v] = LIM_MINMOD
    p.precision = PREC_FP64
    p.gamma = 5.0 / 3.0
    p.smallr, p.smallp = 1e-8, 1e-10
    p.entropy_fix, p.small_b = 0.3, 1e-9
    p.dx = 2.0 / n
    p.factor_ch, p.factor_cp = 0.5, 1.0
    rng = np.random.default_rng(seed)
    p.charge_exchange = 1
    p.ce_scale_vel = 1.0
    p.ce_sigma_scale = 0.1
    p.ce_sigma_a = float(rng.uniform(1.5, 2.5))
    p.ce_sigma_b = float(rng.uniform(0.05, 0.15))
    p.ce_damp_c, p.ce_damp_pow = 0.0, 4.5
    for d in range(3):
        p.sun_center[d] = 1.0
        p.domain_lo[d], p.domain_hi[d], p.periodic[d] = 0, n - 1, 0
    p.sun_r, p.sun_v = 0.1, 10.0
    p.region_t_coeff, p.region_tmlim = 1.0e4, 1.0e5
    p.region_zbot, p.region_ztop = -1e300, 1e300
    p.reinit_sphere, p.reinit_r0, p.sun_int_bc_radius = 1, 0.1, 0.1
    p.sun_rho, p.sun_p, p.sun_b, p.sun_beta, p.dir_br = 1.0, 1.0, 0.1, 2.0, 1.0
    p.bc_kind = BC_FARFIELD
    p.helio_bc = 0
    p.neutral_sun_bc = 1
    wp, wn = helio_inflow()
    for q in range(8):
        p.bc_plasma[q] = wp[q]
    for q in range(5):
        p.bc_neutral1[q] = wn[q]
    p.dedner_ch = 10.0
    p.dedner_cp = float(np.sqrt(10.0 * p.dx))
    p.limiter_ls = LIM_MINMOD
    p.lism_u[0] = -1.0
    p.max_dt_growth = 1.1
    p.sun_b_monopolar = 0
    p.sun_tilt = 0.0
    return p


def max_threads() -> int:
    return load().mf_oracle_max_threads()


class _Level(ctypes.Structure):
    _fields_ = [("p", _PP), ("npatch", ctypes.c_int), ("U", _P(MfFab)),
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
        _pp(p)  # layout check
        arr[lev] = _Level(ctypes.addressof(p), len(arrays), fabs, vb)
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
    return lib.mf_oracle_cf_fill(_pp(pc), _pp(pf), ratio, len(coarse_new), fo,
                                 fn, _boxes(coarse_valid), len(fine_arrays), ff,
                                 _boxes(fine_valid), alpha)


def average_down(pc, pf, ratio, coarse, coarse_fboxes, coarse_valid, fine_arrays, fine_fboxes,
                 fine_valid):
    """Average the fine level onto the coarse cells it covers (in place)."""
    lib = load()
    fc = _fab_array(coarse, coarse_fboxes)
    ff = _fab_array(fine_arrays, fine_fboxes)
    return lib.mf_oracle_average_down(_pp(pc), _pp(pf), ratio, len(coarse), fc,
                                      _boxes(coarse_valid), len(fine_arrays), ff,
                                      _boxes(fine_valid))


def helio_bc_face(p: MfParams, direction: int, side: int, wl, wr):
    """Fluxes and face-normal B of a face on the domain boundary with HELIOBC."""
    lib = load()
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    wr = np.ascontiguousarray(wr, dtype=np.float64)
    f = np.full(num_cons(p), np.nan)
    bn = ctypes.c_double()
    st = lib.mf_oracle_helio_bc_face(_pp(p), direction, side, _dp(wl), _dp(wr), _dp(f),
                                     ctypes.byref(bn))
    assert st == 0, st
    return f, bn.value
