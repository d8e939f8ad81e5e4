"""Tracking surfaces (level sets) and the region tracer.

The reference carries num_tracking_surfaces extra components after the fluids
(EqSysMHDMF, srcIdeal/EqSysMHDMF.cpp:11-48), advected by the plasma velocity:
face values with limiter_LS, the upwind face value of LEVELSETFLUX
(src/LevelSetF.ChF:37-105), the non-conservative UPDATELEVELSET (:200-234;
Hancock: FLUXESHANCOCK_LS :9-35, UPDATELEVELSETHANCOCK :354-388) and the floor
of POSTPROCESSING_LS (:426-465).  With region_tracer the last surface selects
the charge-exchange regions (DEFINE_REGIONS_TRACER_4F, swlism/SWLISMF.ChF:
839-1016).

CPU: known answers of the oracle (a linear surface in a uniform flow moves by
exactly -dt (u . grad phi) in every time scheme and limiter; the floor holds
a +-1 step at -1 while overshoots above +1 stay, as the reference's routine
assigns the upper clip and then overwrites it; the region classification of
chosen states).  GPU: the CUDA path against the oracle on identical inputs at
the per-step tolerance of the FP64 path (single patch, the batched level with
the heliosphere's region tracer, the coupled hierarchy), and the fast and
mixed modes within theirs.
"""
import numpy as np
import pytest

import mfgpu
from mfgpu import amr
from helpers import periodic_fill, rel_err, to_device, to_host, valid_view

RTOL = 1e-12
TAS = [mfgpu.TA_RK2, mfgpu.TA_HANCOCK, mfgpu.TA_FIRST_ORDER]


def _uniform_patch(p, n, u, v, phi):
    """2D fab on [0,n-1]^2 + ghosts: uniform plasma moving with (u, v), the
    surface phi(x, y) at cell centres."""
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    U = np.zeros(mfgpu.fab_shape(lo, hi, mfgpu.num_cons(p)))
    j, i = np.meshgrid(np.arange(lo[1], hi[1] + 1), np.arange(lo[0], hi[0] + 1), indexing="ij")
    x, y = (i + 0.5) * p.dx, (j + 0.5) * p.dx
    rho, pr, B = 1.0, 1.0, (0.2, 0.1, 0.0)
    U[0] = rho
    U[1], U[2] = rho * u, rho * v
    U[5], U[6], U[7] = B
    U[4] = pr / (p.gamma - 1) + 0.5 * rho * (u * u + v * v) + (B[0] ** 2 + B[1] ** 2) / (8 * np.pi)
    U[8] = phi(x, y)[None]
    return U, lo, hi, ng


def _base(ta, n, lim, periodic):
    p = mfgpu._base_params(2, 1)
    p.time_approximation = ta
    p.dx = 1.0 / n
    for d in range(2):
        p.periodic[d] = 1 if periodic else 0
        p.domain_hi[d] = n - 1
    p.num_tracking_surfaces = 1
    p.limiter_ls = lim
    return p


# ---------------------------------------------------------------------------
# CPU: the oracle
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("ta", TAS)
@pytest.mark.parametrize("lim", [mfgpu.LIM_MINMOD, mfgpu.LIM_MC, mfgpu.LIM_VANLEER,
                                 mfgpu.LIM_SUPERBEE])
@pytest.mark.parametrize("uv", [(0.8, 0.3), (-0.6, -0.5)])
def test_linear_surface_moves_by_dt_u_grad(oracle, ta, lim, uv):
    """phi = a + b x + c y in a uniform flow: every limiter reproduces the
    linear face values, the upwind face is the left one for u > 0 and the
    right one for u < 0, and the update is phi - dt (u b + v c).  The fluid
    state does not change.  Cells within 4 of the (non-periodic) domain
    boundary see the unadvanced ghost values in the later stages and are
    left out."""
    n = 32
    p = _base(ta, n, lim, periodic=False)
    a, b, c = 5.0, 0.7, -0.4
    U, lo, hi, ng = _uniform_patch(p, n, uv[0], uv[1], lambda x, y: a + b * x + c * y)
    dt = 0.2 * p.dx
    Uo = U.copy()
    st, _, _ = oracle.patch_update(p, Uo, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)
    assert st == 0
    h = ng + 4
    expect = U[8] - dt * (uv[0] * b + uv[1] * c)
    assert np.max(np.abs(Uo[8][:, h:-h, h:-h] - expect[:, h:-h, h:-h])) <= 4e-15 * a
    assert np.array_equal(valid_view(Uo[:8], ng, 2), valid_view(U[:8], ng, 2))


def _step_surface(p, n, ng):
    U, lo, hi, _ = _uniform_patch(p, n, 1.0, 0.0,
                                  lambda x, y: np.where((x % 1.0 > 0.25) & (x % 1.0 < 0.6),
                                                        -1.0, 1.0))
    return periodic_fill(U, ng, 2), lo, hi


def test_floor_holds_the_lower_extreme_only(oracle):
    """A +-1 step advected at CFL 0.9, first order, minmod: the update
    overshoots on both sides (it is symmetric under phi -> -phi); the floor
    min(Umin, -|Umax|) of the stage-start neighbourhood brings every
    undershoot back to -1, and the overshoots above +1 stay (the reference
    assigns min(LS, Umax) and then max(LS, Umin) from the same LS)."""
    n = 32
    p = _base(mfgpu.TA_FIRST_ORDER, n, mfgpu.LIM_MINMOD, periodic=True)
    ng = mfgpu.num_ghost(p)
    U, lo, hi = _step_surface(p, n, ng)
    dt = 0.9 * p.dx
    for _ in range(6):
        assert oracle.patch_update(p, U, lo, hi, [0, 0, 0], [n - 1, n - 1, 0], dt)[0] == 0
        U = periodic_fill(U, ng, 2)
    v = valid_view(U, ng, 2)[8]
    assert v.min() == -1.0
    assert v.max() > 1.2


def _tracer_params():
    p = mfgpu.helio_params(32, region_tracer=True)
    p.region_zbot, p.region_ztop = -0.5, 0.5
    return p


def _w(p, rho=0.1, u=(-1.0, 0.0, 0.0), pr=0.05, tracer=1.0):
    w = np.zeros(mfgpu.num_cons(p))
    w[0], w[1:4], w[4] = rho, u, pr
    w[5:8] = (0.02, 0.03, 0.0)
    for s in range(9, 24, 5):
        w[s], w[s + 1], w[s + 4] = 0.05, -1.0, 0.025
    w[-1] = tracer
    return w


def test_region_tracer_classification(oracle):
    """DEFINE_REGIONS_TRACER_4F on chosen cells (sun at (1,1,1), dx 1/16,
    LIMSUN = 6, T = 1e4 p/rho).  Interstellar (tracer >= 0): 1, or 4 when
    rho > 1.2, |u| < 0.8, cos(u, lism) < 0.95 or T > 9000.  Solar wind
    (tracer < 0): 3 for a fast radial wind, 2 for a slow one or a fast hot
    one outside sunR, 4 outside the z band."""
    p = _tracer_params()
    i, j, k = 24, 16, 16            # x = 0.53125 from the sun along +x, y = z = 0.03125
    reg = lambda w, ijk=(i, j, k): oracle.region(p, *ijk, w)
    assert reg(_w(p)) == 1
    assert reg(_w(p, tracer=0.0)) == 1
    assert reg(_w(p, rho=1.3)) == 4
    assert reg(_w(p, u=(-0.5, 0.0, 0.0))) == 4
    assert reg(_w(p, u=(-0.866, 0.5, 0.0))) == 4
    assert reg(_w(p, pr=0.1)) == 4               # T = 1e4 * 0.1 / 0.1 = 1e4 > 9000
    fast = (10.0, 0.0, 0.0)
    assert reg(_w(p, rho=1.0, u=fast, pr=1.0, tracer=-1.0)) == 3
    assert reg(_w(p, rho=1.0, u=fast, pr=200.0, tracer=-1.0)) == 2     # T = 2e6
    assert reg(_w(p, rho=1.0, u=(1.0, 0.0, 0.0), pr=1.0, tracer=-1.0)) == 2
    assert reg(_w(p, rho=1.0, u=fast, pr=1.0, tracer=-1.0), (i, j, 30)) == 4   # z = 0.90625
    # without the tracer the same states follow DEFINE_REGIONS_2F
    q = mfgpu.helio_params(32)
    assert oracle.region(q, i, j, k, _w(p, rho=1.3)[:-1]) == 1


def test_tracer_params_validation(gpulib):
    p = mfgpu.helio_params(16)
    p.region_tracer = 1
    with pytest.raises(mfgpu.MfError):          # no surface to hold the tracer
        mfgpu.Context(p)
    p = mfgpu.helio_params(16)
    p.num_tracking_surfaces = 3
    with pytest.raises(mfgpu.MfError):
        mfgpu.Context(p)
    p = mfgpu.helio_params(16, region_tracer=True)
    ctx = mfgpu.Context(p)
    assert ctx.nc == 25
    ctx.close()


# ---------------------------------------------------------------------------
# GPU: the CUDA path against the oracle
# ---------------------------------------------------------------------------
def _gpu_patch(ctx, U, lo, hi, vlo, vhi, dt):
    t = to_device(U)
    st, ndt, _ = ctx.patch_update(t.data_ptr(), lo, hi, vlo, vhi, dt)
    assert st == 0
    return to_host(t), ndt


def _orszag_surface(n, ta, lim, prec=mfgpu.PREC_FP64, **kw):
    p = mfgpu.orszag_params(n, ta, prec)
    p.num_tracking_surfaces = 1
    p.limiter_ls = lim
    for k, v in kw.items():
        setattr(p, k, v)
    ng = mfgpu.num_ghost(p)
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    U = mfgpu.init_host_fab(p, lo, hi, "orszag")
    j, i = np.meshgrid(np.arange(lo[1], hi[1] + 1), np.arange(lo[0], hi[0] + 1), indexing="ij")
    x, y = (i + 0.5) * p.dx, (j + 0.5) * p.dx
    U[8] = (np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y) + 0.2)[None]
    return p, periodic_fill(U, ng, 2), lo, hi, ng


@pytest.mark.gpu
@pytest.mark.parametrize("ta", TAS)
def test_gpu_orszag_surface_vs_oracle(gpulib, oracle, ta):
    n = 48
    p, U, lo, hi, ng = _orszag_surface(n, ta, mfgpu.LIM_MC)
    ctx = mfgpu.Context(p)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    for step in range(3):
        Uo = U.copy()
        st, ndt_o, _ = oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt)
        assert st == 0
        Ug, ndt_g = _gpu_patch(ctx, U, lo, hi, vlo, vhi, dt)
        e = rel_err(valid_view(Ug, ng, 2), valid_view(Uo, ng, 2), nls=1)
        assert np.all(e <= RTOL), (step, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        U = periodic_fill(Uo.copy(), ng, 2)
        dt = 0.4 * ndt_o
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("lim", [mfgpu.LIM_CD, mfgpu.LIM_SUPERBEE, mfgpu.LIM_VANALBADA,
                                 mfgpu.LIM_HARMONIC, mfgpu.LIM_VANLEER, mfgpu.LIM_HYPERBEE,
                                 mfgpu.LIM_VENKATAKRISHNAN, mfgpu.LIM_WENO3])
@pytest.mark.parametrize("char", [0, 1])
@pytest.mark.parametrize("ta", [mfgpu.TA_RK2, mfgpu.TA_HANCOCK])
def test_gpu_surface_limiters(gpulib, oracle, lim, char, ta):
    """Every limiter_LS, with plain and with characteristic reconstruction
    (where the surfaces take the *FACESLOPES form), and the positivity
    fallback on; RK2 and Hancock (face values of the predictor)."""
    n = 32
    p, U, lo, hi, ng = _orszag_surface(n, ta, lim, char_reconstruction=char,
                                       check_positivity=1)
    ctx = mfgpu.Context(p)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    dt = 0.4 * oracle.compute_dt(p, U, lo, hi, vlo, vhi)[1]
    Uo = U.copy()
    assert oracle.patch_update(p, Uo, lo, hi, vlo, vhi, dt)[0] == 0
    Ug, _ = _gpu_patch(ctx, U, lo, hi, vlo, vhi, dt)
    e = rel_err(valid_view(Ug, ng, 2), valid_view(Uo, ng, 2), nls=1)
    assert np.all(e <= RTOL), e
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ta", TAS)
def test_gpu_step_floor_vs_oracle(gpulib, oracle, ta):
    """The +-1 step at CFL 0.9: the floor (and the upwind selection at the
    step) on the device equal the oracle's, bitwise on the surface."""
    n = 32
    p = _base(ta, n, mfgpu.LIM_MINMOD, periodic=True)
    ctx = mfgpu.Context(p)
    ng = ctx.ng
    U, lo, hi = _step_surface(p, n, ng)
    vlo, vhi = [0, 0, 0], [n - 1, n - 1, 0]
    for _ in range(4):
        Uo = U.copy()
        assert oracle.patch_update(p, Uo, lo, hi, vlo, vhi, 0.9 * p.dx)[0] == 0
        Ug, _ = _gpu_patch(ctx, U, lo, hi, vlo, vhi, 0.9 * p.dx)
        assert np.array_equal(valid_view(Ug, ng, 2)[8], valid_view(Uo, ng, 2)[8])
        U = periodic_fill(Uo.copy(), ng, 2)
    ctx.close()


def _helio_level(p, n, arrays_from=None):
    boxes = mfgpu.tile_boxes(n, 16, 3)
    ng = mfgpu.num_ghost(p)
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = mfgpu.grow(lo, hi, ng, 3)
        arrays.append(np.ascontiguousarray(mfgpu.init_host_fab(p, flo, fhi, "helio")))
        fboxes.append((flo, fhi))
    return boxes, arrays, fboxes


def _device_level(p, boxes, arrays):
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
@pytest.mark.parametrize("ta,hbc", [(mfgpu.TA_RK2, 0), (mfgpu.TA_HANCOCK, 0),
                                    (mfgpu.TA_FIRST_ORDER, 0), (mfgpu.TA_RK2, 1)])
def test_gpu_helio_region_tracer_level_vs_oracle(gpulib, oracle, ta, hbc):
    """32^3 heliosphere with the region tracer (8 patches, far-field ghosts
    holding +1), also with the heliosphere boundary fluxes: two level steps,
    each from the oracle's state."""
    n = 32
    p = mfgpu.helio_params(n, time_approximation=ta, region_tracer=True)
    p.helio_bc = hbc
    boxes, arrays, fboxes = _helio_level(p, n)
    ctx, lev, flat, dt0 = _device_level(p, boxes, arrays)
    ng = ctx.ng
    dt = 0.4 * dt0
    for step in range(2):
        st, ndt_o, _, _ = oracle.level_step(p, arrays, fboxes, boxes, dt)
        assert st == 0
        st, ndt_g, _, _ = lev.step(dt)
        assert st == 0
        out = np.zeros(lev.ndoubles)
        lev.download(out.ctypes.data)
        for i in range(len(boxes)):
            e = rel_err(valid_view(lev.patch_view(out, i), ng, 3), valid_view(arrays[i], ng, 3),
                        nls=1)
            assert np.all(e <= RTOL), (step, i, e)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        for i in range(len(boxes)):
            lev.patch_view(flat, i)[:] = arrays[i]
        lev.upload(flat.ctypes.data)
        dt = 0.4 * ndt_o
    # the tracer separates the wind from the interstellar gas
    tr = np.concatenate([valid_view(a, ng, 3)[-1].ravel() for a in arrays])
    assert tr.min() < 0.0 < tr.max()
    lev.close()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(mfgpu.PREC_FP64_FAST, 1e-7), (mfgpu.PREC_MIXED, 1e-5)])
def test_gpu_helio_region_tracer_fast_and_mixed(gpulib, oracle, prec, tol):
    """64^3, 3 steps with the region tracer: fast FP64 pointwise within tol
    of the oracle (psi against the field's scale), mixed within tol in the
    L1 norm of the density and of the tracer."""
    n = 64
    p = mfgpu.helio_params(n, precision=prec, region_tracer=True)
    p64 = mfgpu.helio_params(n, region_tracer=True)
    boxes, arrays, fboxes = _helio_level(p64, n)
    ctx, lev, flat, dt0 = _device_level(p, boxes, arrays)
    p64.dedner_ch, p64.dedner_cp = p.dedner_ch, p.dedner_cp
    ng = ctx.ng
    dt = 0.4 * dt0
    for _ in range(3):
        assert lev.step(dt)[0] == 0
        st, ndt, _, _ = oracle.level_step(p64, arrays, fboxes, boxes, dt)
        assert st == 0
        dt = 0.4 * ndt
    out = np.zeros(lev.ndoubles)
    lev.download(out.ctypes.data)
    num = np.zeros(2)
    den = np.zeros(2)
    for i in range(len(boxes)):
        g = valid_view(lev.patch_view(out, i), ng, 3)
        o = valid_view(arrays[i], ng, 3)
        if prec == mfgpu.PREC_FP64_FAST:
            e = rel_err(g, o, nls=1)
            assert np.all(np.delete(e, 8) <= tol), (i, e)
            assert np.max(np.abs(g[8] - o[8])) <= tol * np.max(np.abs(o[5:8])), i
        for m, q in enumerate((0, -1)):
            num[m] += np.abs(g[q] - o[q]).sum()
            den[m] += np.abs(o[q]).sum()
    if prec == mfgpu.PREC_MIXED:
        assert np.all(num / den <= tol), num / den
    lev.close()
    ctx.close()


# Orszag-Tang 3D hierarchy (base 16^3, levels of ratio 2) with one surface
B0 = mfgpu.tile_boxes(16, 8, 3)
B1 = [((8, 8, 8), (15, 23, 23)), ((16, 8, 8), (23, 23, 23)), ((0, 0, 24), (7, 7, 31))]
B2 = [((22, 22, 22), (29, 29, 37)), ((30, 22, 22), (41, 29, 29))]


def _hier_levels(ta):
    p0 = amr.orszag3d_params(16, ta)
    p0.num_tracking_surfaces = 1
    p0.limiter_ls = mfgpu.LIM_MC
    return [p0, amr.level_params(p0, 2), amr.level_params(p0, 4)], [B0, B1, B2], [2, 2]


def _hier_init(p, lo, hi):
    U = amr.orszag3d_state(p, lo, hi)
    ax = [(np.arange(lo[d], hi[d] + 1) + 0.5) * p.dx for d in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    U[-1] = np.sin(2 * np.pi * X) * np.cos(2 * np.pi * (Y + Z)) + 0.1
    return U


@pytest.mark.gpu
@pytest.mark.parametrize("ta", [mfgpu.TA_RK2, mfgpu.TA_HANCOCK])
def test_gpu_hierarchy_with_surface_vs_oracle(gpulib, oracle, ta):
    """Coupled three-level hierarchy: the surface is interpolated into the
    fine ghosts and averaged down like every state, and left out of the flux
    registers (consInterval only)."""
    params, boxes, ratios = _hier_levels(ta)
    ng = mfgpu.num_ghost(params[0])
    dh = amr.DeviceHierarchy(mfgpu, params, boxes, ratios, _hier_init)
    L = []
    for p, b in zip(params, boxes):
        arrays, fboxes = [], []
        for lo, hi in b:
            flo, fhi = mfgpu.grow(lo, hi, ng, 3)
            arrays.append(np.ascontiguousarray(_hier_init(p, flo, fhi)))
            fboxes.append((flo, fhi))
        L.append((p, arrays, fboxes, b))
    for lv in range(len(L) - 2, -1, -1):
        pc, ac, fbc, bc = L[lv]
        pf, af, fbf, bf = L[lv + 1]
        assert oracle.average_down(pc, pf, ratios[lv], ac, fbc, bc, af, fbf, bf) == 0
    times = [0.0] * 3
    dt = 0.4 * dh.compute_dt()
    for step in range(2):
        dh.step(dt)
        st, ndt_o, _ = oracle.hier_step(L, ratios, times, dt)
        assert st == 0
        R = 1
        for lv, (p, arrays, fboxes, vboxes) in enumerate(L):
            if lv > 0:
                R *= ratios[lv - 1]
            out = dh.download(lv)
            for i in range(len(vboxes)):
                g = dh.levels[lv].patch_view(out, i)[:, ng:-ng, ng:-ng, ng:-ng]
                o = arrays[i][:, ng:-ng, ng:-ng, ng:-ng]
                e = rel_err(g, o, nls=1)
                assert np.all(e <= RTOL * R), (step, lv, i, e)
        dt = 0.4 * ndt_o
    dh.close()
