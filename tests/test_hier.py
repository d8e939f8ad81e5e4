"""Coupled hierarchies (mf_hier_*): the subcycled time step of
AMR_MHDAM::timeStep (srcIdeal/AMR_MHDAM.cpp:1707-1880) with the coarse-fine
ghost interpolation of PiecewiseLinearFillPatchMHDAM
(srcIdeal/PiecewiseLinearFillPatchMHDAM.cpp), the flux-register reflux and the
average down of AMRLevelIdealMHD::postTimeStep
(srcIdeal/AMRLevelIdealMHD.cpp:1633-1646).

CPU: properties of the oracle's restatement (linear data is interpolated
exactly; averaging linear data gives the coarse cell-centre values; a
periodic hierarchy step conserves the composite mass to rounding) and the
proper nesting of the hierarchy builder.  GPU: the interpolation and the
averaging (bitwise) and whole hierarchy steps against the oracle at the
per-step tolerance (RK2, first order, Hancock; 8-wave Orszag-Tang and the GLM
heliosphere with its Ch/Cp update), and conservation of the composite mass.
"""
import numpy as np
import pytest

import mfgpu
from mfgpu import amr
from helpers import rel_err

RTOL = 1e-12

# Orszag-Tang 3D: base 16^3 (8 patches), level 1 (ratio 2) with a region
# crossing the periodic boundary, level 2 (ratio 2) properly nested in level 1.
B0 = mfgpu.tile_boxes(16, 8, 3)
B1 = [((8, 8, 8), (15, 23, 23)), ((16, 8, 8), (23, 23, 23)), ((0, 0, 24), (7, 7, 31))]
B2 = [((22, 22, 22), (29, 29, 37)), ((30, 22, 22), (41, 29, 29))]


def _orszag_levels(ta=mfgpu.TA_RK2, prec=mfgpu.PREC_FP64):
    p0 = amr.orszag3d_params(16, ta, prec)
    return [p0, amr.level_params(p0, 2), amr.level_params(p0, 4)], [B0, B1, B2], [2, 2]


def _empty(p, lo, hi, fill=0.0):
    return np.full((mfgpu.num_cons(p),) + tuple(h - l + 1 for l, h in zip(lo[::-1], hi[::-1])),
                   fill)


def _host_level(p, boxes, ng, init):
    arrays, fboxes = [], []
    for lo, hi in boxes:
        flo, fhi = mfgpu.grow(lo, hi, ng, 3)
        arrays.append(np.ascontiguousarray(init(p, flo, fhi)))
        fboxes.append((flo, fhi))
    return arrays, fboxes


def _oracle_hier(oracle, params, boxes, ratios, init):
    ng = mfgpu.num_ghost(params[0])
    L = []
    for p, b in zip(params, boxes):
        a, fb = _host_level(p, b, ng, init)
        L.append((p, a, fb, b))
    for lv in range(len(L) - 2, -1, -1):
        pc, ac, fbc, bc = L[lv]
        pf, af, fbf, bf = L[lv + 1]
        assert oracle.average_down(pc, pf, ratios[lv], ac, fbc, bc, af, fbf, bf) == 0
    return L


def _composite_mass(L, ng):
    p, a, fb, b = L[0]
    return sum(arr[0, ng:-ng, ng:-ng, ng:-ng].sum() for arr in a) * p.dx ** 3


def _orszag_init(p, lo, hi):
    return amr.orszag3d_state(p, lo, hi)


def _linear_init(p, lo, hi):
    nc = mfgpu.num_cons(p)
    ax = [(np.arange(lo[d], hi[d] + 1) + 0.5) * p.dx for d in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    U = np.zeros((nc,) + X.shape)
    for q in range(nc):
        U[q] = 1.0 + 0.3 * q + (q + 1) * 0.7 * X - 0.2 * Y + 0.05 * q * Z
    return U


# ---------------------------------------------------------------------------
# CPU: the oracle's restatement
# ---------------------------------------------------------------------------
def test_oracle_interpolates_linear_data_exactly(oracle):
    params, boxes, ratios = _orszag_levels()
    p0, p1 = params[0], params[1]
    for p in (p0, p1):
        for d in range(3):
            p.periodic[d] = 0
    ng = mfgpu.num_ghost(p0)
    ca, cfb = _host_level(p0, B0, ng, _linear_init)
    fine = [((8, 8, 8), (15, 15, 23)), ((16, 8, 8), (23, 15, 15))]
    fa, ffb = _host_level(p1, fine, ng, lambda p, lo, hi: _empty(p, lo, hi, np.nan))
    assert oracle.cf_fill(p0, p1, 2, ca, ca, cfb, B0, fa, ffb, fine, 1.0) == 0
    filled = 0
    for a, (lo, hi) in zip(fa, ffb):
        e = _linear_init(p1, lo, hi)
        m = np.isfinite(a[0])
        filled += int(m.sum())
        assert np.max(np.abs(a[:, m] - e[:, m])) < 1e-13
    # every ghost cell of both patches except those inside the sibling
    assert filled == (16 * 16 * 24 - 8 * 8 * 16 - 4 * 8 * 8) + (16 * 16 * 16 - 8 * 8 * 8
                                                                 - 4 * 8 * 12)


def test_oracle_average_of_linear_data_is_cell_centre_value(oracle):
    params, boxes, ratios = _orszag_levels()
    p0, p1 = params[0], params[1]
    ng = mfgpu.num_ghost(p0)
    ca, cfb = _host_level(p0, B0, ng, _empty)
    fa, ffb = _host_level(p1, B1, ng, _linear_init)
    assert oracle.average_down(p0, p1, 2, ca, cfb, B0, fa, ffb, B1) == 0
    checked = 0
    for (lo, hi), a, (vlo, vhi) in zip(cfb, ca, B0):
        e = _linear_init(p0, lo, hi)
        for flo, fhi in B1:
            c0 = [max(vlo[d], flo[d] // 2) - lo[d] for d in range(3)]
            c1 = [min(vhi[d], fhi[d] // 2) - lo[d] for d in range(3)]
            if any(c1[d] < c0[d] for d in range(3)):
                continue
            sl = (slice(None), slice(c0[2], c1[2] + 1), slice(c0[1], c1[1] + 1),
                  slice(c0[0], c1[0] + 1))
            np.testing.assert_allclose(a[sl], e[sl], rtol=1e-14, atol=1e-14)
            checked += a[sl][0].size
    assert checked == sum(np.prod([(h - l + 1) // 2 for l, h in zip(lo, hi)]) for lo, hi in B1)


def test_oracle_hierarchy_conserves_mass(oracle):
    params, boxes, ratios = _orszag_levels()
    ng = mfgpu.num_ghost(params[0])
    L = _oracle_hier(oracle, params, boxes, ratios, _orszag_init)
    m0 = _composite_mass(L, ng)
    times = [0.0, 0.0, 0.0]
    dt = 0.002
    for _ in range(3):
        st, ndt, _ = oracle.hier_step(L, ratios, times, dt)
        assert st == 0
        dt = 0.4 * ndt
        assert abs(_composite_mass(L, ng) - m0) <= 1e-14 * m0
    assert times[0] == times[1] == pytest.approx(times[2], rel=1e-15)


def test_hierarchy_builder_nests_properly():
    n0 = 32
    p = amr.orszag3d_params(n0)
    U = amr.orszag3d_state(p, (0, 0, 0), (n0 - 1,) * 3)
    tags = amr.relgrad_tags(U[0] * (1 + 0.2 * np.sin(np.arange(n0) / 3.0))[None, None, :], 0.05)
    levels = amr.build_hierarchy(tags, ratios=(2, 4), seed=3)
    assert len(levels) == 3 and len(levels[2][2]) > 0
    for lv in (1, 2):
        Rp, npar, bpar = levels[lv - 1]
        R, n, boxes = levels[lv]
        r = R // Rp
        cov = amr.coverage(bpar, npar)
        for lo, hi in boxes:
            assert all(lo[d] % r == 0 and (hi[d] + 1) % r == 0 for d in range(3))
            # the coarsened box grown by ceil(4 / r) + 1 coarse cells is covered
            g = -(-4 // r) + 1
            idx = [np.arange(lo[d] // r - g, hi[d] // r + g + 1) % npar for d in range(3)]
            assert cov[np.ix_(idx[2], idx[1], idx[0])].all()


# ---------------------------------------------------------------------------
# GPU against the oracle
# ---------------------------------------------------------------------------
def _compare_levels(dh, L, ng, tol=RTOL):
    """Valid cells of every level against the oracle.  The parity bar is per
    level step: level l takes prod(ratios[:l]) steps per hierarchy step, so
    its bar is tol times that count (the coarse-fine interpolation itself is
    bitwise; what differs is the last-bit rounding of the transcendentals in
    each level step, e.g. the GLM damping exp, carried into the fine ghosts
    through the time interpolation)."""
    R = 1
    for lv, (p, arrays, fboxes, vboxes) in enumerate(L):
        if lv > 0:
            R *= dh.ratios[lv - 1]
        out = dh.download(lv)
        for i in range(len(vboxes)):
            g = dh.levels[lv].patch_view(out, i)[:, ng:-ng, ng:-ng, ng:-ng]
            o = arrays[i][:, ng:-ng, ng:-ng, ng:-ng]
            e = rel_err(g, o)
            assert np.all(e <= tol * R), (lv, i, e)


@pytest.mark.gpu
def test_gpu_interpolation_and_average_vs_oracle(gpulib, oracle):
    """Fine ghosts interpolated at time fraction 0.3 between two coarse
    states, then the average down, against the oracle (bitwise: the same
    operations in the same order, no transcendentals)."""
    params, boxes, ratios = _orszag_levels()
    ng = mfgpu.num_ghost(params[0])
    dh = amr.DeviceHierarchy(mfgpu, params, boxes, ratios, _orszag_init)
    L = _oracle_hier(oracle, params, boxes, ratios, _orszag_init)
    _compare_levels(dh, L, ng, tol=0.0)
    info = dh.hier.info(1)
    assert info["interpolated"] > 0 and info["register_faces"] > 0
    # old coarse state: the current one; new: a perturbed copy
    dh.hier.snapshot(0)
    p0, a0, fb0, b0 = L[0]
    old = [a.copy() for a in a0]
    new = [a * (1.0 + 0.01 * np.sin(np.arange(a.size)).reshape(a.shape)) for a in a0]
    dh.upload(0, new)
    dh.hier.fill_ghosts(1, 0.3)
    p1, a1, fb1, b1 = L[1]
    assert oracle.cf_fill(p0, p1, 2, old, new, fb0, b0, a1, fb1, b1, 0.3) == 0
    out = dh.download(1)
    for i in range(len(b1)):
        assert np.array_equal(dh.levels[1].patch_view(out, i), a1[i]), i
    dh.hier.average_down(0)
    assert oracle.average_down(p0, p1, 2, new, fb0, b0, a1, fb1, b1) == 0
    out = dh.download(0)
    for i in range(len(b0)):
        g = dh.levels[0].patch_view(out, i)[:, ng:-ng, ng:-ng, ng:-ng]
        assert np.array_equal(g, new[i][:, ng:-ng, ng:-ng, ng:-ng]), i
    dh.close()


@pytest.mark.gpu
@pytest.mark.parametrize("ta", [mfgpu.TA_RK2, mfgpu.TA_FIRST_ORDER, mfgpu.TA_HANCOCK])
def test_gpu_hierarchy_step_vs_oracle(gpulib, oracle, ta):
    params, boxes, ratios = _orszag_levels(ta)
    ng = mfgpu.num_ghost(params[0])
    dh = amr.DeviceHierarchy(mfgpu, params, boxes, ratios, _orszag_init)
    L = _oracle_hier(oracle, params, boxes, ratios, _orszag_init)
    times = [0.0] * 3
    dt = 0.4 * dh.compute_dt()
    for step in range(2):
        ndt_g = dh.step(dt)
        st, ndt_o, _ = oracle.hier_step(L, ratios, times, dt)
        assert st == 0
        _compare_levels(dh, L, ng)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        assert dh.hier.times() == pytest.approx(times, rel=1e-15)
        dt = 0.4 * ndt_o
    dh.close()


@pytest.mark.gpu
def test_gpu_glm_helio_hierarchy_vs_oracle(gpulib, oracle):
    """Two-level GLM heliosphere (far-field boundaries, charge exchange, the
    divergence correction of the interpolated B slopes, Ch/Cp from the base
    level's new dt)."""
    p0 = mfgpu.helio_params(32)
    p1 = amr.level_params(p0, 2)
    b0 = mfgpu.tile_boxes(32, 16, 3)
    b1 = [((16, 16, 16), (31, 31, 47)), ((32, 16, 16), (47, 31, 31))]
    params, boxes, ratios = [p0, p1], [b0, b1], [2]

    def init(p, lo, hi):
        return mfgpu.init_host_fab(p, lo, hi, "helio")

    dh = amr.DeviceHierarchy(mfgpu, params, boxes, ratios, init)
    dt0 = dh.compute_dt()
    dh.set_dedner_from_dt(dt0)
    ng = mfgpu.num_ghost(p0)
    L = _oracle_hier(oracle, params, boxes, ratios, init)
    times = [0.0, 0.0]
    dt = 0.4 * dt0
    for step in range(2):
        ndt_g = dh.step(dt)
        st, ndt_o, ded = oracle.hier_step(L, ratios, times, dt)
        assert st == 0
        _compare_levels(dh, L, ng)
        assert abs(ndt_g - ndt_o) <= RTOL * ndt_o
        # Every step starts from the oracle's state and GLM speeds: a few cells
        # next to the inner sphere are ill-conditioned in this problem (the
        # oracle itself turns a 1e-14 relative perturbation of its state into
        # 1e-9 there within one step, through its region thresholds), so the
        # errors are compared per step, not accumulated.
        for p in params:
            p.dedner_ch, p.dedner_cp = ded
        for c in dh.ctxs:
            c.set_dedner(*ded)
        for lv, (p, arrays, fboxes, vboxes) in enumerate(L):
            dh.upload(lv, arrays)
        dt = 0.4 * ndt_o
    dh.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [(mfgpu.PREC_FP64, 1e-14), (mfgpu.PREC_MIXED, 1e-10)])
def test_gpu_hierarchy_conserves_mass(gpulib, prec, tol):
    """Composite mass over 5 hierarchy steps (reflux + average down make the
    coarse-fine boundary conservative).  FP64: to rounding.  Mixed: the flux
    difference of each cell is formed in FP32 before the FP64 accumulation,
    so the sum telescopes only to FP32 rounding of those differences."""
    params, boxes, ratios = _orszag_levels(prec=prec)
    ng = mfgpu.num_ghost(params[0])
    dh = amr.DeviceHierarchy(mfgpu, params, boxes, ratios, _orszag_init)

    def mass():
        out = dh.download(0)
        return sum(dh.levels[0].patch_view(out, i)[0, ng:-ng, ng:-ng, ng:-ng].sum()
                   for i in range(len(boxes[0]))) * params[0].dx ** 3

    m0 = mass()
    dt = 0.4 * dh.compute_dt()
    for _ in range(5):
        dt = 0.4 * dh.step(dt)
    assert abs(mass() - m0) <= tol * m0
    dh.close()
