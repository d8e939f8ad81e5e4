"""Block-structured AMR hierarchies for the batched level path.

A hierarchy here is a list of levels, each a set of non-overlapping patches
(valid boxes in that level's index space) stepped by one ``mf_level`` in
batched launches.  Levels are built the way the reference regrids
(AMRLevelIdealMHD::tagCells, srcIdeal/AMRLevelIdealMHD.cpp:1782-1870):

* cells are tagged where the undivided relative density gradient reaches a
  threshold: PatchMHDMF::tagCells (srcIdeal/PatchMHDMF.cpp:149-200) with
  GETRELGRAD (src/PatchMHDAMF.ChF:318-415) per direction and MAGNITUDE over
  the directions;
* tags are covered by cubic patches whose edge lengths are drawn from a
  seeded distribution over a set of sizes (8, 16, 24, 32 cells by default),
  on a granule grid of 8 cells, each patch properly nested inside the next
  coarser level's patches: a granule is refined only if the granules around
  it are covered by the coarser level too, so that the coarse-fine
  interpolation, the flux registers and the averaging of mf_hier read coarse
  valid cells only (Chombo's proper nesting).  Chombo's Berger-Rigoutsos
  clustering is replaced by this seeded cover: the sizes of the patches are
  the point of the batched form, not the cluster efficiency.

DeviceHierarchy steps such a hierarchy on the device through mf_hier
(subcycled, coarse-fine ghosts interpolated, refluxed, averaged down).
"""
from __future__ import annotations

import numpy as np

from . import (MfParams, PREC_FP64, TA_RK2, _base_params, grow, fab_shape, num_cons)

GRANULE = 8
SIZES = (8, 16, 24, 32)


# ---------------------------------------------------------------------------
# problem: a three-dimensional Orszag-Tang vortex
# ---------------------------------------------------------------------------
def orszag3d_params(n: int, time_approximation: int = TA_RK2,
                    precision: int = PREC_FP64) -> MfParams:
    """Single-fluid ideal MHD on an n^3 periodic unit cube with the Orszag-Tang
    settings (problems/OrszagF.ChF SETORSZAG :4-25): gamma 5/3, Roe 8-wave
    flux, minmod, 8-wave source, Bn from the face average."""
    p = _base_params(3, 1)
    p.time_approximation = time_approximation
    p.precision = precision
    g = 5.0 / 3.0
    p.gamma = g
    r0 = g * g
    umag = np.sqrt(g * g / r0)
    p.smallr = 1e-8 * r0
    p.smallp = 1e-8 * r0 * 0.5 * umag * umag
    p.dx = 1.0 / n
    for d in range(3):
        p.domain_lo[d] = 0
        p.domain_hi[d] = n - 1
        p.periodic[d] = 1
    return p


def level_params(p0: MfParams, refinement: int) -> MfParams:
    """Parameters of a level refined by `refinement` with respect to p0."""
    p = MfParams()
    ctypes_copy(p, p0)
    p.dx = p0.dx / refinement
    for d in range(p0.space_dim):
        n = p0.domain_hi[d] - p0.domain_lo[d] + 1
        p.domain_lo[d] = p0.domain_lo[d] * refinement
        p.domain_hi[d] = p.domain_lo[d] + n * refinement - 1
    return p


def ctypes_copy(dst, src):
    import ctypes
    ctypes.memmove(ctypes.addressof(dst), ctypes.addressof(src), ctypes.sizeof(src))


def orszag3d_state(p: MfParams, lo, hi, eps: float = 0.2) -> np.ndarray:
    """Conserved state (nc, nz, ny, nx) on the box [lo, hi] (ghosts allowed):
    the reference's Orszag-Tang state (problems/OrszagF.ChF:27-79, Gaussian
    units, rho = gamma^2/4pi, p = gamma/4pi) with the velocity modulated along
    z as in the common three-dimensional variant,
    v = (-(1 + eps sin 2pi z) sin 2pi y, (1 + eps sin 2pi z) sin 2pi x, eps sin 2pi z)."""
    g = p.gamma
    p0 = g / (4.0 * np.pi)
    r0 = p0 * g
    dx = p.dx
    x = (np.arange(lo[0], hi[0] + 1) + 0.5) * dx
    y = (np.arange(lo[1], hi[1] + 1) + 0.5) * dx
    z = (np.arange(lo[2], hi[2] + 1) + 0.5) * dx
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    tp = 2.0 * np.pi
    mod = 1.0 + eps * np.sin(tp * Z)
    ux = -mod * np.sin(tp * Y)
    uy = mod * np.sin(tp * X)
    uz = eps * np.sin(tp * Z)
    bx = -np.sin(tp * Y)
    by = np.sin(2.0 * tp * X)
    nc = num_cons(p)
    U = np.zeros((nc,) + X.shape)
    U[0] = r0
    U[1] = r0 * ux
    U[2] = r0 * uy
    U[3] = r0 * uz
    U[4] = p0 / (g - 1.0) + 0.5 * (r0 * (ux * ux + uy * uy + uz * uz) + (bx * bx + by * by) / (4.0 * np.pi))
    U[5] = bx
    U[6] = by
    return U


# ---------------------------------------------------------------------------
# tagging
# ---------------------------------------------------------------------------
def relgrad(u: np.ndarray, axis: int, periodic: bool) -> np.ndarray:
    """GETRELGRAD (src/PatchMHDAMF.ChF:318-415) along one array axis: centred
    half-difference over half-sum in the interior (0 where |half-sum| <
    1e-32), one-sided at non-periodic domain edges."""
    up = np.roll(u, -1, axis=axis)
    um = np.roll(u, 1, axis=axis)
    diff = 0.5 * (up - um)
    aver = 0.5 * (up + um)
    out = np.where(np.abs(aver) < 1e-32, 0.0, diff / np.where(aver == 0.0, 1.0, aver))
    if not periodic:
        n = u.shape[axis]
        sl = [slice(None)] * u.ndim

        def take(i):
            s = list(sl)
            s[axis] = i
            return tuple(s)

        d_lo = u[take(1)] - u[take(0)]
        a_lo = 0.5 * (u[take(1)] + u[take(0)])
        out[take(0)] = np.where(np.abs(a_lo) < 1e-32, 0.0, d_lo / np.where(a_lo == 0, 1, a_lo))
        d_hi = u[take(n - 1)] - u[take(n - 2)]
        a_hi = 0.5 * (u[take(n - 1)] + u[take(n - 2)])
        out[take(n - 1)] = d_hi / a_hi
    return out


def relgrad_tags(rho: np.ndarray, threshold: float, periodic=(True, True, True)) -> np.ndarray:
    """Tags of PatchMHDMF::tagCells: |(GETRELGRAD_x, _y, _z)| >= threshold
    (srcIdeal/PatchMHDMF.cpp:185-200).  rho is indexed (z, y, x)."""
    sd = rho.ndim
    mag2 = np.zeros_like(rho)
    for d in range(sd):
        axis = sd - 1 - d
        g = relgrad(rho, axis, bool(periodic[d]))
        mag2 += g * g
    return np.sqrt(mag2) >= threshold


# ---------------------------------------------------------------------------
# patch cover
# ---------------------------------------------------------------------------
def cover(gtags: np.ndarray, allowed: np.ndarray, sizes_g, rng: np.random.Generator):
    """Cover the tagged granules with non-overlapping cubes of allowed
    granules.  Granules are visited in (z, y, x) order; an untaken tagged
    granule starts a cube whose edge (in granules) is drawn from sizes_g and
    shrunk until the cube lies in the grid, in `allowed` and clear of earlier
    cubes.  Returns a list of (lo, hi) in granules (inclusive)."""
    G = gtags.shape
    taken = np.zeros(G, dtype=bool)
    out = []
    todo = gtags & allowed
    for k, j, i in np.argwhere(todo):
        if taken[k, j, i]:
            continue
        s = int(rng.choice(sizes_g))
        while s > 1:
            if (k + s <= G[0] and j + s <= G[1] and i + s <= G[2]
                    and allowed[k:k + s, j:j + s, i:i + s].all()
                    and not taken[k:k + s, j:j + s, i:i + s].any()):
                break
            s -= 1
        taken[k:k + s, j:j + s, i:i + s] = True
        out.append(((int(i), int(j), int(k)), (int(i + s - 1), int(j + s - 1), int(k + s - 1))))
    return out


def _block_any(a: np.ndarray, b: int) -> np.ndarray:
    n = a.shape
    return a.reshape(n[0] // b, b, n[1] // b, b, n[2] // b, b).any(axis=(1, 3, 5))


def _block_all(a: np.ndarray, b: int) -> np.ndarray:
    n = a.shape
    return a.reshape(n[0] // b, b, n[1] // b, b, n[2] // b, b).all(axis=(1, 3, 5))


def coverage(boxes, n: int) -> np.ndarray:
    """Boolean (n, n, n) map (z, y, x) of the cells inside the boxes."""
    m = np.zeros((n, n, n), dtype=bool)
    for lo, hi in boxes:
        m[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = True
    return m


def build_hierarchy(tags0: np.ndarray, ratios=(2, 4), sizes=SIZES, granule: int = GRANULE,
                    seed: int = 0, nest: int = 1):
    """Levels of patches over a periodic n0^3 base grid with cell tags tags0
    (z, y, x).

    Level 0 covers the domain; level l (refinement R_l = prod(ratios[:l]))
    covers the granules whose footprint on the base grid holds a tag and
    whose neighbourhood of `nest` granules (periodic) lies inside the patches
    of level l-1.  One granule (8 fine cells, 8/r coarse cells) is enough
    buffer for 4 ghost layers at ratios 2 and 4.  Returns
    [(refinement, n_l, boxes_l), ...] with boxes in cells of level l."""
    rng = np.random.default_rng(seed)
    n0 = tags0.shape[0]
    assert tags0.shape == (n0, n0, n0) and n0 % granule == 0
    sizes_g = [s // granule for s in sizes]
    assert all(s * granule == t for s, t in zip(sizes_g, sizes))
    g0 = n0 // granule
    levels = []
    gb = cover(np.ones((g0,) * 3, bool), np.ones((g0,) * 3, bool), sizes_g, rng)
    levels.append((1, n0, [_cells(b, granule) for b in gb]))
    R = 1
    for r in ratios:
        assert granule % r == 0
        Rp, np_, bp = levels[-1]
        R *= r
        n = n0 * R
        G = n // granule
        # tags: any base-grid tag under the granule (footprint granule / R cells)
        if R <= granule:
            gt = _block_any(tags0, granule // R)
        else:
            rep = R // granule
            gt = np.repeat(np.repeat(np.repeat(tags0, rep, 0), rep, 1), rep, 2)
        # nesting: the footprints on level l-1 (granule / r cells) of the
        # granule and of its neighbours within `nest` granules
        inside = _block_all(coverage(bp, np_), granule // r)
        allowed = inside.copy()
        for dz in range(-nest, nest + 1):
            for dy in range(-nest, nest + 1):
                for dx in range(-nest, nest + 1):
                    allowed &= np.roll(inside, (dz, dy, dx), axis=(0, 1, 2))
        gb = cover(gt, allowed, sizes_g, rng)
        levels.append((R, n, [_cells(b, granule) for b in gb]))
    return levels


def _cells(b, granule):
    lo, hi = b
    return (tuple(x * granule for x in lo), tuple((x + 1) * granule - 1 for x in hi))


# ---------------------------------------------------------------------------
# level data
# ---------------------------------------------------------------------------
def prolong_fab(coarse: np.ndarray, refinement: int, lo, hi) -> np.ndarray:
    """Piecewise-constant prolongation of a periodic base-grid state coarse
    (nc, n0, n0, n0) onto the cells [lo, hi] of a level refined by
    `refinement` (ghost cells wrap around the periodic domain)."""
    n0 = coarse.shape[1]
    ix = [np.floor_divide(np.arange(lo[d], hi[d] + 1), refinement) % n0 for d in range(3)]
    return coarse[:, ix[2][:, None, None], ix[1][None, :, None], ix[0][None, None, :]]


def fill_level_buffer(level, coarse: np.ndarray, refinement: int) -> np.ndarray:
    """A host buffer in the layout of `level` (an mfgpu.Level) holding every
    patch's fab, ghosts included, prolonged from the base-grid state."""
    buf = np.zeros(level.ndoubles)
    for i in range(len(level.boxes)):
        lo, hi = level.fab_box(i)
        level.patch_view(buf, i)[...] = prolong_fab(coarse, refinement, lo, hi)
    return buf


# ---------------------------------------------------------------------------
# a coupled hierarchy on the device
# ---------------------------------------------------------------------------
class DeviceHierarchy:
    """Levels of a hierarchy resident on the device and coupled by mf_hier.

    params: per-level MfParams (level_params of the base parameters);
    boxes: per-level valid boxes; ratios: refinement between consecutive
    levels; init(p, lo, hi) -> conserved state (nc, nz, ny, nx) on a fab box.
    After the upload the coarse cells under finer patches are averaged from
    them, so that the composite state is consistent."""

    def __init__(self, mfgpu, params, boxes, ratios, init):
        self.mfgpu = mfgpu
        self.params = list(params)
        self.boxes = [list(b) for b in boxes]
        self.ratios = list(ratios)
        self.ctxs = [mfgpu.Context(p) for p in self.params]
        self.levels = [mfgpu.Level(c, b) for c, b in zip(self.ctxs, self.boxes)]
        self.bufs = []
        for lev, p in zip(self.levels, self.params):
            buf = np.zeros(lev.ndoubles)
            for i in range(len(lev.boxes)):
                lo, hi = lev.fab_box(i)
                lev.patch_view(buf, i)[...] = init(p, lo, hi)
            lev.upload(buf.ctypes.data)
            self.bufs.append(buf)
        self.hier = mfgpu.Hier(self.levels, self.ratios)
        for lv in range(len(self.levels) - 2, -1, -1):
            self.hier.average_down(lv)

    def set_dedner_from_dt(self, dt_base):
        """GLM speeds of every level from the base level's dt (Ch = factor_ch
        dx0 / dt, Cp = sqrt(Ch dx0 / factor_cp))."""
        p0 = self.params[0]
        ch = p0.factor_ch * p0.dx / dt_base
        cp = float(np.sqrt(ch * p0.dx / p0.factor_cp))
        for c, p in zip(self.ctxs, self.params):
            p.dedner_ch, p.dedner_cp = ch, cp
            c.set_dedner(ch, cp)
        return ch, cp

    def compute_dt(self):
        """min over levels of dx/cmax times the level's refinement."""
        best, R = None, 1
        for lv, lev in enumerate(self.levels):
            if lv > 0:
                R *= self.ratios[lv - 1]
            v = lev.compute_dt()[0] * R
            best = v if best is None else min(best, v)
        return best

    def step(self, dt0, stream=None):
        return self.hier.step(dt0, stream)

    def download(self, lv):
        """Host copy (level layout) of level lv's state."""
        out = np.zeros(self.levels[lv].ndoubles)
        self.levels[lv].download(out.ctypes.data)
        return out

    def upload(self, lv, arrays):
        """Replace level lv's fabs (ghosts included) by host arrays."""
        buf = np.zeros(self.levels[lv].ndoubles)
        for i, a in enumerate(arrays):
            self.levels[lv].patch_view(buf, i)[...] = a
        self.levels[lv].upload(buf.ctypes.data)
        self.bufs[lv] = buf

    def cells_per_step(self):
        """Zone updates of one base step (each level's cells times its steps)."""
        z, R = 0, 1
        for lv, lev in enumerate(self.levels):
            if lv > 0:
                R *= self.ratios[lv - 1]
            z += lev.ncells * R
        return z

    def close(self):
        self.hier.close()
        for lev in self.levels:
            lev.close()
        for c in self.ctxs:
            c.close()
