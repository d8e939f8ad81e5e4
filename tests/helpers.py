"""Shared helpers of the tests: fab construction, periodic ghost fill on the
host, device round trips through torch, and the parity comparison."""
from __future__ import annotations

import numpy as np

import mfgpu


def periodic_fill(U: np.ndarray, ng: int, sd: int) -> np.ndarray:
    """Fill the ghost cells of a single-patch fab that covers a periodic
    domain exactly (valid = fab shrunk by ng)."""
    if sd == 2:
        v = U[:, :, ng:-ng, ng:-ng]
        U[:] = np.pad(v, ((0, 0), (0, 0), (ng, ng), (ng, ng)), mode="wrap")
    else:
        v = U[:, ng:-ng, ng:-ng, ng:-ng]
        U[:] = np.pad(v, ((0, 0), (ng, ng), (ng, ng), (ng, ng)), mode="wrap")
    return U


def valid_view(U: np.ndarray, ng: int, sd: int) -> np.ndarray:
    if sd == 2:
        return U[:, :, ng:-ng, ng:-ng]
    return U[:, ng:-ng, ng:-ng, ng:-ng]


def component_groups(nc: int, nls: int = 0) -> list[list[int]]:
    """Physical groups of the conserved components: density, momentum vector,
    energy, magnetic field vector, psi, then density / momentum / energy of
    each neutral fluid, then each of the nls tracking surfaces."""
    nf = nc - nls
    glm = 1 if (nf - 8) % 5 == 1 else 0
    groups = [[0], [1, 2, 3], [4], [5, 6, 7]]
    if glm:
        groups.append([8])
    s = 8 + glm
    while s + 5 <= nf:
        groups += [[s], [s + 1, s + 2, s + 3], [s + 4]]
        s += 5
    groups += [[q] for q in range(nf, nc)]
    return groups


def rel_err(a: np.ndarray, b: np.ndarray, floor_frac: float = 1e-3, nls: int = 0) -> np.ndarray:
    """Per-component maximum of |a-b| / max(|b|, floor_frac * S): pointwise
    relative error, where S is the largest magnitude of the component's
    physical group (a vector component that is zero, e.g. the z-momentum of a
    2D run, is measured against the magnitude of its vector).  nls: number of
    tracking surfaces after the fluid components."""
    nc = b.shape[0]
    scale = np.zeros(nc)
    for g in component_groups(nc, nls):
        s = max(float(np.max(np.abs(b[c]))) if b[c].size else 0.0 for c in g)
        for c in g:
            scale[c] = s
    out = []
    for c in range(nc):
        bc = b[c]
        den = np.maximum(np.abs(bc), floor_frac * scale[c])
        den = np.where(den == 0.0, 1.0, den)
        out.append(float(np.max(np.abs(a[c] - bc) / den)) if bc.size else 0.0)
    return np.array(out)


def to_device(arr: np.ndarray):
    import torch
    return torch.from_numpy(np.ascontiguousarray(arr)).to("cuda")


def to_host(t) -> np.ndarray:
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def orszag_patch(n: int, ng: int, p) -> np.ndarray:
    """Single periodic patch [0,n-1]^2 + ghosts holding the Orszag-Tang state."""
    lo, hi = mfgpu.grow([0, 0, 0], [n - 1, n - 1, 0], ng, 2)
    U = mfgpu.init_host_fab(p, lo, hi, "orszag")
    return periodic_fill(U, ng, 2)
