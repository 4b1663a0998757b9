"""Absorbing-boundary profiles, same signatures and values as the reference.

Mirrors ``ADFWI/propagator/boundary_condition.py``:
  * ``bc_pml`` (15-47): quadratic PML damping d = kappa (i dx / a)^2, a = (pml-1) dx,
    kappa = -3 vmax ln(1e-6) / (2a). In a corner the reference's strip-by-strip
    overwrite leaves the larger of the x and z values, i.e. d(i, j) =
    prof[max(dist_z(i), dist_x(j))]; it is built here directly in that form.
  * ``bc_sincos`` (50-68): product of per-axis sin^2 tapers.
  * ``bc_gerjan`` (71-95): Gerjan (1985) exp(-(alpha (pml-k))^2) frame.
  * ``bc_pml_xz`` (98-120): separate x / z PML profiles for the elastic split-field scheme.
All return float64 numpy arrays of shape (nz_pml, nx_pml).
"""
from math import log

import numpy as np


def _dims(nx, nz, pml, free_surface):
    return nx + 2 * pml, (nz + pml) if free_surface else (nz + 2 * pml)


def _edge_distance(n, pml, low=True):
    """Distance into the absorbing strip (0 = innermost absorbing cell); -1 in the interior."""
    idx = np.arange(n)
    d = np.full(n, -1, dtype=np.int64)
    if low:
        m = idx < pml
        d[m] = pml - 1 - idx[m]
    m = idx >= n - pml
    d[m] = idx[m] - (n - pml)
    return d


def bc_pml(nx, nz, dx, dz, pml, vmax, free_surface=True):
    nx_pml, nz_pml = _dims(nx, nz, pml, free_surface)
    a = (pml - 1) * dx
    kappa = -3.0 * vmax * log(1e-6) / (2.0 * a)
    # Scalar arithmetic per cell keeps the caller's scalar type (a float32 vmax, as a model's
    # vp.max() is, makes every product float32 like the reference's loop).
    prof = np.zeros(pml + 1)  # prof[-1] = 0 for interior cells
    for ix in range(pml):
        xa = ix * dx / a
        prof[ix] = kappa * xa * xa
    dist = np.maximum(_edge_distance(nz_pml, pml, low=not free_surface)[:, None],
                      _edge_distance(nx_pml, pml)[None, :])
    return prof[dist]


def bc_sincos(nx, nz, dx, dz, pml, free_surface=False):
    nx_pml, nz_pml = _dims(nx, nz, pml, free_surface)
    taper = np.sin(np.pi / 2 * np.arange(pml) / pml) ** 2
    fz = np.ones(nz_pml)
    fx = np.ones(nx_pml)
    for i in range(pml):
        if not free_surface:
            fz[i] *= taper[i]
        fz[nz_pml - 1 - i] *= taper[i]
        fx[i] *= taper[i]
        fx[nx_pml - 1 - i] *= taper[i]
    return fz[:, None] * fx[None, :]


def bc_gerjan(nx, nz, dx, dz, pml, alpha=0.0053, free_surface=True):
    nx_pml, nz_pml = _dims(nx, nz, pml, free_surface)
    wt = np.exp(-(alpha * (pml - np.arange(1, pml + 1))) ** 2)
    damp = np.ones((nz_pml, nx_pml))
    for k in range(1, pml + 1):
        v = wt[k - 1]
        lo, hi = k - 1, nx_pml - k + 1
        if free_surface:
            damp[:nz_pml - k + 1, k - 1] = v
            damp[nz_pml - k, lo:hi] = v
            damp[:nz_pml - k + 1, nx_pml - k] = v
        else:
            damp[k - 1:nz_pml - k + 1, k - 1] = v
            damp[k:nz_pml - k + 1, nx_pml - k] = v
            damp[nz_pml - k, lo:hi] = v
            damp[k - 1, lo:hi] = v
    return damp


def bc_pml_xz(nx, nz, dx, dz, pml, vmax, free_surface=True):
    nx_pml, nz_pml = _dims(nx, nz, pml, free_surface)
    ppml = -np.log(1e-6) * 3 * vmax / (2 * pml ** 3)
    k = np.arange(1, pml + 1)
    vx = (pml - k + 1) ** 2 * ppml / dx
    vz = (pml - k + 1) ** 2 * ppml / dz
    px = np.zeros(nx_pml)
    px[k - 1] = vx
    px[nx_pml - k] = vx
    pz = np.zeros(nz_pml)
    pz[nz_pml - k] = vz
    if not free_surface:
        pz[k - 1] = vz
    bcx = np.broadcast_to(px[None, :], (nz_pml, nx_pml)).copy()
    bcz = np.broadcast_to(pz[:, None], (nz_pml, nx_pml)).copy()
    return bcx, bcz
