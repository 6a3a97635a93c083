"""Algorithmic work of the projector, for roofline figures.

``nnz_per_view`` counts the (ray, voxel) pairs with a positive intersection
length -- the number of nonzeros of one view's system matrix -- from the
ray's crossings of the voxel grid planes (a ray that enters the grid and
crosses k internal planes passes through k + 1 voxels).  The algorithmic
bytes per launch are then (FP32):

* fused Ax  (SART forward step) : 4*nnz + 8*na*nb   (m per nonzero; P in, cor out)
* fused Atx (SART backward step): 4*nnz + 8*N       (cor per nonzero; m in, m out)
* one TV step (one fused pass)  : 8*N               (read m, write m')
"""
from __future__ import annotations

import numpy as np


def _gateway(phi, SO, OD, vxlsize, detsize, na, nb):
    sc = np.float32(vxlsize)
    c = np.cos(np.float32(phi), dtype=np.float32)
    s = np.sin(np.float32(phi), dtype=np.float32)
    so = np.float32(SO) / sc
    od = np.float32(OD) / sc
    det = np.float64(np.float32(detsize) / sc)
    yd = (np.arange(na) - na / 2.0 + 0.5) * det
    zd = (np.arange(nb) - nb / 2.0 + 0.5) * det
    return float(c), float(s), float(so), float(od), yd, zd


def nnz_per_view(phi_deg, SO, OD, vxlsize, detsize, nx, ny, nz, na, nb):
    """Nonzeros of the system matrix of one view (view angle in degrees)."""
    c, s, so, od, yd, zd = _gateway(-phi_deg / 180 * np.pi, SO, OD, vxlsize, detsize,
                                    na, nb)
    A, B = np.meshgrid(yd, zd, indexing="xy")
    S = np.array([c * -so, s * -so, 0.0])
    Dx = c * od - s * A.ravel()
    Dy = s * od + c * A.ravel()
    Dz = B.ravel() if (nz > 1 or nb > 1) else np.zeros(A.size)
    P0 = [np.full(Dx.size, S[0]), np.full(Dx.size, S[1]), np.full(Dx.size, S[2])]
    P1 = [Dx, Dy, Dz]
    dims = [nx, ny, nz]
    axes = 3 if (nz > 1 or nb > 1) else 2
    tmin = np.zeros(Dx.size)
    tmax = np.ones(Dx.size)
    lo = [-(n // 2) for n in dims]
    for k in range(axes):
        d = P1[k] - P0[k]
        with np.errstate(divide="ignore", invalid="ignore"):
            t0 = (lo[k] - P0[k]) / d
            t1 = (lo[k] + dims[k] - P0[k]) / d
        a = np.minimum(t0, t1)
        b = np.maximum(t0, t1)
        inside = (P0[k] >= lo[k]) & (P0[k] <= lo[k] + dims[k])
        a = np.where(d == 0, np.where(inside, -np.inf, np.inf), a)
        b = np.where(d == 0, np.where(inside, np.inf, -np.inf), b)
        tmin = np.maximum(tmin, a)
        tmax = np.minimum(tmax, b)
    hit = tmax > tmin
    count = np.where(hit, 1, 0).astype(np.int64)
    for k in range(axes):
        xa = P0[k] + tmin * (P1[k] - P0[k])
        xb = P0[k] + tmax * (P1[k] - P0[k])
        u = np.maximum(xa, xb)
        v = np.minimum(xa, xb)
        crossings = np.maximum(np.ceil(u) - np.floor(v) - 1, 0)
        count += np.where(hit, crossings, 0).astype(np.int64)
    return int(count.sum())


def atx_bytes(nnz, N):
    return 4 * nnz + 8 * N


def ax_bytes(nnz, M):
    return 4 * nnz + 8 * M


def tv_step_bytes(N):
    return 8 * N
