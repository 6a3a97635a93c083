"""Seeded synthetic inputs: ellipsoid phantoms, view angles and noise.

* ``shepp_logan_3d`` / ``shepp_logan_2d``: the modified Shepp-Logan head
  phantom (Toft's higher-contrast intensities), evaluated like the
  reference's utilities/phantom3d.m: an n^3 grid on [-1, 1] with voxel
  (r, c, k) sampled at (x=g[c], y=g[r], z=g[k]), each ellipsoid adding its
  amplitude where ((p - p0) rotated)^2 / axes^2 <= 1.  The parameter table is
  the published one (Toft 1996, pp. 199-200).
* ``random_ellipses``: seeded piecewise-smooth phantoms for the sparse-view
  and batched workloads.
* ``poisson_noise``: P = -ln(Poisson(I0 e^-p) / I0), zero counts set to 1.

Volumes are returned flat in the projector's x-fastest layout.
"""
from __future__ import annotations

import numpy as np

# A, a, b, c, x0, y0, z0, phi, theta, psi (degrees)
MODIFIED_SHEPP_LOGAN = np.array([
    [1.0, 0.6900, 0.920, 0.810, 0.00, 0.0000, 0.00, 0.0, 0.0, 0.0],
    [-0.8, 0.6624, 0.874, 0.780, 0.00, -0.0184, 0.00, 0.0, 0.0, 0.0],
    [-0.2, 0.1100, 0.310, 0.220, 0.22, 0.0000, 0.00, -18.0, 0.0, 10.0],
    [-0.2, 0.1600, 0.410, 0.280, -0.22, 0.0000, 0.00, 18.0, 0.0, 10.0],
    [0.1, 0.2100, 0.250, 0.410, 0.00, 0.3500, -0.15, 0.0, 0.0, 0.0],
    [0.1, 0.0460, 0.046, 0.050, 0.00, 0.1000, 0.25, 0.0, 0.0, 0.0],
    [0.1, 0.0460, 0.046, 0.050, 0.00, -0.1000, 0.25, 0.0, 0.0, 0.0],
    [0.1, 0.0460, 0.023, 0.050, -0.08, -0.6050, 0.00, 0.0, 0.0, 0.0],
    [0.1, 0.0230, 0.023, 0.020, 0.00, -0.6060, 0.00, 0.0, 0.0, 0.0],
    [0.1, 0.0230, 0.046, 0.020, 0.06, -0.6050, 0.00, 0.0, 0.0, 0.0],
])


def _rot(phi, theta, psi):
    """z-x-z Euler rotation R = Rz(psi) Rx(theta) Rz(phi) (angles in radians)."""
    def rz(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]])

    def rx(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[1.0, 0.0, 0.0], [0.0, c, s], [0.0, -s, c]])

    return rz(psi) @ rx(theta) @ rz(phi)


def ellipsoids(table, nx, ny, nz, zslices=None):
    """Evaluate an ellipsoid table on the phantom3d grid (n = max dims).

    Returns a flat float64 volume with x (the first MATLAB dimension, i.e.
    the grid's y coordinate) fastest.  ``zslices`` selects z planes of the
    full cube (phantom3d's I3d(:,:,k) cropping)."""
    n = max(nx, ny, nz if zslices is None else 1)
    g = (np.arange(n) - (n - 1) / 2) / ((n - 1) / 2) if n > 1 else np.zeros(1)
    gr = g[:nx]
    gc = g[:ny]
    gz = g[np.asarray(zslices)] if zslices is not None else g[:nz]
    # array index (r, c, k) -> point (x=g[c], y=g[r], z=g[k])
    Y, X, Z = np.meshgrid(gr, gc, gz, indexing="ij")
    X, Y, Z = X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F")
    vol = np.zeros(X.size)
    # elementwise, one rounding per operation, in the order the device
    # phantom (asdpocs_phantom_device) evaluates it
    for row in ellipsoid_rows(table):
        A, a, b, c, x0, y0, z0 = row[:7]
        R = row[7:].reshape(3, 3)
        q0 = R[0, 0] * X + R[0, 1] * Y + R[0, 2] * Z
        q1 = R[1, 0] * X + R[1, 1] * Y + R[1, 2] * Z
        q2 = R[2, 0] * X + R[2, 1] * Y + R[2, 2] * Z
        inside = ((q0 - x0) ** 2 / (a * a) + (q1 - y0) ** 2 / (b * b)
                  + (q2 - z0) ** 2 / (c * c)) <= 1
        vol[inside] += A
    return vol


def ellipsoid_rows(table) -> np.ndarray:
    """The table as the device phantom takes it: per ellipsoid A, a, b, c,
    x0, y0, z0 and the 3 x 3 rotation (row-major), float64."""
    rows = []
    for A, a, b, c, x0, y0, z0, ph, th, ps in np.asarray(table, np.float64):
        R = _rot(np.deg2rad(ph), np.deg2rad(th), np.deg2rad(ps))
        rows.append(np.concatenate([[A, a, b, c, x0, y0, z0], R.ravel()]))
    return np.array(rows, np.float64).reshape(-1, 16)


def shepp_logan_3d(n: int) -> np.ndarray:
    return ellipsoids(MODIFIED_SHEPP_LOGAN, n, n, n)


def shepp_logan_2d(n: int) -> np.ndarray:
    """Central (z = 0) section of the 3D phantom on an n x n grid."""
    t = MODIFIED_SHEPP_LOGAN.copy()
    g = (np.arange(n) - (n - 1) / 2) / ((n - 1) / 2)
    Y, X = np.meshgrid(g, g, indexing="ij")
    pts = np.stack([X.ravel(order="F"), Y.ravel(order="F"), np.zeros(n * n)])
    vol = np.zeros(n * n)
    for A, a, b, c, x0, y0, z0, ph, th, ps in t:
        q = _rot(np.deg2rad(ph), np.deg2rad(th), np.deg2rad(ps)) @ pts
        inside = ((q[0] - x0) ** 2 / a ** 2 + (q[1] - y0) ** 2 / b ** 2
                  + (q[2] - z0) ** 2 / c ** 2) <= 1
        vol[inside] += A
    return vol


def random_ellipses(n: int, seed: int, vmax: float = 0.04, count: int = 12) -> np.ndarray:
    """Seeded piecewise-smooth 2D phantom with values in [0, vmax] (1/mm):
    a soft-tissue body ellipse with a smooth gradient plus ``count`` random
    inserts (bone-like, fat-like and cavities), clipped to [0, vmax]."""
    rng = np.random.default_rng(seed)
    g = (np.arange(n) - (n - 1) / 2) / ((n - 1) / 2)
    Y, X = np.meshgrid(g, g, indexing="ij")
    X = X.ravel(order="F")
    Y = Y.ravel(order="F")
    img = np.zeros(n * n)
    a0, b0 = rng.uniform(0.75, 0.92), rng.uniform(0.8, 0.95)
    body = (X / a0) ** 2 + (Y / b0) ** 2 <= 1
    smooth = 0.5 * vmax * (1 + 0.1 * np.cos(np.pi * X * rng.uniform(0.5, 1.5))
                           * np.cos(np.pi * Y * rng.uniform(0.5, 1.5)))
    img[body] = smooth[body]
    for _ in range(count):
        a, b = rng.uniform(0.03, 0.3, size=2)
        x0, y0 = rng.uniform(-0.55, 0.55, size=2)
        th = rng.uniform(0, np.pi)
        c, s = np.cos(th), np.sin(th)
        u = (X - x0) * c + (Y - y0) * s
        v = -(X - x0) * s + (Y - y0) * c
        inside = (u / a) ** 2 + (v / b) ** 2 <= 1
        img[inside & body] += rng.choice([-0.45, -0.2, 0.15, 0.4]) * vmax
    return np.clip(img, 0.0, vmax)


def fov_voxel_size(SO: float, OD: float, det: float, na: int, nx: int) -> float:
    """Voxel size that fits the detector's field of view: SO/(SO+OD)*det*na/nx
    (the reference demos' rule, demo_test.m:25-26)."""
    return SO / (SO + OD) * det * na / nx


def views(nv: int, span: float = 360.0) -> np.ndarray:
    """View angles (degrees) evenly spaced over ``span``: (1:nv)*span/nv."""
    return np.arange(1, nv + 1, dtype=np.float64) * (span / nv)


def poisson_noise(P: np.ndarray, I0: float, seed: int) -> np.ndarray:
    """-ln(Poisson(I0*exp(-P))/I0) with zero counts set to 1."""
    rng = np.random.default_rng(seed)
    counts = rng.poisson(I0 * np.exp(-np.asarray(P, np.float64)))
    counts = np.maximum(counts, 1)
    return -np.log(counts / I0)


# ----------------------------------------------------------------- device
def ellipsoids_device(table, nx, ny, nz, out_ptr: int, scale: float = 1.0,
                      stream: int = 0) -> None:
    """The ellipsoid phantom of ``ellipsoids(table, nx, ny, nz) * scale`` as
    float32, computed on the GPU into the device buffer at ``out_ptr``
    (asdpocs_phantom_device; bit-identical to the host form)."""
    import ctypes as C

    from ._lib import check, load

    rows = np.ascontiguousarray(ellipsoid_rows(table))
    check(load().asdpocs_phantom_device(
        C.c_void_p(out_ptr), int(nx), int(ny), int(nz),
        rows.ctypes.data_as(C.POINTER(C.c_double)), int(rows.shape[0]), float(scale),
        C.c_void_p(stream or None)))


def poisson_noise_device(p_ptr: int, out_ptr: int, n: int, I0: float, seed: int,
                         stream: int = 0) -> None:
    """Poisson-noise sinogram on the GPU (asdpocs_poisson_noise_device): the
    same model as ``poisson_noise``, from a counter-based generator."""
    import ctypes as C

    from ._lib import check, load

    check(load().asdpocs_poisson_noise_device(C.c_void_p(p_ptr), C.c_void_p(out_ptr),
                                              int(n), float(I0), int(seed),
                                              C.c_void_p(stream or None)))
