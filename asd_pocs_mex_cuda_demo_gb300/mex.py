"""MATLAB-level entry points, mirroring the reference's mex functions.

``Ax_cone_gpu`` / ``Atx_cone_gpu`` follow src/AxAtx/Ax_main_test.cpp and
Atx_main_test.cpp (argument checks, ``para`` fields, single-precision
outputs); ``imgTVGradMin`` / ``imgTVGradMin3D`` follow src/tvmin.  Arrays
follow MATLAB's column-major convention: an [nx, ny, nz] volume is a numpy
array of that shape read in Fortran order (or a flat x-fastest vector).
Every call runs on the GPU through the C ABI; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import AsdpocsError, Para, load

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)

GATEWAY_FIELDS = ("SO", "OD", "vxlsize", "nx", "ny", "nz", "phi", "detsize", "na", "nb")


class MexError(AsdpocsError):
    """The error a mex gateway raises through mexErrMsgTxt."""

    def __init__(self, msg: str):
        super().__init__(1, msg)


def check(rc: int):
    """Raise MexError (the gateway's mexErrMsgTxt) for a failed call."""
    if rc != 0:
        msg = load().asdpocs_last_error().decode(errors="replace")
        err = MexError(msg or f"asdpocs status {rc}")
        err.status = rc
        raise err


def _para(para) -> Para:
    if not isinstance(para, dict):
        raise MexError("Error usage!")
    # field order of the checks in Ax_main_test.cpp:48-126
    for f in GATEWAY_FIELDS:
        if f not in para or para[f] is None:
            raise MexError(f"Error input argument parameter.{f}!")
    p = Para()
    p.SO, p.OD, p.vxlsize = float(para["SO"]), float(para["OD"]), float(para["vxlsize"])
    p.detsize, p.phi = float(para["detsize"]), float(para["phi"])
    p.nx, p.ny, p.nz = int(para["nx"]), int(para["ny"]), int(para["nz"])
    p.na, p.nb = int(para["na"]), int(para["nb"])
    return p


def _flat_single(a) -> np.ndarray:
    a = np.asarray(a)
    # the gateways read the data as float* without a class check
    # (Ax_main_test.cpp:45); callers pass single
    return np.ascontiguousarray(a.ravel(order="F"), dtype=np.float32)


def Ax_cone_gpu(X, para, *extra):
    """[y, sr] = Ax_cone_gpu(single(X), para): forward projection of one view.

    Returns the projection ``y`` and the ray sums ``sr`` (row sums of the
    system matrix) as float32 vectors of length na*nb (ia fastest)."""
    if extra:
        raise MexError("Error usage!")
    p = _para(para)
    x = _flat_single(X)
    M = p.na * p.nb
    y = np.empty(M, np.float32)
    sr = np.empty(M, np.float32)
    check(load().Ax_cone_gpu(x.ctypes.data_as(_F), x.size, C.byref(p),
                             y.ctypes.data_as(_F), sr.ctypes.data_as(_F)))
    return y, sr


def Atx_cone_gpu(Y, para, *extra):
    """[x, sc] = Atx_cone_gpu(single(Y), para): backprojection of one view.

    Returns the backprojection ``x`` and the column sums ``sc`` as float32
    vectors of length nx*ny*nz (x fastest)."""
    if extra:
        raise MexError("Error usage!")
    p = _para(para)
    yv = _flat_single(Y)
    N = p.nx * p.ny * p.nz
    x = np.empty(N, np.float32)
    sc = np.empty(N, np.float32)
    check(load().Atx_cone_gpu(yv.ctypes.data_as(_F), yv.size, C.byref(p),
                              x.ctypes.data_as(_F), sc.ctypes.data_as(_F)))
    return x, sc


def adjoint_check(X, Y, para):
    """(<Ax, Y>, <X, A^T Y>) of the view described by para, accumulated in
    FP64 on the GPU: the two agree to the FP32 rounding of the projections."""
    p = _para(para)
    x = _flat_single(X)
    yv = _flat_single(Y)
    dots = np.zeros(2)
    check(load().asdpocs_adjoint_check_para(x.ctypes.data_as(_F), x.size,
                                            yv.ctypes.data_as(_F), yv.size, C.byref(p),
                                            dots.ctypes.data_as(_D)))
    return float(dots[0]), float(dots[1])


def _tv_args(I, I0, ndim):
    I = np.asarray(I)
    if I.dtype != np.float64:
        # imgTVGradMin.cpp:135-139 prints this and returns no output
        raise MexError("Invalid data format. Please make sure the input image data "
                       "is in double format.")
    if ndim == 2 and I.ndim == 1:
        I = I.reshape(-1, 1)
    if I.ndim != ndim:
        raise MexError(f"expected a {ndim}-D image")
    flat = np.ascontiguousarray(I.ravel(order="F"))
    old = None
    if I0 is not None:
        I0 = np.asarray(I0, np.float64)
        if ndim == 2 and I0.ndim == 1:
            I0 = I0.reshape(-1, 1)
        if I0.shape != I.shape:
            raise MexError("img0 dimensions do not match with img")
        old = np.ascontiguousarray(I0.ravel(order="F"))
    return I, flat, old


def imgTVGradMin(I, alpha, nTVIter, pos, I0=None):
    """I2 = imgTVGradMin(I, alpha, nTVIter, pos[, I0]): 2D TV steepest descent
    (FP64 on the GPU).  ``I`` is a double [rowN, colN] array."""
    I, flat, old = _tv_args(I, I0, 2)
    out = np.empty_like(flat)
    check(load().imgTVGradMin(flat.ctypes.data_as(_D), out.ctypes.data_as(_D),
                              I.shape[0], I.shape[1], float(alpha), int(nTVIter),
                              int(pos), None if old is None else old.ctypes.data_as(_D)))
    return out.reshape(I.shape, order="F")


def imgTVGradMin3D(I, alpha, nTVIter, pos, I0=None):
    """I2 = imgTVGradMin3D(I, alpha, nTVIter, pos[, I0]): 3D TV steepest
    descent (FP64 on the GPU).  ``I`` is a double [Nx, Ny, Nz] array."""
    I, flat, old = _tv_args(I, I0, 3)
    out = np.empty_like(flat)
    check(load().imgTVGradMin3D(flat.ctypes.data_as(_D), out.ctypes.data_as(_D),
                                I.shape[0], I.shape[1], I.shape[2], float(alpha),
                                int(nTVIter), int(pos),
                                None if old is None else old.ctypes.data_as(_D)))
    return out.reshape(I.shape, order="F")


def Ax_cone_mf_gpu_new(X, y, sr, cos_phi, sin_phi, y_det, z_det, SO, OD, scale, dz,
                       nx, ny, nz, na, nb):
    """Launcher-level forward projection into caller-owned float32 arrays
    (the C symbol of the same name; host memory, synchronous)."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (X, y_det, z_det)]
    for out in (y, sr):
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size < na * nb:
            raise ValueError("outputs must be contiguous float32 arrays of na*nb")
    L = load()
    L.Ax_cone_mf_gpu_new(arrs[0].ctypes.data_as(_F), y.ctypes.data_as(_F),
                         sr.ctypes.data_as(_F), cos_phi, sin_phi,
                         arrs[1].ctypes.data_as(_F), arrs[2].ctypes.data_as(_F), SO, OD,
                         scale, dz, nx, ny, nz, na, nb)
    check(L.asdpocs_last_status())


def Ax_siddon_mf_gpu(X, y, sr, cos_phi, sin_phi, y_det, z_det, SO, OD, scale, dz,
                     nx, ny, nz, na, nb):
    """Exact (Siddon) forward projection with Ax_cone_mf_gpu_new's arguments:
    the length of each ray inside every voxel it crosses (asdpocs_ax_siddon;
    host memory, synchronous)."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (X, y_det, z_det)]
    for out in (y, sr):
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size < na * nb:
            raise ValueError("outputs must be contiguous float32 arrays of na*nb")
    check(load().asdpocs_ax_siddon(arrs[0].ctypes.data_as(_F), y.ctypes.data_as(_F),
                                   sr.ctypes.data_as(_F), cos_phi, sin_phi,
                                   arrs[1].ctypes.data_as(_F), arrs[2].ctypes.data_as(_F),
                                   SO, OD, scale, dz, nx, ny, nz, na, nb))


def Atx_cone_mf_gpu_new(X, y, sc, cos_phi, sin_phi, y_det, z_det, SO, OD, scale, dy_det,
                        dz_det, dz, nx, ny, nz, na, nb):
    """Launcher-level backprojection: X, sc (outputs, nx*ny*nz float32) from
    the view y (the C symbol of the same name)."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (y, y_det, z_det)]
    for out in (X, sc):
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size < nx * ny * nz:
            raise ValueError("outputs must be contiguous float32 arrays of nx*ny*nz")
    L = load()
    L.Atx_cone_mf_gpu_new(X.ctypes.data_as(_F), arrs[0].ctypes.data_as(_F),
                          sc.ctypes.data_as(_F), cos_phi, sin_phi,
                          arrs[1].ctypes.data_as(_F), arrs[2].ctypes.data_as(_F), SO, OD,
                          scale, dy_det, dz_det, dz, nx, ny, nz, na, nb)
    check(L.asdpocs_last_status())
