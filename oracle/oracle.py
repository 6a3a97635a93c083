"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loaded only by tests/, ``__graft_entry__.smoke()`` and ``bench.py`` (its
``cpu_baseline`` leg and ``--impl reference`` arm), always as the checker or
the timed CPU baseline.  The product package never imports this module.

Two CPU implementations are bound here:

* ``liboracle``: the C restatement in ``asdpocs_oracle.c`` (built by
  ``build_oracle.sh``), available everywhere;
* ``libasdref``: the reference's own ``src/AxAtx`` and ``src/tvmin`` sources
  built for the host by ``build_ref.sh`` (only where the reference checkout
  exists; the golden vectors in ``tests/golden`` carry its results elsewhere).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libasdpocs_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libasdref.so")

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)


class AsdParams(C.Structure):
    """Mirror of ``orc_asd_params`` (ASD_POCS_cuda.m option set)."""

    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("na", C.c_int),
        ("nb", C.c_int), ("nv", C.c_int),
        ("SO", C.c_double), ("OD", C.c_double), ("vxlsize", C.c_double),
        ("detsize", C.c_double),
        ("maxnumIter", C.c_int), ("ng", C.c_int),
        ("alpha", C.c_double), ("alpha_red", C.c_double), ("beta", C.c_double),
        ("beta_red", C.c_double), ("r_max", C.c_double), ("epsilon", C.c_double),
        ("stopRelChg", C.c_double),
    ]


class AsdOut(C.Structure):
    _fields_ = [("iterations", C.c_int), ("dataTolerance", C.c_double),
                ("alpha", C.c_double), ("beta", C.c_double)]


_lib = None
_ref = None


def build():
    """Compile the oracle (and the reference host build when its sources exist)."""
    subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")],
                           check=True, stdout=subprocess.DEVNULL)
        _lib = C.CDLL(ORACLE_SO)
        _declare(_lib)
    return _lib


def ref_available() -> bool:
    """The reference host build exists here and loads (it is built only where
    the reference checkout is, and not for another machine's architecture)."""
    if not os.path.exists(REF_SO):
        return False
    try:
        C.CDLL(REF_SO)
    except OSError:
        return False
    return True


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference host build (oracle/_ref) not present")
        _ref = C.CDLL(REF_SO)
        _ref.stub_numeric.restype = C.c_void_p
        _ref.stub_numeric.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_longlong)]
        _ref.stub_struct.restype = C.c_void_p
        _ref.stub_struct_set.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        _ref.stub_data.restype = C.c_void_p
        _ref.stub_data.argtypes = [C.c_void_p]
        _ref.stub_ndim.argtypes = [C.c_void_p]
        _ref.stub_dim.argtypes = [C.c_void_p, C.c_int]
        _ref.stub_dim.restype = C.c_longlong
        _ref.stub_class.argtypes = [C.c_void_p]
        _ref.stub_free.argtypes = [C.c_void_p]
        _ref.stub_call.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_void_p), C.c_int,
                                   C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
        _ref.ref_set_threads.argtypes = [C.c_int]
        for name in ("Ax_cone_mf_gpu_new",):
            getattr(_ref, name).argtypes = [_F, _F, _F, C.c_float, C.c_float, _F, _F,
                                            C.c_float, C.c_float, C.c_float, C.c_float,
                                            C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _ref.Atx_cone_mf_gpu_new.argtypes = [_F, _F, _F, C.c_float, C.c_float, _F, _F,
                                             C.c_float, C.c_float, C.c_float, C.c_float,
                                             C.c_float, C.c_float, C.c_int, C.c_int,
                                             C.c_int, C.c_int, C.c_int]
    return _ref


def _declare(L):
    L.orc_ax.argtypes = [_F, _F, _F, C.c_float, C.c_float, _F, _F, C.c_float, C.c_float,
                         C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                         C.c_int, C.c_int]
    L.orc_atx.argtypes = [_F, _F, _F, C.c_float, C.c_float, _F, _F, C.c_float, C.c_float,
                          C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                          C.c_int, C.c_int, C.c_int, C.c_int]
    L.orc_tv2d.argtypes = [_D, _D, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, _D]
    L.orc_tv3d.argtypes = [_D, _D, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                           C.c_int, _D, C.c_int]
    L.orc_gateway_geometry.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_int, C.c_int, _F, _F, _F, _F,
                                       _F, _F, _F, _F]
    L.orc_siddon_ax_f64.argtypes = [_F, _D, _D, C.c_float, C.c_float, _F, _F, C.c_float,
                                    C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int]
    L.orc_siddon_atx_f64.argtypes = [_D, _D, _D, C.c_float, C.c_float, _F, _F,
                                     C.c_float, C.c_float, C.c_float, C.c_float,
                                     C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.orc_siddon_nnz.restype = C.c_longlong
    L.orc_siddon_nnz.argtypes = [C.c_float, C.c_float, _F, _F, C.c_float, C.c_float,
                                 C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    L.orc_asdpocs_with.argtypes = [_D, _D, C.POINTER(AsdParams), _D, _D, _D, _D,
                                   C.POINTER(AsdOut), C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_void_p]
    L.orc_sart.argtypes = [_D, _D, C.POINTER(AsdParams), C.c_double, _D, _D, _D, C.c_int]


def _fp(a):
    return a.ctypes.data_as(_F)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32).ravel(order="K")


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---------------------------------------------------------------- geometry
def gateway_geometry(phi, SO, OD, vxlsize, detsize, na, nb):
    """Launcher arguments the mex gateway derives from ``para``."""
    c, s, so, od, sc, det = (np.zeros(1, np.float32) for _ in range(6))
    yd = np.zeros(na, np.float32)
    zd = np.zeros(nb, np.float32)
    lib().orc_gateway_geometry(phi, SO, OD, vxlsize, detsize, na, nb, _fp(c), _fp(s),
                               _fp(so), _fp(od), _fp(sc), _fp(det), _fp(yd), _fp(zd))
    return dict(cos_phi=float(c[0]), sin_phi=float(s[0]), SO=float(so[0]),
                OD=float(od[0]), scale=float(sc[0]), det=float(det[0]),
                y_det=yd, z_det=zd)


# ---------------------------------------------------------------- projectors
def ax(x, g, nx, ny, nz, dz=1.0, nthreads=0):
    """Oracle Ax for launcher-level geometry ``g`` (see gateway_geometry)."""
    na, nb = len(g["y_det"]), len(g["z_det"])
    x = _f32(x)
    y = np.zeros(na * nb, np.float32)
    sr = np.zeros(na * nb, np.float32)
    lib().orc_ax(_fp(x), _fp(y), _fp(sr), g["cos_phi"], g["sin_phi"], _fp(_f32(g["y_det"])),
                 _fp(_f32(g["z_det"])), g["SO"], g["OD"], g["scale"], dz, nx, ny, nz, na,
                 nb, nthreads)
    return y, sr


def atx(yv, g, nx, ny, nz, dz=1.0, nthreads=0):
    na, nb = len(g["y_det"]), len(g["z_det"])
    yv = _f32(yv)
    x = np.zeros(nx * ny * nz, np.float32)
    sc = np.zeros(nx * ny * nz, np.float32)
    lib().orc_atx(_fp(x), _fp(yv), _fp(sc), g["cos_phi"], g["sin_phi"],
                  _fp(_f32(g["y_det"])), _fp(_f32(g["z_det"])), g["SO"], g["OD"],
                  g["scale"], g["det"], g["det"], dz, nx, ny, nz, na, nb, nthreads)
    return x, sc


def siddon_ax(x, g, nx, ny, nz, dz=1.0):
    na, nb = len(g["y_det"]), len(g["z_det"])
    x = _f32(x)
    y = np.zeros(na * nb)
    sr = np.zeros(na * nb)
    lib().orc_siddon_ax_f64(_fp(x), _dp(y), _dp(sr), g["cos_phi"], g["sin_phi"],
                            _fp(_f32(g["y_det"])), _fp(_f32(g["z_det"])), g["SO"], g["OD"],
                            g["scale"], dz, nx, ny, nz, na, nb)
    return y, sr


def siddon_atx(yv, g, nx, ny, nz, dz=1.0):
    na, nb = len(g["y_det"]), len(g["z_det"])
    yv = _f64(yv).ravel()
    x = np.zeros(nx * ny * nz)
    sc = np.zeros(nx * ny * nz)
    lib().orc_siddon_atx_f64(_dp(x), _dp(yv), _dp(sc), g["cos_phi"], g["sin_phi"],
                             _fp(_f32(g["y_det"])), _fp(_f32(g["z_det"])), g["SO"],
                             g["OD"], g["scale"], dz, nx, ny, nz, na, nb)
    return x, sc


def siddon_nnz(g, nx, ny, nz, dz=1.0):
    na, nb = len(g["y_det"]), len(g["z_det"])
    return int(lib().orc_siddon_nnz(g["cos_phi"], g["sin_phi"], _fp(_f32(g["y_det"])),
                                    _fp(_f32(g["z_det"])), g["SO"], g["OD"], dz, nx, ny,
                                    nz, na, nb))


# ---------------------------------------------------------------- TV
def tv(img, alpha, n_iter, pos, img_old=None, nthreads=0):
    """imgTVGradMin (2D array) / imgTVGradMin3D (3D array), MATLAB column-major
    semantics: ``img`` is indexed [x, y(, z)] with x fastest (pass Fortran
    order or a flat vector with explicit shape)."""
    img = np.asarray(img, dtype=np.float64)
    shape = img.shape
    flat = np.ascontiguousarray(img.ravel(order="F"))
    old = None if img_old is None else np.ascontiguousarray(
        np.asarray(img_old, np.float64).ravel(order="F"))
    out = np.zeros_like(flat)
    if len(shape) == 2:
        lib().orc_tv2d(_dp(flat), _dp(out), shape[0], shape[1], alpha, n_iter, pos, _dp(old))
    else:
        lib().orc_tv3d(_dp(flat), _dp(out), shape[0], shape[1], shape[2], alpha, n_iter,
                       pos, _dp(old), nthreads)
    return out.reshape(shape, order="F")


# ---------------------------------------------------------------- drivers
def make_params(para: dict, nv: int) -> AsdParams:
    """Defaults of ASD_POCS_cuda.m:20-96 for absent fields."""
    p = AsdParams()
    p.nx, p.ny, p.nz = int(para["nx"]), int(para["ny"]), int(para["nz"])
    p.na, p.nb, p.nv = int(para["na"]), int(para["nb"]), int(nv)
    p.SO, p.OD = float(para["SO"]), float(para["OD"])
    p.vxlsize, p.detsize = float(para["vxlsize"]), float(para["detsize"])
    eps = float(np.finfo(np.float64).eps)
    p.maxnumIter = int(para.get("maxnumIter", 5))
    p.ng = int(para.get("numOfgradients", 20))
    p.alpha = float(para.get("alpha", 0.02))
    p.alpha_red = float(para.get("alpha_red", 0.95))
    p.beta = float(para.get("beta", 1.0))
    p.beta_red = float(para.get("beta_red", 0.995))
    p.r_max = float(para.get("r_max", 0.95))
    p.epsilon = float(para.get("epsilon", eps))
    p.stopRelChg = float(para.get("stopRelChg", eps))
    return p


def asdpocs(P, para, impl="oracle", nthreads=0):
    """ASD_POCS_cuda(P, para) with FP64 image state.  ``impl`` selects the
    projector/TV code: ``"oracle"`` (restatement), ``"reference"`` (the
    reference's host build) or ``"siddon"`` (the restatement with the FP64
    Siddon forward projection, the oracle of the exact forward mode).
    Returns (m_res flat, out dict)."""
    P = np.asfortranarray(np.asarray(P, np.float64))
    nv = P.shape[1]
    phi = _f64(np.asarray(para["phi_vec"], np.float64).ravel())
    if phi.size != nv:
        raise ValueError("Size of Projection and phi_vec mismatch!")
    p = make_params(para, nv)
    N = p.nx * p.ny * p.nz
    Pflat = np.ascontiguousarray(P.ravel(order="F"))
    m0 = para.get("m0")
    m0 = None if m0 is None else _f64(np.asarray(m0).ravel(order="F"))
    I0 = para.get("I0")
    I0 = None if I0 is None else _f64(np.asarray(I0).ravel(order="F"))
    m_res = np.zeros(N)
    rmse = np.zeros(max(p.maxnumIter, 1))
    out = AsdOut()
    fns = (None, None, None)
    if impl == "reference":
        R = ref()
        fns = tuple(C.cast(getattr(R, n), C.c_void_p)
                    for n in ("ref_ax_for_driver", "ref_atx_for_driver", "ref_tv_for_driver"))
    elif impl == "siddon":
        fns = (C.cast(lib().orc_ax_siddon_for_driver, C.c_void_p), None, None)
    lib().orc_asdpocs_with(_dp(Pflat), _dp(phi), C.byref(p), _dp(m0), _dp(I0), _dp(m_res),
                           _dp(rmse), C.byref(out), nthreads, *fns)
    res = dict(IterationNum=out.iterations, dataTolerance=out.dataTolerance,
               alpha=out.alpha, beta=out.beta)
    if I0 is not None:
        res["RMSE"] = rmse[:out.iterations].copy()
    return m_res, res


def sart(P, para, nthreads=0):
    """SART_cuda_inline(P, para): one sweep, relaxation para.lambda (default 1)."""
    P = np.asfortranarray(np.asarray(P, np.float64))
    nv = P.shape[1]
    phi = _f64(np.asarray(para["phi_vec"], np.float64).ravel())
    p = make_params(para, nv)
    N = p.nx * p.ny * p.nz
    m0 = para.get("m0")
    m0 = None if m0 is None else _f64(np.asarray(m0).ravel(order="F"))
    m = np.zeros(N)
    dt = np.zeros(1)
    lib().orc_sart(_dp(np.ascontiguousarray(P.ravel(order="F"))), _dp(phi), C.byref(p),
                   float(para.get("lambda", 1.0)), _dp(m0), _dp(m), _dp(dt), nthreads)
    return m, float(dt[0])


# ---------------------------------------------------------------- reference host build
def ref_launch_ax(x, g, nx, ny, nz, dz=1.0, nthreads=0):
    """The reference's Ax kernel (host build) through its launcher signature."""
    R = ref()
    R.ref_set_threads(nthreads)
    na, nb = len(g["y_det"]), len(g["z_det"])
    x = _f32(x).copy()
    y = np.zeros(na * nb, np.float32)
    sr = np.zeros(na * nb, np.float32)
    R.Ax_cone_mf_gpu_new(_fp(x), _fp(y), _fp(sr), g["cos_phi"], g["sin_phi"],
                         _fp(_f32(g["y_det"]).copy()), _fp(_f32(g["z_det"]).copy()),
                         g["SO"], g["OD"], g["scale"], dz, nx, ny, nz, na, nb)
    return y, sr


def ref_launch_atx(yv, g, nx, ny, nz, dz=1.0, nthreads=0):
    R = ref()
    R.ref_set_threads(nthreads)
    na, nb = len(g["y_det"]), len(g["z_det"])
    yv = _f32(yv).copy()
    x = np.zeros(nx * ny * nz, np.float32)
    sc = np.zeros(nx * ny * nz, np.float32)
    R.Atx_cone_mf_gpu_new(_fp(x), _fp(yv), _fp(sc), g["cos_phi"], g["sin_phi"],
                          _fp(_f32(g["y_det"]).copy()), _fp(_f32(g["z_det"]).copy()),
                          g["SO"], g["OD"], g["scale"], g["det"], g["det"], dz, nx, ny,
                          nz, na, nb)
    return x, sc


_MX_DOUBLE, _MX_SINGLE = 1, 2


def _mx(R, arr, cls):
    arr = np.asarray(arr)
    dims = arr.shape if arr.ndim >= 2 else (arr.size, 1)
    d = (C.c_longlong * len(dims))(*dims)
    h = R.stub_numeric(cls, len(dims), d)
    dt = np.float64 if cls == _MX_DOUBLE else np.float32
    flat = np.ascontiguousarray(np.asarray(arr, dt).ravel(order="F"))
    C.memmove(R.stub_data(h), flat.ctypes.data, flat.nbytes)
    return h


def _mx_out(R, h):
    cls = R.stub_class(h)
    dims = tuple(R.stub_dim(h, i) for i in range(R.stub_ndim(h)))
    dt = np.float64 if cls == _MX_DOUBLE else np.float32
    n = int(np.prod(dims))
    buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(R.stub_data(h))
    return np.frombuffer(bytes(buf), dtype=dt).reshape(dims, order="F").copy()


def ref_mex(which: str, args, nlhs=1, nthreads=0):
    """Call a reference mexFunction through the stand-in MATLAB API.

    ``which``: 'Ax_cone_gpu' | 'Atx_cone_gpu' | 'imgTVGradMin' | 'imgTVGradMin3D'.
    ``args``: numpy arrays (single for projector data, double otherwise),
    Python numbers (double scalars) or dicts (the para struct).
    Raises RuntimeError with the mexErrMsgTxt message on a gateway error.
    """
    R = ref()
    R.ref_set_threads(nthreads)
    ids = {"Ax_cone_gpu": 0, "Atx_cone_gpu": 1, "imgTVGradMin": 2, "imgTVGradMin3D": 3}
    handles = []
    for a in args:
        if isinstance(a, dict):
            s = R.stub_struct()
            for k, v in a.items():
                R.stub_struct_set(s, k.encode(), _mx(R, np.atleast_2d(np.float64(v)), _MX_DOUBLE))
            handles.append(s)
        elif isinstance(a, np.ndarray):
            cls = _MX_SINGLE if a.dtype == np.float32 else _MX_DOUBLE
            handles.append(_mx(R, a, cls))
        else:
            handles.append(_mx(R, np.atleast_2d(np.float64(a)), _MX_DOUBLE))
    prhs = (C.c_void_p * len(handles))(*handles)
    plhs = (C.c_void_p * max(nlhs, 1))()
    err = C.create_string_buffer(512)
    rc = R.stub_call(ids[which], nlhs, plhs, len(handles), prhs, err, 512)
    try:
        if rc != 0:
            raise RuntimeError(err.value.decode())
        outs = [None if not plhs[i] else _mx_out(R, plhs[i]) for i in range(nlhs)]
    finally:
        for h in handles:
            R.stub_free(h)
        for i in range(nlhs):
            if plhs[i]:
                R.stub_free(plhs[i])
    return outs
