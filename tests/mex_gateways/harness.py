"""Builds and drives the MATLAB gateways against the stand-in mex API (test
infrastructure): this repository's gateways in asd_pocs_mex_cuda_demo_gb300/mex,
linked with the product library, and -- where the reference checkout exists
-- the reference's own Ax/Atx gateway sources linked against the product
library's launcher symbols."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
STUB = os.path.join(ROOT, "oracle", "mexstub")
GW = os.path.join(ROOT, "asd_pocs_mex_cuda_demo_gb300", "mex")
LIBDIR = os.path.join(ROOT, "asd_pocs_mex_cuda_demo_gb300", "lib")
OUT = os.path.join(HERE, "_build")
# the reference checkout: ASDPOCS_REFERENCE_DIR, else "reference" beside the repository
REF = os.environ.get("ASDPOCS_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT),
                                                                "reference")

GATEWAYS = [("imgTVGradMin_gb300.cpp", "gw_tv2d"), ("imgTVGradMin3D_gb300.cpp", "gw_tv3d"),
            ("ASD_POCS_gb300.cpp", "gw_asdpocs")]


def _cxx(args):
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-I", STUB, "-I",
                    os.path.join(ROOT, "include"), *args], check=True)


def build_gateways():
    os.makedirs(OUT, exist_ok=True)
    objs = []
    for src, name in GATEWAYS:
        o = os.path.join(OUT, name + ".o")
        _cxx([f"-DmexFunction={name}", "-c", os.path.join(GW, src), "-o", o])
        objs.append(o)
    for src in (os.path.join(STUB, "mexstub.cpp"), os.path.join(HERE, "gw_lookup.cpp")):
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        _cxx(["-c", src, "-o", o])
        objs.append(o)
    so = os.path.join(OUT, "libgw.so")
    _cxx(["-shared", "-o", so, *objs, "-L", LIBDIR, "-lasdpocs_gb300",
          f"-Wl,-rpath,{LIBDIR}"])
    return so


def link_reference_gateways():
    """The reference's Ax/Atx gateway sources, unmodified, linked against the
    product library (its launchers replace the reference's CUDA ones)."""
    so = os.path.join(OUT, "libref_gw.so")
    objs = []
    for src, name in (("Ax_main_test.cpp", "ref_mex_ax"), ("Atx_main_test.cpp", "ref_mex_atx")):
        o = os.path.join(OUT, name + ".o")
        _cxx([f"-DmexFunction={name}", "-c", os.path.join(REF, "src", "AxAtx", src), "-o", o])
        objs.append(o)
    o = os.path.join(OUT, "mexstub_ref.o")
    _cxx(["-c", os.path.join(STUB, "mexstub.cpp"), "-o", o])
    objs.append(o)
    _cxx(["-shared", "-Wl,--no-undefined", "-o", so, *objs, "-L", LIBDIR,
          "-lasdpocs_gb300", f"-Wl,-rpath,{LIBDIR}"])
    return so


class Mex:
    """Calls mexFunctions of a harness library through the stand-in API."""

    def __init__(self, so):
        L = C.CDLL(so)
        L.stub_numeric.restype = C.c_void_p
        L.stub_numeric.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_longlong)]
        L.stub_struct.restype = C.c_void_p
        L.stub_struct_set.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        L.stub_data.restype = C.c_void_p
        L.stub_data.argtypes = [C.c_void_p]
        L.stub_ndim.argtypes = [C.c_void_p]
        L.stub_dim.argtypes = [C.c_void_p, C.c_int]
        L.stub_dim.restype = C.c_longlong
        L.stub_class.argtypes = [C.c_void_p]
        L.stub_free.argtypes = [C.c_void_p]
        L.stub_get_field.restype = C.c_void_p
        L.stub_get_field.argtypes = [C.c_void_p, C.c_char_p]
        L.stub_call_fn.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.c_int,
                                   C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
        self.L = L

    def _mx(self, arr, cls):
        arr = np.asarray(arr)
        dims = arr.shape if arr.ndim >= 2 else (arr.size, 1)
        d = (C.c_longlong * len(dims))(*dims)
        h = self.L.stub_numeric(cls, len(dims), d)
        dt = np.float64 if cls == 1 else np.float32
        flat = np.ascontiguousarray(np.asarray(arr, dt).ravel(order="F"))
        C.memmove(self.L.stub_data(h), flat.ctypes.data, flat.nbytes)
        return h

    def out(self, h):
        cls = self.L.stub_class(h)
        dims = tuple(self.L.stub_dim(h, i) for i in range(self.L.stub_ndim(h)))
        dt = np.float64 if cls == 1 else np.float32
        n = int(np.prod(dims))
        buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(self.L.stub_data(h))
        return np.frombuffer(bytes(buf), dtype=dt).reshape(dims, order="F").copy()

    def field(self, h, name):
        f = self.L.stub_get_field(h, name.encode())
        return None if not f else self.out(f)

    def call(self, fn, args, nlhs=1):
        hs = []
        for a in args:
            if isinstance(a, dict):
                s = self.L.stub_struct()
                for k, v in a.items():
                    v = np.asarray(v, np.float64)
                    self.L.stub_struct_set(s, k.encode(), self._mx(
                        v.reshape(-1, 1) if v.ndim < 2 else v, 1))
                hs.append(s)
            elif isinstance(a, np.ndarray):
                hs.append(self._mx(a, 2 if a.dtype == np.float32 else 1))
            else:
                hs.append(self._mx(np.atleast_2d(np.float64(a)), 1))
        prhs = (C.c_void_p * len(hs))(*hs)
        plhs = (C.c_void_p * max(nlhs, 1))()
        err = C.create_string_buffer(512)
        rc = self.L.stub_call_fn(fn, nlhs, plhs, len(hs), prhs, err, 512)
        for h in hs:
            self.L.stub_free(h)
        if rc:
            raise RuntimeError(err.value.decode())
        return [plhs[i] for i in range(nlhs)]
