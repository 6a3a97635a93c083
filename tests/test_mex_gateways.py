"""MATLAB-level drop-in: this repository's gateways compile against the mex
API and call the library; the reference's own Ax/Atx gateways link against
the library's launcher symbols (no source change)."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, golden, rel_l2

sys.path.insert(0, os.path.join(ROOT, "tests", "mex_gateways"))
import harness  # noqa: E402


@pytest.fixture(scope="module")
def gw(lib):
    so = harness.build_gateways()
    m = harness.Mex(so)
    look = C.CDLL(so).gw_lookup
    look.restype = C.c_void_p
    look.argtypes = [C.c_int]
    return m, {k: look(i) for i, k in enumerate(("tv2d", "tv3d", "asdpocs"))}


def test_gateways_build_and_link(gw):
    m, fns = gw
    assert all(fns.values())


def test_gateway_argument_errors_without_gpu(gw):
    m, fns = gw
    with pytest.raises(RuntimeError, match="Error usage"):
        m.call(fns["asdpocs"], [np.zeros((4, 2))], nlhs=2)
    with pytest.raises(RuntimeError, match="parameter.SO"):
        m.call(fns["asdpocs"], [np.zeros((4, 2)), dict(nx=2, ny=2, nz=1, na=4, nb=1)], nlhs=2)
    para = dict(nx=2, ny=2, nz=1, na=4, nb=1, SO=541.0, OD=408.0, vxlsize=1.0, detsize=1.0,
                phi_vec=[0.0, 90.0])
    # a sinogram with too few rows for na*nb rays per view is refused before
    # anything reads it (the reference fails on P(:,ii) - proj)
    with pytest.raises(RuntimeError, match="na\\*nb rows"):
        m.call(fns["asdpocs"], [np.zeros((3, 2)), para], nlhs=2)
    with pytest.raises(RuntimeError, match="real double matrix"):
        m.call(fns["asdpocs"], [np.zeros((4, 2), np.float32), para], nlhs=2)
    with pytest.raises(RuntimeError, match="phi_vec mismatch"):
        m.call(fns["asdpocs"], [np.zeros((4, 3)), para], nlhs=2)
    # m0 / I0 of the wrong size are refused, not silently ignored
    for name in ("m0", "I0"):
        with pytest.raises(RuntimeError, match=f"parameter.{name} must be"):
            m.call(fns["asdpocs"], [np.zeros((4, 2)), dict(para, **{name: np.ones(3)})],
                   nlhs=2)


@pytest.mark.skipif(not os.path.exists(os.path.join(harness.REF, "src", "AxAtx",
                                                    "Ax_main_test.cpp")),
                    reason="reference checkout not on this machine")
def test_reference_gateways_link_against_library(lib):
    so = harness.link_reference_gateways()  # --no-undefined: every symbol resolves
    assert os.path.exists(so)


@pytest.mark.gpu
def test_tv_gateways_on_gpu(gpu, gw, oracle_mod):
    m, fns = gw
    d = golden("tv.npz")
    (h,) = m.call(fns["tv2d"], [d["img2"], 0.2, 20, 1, d["old2"]])
    assert rel_l2(m.out(h), d["out2"]) < 1e-12
    (h,) = m.call(fns["tv3d"], [d["img3"], 0.2, 20, 1, d["old3"]])
    assert rel_l2(m.out(h), d["out3"]) < 1e-12


@pytest.mark.gpu
def test_asdpocs_gateway_on_gpu(gpu, gw):
    m, fns = gw
    d = golden("asdpocs.npz")
    n, na, SO, OD, vx, det = d["geo2"]
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=d["phi2"], maxnumIter=6, alpha=0.002, alpha_red=0.95,
                I0=d["x2"].reshape(-1, 1))
    h, o = m.call(fns["asdpocs"], [d["P2"], para], nlhs=2)
    img = m.out(h)
    assert img.shape == (int(n), int(n), 1)
    assert rel_l2(img.ravel(order="F"), d["m2s"]) < 2e-4
    assert int(m.field(o, "IterationNum").item()) == int(d["out2s"][0])
    np.testing.assert_allclose(m.field(o, "RMSE").ravel(), d["rmse2s"], rtol=1e-4)
