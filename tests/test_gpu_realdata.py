"""Real-data realism checks on the GPU (the fixture holds the reference's own
test data, extracted by tests/golden/make_realdata.py):

* utilities/test_asdpocs.m: the swine scan (1537 bins, 90 of its views, SOD
  405.941 / SDD 906.251 mm, 0.148 mm pitch) reconstructed on 512^2 with the
  driver's default options (5 iterations, alpha 0.02);
* demo_head190.m: the head slice as phantom, projected onto a 1024 x 2
  detector over 90 views of 180 degrees (a single-slice geometry with two
  detector rows), then reconstructed with its options for a few iterations.

The GPU runs the image in FP32 where the oracle keeps FP64; at the swine
settings a 1e-7 relative perturbation of the sinogram moves the FP64 result
by 4e-4, so the reconstructions are compared to 1e-2 and the data residual
to 1e-3 (the head slice's chaotic demo options are compared through their
RMSE trajectory)."""
import numpy as np
import pytest

import asd_pocs_mex_cuda_demo_gb300 as pkg
from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def _swine_para(d):
    sod, sdd, dt = (float(v) for v in d["swine_geo"])
    n, Uy = 512, 1537
    return dict(nx=n, ny=n, nz=1, SO=sod, OD=sdd - sod, vxlsize=sod / sdd * dt * Uy / n,
                detsize=dt, na=Uy, nb=1, phi_vec=np.arange(1, 91) * 4.0)


def test_swine_scan(gpu, oracle_mod):
    d = golden("realdata.npz")
    para = _swine_para(d)
    P = d["swine_P"].astype(np.float64)
    m, out = pkg.ASD_POCS_cuda(P, para)
    mo, oo = oracle_mod.asdpocs(P, para)
    assert out["IterationNum"] == oo["IterationNum"] == 5
    assert rel_l2(m.ravel(order="F"), mo) < 1e-2
    assert abs(out["dataTolerance"] / oo["dataTolerance"] - 1) < 1e-3
    assert m.min() >= 0.0


def test_head_slice_single_slice_geometry(gpu, oracle_mod):
    d = golden("realdata.npz")
    img = d["head190"].astype(np.float64)
    I3d = img / img.max()
    n = I3d.shape[0]
    sod, sdd, dt = 405.9410, 906.2510, 0.148
    Uy, Vz, nv = 2 * n, 2, 90
    para = dict(nx=n, ny=n, nz=1, SO=sod, OD=sdd - sod,
                vxlsize=sod / sdd * dt * Uy / n, detsize=dt, na=Uy, nb=Vz,
                phi_vec=np.arange(1, nv + 1) * (180.0 / nv))
    x = I3d.ravel(order="F").astype(np.float32)
    P = np.zeros((Uy * Vz, nv))
    for i, a in enumerate(para["phi_vec"]):
        p = dict(para, phi=-a / 180 * np.pi)
        y, _ = pkg.Ax_cone_gpu(x, p)
        g = oracle_mod.gateway_geometry(p["phi"], sod, sdd - sod, para["vxlsize"], dt, Uy, Vz)
        yo, _ = oracle_mod.ax(x, g, n, n, 1)
        assert rel_l2(y, yo) < 1e-5, a
        P[:, i] = y
    # the demo's options (alpha 0.2) are chaotic here: a 1e-7 relative
    # perturbation of P moves the FP64 image by 3e-2 but its RMSE trajectory
    # by 5e-4; at alpha 0.002 the image moves by 2e-4
    run = dict(para, maxnumIter=4, alpha=0.2, alpha_red=0.95, beta_red=1.0, I0=I3d)
    m, out = pkg.ASD_POCS_cuda(P, run)
    mo, oo = oracle_mod.asdpocs(P, run)
    assert rel_l2(m.ravel(order="F"), mo) < 1e-1
    np.testing.assert_allclose(out["RMSE"], oo["RMSE"], rtol=1e-2)
    assert out["RMSE"][-1] < out["RMSE"][0]
    run = dict(run, alpha=0.002)
    m, out = pkg.ASD_POCS_cuda(P, run)
    mo, oo = oracle_mod.asdpocs(P, run)
    assert rel_l2(m.ravel(order="F"), mo) < 1e-2
    np.testing.assert_allclose(out["RMSE"], oo["RMSE"], rtol=1e-3)
