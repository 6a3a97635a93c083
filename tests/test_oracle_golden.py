"""The CPU oracle against the golden vectors made by the reference's own code
(src/AxAtx gateways + kernels, src/tvmin), and against the reference host
build itself where it is present."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel_l2

PROJ = sorted(glob.glob(os.path.join(GOLDEN, "proj_*.npz")))


def _geo(oracle, d, a):
    nx, ny, nz, na, nb = (int(v) for v in d["dims"])
    SO, OD, vx, det = d["geo"]
    g = oracle.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb)
    return g, nx, ny, nz


@pytest.mark.parametrize("path", PROJ, ids=[os.path.basename(p) for p in PROJ])
def test_oracle_projectors_bit_exact_vs_reference_vectors(oracle_mod, path):
    d = np.load(path)
    for k, a in enumerate(d["angles"]):
        g, nx, ny, nz = _geo(oracle_mod, d, a)
        # the gateway conversion reproduces the reference's cos/sin
        assert np.float32(g["cos_phi"]) == d["trig"][k, 0]
        assert np.float32(g["sin_phi"]) == d["trig"][k, 1]
        y, sr = oracle_mod.ax(d["x"], g, nx, ny, nz)
        b, sc = oracle_mod.atx(d["yview"], g, nx, ny, nz)
        assert np.array_equal(y, d["y"][k]), (a, rel_l2(y, d["y"][k]))
        assert np.array_equal(sr, d["sr"][k])
        assert np.array_equal(b, d["bp"][k]), (a, rel_l2(b, d["bp"][k]))
        assert np.array_equal(sc, d["sc"][k])


def test_oracle_tv_vs_reference_vectors(oracle_mod):
    d = golden("tv.npz")
    out2 = oracle_mod.tv(d["img2"], 0.2, 20, 1, d["old2"])
    assert rel_l2(out2, d["out2"]) < 1e-13
    out2b = oracle_mod.tv(d["img2"] - 0.5, 0.05, 7, 0)
    assert rel_l2(out2b, d["out2_nopos"]) < 1e-13
    assert (out2b < 0).any()  # pos=0 keeps negatives
    out3 = oracle_mod.tv(d["img3"], 0.2, 20, 1, d["old3"])
    assert rel_l2(out3, d["out3"]) < 1e-13


def test_oracle_asdpocs_vs_reference_driven_vectors(oracle_mod):
    d = golden("asdpocs.npz")
    n, na, SO, OD, vx, det = d["geo2"]
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=int(n), ny=int(n), nz=1, na=int(na), nb=1,
                detsize=det, phi_vec=d["phi2"], maxnumIter=6, alpha=0.2, alpha_red=0.95,
                I0=d["x2"])
    m, out = oracle_mod.asdpocs(d["P2"], para)
    assert np.array_equal(m, d["m2"])
    assert out["IterationNum"] == int(d["out2"][0])
    np.testing.assert_allclose([out["dataTolerance"], out["alpha"], out["beta"]],
                               d["out2"][1:], rtol=1e-14)
    np.testing.assert_allclose(out["RMSE"], d["rmse2"], rtol=1e-14)
    n3, na3, nb3, SO3, OD3, vx3, det3 = d["geo3"]
    para3 = dict(SO=SO3, OD=OD3, vxlsize=vx3, nx=int(n3), ny=int(n3), nz=int(n3),
                 na=int(na3), nb=int(nb3), detsize=det3, phi_vec=d["phi3"], maxnumIter=4,
                 alpha=0.2, I0=d["x3"])
    m3, out3 = oracle_mod.asdpocs(d["P3"], para3)
    assert np.array_equal(m3, d["m3"])
    np.testing.assert_allclose(out3["RMSE"], d["rmse3"], rtol=1e-14)


needs_ref = pytest.mark.skipif(
    not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                    "libasdref.so")),
    reason="reference host build (oracle/_ref) not present on this machine")


@needs_ref
@pytest.mark.parametrize("case", [
    (64, 64, 1, 128, 1, 541.0, 408.0, 1.0),
    (31, 20, 1, 77, 1, 541.0, 408.0, 1.0),
    (20, 20, 9, 40, 18, 1000.0, 500.0, 4.0),
    (16, 16, 1, 40, 2, 405.9, 500.3, 0.6),
])
def test_oracle_vs_reference_host_build_random(oracle_mod, case):
    nx, ny, nz, na, nb, SO, OD, det = case
    rng = np.random.default_rng(nx * 1000 + nz)
    vx = SO / (SO + OD) * det * na / nx
    x = rng.random(nx * ny * nz).astype(np.float32)
    yv = rng.standard_normal(na * nb).astype(np.float32)
    for a in rng.uniform(0, 360, size=12).tolist() + [0.0, 90.0, 180.0, 270.0, 45.0]:
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb)
        y1, s1 = oracle_mod.ax(x, g, nx, ny, nz)
        y2, s2 = oracle_mod.ref_launch_ax(x, g, nx, ny, nz)
        b1, c1 = oracle_mod.atx(yv, g, nx, ny, nz)
        b2, c2 = oracle_mod.ref_launch_atx(yv, g, nx, ny, nz)
        assert np.array_equal(y1, y2) and np.array_equal(s1, s2), a
        assert np.array_equal(b1, b2) and np.array_equal(c1, c2), a


@needs_ref
def test_reference_gateway_errors(oracle_mod):
    para = dict(SO=541., OD=408., vxlsize=1.1, nx=8, ny=8, nz=1, phi=0.1, detsize=1.0,
                na=16, nb=1)
    with pytest.raises(RuntimeError, match="Error size of input argument X!"):
        oracle_mod.ref_mex("Ax_cone_gpu", [np.zeros((10, 1), np.float32), para], nlhs=2)
    bad = dict(para)
    del bad["OD"]
    with pytest.raises(RuntimeError, match="parameter.OD"):
        oracle_mod.ref_mex("Ax_cone_gpu", [np.zeros((64, 1), np.float32), bad], nlhs=2)
