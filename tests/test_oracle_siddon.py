"""Known answers for the projector restatement: exact FP64 Siddon in 2D,
adjointness, the central-ray length, and the documented 3D deviation."""
import numpy as np
import pytest

from conftest import rel_l2


def _geom(oracle, a, n=256, na=512, SO=541.0, OD=408.0, det=1.0, nb=1):
    vx = SO / (SO + OD) * det * na / n
    return oracle.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb), vx


@pytest.mark.parametrize("angle", [0, 17, 30, 45, 60, 123])
def test_ax_2d_is_exact_siddon(oracle_mod, angle):
    n = 128
    g, _ = _geom(oracle_mod, angle, n=n, na=256)
    x = np.random.default_rng(angle).random(n * n).astype(np.float32)
    y, sr = oracle_mod.ax(x, g, n, n, 1)
    ye, sre = oracle_mod.siddon_ax(x, g, n, n, 1)
    assert rel_l2(y, ye) < 5e-6
    assert rel_l2(sr, sre) < 5e-6


def test_central_ray_length(oracle_mod):
    # a ray through the centre of a uniform n x n image has length n voxels
    n = 256
    g, vx = _geom(oracle_mod, 0, n=n, na=511)  # odd na: bin 255 is centred
    y, sr = oracle_mod.ax(np.ones(n * n, np.float32), g, n, n, 1)
    assert abs(sr[255] / vx - n) < 1e-3


@pytest.mark.parametrize("angle", [30, 45, 123])
def test_adjointness_2d(oracle_mod, angle):
    n = 96
    g, _ = _geom(oracle_mod, angle, n=n, na=200)
    rng = np.random.default_rng(7)
    x = rng.random(n * n).astype(np.float32)
    yv = rng.random(200).astype(np.float32)
    Ax, _ = oracle_mod.ax(x, g, n, n, 1)
    Aty, _ = oracle_mod.atx(yv, g, n, n, 1)
    lhs = float(np.dot(Ax.astype(np.float64), yv))
    rhs = float(np.dot(x.astype(np.float64), Aty))
    assert abs(lhs - rhs) / abs(lhs) < 2e-5


def test_atx_degenerate_drops(oracle_mod):
    # documented reference behaviour: at some angles (45 deg here) voxels lose
    # a ray in Atx (a corner hit is counted twice by the face tests), so Atx
    # differs from the exact transpose there; at generic angles it agrees
    n = 128
    rng = np.random.default_rng(1)
    yv = rng.random(256).astype(np.float32)
    errs = {}
    for a in (0, 30, 45, 123):
        g, _ = _geom(oracle_mod, a, n=n, na=256)
        b, _ = oracle_mod.atx(yv, g, n, n, 1)
        be, _ = oracle_mod.siddon_atx(yv.astype(np.float64), g, n, n, 1)
        errs[a] = rel_l2(b, be)
    assert max(errs[0], errs[30], errs[123]) < 1e-4
    assert errs[45] > 1e-3


def test_3d_ax_deviates_from_exact_siddon(oracle_mod):
    # documented reference behaviour: the 3D column split is approximate
    n, na, nb = 32, 64, 64
    g, _ = _geom(oracle_mod, 30, n=n, na=na, SO=1000.0, OD=500.0, det=0.8 * 4, nb=nb)
    x = np.random.default_rng(3).random(n ** 3).astype(np.float32)
    y, sr = oracle_mod.ax(x, g, n, n, n)
    ye, sre = oracle_mod.siddon_ax(x, g, n, n, n)
    e = rel_l2(y, ye)
    assert 1e-5 < e < 1e-2
    assert rel_l2(sr, sre) < 1e-3  # total lengths stay right


def test_siddon_nnz_scale(oracle_mod):
    g, _ = _geom(oracle_mod, 30, n=64, na=128)
    nnz = oracle_mod.siddon_nnz(g, 64, 64, 1)
    assert 64 * 128 < nnz < 3 * 64 * 128
