"""The kernels' projector math (csrc/projector.cuh), compiled for the host,
against the oracle -- checks the float logic of the GPU code without a GPU.

* Atx through the staged ray tables is bit-identical to the oracle (and so
  to the reference), planar and 3D, over the reference's whole footprint
  window and over each voxel's shadow only (the kernels' narrowing); so is
  2-D Atx read back from a chord table in the layout of the plans' tables.
* Ax with one partial sum per ray and the reference's weight expressions is
  bit-identical; with the 32-lane split and xor-butterfly combination of the
  warp kernels, and their division-free weights, it stays within 1e-6.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2

SRC = os.path.join(ROOT, "tests", "device_math", "dm_host.cu")
SO_PATH = os.path.join(ROOT, "tests", "device_math", "_build", "libdm_host.so")


@pytest.fixture(scope="module")
def dm():
    os.makedirs(os.path.dirname(SO_PATH), exist_ok=True)
    stale = (not os.path.exists(SO_PATH)) or any(
        os.path.getmtime(p) > os.path.getmtime(SO_PATH)
        for p in (SRC, os.path.join(ROOT, "asd_pocs_mex_cuda_demo_gb300", "csrc",
                                    "projector.cuh")))
    if stale:
        subprocess.run(["nvcc", "-O2", "-std=c++17", "-shared", "-Xcompiler",
                        "-fPIC,-ffp-contract=off", "-o", SO_PATH, SRC], check=True)
    L = C.CDLL(SO_PATH)
    F = C.POINTER(C.c_float)
    L.dm_ax.argtypes = [F, F, F, C.c_float, C.c_float, F, F, C.c_float, C.c_float,
                        C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                        C.c_int, C.c_int]
    L.dm_atx.argtypes = [F, F, F, C.c_float, C.c_float, F, F, C.c_float, C.c_float,
                         C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                         C.c_int, C.c_int, C.c_int, C.c_int]
    L.dm_atx3_zcol.argtypes = [F, F, F, C.c_float, C.c_float, F, F, C.c_float, C.c_float,
                               C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                               C.c_int, C.c_int, C.c_int]
    L.dm_ax_siddon.argtypes = [F, F, F, C.c_float, C.c_float, F, F, C.c_float, C.c_float,
                               C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                               C.c_int, C.c_int]
    L.dm_chord_count.argtypes = [C.c_float, C.c_float, F, C.c_float, C.c_float, C.c_float,
                                 C.c_int, C.c_int, C.c_int]
    L.dm_chord_count.restype = C.c_int
    L.dm_atx_table.argtypes = [F, F, F, C.c_float, C.c_float, F, C.c_float, C.c_float,
                               C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int]
    L.dm_atx_table.restype = C.c_int
    return L


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


CASES = [
    (64, 64, 1, 128, 1, 541.0, 408.0, 1.0),
    (17, 23, 1, 41, 1, 541.0, 408.0, 1.0),
    (40, 40, 1, 80, 2, 405.941, 500.31, 0.6),
    (24, 20, 12, 48, 24, 1000.0, 500.0, 3.2),
    (13, 11, 7, 27, 9, 300.0, 200.0, 1.3),
    # cone beam shaped like 256^3 / 512^2 detector at 0.8 mm, SID 1000 / SDD 1500
    # mm, scaled down (same magnification and bins per voxel)
    (32, 32, 32, 64, 64, 1000.0, 500.0, 0.8 * 256 / 32),
    (31, 33, 9, 60, 20, 1000.0, 500.0, 6.0),
]


@pytest.mark.parametrize("case", CASES, ids=[str(c[:5]) for c in CASES])
def test_device_math_matches_oracle(dm, oracle_mod, case):
    nx, ny, nz, na, nb, SO, OD, det = case
    rng = np.random.default_rng(nx + 7 * nz)
    vx = SO / (SO + OD) * det * na / nx
    x = rng.random(nx * ny * nz).astype(np.float32)
    yv = rng.standard_normal(na * nb).astype(np.float32)
    for a in [0.0, 45.0, 90.0, 135.0, 180.0, 270.0] + rng.uniform(0, 360, 6).tolist():
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb)
        yd, zd = g["y_det"].copy(), g["z_det"].copy()
        yo, so = oracle_mod.ax(x, g, nx, ny, nz)
        bo, co = oracle_mod.atx(yv, g, nx, ny, nz)
        outs = {}
        for lanes, exact in ((1, 1), (32, 1), (32, 0), (32, 2)):
            y = np.zeros(na * nb, np.float32)
            sr = np.zeros(na * nb, np.float32)
            dm.dm_ax(_p(x), _p(y), _p(sr), g["cos_phi"], g["sin_phi"], _p(yd), _p(zd),
                     g["SO"], g["OD"], g["scale"], 1.0, nx, ny, nz, na, nb, lanes, exact)
            outs[exact] = (y, sr)
            if lanes == 1:
                assert np.array_equal(y, yo) and np.array_equal(sr, so), a
            else:
                assert rel_l2(y, yo) < 1e-6 and rel_l2(sr, so) < 1e-6, (a, exact)
        # the grouped, branch-free column march is the per-column one, bit for bit
        assert np.array_equal(outs[0][0], outs[2][0]) and np.array_equal(outs[0][1], outs[2][1])
        for staged in (0, 1, 2):
            b = np.zeros(nx * ny * nz, np.float32)
            sc = np.zeros(nx * ny * nz, np.float32)
            dm.dm_atx(_p(b), _p(yv), _p(sc), g["cos_phi"], g["sin_phi"], _p(yd), _p(zd),
                      g["SO"], g["OD"], g["scale"], g["det"], g["det"], 1.0, nx, ny, nz,
                      na, nb, staged)
            assert np.array_equal(b, bo) and np.array_equal(sc, co), (a, staged)


@pytest.mark.parametrize("dims", [(48, 40, 1, 96, 1), (24, 20, 12, 48, 24)])
def test_narrowing_off_grid_detector(dm, oracle_mod, dims):
    """Detector coordinates off the uniform grid turn the shadow narrowing
    off; the result stays bit-identical to the oracle."""
    nx, ny, nz, na, nb = dims
    SO, OD, det = 541.0, 408.0, 1.0
    rng = np.random.default_rng(nx * nz)
    vx = SO / (SO + OD) * det * na / nx
    yv = rng.standard_normal(na * nb).astype(np.float32)
    for a in (17.0, 133.0, 251.0):
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb)
        yd = (g["y_det"] + rng.uniform(-0.3, 0.3, na) * g["det"]).astype(np.float32)
        zd = (g["z_det"] * (1.07 if nb > 1 else 1.0)).astype(np.float32)
        g["y_det"], g["z_det"] = yd, zd
        bo, co = oracle_mod.atx(yv, g, nx, ny, nz)
        b = np.zeros(nx * ny * nz, np.float32)
        sc = np.zeros(nx * ny * nz, np.float32)
        dm.dm_atx(_p(b), _p(yv), _p(sc), g["cos_phi"], g["sin_phi"], _p(yd), _p(zd),
                  g["SO"], g["OD"], g["scale"], g["det"], g["det"], 1.0, nx, ny, nz, na, nb,
                  2)
        assert np.array_equal(b, bo) and np.array_equal(sc, co), a


@pytest.mark.parametrize("dims", [(64, 64, 128), (17, 23, 41), (50, 31, 77)])
def test_chord_table_layout_matches_oracle(dm, oracle_mod, dims):
    """The 2-D chord table (header, chord sum, slot planes), filled from each
    voxel's shadow and read back in slot order, gives the oracle's Atx and
    chord sums bit for bit; views with an axis-parallel ray have none."""
    nx, ny, na = dims
    SO, OD, det = 541.0, 408.0, 1.0
    vx = SO / (SO + OD) * det * na / nx
    yv = np.random.default_rng(na).standard_normal(na).astype(np.float32)
    tables = 0
    for a in (0.0, 30.0, 45.0, 90.0, 200.0, 333.3):
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, 1)
        yd = g["y_det"].copy()
        K = dm.dm_chord_count(g["cos_phi"], g["sin_phi"], _p(yd), g["SO"], g["OD"],
                              g["det"], nx, ny, na)
        if K == 0:  # an axis-parallel central ray (odd na at 0 and 90 degrees)
            assert na % 2 == 1 and a in (0.0, 90.0)
            continue
        tables += 1
        bo, co = oracle_mod.atx(yv, g, nx, ny, 1)
        b = np.zeros(nx * ny, np.float32)
        sc = np.zeros(nx * ny, np.float32)
        assert dm.dm_atx_table(_p(b), _p(yv), _p(sc), g["cos_phi"], g["sin_phi"], _p(yd),
                               g["SO"], g["OD"], g["scale"], g["det"], nx, ny, na, K) == 0
        assert np.array_equal(b, bo) and np.array_equal(sc, co), a
        # one slot fewer than the largest count does not hold every voxel
        assert dm.dm_atx_table(_p(b), _p(yv), _p(sc), g["cos_phi"], g["sin_phi"], _p(yd),
                               g["SO"], g["OD"], g["scale"], g["det"], nx, ny, na,
                               K - 1) == -1
    assert tables >= 4


def test_chord_slots_of_the_512_fan_beam_protocol(dm, oracle_mod):
    """512^2 voxels of 0.9887 mm, 888 bins of 1 mm, SID 541 / SDD 949 mm, 60
    views: the largest number of pairs of a voxel is 8, the slots (and the
    600 MB of tables) that the GPU plan builds for this protocol."""
    nx = ny = 512
    na, SO, OD, det, vx = 888, 541.0, 408.0, 1.0, 0.9887
    K = 0
    for a in np.arange(1, 61) * 6.0:
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, 1)
        yd = g["y_det"].copy()
        K = max(K, dm.dm_chord_count(g["cos_phi"], g["sin_phi"], _p(yd), g["SO"], g["OD"],
                                     g["det"], nx, ny, na))
    assert K == 8
    assert (2 + K) * nx * ny * 60 * 4 / 2**20 == 600.0


@pytest.mark.parametrize("case", [c for c in CASES if c[2] > 1], ids=lambda c: str(c[:5]))
def test_cone_beam_z_column_walk_matches_oracle(dm, oracle_mod, case):
    """The cone-beam backward step walked down each voxel column, with the
    window's and shadow's columns, the corners' magnifications and the
    in-plane face tests computed once per column, gives the oracle's Atx
    and chord sums bit for bit (the form planned for the cone-beam kernel)."""
    nx, ny, nz, na, nb, SO, OD, det = case
    rng = np.random.default_rng(3 * nx + nz)
    vx = SO / (SO + OD) * det * na / nx
    yv = rng.standard_normal(na * nb).astype(np.float32)
    for a in [0.0, 45.0, 90.0, 200.0] + rng.uniform(0, 360, 4).tolist():
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb)
        yd, zd = g["y_det"].copy(), g["z_det"].copy()
        bo, co = oracle_mod.atx(yv, g, nx, ny, nz)
        b = np.zeros(nx * ny * nz, np.float32)
        sc = np.zeros(nx * ny * nz, np.float32)
        dm.dm_atx3_zcol(_p(b), _p(yv), _p(sc), g["cos_phi"], g["sin_phi"], _p(yd), _p(zd),
                        g["SO"], g["OD"], g["scale"], g["det"], g["det"], 1.0, nx, ny, nz,
                        na, nb)
        assert np.array_equal(b, bo) and np.array_equal(sc, co), a


@pytest.mark.parametrize("case", CASES, ids=lambda c: str(c[:5]))
def test_exact_siddon_columns_match_fp64_siddon(dm, oracle_mod, case):
    """The exact forward mode's device math (FP64 crossing parameters, FP32
    lengths and sums, columns over 32 lanes) against the oracle's FP64
    Siddon projector, in 2-D and 3-D; in 3-D the reference's own march
    deviates from these by about 1e-3."""
    nx, ny, nz, na, nb, SO, OD, det = case
    rng = np.random.default_rng(7 * nx + nz)
    vx = SO / (SO + OD) * det * na / nx
    x = rng.random(nx * ny * nz).astype(np.float32)
    for a in [0.0, 45.0, 90.0, 200.0] + rng.uniform(0, 360, 4).tolist():
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb)
        yd, zd = g["y_det"].copy(), g["z_det"].copy()
        ye, se = oracle_mod.siddon_ax(x, g, nx, ny, nz)
        y = np.zeros(na * nb, np.float32)
        sr = np.zeros(na * nb, np.float32)
        dm.dm_ax_siddon(_p(x), _p(y), _p(sr), g["cos_phi"], g["sin_phi"], _p(yd), _p(zd),
                        g["SO"], g["OD"], g["scale"], 1.0, nx, ny, nz, na, nb, 32)
        assert rel_l2(y, ye) <= 2e-6, (a, rel_l2(y, ye))
        assert rel_l2(sr, se) <= 2e-6, (a, rel_l2(sr, se))
