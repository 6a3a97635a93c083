"""The roofline's work counts.  `roofline.nnz_per_view` (the nonzeros of one
view's system matrix, which define the projectors' algorithmic bytes) is
checked against the oracle's exact FP64 Siddon count, and the byte formulas
against their definitions."""
import numpy as np
import pytest

from asd_pocs_mex_cuda_demo_gb300 import roofline


@pytest.mark.parametrize("case", [
    (64, 64, 1, 128, 1, 541.0, 408.0, 1.0, None),
    (512, 512, 1, 888, 1, 541.0, 408.0, 1.0, 0.9887),   # the 512^2 fan-beam protocol
    (32, 32, 32, 64, 64, 1000.0, 500.0, 6.4, 8.0),      # cone beam, scaled down
])
def test_nnz_per_view_matches_exact_siddon_count(oracle_mod, case):
    nx, ny, nz, na, nb, SO, OD, det, vx = case
    vx = vx or SO / (SO + OD) * det * na / nx
    for a in (13.0, 77.0, 200.0):
        g = oracle_mod.gateway_geometry(-a / 180 * np.pi, SO, OD, vx, det, na, nb)
        exact = oracle_mod.siddon_nnz(g, nx, ny, nz)
        est = roofline.nnz_per_view(a, SO, OD, vx, det, nx, ny, nz, na, nb)
        # plane crossings counted in FP64 without the oracle's length threshold
        assert abs(est / exact - 1) < 1e-2, (a, est, exact)


def test_fan_beam_protocol_nnz():
    """512^2 voxels of 0.9887 mm and 888 bins of 1 mm (SID 541 / SDD 949 mm):
    5.0e5 nonzeros per view along the axes to 6.2e5 along the diagonals, a
    mean of 5.6e5 over the 60 views of the scan -- and over the 10 views the
    bench samples (5.595e5, its reported nnz_per_view)."""
    views = np.arange(1, 61) * 6.0
    nnz = [roofline.nnz_per_view(a, 541.0, 408.0, 0.9887, 1.0, 512, 512, 1, 888, 1)
           for a in views]
    assert 5.0e5 <= min(nnz) and max(nnz) <= 6.3e5
    assert abs(np.mean(nnz) / 5.597e5 - 1) < 1e-3
    assert abs(np.mean(nnz[::6]) / 5.595e5 - 1) < 1e-3


def test_byte_formulas():
    nnz, na, nb, N = 1000, 30, 2, 500
    assert roofline.ax_bytes(nnz, na * nb) == 4 * nnz + 8 * na * nb
    assert roofline.atx_bytes(nnz, N) == 4 * nnz + 8 * N
    assert roofline.tv_step_bytes(N) == 8 * N
