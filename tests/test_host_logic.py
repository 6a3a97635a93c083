"""Host-side argument handling of the mirrored reference interface (no GPU
compute: every call here fails validation before any device work)."""
import numpy as np
import pytest

import asd_pocs_mex_cuda_demo_gb300 as pkg
from asd_pocs_mex_cuda_demo_gb300 import phantoms
from asd_pocs_mex_cuda_demo_gb300.asdpocs import options_from_para

PARA = dict(SO=541.0, OD=408.0, vxlsize=1.14, nx=8, ny=8, nz=1, phi=0.3, detsize=1.0,
            na=16, nb=1)


@pytest.mark.parametrize("field", ["SO", "OD", "vxlsize", "nx", "ny", "nz", "phi",
                                   "detsize", "na", "nb"])
def test_missing_para_field(lib, field):
    p = dict(PARA)
    del p[field]
    with pytest.raises(pkg.MexError, match=f"parameter.{field}!"):
        pkg.Ax_cone_gpu(np.zeros(64, np.float32), p)
    with pytest.raises(pkg.MexError, match=f"parameter.{field}!"):
        pkg.Atx_cone_gpu(np.zeros(16, np.float32), p)


def test_size_mismatch_messages(lib):
    with pytest.raises(pkg.MexError, match="Error size of input argument X!"):
        pkg.Ax_cone_gpu(np.zeros(63, np.float32), PARA)
    with pytest.raises(pkg.MexError, match="Error size of input argument Y!"):
        pkg.Atx_cone_gpu(np.zeros(15, np.float32), PARA)
    with pytest.raises(pkg.MexError, match="Error usage!"):
        pkg.Ax_cone_gpu(np.zeros(64, np.float32), PARA, 1)


def test_tv_argument_checks(lib):
    with pytest.raises(pkg.MexError, match="double format"):
        pkg.imgTVGradMin(np.zeros((4, 4), np.float32), 0.1, 2, 1)
    with pytest.raises(pkg.MexError, match="img0 dimensions"):
        pkg.imgTVGradMin(np.zeros((4, 4)), 0.1, 2, 1, np.zeros((4, 5)))
    with pytest.raises(pkg.AsdpocsError, match="Nz >= 2"):
        pkg.imgTVGradMin3D(np.zeros((4, 4, 1)), 0.1, 2, 1)


def test_tv_rejects_images_beyond_one_launch(lib):
    """A thin volume whose TV tile grid would need more than 65535 launch rows
    (ceil(ny/8) * nz) is rejected with a clear message before device work."""
    with pytest.raises(pkg.AsdpocsError, match="tile rows"):
        pkg.imgTVGradMin3D(np.zeros((4, 1, 65536)), 0.1, 2, 1)


def test_bad_dimensions_are_rejected_before_device_work(lib):
    p = dict(PARA, nx=0)
    with pytest.raises(pkg.AsdpocsError, match="dimensions must be positive"):
        pkg.Ax_cone_gpu(np.zeros(0, np.float32), p)


def test_driver_checks(lib):
    para = dict(PARA, phi_vec=[1.0, 2.0, 3.0])
    with pytest.raises(pkg.AsdpocsError, match="phi_vec mismatch"):
        pkg.ASD_POCS_cuda(np.zeros((16, 2)), para)


def test_option_defaults_match_reference(lib):
    o = options_from_para({})
    assert (o.maxnumIter, o.numOfgradients) == (5, 20)
    assert (o.alpha, o.alpha_red, o.beta, o.beta_red, o.r_max) == (0.02, 0.95, 1.0, 0.995, 0.95)
    assert o.epsilon == np.finfo(float).eps and o.stopRelChg == np.finfo(float).eps
    o = options_from_para(dict(maxnumIter=7, alpha=0.2, beta_red=1.0))
    assert (o.maxnumIter, o.alpha, o.beta_red) == (7, 0.2, 1.0)


def test_plan_rejects_mixed_kinds(lib):
    """Instances of one plan may differ in size but not in kind: 2-D fan
    beam and cone beam need different kernels (rejected before any device
    call)."""
    a = dict(PARA)
    b = dict(PARA, nz=8, nb=4)
    with pytest.raises(pkg.AsdpocsError, match="all 2-D"):
        pkg.Plan([a, b], [np.arange(1, 4.0), np.arange(1, 4.0)])
    with pytest.raises(pkg.AsdpocsError, match="one phi_vec per instance"):
        pkg.Plan([a, a], [np.arange(1, 4.0)])


def test_phantoms():
    sl = phantoms.shepp_logan_2d(64)
    assert sl.shape == (4096,) and 0.9 < sl.max() <= 1.0 + 1e-12 and sl.min() > -1e-12
    sl3 = phantoms.shepp_logan_3d(16)
    assert sl3.shape == (16 ** 3,)
    # the central slice of the 3D phantom matches the 2D section on an odd grid
    r = phantoms.random_ellipses(64, seed=5)
    assert r.min() >= 0 and r.max() <= 0.04
    assert np.array_equal(r, phantoms.random_ellipses(64, seed=5))
    v = phantoms.views(60)
    assert v[0] == 6.0 and v[-1] == 360.0
    P = np.full((10, 3), 2.0)
    n1 = phantoms.poisson_noise(P, 1e5, seed=1)
    assert np.all(np.isfinite(n1)) and abs(n1.mean() - 2.0) < 0.05
