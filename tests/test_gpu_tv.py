"""GPU TV minimisation against the reference's src/tvmin results (golden
vectors) and the oracle.  FP64 entry points: relative L2 <= 1e-12; FP32
device variant: <= 1e-5."""
import numpy as np
import pytest

import asd_pocs_mex_cuda_demo_gb300 as pkg
from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


def test_tv_fp64_vs_reference_vectors(gpu):
    d = golden("tv.npz")
    assert rel_l2(pkg.imgTVGradMin(d["img2"], 0.2, 20, 1, d["old2"]), d["out2"]) < 1e-12
    assert rel_l2(pkg.imgTVGradMin(d["img2"] - 0.5, 0.05, 7, 0), d["out2_nopos"]) < 1e-12
    assert rel_l2(pkg.imgTVGradMin3D(d["img3"], 0.2, 20, 1, d["old3"]), d["out3"]) < 1e-12


@pytest.mark.parametrize("shape", [(1, 1), (5, 3), (64, 48), (257, 130)])
def test_tv2d_fp64_vs_oracle(gpu, oracle_mod, shape):
    rng = np.random.default_rng(shape[0])
    img = rng.random(shape)
    old = rng.random(shape)
    out = pkg.imgTVGradMin(img, 0.1, 5, 1, old)
    assert rel_l2(out, oracle_mod.tv(img, 0.1, 5, 1, old)) < 1e-12


@pytest.mark.parametrize("shape", [(3, 4, 2), (33, 20, 9), (64, 64, 32)])
def test_tv3d_fp64_vs_oracle(gpu, oracle_mod, shape):
    rng = np.random.default_rng(shape[2])
    img = rng.random(shape)
    out = pkg.imgTVGradMin3D(img, 0.05, 4, 1)
    assert rel_l2(out, oracle_mod.tv(img, 0.05, 4, 1)) < 1e-12


def test_tv_zero_iterations_and_constant_image(gpu, oracle_mod):
    img = np.random.default_rng(2).random((8, 8)) - 0.5
    out = pkg.imgTVGradMin(img, 0.2, 0, 1)
    assert np.array_equal(out, img)  # nTVIter == 0: no step and no clamp
    z = np.zeros((6, 6))
    o = pkg.imgTVGradMin(z, 0.2, 3, 0)
    r = oracle_mod.tv(z, 0.2, 3, 0)
    # the reference divides by a zero norm: 0/0 = NaN everywhere
    assert np.isnan(o).all() and np.isnan(r).all()


@pytest.mark.parametrize("shape", [(64, 48, 1), (128, 128, 1), (40, 36, 20)])
def test_tv_fp32_device_vs_oracle(gpu, oracle_mod, shape):
    import torch

    from asd_pocs_mex_cuda_demo_gb300._lib import check, load

    nx, ny, nz = shape
    rng = np.random.default_rng(nx + nz)
    img = rng.random(shape)
    old = rng.random(shape)
    t = torch.tensor(img.ravel(order="F"), dtype=torch.float32, device=gpu)
    o = torch.tensor(old.ravel(order="F"), dtype=torch.float32, device=gpu)
    s = torch.cuda.current_stream().cuda_stream
    check(load().asdpocs_tv_device(t.data_ptr(), o.data_ptr(), nx, ny, nz, 0.2, 10, 1, s))
    torch.cuda.synchronize()
    img32 = img.astype(np.float32).astype(np.float64)
    old32 = old.astype(np.float32).astype(np.float64)
    if nz == 1:
        img32, old32 = img32[:, :, 0], old32[:, :, 0]
    ref = oracle_mod.tv(img32, 0.2, 10, 1, old32)
    assert rel_l2(t.cpu().numpy(), ref.ravel(order="F")) < 1e-5
