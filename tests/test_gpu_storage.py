"""Reduced-precision sinogram storage on the GPU (asdpocs_options
sino_storage): the sinogram is rounded once to FP16 or BF16 on the device and
widened to FP32 on every read; ray sums, residuals and images stay FP32 and
the step-control scalars FP64.  Each reduced-precision reconstruction states
its error against the FP64 oracle (the reference's projectors and TV, FP64
image state) and its RMSE against the phantom, beside the FP32 storage's."""
import json
import os

import numpy as np
import pytest

import asd_pocs_mex_cuda_demo_gb300 as pkg
from asd_pocs_mex_cuda_demo_gb300 import phantoms
from conftest import rel_l2

pytestmark = pytest.mark.gpu

# relative L2 distance to the FP64 oracle's image, and the RMSE against the
# phantom relative to the FP32 storage's.  FP16 meets the matched-RMSE bar
# (within 1 %: measured +0.04 %, 7e-4 from the oracle); BF16's 8-bit
# significand does not (measured +1.5 % RMSE, 6e-3 from the oracle).
BOUND = {"f32": 2e-4, "f16": 1e-3, "bf16": 8e-3}
RMSE_BOUND = {"f32": 0.0, "f16": 0.01, "bf16": 0.03}


def _fan(n=128, na=222, nv=60, iters=12, seed=3):
    SO, OD, det = 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    x = phantoms.random_ellipses(n, seed).astype(np.float32)
    phi = phantoms.views(nv)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=iters, numOfgradients=20, alpha=0.002)
    P = np.stack([pkg.Ax_cone_gpu(x, dict(para, phi=-a / 180 * np.pi))[0] for a in phi],
                 axis=1)
    return x, phantoms.poisson_noise(P, 1e5, seed).astype(np.float32), para


def _run(para, P, x, storage, where=0):
    import torch

    with pkg.Plan(dict(para, sino_storage=storage), para["phi_vec"]) as pl:
        if where:
            d = torch.tensor(P.ravel(order="F"), device="cuda")
            pl.set_sinogram(0, d.data_ptr())
            torch.cuda.synchronize()
        else:
            pl.set_sinogram(0, P.ravel(order="F"))
        pl.set_reference(0, x)
        pl.reset()
        pl.run()
        return pl.image(0), pl.stats(0), pl.nbytes


def test_reduced_precision_sinogram_error_vs_fp64_oracle(gpu, oracle_mod):
    x, P, para = _fan()
    mo, _ = oracle_mod.asdpocs(P.astype(np.float64), para)
    res, report = {}, {}
    for s in ("f32", "f16", "bf16"):
        img, st, nbytes = _run(para, P, x, s)
        res[s] = (img, st, nbytes)
        report[s] = dict(rel_l2_vs_fp64_oracle=rel_l2(img, mo),
                         rmse_vs_phantom=float(st["RMSE"][-1]), plan_bytes=nbytes)
    rep = os.environ.get("ASDPOCS_STORAGE_REPORT")
    if rep:
        with open(rep, "w") as f:
            json.dump(report, f, indent=1)
    for s, r in report.items():
        assert r["rel_l2_vs_fp64_oracle"] <= BOUND[s], (s, r)
        assert abs(r["rmse_vs_phantom"] / report["f32"]["rmse_vs_phantom"] - 1) <= RMSE_BOUND[s], (s, r)
    # the sinogram takes half the bytes
    sino = P.size * 4
    assert res["f32"][2] - res["f16"][2] >= sino // 2 - 256
    assert res["f16"][2] == res["bf16"][2]


def test_device_rounding_equals_host_rounding(gpu):
    """A device sinogram rounded on the GPU gives the same stored bits as the
    host rounding (same images, bit for bit)."""
    x, P, para = _fan(n=64, na=111, nv=24, iters=3)
    for s in ("f16", "bf16"):
        a = _run(para, P, x, s, where=0)[0]
        b = _run(para, P, x, s, where=1)[0]
        assert np.array_equal(a, b), s


def test_served_reduced_precision_job_equals_plan(gpu):
    x, P, para = _fan(n=64, na=111, nv=24, iters=3, seed=5)
    for s in ("f16", "bf16"):
        ref = _run(para, P, x, s)[0]
        with pkg.Server() as srv:
            j = srv.submit(dict(para, sino_storage=s), P, I0=x)
            img, _, _ = srv.wait(j)
        assert np.array_equal(img, ref), s


def test_sinogram_pointer_only_for_fp32_storage(gpu):
    x, P, para = _fan(n=32, na=60, nv=6, iters=1)
    with pkg.Plan(dict(para, sino_storage="f16"), para["phi_vec"]) as pl:
        assert pl.sinogram_ptr(0) == 0
    with pkg.Plan(para, para["phi_vec"]) as pl:
        assert pl.sinogram_ptr(0) != 0
