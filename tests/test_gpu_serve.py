"""Serving queue on the GPU: jobs of mixed kinds, sizes, view counts and
iteration budgets submitted while others run; each result must equal the
same reconstruction run alone in a Plan, bit for bit, and the device memory
the jobs held must return to zero."""
import time

import numpy as np
import pytest

import asd_pocs_mex_cuda_demo_gb300 as pkg
from asd_pocs_mex_cuda_demo_gb300 import phantoms

pytestmark = pytest.mark.gpu


def _job2d(seed, n, na, nv, iters, ng, shift=None):
    """shift: view-angle offset; jobs with equal sizes and offset share a
    scan protocol (and a lane of the server)."""
    SO, OD, det = 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    x = phantoms.random_ellipses(n, seed).astype(np.float32)
    phi = phantoms.views(nv) + (0.25 * seed if shift is None else shift)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=iters, numOfgradients=ng, alpha=0.02)
    P = np.stack([pkg.Ax_cone_gpu(x, dict(para, phi=-a / 180 * np.pi))[0] for a in phi],
                 axis=1)
    return x, phantoms.poisson_noise(P, 1e5, seed).astype(np.float32), para


def _job3d(seed, n, na, nb, nv, iters):
    SO, OD, det = 1000.0, 500.0, 0.8 * 256 / n
    vx = 1.0 * 256 / n
    x = (phantoms.shepp_logan_3d(n) * 0.02).astype(np.float32)
    phi = phantoms.views(nv) + seed
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=n, na=na, nb=nb, detsize=det,
                phi_vec=phi, maxnumIter=iters, numOfgradients=3, alpha=0.02)
    P = np.stack([pkg.Ax_cone_gpu(x, dict(para, phi=-a / 180 * np.pi))[0] for a in phi],
                 axis=1)
    return x, phantoms.poisson_noise(P, 5e4, seed).astype(np.float32), para


def _alone(x, P, para):
    with pkg.Plan(para, para["phi_vec"]) as pl:
        pl.set_sinogram(0, P.ravel(order="F"))
        pl.set_reference(0, x)
        pl.reset()
        pl.run()
        return pl.image(0), pl.stats(0)


def test_server_jobs_equal_alone(gpu):
    # jobs 0, 4, 7 and 8 share one protocol, jobs 3 and 9 another (cone beam)
    jobs = [_job2d(1, 48, 72, 12, 3, 5, shift=1.0), _job2d(2, 64, 96, 20, 4, 10),
            _job2d(3, 40, 60, 9, 2, 0), _job3d(4, 16, 32, 24, 10, 2),
            _job2d(5, 48, 72, 12, 2, 2, shift=1.0), _job2d(6, 33, 50, 7, 5, 1),
            _job3d(7, 20, 40, 30, 12, 3), _job2d(8, 48, 72, 12, 6, 20, shift=1.0),
            _job2d(9, 48, 72, 12, 1, 3, shift=1.0), _job3d(4, 16, 32, 24, 10, 4)]
    ref = [_alone(*j) for j in jobs]
    with pkg.Server(slots_per_lane=3) as srv:  # a fourth job of a protocol waits
        ids = [srv.submit(para, P, I0=x) for x, P, para in jobs[:3]]
        # later arrivals join while the first ones run
        deadline = time.time() + 30
        while srv.poll(ids[0]) == 0 and time.time() < deadline:
            time.sleep(0.001)
        ids += [srv.submit(para, P, I0=x) for x, P, para in jobs[3:]]
        for k, j in enumerate(ids):
            img, out, t = srv.wait(j)
            assert np.array_equal(img, ref[k][0]), k
            assert out["IterationNum"] == ref[k][1]["IterationNum"]
            np.testing.assert_array_equal(out["RMSE"], ref[k][1]["RMSE"])
            assert 0.0 <= t["queued_ms"] <= t["total_ms"] and t["run_ms"] > 0.0
        in_use, peak = srv.memory()
        assert in_use == 0 and peak > 0
        with pytest.raises(pkg.AsdpocsError):
            srv.wait(ids[0])  # released


def test_server_budget_admission(gpu):
    jobs = [_job2d(20 + s, 48, 72, 12, 3, 5) for s in range(4)]
    ref = [_alone(*j) for j in jobs]
    one = None
    with pkg.Server() as probe:
        j = probe.submit(jobs[0][2], jobs[0][1])
        probe.wait(j)
        one = probe.memory()[1]  # device bytes of one such job
    # room for two jobs at a time: the others wait for memory, then run
    with pkg.Server(slots_per_lane=8, hbm_budget_bytes=2 * one + one // 2) as srv:
        ids = [srv.submit(para, P, I0=x) for x, P, para in jobs]
        for k, j in enumerate(ids):
            img, _, _ = srv.wait(j)
            assert np.array_equal(img, ref[k][0]), k
        assert srv.memory()[1] <= 2 * one
    with pkg.Server(hbm_budget_bytes=one // 2) as srv:
        with pytest.raises(pkg.AsdpocsError) as e:
            srv.submit(jobs[0][2], jobs[0][1])
        assert e.value.status == 3


def test_server_cancel_queued_and_running_jobs(gpu):
    """A queued job and a running job are cancelled from the host: the queued
    one never runs, the running one leaves its slot at the end of the
    iteration in flight, and every other job's result equals its run alone,
    bit for bit; the device memory of all jobs returns to zero."""
    jobs = [_job2d(40 + s, 48, 72, 12, 4, 5, shift=2.0) for s in range(4)]
    long_job = _job2d(45, 48, 72, 12, 400, 20, shift=2.0)  # far from done when cancelled
    ref = [_alone(*j) for j in jobs]
    with pkg.Server(slots_per_lane=2) as srv:
        x, P, para = long_job
        run_id = srv.submit(para, P, I0=x)
        deadline = time.time() + 30
        while srv.poll(run_id) != 1 and time.time() < deadline:  # RUNNING
            time.sleep(0.001)
        assert srv.poll(run_id) == 1
        ids = [srv.submit(para_k, P_k, I0=x_k) for x_k, P_k, para_k in jobs]
        queued = srv.submit(para, P, I0=x)  # behind the four: still queued
        assert srv.poll(queued) == 0
        srv.cancel(queued)
        assert srv.poll(queued) == 4  # CANCELLED
        srv.cancel(run_id)
        for k, j in enumerate(ids):
            img, out, _ = srv.wait(j)
            assert np.array_equal(img, ref[k][0]), k
            np.testing.assert_array_equal(out["RMSE"], ref[k][1]["RMSE"])
        for j in (queued, run_id):
            with pytest.raises(pkg.AsdpocsError, match="cancelled"):
                srv.wait(j)
        with pytest.raises(pkg.AsdpocsError):
            srv.cancel(ids[0])  # released
        assert srv.memory()[0] == 0
