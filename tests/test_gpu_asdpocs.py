"""GPU ASD-POCS / SART (device-resident plans through the C ABI) against the
golden reconstructions (reference projector + TV code under the restated
driver) and the oracle.  The GPU keeps the image in FP32 where MATLAB keeps
FP64; the reconstruction tolerance is relative L2 <= 2e-4."""
import numpy as np
import pytest

import asd_pocs_mex_cuda_demo_gb300 as pkg
from asd_pocs_mex_cuda_demo_gb300 import phantoms
from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu
RECON_TOL = 2e-4


def _para2(d, **kw):
    """The 64^2 fixture's para struct (6 iterations, alpha=0.2 unless given)."""
    n, na, SO, OD, vx, det = d["geo2"]
    p = dict(SO=SO, OD=OD, vxlsize=vx, nx=int(n), ny=int(n), nz=1, na=int(na), nb=1,
             detsize=det, phi_vec=d["phi2"], maxnumIter=6, alpha=0.2, alpha_red=0.95,
             I0=d["x2"])
    p.update(kw)
    return p


def test_asdpocs_2d_vs_golden_well_conditioned(gpu):
    d = golden("asdpocs.npz")
    m, out = pkg.ASD_POCS_cuda(d["P2"], _para2(d, alpha=0.002))
    assert rel_l2(m.ravel(order="F"), d["m2s"]) < RECON_TOL
    assert out["IterationNum"] == int(d["out2s"][0])
    np.testing.assert_allclose(out["RMSE"], d["rmse2s"], rtol=1e-4)
    np.testing.assert_allclose([out["alpha"], out["beta"]], d["out2s"][2:], rtol=1e-12)
    assert abs(out["dataTolerance"] / d["out2s"][1] - 1) < 1e-3


def test_asdpocs_2d_vs_golden_reference_settings(gpu):
    # alpha=0.2 with the reference's TV step size is chaotic (a 1e-7 relative
    # perturbation of P moves the FP64 result by ~3e-2): compare the image to
    # 1e-1 and the RMSE trajectory to 3%
    d = golden("asdpocs.npz")
    m, out = pkg.ASD_POCS_cuda(d["P2"], _para2(d))
    assert rel_l2(m.ravel(order="F"), d["m2"]) < 1e-1
    assert out["IterationNum"] == int(d["out2"][0])
    np.testing.assert_allclose(out["RMSE"], d["rmse2"], rtol=3e-2)


def test_asdpocs_3d_vs_golden(gpu):
    d = golden("asdpocs.npz")
    n3, na3, nb3, SO3, OD3, vx3, det3 = d["geo3"]
    para = dict(SO=SO3, OD=OD3, vxlsize=vx3, nx=int(n3), ny=int(n3), nz=int(n3),
                na=int(na3), nb=int(nb3), detsize=det3, phi_vec=d["phi3"], maxnumIter=4,
                alpha=0.2, I0=d["x3"])
    m, out = pkg.ASD_POCS_cuda(d["P3"], para)
    assert rel_l2(m.ravel(order="F"), d["m3"]) < RECON_TOL
    np.testing.assert_allclose(out["RMSE"], d["rmse3"], rtol=1e-4)


def test_stop_rule_and_m0(gpu, oracle_mod):
    d = golden("asdpocs.npz")
    rng = np.random.default_rng(4)
    m0 = rng.random(int(d["geo2"][0]) ** 2) * 0.1
    # dp/N is 2.8e-3 after the first sweep and below 1e-3 after the second
    para = _para2(d, maxnumIter=5, stopRelChg=1e-3, m0=m0, alpha=0.002)
    m, out = pkg.ASD_POCS_cuda(d["P2"], para)
    mo, outo = oracle_mod.asdpocs(d["P2"], para)
    assert out["IterationNum"] == outo["IterationNum"] == 2
    assert len(out["RMSE"]) == 2
    assert rel_l2(m.ravel(order="F"), mo) < RECON_TOL


def test_no_tv_and_sart(gpu, oracle_mod):
    d = golden("asdpocs.npz")
    para = _para2(d, maxnumIter=3, numOfgradients=0)
    m, out = pkg.ASD_POCS_cuda(d["P2"], para)
    mo, outo = oracle_mod.asdpocs(d["P2"], para)
    assert rel_l2(m.ravel(order="F"), mo) < RECON_TOL
    ms, outs = pkg.SART_cuda_inline(d["P2"], dict(para, **{"lambda": 0.7}))
    mso, dto = oracle_mod.sart(d["P2"], dict(para, **{"lambda": 0.7}))
    assert rel_l2(ms, mso) < RECON_TOL
    assert abs(outs["dataTolerance"] / dto - 1) < 1e-4


def test_init_by_sart(gpu, oracle_mod):
    d = golden("asdpocs.npz")
    para = _para2(d, maxnumIter=2, initBySART=True, alpha=0.002)
    m, _ = pkg.ASD_POCS_cuda(d["P2"], para)
    m0, _ = oracle_mod.sart(d["P2"], para)
    mo, _ = oracle_mod.asdpocs(d["P2"], dict(para, m0=m0))
    assert rel_l2(m.ravel(order="F"), mo) < RECON_TOL


def _instance(seed, n=64, na=128, nv=30):
    SO, OD, det = 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    x = phantoms.random_ellipses(n, seed)
    phi = phantoms.views(nv) + seed  # per-instance angles
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=4, alpha=0.002)
    P = np.zeros((na, nv))
    for i, a in enumerate(phi):
        P[:, i] = pkg.Ax_cone_gpu(x.astype(np.float32), dict(para, phi=-a / 180 * np.pi))[0]
    P = phantoms.poisson_noise(P, 1e5, seed)
    return x, P, para


def test_batch_equals_alone_bitwise(gpu):
    insts = [_instance(s) for s in (1, 2, 3)]
    alone = []
    for x, P, para in insts:
        with pkg.Plan(para, para["phi_vec"]) as pl:
            pl.set_sinogram(0, P.ravel(order="F"))
            pl.set_reference(0, x)
            pl.reset()
            pl.run()
            alone.append((pl.image(0), pl.stats(0)))
    paras = [i[2] for i in insts]
    with pkg.Plan(paras, [p["phi_vec"] for p in paras]) as pl:
        for k, (x, P, _) in enumerate(insts):
            pl.set_sinogram(k, P.ravel(order="F"))
            pl.set_reference(k, x)
        pl.reset()
        pl.run(use_graph=True)
        for k in range(3):
            assert np.array_equal(pl.image(k), alone[k][0])
            s = pl.stats(k)
            assert s["IterationNum"] == alone[k][1]["IterationNum"]
            np.testing.assert_array_equal(s["RMSE"], alone[k][1]["RMSE"])
        # replay: reset and run again without the graph gives the same bits
        pl.reset()
        pl.run(use_graph=False)
        for k in range(3):
            assert np.array_equal(pl.image(k), alone[k][0])


def test_plan_vs_oracle_noisy(gpu, oracle_mod):
    x, P, para = _instance(7)
    with pkg.Plan(para, para["phi_vec"]) as pl:
        pl.set_sinogram(0, P.ravel(order="F"))
        pl.reset()
        pl.run()
        m = pl.image(0)
    mo, _ = oracle_mod.asdpocs(P, para)
    assert rel_l2(m, mo) < RECON_TOL


def test_hbm_budget_admission(gpu):
    _, _, para = _instance(1)
    with pytest.raises(pkg.AsdpocsError) as e:
        pkg.Plan(para, para["phi_vec"], hbm_budget_bytes=1024)
    assert e.value.status == 3


def test_shared_geometry_batch_equals_alone_bitwise(gpu, monkeypatch):
    # instances with the same geometry and angles take the shared-coefficient
    # backward step; each result must equal its single-instance run exactly
    n, na, nv = 64, 128, 30
    SO, OD, det = 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    phi = phantoms.views(nv)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=3, alpha=0.002)
    Ps = []
    for s in range(5):
        x = phantoms.random_ellipses(n, 40 + s).astype(np.float32)
        P = np.stack([pkg.Ax_cone_gpu(x, dict(para, phi=-a / 180 * np.pi))[0] for a in phi],
                     axis=1)
        Ps.append(phantoms.poisson_noise(P, 1e5, 40 + s))
    alone = []
    for P in Ps:
        with pkg.Plan(para, phi) as pl:
            pl.set_sinogram(0, P.ravel(order="F"))
            pl.reset()
            pl.run()
            alone.append(pl.image(0))
    for force_per_instance in (False, True):
        if force_per_instance:
            monkeypatch.setenv("ASDPOCS_NO_SHARED_GEOMETRY", "1")
        with pkg.Plan([para] * 5, [phi] * 5) as pl:
            for k, P in enumerate(Ps):
                pl.set_sinogram(k, P.ravel(order="F"))
            pl.reset()
            pl.run()
            for k in range(5):
                assert np.array_equal(pl.image(k), alone[k]), (force_per_instance, k)


def _uneven(seed, n, na, nv, iters, ng, SO=541.0, OD=408.0, det=1.0, gseed=None):
    """An instance: phantom and noise from `seed`, view angles offset by
    `gseed` (default `seed`): instances of equal sizes and `gseed` share
    their geometry."""
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    x = phantoms.random_ellipses(n, seed)
    phi = phantoms.views(nv) + 0.5 * (seed if gseed is None else gseed)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=iters, numOfgradients=ng, alpha=0.002)
    P = np.stack([pkg.Ax_cone_gpu(x.astype(np.float32), dict(para, phi=-a / 180 * np.pi))[0]
                  for a in phi], axis=1)
    return x, phantoms.poisson_noise(P, 1e5, seed), para


def test_uneven_batch_equals_alone_bitwise(gpu, oracle_mod):
    """One plan of instances with different image sizes, bins, view counts,
    iteration counts and TV step counts (the batched uneven-slice pattern):
    every step is one launch for all of them, and each result equals the
    instance's run alone bit for bit and the oracle within the
    reconstruction tolerance."""
    insts = [_uneven(11, 48, 72, 12, 3, 20), _uneven(12, 80, 120, 30, 5, 5),
             _uneven(13, 64, 96, 20, 2, 1), _uneven(14, 33, 50, 7, 4, 0),
             _uneven(15, 80, 120, 30, 5, 5)]
    alone = []
    for x, P, para in insts:
        with pkg.Plan(para, para["phi_vec"]) as pl:
            pl.set_sinogram(0, P.ravel(order="F"))
            pl.set_reference(0, x)
            pl.reset()
            pl.run()
            alone.append((pl.image(0), pl.stats(0)))
    paras = [i[2] for i in insts]
    with pkg.Plan(paras, [p["phi_vec"] for p in paras]) as pl:
        for k, (x, P, _) in enumerate(insts):
            pl.set_sinogram(k, P.ravel(order="F"))
            pl.set_reference(k, x)
        for use_graph in (True, False):
            pl.reset()
            pl.run(use_graph=use_graph)
            for k in range(len(insts)):
                assert np.array_equal(pl.image(k), alone[k][0]), (use_graph, k)
                s = pl.stats(k)
                assert s["IterationNum"] == alone[k][1]["IterationNum"]
                np.testing.assert_array_equal(s["RMSE"], alone[k][1]["RMSE"])
    for k in (0, 1, 3):
        _, P, para = insts[k]
        mo, _ = oracle_mod.asdpocs(P, para)
        assert rel_l2(alone[k][0], mo) < RECON_TOL, k


@pytest.mark.parametrize("tables", [True, False], ids=["chord-tables", "direct"])
def test_mixed_geometry_groups_equal_alone_bitwise(gpu, monkeypatch, tables):
    """A 2-D plan whose instances fall into several geometries, some shared
    by a few instances (one of them by nine: a full group of eight and one
    more), listed out of order and with different iteration and TV-step
    counts: the instances of a geometry run as groups through the
    shared-geometry kernels, several geometries per launch, and each result
    equals the instance's run alone bit for bit."""
    if not tables:
        monkeypatch.setenv("ASDPOCS_NO_CHORD_TABLE", "1")
    A = dict(n=48, na=72, nv=12, gseed=1)
    B = dict(n=64, na=96, nv=20, gseed=2)
    C = dict(n=33, na=50, nv=7, gseed=3)
    D = dict(n=80, na=120, nv=30, gseed=4)
    spec = [(A, 3, 20), (B, 2, 5), (C, 4, 1), (B, 2, 5), (D, 2, 3), (A, 2, 20), (B, 3, 0),
            (B, 2, 5), (C, 3, 2), (B, 2, 5), (B, 4, 5), (A, 4, 10), (B, 2, 5), (B, 2, 5),
            (B, 3, 5)]
    insts = [_uneven(40 + k, g["n"], g["na"], g["nv"], it, ng, gseed=g["gseed"])
             for k, (g, it, ng) in enumerate(spec)]
    alone = []
    for x, P, para in insts:
        with pkg.Plan(para, para["phi_vec"]) as pl:
            pl.set_sinogram(0, P.ravel(order="F"))
            pl.set_reference(0, x)
            pl.reset()
            pl.run()
            alone.append((pl.image(0), pl.stats(0)))
    paras = [i[2] for i in insts]
    with pkg.Plan(paras, [p["phi_vec"] for p in paras]) as pl:
        for k, (x, P, _) in enumerate(insts):
            pl.set_sinogram(k, P.ravel(order="F"))
            pl.set_reference(k, x)
        for use_graph in (True, False):
            pl.reset()
            pl.run(use_graph=use_graph)
            for k in range(len(insts)):
                assert np.array_equal(pl.image(k), alone[k][0]), (use_graph, k)
                s = pl.stats(k)
                assert s["IterationNum"] == alone[k][1]["IterationNum"]
                np.testing.assert_array_equal(s["RMSE"], alone[k][1]["RMSE"])


def test_mixed_geometry_many_classes_storage_and_autotune(gpu):
    """More geometries than sub-batches (ten, most of them shared by two or
    three instances), FP16 sinograms and a plan autotuned before it runs:
    each result still equals its own one-instance FP16 plan bit for bit."""
    spec = []
    for c in range(10):
        g = dict(n=24 + 4 * (c % 5), na=40 + 6 * (c % 4), nv=5 + 2 * c, gseed=100 + c)
        spec += [(g, 2 + (c % 3), 5 * (c % 2))] * (1 + c % 3)
    insts = [_uneven(200 + k, g["n"], g["na"], g["nv"], it, ng, gseed=g["gseed"])
             for k, (g, it, ng) in enumerate(spec)]
    paras = [dict(i[2], sino_storage="f16") for i in insts]
    alone = []
    for (x, P, _), para in zip(insts, paras):
        with pkg.Plan(para, para["phi_vec"]) as pl:
            pl.set_sinogram(0, P.ravel(order="F"))
            pl.set_reference(0, x)
            pl.reset()
            pl.run()
            alone.append(pl.image(0))
    with pkg.Plan(paras, [p["phi_vec"] for p in paras]) as pl:
        assert pl.streams > 1
        for k, (x, P, _) in enumerate(insts):
            pl.set_sinogram(k, P.ravel(order="F"))
            pl.set_reference(k, x)
        pl.autotune_shapes(reps=2)
        pl.reset()
        pl.run()
        for k in range(len(insts)):
            assert np.array_equal(pl.image(k), alone[k]), k


def test_uneven_cone_beam_batch_equals_alone_bitwise(gpu):
    """Cone-beam instances of different volume and detector sizes and view
    counts in one plan (per-instance kernels, sub-batches by size, each
    view's launches over the instances that have it): each result equals the
    instance's run alone bit for bit."""
    spec = [(24, 24, 16, 40, 30, 9, 2, 3), (32, 28, 20, 48, 40, 12, 3, 2),
            (24, 24, 16, 40, 30, 9, 2, 3), (20, 20, 24, 36, 36, 7, 2, 0),
            (32, 28, 20, 48, 40, 5, 1, 4)]
    insts = []
    for k, (nx, ny, nz, na, nb, nv, it, ng) in enumerate(spec):
        phi = phantoms.views(nv) + 3.0 * k
        para = dict(SO=1000.0, OD=500.0, vxlsize=1.0, nx=nx, ny=ny, nz=nz, na=na, nb=nb,
                    detsize=1.6, phi_vec=phi, maxnumIter=it, numOfgradients=ng, alpha=0.05)
        P = np.random.default_rng(300 + k).random(na * nb * nv).astype(np.float32)
        insts.append((para, P))
    alone = []
    for para, P in insts:
        with pkg.Plan(para, para["phi_vec"]) as pl:
            pl.set_sinogram(0, P)
            pl.reset()
            pl.run()
            alone.append(pl.image(0))
    paras = [i[0] for i in insts]
    with pkg.Plan(paras, [p["phi_vec"] for p in paras]) as pl:
        assert pl.streams > 1
        for k, (_, P) in enumerate(insts):
            pl.set_sinogram(k, P)
        pl.reset()
        pl.run()
        for k in range(len(insts)):
            assert np.array_equal(pl.image(k), alone[k]), k
            assert np.isfinite(alone[k]).all()


def test_shared_geometry_cone_beam_instances_finishing_apart(gpu):
    """Cone-beam instances sharing geometry share one per-view ray-slope
    table; the instance that refreshes it keeps doing so after its own
    iterations end, so the others' results still equal their runs alone."""
    n, na, nb, nv = 20, 40, 30, 9
    SO, OD, det, vx = 1000.0, 500.0, 10.24, 12.8
    phi = phantoms.views(nv)
    x = (phantoms.shepp_logan_3d(n) * 0.02).astype(np.float32)
    base = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=n, na=na, nb=nb, detsize=det,
                phi_vec=phi, numOfgradients=3, alpha=0.02)
    P = np.stack([pkg.Ax_cone_gpu(x, dict(base, phi=-a / 180 * np.pi))[0] for a in phi],
                 axis=1)
    paras = [dict(base, maxnumIter=it) for it in (1, 3, 2, 4)]
    Ps = [phantoms.poisson_noise(P, 5e4, 60 + k) for k in range(len(paras))]
    alone = []
    for para, Pk in zip(paras, Ps):
        with pkg.Plan(para, phi) as pl:
            pl.set_sinogram(0, Pk.ravel(order="F"))
            pl.reset()
            pl.run()
            alone.append(pl.image(0))
    with pkg.Plan(paras, [phi] * len(paras)) as pl:
        for k, Pk in enumerate(Ps):
            pl.set_sinogram(k, Pk.ravel(order="F"))
        pl.reset()
        pl.run()
        for k in range(len(paras)):
            assert np.array_equal(pl.image(k), alone[k]), k


@pytest.mark.parametrize("dims", [(1, 1, 1, 3, 1), (3, 17, 1, 1, 1), (17, 9, 5, 33, 7)])
def test_plan_edge_shapes_vs_oracle(gpu, oracle_mod, dims):
    """Degenerate and odd sizes (a single voxel, a single bin, odd cone-beam
    sizes) through the whole device iteration, against the oracle."""
    nx, ny, nz, na, nb = dims
    SO, OD, det = 300.0, 200.0, 1.3
    vx = phantoms.fov_voxel_size(SO, OD, det, max(na, 2), nx)
    rng = np.random.default_rng(sum(dims))
    phi = phantoms.views(6) + 3.0
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=nx, ny=ny, nz=nz, na=na, nb=nb, detsize=det,
                phi_vec=phi, maxnumIter=3, numOfgradients=4, alpha=0.002)
    P = rng.random((na * nb, len(phi)))
    m, out = pkg.ASD_POCS_cuda(P, para)
    mo, oo = oracle_mod.asdpocs(P, para)
    assert out["IterationNum"] == oo["IterationNum"]
    assert rel_l2(m.ravel(order="F"), mo) < 1e-4 or np.abs(m.ravel(order="F") - mo).max() < 1e-6


def test_zero_iterations_returns_initial_image(gpu):
    n, na = 16, 24
    para = dict(SO=541.0, OD=408.0, vxlsize=phantoms.fov_voxel_size(541, 408, 1.0, na, n),
                nx=n, ny=n, nz=1, na=na, nb=1, detsize=1.0, phi_vec=phantoms.views(5),
                maxnumIter=0)
    m0 = np.random.default_rng(3).random((n, n))
    m, out = pkg.ASD_POCS_cuda(np.ones((na, 5)), dict(para, m0=m0))
    assert out["IterationNum"] == 0
    assert np.array_equal(m.ravel(order="F"), m0.ravel(order="F").astype(np.float32))


def test_shared_geometry_groups_with_remainder(gpu):
    """37 instances of one protocol: full groups and a partial last one, each
    result equal to its run alone."""
    n, na, nv = 16, 24, 8
    SO, OD, det = 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    phi = phantoms.views(nv)
    rng = np.random.default_rng(11)
    paras = [dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                  phi_vec=phi, maxnumIter=int(rng.integers(1, 4)),
                  numOfgradients=int(rng.integers(0, 4)), alpha=0.02) for _ in range(37)]
    Ps = [rng.random(na * nv).astype(np.float32) for _ in range(37)]
    with pkg.Plan(paras, [phi] * 37) as pl:
        for k, P in enumerate(Ps):
            pl.set_sinogram(k, P)
        pl.reset()
        pl.run()
        batch = [pl.image(k) for k in range(37)]
    for k in (0, 7, 8, 15, 16, 31, 32, 35, 36):
        with pkg.Plan(paras[k], phi) as pl:
            pl.set_sinogram(0, Ps[k])
            pl.reset()
            pl.run()
            assert np.array_equal(pl.image(0), batch[k]), k


@pytest.mark.parametrize("nx,ny,batch,check", [
    (384, 384, 60, (0, 59)),   # 168 strip bands x 60: three bands per walk in the batch
    (121, 70, 3, (0, 2)),      # odd nx: per-column accesses; ragged strips and bands
    (36, 20, 2, (1,)),         # one strip, one band
    (4, 3, 2, (0,)),
    (1, 5, 2, (1,)),
])
def test_tv_walks_batch_equals_alone(gpu, nx, ny, batch, check):
    """The 2-D TV step walks strips of 60 output columns in bands of 16 rows,
    several bands per walk when the batch is large; each instance's result
    is the same bits as its run alone (one band per walk)."""
    na, nv = 48, 8
    SO, OD, det = 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, max(nx, ny))
    phi = phantoms.views(nv)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=nx, ny=ny, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=2, numOfgradients=3, alpha=0.05)
    rng = np.random.default_rng(nx * 1000 + ny)
    Ps = [rng.random(na * nv).astype(np.float32) for _ in range(batch)]
    with pkg.Plan([para] * batch, [phi] * batch) as pl:
        for k, P in enumerate(Ps):
            pl.set_sinogram(k, P)
        pl.reset()
        pl.run()
        out = [pl.image(k) for k in range(batch)]
    for k in check:
        with pkg.Plan(para, phi) as pl:
            pl.set_sinogram(0, Ps[k])
            pl.reset()
            pl.run()
            assert np.array_equal(pl.image(0), out[k]), k
        assert np.isfinite(out[k]).all()


def test_tv_zwalks_batch_equals_alone(gpu):
    """The cone-beam TV step walks 28 x 30 tiles down z in slabs of 16
    slices (16 tiles x 3 slabs for each of the 20 instances here, walks of
    several slabs in the batch and of one alone); each instance's result is
    the same bits either way."""
    nx, ny, nz, na, nb, nv, batch = 96, 96, 40, 48, 48, 6, 20
    SO, OD, det = 1000.0, 500.0, 1.6
    phi = phantoms.views(nv)
    para = dict(SO=SO, OD=OD, vxlsize=1.0, nx=nx, ny=ny, nz=nz, na=na, nb=nb, detsize=det,
                phi_vec=phi, maxnumIter=2, numOfgradients=3, alpha=0.05)
    rng = np.random.default_rng(5)
    Ps = [rng.random(na * nb * nv).astype(np.float32) for _ in range(batch)]
    with pkg.Plan([para] * batch, [phi] * batch) as pl:
        for k, P in enumerate(Ps):
            pl.set_sinogram(k, P)
        pl.reset()
        pl.run()
        out = [pl.image(k) for k in range(batch)]
    for k in (0, batch - 1):
        with pkg.Plan(para, phi) as pl:
            pl.set_sinogram(0, Ps[k])
            pl.reset()
            pl.run()
            assert np.array_equal(pl.image(0), out[k]), k
        assert np.isfinite(out[k]).all()


@pytest.mark.parametrize("shape", [(200, 150, 1), (60, 44, 40)])
def test_tv_walk_length_and_autotune_do_not_change_results(gpu, shape):
    """Every TV walk length (bands of 16 rows in 2-D, slabs of 16 slices in
    3-D) gives the same bits; the autotuner picks one of them and leaves the
    reconstruction state as it was."""
    nx, ny, nz = shape
    na, nb, nv = 64, (1 if nz == 1 else 48), 6
    phi = phantoms.views(nv)
    para = dict(SO=1000.0, OD=500.0, vxlsize=1.0, nx=nx, ny=ny, nz=nz, na=na, nb=nb,
                detsize=1.6, phi_vec=phi, maxnumIter=2, numOfgradients=4, alpha=0.05)
    P = np.random.default_rng(nz).random(na * nb * nv).astype(np.float32)
    out = {}
    with pkg.Plan(para, phi) as pl:
        pl.set_sinogram(0, P)
        for walk in (0, 1, 2, 3, 100):
            pl.set_tv_walk(walk)
            pl.reset()
            pl.run()
            out[walk] = pl.image(0)
        pl.reset()
        w, ms = pl.autotune(reps=3)
        assert w >= 0 and ms > 0
        pl.run()
        tuned = pl.image(0)
    for walk, img in out.items():
        assert np.array_equal(img, out[0]), walk
    assert np.array_equal(tuned, out[0])


@pytest.mark.parametrize("n,na,det,vx,nv,span,table", [
    (96, 160, 1.0, None, 24, 360.0, True),   # fan beam like the 512^2 protocol, scaled down
    (40, 41, 1.0, None, 8, 360.0, True),     # odd na: the 90-degree views' central rays are axis-parallel
    (50, 64, 1.0, None, 13, 200.0, True),    # nx not a multiple of the 32-voxel tiles
    (24, 400, 0.01, 0.5, 6, 180.0, False),   # ~120 bins per voxel: more pairs than a table holds
])
def test_chord_tables_do_not_change_results(gpu, monkeypatch, n, na, det, vx, nv, span,
                                            table):
    """2-D plans of one instance or of instances sharing geometry read the
    backward step's chords from tables built once per plan; every image
    equals the plan's without the tables, and a residual that is not finite
    (a sinogram with inf) takes the direct form in both."""
    SO, OD = 541.0, 408.0
    vx = vx or phantoms.fov_voxel_size(SO, OD, det, na, n)
    phi = phantoms.views(nv, span)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=3, numOfgradients=3, alpha=0.02)
    rng = np.random.default_rng(n + na)
    B = 11
    Ps = [rng.random(na * nv).astype(np.float32) for _ in range(B)]
    Ps[4][7] = np.inf

    def run(b):  # b instances (1: the per-instance kernels)
        with pkg.Plan([para] * b, [phi] * b) as pl:
            for k in range(b):
                pl.set_sinogram(k, Ps[k])
            pl.reset()
            pl.run()
            return [pl.image(k) for k in range(b)], pl.nbytes, pl.chord_slots

    with_tab, bytes_tab, slots = run(B)
    alone_tab, _, slots1 = run(1)
    monkeypatch.setenv("ASDPOCS_NO_CHORD_TABLE", "1")
    without, bytes_direct, slots_direct = run(B)
    alone, _, _ = run(1)
    assert (slots > 0) == table and slots_direct == 0  # whether the tables were built
    assert slots1 == slots
    assert bytes_tab - bytes_direct == (2 + slots) * n * n * nv * 4 * (slots > 0)
    for k in range(B):
        assert np.array_equal(with_tab[k], without[k], equal_nan=True), k
    assert np.array_equal(alone_tab[0], alone[0]) and np.array_equal(alone[0], without[0])


def test_chord_tables_per_instance_in_uneven_plans(gpu, monkeypatch):
    """A plan of 2-D instances with different sizes, bins and views builds a
    chord table per instance; every image equals the plan's without them."""
    shapes = [(40, 60, 9), (33, 50, 7), (64, 96, 12)]
    paras, Ps = [], []
    for s, (n, na, nv) in enumerate(shapes):
        x, P, para = _uneven(70 + s, n, na, nv, 3, 3)
        paras.append(para)
        Ps.append(P)

    def run():
        with pkg.Plan(paras, [p["phi_vec"] for p in paras]) as pl:
            for k, P in enumerate(Ps):
                pl.set_sinogram(k, P.ravel(order="F"))
            pl.reset()
            pl.run()
            return [pl.image(k) for k in range(len(Ps))], pl.chord_slots

    with_tab, slots = run()
    monkeypatch.setenv("ASDPOCS_NO_CHORD_TABLE", "1")
    without, slots_direct = run()
    assert slots > 0 and slots_direct == 0
    for k in range(len(Ps)):
        assert np.array_equal(with_tab[k], without[k]), k


@pytest.mark.parametrize("dims", [(48, 40, 36, 96, 72, 0.8 * 256 / 48 * 96 / 512),
                                  (17, 13, 11, 41, 9, 1.3)])
def test_cone_beam_z_column_step_equals_per_voxel_step(gpu, monkeypatch, dims):
    """The cone-beam backward step walked down voxel columns gives the same
    images, bit for bit, as the per-voxel step (ASDPOCS_CONE_ATX=voxel),
    through whole reconstructions: one instance, and a batch of instances of
    different sizes.  The odd detector (41 bins) puts an axis-parallel ray in
    the views at 0 and 90 degrees, where both forms walk the reference's
    whole window."""
    nx, ny, nz, na, nb, det = dims
    SO, OD = 1000.0, 500.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, nx)
    phi = np.concatenate([[0.0, 90.0], phantoms.views(6) + 7.0])
    base = dict(SO=SO, OD=OD, vxlsize=vx, nx=nx, ny=ny, nz=nz, na=na, nb=nb, detsize=det,
                phi_vec=phi, maxnumIter=2, numOfgradients=3, alpha=0.02)
    paras = [base, dict(base, nx=nx - 5, nz=nz + 3, maxnumIter=3)]
    rng = np.random.default_rng(nx + nz)
    Ps = [rng.random((na * nb, len(phi))).astype(np.float32) for _ in paras]

    def run(form, ps):
        if form:
            monkeypatch.setenv("ASDPOCS_CONE_ATX", form)
        else:
            monkeypatch.delenv("ASDPOCS_CONE_ATX", raising=False)
        with pkg.Plan(ps, [phi] * len(ps)) as pl:
            for k, Pk in enumerate(Ps[:len(ps)]):
                pl.set_sinogram(k, Pk.ravel(order="F"))
            pl.reset()
            pl.run()
            return [pl.image(k) for k in range(len(ps))]

    for ps in (paras[:1], paras):
        zc, vox = run(None, ps), run("voxel", ps)
        for a, b in zip(zc, vox):
            assert np.array_equal(a, b), rel_l2(a, b)


@pytest.mark.parametrize("dims", [(64, 64, 1, 128, 1, 1.0), (20, 20, 20, 40, 30, 10.24)])
def test_exact_forward_mode_reconstruction_vs_oracle(gpu, oracle_mod, dims):
    """A plan with ax_mode="exact" (SART forward steps through the exact
    Siddon projection) against the oracle's ASD-POCS driver with the FP64
    Siddon forward projector; a batch of exact instances of different sizes
    gives each instance's image alone, bit for bit."""
    nx, ny, nz, na, nb, det = dims
    SO, OD = (541.0, 408.0) if nz == 1 else (1000.0, 500.0)
    vx = phantoms.fov_voxel_size(SO, OD, det, na, nx)
    x = (phantoms.shepp_logan_2d(nx) if nz == 1 else phantoms.shepp_logan_3d(nx) * 0.02)
    x = x.astype(np.float32)
    phi = phantoms.views(9)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=nx, ny=ny, nz=nz, na=na, nb=nb, detsize=det,
                phi_vec=phi, maxnumIter=3, numOfgradients=5, alpha=0.002, ax_mode="exact")
    P = np.stack([oracle_mod.siddon_ax(x, oracle_mod.gateway_geometry(
        -a / 180 * np.pi, SO, OD, vx, det, na, nb), nx, ny, nz)[0] for a in phi], axis=1)
    m, out = pkg.ASD_POCS_cuda(P, dict(para, I0=x))
    mo, oo = oracle_mod.asdpocs(P, dict(para, I0=x.astype(np.float64)), impl="siddon")
    assert out["IterationNum"] == oo["IterationNum"]
    assert rel_l2(m.ravel(order="F"), mo) < RECON_TOL, rel_l2(m.ravel(order="F"), mo)
    np.testing.assert_allclose(out["RMSE"], oo["RMSE"], rtol=1e-4)
    # a batch: this instance and a smaller one, both exact
    other = dict(para, nx=nx - 3, na=na - 5)
    Po = np.random.default_rng(1).random(((na - 5) * nb, len(phi))).astype(np.float32)
    alone = []
    for pa, Pk in ((para, P), (other, Po)):
        with pkg.Plan(pa, phi) as pl:
            pl.set_sinogram(0, np.asarray(Pk, np.float32).ravel(order="F"))
            pl.reset()
            pl.run()
            alone.append(pl.image(0))
    with pkg.Plan([para, other], [phi, phi]) as pl:
        for k, Pk in enumerate((P, Po)):
            pl.set_sinogram(k, np.asarray(Pk, np.float32).ravel(order="F"))
        pl.reset()
        pl.run()
        for k in range(2):
            assert np.array_equal(pl.image(k), alone[k]), k


def test_exact_mode_rules(gpu):
    """One forward mode per plan; the serving queue refuses exact-mode jobs."""
    para = dict(SO=541.0, OD=408.0, vxlsize=1.0, nx=16, ny=16, nz=1, na=32, nb=1,
                detsize=1.0, phi_vec=phantoms.views(4), maxnumIter=1)
    with pytest.raises(pkg.AsdpocsError, match="one forward mode"):
        pkg.Plan([para, dict(para, ax_mode="exact")], [para["phi_vec"]] * 2)
    with pkg.Server() as srv:
        with pytest.raises(pkg.AsdpocsError, match="reference forward mode only"):
            srv.submit(dict(para, ax_mode="exact"), np.zeros((32, 4), np.float32))


def test_headline_fan_beam_geometry_vs_oracle(gpu, oracle_mod):
    """The measured fan-beam workload's geometry at full size -- a 512^2
    random-ellipse phantom (0-0.04 /mm, 0.9887 mm voxels), 60 views over 360
    degrees, 888 bins at 1.0 mm, SID 541 / SDD 949 mm, Poisson noise at
    I0 = 1e5 -- reconstructed on the GPU and by the oracle (FP64 image
    state): 4 iterations of 20 TV steps at a well-conditioned alpha, within
    the 2e-4 bar, with the same RMSE trajectory.  (At the workload's own
    alpha = 0.2 the iteration is chaotic: a 1e-7 change of P moves the
    oracle's image by ~3e-2, so only the RMSE can be compared there.)"""
    n, na, nv = 512, 888, 60
    SO, OD, det = 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    x = phantoms.random_ellipses(n, 0).astype(np.float32)
    phi = phantoms.views(nv)
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=4, numOfgradients=20, alpha=0.002, r_max=0.95,
                alpha_red=0.95)
    P = np.stack([pkg.Ax_cone_gpu(x, dict(para, phi=-a / 180 * np.pi))[0] for a in phi],
                 axis=1)
    P = phantoms.poisson_noise(P, 1e5, 0)
    m, out = pkg.ASD_POCS_cuda(P, dict(para, I0=x))
    mo, oo = oracle_mod.asdpocs(P, dict(para, I0=x.astype(np.float64)))
    assert out["IterationNum"] == oo["IterationNum"] == 4
    assert rel_l2(m.ravel(order="F"), mo) < RECON_TOL, rel_l2(m.ravel(order="F"), mo)
    np.testing.assert_allclose(out["RMSE"], oo["RMSE"], rtol=1e-4)


def test_launch_shapes_do_not_change_results(gpu):
    """Every launch shape the autotuner chooses from gives the same images,
    bit for bit: the shared forward step's loads per round and quads per
    block (fan and cone beams), the cone-beam backward step's column segment,
    and programmatic dependent launches; so does the autotuner's pick."""
    def recon(paras, phis, Ps, **shape):
        with pkg.Plan(paras, phis) as pl:
            for k, Pk in enumerate(Ps):
                pl.set_sinogram(k, Pk)
            if shape.pop("auto", False):
                chosen = pl.autotune_shapes(reps=2)
                assert chosen["iteration_ms"] > 0
            elif shape:
                pl.set_shapes(**shape)
            pl.reset()
            pl.run()
            return [pl.image(k) for k in range(len(Ps))]

    rng = np.random.default_rng(12)
    fan = dict(SO=541.0, OD=408.0, vxlsize=1.2, nx=48, ny=40, nz=1, na=80, nb=1, detsize=1.0,
               maxnumIter=2, numOfgradients=4, alpha=0.02)
    cone = dict(SO=1000.0, OD=500.0, vxlsize=1.0, nx=24, ny=20, nz=30, na=48, nb=40,
                detsize=1.5, maxnumIter=2, numOfgradients=3, alpha=0.02)
    phi = phantoms.views(7)
    for base, batch in ((fan, 11), (cone, 9), (cone, 1)):
        paras = [base] * batch
        Ps = [rng.random(base["na"] * base["nb"] * len(phi)).astype(np.float32)
              for _ in range(batch)]
        ref = recon(paras, [phi] * batch, Ps)
        shapes = [dict(ax_cols=u, ax_quads=q) for u in (1, 2) for q in (1, 2)]
        shapes += [dict(zcol_segment=z) for z in (8, 16, 64)]
        shapes += [dict(pdl=0), dict(pdl=1), dict(auto=True)]
        for sh in shapes:
            out = recon(paras, [phi] * batch, Ps, **dict(sh))
            for a, b in zip(ref, out):
                assert np.array_equal(a, b), (batch, sh)
