"""Generate the golden vectors in this directory from the REFERENCE'S OWN CODE.

Run where the reference checkout exists (its sources are compiled for the host
by oracle/build_ref.sh into oracle/_ref/libasdref.so):

    python tests/golden/make_golden.py

Each fixture stores the inputs and the outputs of the reference's
src/AxAtx gateway+kernels or src/tvmin functions; the ASD-POCS fixture runs
the oracle's restatement of utilities/ASD_POCS_cuda.m with the reference's
projector and TV code plugged in.  Sizes are small so the files stay a few
hundred KB.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from asd_pocs_mex_cuda_demo_gb300 import phantoms  # noqa: E402

# (name, nx, ny, nz, na, nb, SO, OD, detsize, angles in degrees)
PROJ_CASES = [
    ("fan2d_64", 64, 64, 1, 128, 1, 541.0, 408.0, 1.0, [0, 17, 30, 45, 60, 90, 123, 180, 271.5]),
    ("fan2d_odd", 17, 23, 1, 41, 1, 541.0, 408.0, 1.0, [0, 33, 90, 200]),
    ("fan2d_nb2", 48, 48, 1, 96, 2, 405.941, 500.31, 0.148 * 4, [0, 45, 100]),
    ("cone3d_24", 24, 24, 12, 48, 24, 1000.0, 500.0, 0.8 * 4, [0, 30, 45, 123]),
    ("cone3d_odd", 13, 11, 7, 27, 9, 300.0, 200.0, 1.3, [0, 77, 250]),
]


def proj_fixture(name, nx, ny, nz, na, nb, SO, OD, det, angles, rng):
    vx = phantoms.fov_voxel_size(SO, OD, det, na, nx)
    x = rng.random(nx * ny * nz).astype(np.float32)
    yv = rng.random(na * nb).astype(np.float32)
    out = dict(dims=np.array([nx, ny, nz, na, nb]), geo=np.array([SO, OD, vx, det]),
               angles=np.array(angles, np.float64), x=x, yview=yv)
    ys, srs, bs, scs, trig = [], [], [], [], []
    for a in angles:
        phi = -a / 180 * np.pi
        para = dict(SO=SO, OD=OD, vxlsize=vx, nx=nx, ny=ny, nz=nz, phi=phi, detsize=det,
                    na=na, nb=nb)
        y, sr = oracle.ref_mex("Ax_cone_gpu", [x.reshape(-1, 1), para], nlhs=2)
        b, sc = oracle.ref_mex("Atx_cone_gpu", [yv.reshape(-1, 1), para], nlhs=2)
        g = oracle.gateway_geometry(phi, SO, OD, vx, det, na, nb)
        trig.append([g["cos_phi"], g["sin_phi"]])
        ys.append(y.ravel()); srs.append(sr.ravel()); bs.append(b.ravel()); scs.append(sc.ravel())
    out.update(y=np.array(ys), sr=np.array(srs), bp=np.array(bs), sc=np.array(scs),
               trig=np.array(trig, np.float32))
    np.savez_compressed(os.path.join(HERE, f"proj_{name}.npz"), **out)


def tv_fixtures(rng):
    img2 = rng.random((40, 30)); old2 = rng.random((40, 30))
    out2 = oracle.ref_mex("imgTVGradMin", [img2, 0.2, 20, 1, old2])[0]
    out2b = oracle.ref_mex("imgTVGradMin", [img2 - 0.5, 0.05, 7, 0])[0]
    img3 = rng.random((20, 18, 7)); old3 = rng.random((20, 18, 7))
    out3 = oracle.ref_mex("imgTVGradMin3D", [img3, 0.2, 20, 1, old3])[0]
    np.savez_compressed(os.path.join(HERE, "tv.npz"), img2=img2, old2=old2, out2=out2,
                        out2_nopos=out2b, img3=img3, old3=old3, out3=out3)


def asdpocs_fixture():
    # 2D fan-beam, 64^2 modified Shepp-Logan, 36 views, noiseless
    n, na, nv, SO, OD, det = 64, 128, 36, 541.0, 408.0, 1.0
    vx = phantoms.fov_voxel_size(SO, OD, det, na, n)
    x = phantoms.shepp_logan_2d(n)
    phi = phantoms.views(nv)
    P = np.zeros((na, nv))
    for i, a in enumerate(phi):
        para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, phi=-a / 180 * np.pi,
                    detsize=det, na=na, nb=1)
        P[:, i] = oracle.ref_mex("Ax_cone_gpu", [x.astype(np.float32).reshape(-1, 1), para],
                                 nlhs=2)[0].ravel()
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=n, ny=n, nz=1, na=na, nb=1, detsize=det,
                phi_vec=phi, maxnumIter=6, alpha=0.2, alpha_red=0.95, I0=x)
    m, out = oracle.asdpocs(P, para, impl="reference")
    # The reference's TV step (alpha*||m - m0||, ASD_POCS_cuda.m:151-158) is so
    # large at alpha=0.2 that the iteration is chaotic: a 1e-7 relative change
    # of P moves m by ~3e-2.  A second run at alpha=0.002 is well conditioned
    # and pins the reconstruction tightly.
    paras = dict(para, alpha=0.002)
    ms, outs = oracle.asdpocs(P, paras, impl="reference")
    # 3D cone-beam, 16^3, 20 views, Poisson noise
    n3, na3, nb3, nv3 = 16, 32, 16, 20
    SO3, OD3, det3 = 1000.0, 500.0, 0.8 * 16
    vx3 = phantoms.fov_voxel_size(SO3, OD3, det3, na3, n3)
    x3 = phantoms.shepp_logan_3d(n3) * 0.02
    phi3 = phantoms.views(nv3)
    P3 = np.zeros((na3 * nb3, nv3))
    for i, a in enumerate(phi3):
        para3 = dict(SO=SO3, OD=OD3, vxlsize=vx3, nx=n3, ny=n3, nz=n3,
                     phi=-a / 180 * np.pi, detsize=det3, na=na3, nb=nb3)
        P3[:, i] = oracle.ref_mex("Ax_cone_gpu", [x3.astype(np.float32).reshape(-1, 1),
                                                  para3], nlhs=2)[0].ravel()
    P3 = phantoms.poisson_noise(P3, 5e4, seed=3)
    para3 = dict(SO=SO3, OD=OD3, vxlsize=vx3, nx=n3, ny=n3, nz=n3, na=na3, nb=nb3,
                 detsize=det3, phi_vec=phi3, maxnumIter=4, alpha=0.2, I0=x3)
    m3, out3 = oracle.asdpocs(P3, para3, impl="reference")
    np.savez_compressed(
        os.path.join(HERE, "asdpocs.npz"),
        P2=P, phi2=phi, geo2=np.array([n, na, SO, OD, vx, det]), x2=x, m2=m,
        out2=np.array([out["IterationNum"], out["dataTolerance"], out["alpha"], out["beta"]]),
        rmse2=out["RMSE"],
        m2s=ms, rmse2s=outs["RMSE"],
        out2s=np.array([outs["IterationNum"], outs["dataTolerance"], outs["alpha"],
                        outs["beta"]]),
        P3=P3, phi3=phi3, geo3=np.array([n3, na3, nb3, SO3, OD3, vx3, det3]), x3=x3, m3=m3,
        out3=np.array([out3["IterationNum"], out3["dataTolerance"], out3["alpha"],
                       out3["beta"]]),
        rmse3=out3["RMSE"])


def main():
    if not oracle.ref_available():
        oracle.build()
    if not oracle.ref_available():
        sys.exit("reference host build unavailable: cannot regenerate golden vectors")
    rng = np.random.default_rng(20261203)
    for c in PROJ_CASES:
        proj_fixture(*c, rng=rng)
    tv_fixtures(rng)
    asdpocs_fixture()
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
