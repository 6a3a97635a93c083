"""The bounds-checked build (libasdpocs_gb300_checked.so, -DASDPOCS_CHECKED):
every volume, sinogram, residual and table index of the projector and TV
kernels is checked before its access, a bad one counted and skipped (never
trapped).  Odd and degenerate sizes -- n = 1, 3, 17; na = 1; nz = 1; nb = 1
and 2; cone beams with single detector rows or columns -- run through the
launchers, the exact projector, the TV entry points, ASD-POCS plans (single,
shared-geometry and uneven batches, both forward modes) and a served job,
and the count must stay 0.  The run uses a child process because the
checked library is selected at load time (ASDPOCS_LIB=checked)."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import ctypes as C, json, sys
import numpy as np
sys.path.insert(0, ROOT)
import asd_pocs_mex_cuda_demo_gb300 as pkg
from asd_pocs_mex_cuda_demo_gb300 import phantoms
from asd_pocs_mex_cuda_demo_gb300._lib import check, load

L = load()
assert b"bounds-checked" in L.asdpocs_version()
rng = np.random.default_rng(0)
CASES = [(1, 1, 1, 3, 1), (3, 3, 1, 1, 1), (17, 17, 1, 33, 1), (3, 17, 1, 5, 2),
         (17, 3, 1, 1, 2), (3, 3, 3, 5, 5), (17, 9, 5, 33, 7), (1, 1, 17, 3, 3),
         (17, 17, 17, 1, 1), (3, 17, 9, 1, 2), (16, 16, 33, 7, 9)]
done = []
for (nx, ny, nz, na, nb) in CASES:
    SO, OD, det = 300.0, 200.0, 1.3
    vx = phantoms.fov_voxel_size(SO, OD, det, max(na, 2), nx)
    x = rng.random(nx * ny * nz).astype(np.float32)
    yv = rng.standard_normal(na * nb).astype(np.float32)
    for a in (0.0, 33.0, 90.0, 217.0):
        para = dict(SO=SO, OD=OD, vxlsize=vx, nx=nx, ny=ny, nz=nz, na=na, nb=nb,
                    phi=-a / 180 * np.pi, detsize=det)
        pkg.Ax_cone_gpu(x, para)
        pkg.Atx_cone_gpu(yv, para)
    phi = phantoms.views(5) + 3.0
    para = dict(SO=SO, OD=OD, vxlsize=vx, nx=nx, ny=ny, nz=nz, na=na, nb=nb, detsize=det,
                phi_vec=phi, maxnumIter=2, numOfgradients=3, alpha=0.002)
    P = rng.random((na * nb, len(phi)))
    pkg.ASD_POCS_cuda(P, para)
    pkg.ASD_POCS_cuda(P, dict(para, ax_mode="exact"))
    pkg.ASD_POCS_cuda(P, dict(para, sino_storage="f16"))
    # shared geometry (identical instances) and an uneven batch
    other = dict(para, nx=nx + 2, na=na + 1)
    for ps in ([para, para, para], [para, other]):
        with pkg.Plan(ps, [phi] * len(ps)) as pl:
            for k, p in enumerate(ps):
                pl.set_sinogram(k, rng.random(p["na"] * p["nb"] * len(phi)).astype(np.float32))
            pl.reset()
            pl.run()
    img = rng.random((nx, ny, nz)) if nz > 1 else rng.random((nx, ny))
    if nz > 1:
        pkg.imgTVGradMin3D(img, 0.2, 4, 1, img * 0.9)
    else:
        pkg.imgTVGradMin(img, 0.2, 4, 1, img * 0.9)
    done.append([nx, ny, nz, na, nb])
with pkg.Server(slots_per_lane=2) as srv:
    for (nx, ny, nz, na, nb) in CASES[:6]:
        vx = phantoms.fov_voxel_size(300.0, 200.0, 1.3, max(na, 2), nx)
        p = dict(SO=300.0, OD=200.0, vxlsize=vx, nx=nx, ny=ny, nz=nz, na=na, nb=nb,
                 detsize=1.3, phi_vec=phantoms.views(4), maxnumIter=2, numOfgradients=2)
        srv.wait(srv.submit(p, rng.random((na * nb, 4)).astype(np.float32)))
cnt = C.c_ulonglong()
first = (C.c_longlong * 2)()
check(L.asdpocs_checked_errors(C.byref(cnt), first))
print(json.dumps({"count": cnt.value, "first": [first[0], first[1]], "cases": done}))
"""


def test_bounds_checked_build_sees_no_bad_index(gpu):
    from asd_pocs_mex_cuda_demo_gb300 import build

    build.build(checked=True)
    env = dict(os.environ, ASDPOCS_LIB="checked")
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + SCRIPT], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert len(out["cases"]) == 11
    assert out["count"] == 0, out
