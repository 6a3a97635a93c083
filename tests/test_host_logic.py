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


def _fan(n, nv, gseed, na=None):
    """A 2-D instance's para and angles: equal (n, nv, gseed) means equal
    geometry."""
    para = dict(SO=541.0, OD=408.0, vxlsize=1.0, nx=n, ny=n, nz=1, na=na or 2 * n, nb=1,
                detsize=1.0, maxnumIter=5, numOfgradients=4)
    return para, phantoms.views(nv) + 0.5 * gseed


def _layout(insts):
    return pkg.plan_layout([p for p, _ in insts], [ph for _, ph in insts])


def _check_layout(insts, group_of, sub_of, nsub):
    """Invariants of any plan layout: a group's instances share sizes, views
    and angles, at most eight per group, each group in one sub-batch; every
    instance in one sub-batch; at most eight sub-batches."""
    assert 1 <= nsub <= 8
    assert all(0 <= s < nsub for s in sub_of)
    groups = {}
    for i, g in enumerate(group_of):
        if g >= 0:
            groups.setdefault(g, []).append(i)
    for members in groups.values():
        assert len(members) <= 8
        p0, ph0 = insts[members[0]]
        for i in members:
            p, ph = insts[i]
            assert (p["nx"], p["na"], len(ph)) == (p0["nx"], p0["na"], len(ph0))
            assert np.array_equal(ph, ph0)
            assert sub_of[i] == sub_of[members[0]]
    return groups


def test_plan_layout_uniform_batch(lib):
    """64 instances of one geometry: groups of eight in instance order, two
    sub-batches of whole groups."""
    insts = [_fan(64, 12, 0)] * 64
    group_of, sub_of, nsub = _layout(insts)
    _check_layout(insts, group_of, sub_of, nsub)
    assert group_of == [i // 8 for i in range(64)]
    assert nsub == 2 and sub_of == [i // 32 for i in range(64)]


def test_plan_layout_mixed_geometries(lib):
    """Instances of several geometries listed out of order: each geometry's
    instances form groups of up to eight in instance order, a geometry of
    one instance a group of one; equal sizes share sub-batches, which split
    the work of the largest size class."""
    A, B, C = (48, 12, 1), (64, 20, 2), (33, 7, 3)
    spec = [A, B, C, B, A, B, B, C, B, B, B, A, B, B, B, (80, 30, 4)]
    insts = [_fan(*g) for g in spec]
    group_of, sub_of, nsub = _layout(insts)
    groups = _check_layout(insts, group_of, sub_of, nsub)
    b = [i for i, g in enumerate(spec) if g == B]  # ten instances of B
    assert sorted(len(m) for m in groups.values()) == [1, 2, 2, 3, 8]
    assert group_of[b[8]] == group_of[b[9]] != group_of[b[0]]  # eight, then two
    assert all(group_of[i] == group_of[b[0]] for i in b[:8])
    assert nsub == 5  # five groups, dealt over at most eight sub-batches


def test_plan_layout_without_shared_geometry(lib, monkeypatch):
    """Every instance of its own geometry runs through the per-instance
    kernels (no groups), sizes dealt to sub-batches by class; exact-mode
    plans and cone beams are never grouped."""
    insts = [_fan(32 + 8 * (k % 4), 5 + k, k) for k in range(12)]
    group_of, sub_of, nsub = _layout(insts)
    _check_layout(insts, group_of, sub_of, nsub)
    assert group_of == [-1] * 12 and nsub == 8
    for s in range(nsub):  # a sub-batch holds one size only (four classes)
        assert len({insts[i][0]["nx"] for i in range(12) if sub_of[i] == s}) == 1
    same = [_fan(48, 12, 1)] * 5 + [_fan(64, 20, 2)] * 3
    exact = [(dict(p, ax_mode="exact"), ph) for p, ph in same]
    group_of, sub_of, nsub = _layout(exact)
    assert group_of == [-1] * 8 and nsub == 8
    cone = [(dict(p, nz=p["nx"], nb=16), ph) for p, ph in same]
    group_of, _, _ = _layout(cone)
    assert group_of == [-1] * 8
    monkeypatch.setenv("ASDPOCS_NO_SHARED_GEOMETRY", "1")
    assert _layout(same)[0] == [-1] * 8


def test_plan_layout_rejects_like_create(lib):
    """The layout query checks its arguments as plan creation does."""
    p2, ph2 = _fan(32, 5, 0)
    p3 = dict(p2, nz=32, nb=16)
    with pytest.raises(pkg.AsdpocsError, match="all 2-D"):
        _layout([(p2, ph2), (p3, ph2)])
    with pytest.raises(pkg.AsdpocsError, match="forward mode"):
        _layout([(p2, ph2), (dict(p2, ax_mode="exact"), ph2)])
