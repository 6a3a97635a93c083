"""ASD-POCS drivers mirroring utilities/ASD_POCS_cuda.m and
utilities/SART_cuda_inline.m, plus the batched device-resident ``Plan``.

The whole iteration (per-view SART with row/column normalisation and
positivity, the data residual, the TV steepest descent and the adaptive
alpha/beta step control) runs on the GPU; FP64 is used on the device only
for the scalars (dd2, dp, dg, TV norms, alpha, beta).  Images and sinograms
are FP32 on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (AX_MODE, SINO_STORAGE, AsdpocsError, Geometry, Options, Shapes, Stats,
                   check, load)

_D = C.POINTER(C.c_double)
_EPS = float(np.finfo(np.float64).eps)


def options_from_para(para: dict) -> Options:
    """ASD_POCS_cuda.m:34-96: absent fields take the reference defaults."""
    o = Options()
    load().asdpocs_options_default(C.byref(o))

    def get(name, default):
        v = para.get(name)
        return default if v is None else v

    o.maxnumIter = int(get("maxnumIter", 5))
    o.numOfgradients = int(get("numOfgradients", 20))
    o.alpha = float(get("alpha", 0.02))
    o.alpha_red = float(get("alpha_red", 0.95))
    o.beta = float(get("beta", 1.0))
    o.beta_red = float(get("beta_red", 0.995))
    o.r_max = float(get("r_max", 0.95))
    o.epsilon = float(get("epsilon", _EPS))
    o.stopRelChg = float(get("stopRelChg", _EPS))
    # not in the reference: "f32" (default), "f16" or "bf16" device storage of P
    s = get("sino_storage", "f32")
    o.sino_storage = SINO_STORAGE[s] if isinstance(s, str) else int(s)
    # not in the reference: "reference" column march (default) or "exact" Siddon
    a = get("ax_mode", "reference")
    o.ax_mode = AX_MODE[a] if isinstance(a, str) else int(a)
    return o


def geometry_from_para(para: dict, nv: int) -> Geometry:
    g = Geometry()
    g.nx, g.ny, g.nz = int(para["nx"]), int(para["ny"]), int(para["nz"])
    g.na, g.nb, g.nv = int(para["na"]), int(para["nb"]), int(nv)
    g.SO, g.OD = float(para["SO"]), float(para["OD"])
    g.vxlsize, g.detsize = float(para["vxlsize"]), float(para["detsize"])
    return g


def _prep(P, para):
    P = np.asarray(P, dtype=np.float64)
    if P.ndim == 1:
        P = P.reshape(-1, 1)
    nv = P.shape[1]
    phi = np.ascontiguousarray(np.asarray(para["phi_vec"], np.float64).ravel())
    if nv != phi.size:
        raise AsdpocsError(1, "Size of Projection and phi_vec mismatch!")
    g = geometry_from_para(para, nv)
    if P.shape[0] != g.na * g.nb:
        raise AsdpocsError(1, "Size of Projection and na*nb mismatch!")
    return np.ascontiguousarray(P.ravel(order="F")), phi, g


def _vol(a, g):
    if a is None:
        return None
    a = np.asarray(a, np.float64)
    if a.size != g.nx * g.ny * g.nz:
        raise AsdpocsError(1, "image size does not match nx*ny*nz")
    return np.ascontiguousarray(a.ravel(order="F"))


def ASD_POCS_cuda(P, para: dict):
    """[m_res, out] = ASD_POCS_cuda(P, para).

    P: (na*nb) x nv projections (column per view); para: the reference's
    struct as a dict (nx ny nz SO OD vxlsize detsize na nb phi_vec and the
    optional maxnumIter numOfgradients alpha alpha_red beta beta_red r_max
    epsilon stopRelChg m0 initBySART lambda I0).  Returns m_res as an
    [nx, ny, nz] array (the post-SART image of the last iteration, as the
    reference returns) and the ``out`` struct as a dict.
    """
    Pf, phi, g = _prep(P, para)
    o = options_from_para(para)
    m0 = _vol(para.get("m0"), g)
    if m0 is None and para.get("initBySART"):
        m0, _ = SART_cuda_inline(P, {**para, "m0": None})
        m0 = _vol(m0, g)
    I0 = _vol(para.get("I0"), g)
    N = g.nx * g.ny * g.nz
    m_res = np.zeros(N)
    rmse = np.zeros(max(o.maxnumIter, 1))
    st = Stats()
    check(load().ASD_POCS_cuda(Pf.ctypes.data_as(_D), phi.ctypes.data_as(_D), C.byref(g),
                               C.byref(o), None if m0 is None else m0.ctypes.data_as(_D),
                               None if I0 is None else I0.ctypes.data_as(_D),
                               m_res.ctypes.data_as(_D), rmse.ctypes.data_as(_D),
                               C.byref(st)))
    out = dict(IterationNum=st.IterationNum, dataTolerance=st.dataTolerance,
               beta=st.beta, alpha=st.alpha, reconImg=None)
    m_res = m_res.reshape((g.nx, g.ny, g.nz), order="F")
    out["reconImg"] = m_res
    if I0 is not None:
        out["RMSE"] = rmse[:st.IterationNum].copy()
    return m_res, out


def SART_cuda_inline(P, para: dict):
    """[m, out] = SART_cuda_inline(P, para): one SART sweep, relaxation
    ``para['lambda']`` (default 1), starting from ``para['m0']`` or zeros."""
    Pf, phi, g = _prep(P, para)
    lam = para.get("lambda")
    lam = 1.0 if lam is None else float(lam)
    m0 = _vol(para.get("m0"), g)
    N = g.nx * g.ny * g.nz
    m = np.zeros(N)
    dt = np.zeros(1)
    check(load().SART_cuda_inline(Pf.ctypes.data_as(_D), phi.ctypes.data_as(_D),
                                  C.byref(g), lam,
                                  None if m0 is None else m0.ctypes.data_as(_D),
                                  m.ctypes.data_as(_D), dt.ctypes.data_as(_D)))
    out = dict(IterationNum=1, dataTolerance=float(dt[0]), **{"lambda": lam})
    return m, out


def _plan_args(paras, phi_vecs):
    """The batch descriptor of asdpocs_plan_create: geometries, options and
    the concatenated angle lists."""
    if isinstance(paras, dict):
        paras = [paras]
    batch = len(paras)
    phis = [np.asarray(p, np.float64).ravel() for p in
            (phi_vecs if isinstance(phi_vecs, (list, tuple)) else [phi_vecs] * batch)]
    if len(phis) != batch:
        raise AsdpocsError(1, "one phi_vec per instance")
    geoms = (Geometry * batch)(*[geometry_from_para(p, ph.size) for p, ph in zip(paras, phis)])
    opts = (Options * batch)(*[options_from_para(p) for p in paras])
    return geoms, opts, np.ascontiguousarray(np.concatenate(phis))


def plan_layout(paras, phi_vecs):
    """How a Plan of these instances would run, computed on the host without
    a GPU (asdpocs_plan_layout): (group of each instance, -1 when it runs
    through the per-instance kernels; sub-batch of each instance; number of
    sub-batches)."""
    geoms, opts, phi = _plan_args(paras, phi_vecs)
    n = len(geoms)
    group_of = (C.c_int * n)()
    sub_of = (C.c_int * n)()
    rc = load().asdpocs_plan_layout(n, geoms, phi.ctypes.data_as(_D), opts, group_of, sub_of)
    if rc < 0:
        check(-rc)
    return list(group_of), list(sub_of), rc


class Plan:
    """A batch of device-resident ASD-POCS reconstructions (per-instance
    sizes, geometry values, angles and options).  Instances of one plan are
    all 2-D (nz == nb == 1) or all cone-beam; the kernels run every instance
    in one launch per step, each at its own sizes, and an instance gives the
    same result bit for bit alone or in any batch.

    Data go in as float32 (host numpy arrays or device pointers as ints) and
    the whole iteration runs on the plan's CUDA stream, optionally replayed
    from a CUDA graph."""

    def __init__(self, paras, phi_vecs, hbm_budget_bytes: int = 0, stream: int = 0):
        geoms, opts, phi = _plan_args(paras, phi_vecs)
        self.batch = len(geoms)
        self._geoms = geoms
        self._opts = opts
        h = C.c_void_p()
        check(load().asdpocs_plan_create(C.byref(h), self.batch, geoms,
                                         phi.ctypes.data_as(_D), opts,
                                         int(hbm_budget_bytes), C.c_void_p(stream or None)))
        self._h = h
        g0 = geoms[0]
        # sizes of instance 0 (every instance of a uniform plan)
        self.nx, self.ny, self.nz = g0.nx, g0.ny, g0.nz
        self.na, self.nb, self.nv = g0.na, g0.nb, g0.nv

    def voxels(self, inst: int) -> int:
        g = self._geoms[inst]
        return g.nx * g.ny * g.nz

    def sinogram_size(self, inst: int) -> int:
        g = self._geoms[inst]
        return g.na * g.nb * g.nv

    @property
    def nbytes(self) -> int:
        return int(load().asdpocs_plan_bytes(self._h))

    def close(self):
        if getattr(self, "_h", None):
            load().asdpocs_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- data
    def _put(self, fn, inst, arr, n):
        L = load()
        if arr is None:
            check(getattr(L, fn)(self._h, inst, None, 0))
        elif isinstance(arr, int):
            check(getattr(L, fn)(self._h, inst, C.c_void_p(arr), 1))
        else:
            a = np.asarray(arr)
            if a.ndim > 1:
                a = a.ravel(order="F")
            a = np.ascontiguousarray(a, np.float32)
            if a.size != n:
                raise AsdpocsError(1, f"expected {n} values, got {a.size}")
            check(getattr(L, fn)(self._h, inst, C.c_void_p(a.ctypes.data), 0))

    def set_sinogram(self, inst: int, P):
        self._put("asdpocs_plan_set_sinogram", inst, P, self.sinogram_size(inst))

    def set_initial(self, inst: int, m0):
        self._put("asdpocs_plan_set_initial", inst, m0, self.voxels(inst))

    def set_reference(self, inst: int, I0):
        self._put("asdpocs_plan_set_reference", inst, I0, self.voxels(inst))

    def reset(self):
        check(load().asdpocs_plan_reset(self._h))

    def run(self, use_graph: bool = True, sync: bool = True):
        check(load().asdpocs_plan_run(self._h, 1 if use_graph else 0))
        if sync:
            self.sync()

    def sync(self):
        check(load().asdpocs_plan_sync(self._h))

    def image(self, inst: int) -> np.ndarray:
        out = np.empty(self.voxels(inst), np.float32)
        check(load().asdpocs_plan_get_image(self._h, inst, C.c_void_p(out.ctypes.data), 0))
        return out

    def stats(self, inst: int):
        st = Stats()
        n = max(self._opts[inst].maxnumIter, 1)
        rmse = np.zeros(n)
        check(load().asdpocs_plan_get_stats(self._h, inst, C.byref(st),
                                            rmse.ctypes.data_as(_D)))
        return dict(IterationNum=st.IterationNum, dataTolerance=st.dataTolerance,
                    alpha=st.alpha, beta=st.beta, dp=st.dp, dg=st.dg,
                    RMSE=rmse[:st.IterationNum].copy())

    def time_phase(self, phase: int, reps: int = 20) -> float:
        """Average device milliseconds per launch of one phase kernel
        (0 SART forward, 1 SART backward, 2 TV step, 3 sweep scalars) for the
        whole batch; leaves the state modified (call reset())."""
        ms = C.c_double()
        check(load().asdpocs_plan_time_phase(self._h, int(phase), int(reps), C.byref(ms)))
        return ms.value

    def autotune(self, reps: int = 20):
        """Times the TV step at each candidate walk length and keeps the
        fastest (results do not depend on it); returns (walk, ms per step),
        walk 0 meaning the batch-size rule.  Leaves the reconstruction state
        unchanged."""
        w, ms = C.c_int(), C.c_double()
        check(load().asdpocs_plan_autotune(self._h, int(reps), C.byref(w), C.byref(ms)))
        return w.value, ms.value

    def autotune_shapes(self, reps: int = 10) -> dict:
        """Times every launch shape that applies to the plan (TV walk, the
        shared forward step's loads per round and quads per block, the
        cone-beam backward step's column segment, programmatic launches) on
        its own data and keeps the fastest; no shape changes a result bit.
        Resets the plan.  Returns the chosen shapes and the iteration's
        device milliseconds."""
        sh = Shapes()
        check(load().asdpocs_plan_autotune_shapes(self._h, int(reps), C.byref(sh)))
        return {f: getattr(sh, f) for f, _ in Shapes._fields_}

    @property
    def shapes(self) -> dict:
        sh = Shapes()
        check(load().asdpocs_plan_get_shapes(self._h, C.byref(sh)))
        return {f: getattr(sh, f) for f, _ in Shapes._fields_ if f != "iteration_ms"}

    def set_shapes(self, **kw):
        """Sets launch shapes by name (tv_walk, ax_cols, ax_quads,
        zcol_segment, pdl); 0 = the default, pdl -1 = auto."""
        sh = Shapes()
        check(load().asdpocs_plan_get_shapes(self._h, C.byref(sh)))
        for k, v in kw.items():
            setattr(sh, k, int(v))
        check(load().asdpocs_plan_set_shapes(self._h, C.byref(sh)))

    @property
    def streams(self) -> int:
        """Sub-batches run concurrently on their own streams."""
        return int(load().asdpocs_plan_streams(self._h))

    @property
    def chord_slots(self) -> int:
        """Chord slots per voxel of the backward step's chord tables (2-D
        plans of one instance or of instances sharing geometry), 0 when the
        plan computes chords every step."""
        return int(load().asdpocs_plan_chord_slots(self._h))

    def set_tv_walk(self, walk: int):
        """Pins the TV walk length (bands or slabs per walk; 0: the
        batch-size rule)."""
        check(load().asdpocs_plan_set_tv_walk(self._h, int(walk)))

    def sinogram_ptr(self, inst: int) -> int:
        """Device pointer of the instance's FP32 sinogram; 0 for FP16 / BF16
        storage (load those through set_sinogram)."""
        return int(load().asdpocs_plan_sinogram_ptr(self._h, inst) or 0)

    def image_ptr(self, inst: int) -> int:
        return int(load().asdpocs_plan_image_ptr(self._h, inst))
