"""Serving queue: ASD-POCS jobs of any geometry submitted at any time,
continuously batched on one GPU (asdpocs_server_* in the C ABI).

    with Server(slots_per_lane=32) as srv:
        job = srv.submit(para, P, I0=phantom)      # para as for ASD_POCS_cuda
        m_res, out, times = srv.wait(job)

A job's image is the same, bit for bit, as the same reconstruction run
alone in a ``Plan``; ``times`` gives its queueing, run and total latency.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import JobTimes, ServerConfig, Stats, check, load
from .asdpocs import geometry_from_para, options_from_para

_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3


def _f32(a, n, what):
    a = np.asarray(a)
    if a.ndim > 1:
        a = a.ravel(order="F")
    a = np.ascontiguousarray(a, np.float32)
    if a.size != n:
        raise ValueError(f"{what}: expected {n} values, got {a.size}")
    return a


class Server:
    def __init__(self, slots_per_lane: int = 32, hbm_budget_bytes: int = 0,
                 inflight: int = 2):
        L = load()
        cfg = ServerConfig()
        L.asdpocs_server_config_default(C.byref(cfg))
        cfg.slots_per_lane = int(slots_per_lane)
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.inflight = int(inflight)
        h = C.c_void_p()
        check(L.asdpocs_server_create(C.byref(h), C.byref(cfg)))
        self._h = h
        self._jobs = {}

    def submit(self, para: dict, P, m0=None, I0=None) -> int:
        """Queue one reconstruction: ``para`` with ``phi_vec`` (degrees) and
        the ASD_POCS_cuda options, sinogram P ((na*nb) x nv)."""
        phi = np.ascontiguousarray(np.asarray(para["phi_vec"], np.float64).ravel())
        g = geometry_from_para(para, phi.size)
        o = options_from_para(para)
        N = g.nx * g.ny * g.nz
        Pf = _f32(P, g.na * g.nb * g.nv, "sinogram")
        m0f = None if m0 is None else _f32(m0, N, "m0")
        I0f = None if I0 is None else _f32(I0, N, "I0")
        job = C.c_longlong()
        check(load().asdpocs_server_submit(
            self._h, C.byref(g), phi.ctypes.data_as(_D), C.byref(o), Pf.ctypes.data_as(_F),
            None if m0f is None else m0f.ctypes.data_as(_F),
            None if I0f is None else I0f.ctypes.data_as(_F), C.byref(job)))
        self._jobs[job.value] = (N, o.maxnumIter, I0 is not None)
        return job.value

    def poll(self, job: int) -> int:
        st = C.c_int()
        check(load().asdpocs_server_poll(self._h, int(job), C.byref(st)))
        return st.value

    def cancel(self, job: int):
        """Cancel a queued or running job (its slot and memory are released in
        stream order; the other jobs are unaffected).  The job must still be
        collected with wait(), which then raises AsdpocsError."""
        check(load().asdpocs_server_cancel(self._h, int(job)))

    def wait(self, job: int):
        """Block until the job is done; returns (m_res, out, times)."""
        info = self._jobs.pop(job, None)
        if info is None:  # unknown or already taken: the library reports it
            check(load().asdpocs_server_wait(self._h, int(job), None, None, None, None))
        N, iters, has_ref = info
        img = np.empty(N, np.float32)
        rmse = np.zeros(max(iters, 1))
        st = Stats()
        t = JobTimes()
        check(load().asdpocs_server_wait(self._h, int(job), img.ctypes.data_as(_F),
                                         C.byref(st), rmse.ctypes.data_as(_D),
                                         C.byref(t)))
        out = dict(IterationNum=st.IterationNum, dataTolerance=st.dataTolerance,
                   alpha=st.alpha, beta=st.beta, dp=st.dp, dg=st.dg)
        if has_ref:
            out["RMSE"] = rmse[:st.IterationNum].copy()
        return img, out, dict(queued_ms=t.queued_ms, run_ms=t.run_ms,
                              total_ms=t.total_ms)

    def memory(self):
        """(device bytes held by admitted jobs, peak)."""
        a, b = C.c_ulonglong(), C.c_ulonglong()
        check(load().asdpocs_server_memory(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if getattr(self, "_h", None):
            load().asdpocs_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
