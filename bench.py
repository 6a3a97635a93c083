#!/usr/bin/env python
"""ASD-POCS reconstructions per second on one GB300 (or N replicas).

Workload (the sparse-view clinical-head-slice configuration): 512x512
seeded random-ellipse phantoms (0-0.04 /mm), 60 views evenly spaced over
360 deg, 888 detector bins at 1.0 mm, SID 541 / SDD 949 mm (voxel 0.9887 mm
by the field-of-view rule), Poisson noise at I0 = 1e5 photons per bin,
100 ASD-POCS iterations (20 TV steps each, alpha 0.2, alpha_red 0.95,
r_max 0.95).  Synthetic seeded inputs stand in for real scans.

One step = one batch of --batch reconstructions run to completion from
their sinograms.  ``value`` is device-resident throughput (inputs in HBM,
CUDA events on the plan's stream); ``e2e`` runs the same batch through the
C ABI with host buffers, the sinogram upload and the image download inside
the timed region.  ``--impl reference`` times the reference's CPU path
instead (its host build where present, else the C restatement of it), on
all host cores, over a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ASD-POCS recons/s and p99 latency, batched/served vs plain, same GPU at matched RMSE"
N_PIX, N_BINS, N_VIEWS, SO, OD, DET = 512, 888, 60, 541.0, 408.0, 1.0
I0_PHOTONS = 1e5
WORKLOAD = "2D fan-beam sparse-view ASD-POCS, 512^2, 60 views/360deg, 888 bins, I0=1e5, 100 it"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")  # host-side barrier and max; no data collective
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch

    t = torch.tensor([float(v)])
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def para_for(seed):
    from asd_pocs_mex_cuda_demo_gb300 import phantoms

    vx = phantoms.fov_voxel_size(SO, OD, DET, N_BINS, N_PIX)
    return dict(SO=SO, OD=OD, vxlsize=vx, detsize=DET, nx=N_PIX, ny=N_PIX, nz=1,
                na=N_BINS, nb=1, maxnumIter=0, numOfgradients=20, alpha=0.2,
                alpha_red=0.95, r_max=0.95, beta=1.0, beta_red=0.995)


def make_inputs(B, iters, seed0, device):
    """Seeded phantoms, their noiseless projections (GPU projector) and
    Poisson-noise sinograms.  Setup only; not timed."""
    import torch

    from asd_pocs_mex_cuda_demo_gb300 import phantoms
    from asd_pocs_mex_cuda_demo_gb300._lib import check, load

    L = load()
    phi = phantoms.views(N_VIEWS)
    paras, Ps, I0s = [], [], []
    st = torch.cuda.current_stream().cuda_stream
    for b in range(B):
        p = para_for(seed0 + b)
        p["maxnumIter"] = iters
        x = phantoms.random_ellipses(N_PIX, seed0 + b).astype(np.float32)
        xd = torch.tensor(x, device=device)
        y = torch.empty(N_BINS * N_VIEWS, device=device)
        sr = torch.empty(N_BINS, device=device)
        vx = p["vxlsize"]
        sc = np.float32(vx)
        det = np.float32(DET) / sc
        ydet = torch.tensor(((np.arange(N_BINS) - N_BINS / 2.0 + 0.5) * np.float64(det))
                            .astype(np.float32), device=device)
        zdet = torch.zeros(1, device=device)
        for v, a in enumerate(phi):
            ph = np.float32(-(a / 180.0 * np.pi))
            check(L.asdpocs_ax_device(xd.data_ptr(), y.data_ptr() + 4 * N_BINS * v,
                                      sr.data_ptr(), float(np.cos(ph)), float(np.sin(ph)),
                                      ydet.data_ptr(), zdet.data_ptr(),
                                      float(np.float32(SO) / sc), float(np.float32(OD) / sc),
                                      float(sc), 1.0, N_PIX, N_PIX, 1, N_BINS, 1, st))
        torch.cuda.synchronize()
        P = phantoms.poisson_noise(y.cpu().numpy().astype(np.float64), I0_PHOTONS,
                                   seed=1000 + seed0 + b)
        paras.append(p)
        Ps.append(P.astype(np.float32))
        I0s.append(x)
    return paras, [phi] * B, Ps, I0s


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(paras, phis, Ps, sample_iters):
    """The C restatement of the reference's CPU path (OpenMP, all host
    threads) on one reconstruction of the workload, `sample_iters` iterations,
    extrapolated to the full iteration count."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    kind = "port"
    cores = os.cpu_count() or 1
    p = dict(paras[0], phi_vec=phis[0], maxnumIter=sample_iters)
    P = Ps[0].astype(np.float64).reshape(N_BINS, N_VIEWS, order="F")
    t = time.perf_counter()
    oracle.asdpocs(P, p, nthreads=cores)
    dt = time.perf_counter() - t
    full = paras[0]["maxnumIter"]
    per_recon = dt * full / sample_iters
    return {"value": 1.0 / per_recon, "unit": "recons/s", "cores": cores, "kind": kind,
            "sample": f"{sample_iters} of {full} ASD-POCS iterations of one 512^2 "
                      f"reconstruction ({dt:.1f} s), extrapolated"}


def main():
    args = parse()
    rank, world, local, pg = dist_init(args.gpus)
    if args.impl == "reference":
        return reference_arm(args, rank, world, pg)
    import torch

    import asd_pocs_mex_cuda_demo_gb300 as pkg
    from asd_pocs_mex_cuda_demo_gb300 import roofline

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pkg.load()
    B, iters = args.batch, args.iters
    paras, phis, Ps, I0s = make_inputs(B, iters, seed0=100 * rank, device=dev)
    stream = torch.cuda.Stream(device=dev)
    plan = pkg.Plan(paras, phis, stream=stream.cuda_stream)
    for b in range(B):
        plan.set_sinogram(b, Ps[b])
        plan.set_reference(b, I0s[b])
    flush = torch.empty(256 * 1024 * 1024 // 4, device=dev)  # > L2 (129 MB)

    def step():
        plan.reset()
        plan.run(use_graph=True, sync=False)

    for _ in range(args.warmup):
        step()
        plan.sync()
    clocks = ClockSampler(local)
    times = []
    barrier(pg)
    torch.cuda.synchronize()
    clocks.start()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        plan.reset()
        e0.record(stream)
        plan.run(use_graph=True, sync=False)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(pg)
    clk = clocks.stop()
    ms = allmax(pg, statistics.mean(times))
    value = B * world / (ms / 1e3)
    rmse = [plan.stats(b)["RMSE"][-1] for b in range(B)]
    kernels_per_step = iters * (2 * N_VIEWS + 1 + 2 * 20 + 1)

    # ---- plain path (one reconstruction per plan, same kernels) for context
    plain = pkg.Plan(paras[:1], phis[:1], stream=stream.cuda_stream)
    plain.set_sinogram(0, Ps[0])
    plain.set_reference(0, I0s[0])
    plain.reset()
    plain.run()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    plain.reset()
    e0.record(stream)
    plain.run(use_graph=True, sync=False)
    e1.record(stream)
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_rmse = plain.stats(0)["RMSE"][-1]
    plain_img = plain.image(0)
    batch_img = plan.image(0)
    plain.close()

    # ---- per-kernel device times (CUDA events on the plan's stream)
    vx = paras[0]["vxlsize"]
    nnz = statistics.mean(roofline.nnz_per_view(a, SO, OD, vx, DET, N_PIX, N_PIX, 1,
                                                N_BINS, 1) for a in phis[0][::6])
    N, M = N_PIX * N_PIX, N_BINS
    plan.reset()
    t_ax = plan.time_phase(0, 30)
    t_atx = plan.time_phase(1, 30)
    t_tv = plan.time_phase(2, 20)
    plan.reset()
    kern = {
        "sart_ax": {"ms": t_ax, "per_iter_ms": t_ax * N_VIEWS,
                    "bytes": B * roofline.ax_bytes(nnz, M)},
        "sart_atx": {"ms": t_atx, "per_iter_ms": t_atx * N_VIEWS,
                     "bytes": B * roofline.atx_bytes(nnz, N)},
        "tv_step": {"ms": t_tv, "per_iter_ms": t_tv * 20,
                    "bytes": B * roofline.tv_step_bytes(N)},
    }
    top = max(kern, key=lambda k: kern[k]["per_iter_ms"])
    peak, peak_kind = measured_peaks()
    achieved = kern[top]["bytes"] / (kern[top]["ms"] / 1e3) / 1e9
    tot_iter = sum(k["per_iter_ms"] for k in kern.values())

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        pinned_P = [torch.from_numpy(P.ravel(order="F")).pin_memory() for P in Ps]
        out_img = [torch.empty(N, dtype=torch.float32).pin_memory() for _ in range(B)]
        from asd_pocs_mex_cuda_demo_gb300._lib import check, load
        import ctypes as C

        L = load()
        et = []
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for b in range(B):
                check(L.asdpocs_plan_set_sinogram(plan._h, b, C.c_void_p(pinned_P[b].data_ptr()), 0))
            plan.reset()
            plan.run(use_graph=True, sync=False)
            for b in range(B):
                check(L.asdpocs_plan_get_image(plan._h, b, C.c_void_p(out_img[b].data_ptr()), 0))
            et.append(time.perf_counter() - t0)
        e_s = allmax(pg, statistics.mean(et))
        e2e = {"value": B * world / e_s, "unit": "recons/s",
               "h2d_bytes_per_step": B * N_BINS * N_VIEWS * 4,
               "d2h_bytes_per_step": B * N * 4}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(paras, phis, Ps, sample_iters=2)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "recons/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded random-ellipse phantoms, Poisson noise)",
            "config": {"workload": WORKLOAD, "batch_per_gpu": B, "iterations": iters,
                       "nx": N_PIX, "views": N_VIEWS, "bins": N_BINS, "tv_steps": 20,
                       "parallelism": f"replicas x{world}",
                       "l2": "256 MB buffer written between timed steps; resident set "
                             f"{plan.nbytes / 2**20:.0f} MB > 129 MB L2",
                       "graph": "one ASD-POCS iteration captured, replayed per iteration"},
            "latency_ms": {"p50": ms, "p99": max(times),
                           "note": "every reconstruction of a batch completes at the end "
                                   "of its step"},
            "plain": {"recons_per_s": 1e3 / plain_ms, "ms_per_recon": plain_ms,
                      "rmse": plain_rmse, "batched_rmse": rmse[0],
                      "batch_equals_plain_bitwise": bool(np.array_equal(plain_img, batch_img)),
                      "batched_speedup": value / world / (1e3 / plain_ms)},
            "rmse_vs_phantom": {"mean": float(np.mean(rmse)), "max": float(np.max(rmse))},
            "roofline": {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": None,
                         "bytes_per_launch": kern[top]["bytes"],
                         "ms_per_launch": kern[top]["ms"],
                         "share_of_iteration": kern[top]["per_iter_ms"] / tot_iter,
                         "kernels": kern},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": kernels_per_step * args.steps,
        }
        print(json.dumps(line))
    plan.close()


def reference_arm(args, rank, world, pg):
    """The reference's CPU implementation of the path on the host cores."""
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    from asd_pocs_mex_cuda_demo_gb300 import phantoms

    cores = os.cpu_count() or 1
    impl = "reference" if oracle.ref_available() else "oracle"
    kind = "reference" if impl == "reference" else "port"
    p = para_for(0)
    p["maxnumIter"] = 1
    phi = phantoms.views(N_VIEWS)
    x = phantoms.random_ellipses(N_PIX, 0)
    P = np.zeros((N_BINS, N_VIEWS))
    for v, a in enumerate(phi):
        g = oracle.gateway_geometry(-a / 180 * np.pi, SO, OD, p["vxlsize"], DET, N_BINS, 1)
        P[:, v] = oracle.ax(x.astype(np.float32), g, N_PIX, N_PIX, 1, nthreads=cores)[0]
    P = phantoms.poisson_noise(P, I0_PHOTONS, seed=1000)
    p["phi_vec"] = phi
    for _ in range(args.warmup):
        oracle.asdpocs(P, dict(p, maxnumIter=1), impl=impl, nthreads=cores)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.asdpocs(P, dict(p, maxnumIter=1), impl=impl, nthreads=cores)
        times.append(time.perf_counter() - t)
    per_iter = statistics.mean(times)
    value = 1.0 / (per_iter * args.iters)
    sample = (f"one of {args.iters} ASD-POCS iterations per step (60 views SART + 20 TV "
              f"steps) of one 512^2 reconstruction, extrapolated")
    print(json.dumps({
        "metric": METRIC, "impl": "reference", "value": value, "unit": "recons/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per_iter * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "iterations": args.iters},
        "cpu_baseline": {"value": value, "unit": "recons/s", "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "recons/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))
    return 0


if __name__ == "__main__":
    sys.exit(main() or 0)
