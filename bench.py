#!/usr/bin/env python
"""Throughput of the rotation-based SPECT projector/backprojector on GB300.

Workload (one "pair"): activity 128^3 (seeded ellipsoid phantom), mu map 128^3,
depth-dependent Gaussian PSF 11 x 11 per depth plane (sigma = 0.5 + 0.02 z),
120 camera angles k * 3 degrees about the gantry axis; project all 120 angles
and backproject all 120 angles (the reference's inverse-rotation
backprojector).  Synthetic inputs with the benchmark's shapes and value
ranges stand in for a dataset (none is involved).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on stdout (rank 0).  `value` is device-resident throughput
(inputs already in HBM, L2 flushed between steps, CUDA events on the launching
stream); `e2e` is the same pair through the reference-facing C-ABI with host
buffers (SPECT_project_parallelholes + SPECT_backproject_parallelholes, all
host<->device copies inside the timed region).  With --gpus N (torchrun), each
rank runs its own independent pairs on its own GPU (weak scaling; no
collective on the data path) and the slowest rank's time is reported.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "128³×120-angle atten+PSF project+backproject pairs/s vs plain; % HBM peak"
UNIT = "pairs/s"
N = 128
NCAM = 120
K = 11
# Algorithmic bytes (float32): per angle the projector reads activity and mu
# once and writes one projection plane; the backprojector reads mu and the
# projection plane and read-modify-writes the accumulator.
P_ANGLE = N ** 3 * 8 + N ** 2 * 4
B_ANGLE = N ** 3 * 12 + N ** 2 * 4
PAIR_BYTES = NCAM * (P_ANGLE + B_ANGLE)  # 5,048,893,440
FLUSH_BYTES = 256 << 20  # > 129 MB L2
DOMINANT = "k_project_yg"  # the pair's largest kernel (per-kernel pass); timed inside the timed region


def algorithmic_bytes(kernel: str, launches: int, ncam_total: int) -> float:
    """Algorithmic bytes of all launches of one kernel within the timed region."""
    if kernel == "k_project_yg":
        return ncam_total * P_ANGLE
    if kernel in ("k_spread_yg", "k_spread_pair_yg"):  # reads mu and the projection plane per angle
        return ncam_total * (N ** 3 * 4 + N ** 2 * 4)
    if kernel == "k_gather_yg":  # accumulator read-modify-write per angle
        return ncam_total * (N ** 3 * 8)
    return float("nan")


def workload(seed=0):
    from niftyrec_gb300 import synthetic as S

    act = S.ellipsoid_phantom((N, N, N), seed=seed)
    mu = S.mu_map((N, N, N), seed=seed)
    psf = S.gaussian_psf(K, N, 0.5, 0.02)
    cams = S.cameras_about_y(NCAM, 0.0, 3.0)[1].copy()  # [n] theta_y only
    return act, mu, psf, cams


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(kernel: str):
    """dram bytes per launch of `kernel` from the committed ncu summary, or None."""
    for fn in sorted(os.listdir(os.path.join(ROOT, "profiles"))) if os.path.isdir(os.path.join(ROOT, "profiles")) else []:
        if not fn.endswith(".md") or not fn.startswith(kernel):
            continue
        txt = open(os.path.join(ROOT, "profiles", fn)).read()
        m = re.search(r"traffic_bytes_per_launch_full\s*\|\s*([0-9.eE+]+)", txt)
        if m:
            return float(m.group(1))
    return None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        self.device = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        self.file.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ----------------------------------------------------------------- our arm
def run_ours(args):
    import torch

    from niftyrec_gb300 import _lib
    from niftyrec_gb300 import array_api as A

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo", init_method="env://")
    torch.cuda.set_device(local)
    L = _lib.load()
    if L.et_array_set_gpu(local) != 0:
        raise RuntimeError("et_array_set_gpu failed")
    dev = torch.device("cuda", local)
    act, mu, psf, cams = workload(seed=rank)
    t_act = torch.from_numpy(act).to(dev)
    t_mu = torch.from_numpy(mu).to(dev)
    t_sino = torch.empty((NCAM, N, N), dtype=torch.float32, device=dev)
    t_bk = torch.empty((N, N, N), dtype=torch.float32, device=dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    size = (ctypes.c_int * 3)(N, N, N)
    csize = (ctypes.c_int * 2)(NCAM, 1)
    psize = (ctypes.c_int * 3)(K, K, N)
    cams_c = np.ascontiguousarray(cams, np.float32)
    psf_c = np.ascontiguousarray(psf, np.float32)
    vp = ctypes.c_void_p

    def pair(use_psf=True, use_att=True, mode=0):
        sp = vp(stream.cuda_stream)
        st = L.nrgb_project_device(vp(t_act.data_ptr()), vp(t_mu.data_ptr()) if use_att else None, size,
                                   vp(t_sino.data_ptr()), cams_c.ctypes.data_as(vp), csize,
                                   psf_c.ctypes.data_as(vp) if use_psf else None,
                                   psize if use_psf else (ctypes.c_int * 3)(0, 0, 0), 0.0, 0.0, 1, sp)
        if st:
            raise RuntimeError(f"nrgb_project_device status {st}")
        st = L.nrgb_backproject_device(vp(t_sino.data_ptr()), vp(t_mu.data_ptr()) if use_att else None, size,
                                       vp(t_bk.data_ptr()), cams_c.ctypes.data_as(vp), csize,
                                       psf_c.ctypes.data_as(vp) if use_psf else None,
                                       psize if use_psf else (ctypes.c_int * 3)(0, 0, 0), 0.0, 0.0, 1, mode, sp)
        if st:
            raise RuntimeError(f"nrgb_backproject_device status {st}")

    def timed(steps, use_psf=True, use_att=True, profile=False, mode=0, only=None):
        """profile: per-kernel CUDA events on the launching stream (`only`: that
        kernel's launches alone; events around every launch add about 0.06 ms
        per pair)."""
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier(world)
        torch.cuda.synchronize(dev)
        n0 = L.nrgb_launch_count()
        if profile:
            L.nrgb_profile_only(only.encode() if only else None)
            L.nrgb_profile_enable(1)
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            pair(use_psf, use_att, mode)
            b.record(stream)
        torch.cuda.synchronize(dev)
        barrier(world)
        launches = L.nrgb_launch_count() - n0
        prof = None
        if profile:
            buf = ctypes.create_string_buffer(1 << 16)
            L.nrgb_profile_summary(buf, len(buf))
            L.nrgb_profile_enable(0)
            L.nrgb_profile_only(None)
            prof = {}
            for line in buf.value.decode().splitlines():
                name, cnt, ms = line.split()
                prof[name] = (int(cnt), float(ms))
        ms = [a.elapsed_time(b) for a, b in evs]
        return ms, launches, prof

    # warm-up (both variants)
    for _ in range(args.warmup):
        pair()
        pair(False, False)
    torch.cuda.synchronize(dev)

    # timed region: full model with clock sampling; CUDA events around the
    # projector's launches only (the dominant kernel's duration for the roofline)
    with Clocks(local) as clk:
        ms, launches, prof_dom = timed(args.steps, profile=True, only=DOMINANT)
    clocks = clk.summary()
    ms_step = reduce_max(sum(ms) / len(ms), world)
    value = world * 1000.0 / ms_step
    # per-kernel split of the same pair: a second pass with events around every launch
    ms_prof, _, prof = timed(max(3, args.steps // 2), profile=True)

    # "vs plain": the same pair without PSF and attenuation
    ms_plain, _, _ = timed(max(3, args.steps // 2), use_psf=False, use_att=False)
    plain = world * 1000.0 / reduce_max(sum(ms_plain) / len(ms_plain), world)
    # the same pair with the exact-transpose backprojector (gradient form)
    pair(mode=1)
    ms_adj, _, _ = timed(max(3, args.steps // 2), mode=1)
    adjoint = world * 1000.0 / reduce_max(sum(ms_adj) / len(ms_adj), world)

    grad = None if args.no_grad else grad_compare(L, t_act, t_mu, t_sino, t_bk, cams, psf, stream, flush, dev)

    # end to end through the reference-facing C-ABI with host buffers
    y = t_sino.cpu().numpy()
    A.project(act, cams, psf, mu)
    A.backproject(y, cams, psf, mu)
    barrier(world)
    e2e_t = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        s = A.project(act, cams, psf, mu)
        A.backproject(s, cams, psf, mu)
        e2e_t.append(time.perf_counter() - t0)
    barrier(world)
    e2e_s = reduce_max(statistics.median(e2e_t), world)
    # copied per pair: activity, mu, sinogram, mu again, and twice the camera
    # matrices (2 x 3x4 floats per camera) plus the separated PSF (2k floats per plane)
    params = NCAM * 24 * 4 + N * 2 * K * 4
    h2d = act.nbytes + mu.nbytes + y.nbytes + mu.nbytes + 2 * params
    d2h = y.nbytes + act.nbytes

    # rooflines of the kernels with algorithmic bytes: the projector timed in the
    # timed region, the others in the per-kernel pass; `roofline` is the
    # dominant kernel's (the largest total of the per-kernel pass)
    peak, peak_kind = measured_peak()
    rooflines = {}
    for name in (prof or {}):
        src, steps_src = (prof_dom, args.steps) if name in (prof_dom or {}) else (prof, max(3, args.steps // 2))
        cnt, tot_ms = src[name]
        alg = algorithmic_bytes(name, cnt, NCAM * steps_src)
        if alg != alg or cnt == 0:  # NaN: no algorithmic-byte model for this kernel
            continue
        per_launch_bytes = alg / cnt
        avg_s = tot_ms / cnt / 1e3
        achieved = per_launch_bytes / avg_s / 1e9
        rooflines[name] = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
                           "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                           "bytes_per_launch": per_launch_bytes, "avg_launch_ms": round(avg_s * 1e3, 4),
                           "timed_in": "timed region" if src is prof_dom else "per-kernel pass",
                           "traffic": committed_traffic(name)}
    roof = None
    if prof:
        dom = max(prof, key=lambda k: prof[k][1])
        roof = rooflines.get(dom)
    kernels = {k: {"launches": v[0], "ms_total": round(v[1], 3)} for k, v in (prof or {}).items()}

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipsoid phantom, mu map, Gaussian PSF)",
        "config": {"workload": "128^3 activity + mu, PSF 11x11 sigma=0.5+0.02*z, 120 angles x 3 deg, "
                               "project + reference backproject", "volume": [N, N, N], "angles": NCAM,
                   "psf": [K, K, N], "l2": "flushed (256 MB write) before every step", "parallelism": f"replicas{world}"},
        "plain_pairs_per_s": round(plain, 3),
        "adjoint_backprojector_pairs_per_s": round(adjoint, 3),
        "vs_plain": round(value / plain, 4),
        "pair_hbm": {"bytes_per_pair": PAIR_BYTES, "achieved_gbs": round(PAIR_BYTES * value / world / 1e9, 1),
                     "frac_of_peak": round(PAIR_BYTES * value / world / 1e9 / peak, 4), "peak_source": peak_kind},
        "roofline": roof,
        "rooflines": rooflines,
        "rooflines_note": "algorithmic bytes per camera angle as the reference moves them; a mirror unit serves "
                          "two angles from one pass, so the gather can read above its physical rate",
        "kernels": kernels,
        "kernels_pass": {"ms_per_step": round(sum(ms_prof) / len(ms_prof), 4),
                         "note": "separate pass with CUDA events around every launch"},
        "e2e": {"value": round(world / e2e_s, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "api": "SPECT_project_parallelholes + SPECT_backproject_parallelholes"},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if grad:
        out["attenuation_gradient"] = grad
    if not args.no_osem:
        out["osem"] = osem_compare(act, mu, psf, cams, dev)
    if not args.no_batch:
        out["batch_osem"] = batch_compare(dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(act, mu, psf, cams, args.cpu_angles)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


# --------------------------------------------------- attenuation gradient
def grad_compare(L, t_act, t_mu, t_sino, t_out, cams, psf, stream, flush, dev, reps=3):
    """The reference attenuation gradient (et_array_gradient_attenuation
    semantics) on device buffers at the bench workload: the gantry kernels
    against the general-orientation path (the same cameras tilted by 1e-9 rad
    about z, which leaves the gantry form)."""
    import torch

    vp = ctypes.c_void_p
    size = (ctypes.c_int * 3)(N, N, N)
    psize = (ctypes.c_int * 3)(K, K, N)
    psf_c = np.ascontiguousarray(psf, np.float32)
    gantry = np.zeros((3, NCAM), np.float32)
    gantry[1] = cams
    tilted = gantry.copy()
    tilted[2] = 1e-9

    def run(cm):
        cs = (ctypes.c_int * 2)(cm.shape[1], cm.shape[0])
        st = L.nrgb_gradient_attenuation_device(vp(t_sino.data_ptr()), vp(t_act.data_ptr()), vp(t_mu.data_ptr()),
                                                size, vp(t_out.data_ptr()), cm.ctypes.data_as(vp), cs,
                                                psf_c.ctypes.data_as(vp), psize, 0.0, 0.0, 0, vp(stream.cuda_stream))
        if st:
            raise RuntimeError(f"nrgb_gradient_attenuation_device status {st}")
        return L.nrgb_last_path()

    def timed(cm, n):
        ms = []
        for _ in range(n):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            run(cm)
            b.record(stream)
            torch.cuda.synchronize(dev)
            ms.append(a.elapsed_time(b))
        return statistics.median(ms)

    paths = (run(gantry), run(tilted))
    torch.cuda.synchronize(dev)
    fused_ms = timed(gantry, reps)
    L.nrgb_profile_enable(1)
    run(gantry)
    torch.cuda.synchronize(dev)
    buf = ctypes.create_string_buffer(1 << 16)
    L.nrgb_profile_summary(buf, len(buf))
    L.nrgb_profile_enable(0)
    kernels = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        kernels[name] = {"launches": int(cnt), "ms_total": round(float(ms), 3)}
    general_ms = timed(tilted, 2)
    return {"workload": "et_array_gradient_attenuation semantics, 128^3, 120 angles, PSF 11x11, mu, device buffers",
            "paths": list(paths), "fused_ms": round(fused_ms, 3), "general_ms": round(general_ms, 3),
            "speedup": round(general_ms / fused_ms, 2), "fused_kernels": kernels}


# ------------------------------------------------------------------- OSEM
def osem_compare(act, mu, psf, cams, dev, n_subsets=8, iterations=3):
    """One OSEM iteration (all subsets) at 128^3 x 120 angles: the plain
    per-call drop-in (et_array_osem_step_subset with host buffers, one call per
    subset) against a plan with cached carries/sensitivities whose iteration is
    captured once as a CUDA graph and replayed."""
    import torch

    from niftyrec_gb300 import array_api as A
    from niftyrec_gb300 import synthetic as S
    from niftyrec_gb300.plan import Plan

    counts = S.poisson_counts(A.project(act, cams, psf, mu), 50, seed=1)
    x = np.ones_like(act)
    cams3 = np.zeros((3, NCAM), np.float32)
    cams3[1] = cams
    subsets = [list(range(s, NCAM, n_subsets)) for s in range(n_subsets)]
    x = A.osem_step_subset(x, counts, cams3, subsets[0], mu, psf)  # warm-up
    t0 = time.perf_counter()
    for _ in range(iterations):
        for idx in subsets:
            x = A.osem_step_subset(x, counts, cams3, idx, mu, psf)
    per_call = (time.perf_counter() - t0) / iterations * 1e3

    plan = Plan((N, N, N), cams, psf, torch.from_numpy(mu).to(dev), subsets=n_subsets)
    y = torch.from_numpy(counts).to(dev)
    plan.osem(y, iterations=1, layout="column", graph=True)  # prepare + capture
    g, xc, ys = plan._graph
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(iterations):
        g.replay()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    graph_ms = e0.elapsed_time(e1) / iterations
    e0.record(stream)
    for _ in range(iterations):
        for s in range(n_subsets):
            plan.osem_step(xc, ys[s], s)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    eager_ms = e0.elapsed_time(e1) / iterations
    # the same iteration with opposite cameras in the same subset (mirror units)
    from niftyrec_gb300.plan import opposed_subsets

    plan2 = Plan((N, N, N), cams, psf, torch.from_numpy(mu).to(dev), subsets=opposed_subsets(NCAM, n_subsets))
    plan2.osem(y, iterations=1, layout="column", graph=True)
    g2 = plan2._graph[0]
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(iterations):
        g2.replay()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    opposed_ms = e0.elapsed_time(e1) / iterations
    return {"workload": f"OSEM iteration, 128^3, {NCAM} angles, {n_subsets} interleaved subsets, PSF 11x11, mu",
            "per_call_iteration_ms": round(per_call, 3), "plan_eager_iteration_ms": round(eager_ms, 3),
            "plan_graph_iteration_ms": round(graph_ms, 3), "speedup_graph_vs_per_call": round(per_call / graph_ms, 2),
            "plan_graph_opposed_subsets_iteration_ms": round(opposed_ms, 3)}


# ------------------------------------------------------------ batched OSEM
def batch_compare(dev, n_volumes=24, reps=5):
    """One OSEM subset step of 24 volumes of uneven size (64^3, 96x96x80,
    128^3, 160x160x128; 60/90/120/180 angles; 4-16 interleaved subsets; PSF
    11x11 with per-volume sigma slope; mu): the plain per-call drop-in
    (et_array_osem_step_subset with host buffers, one call per volume) against
    per-volume plan steps (eager and in one CUDA graph) and the batch (one
    persistent projector launch for all volumes; eager and graph-replayed)."""
    import torch

    from niftyrec_gb300 import array_api as A
    from niftyrec_gb300 import synthetic as S
    from niftyrec_gb300.batch import Batch, config_volumes
    from niftyrec_gb300.plan import Plan

    vols = []
    for c in config_volumes(n_volumes):
        shape = c["shape"]
        act = S.ellipsoid_phantom(shape, seed=c["seed"])
        mu = S.mu_map(shape, seed=c["seed"])
        psf = S.gaussian_psf(K, shape[2], 0.5, c["slope"])
        cams = S.cameras_about_y(c["ncam"], 0.0, 360.0 / c["ncam"])
        y = S.poisson_counts(A.project(act, cams, psf, mu), 50, seed=c["seed"])
        vols.append((c, act, mu, psf, cams, y))
    stream = torch.cuda.current_stream(dev)

    def dev_ms(fn, n=reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / n

    # plain per-call drop-in: one subset step per volume composed from the host
    # C-ABI projection / backprojection calls with the update on the host, as
    # et_array_osem_step does (emission-lib/_et_array_interface.cpp:1017-1044;
    # the entry itself takes cubic-in-x volumes only)
    def per_call():
        for c, act, mu, psf, cams, y in vols:
            idx = list(range(0, c["ncam"], c["subsets"]))
            sub = np.ascontiguousarray(cams[:, idx])
            x = np.ones_like(act)
            p = A.project(x, sub, psf, mu)
            r = np.where(p < 1e-6, y[idx] / np.float32(1e-6), y[idx] / np.maximum(p, 1e-6)).astype(np.float32)
            num = A.backproject(r, sub, psf, mu, nz=act.shape[0])
            den = A.backproject(np.ones_like(r), sub, psf, mu, nz=act.shape[0])
            x *= num / np.maximum(den, np.float32(1e-6))

    per_call()
    t0 = time.perf_counter()
    for _ in range(2):
        per_call()
    per_call_ms = (time.perf_counter() - t0) / 2 * 1e3

    plans = [Plan(c["shape"], cams, psf, torch.from_numpy(mu).to(dev), subsets=c["subsets"])
             for c, act, mu, psf, cams, y in vols]
    for p in plans:
        p.osem_prepare("column")
    ys = [p.split_counts(torch.from_numpy(v[5]).to(dev), "column") for p, v in zip(plans, vols)]
    xs = [p.to_column(torch.ones(p.shape, dtype=torch.float32, device=dev)) for p in plans]

    def plan_steps():
        for p, x, y in zip(plans, xs, ys):
            p.osem_step(x, y[0], 0)

    plan_eager = dev_ms(plan_steps)
    g_plans = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_plans):
        plan_steps()
    plan_graph = dev_ms(g_plans.replay)

    b = Batch(plans)
    for v, vv in enumerate(vols):
        b.set_counts(v, torch.from_numpy(vv[5]).to(dev))
        b.set_activity(v, torch.ones(plans[v].shape, dtype=torch.float32, device=dev))
    batch_eager = dev_ms(lambda: b.step(0))
    g_batch = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_batch):
        b.step(0)
    batch_graph = dev_ms(g_batch.replay)
    n_angles = sum(len(range(0, c["ncam"], c["subsets"])) for c, *_ in vols)
    return {"workload": f"one OSEM subset step of {n_volumes} volumes (64^3, 96x96x80, 128^3, 160x160x128; "
                        f"60/90/120/180 angles; 4-16 subsets; PSF 11x11; mu), {n_angles} angles in the step",
            "per_call_ms": round(per_call_ms, 3), "plan_eager_ms": round(plan_eager, 3),
            "plan_graph_ms": round(plan_graph, 3), "batch_eager_ms": round(batch_eager, 3),
            "batch_graph_ms": round(batch_graph, 3),
            "speedup_batch_graph_vs_per_call": round(per_call_ms / batch_graph, 2),
            "speedup_batch_graph_vs_plan_graph": round(plan_graph / batch_graph, 3)}


# ----------------------------------------------------------- CPU baselines
def cpu_baseline(act, mu, psf, cams, n_angles):
    """Single-core CPU time of the reference algorithm on a bounded sample:
    project + backproject of n_angles of the 120 angles, scaled to pairs/s."""
    from oracle.oracle import Reference, Restated

    if Reference.available:
        impl, kind = Reference(), "reference"
    else:
        impl, kind = Restated("f32"), "port"
    sub = cams[:n_angles]
    t0 = time.perf_counter()
    s = impl.project(act, sub, psf, mu)
    impl.backproject(s, sub, psf, mu)
    dt = time.perf_counter() - t0
    return {"value": round(n_angles / NCAM / dt, 6), "unit": UNIT, "cores": 1, "kind": kind,
            "sample": f"{n_angles} of {NCAM} angles projected and backprojected (128^3, PSF 11x11, mu), "
                      f"{dt:.1f} s, scaled to one pair"}


def _ref_worker_init(kind):
    global _W
    from oracle.oracle import Reference, Restated

    act, mu, psf, cams = workload(0)
    _W = (Reference() if kind == "reference" else Restated("f32"), act, mu, psf, cams)


def _ref_worker(angle_idx):
    impl, act, mu, psf, cams = _W
    sub = cams[list(angle_idx)]
    s = impl.project(act, sub, psf, mu)
    return impl.backproject(s, sub, psf, mu)


def run_reference(args):
    """The reference's CPU implementation of the pair on all host cores: angles
    split across worker processes, partial backprojections summed."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp

    from oracle.oracle import Reference

    kind = "reference" if Reference.available else "port"
    workers = os.cpu_count() or 1
    per_step = min(NCAM, 2 * workers)
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers, initializer=_ref_worker_init, initargs=(kind,)) as pool:
        def step(k):
            idx = [(k * per_step + i) % NCAM for i in range(per_step)]
            chunks = [idx[w::workers] for w in range(workers) if idx[w::workers]]
            parts = pool.map(_ref_worker, chunks)
            return np.sum(parts, axis=0)

        for k in range(args.warmup):
            step(k)
        t0 = time.perf_counter()
        for k in range(args.steps):
            step(k)
        dt = time.perf_counter() - t0
    pairs = args.steps * per_step / NCAM
    value = pairs / dt
    out = {
        "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipsoid phantom, mu map, Gaussian PSF)",
        "config": {"workload": "128^3 activity + mu, PSF 11x11 sigma=0.5+0.02*z, 120 angles x 3 deg, "
                               "project + reference backproject", "volume": [N, N, N], "angles": NCAM,
                   "psf": [K, K, N]},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": workers, "kind": kind,
                         "sample": f"{per_step} of {NCAM} angles per step over {workers} processes"},
        "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-angles", type=int, default=24)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-osem", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
