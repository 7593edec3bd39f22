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
stream) of nrgb_project_backproject_device, which projects and then
backprojects the projection in one call (the two separate device calls are
reported beside it); `e2e` is the same pair through the reference-facing C-ABI
with host buffers (SPECT_project_parallelholes + SPECT_backproject_parallelholes,
all host<->device copies inside the timed region).  With --gpus N (torchrun), each
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
DOMINANT = "k_project_yg"  # the pair's largest kernel (serialised ncu launch list); timed inside the timed region


def algorithmic_bytes(kernel: str, launches: int, ncam_total: int) -> float:
    """Algorithmic bytes of all launches of one kernel within the timed region."""
    if kernel == "k_project_yg":
        return ncam_total * P_ANGLE
    if kernel in ("k_spread_yg", "k_spread_pair_yg"):  # reads mu and the projection plane per angle
        return ncam_total * (N ** 3 * 4 + N ** 2 * 4)
    # k_gather_yg reads the scratch the spread wrote and gathers once per camera
    # group (a mirror unit serves two angles), overlapping the next spread on a
    # second stream: it has no per-angle algorithmic-byte model and no
    # isolated duration here (its ncu summary gives both)
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


def cpu_model() -> str:
    """Host CPU model name (lscpu / /proc/cpuinfo), for the CPU baselines."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


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

    def pair(use_psf=True, use_att=True, mode=0, separate=False):
        """One pair: nrgb_project_backproject_device (projection, then the
        backprojection of that projection), or the two separate calls."""
        sp = vp(stream.cuda_stream)
        if not separate:
            st = L.nrgb_project_backproject_device(vp(t_act.data_ptr()), vp(t_mu.data_ptr()) if use_att else None,
                                                   size, vp(t_sino.data_ptr()), None, vp(t_bk.data_ptr()),
                                                   cams_c.ctypes.data_as(vp), csize,
                                                   psf_c.ctypes.data_as(vp) if use_psf else None,
                                                   psize if use_psf else (ctypes.c_int * 3)(0, 0, 0), 0.0, 0.0, 1,
                                                   mode, sp)
            if st:
                raise RuntimeError(f"nrgb_project_backproject_device status {st}")
            return
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

    def timed(steps, use_psf=True, use_att=True, profile=False, mode=0, only=None, separate=False):
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
            pair(use_psf, use_att, mode, separate)
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

    # warm-up (every variant)
    for _ in range(args.warmup):
        pair()
        pair(False, False)
        pair(separate=True)
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

    # the same pair as two separate calls (nrgb_project_device + nrgb_backproject_device)
    ms_sep, _, _ = timed(max(3, args.steps // 2), separate=True)
    separate = world * 1000.0 / reduce_max(sum(ms_sep) / len(ms_sep), world)
    # "vs plain": the same pair without PSF and attenuation
    ms_plain, _, _ = timed(max(3, args.steps // 2), use_psf=False, use_att=False)
    plain = world * 1000.0 / reduce_max(sum(ms_plain) / len(ms_plain), world)
    # the same pair with the exact-transpose backprojector (gradient form)
    pair(mode=1)
    ms_adj, _, _ = timed(max(3, args.steps // 2), mode=1)
    adjoint = world * 1000.0 / reduce_max(sum(ms_adj) / len(ms_adj), world)
    # the same in the deterministic form (group scratch + transposed gather)
    L.nrgb_set_deterministic(1)
    pair(mode=1)
    ms_det, _, _ = timed(max(3, args.steps // 2), mode=1)
    L.nrgb_set_deterministic(0)
    adjoint_det = world * 1000.0 / reduce_max(sum(ms_det) / len(ms_det), world)

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
    # dominant kernel's: the projector, the largest share of the serialised ncu
    # launch list (the two camera groups' spreads run concurrently on two
    # streams, so their event durations include each other's)
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
    roof = rooflines.get(DOMINANT)
    kernels = {k: {"launches": v[0], "ms_total": round(v[1], 3)} for k, v in (prof or {}).items()}

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipsoid phantom, mu map, Gaussian PSF)",
        "config": {"workload": "128^3 activity + mu, PSF 11x11 sigma=0.5+0.02*z, 120 angles x 3 deg, "
                               "project + reference backproject", "volume": [N, N, N], "angles": NCAM,
                   "psf": [K, K, N], "l2": "flushed (256 MB write) before every step", "parallelism": f"replicas{world}"},
        "api": "nrgb_project_backproject_device (device buffers; projection, then backprojection of it)",
        "separate_calls_pairs_per_s": round(separate, 3),
        "plain_pairs_per_s": round(plain, 3),
        "adjoint_backprojector_pairs_per_s": round(adjoint, 3),
        "adjoint_deterministic_pairs_per_s": round(adjoint_det, 3),
        "vs_plain": round(value / plain, 4),
        "pair_hbm": {"bytes_per_pair": PAIR_BYTES, "achieved_gbs": round(PAIR_BYTES * value / world / 1e9, 1),
                     "frac_of_peak": round(PAIR_BYTES * value / world / 1e9 / peak, 4), "peak_source": peak_kind},
        "roofline": roof,
        "rooflines": rooflines,
        "rooflines_note": "algorithmic bytes per camera angle as the reference moves them (a mirror unit serves "
                          "two angles from one pass); the spreads of the two camera groups overlap each other "
                          "(two streams), so their per-kernel-pass durations include the sharing; the gather, an "
                          "intermediate that overlaps the spread, is left out (its one-kernel ncu summary is under "
                          "profiles/)",
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
    out["error_vs_fp64"] = fp64_errors(act, mu, psf, cams, dev)
    if not args.no_config1:
        out["config1"] = config1_leg(dev, flush, stream, args, cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
    if not args.no_config5:
        out["config5"] = config5_leg(dev, flush, stream, args, cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
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


# ------------------------------------------------------- error vs float64
def fp64_errors(act, mu, psf, cams, dev):
    """Relative L2 error of the timed pair's float32 results against the
    float64 GPU run of the reference algorithm (computed once, outside the
    timed region): the projection, and the backprojection of that projection."""
    import torch

    from niftyrec_gb300 import precision as pr

    a32, m32 = torch.from_numpy(act).to(dev), torch.from_numpy(mu).to(dev)
    p32 = pr.project(a32, m32, cams, psf, truncate=True)
    p64 = pr.project(a32.double(), m32.double(), cams, psf, truncate=True)
    b32 = pr.backproject(p32, m32, cams, psf, nz=N, truncate=True)
    b64 = pr.backproject(p32.double(), m32.double(), cams, psf, nz=N, truncate=True)
    ep, wp = pr.rel_error(p32, p64)
    eb, wb = pr.rel_error(b32, b64)
    return {"projection_rel_l2": ep, "projection_worst_plane": wp, "backprojection_rel_l2": eb,
            "backprojection_worst_plane": wb,
            "reference": "float64 GPU run of the reference algorithm (general-orientation kernels in double)"}


def _time_ms(fn, flush, stream, reps):
    """Mean device time of fn() over reps runs (CUDA events on the stream, L2
    flushed before each run)."""
    import torch

    ms = []
    for _ in range(reps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        ms.append((a, b))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ms) / reps


# ------------------------------------------------- config 1: 64^3 x 60 MLEM
C1_N, C1_NCAM = 64, 60
# per angle: projector N^3*4 + N^2*4, each backprojector 2*N^3*4 + N^2*4; one
# projection and two backprojections per MLEM iteration
C1_BYTES = C1_NCAM * ((C1_N ** 3 * 4 + C1_N ** 2 * 4) + 2 * (2 * C1_N ** 3 * 4 + C1_N ** 2 * 4))  # 317,521,920


def config1_workload():
    from niftyrec_gb300 import synthetic as S
    from niftyrec_gb300.array_api import make_cameras

    act = S.ellipsoid_phantom((C1_N,) * 3, seed=0)
    cams3 = np.ascontiguousarray(make_cameras(0.0, 354.0, C1_NCAM, 1), np.float32)  # [3, 60]
    return act, cams3


def config1_leg(dev, flush, stream, args, cpu=True):
    """Plain SPECT MLEM at 64^3 x 60 cameras (0..354 degrees, no PSF, no mu;
    counts Poisson(100 A x), seed 1): device-resident MLEM iterations/s with
    et_array_mlem_step's work (one projection, two backprojections, ratio and
    update) through the device entry points, the same through
    et_array_mlem_step with host buffers (e2e), a plan whose normaliser is
    computed once (graph-replayed), error of one step against float64, and the
    CPU reference step."""
    import torch

    from niftyrec_gb300 import _lib
    from niftyrec_gb300 import array_api as A
    from niftyrec_gb300 import precision as pr
    from niftyrec_gb300 import synthetic as S
    from niftyrec_gb300.plan import Plan

    L = _lib.load()
    n, ncam = C1_N, C1_NCAM
    act, cams3 = config1_workload()
    y = S.poisson_counts(A.project(act, cams3), 100, seed=1)
    vp = ctypes.c_void_p
    size = (ctypes.c_int * 3)(n, n, n)
    csize = (ctypes.c_int * 2)(ncam, 3)
    nopsf = (ctypes.c_int * 3)(0, 0, 0)
    t_y = torch.from_numpy(y).to(dev)
    t_x = torch.ones((n, n, n), dtype=torch.float32, device=dev)
    t_p = torch.empty((ncam, n, n), dtype=torch.float32, device=dev)
    t_ones = torch.ones((ncam, n, n), dtype=torch.float32, device=dev)
    t_num = torch.empty((n, n, n), dtype=torch.float32, device=dev)
    t_den = torch.empty((n, n, n), dtype=torch.float32, device=dev)
    cp = cams3.ctypes.data_as(vp)
    launches = [0]

    def iteration():
        sp = vp(stream.cuda_stream)
        n0 = L.nrgb_launch_count()
        st = [L.nrgb_project_device(vp(t_x.data_ptr()), None, size, vp(t_p.data_ptr()), cp, csize, None, nopsf,
                                    0.0, 0.0, 1, sp),
              L.nrgb_osem_ratio_device(vp(t_y.data_ptr()), vp(t_p.data_ptr()), t_p.numel(), 1e-6, sp),
              L.nrgb_backproject_device(vp(t_p.data_ptr()), None, size, vp(t_num.data_ptr()), cp, csize, None,
                                        nopsf, 0.0, 0.0, 1, 0, sp),
              L.nrgb_backproject_device(vp(t_ones.data_ptr()), None, size, vp(t_den.data_ptr()), cp, csize, None,
                                        nopsf, 0.0, 0.0, 1, 0, sp),
              L.nrgb_osem_update_device(vp(t_x.data_ptr()), vp(t_num.data_ptr()), vp(t_den.data_ptr()),
                                        t_x.numel(), 1e-6, sp)]
        launches[0] = L.nrgb_launch_count() - n0
        if any(st):
            raise RuntimeError(f"config-1 MLEM iteration status {st}")

    for _ in range(args.warmup):
        iteration()
    t_x.fill_(1.0)
    reps = max(5, args.steps)
    ms = _time_ms(iteration, flush, stream, reps)
    peak, peak_kind = measured_peak()
    achieved = C1_BYTES / (ms / 1e3) / 1e9

    # e2e: et_array_mlem_step with host buffers (copies inside the timed region)
    x = np.ones((n, n, n), np.float32)
    A.mlem_step(x, y, cams3)
    e2e_t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        x = A.mlem_step(x, y, cams3)
        e2e_t.append(time.perf_counter() - t0)

    # a plan (normaliser computed once, the iteration captured as a CUDA graph)
    plan = Plan((n, n, n), cams3[1].copy(), None, None, subsets=1)
    plan.osem(t_y, iterations=1, layout="column", graph=True)
    g = plan._graph[0]
    plan_ms = _time_ms(g.replay, flush, stream, reps)

    # error of one step against the float64 run (float32 vs float64 MLEM from ones)
    x32 = pr.osem(t_y, cams3, None, None, 1, 1, storage="float32")
    x64 = pr.osem(t_y, cams3, None, None, 1, 1, storage="float64")
    err = pr.rel_error(x32, x64)[0]

    out = {"workload": "plain SPECT MLEM, 64^3 activity (seeded ellipsoid phantom), 60 cameras 0..354 deg about "
                       "the gantry axis, no PSF, no mu, counts Poisson(100 A x) seed 1",
           "metric": "MLEM iterations/s (1 projection + 2 backprojections)", "unit": "iterations/s",
           "value": round(1000.0 / ms, 2), "ms_per_iteration": round(ms, 4), "gpu_launches_per_iteration":
               launches[0],
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "peak_source": peak_kind, "bytes_per_iteration": C1_BYTES,
                        "note": "whole iteration (several kernels); the volumes fit in L2, flushed before every "
                                "iteration"},
           "e2e": {"value": round(1.0 / statistics.median(e2e_t), 2), "unit": "iterations/s",
                   "api": "et_array_mlem_step", "h2d_bytes_per_step": int(x.nbytes + y.nbytes),
                   "d2h_bytes_per_step": int(x.nbytes)},
           "plan_graph": {"value": round(1000.0 / plan_ms, 2), "unit": "iterations/s",
                          "note": "normaliser B^T 1 computed once per plan (one projection and one backprojection "
                                  "per iteration), iteration replayed as a CUDA graph"},
           "error_vs_fp64": {"mlem_step_rel_l2": err}}
    if cpu:
        from oracle.oracle import Reference, Restated

        impl, kind = (Reference(), "reference") if Reference.available else (Restated("f32"), "port")
        x0 = np.ones((n, n, n), np.float32)
        t0 = time.perf_counter()
        k = 0
        while True:
            if kind == "reference":
                impl.mlem_step(x0, y, cams3)
            else:
                impl.osem_step(x0, y, cams3, list(range(ncam)))
            k += 1
            if time.perf_counter() - t0 > 4.0:
                break
        dt = (time.perf_counter() - t0) / k
        out["cpu_baseline"] = {"value": round(1.0 / dt, 4), "unit": "iterations/s", "cores": 1, "kind": kind,
                               "cpu_model": cpu_model(), "sample": f"{k} full MLEM iteration(s), {dt:.2f} s each"}
    return out


# ------------------------------- config 5: 256^3 x 180, PSF 15, BF16 vs FP32
C5_N, C5_NCAM, C5_K, C5_SLOPE = 256, 180, 15, 0.015


def _c5_bytes(s_vol):
    """Algorithmic bytes of one pair: per angle the projector reads activity and
    mu (s_vol bytes each) and writes a float32 plane; the backprojector reads
    mu, read-modify-writes the float32 accumulator and reads a plane."""
    n3, n2 = C5_N ** 3, C5_N ** 2
    return C5_NCAM * ((n3 * 2 * s_vol + n2 * 4) + (n3 * (s_vol + 8) + n2 * 4))


def config5_workload():
    from niftyrec_gb300 import synthetic as S

    n = C5_N
    act = S.ellipsoid_phantom((n, n, n), seed=0)
    mu = S.mu_map((n, n, n), seed=0)
    psf = S.gaussian_psf(C5_K, n, 0.5, C5_SLOPE)
    cams = S.cameras_about_y(C5_NCAM, 0.0, 2.0)[1].copy()
    return act, mu, psf, cams


def config5_leg(dev, flush, stream, args, cpu=True):
    """Precision at scale: one project + backproject pair of 256^3 x 180
    cameras, PSF 15 (sigma = 0.5 + 0.015 z), mu, with float32 storage and with
    bfloat16 activity / mu (float32 accumulation, Kahan depth sums); pairs/s,
    HBM fraction of each against its algorithmic bytes, and the error of each
    result against the float64 GPU run."""
    import torch

    from niftyrec_gb300 import _lib
    from niftyrec_gb300 import precision as pr

    L = _lib.load()
    n, ncam, k = C5_N, C5_NCAM, C5_K
    act, mu, psf, cams = config5_workload()
    vp = ctypes.c_void_p
    size = (ctypes.c_int * 3)(n, n, n)
    csize = (ctypes.c_int * 2)(ncam, 1)
    psize = (ctypes.c_int * 3)(k, k, n)
    cp = np.ascontiguousarray(cams, np.float32)
    pp = np.ascontiguousarray(psf, np.float32)
    a32, m32 = torch.from_numpy(act).to(dev), torch.from_numpy(mu).to(dev)
    a16, m16 = a32.to(torch.bfloat16), m32.to(torch.bfloat16)
    sino = torch.empty((ncam, n, n), dtype=torch.float32, device=dev)
    bk = torch.empty((n, n, n), dtype=torch.float32, device=dev)

    def pair(bf16):
        """One pair through nrgb_project_backproject_device(_bf16), as the headline."""
        sp = vp(stream.cuda_stream)
        fn = L.nrgb_project_backproject_device_bf16 if bf16 else L.nrgb_project_backproject_device
        a, m = (a16, m16) if bf16 else (a32, m32)
        st = fn(vp(a.data_ptr()), vp(m.data_ptr()), size, vp(sino.data_ptr()), None, vp(bk.data_ptr()),
                cp.ctypes.data_as(vp), csize, pp.ctypes.data_as(vp), psize, 0.0, 0.0, 1, 0, sp)
        if st:
            raise RuntimeError(f"config-5 pair status {st}")

    peak, peak_kind = measured_peak()
    reps = max(3, args.steps // 3)
    res = {}
    for name, bf16, sv in (("float32", False, 4), ("bfloat16", True, 2)):
        for _ in range(2):
            pair(bf16)
        ms = _time_ms(lambda: pair(bf16), flush, stream, reps)
        byts = _c5_bytes(sv)
        ach = byts / (ms / 1e3) / 1e9
        res[name] = {"pairs_per_s": round(1000.0 / ms, 3), "ms_per_pair": round(ms, 3),
                     "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                                  "frac": round(ach / peak, 4), "peak_source": peak_kind, "bytes_per_pair": byts}}
    # errors against float64 (outside the timed region)
    p64 = pr.project(a32.double(), m32.double(), cams, psf, truncate=True)
    b64 = pr.backproject(p64, m32.double(), cams, psf, nz=n, truncate=True)
    s32 = p64.float()
    for name, (a, m) in (("float32", (a32, m32)), ("bfloat16", (a16, m16))):
        p = pr.project(a, m, cams, psf, truncate=True)
        b = pr.backproject(s32, m, cams, psf, nz=n, truncate=True)
        ep, wp = pr.rel_error(p, p64)
        eb, wb = pr.rel_error(b, b64)
        res[name]["error_vs_fp64"] = {"projection_rel_l2": ep, "projection_worst_plane": wp,
                                      "backprojection_rel_l2": eb, "backprojection_worst_plane": wb}
        del p, b
    del p64, b64, s32
    out = {"workload": "256^3 activity + mu (seeded ellipsoid phantom, mu map), PSF 15x15 sigma=0.5+0.015*z, "
                       "180 angles x 2 deg, project + reference backproject; float32 vs bfloat16 storage",
           "unit": "pairs/s", "api": "nrgb_project_backproject_device(_bf16), device buffers", **res,
           "bf16_speedup": round(res["bfloat16"]["pairs_per_s"] / res["float32"]["pairs_per_s"], 3)}
    if cpu:
        out["cpu_baseline"] = cpu_pair_sample("config5", 16)
    return out


def _pool_init(which, kind):
    global _W
    from oracle.oracle import Reference, Restated

    wl = workload(0) if which == "headline" else config5_workload()
    _W = (Reference() if kind == "reference" else Restated("f32"),) + tuple(wl)


def _pool_noop(_):
    return 0


def _pool_pair(angle_idx):
    impl, act, mu, psf, cams = _W
    sub = cams[list(angle_idx)]
    s = impl.project(act, sub, psf, mu)
    return float(np.sum(impl.backproject(s, sub, psf, mu)))


def cpu_pair_sample(which, n_angles, workers=None):
    """Project + backproject of n_angles cameras of a workload on all host
    cores (one process per share of the angles), scaled to pairs/s."""
    import multiprocessing as mp

    from oracle.oracle import Reference

    kind = "reference" if Reference.available else "port"
    workers = workers or os.cpu_count() or 1
    ncam = NCAM if which == "headline" else C5_NCAM
    idx = list(range(n_angles))
    chunks = [idx[w::workers] for w in range(workers) if idx[w::workers]]
    with mp.get_context("spawn").Pool(len(chunks), initializer=_pool_init, initargs=(which, kind)) as pool:
        pool.map(_pool_noop, range(len(chunks)))
        t0 = time.perf_counter()
        pool.map(_pool_pair, chunks)
        dt = time.perf_counter() - t0
    return {"value": round(n_angles / ncam / dt, 6), "unit": "pairs/s", "cores": len(chunks), "kind": kind,
            "cpu_model": cpu_model(),
            "sample": f"{n_angles} of {ncam} angles projected and backprojected over {len(chunks)} processes, "
                      f"{dt:.1f} s, scaled to one pair"}


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
    # algorithmic bytes of the step: per angle the projector's 8 B and the
    # backprojector's 12 B per voxel plus 4 B per plane each; the ratio's 12 B
    # per sinogram element, the update's 16 B per voxel
    step_bytes = 0
    for c, *_ in vols:
        nz, ny, nx = c["shape"]
        na = len(range(0, c["ncam"], c["subsets"]))
        step_bytes += na * (20 * nz * ny * nx + 8 * ny * nx) + 12 * na * ny * nx + 16 * nz * ny * nx
    peak, peak_kind = measured_peak()
    ach = step_bytes / (batch_graph / 1e3) / 1e9
    return {"workload": f"one OSEM subset step of {n_volumes} volumes (64^3, 96x96x80, 128^3, 160x160x128; "
                        f"60/90/120/180 angles; 4-16 subsets; PSF 11x11; mu), {n_angles} angles in the step",
            "per_call_ms": round(per_call_ms, 3), "plan_eager_ms": round(plan_eager, 3),
            "plan_graph_ms": round(plan_graph, 3), "batch_eager_ms": round(batch_eager, 3),
            "batch_graph_ms": round(batch_graph, 3),
            "speedup_batch_graph_vs_per_call": round(per_call_ms / batch_graph, 2),
            "speedup_batch_graph_vs_plan_graph": round(plan_graph / batch_graph, 3),
            "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(ach / peak, 4), "peak_source": peak_kind, "bytes_per_step": step_bytes,
                         "note": "batch graph step; algorithmic bytes summed over the volumes"}}


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
            "cpu_model": cpu_model(),
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
                         "cpu_model": cpu_model(),
                         "sample": f"{per_step} of {NCAM} angles per step over {workers} processes"},
        "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_config1:
        out["config1"] = cpu_mlem_all_cores(kind, workers, iterations=max(2, min(args.steps, 5)))
    if not args.no_config5:
        out["config5"] = {"workload": "256^3 activity + mu, PSF 15x15 sigma=0.5+0.015*z, 180 angles x 2 deg, "
                                      "project + reference backproject, float32",
                          "cpu_baseline": cpu_pair_sample("config5", 2 * workers, workers)}
    print(json.dumps(out), flush=True)


def _mlem_init(kind):
    global _W
    from oracle.oracle import Reference, Restated

    act, cams3 = config1_workload()
    impl = Reference() if kind == "reference" else Restated("f32")
    y = np.clip(impl.project(act, cams3), 0, None).astype(np.float64) * 100.0
    y = np.random.default_rng(1).poisson(y).astype(np.float32)
    _W = (impl, cams3, y)


def _mlem_part(task):
    """Numerator and normaliser of one share of the cameras (the reference's
    MLEM step restricted to them: emission-lib/_et_array_interface.cpp:1080-1131)."""
    idx, x = task
    impl, cams3, y = _W
    sub = np.ascontiguousarray(cams3[:, idx])
    p = impl.project(x, sub)
    ys = y[idx]
    r = np.where(p < 1e-6, ys / np.float32(1e-6), ys / np.where(p < 1e-6, 1, p)).astype(np.float32)
    num = impl.backproject(r, sub, nz=x.shape[0])
    den = impl.backproject(np.ones_like(r), sub, nz=x.shape[0])
    return num, den


def cpu_mlem_all_cores(kind, workers, iterations):
    """Config 1 (64^3 x 60, plain MLEM) on all host cores: every iteration
    splits the cameras over the processes and sums their numerators and
    normalisers before the update."""
    import multiprocessing as mp

    idx = list(range(C1_NCAM))
    chunks = [idx[w::workers] for w in range(workers) if idx[w::workers]]
    x = np.ones((C1_N,) * 3, np.float32)
    with mp.get_context("spawn").Pool(len(chunks), initializer=_mlem_init, initargs=(kind,)) as pool:
        pool.map(_pool_noop, range(len(chunks)))
        t0 = time.perf_counter()
        for _ in range(iterations):
            parts = pool.map(_mlem_part, [(c, x) for c in chunks])
            num = np.sum([p[0] for p in parts], axis=0)
            den = np.sum([p[1] for p in parts], axis=0)
            x = (x * num / np.maximum(den, np.float32(1e-6))).astype(np.float32)
        dt = (time.perf_counter() - t0) / iterations
    return {"workload": "plain SPECT MLEM, 64^3, 60 cameras 0..354 deg, no PSF, no mu",
            "metric": "MLEM iterations/s (1 projection + 2 backprojections)", "unit": "iterations/s",
            "cpu_baseline": {"value": round(1.0 / dt, 4), "unit": "iterations/s", "cores": len(chunks),
                             "kind": kind, "cpu_model": cpu_model(),
                             "sample": f"{iterations} MLEM iterations, cameras split over {len(chunks)} processes"}}


# ------------------------------------------------- angle-sharded OSEM mode
def headline_sharded_workload():
    """The headline volume with counts Poisson(50 A x) (seed 1) from this
    rank's GPU projector; every rank draws the same counts."""
    from niftyrec_gb300 import array_api as A
    from niftyrec_gb300 import synthetic as S

    act, mu, psf, cams = workload(0)
    y = S.poisson_counts(A.project(act, cams, psf, mu), 50, seed=1)
    return act, mu, psf, cams, y


def run_sharded(args, make_operator=None, make_workload=None, device=None, out=None):
    """OSEM whose every subset's cameras are dealt over the ranks (one
    all_reduce of the numerator volume per subset step; niftyrec_gb300.sharded).
    Default: the headline workload (128^3 x 120, PSF 11, mu) with 8 interleaved
    subsets on CUDA with NCCL; make_operator / make_workload / device replace
    the GPU operator, the workload and the device (CPU ranks over gloo in the
    tests).  Rank 0 prints one JSON line (and stores it in `out` if given)."""
    import torch
    import torch.distributed as dist

    from niftyrec_gb300 import sharded as SH

    world, rank, local = dist_env()
    cuda = make_operator is None
    if cuda:
        torch.cuda.set_device(local)
        device = torch.device("cuda", local)
    device = device or torch.device("cpu")
    if world > 1 and not dist.is_initialized():
        dist.init_process_group("nccl" if cuda else "gloo", init_method="env://")
    sync = (lambda: torch.cuda.synchronize(device)) if cuda else (lambda: None)
    act, mu, psf, cams, y = (make_workload or headline_sharded_workload)()
    n_subsets = args.subsets
    ncam = cams.shape[-1]
    shape = act.shape
    ids, sids = SH.camera_shares(np.arange(ncam) % n_subsets, rank, world)
    if make_operator is None:
        cams3 = np.zeros((3, ncam), np.float32)
        cams3[1] = cams if cams.ndim == 1 else cams[1]
        op = SH.PlanOperator(shape, cams3, ids, sids, n_subsets, psf, torch.from_numpy(mu).to(device))
    else:
        op = make_operator(cams, ids, sids, n_subsets, psf, mu)
    counts = SH.split_counts(torch.from_numpy(y).to(device), ids, sids, n_subsets)
    rec = SH.ShardedOSEM(op, counts, n_subsets, rank=rank, world=world, sync=sync)
    x = torch.ones(shape, dtype=torch.float32, device=device)
    for _ in range(args.warmup):
        rec.run(x, 1)
    x.fill_(1.0)

    def reduce_max_dev(v):
        if world == 1:
            return v
        t = torch.tensor([v], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    if world > 1:
        dist.barrier()
    sync()
    t0 = time.perf_counter()
    rec.run(x, args.steps)
    sync()
    dt = time.perf_counter() - t0
    if world > 1:
        dist.barrier()
    dt = reduce_max_dev(dt)
    # a second pass with the collectives timed on their own (device synchronised around each)
    rec.timing_collectives = True
    rec.collective_seconds = 0.0
    rec.run(x.clone(), 1)
    coll_ms = reduce_max_dev(rec.collective_seconds / max(1, n_subsets) * 1e3)
    line = {"metric": f"OSEM iterations/s, angle-sharded over {world} rank(s) ({shape[2]}x{shape[1]}x{shape[0]}, "
                      f"{ncam} angles, {n_subsets} subsets)", "value": round(args.steps / dt, 4),
            "unit": "iterations/s", "n_gpus": world if cuda else 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt / args.steps * 1e3, 4), "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipsoid phantom, mu map, Gaussian PSF)",
            "mode": "sharded", "backend": (dist.get_backend() if world > 1 else "none"),
            "config": {"workload": "angle-sharded OSEM", "volume": list(shape[::-1]), "angles": ncam,
                       "subsets": n_subsets, "parallelism": f"angles{world}"},
            "cameras_this_rank": int(len(ids)),
            "collectives_per_iteration": n_subsets if world > 1 else 0,
            "allreduce_ms_per_step": round(coll_ms, 4) if world > 1 else 0.0,
            "allreduce_bytes_per_step": int(np.prod(shape) * 4) if world > 1 else 0}
    if rank == 0:
        print(json.dumps(line), flush=True)
        if out is not None:
            out.update(line)
    return x


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
    ap.add_argument("--no-config1", action="store_true")
    ap.add_argument("--no-config5", action="store_true")
    ap.add_argument("--sharded", action="store_true",
                    help="angle-sharded OSEM over the ranks (one all_reduce per subset step) instead of the pair")
    ap.add_argument("--subsets", type=int, default=8)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.sharded:
        run_sharded(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
