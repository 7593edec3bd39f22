"""Named workloads of the projector/backprojector, runnable from the command
line (e.g. under a profiler) through the device-pointer C-ABI:

    python -m niftyrec_gb300.workloads pair --n 128 --ncam 120 --psf 11 --reps 2   # one-call pair
    python -m niftyrec_gb300.workloads pair2 --n 128 --ncam 120 --reps 2           # two separate calls
    python -m niftyrec_gb300.workloads project --n 64 --ncam 60 --psf 0 --no-att
    python -m niftyrec_gb300.workloads dmu --reps 1       # exact d/dmu (autograd's attenuation gradient)
    python -m niftyrec_gb300.workloads pair --mode 1 --det   # exact transpose, deterministic form
    python -m niftyrec_gb300.workloads fisher --reps 1    # Fisher information of a 64-point grid
    python -m niftyrec_gb300.workloads osem --subsets 8 --reps 1     # plan OSEM iterations
    python -m niftyrec_gb300.workloads batch --volumes 8 --reps 1    # batched OSEM steps
    python -m niftyrec_gb300.workloads gradient --ncam 40 --reps 1   # et_array_gradient_attenuation

Inputs are the seeded synthetic phantom, mu map and depth-dependent Gaussian
PSF of niftyrec_gb300.synthetic; cameras rotate about the gantry axis in
360/ncam degree steps.  Prints the mean device time per repetition.
"""
from __future__ import annotations

import argparse
import ctypes

import numpy as np


def main(argv=None):
    import torch

    from . import _lib
    from . import synthetic as S

    ap = argparse.ArgumentParser()
    ap.add_argument("op", choices=["project", "backproject", "pair", "pair2", "osem", "batch", "gradient", "dmu",
                                   "fisher"])
    ap.add_argument("--subsets", type=int, default=8, help="osem: interleaved subsets")
    ap.add_argument("--volumes", type=int, default=8, help="batch: volumes of the batched workload")
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--ncam", type=int, default=120)
    ap.add_argument("--psf", type=int, default=11, help="PSF width (0: none)")
    ap.add_argument("--no-att", action="store_true")
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--mode", type=int, default=0, help="backprojector: 0 reference, 1 exact transpose")
    ap.add_argument("--bf16", action="store_true", help="activity and mu stored in bfloat16")
    ap.add_argument("--slope", type=float, default=0.02, help="PSF sigma = 0.5 + slope * depth")
    ap.add_argument("--group", type=int, default=0, help="backprojector cameras per scratch group (0: tuned)")
    ap.add_argument("--slabs", type=int, default=0, help="projector depth slabs 2/4/8 (0: tuned)")
    ap.add_argument("--no-mirror", action="store_true", help="every camera from its own matrix")
    ap.add_argument("--det", action="store_true",
                    help="deterministic exact-transpose backprojection and d/dmu (nrgb_set_deterministic)")
    a = ap.parse_args(argv)

    L = _lib.load()
    if a.group:
        L.nrgb_set_backproject_group(a.n, a.n, a.n, a.ncam, a.group)
    if a.slabs:
        L.nrgb_set_project_slabs(a.n, a.n, a.n, a.ncam, a.slabs)
    L.nrgb_set_mirror_pairs(0 if a.no_mirror else 1)
    L.nrgb_set_deterministic(1 if a.det else 0)
    n = a.n
    act = S.ellipsoid_phantom((n, n, n), seed=0)
    mu = S.mu_map((n, n, n), seed=0)
    psf = S.gaussian_psf(a.psf, n, 0.5, a.slope) if a.psf else None
    cams = S.cameras_about_y(a.ncam)[1].copy()
    dev = torch.device("cuda", 0)
    store = torch.bfloat16 if a.bf16 else torch.float32
    t_act = torch.from_numpy(act).to(dev).to(store)
    t_mu = None if a.no_att else torch.from_numpy(mu).to(dev).to(store)
    t_sino = torch.zeros((a.ncam, n, n), dtype=torch.float32, device=dev)
    t_bk = torch.zeros((n, n, n), dtype=torch.float32, device=dev)
    vp = ctypes.c_void_p
    size = (ctypes.c_int * 3)(n, n, n)
    csize = (ctypes.c_int * 2)(a.ncam, 1)
    psize = (ctypes.c_int * 3)(a.psf, a.psf, n) if a.psf else (ctypes.c_int * 3)(0, 0, 0)
    psf_p = psf.ctypes.data_as(vp) if psf is not None else None
    mu_p = vp(t_mu.data_ptr()) if t_mu is not None else None
    stream = torch.cuda.current_stream(dev)

    if a.op == "osem":
        from .plan import Plan

        plan = Plan((n, n, n), cams, psf, t_mu, subsets=a.subsets)
        counts = torch.from_numpy(S.poisson_counts(act_proj(L, act, mu, cams, psf), 50, seed=1)).to(dev)
        state = {}

        def run_osem():
            state["x"] = plan.osem(counts, iterations=1, activity=state.get("x"))
        run = run_osem
    elif a.op == "batch":
        from .batch import Batch, config_volumes
        from .plan import Plan

        vols, ys = [], []
        for c in config_volumes(a.volumes):
            shape = c["shape"]
            va, vm = S.ellipsoid_phantom(shape, seed=c["seed"]), S.mu_map(shape, seed=c["seed"])
            vp_ = S.gaussian_psf(a.psf or 11, shape[2], 0.5, c["slope"])
            vc = S.cameras_about_y(c["ncam"], 0.0, 360.0 / c["ncam"])
            vols.append(Plan(shape, vc, vp_, torch.from_numpy(vm).to(dev), subsets=c["subsets"]))
            ys.append(torch.from_numpy(S.poisson_counts(act_proj(L, va, vm, vc, vp_), 50, seed=c["seed"])).to(dev))
        batch = Batch(vols)

        def run_batch():
            batch.osem(ys, iterations=1)
        run = run_batch
    elif a.op == "gradient":  # the reference attenuation gradient of the projection (float32, mu required)
        if a.bf16 or t_mu is None:
            raise SystemExit("gradient: float32 activity and mu required")
        st = L.nrgb_project_device(vp(t_act.data_ptr()), mu_p, size, vp(t_sino.data_ptr()), cams.ctypes.data_as(vp),
                                   csize, psf_p, psize, 0.0, 0.0, 1, vp(stream.cuda_stream))
        assert st == 0, st

        def run_gradient():
            st = L.nrgb_gradient_attenuation_device(vp(t_sino.data_ptr()), vp(t_act.data_ptr()), mu_p, size,
                                                    vp(t_bk.data_ptr()), cams.ctypes.data_as(vp), csize, psf_p,
                                                    psize, 0.0, 0.0, 0, vp(stream.cuda_stream))
            assert st == 0, st
        run = run_gradient
    elif a.op == "dmu":  # d/dmu of sum(g * project(act, mu)), the fused recomputed-scan kernel
        if a.bf16 or t_mu is None:
            raise SystemExit("dmu: float32 activity and mu required")
        g = torch.from_numpy(np.random.default_rng(3).uniform(0.5, 1.5, (a.ncam, n, n)).astype(np.float32)).to(dev)

        def run_dmu():
            st = L.nrgb_attenuation_grad_device(vp(g.data_ptr()), vp(t_act.data_ptr()), mu_p, size,
                                                vp(t_bk.data_ptr()), cams.ctypes.data_as(vp), csize, psf_p, psize,
                                                0.0, 0.0, vp(stream.cuda_stream))
            assert st == 0, st
        run = run_dmu
    elif a.op == "fisher":  # et_array_fisher_grid of 64 grid points (host buffers)
        from . import array_api as A

        grid = np.zeros((n, n, n), np.float32)
        pts = np.random.default_rng(5).choice(n ** 3, size=64, replace=False)
        grid.flat[pts] = np.arange(1, 65, dtype=np.float32)
        psf_f = psf if psf is not None else S.gaussian_psf(3, n)

        def run_fisher():
            A.fisher_grid(act, S.cameras_about_y(a.ncam), psf_f, grid, 64, mu if not a.no_att else None)
        run = run_fisher
    else:
        run = None

    def run_pair():
        sp = vp(stream.cuda_stream)
        if a.op == "pair":
            fn = L.nrgb_project_backproject_device_bf16 if a.bf16 else L.nrgb_project_backproject_device
            st = fn(vp(t_act.data_ptr()), mu_p, size, vp(t_sino.data_ptr()), None, vp(t_bk.data_ptr()),
                    cams.ctypes.data_as(vp), csize, psf_p, psize, 0.0, 0.0, 1, a.mode, sp)
            assert st == 0, st
            return
        if a.op in ("project", "pair", "pair2"):
            fn = L.nrgb_project_device_bf16 if a.bf16 else L.nrgb_project_device
            st = fn(vp(t_act.data_ptr()), mu_p, size, vp(t_sino.data_ptr()), cams.ctypes.data_as(vp), csize, psf_p,
                    psize, 0.0, 0.0, 1, sp)
            assert st == 0, st
        if a.op in ("backproject", "pair", "pair2"):
            fn = L.nrgb_backproject_device_bf16 if a.bf16 else L.nrgb_backproject_device
            st = fn(vp(t_sino.data_ptr()), mu_p, size, vp(t_bk.data_ptr()), cams.ctypes.data_as(vp), csize, psf_p,
                    psize, 0.0, 0.0, 1, a.mode, sp)
            assert st == 0, st

    if run is None:
        run = run_pair

    run()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    for _ in range(a.reps):
        run()
    ev[1].record(stream)
    torch.cuda.synchronize()
    print(f"{a.op} n={n} ncam={a.ncam} psf={a.psf} att={not a.no_att} bf16={a.bf16} slabs={a.slabs} "
          f"mirror={not a.no_mirror}: "
          f"{ev[0].elapsed_time(ev[1]) / a.reps:.3f} ms per repetition")
    return 0


def act_proj(L, act, mu, cams, psf):
    """Projection of a host activity through the host-buffer C-ABI (counts for the OSEM workloads)."""
    from . import array_api as A

    return A.project(act, cams, psf, mu)


if __name__ == "__main__":
    raise SystemExit(main())
