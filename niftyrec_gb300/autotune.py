"""Autotuner of the fused backprojector's camera-group size.

The reference-mode backprojector materialises the rotated-frame spread of a
group of cameras in an L2-sized scratch and gathers it back (two scratch
slots, spread of group g+1 overlapping the gather of group g).  The best group
size trades L2 residency of the scratch against launch count and per-launch
parallelism; it depends on the grid, the camera count and the GPU.  This
module times candidate sizes on the real problem shape (device buffers, CUDA
events), records the fastest in the library's tuning table
(nrgb_set_backproject_group) and keeps the result in a JSON cache so later
processes start tuned.

    python -m niftyrec_gb300.autotune --n 128 --ncam 120 --psf 11
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os

import numpy as np

CANDIDATES = (8, 16, 24, 32, 40, 48, 64)
CACHE = os.path.join(os.path.expanduser("~"), ".cache", "niftyrec_gb300", "tune.json")


def _key(nx, ny, nz, ncam):
    return f"{nx}x{ny}x{nz}x{ncam}"


def load_cache(path=CACHE):
    """Apply every cached entry to the library's tuning table; returns the cache."""
    from . import _lib

    try:
        with open(path) as f:
            cache = json.load(f)
    except (OSError, ValueError):
        return {}
    L = _lib.load()
    for k, v in cache.items():
        nx, ny, nz, ncam = (int(t) for t in k.split("x"))
        L.nrgb_set_backproject_group(nx, ny, nz, ncam, int(v["group"]))
    return cache


def tune_backproject_group(nx, ny, nz, ncam, psf_k=11, attenuation=True, candidates=CANDIDATES, reps=3,
                           cache_path=CACHE):
    """Time the backprojection for each candidate group size; record and return the best."""
    import torch

    from . import _lib
    from . import synthetic as S

    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    shape = (nz, ny, nx)
    mu = torch.from_numpy(S.mu_map(shape, seed=0)).to(dev) if attenuation else None
    sino = torch.rand((ncam, ny, nx), dtype=torch.float32, device=dev)
    out = torch.empty(shape, dtype=torch.float32, device=dev)
    cams = np.ascontiguousarray(S.cameras_about_y(ncam)[1])
    psf = S.gaussian_psf(psf_k, max(nx, nz)) if psf_k else None
    vp = ctypes.c_void_p
    size = (ctypes.c_int * 3)(nx, ny, nz)
    csize = (ctypes.c_int * 2)(ncam, 1)
    psize = (ctypes.c_int * 3)(psf_k, psf_k, max(nx, nz)) if psf_k else (ctypes.c_int * 3)(0, 0, 0)
    stream = torch.cuda.current_stream(dev)

    def run():
        st = L.nrgb_backproject_device(vp(sino.data_ptr()), vp(mu.data_ptr()) if mu is not None else None, size,
                                       vp(out.data_ptr()), cams.ctypes.data_as(vp), csize,
                                       psf.ctypes.data_as(vp) if psf is not None else None, psize, 0.0, 0.0, 1, 0,
                                       vp(stream.cuda_stream))
        if st:
            raise RuntimeError(f"nrgb_backproject_device status {st}")

    times = {}
    for g in candidates:
        if g > ncam:
            continue
        L.nrgb_set_backproject_group(nx, ny, nz, ncam, g)
        run()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            run()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        times[g] = e0.elapsed_time(e1) / reps
    best = min(times, key=times.get)
    L.nrgb_set_backproject_group(nx, ny, nz, ncam, best)
    if cache_path:
        try:
            os.makedirs(os.path.dirname(cache_path), exist_ok=True)
            try:
                with open(cache_path) as f:
                    cache = json.load(f)
            except (OSError, ValueError):
                cache = {}
            cache[_key(nx, ny, nz, ncam)] = {"group": best, "ms": times}
            with open(cache_path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return best, times


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--ncam", type=int, default=120)
    ap.add_argument("--psf", type=int, default=11)
    ap.add_argument("--no-att", action="store_true")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--no-cache", action="store_true")
    a = ap.parse_args(argv)
    best, times = tune_backproject_group(a.n, a.n, a.n, a.ncam, a.psf, not a.no_att, reps=a.reps,
                                         cache_path=None if a.no_cache else CACHE)
    print(json.dumps({"shape": [a.n, a.n, a.n, a.ncam], "best_group": best,
                      "ms": {str(k): round(v, 4) for k, v in times.items()}}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
