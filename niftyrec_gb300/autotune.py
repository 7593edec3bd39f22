"""Autotuner of the fused kernels' two shape-dependent launch choices.

* Backprojector camera-group size.  The reference-mode backprojector
  materialises the rotated-frame spread of a group of cameras in a scratch
  and gathers it back (two scratch slots, spread of group g+1 overlapping the
  gather of group g).  The best group size trades L2 residency of the scratch
  against launch count and per-launch parallelism.
* Projector depth slabs.  Each (camera, x-tile) item of the projector is
  split into 2, 4, 8 or 16 depth slabs, one thread block each, merged through
  distributed shared memory inside a thread-block cluster of that size.  More
  slabs mean more thread blocks in flight (better latency hiding on small
  grids) and a longer merge.

Both depend on the grid, the camera count and the GPU.  This module times the
candidates on the real problem shape (device buffers, CUDA events), records
the fastest in the library's tuning tables (nrgb_set_backproject_group,
nrgb_set_project_slabs) and keeps the results in a JSON cache so later
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
SLAB_CANDIDATES = (2, 4, 8, 16)
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
        if "group" in v:
            L.nrgb_set_backproject_group(nx, ny, nz, ncam, int(v["group"]))
        if "slabs" in v:
            L.nrgb_set_project_slabs(nx, ny, nz, ncam, int(v["slabs"]))
    return cache


def _record(cache_path, key, entry):
    """Merge `entry` into the cache's record of `key` (best effort)."""
    if not cache_path:
        return
    try:
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        try:
            with open(cache_path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        cache.setdefault(key, {}).update(entry)
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    except OSError:
        pass


def _time(run, reps, stream, dev):
    """Average milliseconds of `run` over `reps` calls after one untimed call."""
    import torch

    run()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    return e0.elapsed_time(e1) / reps


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
        times[g] = _time(run, reps, stream, dev)
    best = min(times, key=times.get)
    L.nrgb_set_backproject_group(nx, ny, nz, ncam, best)
    _record(cache_path, _key(nx, ny, nz, ncam), {"group": best, "ms": times})
    return best, times


def tune_project_slabs(nx, ny, nz, ncam, psf_k=11, attenuation=True, candidates=SLAB_CANDIDATES, reps=3,
                       cache_path=CACHE):
    """Time the projection for each depth-slab count; record and return the best."""
    import torch

    from . import _lib
    from . import synthetic as S

    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    shape = (nz, ny, nx)
    act = torch.from_numpy(S.ellipsoid_phantom(shape, seed=0)).to(dev)
    mu = torch.from_numpy(S.mu_map(shape, seed=0)).to(dev) if attenuation else None
    sino = torch.empty((ncam, ny, nx), dtype=torch.float32, device=dev)
    cams = np.ascontiguousarray(S.cameras_about_y(ncam)[1])
    psf = S.gaussian_psf(psf_k, max(nx, nz)) if psf_k else None
    vp = ctypes.c_void_p
    size = (ctypes.c_int * 3)(nx, ny, nz)
    csize = (ctypes.c_int * 2)(ncam, 1)
    psize = (ctypes.c_int * 3)(psf_k, psf_k, max(nx, nz)) if psf_k else (ctypes.c_int * 3)(0, 0, 0)
    stream = torch.cuda.current_stream(dev)

    def run():
        st = L.nrgb_project_device(vp(act.data_ptr()), vp(mu.data_ptr()) if mu is not None else None, size,
                                   vp(sino.data_ptr()), cams.ctypes.data_as(vp), csize,
                                   psf.ctypes.data_as(vp) if psf is not None else None, psize, 0.0, 0.0, 0,
                                   vp(stream.cuda_stream))
        if st:
            raise RuntimeError(f"nrgb_project_device status {st}")

    times = {}
    for s in candidates:
        if L.nrgb_set_project_slabs(nx, ny, nz, ncam, s):
            continue
        times[s] = _time(run, reps, stream, dev)
    best = min(times, key=times.get)
    L.nrgb_set_project_slabs(nx, ny, nz, ncam, best)
    _record(cache_path, _key(nx, ny, nz, ncam), {"slabs": best, "slab_ms": times})
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
    cache = None if a.no_cache else CACHE
    best, times = tune_backproject_group(a.n, a.n, a.n, a.ncam, a.psf, not a.no_att, reps=a.reps, cache_path=cache)
    slabs, stimes = tune_project_slabs(a.n, a.n, a.n, a.ncam, a.psf, not a.no_att, reps=a.reps, cache_path=cache)
    print(json.dumps({"shape": [a.n, a.n, a.n, a.ncam], "best_group": best,
                      "ms": {str(k): round(v, 4) for k, v in times.items()}, "best_slabs": slabs,
                      "slab_ms": {str(k): round(v, 4) for k, v in stimes.items()}}))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
