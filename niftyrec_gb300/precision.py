"""Storage precision and the float64 reference run.

Three arithmetic variants of the same projector / backprojector, selected by
the dtype of the torch tensors given:

* float32  - the reference's type (nrgb_project_device, ...);
* bfloat16 - activity and mu stored in bfloat16 (half the bytes), widened
  exactly on load; float32 arithmetic with Kahan-compensated depth sums;
  sinograms and backprojections float32 (nrgb_*_device_bf16);
* float64  - the reference algorithm with positions, weights, PSF, exp and
  every sum in double (nrgb_*_device_f64): the reference run the other two are
  measured against.

``osem`` runs the reference's OSEM update (emission-lib/_et_array_interface.cpp:972-1054)
in any of the three; ``rel_error`` states the error of a result against the
float64 run.  ``python -m niftyrec_gb300.precision`` reports, for a seeded
phantom, the error of every projection and reconstruction of the float32 and
bfloat16 variants against float64, with their timings.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import time

import numpy as np

from ._lib import NiftyRecError, load

_vp = ctypes.c_void_p


def _cams(cameras):
    c = np.ascontiguousarray(np.asarray(cameras, dtype=np.float32))
    size = (ctypes.c_int * 2)(*((c.shape[0], 1) if c.ndim == 1 else (c.shape[1], c.shape[0])))
    return c, size


def _psf(psf):
    if psf is None:
        return None, (ctypes.c_int * 3)(0, 0, 0)
    p = np.ascontiguousarray(np.asarray(psf, dtype=np.float32))
    return p, (ctypes.c_int * 3)(*p.shape[::-1])


def _ptr(t):
    return _vp(t.data_ptr()) if t is not None else None


def _stream(t):
    import torch

    return _vp(torch.cuda.current_stream(t.device).cuda_stream)


def project(activity, attenuation, cameras, psf=None, truncate=False):
    """Projection (n_cameras, ny, nx); float64 for float64 inputs, else float32."""
    import torch

    L = load()
    nz, ny, nx = activity.shape
    c, csize = _cams(cameras)
    p, psize = _psf(psf)
    size = (ctypes.c_int * 3)(nx, ny, nz)
    dt = activity.dtype
    if attenuation is not None and attenuation.dtype != dt:
        raise TypeError("activity and attenuation must share a dtype")
    out = torch.empty((csize[0], ny, nx), dtype=torch.float64 if dt == torch.float64 else torch.float32,
                      device=activity.device)
    args = (_ptr(activity), _ptr(attenuation), size, _ptr(out), c.ctypes.data_as(_vp), csize,
            p.ctypes.data_as(_vp) if p is not None else None, psize)
    if dt == torch.float32:
        st = L.nrgb_project_device(*args, 0.0, 0.0, int(truncate), _stream(activity))
    elif dt == torch.bfloat16:
        st = L.nrgb_project_device_bf16(*args, 0.0, 0.0, int(truncate), _stream(activity))
    elif dt == torch.float64:
        st = L.nrgb_project_device_f64(*args, 0.0, 0.0, int(truncate), _stream(activity))
    else:
        raise TypeError(f"unsupported dtype {dt}")
    if st:
        raise NiftyRecError("project", st)
    return out


def backproject(sinogram, attenuation, cameras, psf=None, nz=None, truncate=False):
    """Reference backprojection (nz, ny, nx).  The storage variant follows the
    attenuation's dtype (bfloat16 mu with a float32 sinogram selects the
    bfloat16 kernels); float64 sinograms select the float64 run."""
    import torch

    L = load()
    n, ny, nx = sinogram.shape
    nz = nx if nz is None else nz
    c, csize = _cams(cameras)
    p, psize = _psf(psf)
    size = (ctypes.c_int * 3)(nx, ny, nz)
    out = torch.empty((nz, ny, nx), dtype=sinogram.dtype, device=sinogram.device)
    args = (_ptr(sinogram), _ptr(attenuation), size, _ptr(out), c.ctypes.data_as(_vp), csize,
            p.ctypes.data_as(_vp) if p is not None else None, psize)
    if sinogram.dtype == torch.float64:
        st = L.nrgb_backproject_device_f64(*args, 0.0, 0.0, int(truncate), _stream(sinogram))
    elif attenuation is not None and attenuation.dtype == torch.bfloat16:
        st = L.nrgb_backproject_device_bf16(*args, 0.0, 0.0, int(truncate), 0, _stream(sinogram))
    else:
        st = L.nrgb_backproject_device(*args, 0.0, 0.0, int(truncate), 0, _stream(sinogram))
    if st:
        raise NiftyRecError("backproject", st)
    return out


def _ratio(y, p, eps):
    L = load()
    f = L.nrgb_osem_ratio_device_f64 if p.dtype.itemsize == 8 else L.nrgb_osem_ratio_device
    st = f(_ptr(y), _ptr(p), p.numel(), float(eps), _stream(p))
    if st:
        raise NiftyRecError("osem_ratio", st)


def _update(x, num, den, eps):
    L = load()
    f = L.nrgb_osem_update_device_f64 if x.dtype.itemsize == 8 else L.nrgb_osem_update_device
    st = f(_ptr(x), _ptr(num), _ptr(den), x.numel(), float(eps), _stream(x))
    if st:
        raise NiftyRecError("osem_update", st)


def osem(counts, cameras, psf, attenuation, n_subsets, iterations, storage="float32", epsilon=1e-6,
         callback=None):
    """OSEM with interleaved subsets (camera k in subset k % n_subsets).

    storage: "float32", "bfloat16" (activity re-stored in bfloat16 before every
    projection, mu stored in bfloat16; the estimate itself and the update stay
    float32) or "float64" (everything double: the reference run).
    counts: (n_cameras, ny, nx) tensor; attenuation: (nz, ny, nx) float32 or
    float64 tensor or None.  callback(iteration, x) after every iteration."""
    import torch

    cams = np.asarray(cameras, dtype=np.float32)
    cams = cams[None, :] if cams.ndim == 1 else cams
    ncam = cams.shape[1]
    nz = counts.shape[2]
    wide = storage == "float64"
    dt = torch.float64 if wide else torch.float32
    y = counts.to(dt)
    mu = None
    if attenuation is not None:
        mu = attenuation.to(torch.bfloat16 if storage == "bfloat16" else dt)
    subsets = [np.flatnonzero(np.arange(ncam) % n_subsets == s) for s in range(n_subsets)]
    ys = [y.index_select(0, torch.as_tensor(idx, device=y.device)).contiguous() for idx in subsets]
    sens = []
    for idx in subsets:
        ones = torch.ones((len(idx),) + tuple(y.shape[1:]), dtype=dt, device=y.device)
        sens.append(backproject(ones, mu, cams[:, idx], psf, nz=nz, truncate=True))
    x = torch.ones((nz,) + tuple(y.shape[1:]), dtype=dt, device=y.device)
    for it in range(iterations):
        for s, idx in enumerate(subsets):
            xs = x.to(torch.bfloat16) if storage == "bfloat16" else x
            p = project(xs, mu, cams[:, idx], psf, truncate=True)
            _ratio(ys[s], p, epsilon)
            num = backproject(p, mu, cams[:, idx], psf, nz=nz, truncate=True)
            _update(x, num, sens[s], epsilon)
        if callback is not None:
            callback(it, x)
    return x


def rel_error(result, reference):
    """Relative L2 error of a result against the float64 reference run:
    (global, worst plane along the first axis)."""
    a = result.double()
    b = reference.double()
    d = (a - b).flatten(1).norm(dim=1)
    r = b.flatten(1).norm(dim=1).clamp_min(1e-300)
    return float((a - b).norm() / b.norm().clamp_min(1e-300)), float((d / r).max())


def report(n=256, ncam=180, k=15, slope=0.015, n_subsets=10, iterations=10, seed=0, osem_size=None):
    """Errors of float32 and bfloat16 storage against the float64 run on the
    seeded phantom: one projection and one backprojection of all cameras, and
    OSEM (osem_size^3 grid, default n) after every iteration; with timings."""
    import torch

    from . import synthetic as S

    dev = torch.device("cuda", 0)
    out = {"shape": [n, n, n], "cameras": ncam, "psf": [k, k, n], "sigma": f"0.5 + {slope} * depth"}

    def timed(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t

    act = torch.from_numpy(S.ellipsoid_phantom((n, n, n), seed=seed)).to(dev)
    mu = torch.from_numpy(S.mu_map((n, n, n), seed=seed)).to(dev)
    psf = S.gaussian_psf(k, n, 0.5, slope)
    cams = S.cameras_about_y(ncam)
    p64, t64 = timed(lambda: project(act.double(), mu.double(), cams, psf))
    p32, t32 = timed(lambda: project(act, mu, cams, psf))
    p16, t16 = timed(lambda: project(act.to(torch.bfloat16), mu.to(torch.bfloat16), cams, psf))
    out["project"] = {"float32": dict(zip(("rel_l2", "worst_plane"), rel_error(p32, p64)), seconds=t32),
                      "bfloat16": dict(zip(("rel_l2", "worst_plane"), rel_error(p16, p64)), seconds=t16),
                      "float64_seconds": t64}
    sino = p64.float()
    b64, t64 = timed(lambda: backproject(p64, mu.double(), cams, psf, nz=n))
    b32, t32 = timed(lambda: backproject(sino, mu, cams, psf, nz=n))
    b16, t16 = timed(lambda: backproject(sino, mu.to(torch.bfloat16), cams, psf, nz=n))
    out["backproject"] = {"float32": dict(zip(("rel_l2", "worst_plane"), rel_error(b32, b64)), seconds=t32),
                          "bfloat16": dict(zip(("rel_l2", "worst_plane"), rel_error(b16, b64)), seconds=t16),
                          "float64_seconds": t64}
    del p64, p32, p16, b64, b32, b16
    m = osem_size or n
    if m != n:
        act = torch.from_numpy(S.ellipsoid_phantom((m, m, m), seed=seed)).to(dev)
        mu = torch.from_numpy(S.mu_map((m, m, m), seed=seed)).to(dev)
        psf = S.gaussian_psf(k, m, 0.5, slope)
    counts = torch.from_numpy(S.poisson_counts(project(act, mu, cams, psf, truncate=True).cpu().numpy(), 50,
                                               seed=seed + 1)).to(dev)
    hist = {s: [] for s in ("float64", "float32", "bfloat16")}
    recs = {}
    times = {}
    for s in ("float64", "float32", "bfloat16"):
        keep = hist[s]
        x, t = timed(lambda: osem(counts, cams, psf, mu, n_subsets, iterations, storage=s,
                                  callback=lambda it, x: keep.append(x.double().clone())))
        recs[s], times[s] = x, t
    per_iter = {s: [rel_error(hist[s][i], hist["float64"][i])[0] for i in range(iterations)]
                for s in ("float32", "bfloat16")}
    out["osem"] = {"shape": [m, m, m], "subsets": n_subsets, "iterations": iterations,
                   "rel_l2_per_iteration": per_iter, "seconds": times}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--ncam", type=int, default=180)
    ap.add_argument("--psf", type=int, default=15)
    ap.add_argument("--slope", type=float, default=0.015)
    ap.add_argument("--subsets", type=int, default=10)
    ap.add_argument("--iterations", type=int, default=10)
    ap.add_argument("--osem-size", type=int, default=None)
    a = ap.parse_args(argv)
    print(json.dumps(report(a.n, a.ncam, a.psf, a.slope, a.subsets, a.iterations, osem_size=a.osem_size)))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
