"""Differentiable SPECT projector for PyTorch.

``project(activity, attenuation, cameras, psf)`` returns the sinogram (no
negative truncation: it is not differentiable) of the rotation-based
projector with depth-dependent PSF and attenuation.  Its backward pass uses

* d/d(activity): the library's exact-transpose backprojector (mode 1 of
  nrgb_backproject_device: transposed PSF and transposed bilinear weights);
* d/d(mu): nrgb_attenuation_grad_device, which recomputes the depth scan of
  every ray instead of storing per-angle transmission.

Both sum rotated-frame values into the volume with vector reductions, whose
order varies between runs; ``set_deterministic(True)`` switches the fused
gantry kernels to a scratch + transposed-gather form with a fixed order
(bit-identical gradients from run to run).

Tensors are CUDA float32 in nifti memory order: volumes (nz, ny, nx),
sinograms (n_cameras, ny, nx).  Cameras and PSF are numpy arrays (see
niftyrec_gb300.array_api for the conventions).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import NiftyRecError, load

_vp = ctypes.c_void_p


def set_deterministic(on=True):
    """Deterministic exact-transpose backprojection and d/dmu (library-wide,
    for calls made afterwards); returns the previous setting."""
    L = load()
    prev = bool(L.nrgb_get_deterministic())
    L.nrgb_set_deterministic(1 if on else 0)
    return prev


def _cams(cameras):
    c = np.ascontiguousarray(np.asarray(cameras, dtype=np.float32))
    size = (ctypes.c_int * 2)(*((c.shape[0], 1) if c.ndim == 1 else (c.shape[1], c.shape[0])))
    return c, size


def _psf(psf, nz):
    if psf is None:
        return None, (ctypes.c_int * 3)(0, 0, 0)
    p = np.ascontiguousarray(np.asarray(psf, dtype=np.float32))
    return p, (ctypes.c_int * 3)(*p.shape[::-1])


def _stream(t):
    import torch

    return _vp(torch.cuda.current_stream(t.device).cuda_stream)


def project_raw(activity, attenuation, cameras, psf=None, background=0.0, background_attenuation=0.0):
    import torch

    L = load()
    nz, ny, nx = activity.shape
    c, csize = _cams(cameras)
    p, psize = _psf(psf, nz)
    n = csize[0]
    out = torch.empty((n, ny, nx), dtype=torch.float32, device=activity.device)
    st = L.nrgb_project_device(_vp(activity.data_ptr()), _vp(attenuation.data_ptr()) if attenuation is not None else None,
                               (ctypes.c_int * 3)(nx, ny, nz), _vp(out.data_ptr()), c.ctypes.data_as(_vp), csize,
                               p.ctypes.data_as(_vp) if p is not None else None, psize, float(background),
                               float(background_attenuation), 0, _stream(activity))
    if st:
        raise NiftyRecError("nrgb_project_device", st)
    return out


def backproject_raw(sinogram, attenuation, cameras, psf=None, nz=None, mode=1, truncate=0):
    """mode 1: exact transpose of the projector; mode 0: the reference backprojector."""
    import torch

    L = load()
    n, ny, nx = sinogram.shape
    nz = nx if nz is None else nz
    c, csize = _cams(cameras)
    p, psize = _psf(psf, nz)
    out = torch.empty((nz, ny, nx), dtype=torch.float32, device=sinogram.device)
    st = L.nrgb_backproject_device(_vp(sinogram.data_ptr()),
                                   _vp(attenuation.data_ptr()) if attenuation is not None else None,
                                   (ctypes.c_int * 3)(nx, ny, nz), _vp(out.data_ptr()), c.ctypes.data_as(_vp), csize,
                                   p.ctypes.data_as(_vp) if p is not None else None, psize, 0.0, 0.0, int(truncate),
                                   int(mode), _stream(sinogram))
    if st:
        raise NiftyRecError("nrgb_backproject_device", st)
    return out


def attenuation_grad_raw(grad_sino, activity, attenuation, cameras, psf=None, background=0.0,
                         background_attenuation=0.0):
    import torch

    L = load()
    nz, ny, nx = activity.shape
    c, csize = _cams(cameras)
    p, psize = _psf(psf, nz)
    out = torch.empty_like(activity)
    st = L.nrgb_attenuation_grad_device(_vp(grad_sino.data_ptr()), _vp(activity.data_ptr()),
                                        _vp(attenuation.data_ptr()), (ctypes.c_int * 3)(nx, ny, nz),
                                        _vp(out.data_ptr()), c.ctypes.data_as(_vp), csize,
                                        p.ctypes.data_as(_vp) if p is not None else None, psize, float(background),
                                        float(background_attenuation), _stream(activity))
    if st:
        raise NiftyRecError("nrgb_attenuation_grad_device", st)
    return out


def _function():
    import torch

    class SPECTProject(torch.autograd.Function):
        @staticmethod
        def forward(ctx, activity, attenuation, cameras, psf, background, background_attenuation):
            activity = activity.contiguous()
            attenuation = attenuation.contiguous() if attenuation is not None else None
            ctx.save_for_backward(activity, attenuation)
            ctx.args = (cameras, psf, background, background_attenuation)
            return project_raw(activity, attenuation, cameras, psf, background, background_attenuation)

        @staticmethod
        def backward(ctx, grad):
            activity, attenuation = ctx.saved_tensors
            cameras, psf, background, background_attenuation = ctx.args
            grad = grad.contiguous()
            g_act = g_mu = None
            if ctx.needs_input_grad[0]:
                g_act = backproject_raw(grad, attenuation, cameras, psf, nz=activity.shape[0], mode=1)
            if attenuation is not None and ctx.needs_input_grad[1]:
                g_mu = attenuation_grad_raw(grad, activity, attenuation, cameras, psf, background,
                                            background_attenuation)
            return g_act, g_mu, None, None, None, None

    return SPECTProject


_FN = None


def project(activity, attenuation=None, cameras=None, psf=None, background=0.0, background_attenuation=0.0):
    """Differentiable projection (see module docstring)."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(activity, attenuation, cameras, psf, background, background_attenuation)


def poisson_nll(projection, counts, eps=1e-9):
    """sum(p - y log p), the Poisson negative log-likelihood up to a constant."""
    import torch

    return torch.sum(projection - counts * torch.log(projection.clamp_min(eps)))
