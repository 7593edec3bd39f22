"""numpy front end of the C-ABI (host buffers; every call goes through the
reference-compatible entry points of lib_et_array_interface.so).

Array convention: C-order numpy arrays whose memory is nifti order -- volumes
(nz, ny, nx), sinograms (n_cameras, ny, nx), PSF (planes, k, k); the size
vectors handed to the library are the reversed shapes.  Cameras: [n] (theta_y
only), [3, n] (theta_x, theta_y, theta_z rows) or [6, n] (angles then
centres), in radians, axis-major like the reference's ``cameras[axis*n+cam]``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import NiftyRecError, load

_PI = ctypes.POINTER(ctypes.c_int)


def _f32(a):
    return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _ints(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.int32))


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _pi(a):
    return a.ctypes.data_as(_PI)


def _cam_size(cams):
    return [cams.shape[0], 1] if cams.ndim == 1 else [cams.shape[1], cams.shape[0]]


def _check(fn, st):
    if st != 0:
        raise NiftyRecError(fn, st)


def project(activity, cameras, psf=None, attenuation=None, background=0.0, background_attenuation=0.0,
            truncate_negative_values=1):
    """SPECT_project_parallelholes; returns the sinogram (n_cameras, ny, nx)."""
    L = load()
    act, att, psf, cams = _f32(activity), _f32(attenuation), _f32(psf), _f32(cameras)
    ref = act if act is not None else att
    nz, ny, nx = ref.shape
    cs = _cam_size(cams)
    sino = np.empty((cs[0], ny, nx), np.float32)  # every element is written
    asz = _ints([nx, ny, nz] if act is not None else [0, 0, 0])
    tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
    psz = _ints(psf.shape[::-1] if psf is not None else [0, 0, 0])
    st = L.SPECT_project_parallelholes(_p(act), _pi(asz), _p(sino), _pi(_ints([nx, ny, cs[0]])), _p(cams),
                                       _pi(_ints(cs)), _p(psf), _pi(psz), _p(att), _pi(tsz),
                                       ctypes.byref(ctypes.c_float(background)),
                                       ctypes.byref(ctypes.c_float(background_attenuation)),
                                       ctypes.byref(ctypes.c_int(1)),
                                       ctypes.byref(ctypes.c_int(truncate_negative_values)))
    _check("SPECT_project_parallelholes", st)
    return sino


def project_partial(activity, cameras, psf=None, attenuation=None, background=0.0, background_image=None,
                    background_attenuation=0.0, truncate_negative_values=1, rotate_partial=0):
    """et_array_project_partial; returns (sinogram (n_cameras, ny, nx),
    partial sums (n_cameras, nz, ny, nx)): per camera the emission reaching
    each depth from the far side, in the rotated frame or (rotate_partial=1)
    rotated back to the image frame."""
    L = load()
    act, att, psf, cams = _f32(activity), _f32(attenuation), _f32(psf), _f32(cameras)
    bgi = _f32(background_image)
    ref = act if act is not None else att
    nz, ny, nx = ref.shape
    cs = _cam_size(cams)
    sino = np.zeros((cs[0], ny, nx), np.float32)
    part = np.zeros((cs[0], nz, ny, nx), np.float32)
    asz = _ints([nx, ny, nz] if act is not None else [0, 0, 0])
    tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
    psz = _ints(psf.shape[::-1] if psf is not None else [0, 0, 0])
    st = L.et_array_project_partial(_p(act), _pi(asz), _p(sino), _pi(_ints([nx, ny, cs[0]])), _p(part),
                                    _pi(_ints([nx, ny, nz, cs[0]])), _p(cams), _pi(_ints(cs)), _p(psf), _pi(psz),
                                    _p(att), _pi(tsz), background, _p(bgi), background_attenuation, 1,
                                    truncate_negative_values, rotate_partial)
    _check("et_array_project_partial", st)
    return sino, part


def fisher_grid(activity, cameras, psf, grid, n, attenuation=None, background=0.0, background_attenuation=0.0,
                prior=True):
    """et_array_fisher_grid: Fisher information [n, n] of the grid points
    (grid: volume with values 1..n at the points, 0 elsewhere) for the
    projection of the activity, and the 26-neighbour prior matrix (or None)."""
    L = load()
    act, att, psf, grid, cams = _f32(activity), _f32(attenuation), _f32(psf), _f32(grid), _f32(cameras)
    nz, ny, nx = act.shape
    cs = _cam_size(cams)
    f = np.zeros((n, n), np.float32)
    pr = np.zeros((n, n), np.float32) if prior else None
    tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
    st = L.et_array_fisher_grid(_p(act), _pi(_ints([nx, ny, nz])), _p(cams), _pi(_ints(cs)), _p(psf),
                                _pi(_ints(psf.shape[::-1])), _p(grid), _p(f), _p(pr), _pi(_ints([n, n])), _p(att),
                                _pi(tsz), 0.0, background, background_attenuation, 1)
    _check("et_array_fisher_grid", st)
    return f, pr


def fisher_grid_projection(sinogram, cameras, psf, grid, n, prior=True):
    """et_array_fisher_grid_projection: as fisher_grid from a given projection
    (n_cameras, ny, nx); grid is the volume (nz, ny, nx) of grid indexes."""
    L = load()
    sino, psf, grid, cams = _f32(sinogram), _f32(psf), _f32(grid), _f32(cameras)
    ncam, ny, nx = sino.shape
    gz, gy, gx = grid.shape
    cs = _cam_size(cams)
    f = np.zeros((n, n), np.float32)
    pr = np.zeros((n, n), np.float32) if prior else None
    st = L.et_array_fisher_grid_projection(_p(sino), _pi(_ints([nx, ny, ncam])), _pi(_ints([gx, gy, gz])), _p(cams),
                                           _pi(_ints(cs)), _p(psf), _pi(_ints(psf.shape[::-1])), _p(grid), _p(f),
                                           _p(pr), _pi(_ints([n, n])), None, _pi(_ints([0, 0, 0])), 0.0, 0.0, 0.0, 1)
    _check("et_array_fisher_grid_projection", st)
    return f, pr


def backproject(sinogram, cameras, psf=None, attenuation=None, background=0.0, background_attenuation=0.0,
                truncate_negative_values=1, nz=None):
    """SPECT_backproject_parallelholes; returns the volume (nz, ny, nx), nz defaults to nx."""
    L = load()
    sino, att, psf, cams = _f32(sinogram), _f32(attenuation), _f32(psf), _f32(cameras)
    ncam, ny, nx = sino.shape
    nz = nx if nz is None else nz
    out = np.empty((nz, ny, nx), np.float32)  # every element is written
    cs = _cam_size(cams)
    tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
    psz = _ints(psf.shape[::-1] if psf is not None else [0, 0, 0])
    st = L.SPECT_backproject_parallelholes(_p(sino), _pi(_ints([nx, ny, ncam])), _p(out), _pi(_ints([nx, ny, nz])),
                                           _p(cams), _pi(_ints(cs)), _p(psf), _pi(psz), _p(att), _pi(tsz),
                                           ctypes.byref(ctypes.c_float(background)),
                                           ctypes.byref(ctypes.c_float(background_attenuation)),
                                           ctypes.byref(ctypes.c_int(1)),
                                           ctypes.byref(ctypes.c_int(truncate_negative_values)))
    _check("SPECT_backproject_parallelholes", st)
    return out


def gradient_attenuation(sinogram, activity, attenuation, cameras, psf=None, background=0.0,
                         background_attenuation=0.0, truncate_negative_values=0):
    """et_array_gradient_attenuation (the reference's GPU attenuation-gradient semantics)."""
    L = load()
    sino, act, att, psf, cams = _f32(sinogram), _f32(activity), _f32(attenuation), _f32(psf), _f32(cameras)
    nz, ny, nx = act.shape
    out = np.empty_like(act)  # every element is written
    cs = _cam_size(cams)
    psz = _ints(psf.shape[::-1] if psf is not None else [0, 0, 0])
    vs = _ints([nx, ny, nz])
    st = L.et_array_gradient_attenuation(_p(sino), _pi(_ints([nx, ny, sino.shape[0]])), _p(act), _pi(vs), _p(out),
                                         _pi(vs), _p(cams), _pi(_ints(cs)), _p(psf), _pi(psz), _p(att), _pi(vs),
                                         background, background_attenuation, 1, truncate_negative_values)
    _check("et_array_gradient_attenuation", st)
    return out


def mlem_step(activity, sinogram, cameras3, attenuation=None, psf=None, background=0.0, background_attenuation=0.0,
              epsilon=1e-6):
    """et_array_mlem_step; returns the updated activity (the input is not modified)."""
    L = load()
    act = _f32(activity).copy()
    sino, att, psf, cams = _f32(sinogram), _f32(attenuation), _f32(psf), _f32(cameras3)
    nz, ny, nx = act.shape
    kx, ky = (psf.shape[2], psf.shape[1]) if psf is not None else (0, 0)
    st = L.et_array_mlem_step(_p(act), nx, ny, _p(sino), sino.shape[0], _p(cams), int(att is not None), _p(att),
                              int(psf is not None), _p(psf), kx, ky, background, background_attenuation, epsilon, 1)
    _check("et_array_mlem_step", st)
    return act


def osem_step_subset(activity, sinogram, cameras3, indexes, attenuation=None, psf=None, background=0.0,
                     background_attenuation=0.0, epsilon=1e-6):
    """et_array_osem_step_subset: one OSEM step over the given camera indexes."""
    L = load()
    act = _f32(activity).copy()
    sino, att, psf, cams = _f32(sinogram), _f32(attenuation), _f32(psf), _f32(cameras3)
    idx = _ints(indexes)
    nz, ny, nx = act.shape
    kx, ky = (psf.shape[2], psf.shape[1]) if psf is not None else (0, 0)
    st = L.et_array_osem_step_subset(_p(act), nx, ny, _p(sino), sino.shape[0], _p(cams), _pi(idx), len(idx),
                                     int(att is not None), _p(att), int(psf is not None), _p(psf), kx, ky,
                                     background, background_attenuation, epsilon)
    _check("et_array_osem_step_subset", st)
    return act


def rotate(volume, angles, center, background=0.0, axis_order=0):
    """et_array_rotate."""
    L = load()
    vol = _f32(volume)
    nz, ny, nx = vol.shape
    out = np.zeros_like(vol)
    st = L.et_array_rotate(_p(vol), _pi(_ints([nx, ny, nz])), _p(out), _p(_f32(angles)), _p(_f32(center)),
                           background, axis_order, 1)
    _check("et_array_rotate", st)
    return out


def affine(volume, matrix, background=0.0):
    """et_array_affine: out(x) = trilinear(volume, matrix @ x) in voxel
    coordinates (x, y, z, 1), `background` outside; volume (nz, ny, nx)."""
    L = load()
    vol = _f32(volume)
    nz, ny, nx = vol.shape
    out = np.zeros_like(vol)
    a = np.asfortranarray(np.asarray(matrix, dtype=np.float32).reshape(4, 4)).ravel(order="F")
    size = _ints([nx, ny, nz])
    st = L.et_array_affine(_p(vol), _pi(size), _p(out), _pi(size), _p(a), _pi(_ints([4, 4])), background, 1)
    _check("et_array_affine", st)
    return out


def convolve(volume, kernels):
    """et_array_convolve: per-slice 2D convolution; volume (nz, ny, nx),
    kernels (nz, ky, kx) with odd kx, ky; the image is clamped at its border."""
    L = load()
    vol = _f32(volume)
    k = _f32(kernels)
    nz, ny, nx = vol.shape
    out = np.zeros_like(vol)
    size = _ints([nx, ny, nz])
    st = L.et_array_convolve(_p(vol), _pi(size), _p(out), _pi(size), _p(k), _pi(_ints([k.shape[2], k.shape[1], k.shape[0]])),
                             1)
    _check("et_array_convolve", st)
    return out


def make_cameras(first_deg, last_deg, n, axis=1):
    """et_array_make_cameras -> [3, n]."""
    L = load()
    cams = np.zeros(3 * n, np.float32)
    L.et_array_make_cameras(_p(cams), first_deg, last_deg, n, axis)
    return cams.reshape(3, n)


def last_path():
    """1: the last call ran the fused y-gantry kernels; 2: the general path."""
    return load().nrgb_last_path()
