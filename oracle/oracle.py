"""ctypes front end of the two CPU oracles.  Test infrastructure only.

* ``Restated`` -- the oracle's own C restatement (``et_oracle.c``), float
  (``"f32"``, follows the reference's float arithmetic) or double (``"f64"``,
  the FP64 oracle).  Built by ``make -C oracle`` into
  ``oracle/_build/libet_oracle.so``; travels anywhere gcc exists.
* ``Reference`` -- the reference's own CPU path compiled from its sources by
  ``oracle/Makefile.ref`` into ``oracle/_ref/libref_et.so``; exists only where
  the reference sources were available at build time.

Array convention (both): numpy C-order arrays whose memory is nifti order,
i.e. volumes have shape (nz, ny, nx) and sinograms (n_cameras, ny, nx); the
reference size vectors are then [nx, ny, nz] and [nx, ny, n_cameras].
Cameras are given as [3, n] (axis-major, rows theta_x, theta_y, theta_z) or
[n] (theta_y only) or [6, n] (angles then centres), matching the reference's
``cameras[axis * n + cam]`` layout.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
RESTATED_SO = os.path.join(_HERE, "_build", "libet_oracle.so")
REFERENCE_SO = os.path.join(_HERE, "_ref", "libref_et.so")

_P = ctypes.c_void_p
_I = ctypes.c_int


def build_restated() -> str:
    """Compile et_oracle.c (float + double) if the shared library is missing or stale."""
    src = os.path.join(_HERE, "et_oracle.c")
    if not os.path.exists(RESTATED_SO) or os.path.getmtime(RESTATED_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return RESTATED_SO


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _ints(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.int32))


def _cam_size(cameras: np.ndarray):
    cameras = np.asarray(cameras)
    if cameras.ndim == 1:
        return [cameras.shape[0], 1]
    return [cameras.shape[1], cameras.shape[0]]


def _psf_size(psf, nz):
    """PSF size in the reference's order; a PSF with fewer planes than the
    volume's depth would be read past its end by the restated convolution
    (as by the reference), so it is refused here."""
    if psf is None:
        return [0, 0, 0]
    if psf.shape[0] < nz:
        raise ValueError(f"PSF has {psf.shape[0]} planes, the volume {nz}")
    return list(psf.shape[::-1])


class Restated:
    """The C restatement, float or double."""

    def __init__(self, precision: str = "f32"):
        assert precision in ("f32", "f64")
        self.precision = precision
        self.dtype = np.float32 if precision == "f32" else np.float64
        self.real = ctypes.c_float if precision == "f32" else ctypes.c_double
        self.lib = ctypes.CDLL(build_restated())

    def _f(self, name):
        fn = getattr(self.lib, f"orc_{name}_{self.precision}")
        fn.restype = _I
        return fn

    def _arr(self, a):
        return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=self.dtype))

    def rotation_matrix(self, angles, center, axis_order=0):
        fn = getattr(self.lib, f"orc_rotation_matrix_{self.precision}")
        fn.restype = None
        M = np.zeros(16, dtype=self.dtype)
        R = self.real
        fn(_ptr(M), R(angles[0]), R(angles[1]), R(angles[2]), R(center[0]), R(center[1]), R(center[2]), _I(axis_order))
        return M.reshape(4, 4)

    def affine_resample(self, vol, A, bg=0.0):
        vol = self._arr(vol)
        A = self._arr(np.asarray(A).reshape(16))
        out = np.zeros_like(vol)
        nz, ny, nx = vol.shape
        fn = getattr(self.lib, f"orc_affine_resample_{self.precision}")
        fn.restype = None
        fn(_ptr(vol), _ptr(out), _I(nx), _I(ny), _I(nz), _ptr(A), self.real(bg))
        return out

    def convolve2d(self, vol, psf):
        """Per-slice 2D convolution (et_array_convolve): vol (nz, ny, nx), psf
        (nz, ky, kx); clamp-to-border."""
        vol = self._arr(vol)
        psf = self._arr(psf)
        nz, ny, nx = vol.shape
        _, ky, kx = psf.shape
        out = np.zeros_like(vol)
        fn = getattr(self.lib, f"orc_convolve2d_{self.precision}")
        fn.restype = None
        fn(_ptr(vol), _ptr(out), _I(nx), _I(ny), _I(nz), _ptr(psf), _I(kx), _I(ky))
        return out

    def project(self, act, cameras, psf=None, att=None, bg=0.0, bg_att=0.0, truncate=1):
        act = self._arr(act)
        att = self._arr(att)
        psf = self._arr(psf)
        cams = self._arr(cameras)
        ref = act if act is not None else att
        nz, ny, nx = ref.shape
        cs = _cam_size(cams)
        sino = np.zeros((cs[0], ny, nx), dtype=self.dtype)
        asz = _ints([nx, ny, nz] if act is not None else [0, 0, 0])
        tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
        psz = _ints(_psf_size(psf, nz))
        st = self._f("spect_project")(_ptr(act), _ptr(asz), _ptr(sino), _ptr(_ints([nx, ny, cs[0]])),
                                      _ptr(cams), _ptr(_ints(cs)), _ptr(psf), _ptr(psz), _ptr(att), _ptr(tsz),
                                      self.real(bg), self.real(bg_att), _I(truncate))
        if st:
            raise RuntimeError(f"oracle project status {st}")
        return sino

    def backproject(self, sino, cameras, psf=None, att=None, bg=0.0, bg_att=0.0, truncate=1, adjoint=False,
                    nz=None):
        sino = self._arr(sino)
        att = self._arr(att)
        psf = self._arr(psf)
        cams = self._arr(cameras)
        ncam, ny, nx = sino.shape
        nz = nx if nz is None else nz
        out = np.zeros((nz, ny, nx), dtype=self.dtype)
        cs = _cam_size(cams)
        tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
        psz = _ints(_psf_size(psf, nz))
        st = self._f("spect_backproject")(_ptr(sino), _ptr(_ints([nx, ny, ncam])), _ptr(out), _ptr(_ints([nx, ny, nz])),
                                          _ptr(cams), _ptr(_ints(cs)), _ptr(psf), _ptr(psz), _ptr(att), _ptr(tsz),
                                          self.real(bg), self.real(bg_att), _I(truncate), _I(1 if adjoint else 0))
        if st:
            raise RuntimeError(f"oracle backproject status {st}")
        return out

    def project_partial(self, act, cameras, psf=None, att=None, bg=0.0, bg_image=None, bg_att=0.0, truncate=1,
                        rotate=0):
        """et_array_project_partial: (sinogram [ncam, ny, nx], partial sums [ncam, nz, ny, nx])."""
        act = self._arr(act)
        att = self._arr(att)
        psf = self._arr(psf)
        bgi = self._arr(bg_image)
        cams = self._arr(cameras)
        ref = act if act is not None else att
        nz, ny, nx = ref.shape
        cs = _cam_size(cams)
        sino = np.zeros((cs[0], ny, nx), dtype=self.dtype)
        part = np.zeros((cs[0], nz, ny, nx), dtype=self.dtype)
        asz = _ints([nx, ny, nz] if act is not None else [0, 0, 0])
        tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
        psz = _ints(_psf_size(psf, nz))
        st = self._f("spect_project_partial")(_ptr(act), _ptr(asz), _ptr(sino), _ptr(part), _ptr(cams),
                                              _ptr(_ints(cs)), _ptr(psf), _ptr(psz), _ptr(att), _ptr(tsz),
                                              self.real(bg), _ptr(bgi), self.real(bg_att), _I(truncate), _I(rotate))
        if st:
            raise RuntimeError(f"oracle project_partial status {st}")
        return sino, part

    def fisher_grid(self, act, cameras, psf, grid, n, att=None, bg=0.0, bg_att=0.0, prior=True):
        """et_array_fisher_grid: (Fisher matrix [n, n], prior matrix [n, n] or None)."""
        act, att, psf, grid, cams = (self._arr(a) for a in (act, att, psf, grid, cameras))
        nz, ny, nx = act.shape
        cs = _cam_size(cams)
        fisher = np.zeros((n, n), dtype=self.dtype)
        pr = np.zeros((n, n), dtype=self.dtype) if prior else None
        tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
        st = self._f("spect_fisher_grid")(_ptr(act), _ptr(_ints([nx, ny, nz])), _ptr(cams), _ptr(_ints(cs)), _ptr(psf),
                                          _ptr(_ints(_psf_size(psf, nz))), _ptr(grid), _ptr(fisher), _ptr(pr),
                                          _I(n), _ptr(att), _ptr(tsz), self.real(bg), self.real(bg_att))
        if st:
            raise RuntimeError(f"oracle fisher_grid status {st}")
        return fisher, pr

    def gradient_attenuation(self, sino, act, att, cameras, psf=None, bg=0.0, bg_att=0.0, truncate=0):
        sino = self._arr(sino)
        act = self._arr(act)
        att = self._arr(att)
        psf = self._arr(psf)
        cams = self._arr(cameras)
        nz, ny, nx = act.shape
        ncam = sino.shape[0]
        out = np.zeros_like(act)
        cs = _cam_size(cams)
        psz = _ints(_psf_size(psf, nz))
        st = self._f("spect_gradient_attenuation")(_ptr(sino), _ptr(_ints([nx, ny, ncam])), _ptr(act),
                                                   _ptr(_ints([nx, ny, nz])), _ptr(out), _ptr(_ints([nx, ny, nz])),
                                                   _ptr(cams), _ptr(_ints(cs)), _ptr(psf), _ptr(psz), _ptr(att),
                                                   self.real(bg), self.real(bg_att), _I(truncate))
        if st:
            raise RuntimeError(f"oracle gradient status {st}")
        return out

    def osem_step(self, act, sino, cameras3, idx, att=None, psf=None, bg=0.0, bg_att=0.0, eps=1e-6):
        act = self._arr(act).copy()
        sino = self._arr(sino)
        att = self._arr(att)
        psf = self._arr(psf)
        cams = self._arr(cameras3)
        nz, ny, nx = act.shape
        ncam = sino.shape[0]
        idx = _ints(idx)
        _psf_size(psf, act.shape[0])  # refuses a PSF with fewer planes than nz
        kx, ky = (psf.shape[2], psf.shape[1]) if psf is not None else (0, 0)
        self._f("osem_step_subset")(_ptr(act), _I(nx), _I(ny), _ptr(sino), _I(ncam), _ptr(cams), _ptr(idx),
                                    _I(len(idx)), _ptr(att), _ptr(psf), _I(kx), _I(ky), self.real(bg),
                                    self.real(bg_att), self.real(eps))
        return act

    def make_cameras(self, first_deg, last_deg, n, axis=1):
        cams = np.zeros(3 * n, dtype=self.dtype)
        fn = getattr(self.lib, f"orc_make_cameras_{self.precision}")
        fn.restype = None
        fn(_ptr(cams), self.real(first_deg), self.real(last_deg), _I(n), _I(axis))
        return cams.reshape(3, n)


class Reference:
    """The reference's own CPU path (float32 only), called through its C-ABI."""

    available = os.path.exists(REFERENCE_SO)

    def __init__(self):
        if not os.path.exists(REFERENCE_SO):
            raise FileNotFoundError(REFERENCE_SO)
        self.lib = ctypes.CDLL(REFERENCE_SO)

    @staticmethod
    def _f32(a):
        return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float32))

    def project(self, act, cameras, psf=None, att=None, bg=0.0, bg_att=0.0, truncate=1):
        act, att, psf, cams = self._f32(act), self._f32(att), self._f32(psf), self._f32(cameras)
        nz, ny, nx = act.shape
        cs = _cam_size(cams)
        sino = np.zeros((cs[0], ny, nx), dtype=np.float32)
        tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
        psz = _ints(_psf_size(psf, nz))
        fn = self.lib.SPECT_project_parallelholes
        fn.restype = _I
        st = fn(_ptr(act), _ptr(_ints([nx, ny, nz])), _ptr(sino), _ptr(_ints([nx, ny, cs[0]])), _ptr(cams),
                _ptr(_ints(cs)), _ptr(psf), _ptr(psz), _ptr(att), _ptr(tsz),
                ctypes.byref(ctypes.c_float(bg)), ctypes.byref(ctypes.c_float(bg_att)), ctypes.byref(_I(0)),
                ctypes.byref(_I(truncate)))
        if st:
            raise RuntimeError(f"reference project status {st}")
        return sino

    def backproject(self, sino, cameras, psf=None, att=None, bg=0.0, bg_att=0.0, truncate=1, nz=None):
        sino, att, psf, cams = self._f32(sino), self._f32(att), self._f32(psf), self._f32(cameras)
        ncam, ny, nx = sino.shape
        nz = nx if nz is None else nz
        out = np.zeros((nz, ny, nx), dtype=np.float32)
        cs = _cam_size(cams)
        tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
        psz = _ints(_psf_size(psf, nz))
        fn = self.lib.SPECT_backproject_parallelholes
        fn.restype = _I
        st = fn(_ptr(sino), _ptr(_ints([nx, ny, ncam])), _ptr(out), _ptr(_ints([nx, ny, nz])), _ptr(cams),
                _ptr(_ints(cs)), _ptr(psf), _ptr(psz), _ptr(att), _ptr(tsz),
                ctypes.byref(ctypes.c_float(bg)), ctypes.byref(ctypes.c_float(bg_att)), ctypes.byref(_I(0)),
                ctypes.byref(_I(truncate)))
        if st:
            raise RuntimeError(f"reference backproject status {st}")
        return out

    def mlem_step(self, act, sino, cameras3, att=None, psf=None, bg=0.0, bg_att=0.0, eps=1e-6):
        act = self._f32(act).copy()
        sino, att, psf, cams = self._f32(sino), self._f32(att), self._f32(psf), self._f32(cameras3)
        nz, ny, nx = act.shape
        ncam = sino.shape[0]
        _psf_size(psf, act.shape[0])  # refuses a PSF with fewer planes than nz
        kx, ky = (psf.shape[2], psf.shape[1]) if psf is not None else (0, 0)
        fn = self.lib.et_array_mlem_step
        fn.restype = _I
        st = fn(_ptr(act), _I(nx), _I(ny), _ptr(sino), _I(ncam), _ptr(cams), _I(att is not None), _ptr(att),
                _I(psf is not None), _ptr(psf), ctypes.c_uint(kx), ctypes.c_uint(ky), ctypes.c_float(bg),
                ctypes.c_float(bg_att), ctypes.c_float(eps), _I(0))
        if st:
            raise RuntimeError(f"reference mlem status {st}")
        return act

    def fisher_grid(self, act, cameras, psf, grid, n, att=None, bg=0.0, bg_att=0.0, prior=True):
        act, att, psf, grid, cams = (self._f32(a) for a in (act, att, psf, grid, cameras))
        nz, ny, nx = act.shape
        cs = _cam_size(cams)
        fisher = np.zeros((n, n), dtype=np.float32)
        pr = np.zeros((n, n), dtype=np.float32) if prior else None
        tsz = _ints([nx, ny, nz] if att is not None else [0, 0, 0])
        fn = self.lib.et_array_fisher_grid
        fn.restype = _I
        st = fn(_ptr(act), _ptr(_ints([nx, ny, nz])), _ptr(cams), _ptr(_ints(cs)), _ptr(psf),
                _ptr(_ints(_psf_size(psf, nz))), _ptr(grid), _ptr(fisher), _ptr(pr), _ptr(_ints([n, n])), _ptr(att),
                _ptr(tsz), ctypes.c_float(0.0), ctypes.c_float(bg), ctypes.c_float(bg_att), _I(0))
        if st:
            raise RuntimeError(f"reference fisher_grid status {st}")
        return fisher, pr

    def make_cameras(self, first_deg, last_deg, n, axis=1):
        cams = np.zeros(3 * n, dtype=np.float32)
        fn = self.lib.et_array_make_cameras
        fn.restype = _I
        fn(_ptr(cams), ctypes.c_float(first_deg), ctypes.c_float(last_deg), ctypes.c_uint(n), ctypes.c_uint(axis))
        return cams.reshape(3, n)

    def rotate(self, vol, angles, center, bg=0.0, axis_order=0):
        vol = self._f32(vol)
        nz, ny, nx = vol.shape
        out = np.zeros_like(vol)
        fn = self.lib.et_array_rotate
        fn.restype = _I
        st = fn(_ptr(vol), _ptr(_ints([nx, ny, nz])), _ptr(out), _ptr(self._f32(angles)), _ptr(self._f32(center)),
                ctypes.c_float(bg), _I(axis_order), _I(0))
        if st:
            raise RuntimeError(f"reference rotate status {st}")
        return out
