"""Python 3 restatement of the NiftyRec package's emission API
(Python/NiftyRec/NiftyRec/NiftyRec.py) on the GB300 library.

Same function names, arguments, defaults and array conventions as the
reference package: arrays are passed to the C-ABI as raw buffers whose size
vector is ``array.shape`` (so for cubic volumes numpy axis 0 is nifti x),
cameras are given as a [3, n] array of angles in radians and transposed
before the call, and a non-zero status returns None.  The reference's GPU
block-size restriction no longer applies (every size is accepted).
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER as P
from ctypes import c_float, c_int

import numpy as np

from ._lib import load

ET_BACKGROUND_ACTIVITY = 0.0
ET_BACKGROUND_ATTENUATION = 0.0
ET_EPSILON = 0.000001
MAX_DEVICES = 16
SIZE_INFO = 5


def _pf(a):
    return None if a is None else a.ctypes.data_as(P(c_float))


def _size(shape):
    s = np.asarray(shape, dtype=np.int32)
    return s, s.ctypes.data_as(P(c_int))


def _f32(a):
    return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def et_project(activity, cameras, psf=None, attenuation=None, gpu=1, background=0.0, background_attenuation=0.0,
               truncate_negative_values=1):
    """Project activity to multiple cameras (NiftyRec.py:58-118)."""
    L = load()
    activity = _f32(activity)
    attenuation = _f32(attenuation)
    psf = _f32(psf)
    cameras = np.ascontiguousarray(np.asarray(cameras, dtype=np.float32))
    cams_t = cameras.transpose()  # [n, 3] view of the axis-major buffer
    a_size, a_p = _size(activity.shape)
    c_size, c_p = _size(cams_t.shape)
    if psf is not None:
        p_size, p_p = _size(psf.shape)
    else:
        p_size, p_p = _size([0, 0, 0])
    if attenuation is not None:
        t_size, t_p = _size(attenuation.shape)
    else:
        t_size, t_p = _size([0, 0, 0])
    projection = np.empty([activity.shape[0], activity.shape[1], cams_t.shape[0]], dtype=np.float32)
    s_size, s_p = _size(projection.shape)
    status = L.et_array_project(_pf(activity), a_p, _pf(projection), s_p, cameras.ctypes.data_as(P(c_float)), c_p,
                                _pf(psf), p_p, _pf(attenuation), t_p, float(background),
                                float(background_attenuation), int(gpu), int(truncate_negative_values))
    return None if status else projection


def et_backproject(projections, cameras, psf=None, attenuation=None, gpu=1, background=0, background_attenuation=0.0,
                   truncate_negative_values=1):
    """Backproject from multiple cameras to body space (NiftyRec.py:121-180)."""
    L = load()
    projections = _f32(projections)
    attenuation = _f32(attenuation)
    psf = _f32(psf)
    cameras = np.ascontiguousarray(np.asarray(cameras, dtype=np.float32))
    cams_t = cameras.transpose()
    s_size, s_p = _size(projections.shape)
    c_size, c_p = _size(cams_t.shape)
    if psf is not None:
        p_size, p_p = _size(psf.shape)
    else:
        p_size, p_p = _size([0, 0, 0])
    if attenuation is not None:
        t_size, t_p = _size(attenuation.shape)
    else:
        t_size, t_p = _size([0, 0, 0])
    bk = np.empty([projections.shape[0], projections.shape[1], projections.shape[0]], dtype=np.float32)
    b_size, b_p = _size(bk.shape)
    status = L.et_array_backproject(_pf(projections), s_p, _pf(bk), b_p, cameras.ctypes.data_as(P(c_float)), c_p,
                                    _pf(psf), p_p, _pf(attenuation), t_p, float(background),
                                    float(background_attenuation), int(gpu), int(truncate_negative_values))
    return None if status else bk


def et_set_gpu(gpu_id):
    """Select the GPU used by the library (NiftyRec.py:184-189)."""
    return load().et_array_set_gpu(int(gpu_id))


def et_list_gpus():
    """[gpu_count, [id, SMs*clock, SMs, clock_kHz, memory_MB] * count] (NiftyRec.py:193-207)."""
    L = load()
    count = ctypes.c_int(0)
    info = np.zeros(MAX_DEVICES * SIZE_INFO, dtype=np.int32)
    status = L.et_array_list_gpus(ctypes.byref(count), info.ctypes.data_as(P(c_int)))
    if status:
        return None
    return [count.value, info[:SIZE_INFO * count.value].tolist()]


def et_is_block_multiple(integer_value):
    return load().et_array_is_block_multiple(int(integer_value))


def et_get_block_size():
    return load().et_array_get_block_size()


def et_osmapem_step(subset_order, activity_old, sinogram, cameras, attenuation, psf, beta_osl, gradient_prior,
                    use_gpu, background_activity=ET_BACKGROUND_ACTIVITY,
                    background_attenuation=ET_BACKGROUND_ATTENUATION, epsilon=ET_EPSILON, rng=None):
    """One-step-late MAP-EM step over a random camera subset (NiftyRec.py:224-246).

    ``rng`` (a numpy Generator) makes the subset draw reproducible; the
    reference draws from numpy's global state."""
    n1, n2 = activity_old.shape[0], activity_old.shape[1]
    n_cameras = cameras.shape[1]
    n_sub = int(np.round(n_cameras / subset_order))
    r = (rng.random(n_sub) if rng is not None else np.random.rand(n_sub))
    idx = np.int32(np.round(0.5 + (n_cameras - 0.5) * r) - 1)
    cameras_sub = np.zeros((3, n_sub), dtype=np.float32)
    cameras_sub[:, :] = cameras[:, idx]
    normalization = et_backproject(np.ones((n1, n2, n_sub), dtype=np.float32), cameras_sub, psf, attenuation,
                                   use_gpu, background_activity, background_attenuation)
    normalization = normalization - beta_osl * gradient_prior
    normalization = normalization * (normalization > 0) + epsilon
    proj = et_project(activity_old, cameras_sub, psf, attenuation, use_gpu, background_activity,
                      background_attenuation)
    proj = proj * (proj > 0) + epsilon
    update = et_backproject(sinogram[idx, :, :].reshape(n1, n2, n_sub) / proj, cameras_sub, psf, attenuation,
                            use_gpu, background_activity, background_attenuation)
    update = update * (update > 0)
    return activity_old * update / normalization


class Reconstructor:
    """Background-thread reconstructor of NiftyRec.py:252-410 (OSEM and OSL-MAP
    with a quadratic MRF prior)."""

    def __init__(self, volume_size):
        self._reconstructing = False
        self._stop = False
        self.volume_size = tuple(volume_size)
        self.clear_activity()
        self.N_cameras = 0
        self.cameras = None
        self.psf = None
        self.attenuation = np.zeros(self.volume_size, dtype=np.float32)
        self.sinogram = None
        self.use_gpu = True
        self.background_activity = np.float32(ET_BACKGROUND_ACTIVITY)
        self.background_attenuation = np.float32(ET_BACKGROUND_ATTENUATION)
        self.epsilon = ET_EPSILON
        self.callback_status = lambda msg, frac: None
        self.callback_updateactivity = lambda activity: None
        self._thread = None

    def set_callback_status(self, function):
        self.callback_status = function

    def set_callback_updateactivity(self, function):
        self.callback_updateactivity = function

    def set_activity(self, activity):
        self.activity = np.float32(activity)

    def clear_activity(self):
        self.activity = np.ones(self.volume_size, dtype=np.float32)

    def set_attenuation(self, attenuation):
        self.attenuation = np.float32(attenuation)

    def set_sinogram(self, sinogram):
        if sinogram.shape[1] != self.volume_size[0] or sinogram.shape[2] != self.volume_size[1]:
            return
        self.sinogram = np.float32(sinogram)

    def set_psf_matrix(self, psf):
        self.psf = np.float32(psf)

    def set_cameras_matrix(self, cameras):
        self.cameras = np.float32(cameras)
        self.N_cameras = cameras.shape[1]

    def set_cameras_equispaced(self, first_camera, last_camera, n_cameras, axis=1):
        cams = np.zeros((3, n_cameras))
        cams[axis, :] = np.linspace(first_camera * np.pi / 180.0, last_camera * np.pi / 180.0, n_cameras)
        self.N_cameras = n_cameras
        self.cameras = np.float32(cams)

    def set_use_gpu(self, enable):
        self.use_gpu = int(enable)

    def set_background_activity(self, bg):
        self.background_activity = np.float32(bg)

    def set_background_attenuation(self, bg):
        self.background_attenuation = np.float32(bg)

    def set_epsilon(self, epsilon):
        self.epsilon = np.float32(epsilon)

    def has_all_parameters(self):
        return self.N_cameras != 0 and self.cameras is not None and self.sinogram is not None

    def is_reconstructing(self):
        return self._reconstructing

    def reconstruct(self, method, parameters, blocking=False):
        if self.is_reconstructing() or not self.has_all_parameters():
            return
        self._stop = False
        if blocking:
            self._reconstruct(method, parameters)
        else:
            self._thread = threading.Thread(target=self._reconstruct, args=(method, parameters), daemon=True)
            self._thread.start()

    def _reconstruct(self, method, parameters):
        steps = parameters["steps"]
        subset_order = parameters["subset_order"]
        self._reconstructing = True
        try:
            for step in range(steps):
                self.callback_status(f"{100.0 * step / steps:.0f}% {method} reconstruction", step / steps)
                beta, prior = 0.0, 0.0
                if method == "quadratic_MRF":
                    from scipy.signal import convolve

                    beta = parameters["beta"] / 1000.0
                    kernel = -np.ones((3, 3, 3))
                    kernel[1, 1, 1] = 26
                    prior = convolve(self.activity, kernel, "same")
                elif method != "osem":
                    break
                self.activity = et_osmapem_step(subset_order, self.activity, self.sinogram, self.cameras,
                                                self.attenuation, self.psf, beta, prior, self.use_gpu,
                                                self.background_activity, self.background_attenuation,
                                                self.epsilon)
                self.callback_updateactivity(self.activity)
                if self._stop:
                    break
        finally:
            self._reconstructing = False
            self.callback_status(" ", 0.0)

    def stop(self):
        if self.is_reconstructing():
            self._stop = True
