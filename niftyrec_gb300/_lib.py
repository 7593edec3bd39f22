"""Loader of the in-tree CUDA library ``lib_et_array_interface.so`` and the
ctypes prototypes of its C-ABI (declared in include/et_array_interface.h).

The library is the product: there is no CPU fallback.  If it is missing, every
call raises; on a machine without a GPU the compute entry points return
status 8 (no GPU installed).
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib_et_array_interface.so")

_P = ctypes.c_void_p
_I = ctypes.c_int
_U = ctypes.c_uint
_F = ctypes.c_float
_PF = ctypes.POINTER(ctypes.c_float)
_PI = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes)
PROTOTYPES = {
    "status_success": (_I, [_PI]),
    "status_io_error": (_I, [_PI]),
    "status_initialisation_error": (_I, [_PI]),
    "status_parameter_error": (_I, [_PI]),
    "status_unhandled_error": (_I, [_PI]),
    "echo": (_I, [_PI, _PI]),
    "niftyrec_error_msg": (ctypes.c_char_p, [_I]),
    "et_array_isinstalled": (_I, []),
    "et_array_list_gpus": (_I, [_PI, _PI]),
    "et_array_set_gpu": (_I, [_I]),
    "et_array_set_gpu_pointer": (_I, [_PI]),
    "et_array_reset_gpu": (_I, []),
    "et_array_is_block_multiple": (ctypes.c_ushort, [ctypes.c_ushort]),
    "et_array_get_block_size": (ctypes.c_ushort, []),
    "SPECT_project_parallelholes": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _PF, _PF, _PI, _PI]),
    "SPECT_backproject_parallelholes": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _PF, _PF, _PI, _PI]),
    "et_array_project": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _F, _F, _I, _I]),
    "et_array_backproject": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _F, _F, _I, _I]),
    "et_array_gradient_attenuation": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _F, _F, _I, _I]),
    "et_array_attenuation_gradient": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _F, _F, _I, _I]),
    "et_array_project_partial": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _P, _PI, _F, _P, _F, _I, _I,
                                      _I]),
    "et_array_fisher_grid": (_I, [_P, _PI, _P, _PI, _P, _PI, _P, _P, _P, _PI, _P, _PI, _F, _F, _F, _I]),
    "et_array_fisher_grid_projection": (_I, [_P, _PI, _PI, _P, _PI, _P, _PI, _P, _P, _P, _PI, _P, _PI, _F, _F, _F,
                                             _I]),
    "et_array_calculate_size_psf": (_I, [ctypes.POINTER(_U), ctypes.POINTER(_U), _F, _F, _F, _F, _F, _F]),
    "et_array_make_psf": (_I, [_P, _U, _U, _F, _F, _F, _F, _F, _F, _U]),
    "et_array_make_cameras": (_I, [_P, _F, _F, _U, _U]),
    "et_array_rotate": (_I, [_P, _PI, _P, _P, _P, _F, _I, _I]),
    "et_array_affine": (_I, [_P, _PI, _P, _PI, _P, _PI, _F, _I]),
    "et_array_convolve": (_I, [_P, _PI, _P, _PI, _P, _PI, _I]),
    "et_array_osem_step": (_I, [_P, _I, _I, _U, _P, _I, _P, _I, _P, _I, _P, _U, _U, _F, _F, _F, _I]),
    "et_array_osem_step_subset": (_I, [_P, _I, _I, _P, _I, _P, _PI, _I, _I, _P, _I, _P, _U, _U, _F, _F, _F]),
    "et_array_mlem_step": (_I, [_P, _I, _I, _P, _I, _P, _I, _P, _I, _P, _U, _U, _F, _F, _F, _I]),
    "et_array_osem": (_I, [_P, _U, _U, _U, _P, _I, _F, _F, _U, _I, _I, _P, _I, _P, _U, _U, _F, _F, _F, _I]),
    "et_array_mlem": (_I, [_P, _U, _U, _P, _I, _F, _F, _U, _I, _I, _P, _I, _P, _U, _U, _F, _F, _F, _I]),
    "nrgb_project_device": (_I, [_P, _P, _PI, _P, _P, _PI, _P, _PI, _F, _F, _I, _P]),
    "nrgb_backproject_device": (_I, [_P, _P, _PI, _P, _P, _PI, _P, _PI, _F, _F, _I, _I, _P]),
    "nrgb_debug_fail_allocations": (_I, [_I]),
    "nrgb_project_backproject_device": (_I, [_P, _P, _PI, _P, _P, _P, _P, _PI, _P, _PI, _F, _F, _I, _I, _P]),
    "nrgb_project_backproject_device_bf16": (_I, [_P, _P, _PI, _P, _P, _P, _P, _PI, _P, _PI, _F, _F, _I, _I, _P]),
    "nrgb_project_device_bf16": (_I, [_P, _P, _PI, _P, _P, _PI, _P, _PI, _F, _F, _I, _P]),
    "nrgb_backproject_device_bf16": (_I, [_P, _P, _PI, _P, _P, _PI, _P, _PI, _F, _F, _I, _I, _P]),
    "nrgb_backproject_device_noalloc":(_I, [_P, _P, _PI, _P, _P, _PI, _P, _PI, _F, _F, _I, _P]),
    "nrgb_attenuation_grad_device": (_I, [_P, _P, _P, _PI, _P, _P, _PI, _P, _PI, _F, _F, _P]),
    "nrgb_gradient_attenuation_device": (_I, [_P, _P, _P, _PI, _P, _P, _PI, _P, _PI, _F, _F, _I, _P]),
    "nrgb_project_device_f64": (_I, [_P, _P, _PI, _P, _P, _PI, _P, _PI, ctypes.c_double, ctypes.c_double, _I, _P]),
    "nrgb_backproject_device_f64": (_I, [_P, _P, _PI, _P, _P, _PI, _P, _PI, ctypes.c_double, ctypes.c_double, _I,
                                         _P]),
    "nrgb_osem_ratio_device_f64": (_I, [_P, _P, ctypes.c_longlong, ctypes.c_double, _P]),
    "nrgb_osem_update_device_f64": (_I, [_P, _P, _P, ctypes.c_longlong, ctypes.c_double, _P]),
    "nrgb_osem_ratio_device": (_I, [_P, _P, ctypes.c_longlong, _F, _P]),
    "nrgb_osem_update_device": (_I, [_P, _P, _P, ctypes.c_longlong, _F, _P]),
    "nrgb_plan_create": (_I, [ctypes.POINTER(_P), _PI, _P, _PI, _P, _PI, _P, _F, _F, _PI, _I, _P]),
    "nrgb_plan_destroy": (_I, [_P]),
    "nrgb_plan_shape": (_I, [_P, _PI]),
    "nrgb_plan_subset_cameras": (_I, [_P, _I, _PI]),
    "nrgb_plan_project": (_I, [_P, _I, _P, _P, _I, _I, _P]),
    "nrgb_plan_backproject": (_I, [_P, _I, _P, _P, _I, _I, _P]),
    "nrgb_plan_osem_prepare": (_I, [_P, _I, _P]),
    "nrgb_plan_osem_step": (_I, [_P, _I, _P, _P, _F, _P]),
    "nrgb_batch_create": (_I, [ctypes.POINTER(_P), ctypes.POINTER(_P), _I, _P]),
    "nrgb_batch_destroy": (_I, [_P]),
    "nrgb_batch_set_counts": (_I, [_P, _I, _P, _P]),
    "nrgb_batch_set_activity": (_I, [_P, _I, _P, _P]),
    "nrgb_batch_get_activity": (_I, [_P, _I, _P, _P]),
    "nrgb_batch_osem_step": (_I, [_P, _I, _I, _F, _P]),
    "nrgb_plan_osmapem_step": (_I, [_P, _I, _P, _P, _F, _F, _P]),
    "nrgb_mrf_gradient_device": (_I, [_P, _P, _PI, _P]),
    "nrgb_layout_convert": (_I, [_P, _P, _I, _I, _I, _I, _I, _P]),
    "nrgb_set_backproject_group": (_I, [_I, _I, _I, _I, _I]),
    "nrgb_get_backproject_group": (_I, [_I, _I, _I, _I]),
    "nrgb_set_project_slabs": (_I, [_I, _I, _I, _I, _I]),
    "nrgb_get_project_slabs": (_I, [_I, _I, _I, _I]),
    "nrgb_set_mirror_pairs": (_I, [_I]),
    "nrgb_get_mirror_pairs": (_I, []),
    "nrgb_set_deterministic": (_I, [_I]),
    "nrgb_get_deterministic": (_I, []),
    "nrgb_nifti_info": (_I, [ctypes.c_char_p, _PI]),
    "nrgb_nifti_read": (_I, [ctypes.c_char_p, _P, ctypes.c_longlong]),
    "nrgb_nifti_write": (_I, [ctypes.c_char_p, _P, _PI]),
    "nrgb_nifti_gzip_supported": (_I, []),
    "nrgb_last_path": (_I, []),
    "nrgb_launch_count": (ctypes.c_longlong, []),
    "nrgb_profile_enable": (_I, [_I]),
    "nrgb_profile_summary": (_I, [ctypes.c_char_p, _I]),
    "nrgb_profile_only": (_I, [ctypes.c_char_p]),
    "nrgb_mirror_units": (_I, [_P, _PI, _PI, _PI, _I, _PI]),
    "nrgb_row_windows": (_I, [_I, _I, _PI, _I, _PI]),
}

_lib = None


class LibraryMissing(RuntimeError):
    pass


def load() -> ctypes.CDLL:
    """Load the CUDA library (once) and attach the prototypes."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise LibraryMissing(f"{LIB_PATH} is not built; run `python -m niftyrec_gb300.build`")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


STATUS = {
    0: "success", 1: "unspecified", 2: "parameters", 3: "kernel", 4: "allocgpu", 5: "alloccpu", 10: "scratch",
    6: "transfergpu", 7: "nogpubuilt", 8: "nogpuinstalled", 9: "timeout",
}


class NiftyRecError(RuntimeError):
    def __init__(self, fn, status):
        super().__init__(f"{fn} returned status {status} ({STATUS.get(status, 'unknown')})")
        self.status = status
