"""The drop-in boundary without a GPU: the library loads and exports every
function declared in include/*.h, and the pure host helpers behave like the
reference's."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:unsigned\s+)?(?:long long|int|char|short|void|float)\s*\*?\s*(\w+)\s*\(",
                             src, re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    from niftyrec_gb300 import _lib
    return _lib.load()


def test_header_declares_reference_entry_points():
    names = _declared_functions()
    for n in ["SPECT_project_parallelholes", "SPECT_backproject_parallelholes", "et_array_project",
              "et_array_backproject", "et_array_gradient_attenuation", "et_array_attenuation_gradient",
              "et_array_osem_step", "et_array_mlem_step", "et_array_osem", "et_array_mlem",
              "et_array_make_cameras", "et_array_list_gpus", "et_array_set_gpu", "et_array_isinstalled",
              "et_array_reset_gpu", "et_array_is_block_multiple", "et_array_get_block_size", "niftyrec_error_msg"]:
        assert n in names, n


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in sorted(_declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_prototypes_cover_header():
    from niftyrec_gb300 import _lib
    assert _declared_functions() <= set(_lib.PROTOTYPES), _declared_functions() - set(_lib.PROTOTYPES)


def test_status_helpers(lib):
    s = ctypes.c_int(-1)
    assert lib.status_success(ctypes.byref(s)) == 0 and s.value == 0
    assert lib.status_io_error(ctypes.byref(s)) == 0 and s.value == 101
    assert lib.status_parameter_error(ctypes.byref(s)) == 0 and s.value == 104
    out = ctypes.c_int(0)
    lib.echo(ctypes.byref(ctypes.c_int(42)), ctypes.byref(out))
    assert out.value == 42
    assert b"parameters" in lib.niftyrec_error_msg(2)


def test_make_cameras_matches_reference_fixture(golden):
    from niftyrec_gb300 import array_api
    g = golden("make_cameras")
    assert np.array_equal(array_api.make_cameras(0.0, 354.0, 60, 1), g["c60"])
    assert np.array_equal(array_api.make_cameras(-30.0, 45.0, 7, 0), g["c7x"])
    assert np.array_equal(array_api.make_cameras(10.0, 100.0, 5, 2), g["c5z"])


def test_psf_stub_like_reference(lib):
    sx, sy = ctypes.c_uint(0), ctypes.c_uint(0)
    lib.et_array_calculate_size_psf(ctypes.byref(sx), ctypes.byref(sy), 1, 1, 1, 1, 1, 1)
    assert (sx.value, sy.value) == (5, 5)
    buf = np.zeros(5 * 5 * 3, np.float32)
    assert lib.et_array_make_psf(buf.ctypes.data_as(ctypes.c_void_p), 5, 5, 1, 1, 1, 1, 1, 1, 3) == 0
    assert np.all(buf == 1)


def test_tuning_tables(lib):
    """The host-side tuning tables: set, read back, reject bad values, clear."""
    shape = (40, 44, 36, 7)
    assert lib.nrgb_get_project_slabs(*shape) == 0
    for s in (2, 4, 8, 16):
        assert lib.nrgb_set_project_slabs(*shape, s) == 0
        assert lib.nrgb_get_project_slabs(*shape) == s
    for bad in (1, 3, 32, -2):
        assert lib.nrgb_set_project_slabs(*shape, bad) == 2
    assert lib.nrgb_get_project_slabs(*shape) == 16
    assert lib.nrgb_set_project_slabs(*shape, 0) == 0
    assert lib.nrgb_get_project_slabs(*shape) == 0
    g0 = lib.nrgb_get_backproject_group(*shape)
    assert lib.nrgb_set_backproject_group(*shape, 5) == 0
    assert lib.nrgb_get_backproject_group(*shape) == 5
    assert lib.nrgb_set_backproject_group(*shape, 0) == 0
    assert lib.nrgb_get_backproject_group(*shape) == g0


def test_opposed_subsets():
    from niftyrec_gb300.plan import interleaved_subsets, opposed_subsets

    s = opposed_subsets(120, 8)
    assert s.shape == (120,) and s.min() == 0 and s.max() == 7
    assert (s[:60] == s[60:]).all()  # camera k and k + 60 share a subset
    counts = np.bincount(s)
    assert counts.max() - counts.min() <= 2
    np.testing.assert_array_equal(opposed_subsets(9, 3), interleaved_subsets(9, 3))
