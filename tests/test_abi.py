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


def _windows(lib, ny, k):
    out = (ctypes.c_int * (4 * (ny + 1)))()
    n = ctypes.c_int(0)
    assert lib.nrgb_row_windows(ny, k, out, ny + 1, ctypes.byref(n)) == 0
    return [tuple(out[4 * i:4 * i + 4]) for i in range(n.value)]


@pytest.mark.parametrize("k", [0, 1, 3, 5, 11, 15])
def test_row_windows_partition_rows(lib, k):
    """Row windows of the fused kernels: at most 128 rows, starts and valid
    ranges on multiples of 4 (except at the volume's end), valid ranges
    partition [0, ny) in order, and every valid row's PSF support lies inside
    its window or past the volume's edge."""
    r = (k - 1) // 2 if k else 0
    for ny in list(range(1, 300)) + [511, 512, 513, 1000]:
        wins = _windows(lib, ny, k)
        assert wins
        expect = 0
        for row0, rows, lo, hi in wins:
            assert row0 % 4 == 0 and 0 < rows <= 128 and row0 + rows <= ny
            assert 0 <= lo < hi <= rows
            assert row0 + lo == expect
            assert (row0 + lo) % 4 == 0 and ((row0 + hi) % 4 == 0 or row0 + hi == ny)
            for y in (row0 + lo, row0 + hi - 1):
                assert max(0, y - r) >= row0 and min(ny - 1, y + r) < row0 + rows, (ny, k, y)
            expect = row0 + hi
        assert expect == ny
    if k == 15:
        assert [w[3] - w[2] for w in _windows(lib, 256, 15)] == [120, 112, 24]
    out, n = (ctypes.c_int * 4)(), ctypes.c_int(0)
    assert lib.nrgb_row_windows(300, k, out, 1, ctypes.byref(n)) == 2 and n.value > 1  # too small an output
    assert lib.nrgb_row_windows(0, k, out, 1, ctypes.byref(n)) == 2


def _units(lib, cams, size):
    cams = np.ascontiguousarray(cams, np.float32)
    cs = (ctypes.c_int * 2)(*((cams.shape[0], 1) if cams.ndim == 1 else (cams.shape[1], cams.shape[0])))
    out = (ctypes.c_int * (2 * 4096))()
    n = ctypes.c_int(0)
    st = lib.nrgb_mirror_units(cams.ctypes.data_as(ctypes.c_void_p), cs, (ctypes.c_int * 3)(*size), out, 4096,
                               ctypes.byref(n))
    assert st == 0
    return [tuple(out[2 * i:2 * i + 2]) for i in range(n.value)]


def test_mirror_units_of_camera_tables(lib):
    """Cameras at opposite angles about the grid centre pair up; odd counts
    leave cameras unpaired; tilted or off-centre cameras and the switch off
    form no units; cameras about x pair on the x-gantry form."""
    from niftyrec_gb300 import synthetic as S

    size = (32, 24, 32)
    u = _units(lib, S.cameras_about_y(120, 0.0, 3.0)[1], size)
    assert u == [(k, k + 60) for k in range(60)]
    u = _units(lib, S.cameras_about_y(7, 10.0), size)  # 360/7 deg steps: no opposite pairs
    assert u == []
    cams = S.cameras_about_y(5, 0.0, 45.0)  # 0, 45, 90, 135, 180 deg
    u = _units(lib, cams, size)
    assert u == [(0, 4), (1, -1), (2, -1), (3, -1)]
    tilted = S.cameras_about_y(4, 0.0)
    tilted[2] = 1e-3
    assert _units(lib, tilted, size) == []
    six = np.zeros((6, 4), np.float32)
    six[1] = np.deg2rad([0, 180, 90, 270])
    six[3:] = 5.0  # centres away from the grid centre
    assert _units(lib, six, size) == []
    about_x = np.zeros((3, 4), np.float32)
    about_x[0] = np.deg2rad([0, 90, 180, 270])
    assert _units(lib, about_x, size) == [(0, 2), (1, 3)]
    assert lib.nrgb_set_mirror_pairs(0) == 0
    try:
        assert _units(lib, S.cameras_about_y(120, 0.0, 3.0)[1], size) == []
    finally:
        lib.nrgb_set_mirror_pairs(1)


def _greedy_units(theta, centred):
    """Restatement of the pairing rule: camera i (in order) takes the first
    later free camera whose angle differs by pi within 1e-6 rad (modulo 2 pi)."""
    n = len(theta)
    mate, taken = [-1] * n, [False] * n
    for i in range(n):
        if taken[i] or not centred[i]:
            continue
        for j in range(i + 1, n):
            if taken[j] or not centred[j]:
                continue
            d = float(theta[j]) - float(theta[i]) - np.pi
            if abs(d - 2 * np.pi * round(d / (2 * np.pi))) <= 1e-6:
                mate[i], taken[i], taken[j] = j, True, True
                break
    if not any(taken):
        return []
    return [(i, mate[i]) for i in range(n) if not (taken[i] and mate[i] < 0)]


@pytest.mark.parametrize("seed", range(6))
def test_mirror_units_match_greedy_rule(lib, seed):
    """The angle-sorted lookup pairs exactly like a scan over all later
    cameras: repeated angles, pairs across the 0 / 2 pi seam, differences just
    inside and just outside the tolerance, off-centre cameras."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 400))
    base = rng.choice(np.deg2rad(np.arange(0.0, 360.0, 1.5)), n)
    jitter = rng.choice([0.0, 0.0, 4e-7, -9e-7, 3e-6, 2 * np.pi, -2 * np.pi], n)
    theta = (base + jitter).astype(np.float32)
    theta[: n // 10] = np.float32(np.pi) * rng.choice([1.0, -1.0, 3.0], n // 10).astype(np.float32)
    six = np.zeros((6, n), np.float32)
    six[1] = theta
    size = (40, 20, 40)
    six[3] = (size[0] - 1) / 2.0
    six[4] = (size[1] - 1) / 2.0
    six[5] = (size[2] - 1) / 2.0
    off = rng.random(n) < 0.1
    six[5, off] += 1.0
    got = _units(lib, six, size)
    assert got == _greedy_units(theta, ~off)


def test_autotune_cache_round_trip(lib, tmp_path):
    """Tuning results recorded in the JSON cache are applied to the library's
    tables by load_cache in a later process; a broken cache file is ignored."""
    from niftyrec_gb300 import autotune as AT

    path = str(tmp_path / "tune.json")
    key = AT._key(44, 40, 36, 9)
    AT._record(path, key, {"group": 6})
    AT._record(path, key, {"slabs": 4, "slabs_ms": {"4": 0.1}})
    cache = AT.load_cache(path)
    assert cache[key]["group"] == 6 and cache[key]["slabs"] == 4
    try:
        assert lib.nrgb_get_backproject_group(44, 40, 36, 9) == 6
        assert lib.nrgb_get_project_slabs(44, 40, 36, 9) == 4
    finally:
        lib.nrgb_set_backproject_group(44, 40, 36, 9, 0)
        lib.nrgb_set_project_slabs(44, 40, 36, 9, 0)
    (tmp_path / "bad.json").write_text("{not json")
    assert AT.load_cache(str(tmp_path / "bad.json")) == {}
    assert AT.load_cache(str(tmp_path / "missing.json")) == {}


def test_niftyrec_log_one_json_line_per_call():
    """NIFTYREC_LOG=1: every C-ABI call writes one JSON line on stderr (entry
    point, host time, path); unset, nothing is written."""
    import json
    import subprocess
    import sys

    code = ("import sys; sys.path.insert(0, %r); from niftyrec_gb300 import array_api as A; "
            "A.make_cameras(0.0, 90.0, 4, 1); A.make_cameras(0.0, 180.0, 3, 0)") % ROOT
    for env_val, expect in (("1", 2), ("0", 0)):
        env = dict(os.environ, NIFTYREC_LOG=env_val)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)
        assert r.returncode == 0, r.stderr
        lines = [json.loads(x) for x in r.stderr.splitlines() if x.startswith('{"niftyrec"')]
        assert len(lines) == expect
        for rec in lines:
            assert rec["niftyrec"] == "et_array_make_cameras" and rec["host_ms"] >= 0


def test_deterministic_switch_round_trip(lib):
    """nrgb_set_deterministic / nrgb_get_deterministic (a library-wide switch,
    host only; 0 by default)."""
    prev = lib.nrgb_get_deterministic()
    try:
        assert lib.nrgb_set_deterministic(1) == 0
        assert lib.nrgb_get_deterministic() == 1
        assert lib.nrgb_set_deterministic(0) == 0
        assert lib.nrgb_get_deterministic() == 0
    finally:
        lib.nrgb_set_deterministic(prev)


def test_affine_and_convolve_reject_bad_arguments(lib):
    """Argument checks that come before any GPU work: a matrix size other than
    {4, 4}, missing arrays, even or mismatched kernels -> status 2."""
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    vol = np.zeros((4, 5, 6), np.float32)
    out = np.zeros_like(vol)
    size = (ctypes.c_int * 3)(6, 5, 4)
    eye = np.eye(4, dtype=np.float32)
    assert lib.et_array_affine(p(vol), size, p(out), size, p(eye), (ctypes.c_int * 2)(4, 3), 0.0, 1) == 2
    assert lib.et_array_affine(p(vol), size, p(out), size, None, (ctypes.c_int * 2)(4, 4), 0.0, 1) == 2
    assert lib.et_array_affine(p(vol), (ctypes.c_int * 3)(6, 5, 0), p(out), size, p(eye), (ctypes.c_int * 2)(4, 4),
                               0.0, 1) == 2
    ker = np.zeros((4, 3, 3), np.float32)
    assert lib.et_array_convolve(p(vol), size, p(out), size, p(ker), (ctypes.c_int * 3)(4, 3, 4), 1) == 2
    assert lib.et_array_convolve(p(vol), size, p(out), size, p(ker), (ctypes.c_int * 3)(3, 3, 3), 1) == 2
    assert lib.et_array_convolve(p(vol), size, None, size, p(ker), (ctypes.c_int * 3)(3, 3, 4), 1) == 2
