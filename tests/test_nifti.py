"""NIfTI-1 image I/O of the library (nrgb_nifti_*) and the rec_spect command
line without a GPU: files written here from the NIfTI-1 header layout are
read by the library, files the library writes are parsed here, and the
command line parses the reference tool's options."""
import gzip
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from niftyrec_gb300 import _lib
    return _lib.load()


def write_nifti(path, arr, dtype_code, np_dtype, endian="<", slope=0.0, inter=0.0, offset=352):
    """A single-file NIfTI-1 image from the format definition (348-byte header,
    dims x fastest: arr is indexed [z][y][x])."""
    dims = arr.shape[::-1]
    hdr = bytearray(348)
    struct.pack_into(endian + "i", hdr, 0, 348)
    struct.pack_into(endian + "8h", hdr, 40, len(dims), *dims, *([1] * (7 - len(dims))))
    struct.pack_into(endian + "hh", hdr, 70, dtype_code, np.dtype(np_dtype).itemsize * 8)
    struct.pack_into(endian + "8f", hdr, 76, 1, 1, 1, 1, 1, 1, 1, 1)
    struct.pack_into(endian + "fff", hdr, 108, float(offset), slope, inter)
    hdr[344:348] = b"n+1\0"
    data = np.ascontiguousarray(arr, dtype=np.dtype(np_dtype).newbyteorder(endian)).tobytes()
    blob = bytes(hdr) + b"\0" * (offset - 348) + data
    if path.endswith(".gz"):
        with gzip.open(path, "wb") as f:
            f.write(blob)
    else:
        with open(path, "wb") as f:
            f.write(blob)


def read_nifti(path):
    """Parse a little-endian float32 single-file NIfTI-1 image."""
    blob = gzip.open(path).read() if path.endswith(".gz") else open(path, "rb").read()
    assert struct.unpack_from("<i", blob, 0)[0] == 348 and blob[344:348] == b"n+1\0"
    nd = struct.unpack_from("<h", blob, 40)[0]
    dims = struct.unpack_from("<7h", blob, 42)[:nd]
    dtype, bitpix = struct.unpack_from("<hh", blob, 70)
    assert (dtype, bitpix) == (16, 32)
    off = int(struct.unpack_from("<f", blob, 108)[0])
    return np.frombuffer(blob, "<f4", int(np.prod(dims)), off).reshape(dims[::-1])


def lib_read(lib, path):
    import ctypes

    dims = (ctypes.c_int * 8)()
    assert lib.nrgb_nifti_info(path.encode(), dims) == 0
    shape = tuple(dims[1:1 + dims[0]])[::-1]
    out = np.empty(shape, np.float32)
    assert lib.nrgb_nifti_read(path.encode(), out.ctypes.data_as(ctypes.c_void_p), out.size) == 0
    return out


@pytest.mark.parametrize("code,dt,endian,slope,inter", [
    (16, "f4", "<", 0.0, 0.0), (16, "f4", ">", 0.0, 0.0), (4, "i2", "<", 0.5, -3.0), (64, "f8", "<", 0.0, 0.0),
    (2, "u1", ">", 2.0, 0.0), (512, "u2", "<", 1.0, 0.0), (8, "i4", ">", 0.0, 0.0)])
def test_read_datatypes(tmp_path, lib, code, dt, endian, slope, inter):
    rng = np.random.default_rng(code)
    arr = (rng.uniform(0, 100, (5, 4, 3)) if dt.startswith("f") else rng.integers(0, 100, (5, 4, 3))).astype(dt)
    p = str(tmp_path / "img.nii")
    write_nifti(p, arr, code, dt, endian, slope, inter, offset=368)
    got = lib_read(lib, p)
    want = arr.astype(np.float64) * slope + inter if slope not in (0.0, 1.0) else arr.astype(np.float64)
    np.testing.assert_allclose(got, want.astype(np.float32), rtol=1e-6)


def test_write_roundtrip(tmp_path, lib):
    import ctypes

    arr = np.random.default_rng(3).standard_normal((6, 5, 7)).astype(np.float32)
    p = str(tmp_path / "out.nii")
    dims = (ctypes.c_int * 4)(3, 7, 5, 6)
    assert lib.nrgb_nifti_write(p.encode(), arr.ctypes.data_as(ctypes.c_void_p), dims) == 0
    np.testing.assert_array_equal(read_nifti(p), arr)
    np.testing.assert_array_equal(lib_read(lib, p), arr)
    if lib.nrgb_nifti_gzip_supported():
        pz = str(tmp_path / "out.nii.gz")
        assert lib.nrgb_nifti_write(pz.encode(), arr.ctypes.data_as(ctypes.c_void_p), dims) == 0
        np.testing.assert_array_equal(read_nifti(pz), arr)
        np.testing.assert_array_equal(lib_read(lib, pz), arr)
        write_nifti(str(tmp_path / "in.nii.gz"), arr, 16, "f4")
        np.testing.assert_array_equal(lib_read(lib, str(tmp_path / "in.nii.gz")), arr)


def test_bad_files(tmp_path, lib):
    import ctypes

    dims = (ctypes.c_int * 8)()
    assert lib.nrgb_nifti_info(str(tmp_path / "missing.nii").encode(), dims) == 2
    p = tmp_path / "junk.nii"
    p.write_bytes(b"x" * 400)
    assert lib.nrgb_nifti_info(str(p).encode(), dims) == 2
    arr = np.ones((2, 2, 2), np.float32)
    write_nifti(str(p), arr, 16, "f4")
    out = np.empty(7, np.float32)
    assert lib.nrgb_nifti_read(str(p).encode(), out.ctypes.data_as(ctypes.c_void_p), 7) == 2  # count mismatch


TOOL = os.path.join(ROOT, "niftyrec_gb300", "rec_spect")


@pytest.mark.skipif(not os.path.exists(TOOL), reason="rec_spect not built")
def test_rec_spect_options(tmp_path):
    r = subprocess.run([TOOL, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--sinogram" in r.stdout and "--subsets" in r.stdout
    r = subprocess.run([TOOL, "--xml"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("<?xml")
    assert subprocess.run([TOOL, "-o", "x.nii"], capture_output=True).returncode == 1  # no sinogram
    assert subprocess.run([TOOL, "-s", "a.png", "-o", "x.nii"], capture_output=True).returncode == 1
    assert subprocess.run([TOOL, "--bogus"], capture_output=True).returncode == 1
    r = subprocess.run([TOOL, "-s", str(tmp_path / "none.nii"), "-o", str(tmp_path / "o.nii")], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "Couldn't load the sinogram" in r.stdout
