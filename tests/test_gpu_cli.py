"""rec_spect on the GPU: the command-line MLEM equals the library's MLEM steps
on the same sinogram, cameras and PSF; OSEM and attenuation runs finish."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from niftyrec_gb300 import array_api as A
from niftyrec_gb300 import synthetic as S
from test_nifti import read_nifti, write_nifti

pytestmark = pytest.mark.gpu
TOOL = os.path.join(ROOT, "niftyrec_gb300", "rec_spect")


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    shape = (24, 20, 24)  # [N][M][N]
    act = S.ellipsoid_phantom(shape, seed=5)
    cams = A.make_cameras(0.0, 180.0, 16, 1)  # the tool's default first / last camera, gantry axis
    psf = np.ones((24, 5, 5), np.float32)  # et_array_make_psf: 5 x 5 ones per plane
    sino = A.project(act, cams, psf)
    write_nifti(str(d / "sino.nii"), sino, 16, "f4")
    mu = S.mu_map(shape, seed=5)
    write_nifti(str(d / "mu.nii"), mu, 16, "f4")
    return d, sino, cams, psf


def run(args):
    r = subprocess.run([TOOL] + args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def test_mlem_matches_library_steps(case):
    d, sino, cams, psf = case
    run(["-s", str(d / "sino.nii"), "-o", str(d / "mlem.nii"), "-x", "1", "-u", "1", "-i", "3"])
    got = read_nifti(str(d / "mlem.nii"))
    x = np.ones((24, 20, 24), np.float32)
    for _ in range(3):
        x = A.mlem_step(x, sino, cams, None, psf, epsilon=1e-7)
    assert got.shape == x.shape
    assert rel_l2(got, x) < 1e-6


def test_osem_and_attenuation_runs(case):
    d, sino, cams, psf = case
    run(["-s", str(d / "sino.nii"), "-o", str(d / "osem.nii"), "-x", "1", "-u", "4", "-i", "2",
         "--attenuation", str(d / "mu.nii")])
    got = read_nifti(str(d / "osem.nii"))
    assert got.shape == (24, 20, 24) and np.isfinite(got).all() and got.min() >= 0
    # the reference's default axis (0: rotation about x) runs on the general path
    run(["-s", str(d / "sino.nii"), "-o", str(d / "axis0.nii"), "-u", "1", "-i", "1"])
    assert np.isfinite(read_nifti(str(d / "axis0.nii"))).all()
