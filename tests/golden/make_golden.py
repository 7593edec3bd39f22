"""Generate the golden fixtures in this folder from the reference's own CPU
path (oracle/_ref/libref_et.so, built from the reference sources by
oracle/Makefile.ref).  Run from the repository root:

    make -C oracle ref && python tests/golden/make_golden.py

Every fixture is an .npz holding the seeded inputs and the reference's float32
outputs, in nifti memory order (volumes (nz, ny, nx), sinograms
(n_cameras, ny, nx), cameras [3, n] or [6, n] axis-major, PSF (planes, k, k)).
The reference cannot run where the fixtures are consumed, so these files are
the travelling pin of the oracle and the parity target of the CUDA path.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402
from niftyrec_gb300 import synthetic as S  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, **arrays):
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(f"{name}: {os.path.getsize(path)} bytes")


def main():
    R = Reference()

    # 1. y-gantry, cubic, PSF + attenuation, the headline model at small size.
    shape = (24, 24, 24)
    act = S.ellipsoid_phantom(shape, seed=11)
    mu = S.mu_map(shape, seed=11)
    psf = S.gaussian_psf(7, 24, 0.5, 0.05)
    cams = S.cameras_about_y(10, 3.0)
    sino = R.project(act, cams[1], psf, mu)
    y = S.poisson_counts(sino, 50, seed=5)
    bk = R.backproject(y, cams[1], psf, mu)
    save("ygantry_psf_att_24", act=act, mu=mu, psf=psf, cameras=cams[1], sino=sino, counts=y, bkpr=bk)

    # 2. y-gantry, plain (no PSF, no attenuation), 1-column cameras, config-1 angles.
    shape = (20, 20, 20)
    act = S.ellipsoid_phantom(shape, seed=12)
    cams = R.make_cameras(0.0, 354.0, 12, 1)
    sino = R.project(act, cams[1])
    bk = R.backproject(sino, cams[1])
    save("ygantry_plain_20", act=act, cameras=cams[1], cameras3=cams, sino=sino, bkpr=bk)

    # 3. Non-cubic grid (nx=24, ny=20, nz=16), PSF + attenuation, 3-column cameras about y.
    shape = (16, 20, 24)
    act = S.ellipsoid_phantom(shape, seed=13)
    mu = S.mu_map(shape, seed=13)
    psf = S.gaussian_psf(5, 24, 0.6, 0.04)
    cams = S.cameras_about_y(7, 11.0)
    sino = R.project(act, cams, psf, mu)
    bk = R.backproject(sino, cams, psf, mu, nz=16)
    save("noncubic_24x20x16", act=act, mu=mu, psf=psf, cameras=cams, sino=sino, bkpr=bk)

    # 4. General 3-axis cameras with per-camera centres (6 columns), attenuation,
    #    non-zero backgrounds (exercises the reference's background resampling rule).
    shape = (18, 18, 18)
    act = S.ellipsoid_phantom(shape, seed=14)
    mu = S.mu_map(shape, seed=14)
    rng = np.random.default_rng(14)
    ang = rng.uniform(-1.2, 1.2, (3, 5)).astype(np.float32)
    cen = rng.uniform(6.0, 11.0, (3, 5)).astype(np.float32)
    cams6 = np.concatenate([ang, cen]).astype(np.float32)
    sino = R.project(act, cams6, None, mu, 0.25, 0.01)
    bk = R.backproject(sino, cams6, None, mu, 0.25, 0.01)
    sino0 = R.project(act, ang, None, mu)
    bk0 = R.backproject(sino0, ang, None, mu)
    save("general_cams_18", act=act, mu=mu, cameras6=cams6, cameras3=ang, bg=np.float32(0.25),
         bg_att=np.float32(0.01), sino_bg=sino, bkpr_bg=bk, sino=sino0, bkpr=bk0)

    # 5. One MLEM step (et_array_mlem_step) with PSF + attenuation.
    shape = (16, 16, 16)
    act = S.ellipsoid_phantom(shape, seed=15)
    mu = S.mu_map(shape, seed=15)
    psf = S.gaussian_psf(5, 16, 0.5, 0.05)
    cams = R.make_cameras(0.0, 350.0, 8, 1)
    y = S.poisson_counts(R.project(act, cams, psf, mu), 100, seed=2)
    x0 = np.ones(shape, np.float32)
    x1 = R.mlem_step(x0, y, cams, mu, psf)
    x2 = R.mlem_step(x1, y, cams, mu, psf)
    save("mlem_16", mu=mu, psf=psf, cameras3=cams, counts=y, x1=x1, x2=x2)

    # 6. Rotation alone (et_array_rotate), XYZ and ZYX orders.
    shape = (12, 14, 16)
    vol = S.ellipsoid_phantom(shape, seed=16)
    rot_xyz = R.rotate(vol, np.array([0.3, -0.7, 0.2], np.float32), np.array([7.5, 6.5, 5.5], np.float32), 0.0, 0)
    rot_zyx = R.rotate(vol, np.array([-0.3, 0.7, -0.2], np.float32), np.array([7.5, 6.5, 5.5], np.float32), 0.0, 5)
    save("rotate_16x14x12", vol=vol, rot_xyz=rot_xyz, rot_zyx=rot_zyx)

    # 7. make_cameras.
    save("make_cameras", c60=R.make_cameras(0.0, 354.0, 60, 1), c7x=R.make_cameras(-30.0, 45.0, 7, 0),
         c5z=R.make_cameras(10.0, 100.0, 5, 2))

    fisher(R)


def fisher(R):
    # 8. Fisher information of a 24-point grid (et_array_fisher_grid), PSF + attenuation.
    shape = (16, 16, 16)
    act = S.ellipsoid_phantom(shape, seed=17)
    mu = S.mu_map(shape, seed=17)
    psf = S.gaussian_psf(5, 16, 0.5, 0.05)
    cams = S.cameras_about_y(8, 5.0)
    grid = np.zeros(shape, np.float32)
    pts = np.random.default_rng(17).choice(grid.size, 24, replace=False)
    grid.flat[pts] = np.arange(1, 25, dtype=np.float32)
    f, pr = R.fisher_grid(act, cams, psf, grid, 24, mu)
    save("fisher_16", act=act, mu=mu, psf=psf, cameras=cams, grid=grid, fisher=f, prior=pr)


if __name__ == "__main__":
    # `python tests/golden/make_golden.py fisher` regenerates that fixture only
    if len(sys.argv) > 1 and sys.argv[1] == "fisher":
        fisher(Reference())
    else:
        main()
