"""The seeded synthetic inputs that stand in for the benchmark's data: shapes,
value ranges, determinism and the PSF's normalisation (no GPU)."""
import numpy as np

from niftyrec_gb300 import synthetic as S


def test_phantom_and_mu_map_ranges_and_determinism():
    shape = (20, 16, 24)
    a = S.ellipsoid_phantom(shape, seed=5)
    m = S.mu_map(shape, seed=5)
    assert a.shape == shape and m.shape == shape and a.dtype == np.float32
    assert np.array_equal(a, S.ellipsoid_phantom(shape, seed=5))
    assert not np.array_equal(a, S.ellipsoid_phantom(shape, seed=6))
    assert a.min() >= 0.0 and a.max() > 0.5  # background 0.1 plus inserts of 0.5..2 each
    assert set(np.unique(m)) <= {0.0, np.float32(0.005), np.float32(0.015), np.float32(0.03)}
    assert m[shape[0] // 2, shape[1] // 2, shape[2] // 2] > 0  # the body covers the centre
    assert a[0, 0, 0] == 0.0 and m[0, 0, 0] == 0.0  # corners lie outside the body


def test_gaussian_psf_planes():
    p = S.gaussian_psf(11, 30, 0.5, 0.02)
    assert p.shape == (30, 11, 11)
    np.testing.assert_allclose(p.sum(axis=(1, 2)), 1.0, rtol=1e-6)
    assert np.allclose(p, p[:, ::-1, :]) and np.allclose(p, p.transpose(0, 2, 1))  # symmetric
    centre = p[:, 5, 5]
    assert np.all(np.diff(centre) < 0)  # wider with depth
    assert np.allclose(p[0], np.outer(p[0, 5], p[0, :, 5]) / p[0, 5, 5])  # separable


def test_cameras_and_counts():
    c = S.cameras_about_y(120, 0.0, 3.0)
    assert c.shape == (3, 120) and not c[0].any() and not c[2].any()
    np.testing.assert_allclose(np.rad2deg(c[1]), 3.0 * np.arange(120), atol=1e-4)
    np.testing.assert_allclose(np.rad2deg(S.cameras_about_y(8)[1]), 45.0 * np.arange(8), atol=1e-4)
    proj = np.full((2, 4, 4), 2.0, np.float32)
    y = S.poisson_counts(proj, 50, seed=3)
    assert y.dtype == np.float32 and np.array_equal(y, S.poisson_counts(proj, 50, seed=3))
    assert abs(y.mean() - 100.0) < 10.0
    assert not S.poisson_counts(-proj, 50).any()  # negative projections clip to zero
