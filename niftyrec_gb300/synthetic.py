"""Seeded synthetic SPECT inputs: ellipsoid phantoms, attenuation maps,
depth-dependent Gaussian PSFs, camera sets and Poisson sinograms.

The reference's sample data files are not available, so these stand in for
them with the shapes and value ranges of the benchmark workloads:

* activity: a body ellipsoid (semi-axes 0.45 * dims) at 0.1 plus six random
  ellipsoids (centres U[0.3, 0.7] * dims, semi-axes U[0.08, 0.25] * dims,
  random orientation) adding U(0.5, 2) each;
* mu: the body ellipsoid at 0.015 / voxel with two ellipsoid inserts at 0.03
  and 0.005;
* PSF: per depth plane z an k x k Gaussian with sigma = s0 + slope * z,
  normalised to sum 1.

All volumes are C-order numpy arrays with shape (nz, ny, nx), i.e. their
memory is in nifti order (x fastest).  PSFs have shape (nplanes, k, k) (nifti
[k, k, nplanes]).  Camera arrays are [3, n] axis-major (theta_x, theta_y,
theta_z rows) in radians.
"""
from __future__ import annotations

import numpy as np


def _grid(shape):
    nz, ny, nx = shape
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return np.stack([x, y, z], axis=-1).astype(np.float64)


def _random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d],
    ])


def _inside(pts, center, semi, rot=None):
    d = pts - center
    if rot is not None:
        d = d @ rot
    return np.sum((d / semi) ** 2, axis=-1) <= 1.0


def ellipsoid_phantom(shape, seed=0, n_ellipsoids=6, dtype=np.float32):
    """Activity phantom of shape (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    dims = np.array([nx, ny, nz], dtype=np.float64)
    pts = _grid(shape)
    centre = (dims - 1) / 2.0
    vol = np.where(_inside(pts, centre, 0.45 * dims), 0.1, 0.0)
    for _ in range(n_ellipsoids):
        c = rng.uniform(0.3, 0.7, size=3) * dims
        semi = rng.uniform(0.08, 0.25, size=3) * dims
        rot = _random_rotation(rng)
        val = rng.uniform(0.5, 2.0)
        vol = vol + np.where(_inside(pts, c, semi, rot), val, 0.0)
    return vol.astype(dtype)


def mu_map(shape, seed=0, dtype=np.float32):
    """Attenuation map of shape (nz, ny, nx): body 0.015, inserts 0.03 and 0.005 per voxel."""
    rng = np.random.default_rng(seed + 1000)
    nz, ny, nx = shape
    dims = np.array([nx, ny, nz], dtype=np.float64)
    pts = _grid(shape)
    centre = (dims - 1) / 2.0
    body = _inside(pts, centre, 0.45 * dims)
    mu = np.where(body, 0.015, 0.0)
    for val in (0.03, 0.005):
        c = centre + rng.uniform(-0.15, 0.15, size=3) * dims
        semi = rng.uniform(0.08, 0.15, size=3) * dims
        mu = np.where(body & _inside(pts, c, semi, _random_rotation(rng)), val, mu)
    return mu.astype(dtype)


def gaussian_psf(k, nplanes, sigma0=0.5, slope=0.02, dtype=np.float32):
    """Depth-dependent Gaussian PSF of shape (nplanes, k, k), each plane summing to 1."""
    r = (k - 1) / 2.0
    u = np.arange(k) - r
    out = np.empty((nplanes, k, k), dtype=np.float64)
    for z in range(nplanes):
        s = sigma0 + slope * z
        g = np.exp(-0.5 * (u / s) ** 2)
        p = np.outer(g, g)
        out[z] = p / p.sum()
    return out.astype(dtype)


def cameras_about_y(n, first_deg=0.0, step_deg=None, dtype=np.float32):
    """[3, n] cameras rotating about the gantry axis (nifti y): angles first + k*step degrees."""
    step = 360.0 / n if step_deg is None else step_deg
    cams = np.zeros((3, n), dtype=np.float64)
    cams[1] = np.deg2rad(first_deg + step * np.arange(n))
    return cams.astype(dtype)


def poisson_counts(projection, scale, seed=1):
    """Seeded Poisson counts of scale * projection, float32."""
    rng = np.random.default_rng(seed)
    lam = np.clip(np.asarray(projection, dtype=np.float64) * scale, 0, None)
    return rng.poisson(lam).astype(np.float32)
