"""Differentiation of the projector.

* Adjoint identity <A x, y> = <x, A^T y> for the transpose backprojector
  (mode 1), fused and general-orientation kernels: relative mismatch <= 1e-6.
* Autograd gradients (d/d activity via the transpose backprojector, d/d mu via
  the recomputed-scan kernel) against central finite differences with
  h = 1e-3 at 64 seeded voxels, the differences taken on the oracle's FP64
  restatement of the reference projector: relative error <= 1e-3.
* The reference's own attenuation-gradient semantics (et_array_gradient_attenuation,
  inverse-rotation gather, no PSF coupling) against the exact gradient of the
  Poisson log-likelihood: same direction (cosine >= 0.98).
"""
import numpy as np
import pytest

from niftyrec_gb300 import array_api as A
from niftyrec_gb300 import synthetic as S
from oracle.oracle import Restated

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHAPE = (24, 24, 24)


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def setup(seed=41, k=5, ncam=12, general=False):
    act = S.ellipsoid_phantom(SHAPE, seed=seed)
    mu = S.mu_map(SHAPE, seed=seed)
    psf = S.gaussian_psf(k, SHAPE[2], 0.5, 0.05) if k else None
    if general:
        cams = np.random.default_rng(seed).uniform(-1, 1, (3, ncam)).astype(np.float32)
    else:
        cams = S.cameras_about_y(ncam, 4.0)
    return act, mu, psf, cams


@pytest.mark.parametrize("general", [False, True])
def test_adjoint_identity(general):
    from niftyrec_gb300.autograd import backproject_raw, project_raw

    act, mu, psf, cams = setup(general=general)
    rng = np.random.default_rng(3)
    x = rng.random(SHAPE).astype(np.float32)
    y = rng.random((cams.shape[-1],) + SHAPE[1:]).astype(np.float32)
    Ax = project_raw(cuda(x), cuda(mu), cams, psf).cpu().numpy().astype(np.float64)
    Aty = backproject_raw(cuda(y), cuda(mu), cams, psf, nz=SHAPE[0], mode=1).cpu().numpy().astype(np.float64)
    lhs = float(np.sum(Ax * y))
    rhs = float(np.sum(x * Aty))
    assert abs(lhs - rhs) / abs(lhs) < 1e-6, (lhs, rhs)


def _fd_voxels(mask, n=64, seed=5):
    idx = np.argwhere(mask)
    sel = np.random.default_rng(seed).choice(len(idx), size=n, replace=False)
    return [tuple(v) for v in idx[sel]]


def test_autograd_matches_finite_differences():
    from niftyrec_gb300 import autograd as AG

    act, mu, psf, cams = setup()
    g = np.random.default_rng(11).random((cams.shape[-1],) + SHAPE[1:]).astype(np.float32)
    xa = cuda(act).requires_grad_(True)
    ma = cuda(mu).requires_grad_(True)
    p = AG.project(xa, ma, cams, psf)
    (p * cuda(g)).sum().backward()
    gx = xa.grad.cpu().numpy()
    gm = ma.grad.cpu().numpy()

    o64 = Restated("f64")
    g64 = g.astype(np.float64)

    def L(a, m):
        return float(np.sum(o64.project(a, cams, psf, m, truncate=0) * g64))

    h = 1e-3
    a64, m64 = act.astype(np.float64), mu.astype(np.float64)
    fdx, anx, fdm, anm = [], [], [], []
    for v in _fd_voxels(act > 0.2):
        ap, am = a64.copy(), a64.copy()
        ap[v] += h
        am[v] -= h
        fdx.append((L(ap, m64) - L(am, m64)) / (2 * h))
        anx.append(gx[v])
    for v in _fd_voxels(mu > 0.01, seed=6):
        mp, mm = m64.copy(), m64.copy()
        mp[v] += h
        mm[v] -= h
        fdm.append((L(a64, mp) - L(a64, mm)) / (2 * h))
        anm.append(gm[v])
    fdx, anx, fdm, anm = map(np.asarray, (fdx, anx, fdm, anm))
    assert np.linalg.norm(anx - fdx) / np.linalg.norm(fdx) < 1e-3
    assert np.linalg.norm(anm - fdm) / np.linalg.norm(fdm) < 1e-3


def test_poisson_nll_gradients_finite_differences():
    """Config-3 form at small size: Poisson NLL of the projection against counts."""
    from niftyrec_gb300 import autograd as AG

    act, mu, psf, cams = setup(seed=43)
    y = S.poisson_counts(A.project(act, cams, psf, mu, truncate_negative_values=0), 50, seed=4)
    x0 = np.clip(act * 0.9 + 0.05, 0, None).astype(np.float32)
    xa = cuda(x0).requires_grad_(True)
    ma = cuda(mu).requires_grad_(True)
    AG.poisson_nll(AG.project(xa, ma, cams, psf), cuda(y)).backward()
    gx, gm = xa.grad.cpu().numpy(), ma.grad.cpu().numpy()
    o64 = Restated("f64")
    y64 = y.astype(np.float64)

    def L(a, m):
        p = o64.project(a, cams, psf, m, truncate=0)
        return float(np.sum(p - y64 * np.log(np.maximum(p, 1e-9))))

    h = 1e-3
    a64, m64 = x0.astype(np.float64), mu.astype(np.float64)
    fd, an = [], []
    for v in _fd_voxels(x0 > 0.2, n=32, seed=8):
        ap, am = a64.copy(), a64.copy()
        ap[v] += h
        am[v] -= h
        fd.append((L(ap, m64) - L(am, m64)) / (2 * h))
        an.append(gx[v])
    for v in _fd_voxels(mu > 0.01, n=32, seed=9):
        mp, mm = m64.copy(), m64.copy()
        mp[v] += h
        mm[v] -= h
        fd.append((L(a64, mp) - L(a64, mm)) / (2 * h))
        an.append(gm[v])
    fd, an = np.asarray(fd), np.asarray(an)
    assert np.linalg.norm(an - fd) / np.linalg.norm(fd) < 1e-3


def test_reference_attenuation_gradient_direction():
    """Without PSF and background, the reference's G(y/p) - G(1) approximates the
    exact NLL gradient in mu up to its inverse-rotation gather."""
    from niftyrec_gb300 import autograd as AG

    act, mu, _, cams = setup(seed=44, k=0)
    y = S.poisson_counts(A.project(act, cams, None, mu, truncate_negative_values=0), 50, seed=2)
    xa = cuda(act)
    ma = cuda(mu).requires_grad_(True)
    p = AG.project(xa, ma, cams, None)
    AG.poisson_nll(p, cuda(y)).backward()
    exact = ma.grad.cpu().numpy()
    ratio = y / np.maximum(p.detach().cpu().numpy(), 1e-9)
    ref = (A.gradient_attenuation(ratio, act, mu, cams, None, truncate_negative_values=0)
           - A.gradient_attenuation(np.ones_like(ratio), act, mu, cams, None, truncate_negative_values=0))
    cos = float(np.sum(exact * ref) / (np.linalg.norm(exact) * np.linalg.norm(ref)))
    assert cos > 0.98, cos


@pytest.mark.parametrize("shape,k", [((24, 24, 24), 5), ((20, 140, 28), 7), ((24, 20, 24), 0)])
def test_fused_dmu_matches_general_path(shape, k):
    """The fused y-gantry d/dmu kernel (clusters of depth slabs, two walks)
    against the general-orientation kernels: the same cameras with theta_z =
    1e-9 rad (a rotation far below float resolution) take the general path."""
    from niftyrec_gb300 import _lib
    from niftyrec_gb300.autograd import attenuation_grad_raw

    L = _lib.load()
    act = S.ellipsoid_phantom(shape, seed=52)
    mu = S.mu_map(shape, seed=52)
    psf = S.gaussian_psf(k, shape[2], 0.5, 0.05) if k else None
    cams = np.zeros((3, 10), np.float32)
    cams[1] = np.deg2rad(7.0 + 36.0 * np.arange(10)).astype(np.float32)
    g = cuda(np.random.default_rng(3).uniform(0.5, 1.5, (10, shape[1], shape[2])))
    fused = attenuation_grad_raw(g, cuda(act), cuda(mu), cams, psf).cpu().numpy()
    assert L.nrgb_last_path() == 1
    tilted = cams.copy()
    tilted[2] = 1e-9
    general = attenuation_grad_raw(g, cuda(act), cuda(mu), tilted, psf).cpu().numpy()
    assert L.nrgb_last_path() == 2
    assert np.linalg.norm(fused - general) / np.linalg.norm(general) < 1e-5
