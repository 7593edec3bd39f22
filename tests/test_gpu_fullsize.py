"""Parity at the benchmark configurations' own sizes, through the C-ABI.

* Headline workload (128^3 activity and mu, depth-dependent Gaussian PSF
  11 x 11 with sigma = 0.5 + 0.02 z, 120 cameras k * 3 degrees about the
  gantry axis): every one of the 120 projection planes and the reference
  backprojection of all 120 cameras against the oracle's float32
  restatement, relative L2 <= 1e-5 per plane / per volume.  At this size the
  launchers take the paths the benchmark times: 60 mirror units (cameras k and
  k + 60), projector clusters of several depth slabs, two camera groups of 30
  units in the backprojector, the PSF as a kernel-parameter table.  Both the
  host-buffer entry points (SPECT_project_parallelholes /
  SPECT_backproject_parallelholes) and the device-buffer ones the benchmark
  calls are checked.
* The reference attenuation gradient (et_array_gradient_attenuation) at the
  same size against the oracle's restatement, <= 1e-5.
* One and two MLEM steps (et_array_mlem_step) at 64^3 x 60 cameras
  (0..354 degrees, no PSF, no mu; counts Poisson(100 A x), seed 1) against the
  oracle's step, <= 1e-5 / 2e-5.
* Differentiation at 128^3 x 120 (PSF 11, mu, Poisson NLL against seeded
  counts): autograd gradients in activity and mu against central finite
  differences (h = 1e-3, 64 seeded voxels each), evaluated with the float64
  GPU run of the reference projector (itself equal to the oracle's float64
  build to 1e-12 at small sizes), relative L2 <= 1e-3.

The oracle runs in a pool of spawned processes over the host's cores, one
share of the cameras each.
"""
import numpy as np
import pytest

from conftest import rel_l2
from niftyrec_gb300 import array_api as A
from niftyrec_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL = 1e-5
FUSED = 1
N = 128
NCAM = 120
K = 11


@pytest.fixture(scope="module")
def pool():
    from oracle.parallel import Pool

    p = Pool(precision="f32")
    yield p
    p.close()


@pytest.fixture(scope="module")
def headline():
    act = S.ellipsoid_phantom((N, N, N), seed=0)
    mu = S.mu_map((N, N, N), seed=0)
    psf = S.gaussian_psf(K, N, 0.5, 0.02)
    cams = S.cameras_about_y(NCAM, 0.0, 3.0)
    return act, mu, psf, cams


@pytest.fixture(scope="module")
def headline_oracle(pool, headline):
    act, mu, psf, cams = headline
    so = pool.project(act, cams, psf, mu)
    bo = pool.backproject(so, cams, psf, mu, nz=N)
    return so, bo


def per_plane_rel(a, b):
    return max(rel_l2(a[i], b[i]) for i in range(b.shape[0]))


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def test_headline_projection_all_angles(headline, headline_oracle):
    from niftyrec_gb300 import precision as pr

    act, mu, psf, cams = headline
    so, _ = headline_oracle
    s = A.project(act, cams, psf, mu)
    assert A.last_path() == FUSED
    assert per_plane_rel(s, so) < RTOL
    sd = pr.project(cuda(act), cuda(mu), cams[1], psf, truncate=True).cpu().numpy()
    assert A.last_path() == FUSED
    assert per_plane_rel(sd, so) < RTOL


def test_headline_backprojection_all_angles(headline, headline_oracle):
    from niftyrec_gb300 import precision as pr

    act, mu, psf, cams = headline
    so, bo = headline_oracle
    b = A.backproject(so, cams, psf, mu, nz=N)
    assert A.last_path() == FUSED
    assert rel_l2(b, bo) < RTOL
    bd = pr.backproject(cuda(so), cuda(mu), cams[1], psf, nz=N, truncate=True).cpu().numpy()
    assert A.last_path() == FUSED
    assert rel_l2(bd, bo) < RTOL
    # per depth plane as well: no slab or group seam
    assert per_plane_rel(bd, bo) < 10 * RTOL


def test_headline_reference_attenuation_gradient(pool, headline):
    act, mu, psf, cams = headline
    sino = np.random.default_rng(7).uniform(0.5, 1.5, (NCAM, N, N)).astype(np.float32)
    g = A.gradient_attenuation(sino, act, mu, cams, psf, truncate_negative_values=0)
    assert A.last_path() == FUSED
    go = pool.gradient_attenuation(sino, act, mu, cams, psf, truncate=0)
    assert rel_l2(g, go) < RTOL


def test_config1_mlem_steps_64():
    from oracle.oracle import Restated

    o = Restated("f32")
    shape = (64, 64, 64)
    x_true = S.ellipsoid_phantom(shape, seed=0)
    cams3 = A.make_cameras(0.0, 354.0, 60, 1)
    assert cams3.shape == (3, 60)
    y = S.poisson_counts(o.project(x_true, cams3), 100, seed=1)
    x0 = np.ones(shape, np.float32)
    x1 = A.mlem_step(x0, y, cams3)
    assert A.last_path() == FUSED
    x1o = o.osem_step(x0, y, cams3, list(range(60)))
    assert rel_l2(x1, x1o) < RTOL
    x2 = A.mlem_step(x1, y, cams3)
    x2o = o.osem_step(x1o, y, cams3, list(range(60)))
    assert rel_l2(x2, x2o) < 2 * RTOL


def _fd_voxels(mask, n=64, seed=5):
    idx = np.argwhere(mask)
    sel = np.random.default_rng(seed).choice(len(idx), size=n, replace=False)
    return [tuple(int(c) for c in v) for v in idx[sel]]


def test_config3_gradients_finite_differences_128(headline):
    """Poisson NLL L(x, mu) = sum(p - y log p) with p the projection; the
    difference L(+h) - L(-h) is summed from per-pixel differences in float64,
    so the 2M-term sums do not drown it in rounding."""
    from niftyrec_gb300 import autograd as AG
    from niftyrec_gb300 import precision as pr

    act, mu, psf, cams = headline
    y = S.poisson_counts(A.project(act, cams, psf, mu, truncate_negative_values=0), 50, seed=3)
    x0 = (0.9 * act + 0.05).astype(np.float32)
    xa = cuda(x0).requires_grad_(True)
    ma = cuda(mu).requires_grad_(True)
    AG.poisson_nll(AG.project(xa, ma, cams[1], psf), cuda(y)).backward()
    gx, gm = xa.grad.cpu().numpy(), ma.grad.cpu().numpy()

    dev = xa.device
    y64 = torch.from_numpy(y.astype(np.float64)).to(dev)
    x64 = torch.from_numpy(x0.astype(np.float64)).to(dev)
    m64 = torch.from_numpy(mu.astype(np.float64)).to(dev)
    h = 1e-3

    def dL(xp, mp, xm, mm):
        pp = pr.project(xp, mp, cams[1], psf)
        pm = pr.project(xm, mm, cams[1], psf)
        d = (pp - pm) - y64 * torch.log1p((pp - pm) / pm)
        return float(d.sum()) / (2 * h)

    fdx, anx = [], []
    for v in _fd_voxels(x0 > 0.2, seed=5):
        xp, xm = x64.clone(), x64.clone()
        xp[v] += h
        xm[v] -= h
        fdx.append(dL(xp, m64, xm, m64))
        anx.append(gx[v])
    fdm, anm = [], []
    for v in _fd_voxels(mu > 0.01, seed=6):
        mp, mm = m64.clone(), m64.clone()
        mp[v] += h
        mm[v] -= h
        fdm.append(dL(x64, mp, x64, mm))
        anm.append(gm[v])
    fdx, anx, fdm, anm = map(np.asarray, (fdx, anx, fdm, anm))
    assert np.linalg.norm(anx - fdx) / np.linalg.norm(fdx) < 1e-3
    assert np.linalg.norm(anm - fdm) / np.linalg.norm(fdm) < 1e-3


def test_config3_reference_gradient_direction_128(headline):
    """Without PSF the reference's attenuation gradient G(y/p) - G(1) points
    along the exact Poisson-NLL gradient in mu at the full size as well."""
    from niftyrec_gb300 import autograd as AG

    act, mu, _, cams = headline
    y = S.poisson_counts(A.project(act, cams, None, mu, truncate_negative_values=0), 50, seed=2)
    ma = cuda(mu).requires_grad_(True)
    p = AG.project(cuda(act), ma, cams[1], None)
    AG.poisson_nll(p, cuda(y)).backward()
    exact = ma.grad.cpu().numpy()
    ratio = y / np.maximum(p.detach().cpu().numpy(), 1e-9)
    ref = (A.gradient_attenuation(ratio, act, mu, cams, None, truncate_negative_values=0)
           - A.gradient_attenuation(np.ones_like(ratio), act, mu, cams, None, truncate_negative_values=0))
    cos = float(np.sum(exact * ref) / (np.linalg.norm(exact) * np.linalg.norm(ref)))
    assert cos > 0.98, cos


def test_headline_adjoint_identity_128(headline):
    """The exact-transpose backprojector at the headline size: <Ax, y> = <x, A^T y>."""
    from niftyrec_gb300.autograd import backproject_raw, project_raw

    _, mu, psf, cams = headline
    rng = np.random.default_rng(3)
    x = rng.random((N, N, N)).astype(np.float32)
    yv = rng.random((NCAM, N, N)).astype(np.float32)
    Ax = project_raw(cuda(x), cuda(mu), cams[1], psf).double()
    Aty = backproject_raw(cuda(yv), cuda(mu), cams[1], psf, nz=N, mode=1).double()
    lhs = float((Ax * cuda(yv).double()).sum())
    rhs = float((cuda(x).double() * Aty).sum())
    assert abs(lhs - rhs) / abs(lhs) < 1e-6, (lhs, rhs)
