"""Storage precision and the float64 reference run (niftyrec_gb300.precision).

* The GPU float64 run equals the oracle's float64 C restatement of the
  reference algorithm (relative L2 <= 1e-12: only exp and fused operations may
  differ in the last bits).
* float32 (the reference's type) against float64: <= 1e-5 relative L2 per
  projection plane and per backprojection.
* bfloat16 storage: exact on bfloat16-representable inputs up to float32
  arithmetic (<= 1e-5 against float64 on the same rounded inputs); against
  the unrounded inputs the error is the storage rounding (<= 4e-3).
* OSEM in the three variants: float32 and bfloat16 reconstructions stay
  within the stated bounds of the float64 one.
"""
import numpy as np
import pytest

from conftest import rel_l2
from niftyrec_gb300 import synthetic as S
from oracle.oracle import Restated

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SHAPE = (24, 20, 24)


def setup(seed=51, k=5, ncam=10, general=False):
    act = S.ellipsoid_phantom(SHAPE, seed=seed)
    mu = S.mu_map(SHAPE, seed=seed)
    psf = S.gaussian_psf(k, SHAPE[2], 0.5, 0.05) if k else None
    if general:
        cams = np.random.default_rng(seed).uniform(-1, 1, (3, ncam)).astype(np.float32)
    else:
        cams = S.cameras_about_y(ncam, 3.0)
    return act, mu, psf, cams


def dev(a, dtype=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda().to(dtype)


def per_plane(a, b):
    return max(rel_l2(a[i], b[i]) for i in range(b.shape[0]))


@pytest.mark.parametrize("general", [False, True])
def test_float64_run_matches_float64_oracle(general):
    from niftyrec_gb300 import precision as P

    act, mu, psf, cams = setup(general=general)
    o = Restated("f64")
    s = P.project(dev(act, torch.float64), dev(mu, torch.float64), cams, psf).cpu().numpy()
    so = o.project(act, cams, psf, mu, truncate=0)
    assert per_plane(s, so) < 1e-12
    b = P.backproject(dev(so, torch.float64), dev(mu, torch.float64), cams, psf, nz=SHAPE[0]).cpu().numpy()
    bo = o.backproject(so, cams, psf, mu, truncate=0, nz=SHAPE[0])
    assert rel_l2(b, bo) < 1e-12


def test_float32_within_1e5_of_float64():
    from niftyrec_gb300 import precision as P

    act, mu, psf, cams = setup(seed=52, k=7)
    p64 = P.project(dev(act, torch.float64), dev(mu, torch.float64), cams, psf)
    p32 = P.project(dev(act), dev(mu), cams, psf)
    assert P.rel_error(p32, p64)[1] < 1e-5
    b64 = P.backproject(p64, dev(mu, torch.float64), cams, psf, nz=SHAPE[0])
    b32 = P.backproject(p64.float(), dev(mu), cams, psf, nz=SHAPE[0])
    assert P.rel_error(b32, b64)[0] < 1e-5


@pytest.mark.parametrize("shape,ncam", [(SHAPE, 8), ((16, 140, 16), 8), ((64, 64, 64), 60), ((48, 48, 48), 7)])
def test_bfloat16_storage(shape, ncam):
    """Opposite cameras form mirror units in the bfloat16 kernels too (8 and
    60 cameras; 7 cameras have no opposite pairs); shape 2 has ny > 128: row
    windows of the bfloat16 kernels."""
    from niftyrec_gb300 import precision as P

    act = S.ellipsoid_phantom(shape, seed=53)
    mu = S.mu_map(shape, seed=53)
    psf = S.gaussian_psf(7, shape[2], 0.5, 0.05)
    cams = S.cameras_about_y(ncam, 3.0)
    a16, m16 = dev(act, torch.bfloat16), dev(mu, torch.bfloat16)
    p16 = P.project(a16, m16, cams, psf)
    assert p16.dtype == torch.float32
    from niftyrec_gb300 import array_api as A

    assert A.last_path() == 1
    # same (rounded) inputs in float64: only float32 arithmetic differs
    p64r = P.project(a16.double(), m16.double(), cams, psf)
    assert P.rel_error(p16, p64r)[1] < 1e-5
    # against the unrounded inputs: the bfloat16 rounding of activity and mu
    p64 = P.project(dev(act, torch.float64), dev(mu, torch.float64), cams, psf)
    assert P.rel_error(p16, p64)[1] < 4e-3
    b16 = P.backproject(p64r.float(), m16, cams, psf, nz=shape[0])
    b64r = P.backproject(p64r, m16.double(), cams, psf, nz=shape[0])
    assert P.rel_error(b16, b64r)[0] < 1e-5


def test_bfloat16_general_cameras_widen():
    from niftyrec_gb300 import precision as P

    act, mu, psf, cams = setup(seed=54, general=True)
    a16, m16 = dev(act, torch.bfloat16), dev(mu, torch.bfloat16)
    p16 = P.project(a16, m16, cams, psf)
    p64r = P.project(a16.double(), m16.double(), cams, psf)
    assert P.rel_error(p16, p64r)[1] < 1e-5


def test_osem_three_storages():
    from niftyrec_gb300 import precision as P

    act, mu, psf, cams = setup(seed=55, k=5, ncam=12)
    counts = dev(S.poisson_counts(Restated("f32").project(act, cams, psf, mu), 60, seed=3))
    m = dev(mu)
    x64 = P.osem(counts, cams, psf, m.double(), 3, 2, storage="float64")
    x32 = P.osem(counts, cams, psf, m, 3, 2, storage="float32")
    x16 = P.osem(counts, cams, psf, m, 3, 2, storage="bfloat16")
    assert x64.dtype == torch.float64 and x32.dtype == torch.float32
    assert P.rel_error(x32, x64)[0] < 1e-5
    assert P.rel_error(x16, x64)[0] < 1e-2
