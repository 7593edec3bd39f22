"""Deterministic gradients (nrgb_set_deterministic).

With the switch on, the exact-transpose backprojector (mode 1) and the exact
d/dmu (nrgb_attenuation_grad_device) on the fused gantry kernels write their
rotated-frame values into camera-group scratch volumes and sum them with a
transposed bilinear gather in a fixed order.  Checked here:

* repeated calls give bit-identical volumes;
* the result equals the vector-reduction form to 1e-6 relative L2 (only the
  float32 summation order differs);
* the adjoint identity <A x, y> = <x, A^T y> holds to 1e-6 in the
  deterministic form;
* autograd gradients of a Poisson NLL are bit-identical across runs.

Cases: mirror units (even camera count, PSF, mu), unpaired cameras (odd
count), no PSF / no mu, row windows (ny > 128) and cameras rotating about x
(the gantry kernels with x and y exchanged)."""
import numpy as np
import pytest

from niftyrec_gb300 import _lib
from niftyrec_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _rel(a, b):
    a, b = a.double(), b.double()
    return float((a - b).norm() / b.norm().clamp_min(1e-300))


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.fixture
def det():
    from niftyrec_gb300.autograd import set_deterministic

    prev = set_deterministic(True)
    yield
    set_deterministic(prev)


def _cams(ncam, axis):
    cams = np.zeros((3, ncam), np.float32)
    cams[axis] = np.deg2rad(2.0 + 360.0 / ncam * np.arange(ncam))
    return cams


CASES = [
    ((64, 64, 64), 60, 7, True, 1),
    ((48, 40, 56), 7, 5, True, 1),
    ((40, 40, 40), 12, 0, False, 1),
    ((20, 150, 24), 8, 9, True, 1),
    ((32, 24, 40), 10, 5, True, 0),
]


@pytest.mark.parametrize("shape,ncam,k,att,axis", CASES)
def test_adjoint_backprojection_deterministic(shape, ncam, k, att, axis):
    from niftyrec_gb300.autograd import backproject_raw, project_raw, set_deterministic

    nz, ny, nx = shape
    rng = np.random.default_rng(ncam)
    mu = cuda(S.mu_map(shape, seed=nz)) if att else None
    psf = S.gaussian_psf(k, nz, 0.5, 0.03) if k else None
    cams = _cams(ncam, axis)
    y = cuda(rng.uniform(0.5, 1.5, (ncam, ny, nx)))
    x = cuda(rng.random(shape))
    L = _lib.load()
    prev = set_deterministic(False)
    try:
        ref = backproject_raw(y, mu, cams, psf, nz=nz, mode=1)
        set_deterministic(True)
        assert L.nrgb_get_deterministic() == 1
        b1 = backproject_raw(y, mu, cams, psf, nz=nz, mode=1)
        b2 = backproject_raw(y, mu, cams, psf, nz=nz, mode=1)
        torch.cuda.synchronize()
        assert torch.isfinite(b1).all()
        assert torch.equal(b1, b2)
        assert _rel(b1, ref) < 1e-6
        Ax = project_raw(x, mu, cams, psf).double()
        lhs = float((Ax * y.double()).sum())
        rhs = float((x.double() * b1.double()).sum())
        assert abs(lhs - rhs) / abs(lhs) < 1e-6, (lhs, rhs)
    finally:
        set_deterministic(prev)


@pytest.mark.parametrize("shape,ncam,k,axis", [((64, 64, 64), 60, 7, 1), ((20, 150, 24), 8, 9, 1),
                                               ((32, 24, 40), 10, 5, 0)])
def test_dmu_deterministic(shape, ncam, k, axis):
    from niftyrec_gb300.autograd import attenuation_grad_raw, set_deterministic

    nz, ny, nx = shape
    act = cuda(S.ellipsoid_phantom(shape, seed=3))
    mu = cuda(S.mu_map(shape, seed=3))
    psf = S.gaussian_psf(k, nz, 0.5, 0.03)
    cams = _cams(ncam, axis)
    g = cuda(np.random.default_rng(4).uniform(-1.0, 1.0, (ncam, ny, nx)))
    prev = set_deterministic(False)
    try:
        ref = attenuation_grad_raw(g, act, mu, cams, psf)
        set_deterministic(True)
        d1 = attenuation_grad_raw(g, act, mu, cams, psf)
        d2 = attenuation_grad_raw(g, act, mu, cams, psf)
        torch.cuda.synchronize()
        assert torch.equal(d1, d2)
        assert _rel(d1, ref) < 1e-6
    finally:
        set_deterministic(prev)


def test_autograd_gradients_bit_identical(det):
    from niftyrec_gb300 import autograd as AG

    shape = (48, 48, 48)
    act = S.ellipsoid_phantom(shape, seed=8)
    mu = S.mu_map(shape, seed=8)
    psf = S.gaussian_psf(7, 48, 0.5, 0.03)
    cams = S.cameras_about_y(30, 1.0)
    y = cuda(S.poisson_counts(np.ones((30, 48, 48), np.float32), 20, seed=2))
    grads = []
    for _ in range(2):
        xa = cuda(act).requires_grad_(True)
        ma = cuda(mu).requires_grad_(True)
        AG.poisson_nll(AG.project(xa, ma, cams[1], psf), y).backward()
        grads.append((xa.grad.clone(), ma.grad.clone()))
    assert torch.equal(grads[0][0], grads[1][0])
    assert torch.equal(grads[0][1], grads[1][1])


def test_pair_call_exact_transpose_deterministic(det):
    """nrgb_project_backproject_device in mode 1 with the switch on: repeated
    calls are bit-identical and equal the separate deterministic calls to 1e-6
    (the pair takes its carries from the projector)."""
    import ctypes

    vp = ctypes.c_void_p
    L = _lib.load()
    dev = torch.device("cuda", 0)
    sp = vp(torch.cuda.current_stream(dev).cuda_stream)
    shape = (64, 64, 64)
    nz, ny, nx = shape
    act = cuda(S.ellipsoid_phantom(shape, seed=9))
    mu = cuda(S.mu_map(shape, seed=9))
    psf = S.gaussian_psf(7, nz, 0.5, 0.03)
    cams = np.ascontiguousarray(S.cameras_about_y(40, 1.0)[1])
    size = (ctypes.c_int * 3)(nx, ny, nz)
    csize = (ctypes.c_int * 2)(40, 1)
    psize = (ctypes.c_int * 3)(*psf.shape[::-1])
    args = (cams.ctypes.data_as(vp), csize, psf.ctypes.data_as(vp), psize, 0.0, 0.0, 0, 1, sp)
    outs = []
    for _ in range(2):
        s = torch.empty((40, ny, nx), dtype=torch.float32, device=dev)
        b = torch.empty(shape, dtype=torch.float32, device=dev)
        assert L.nrgb_project_backproject_device(vp(act.data_ptr()), vp(mu.data_ptr()), size, vp(s.data_ptr()), None,
                                                 vp(b.data_ptr()), *args) == 0
        outs.append((s, b))
    bs = torch.empty(shape, dtype=torch.float32, device=dev)
    assert L.nrgb_backproject_device(vp(outs[0][0].data_ptr()), vp(mu.data_ptr()), size, vp(bs.data_ptr()), *args) == 0
    torch.cuda.synchronize(dev)
    assert torch.equal(outs[0][1], outs[1][1])
    assert _rel(outs[0][1], bs) < 1e-6


def test_bf16_exact_transpose_deterministic():
    """bfloat16 mu (the non-mirror bfloat16 spread): the deterministic exact
    transpose repeats bit for bit and equals the vector-reduction form to 1e-6."""
    import ctypes

    vp = ctypes.c_void_p
    L = _lib.load()
    dev = torch.device("cuda", 0)
    sp = vp(torch.cuda.current_stream(dev).cuda_stream)
    shape = (48, 48, 48)
    nz, ny, nx = shape
    mu = torch.from_numpy(S.mu_map(shape, seed=4)).to(dev).to(torch.bfloat16)
    psf = S.gaussian_psf(5, nz, 0.5, 0.03)
    cams = np.ascontiguousarray(S.cameras_about_y(24, 1.0)[1])
    size = (ctypes.c_int * 3)(nx, ny, nz)
    csize = (ctypes.c_int * 2)(24, 1)
    psize = (ctypes.c_int * 3)(*psf.shape[::-1])
    y = torch.from_numpy(np.random.default_rng(3).uniform(0.5, 1.5, (24, ny, nx)).astype(np.float32)).to(dev)
    args = (cams.ctypes.data_as(vp), csize, psf.ctypes.data_as(vp), psize, 0.0, 0.0, 0, 1, sp)
    prev = L.nrgb_get_deterministic()
    outs = []
    try:
        for det in (0, 1, 1):
            L.nrgb_set_deterministic(det)
            b = torch.empty(shape, dtype=torch.float32, device=dev)
            assert L.nrgb_backproject_device_bf16(vp(y.data_ptr()), vp(mu.data_ptr()), size, vp(b.data_ptr()),
                                                  *args) == 0
            outs.append(b)
        torch.cuda.synchronize(dev)
    finally:
        L.nrgb_set_deterministic(prev)
    ref, d1, d2 = (o.double() for o in outs)
    assert torch.isfinite(d1).all()
    assert torch.equal(outs[1], outs[2])
    assert float((d1 - ref).norm() / ref.norm()) < 1e-6
