"""nrgb_project_backproject_device (projection and backprojection in one call)
against the two separate device calls, through the C-ABI.

The one-call form lays the volumes out once, takes the backprojector's
transmission carries from the projector (at the projector's depth slabs) and
feeds it the projection without another layout pass; only the float32
summation order of the carries differs from the separate calls, so results
agree to 1e-6 relative L2 (and both are within the 1e-5 of the oracle checked
elsewhere).  Cases: the headline size, unpaired cameras (odd count), no mu,
no PSF, an explicit backprojection input, the exact-transpose mode, row
windows (ny > 128), non-cubic grids and a general-orientation camera set
(which runs the two calls in sequence)."""
import ctypes

import numpy as np
import pytest

from niftyrec_gb300 import _lib
from niftyrec_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

vp = ctypes.c_void_p
TOL = 1e-6


def _rel(a, b):
    a, b = a.double(), b.double()
    return float((a - b).norm() / b.norm().clamp_min(1e-300))


def _call(L, fn, *args):
    st = fn(*args)
    assert st == 0, (fn.__name__, st)


@pytest.mark.parametrize("shape,ncam,k,att,inp,mode,general", [
    ((128, 128, 128), 120, 11, True, False, 0, False),
    ((64, 64, 64), 31, 7, True, False, 0, False),
    ((64, 64, 64), 30, 7, False, False, 0, False),
    ((48, 40, 56), 24, 0, True, True, 0, False),
    ((40, 40, 40), 20, 5, True, False, 1, False),
    ((20, 150, 24), 8, 9, True, True, 0, False),
    ((24, 24, 24), 6, 5, True, False, 0, True),
])
def test_pair_call_matches_separate_calls(shape, ncam, k, att, inp, mode, general):
    L = _lib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    sp = vp(stream.cuda_stream)
    nz, ny, nx = shape
    act = torch.from_numpy(S.ellipsoid_phantom(shape, seed=nz + ncam)).to(dev)
    mu = torch.from_numpy(S.mu_map(shape, seed=nz)).to(dev) if att else None
    psf = S.gaussian_psf(k, nz, 0.5, 0.03) if k else None
    if general:
        cams = np.random.default_rng(4).uniform(-1, 1, (3, ncam)).astype(np.float32)
        csize = (ctypes.c_int * 2)(ncam, 3)
    else:
        cams = np.ascontiguousarray(S.cameras_about_y(ncam, 1.0)[1])
        csize = (ctypes.c_int * 2)(ncam, 1)
    size = (ctypes.c_int * 3)(nx, ny, nz)
    psize = (ctypes.c_int * 3)(*(psf.shape[::-1] if psf is not None else (0, 0, 0)))
    pp = psf.ctypes.data_as(vp) if psf is not None else None
    mp = vp(mu.data_ptr()) if mu is not None else None
    cp = cams.ctypes.data_as(vp)
    y = None
    if inp:
        y = torch.from_numpy(np.random.default_rng(2).uniform(0.5, 1.5, (ncam, ny, nx)).astype(np.float32)).to(dev)

    s_ref = torch.empty((ncam, ny, nx), dtype=torch.float32, device=dev)
    b_ref = torch.empty(shape, dtype=torch.float32, device=dev)
    _call(L, L.nrgb_project_device, vp(act.data_ptr()), mp, size, vp(s_ref.data_ptr()), cp, csize, pp, psize, 0.0,
          0.0, 1, sp)
    src = y if y is not None else s_ref
    _call(L, L.nrgb_backproject_device, vp(src.data_ptr()), mp, size, vp(b_ref.data_ptr()), cp, csize, pp, psize,
          0.0, 0.0, 1, mode, sp)

    for _ in range(2):  # twice: the arena and carries are reused
        s = torch.full((ncam, ny, nx), float("nan"), dtype=torch.float32, device=dev)
        b = torch.full(shape, float("nan"), dtype=torch.float32, device=dev)
        _call(L, L.nrgb_project_backproject_device, vp(act.data_ptr()), mp, size, vp(s.data_ptr()),
              vp(y.data_ptr()) if y is not None else None, vp(b.data_ptr()), cp, csize, pp, psize, 0.0, 0.0, 1, mode,
              sp)
        assert L.nrgb_last_path() == (2 if general else 1)
        torch.cuda.synchronize(dev)
        assert torch.isfinite(s).all() and torch.isfinite(b).all()
        assert _rel(s, s_ref) < TOL
        assert _rel(b, b_ref) < TOL


def test_pair_call_rejects_bad_arguments():
    L = _lib.load()
    size = (ctypes.c_int * 3)(8, 8, 8)
    cams = np.zeros(4, np.float32)
    csize = (ctypes.c_int * 2)(4, 1)
    nopsf = (ctypes.c_int * 3)(0, 0, 0)
    buf = torch.zeros(8 * 8 * 8, dtype=torch.float32, device="cuda")
    p = vp(buf.data_ptr())
    assert L.nrgb_project_backproject_device(None, None, size, p, None, p, cams.ctypes.data_as(vp), csize, None, nopsf,
                                             0.0, 0.0, 1, 0, None) == 2
    assert L.nrgb_project_backproject_device(p, None, size, p, None, p, cams.ctypes.data_as(vp), csize, None, nopsf,
                                             0.0, 0.0, 1, 7, None) == 2


@pytest.mark.parametrize("shape,ncam", [((64, 64, 64), 60), ((48, 40, 48), 9)])
def test_pair_call_bf16_matches_separate_bf16_calls(shape, ncam):
    """nrgb_project_backproject_device_bf16 (bfloat16 activity and mu) against
    nrgb_project_device_bf16 + nrgb_backproject_device_bf16."""
    L = _lib.load()
    dev = torch.device("cuda", 0)
    sp = vp(torch.cuda.current_stream(dev).cuda_stream)
    nz, ny, nx = shape
    act = torch.from_numpy(S.ellipsoid_phantom(shape, seed=5)).to(dev).to(torch.bfloat16)
    mu = torch.from_numpy(S.mu_map(shape, seed=5)).to(dev).to(torch.bfloat16)
    psf = S.gaussian_psf(7, nz, 0.5, 0.03)
    cams = np.ascontiguousarray(S.cameras_about_y(ncam, 2.0)[1])
    size = (ctypes.c_int * 3)(nx, ny, nz)
    csize = (ctypes.c_int * 2)(ncam, 1)
    psize = (ctypes.c_int * 3)(*psf.shape[::-1])
    args = (cams.ctypes.data_as(vp), csize, psf.ctypes.data_as(vp), psize, 0.0, 0.0, 1)
    s_ref = torch.empty((ncam, ny, nx), dtype=torch.float32, device=dev)
    b_ref = torch.empty(shape, dtype=torch.float32, device=dev)
    _call(L, L.nrgb_project_device_bf16, vp(act.data_ptr()), vp(mu.data_ptr()), size, vp(s_ref.data_ptr()), *args, sp)
    _call(L, L.nrgb_backproject_device_bf16, vp(s_ref.data_ptr()), vp(mu.data_ptr()), size, vp(b_ref.data_ptr()),
          *args, 0, sp)
    s = torch.empty_like(s_ref)
    b = torch.empty_like(b_ref)
    _call(L, L.nrgb_project_backproject_device_bf16, vp(act.data_ptr()), vp(mu.data_ptr()), size, vp(s.data_ptr()),
          None, vp(b.data_ptr()), *args, 0, sp)
    torch.cuda.synchronize(dev)
    assert _rel(s, s_ref) < TOL
    assert _rel(b, b_ref) < TOL


@pytest.mark.parametrize("group", [3, 5, 7])
def test_many_camera_groups_reuse_scratch_slots(group):
    """Small camera groups (group 0, 2, 4, ... spread on the caller's stream,
    1, 3, 5, ... on the second spread stream, each slot spread again only after
    its gather): reference and exact-transpose backprojections, separate and
    one-call, against the default grouping (only the float32 order of the group
    sums differs) at 48^3 x 40 cameras with PSF and mu."""
    L = _lib.load()
    dev = torch.device("cuda", 0)
    sp = vp(torch.cuda.current_stream(dev).cuda_stream)
    shape = (48, 48, 48)
    nz, ny, nx = shape
    ncam = 40
    act = torch.from_numpy(S.ellipsoid_phantom(shape, seed=21)).to(dev)
    mu = torch.from_numpy(S.mu_map(shape, seed=21)).to(dev)
    psf = S.gaussian_psf(5, nz, 0.5, 0.03)
    cams = np.ascontiguousarray(S.cameras_about_y(ncam, 1.0)[1])
    size = (ctypes.c_int * 3)(nx, ny, nz)
    csize = (ctypes.c_int * 2)(ncam, 1)
    psize = (ctypes.c_int * 3)(*psf.shape[::-1])
    args = (cams.ctypes.data_as(vp), csize, psf.ctypes.data_as(vp), psize, 0.0, 0.0, 1)
    y = torch.from_numpy(np.random.default_rng(5).uniform(0.5, 1.5, (ncam, ny, nx)).astype(np.float32)).to(dev)

    def run():
        out = {}
        for mode in (0, 1):
            b = torch.empty(shape, dtype=torch.float32, device=dev)
            _call(L, L.nrgb_backproject_device, vp(y.data_ptr()), vp(mu.data_ptr()), size, vp(b.data_ptr()), *args,
                  mode, sp)
            s = torch.empty((ncam, ny, nx), dtype=torch.float32, device=dev)
            bp = torch.empty(shape, dtype=torch.float32, device=dev)
            _call(L, L.nrgb_project_backproject_device, vp(act.data_ptr()), vp(mu.data_ptr()), size, vp(s.data_ptr()),
                  None, vp(bp.data_ptr()), *args, mode, sp)
            out[mode] = (b, bp)
        torch.cuda.synchronize(dev)
        return out

    ref = run()
    try:
        assert L.nrgb_set_backproject_group(nx, ny, nz, ncam, group) == 0
        got = run()
    finally:
        L.nrgb_set_backproject_group(nx, ny, nz, ncam, 0)
    for mode in (0, 1):
        for r, g in zip(ref[mode], got[mode]):
            assert torch.isfinite(g).all()
            assert _rel(g, r) < TOL
