"""nrgb_backproject_device_noalloc -- the backprojection for callers that
cannot allocate device memory (a plug-in whose host application's allocator
already holds the GPU's memory, a real-time loop that must not enter the
driver's allocator) -- called through the C-ABI and checked against the
allocating entry point nrgb_backproject_device on two calls in a row, with the
same relative-L2 tolerance as the other parity tests.  Collected last on
purpose; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from niftyrec_gb300 import _lib
from niftyrec_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

RTOL = 1e-5
vp = ctypes.c_void_p


def _rel(a, b):
    a = a.double()
    b = b.double()
    return float((a - b).norm() / b.norm().clamp_min(1e-300))


def _run(fn, sino, mu, out, n, cams, ncols, psf, stream, extra_mode):
    size = (ctypes.c_int * 3)(n[0], n[1], n[2])
    ncam = cams.shape[-1] if cams.ndim > 1 else cams.shape[0]
    csize = (ctypes.c_int * 2)(ncam, ncols)
    psize = (ctypes.c_int * 3)(*(psf.shape[::-1] if psf is not None else (0, 0, 0)))
    args = [vp(sino.data_ptr()), vp(mu.data_ptr()) if mu is not None else None, size, vp(out.data_ptr()),
            cams.ctypes.data_as(vp), csize, psf.ctypes.data_as(vp) if psf is not None else None, psize, 0.0, 0.0, 1]
    if extra_mode:
        args.append(0)
    args.append(vp(stream.cuda_stream))
    return fn(*args)


@pytest.mark.parametrize("case", ["gantry_psf_att", "general_cameras"])
def test_noalloc_matches_allocating_entry_point_twice(case):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    if case == "gantry_psf_att":
        n = (64, 64, 64)  # (nx, ny, nz)
        cams = np.ascontiguousarray(S.cameras_about_y(60, 1.0)[1])
        ncols = 1
        psf = S.gaussian_psf(7, 64, 0.5, 0.04)
    else:
        n = (24, 24, 24)
        cams = np.ascontiguousarray(np.random.default_rng(5).uniform(-1, 1, (3, 6)).astype(np.float32))
        ncols = 3
        psf = S.gaussian_psf(5, 24)
    shape = (n[2], n[1], n[0])
    mu = torch.from_numpy(S.mu_map(shape, seed=3)).to(dev)
    ncam = cams.shape[-1]
    for call in range(2):  # two calls in a row, different data each time
        act = S.ellipsoid_phantom(shape, seed=10 + call)
        sino_np = np.stack([act.sum(axis=0)] * ncam) * (1.0 + 0.01 * np.arange(ncam))[:, None, None]
        sino = torch.from_numpy(np.ascontiguousarray(sino_np, dtype=np.float32)).to(dev)
        ref = torch.zeros(shape, dtype=torch.float32, device=dev)
        out = torch.full(shape, float("nan"), dtype=torch.float32, device=dev)
        st = _run(L.nrgb_backproject_device, sino, mu, ref, n, cams, ncols, psf, stream, True)
        assert st == 0, st
        st = _run(L.nrgb_backproject_device_noalloc, sino, mu, out, n, cams, ncols, psf, stream, False)
        assert st == 0, st
        assert L.nrgb_last_path() == (1 if case == "gantry_psf_att" else 2)
        torch.cuda.synchronize(dev)
        assert torch.isfinite(out).all()
        assert _rel(out, ref) < RTOL


def test_noalloc_rejects_psf_without_size():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda", 0)
    n = (16, 16, 16)
    cams = np.ascontiguousarray(S.cameras_about_y(4)[1])
    psf = S.gaussian_psf(3, 16)
    sino = torch.zeros((4, 16, 16), dtype=torch.float32, device=dev)
    out = torch.zeros((16, 16, 16), dtype=torch.float32, device=dev)
    st = L.nrgb_backproject_device_noalloc(vp(sino.data_ptr()), None, (ctypes.c_int * 3)(*n), vp(out.data_ptr()),
                                           cams.ctypes.data_as(vp), (ctypes.c_int * 2)(4, 1),
                                           psf.ctypes.data_as(vp), None, 0.0, 0.0, 1,
                                           vp(torch.cuda.current_stream(dev).cuda_stream))
    assert st == 2


def test_noalloc_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda", 0)
    n = (128, 128, 128)
    cams = np.ascontiguousarray(S.cameras_about_y(120)[1])
    sino = torch.zeros((120, 128, 128), dtype=torch.float32, device=dev)
    mu = torch.zeros((128, 128, 128), dtype=torch.float32, device=dev)
    out = torch.zeros((128, 128, 128), dtype=torch.float32, device=dev)
    st = _run(L.nrgb_backproject_device_noalloc, sino, mu, out, n, cams, 1, None,
              torch.cuda.current_stream(dev), False)
    assert st == 10
    assert b"64 MiB" in L.niftyrec_error_msg(10)
