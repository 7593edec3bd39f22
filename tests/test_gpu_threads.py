"""Calls from several host threads: the host-buffer entry points (serialised
per device) and plans working on their own CUDA streams concurrently give
the results of the same calls made one after another."""
import threading

import numpy as np
import pytest

from niftyrec_gb300 import array_api as A
from niftyrec_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def inputs(shape, seed, ncam):
    act = S.ellipsoid_phantom(shape, seed=seed)
    mu = S.mu_map(shape, seed=seed)
    psf = S.gaussian_psf(7, shape[2], 0.5, 0.05)
    cams = S.cameras_about_y(ncam, 1.0 + seed)
    return act, mu, psf, cams


def run_threads(fns):
    errors = []

    def wrap(f):
        try:
            f()
        except Exception as e:  # reported by the main thread
            errors.append(e)

    ts = [threading.Thread(target=wrap, args=(f,)) for f in fns]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not errors, errors


def test_host_buffer_calls_from_two_threads():
    cases = [inputs((40, 36, 40), 1, 12), inputs((32, 28, 36), 2, 10)]
    want = []
    for act, mu, psf, cams in cases:
        s = A.project(act, cams, psf, mu)
        want.append((s, A.backproject(s, cams, psf, mu, nz=act.shape[0])))
    got = [[], []]

    def worker(i):
        act, mu, psf, cams = cases[i]
        for _ in range(4):
            s = A.project(act, cams, psf, mu)
            got[i].append((s, A.backproject(s, cams, psf, mu, nz=act.shape[0])))

    run_threads([lambda: worker(0), lambda: worker(1)])
    for i in range(2):
        for s, b in got[i]:
            np.testing.assert_array_equal(s, want[i][0])
            np.testing.assert_array_equal(b, want[i][1])


def test_plans_on_their_own_streams():
    from niftyrec_gb300.plan import Plan

    cases = [inputs((48, 40, 48), 3, 24), inputs((40, 32, 40), 4, 16)]
    plans = [Plan(c[0].shape, c[3], c[2], torch.from_numpy(c[1]).cuda(), subsets=2) for c in cases]
    acts = [torch.from_numpy(c[0]).cuda() for c in cases]
    want = []
    for p, x in zip(plans, acts):
        s = p.project(x)
        want.append((s.cpu().numpy(), p.backproject(s).cpu().numpy()))
    torch.cuda.synchronize()
    got = [[], []]

    def worker(i):
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            for _ in range(6):
                s = plans[i].project(acts[i])
                b = plans[i].backproject(s)
                got[i].append((s, b))
        stream.synchronize()

    run_threads([lambda: worker(0), lambda: worker(1)])
    torch.cuda.synchronize()
    for i in range(2):
        for s, b in got[i]:
            np.testing.assert_array_equal(s.cpu().numpy(), want[i][0])
            np.testing.assert_array_equal(b.cpu().numpy(), want[i][1])


def test_injected_allocation_failure_is_a_status_not_a_fault():
    """Host-side fault injection: with the arena released, an injected
    allocation failure makes the next call return status 4 (allocgpu); the
    call after it succeeds and matches the result before the failure."""
    from niftyrec_gb300 import _lib
    from niftyrec_gb300 import array_api as A
    from niftyrec_gb300 import synthetic as S

    L = _lib.load()
    shape = (24, 24, 24)
    act = S.ellipsoid_phantom(shape, seed=2)
    cams = S.cameras_about_y(6)
    ref = A.project(act, cams)
    assert L.et_array_reset_gpu() == 0
    L.nrgb_debug_fail_allocations(1)
    from niftyrec_gb300._lib import NiftyRecError

    with pytest.raises(NiftyRecError) as e:
        A.project(act, cams)
    assert e.value.status == 4
    np.testing.assert_array_equal(A.project(act, cams), ref)
    L.nrgb_debug_fail_allocations(0)
