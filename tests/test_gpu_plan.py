"""Plans (precomputed device state) against the stateless reference-compatible
C-ABI: projections, backprojections, camera subsets, the column layout, and
OSEM (eager and CUDA-graph-captured) against et_array_osem_step_subset."""
import numpy as np
import pytest

from conftest import rel_l2
from niftyrec_gb300 import array_api as A
from niftyrec_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL = 1e-5
SHAPE = (40, 40, 40)
NCAM = 24


@pytest.fixture(scope="module")
def data():
    act = S.ellipsoid_phantom(SHAPE, seed=31)
    mu = S.mu_map(SHAPE, seed=31)
    psf = S.gaussian_psf(7, SHAPE[2], 0.5, 0.05)
    cams = S.cameras_about_y(NCAM, 2.0)
    y = S.poisson_counts(A.project(act, cams, psf, mu), 80, seed=9)
    return act, mu, psf, cams, y


def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def make_plan(data, subsets=4, cams=None):
    from niftyrec_gb300.plan import Plan

    act, mu, psf, c3, y = data
    return Plan(SHAPE, c3 if cams is None else cams, psf, cuda(mu), subsets=subsets)


def test_plan_project_backproject_match_stateless(data):
    act, mu, psf, cams, y = data
    p = make_plan(data)
    assert p.fused
    order = p.subset_cameras(-1)  # all cameras, subset by subset
    assert sorted(order.tolist()) == list(range(NCAM))
    s = p.project(cuda(act)).cpu().numpy()
    sr = A.project(act, cams, psf, mu)
    assert rel_l2(s, sr[order]) < RTOL
    b = p.backproject(cuda(y[order])).cpu().numpy()
    br = A.backproject(y, cams, psf, mu)
    assert rel_l2(b, br) < RTOL
    for sub in range(p.n_subsets):
        idx = p.subset_cameras(sub)
        ss = p.project(cuda(act), subset=sub).cpu().numpy()
        assert rel_l2(ss, sr[idx]) < RTOL
        bs = p.backproject(cuda(y[idx]), subset=sub).cpu().numpy()
        assert rel_l2(bs, A.backproject(y[idx], cams[:, idx], psf, mu)) < RTOL


def test_plan_column_layout(data):
    act, mu, psf, cams, y = data
    p = make_plan(data, subsets=None)
    sc = p.project(p.to_column(cuda(act)), layout="column")
    s = p.from_column(sc).cpu().numpy()
    assert rel_l2(s, A.project(act, cams, psf, mu)) < RTOL
    bc = p.backproject(p.to_column(cuda(y)), layout="column")
    b = p.from_column(bc).cpu().numpy()
    assert rel_l2(b, A.backproject(y, cams, psf, mu)) < RTOL


@pytest.mark.parametrize("layout,graph", [("nifti", False), ("column", False), ("column", True)])
def test_plan_osem_matches_c_abi_steps(data, layout, graph):
    act, mu, psf, cams, y = data
    p = make_plan(data, subsets=4)
    x = p.osem(cuda(y), iterations=2, layout=layout, graph=graph).cpu().numpy()
    xr = np.ones(SHAPE, np.float32)
    for _ in range(2):
        for sub in range(4):
            xr = A.osem_step_subset(xr, y, cams, p.subset_cameras(sub), mu, psf)
    assert rel_l2(x, xr) < 2 * RTOL


def test_plan_general_orientation(data):
    act, mu, psf, _, y = data
    cams = np.random.default_rng(7).uniform(-1, 1, (3, 6)).astype(np.float32)
    p = make_plan(data, subsets=2, cams=cams)
    assert not p.fused
    order = p.subset_cameras(-1)
    s = p.project(cuda(act)).cpu().numpy()
    yy = A.project(act, cams, psf, mu)
    assert rel_l2(s, yy[order]) < RTOL
    b = p.backproject(cuda(yy[order])).cpu().numpy()
    assert rel_l2(b, A.backproject(yy, cams, psf, mu)) < RTOL


@pytest.mark.parametrize("world", [1, 2])
def test_sharded_osem_plan_operator(data, world):
    """Angle-sharded OSEM on the GPU operator.  world=1 is the plain step;
    world=2 runs both ranks' operators in this one process and sums their
    partial volumes by hand (the all_reduce of a real run), which must give
    the single-process step up to float32 summation order."""
    from niftyrec_gb300 import sharded as SH

    act, mu, psf, cams, y = data
    n_sub = 4
    sub = np.arange(NCAM) % n_sub
    ops, counts = [], []
    for r in range(world):
        ids, sids = SH.camera_shares(sub, r, world)
        ops.append(SH.PlanOperator(SHAPE, cams, ids, sids, n_sub, psf, cuda(mu)))
        counts.append(SH.split_counts(cuda(y), ids, sids, n_sub))
    sens = [sum(op.sensitivity(s) for op in ops) for s in range(n_sub)]
    x = torch.ones(SHAPE, dtype=torch.float32, device="cuda")
    for _ in range(2):
        for s in range(n_sub):
            num = sum(op.numerator(x, c[s], s, 1e-6) for op, c in zip(ops, counts))
            ops[0].update(x, num, sens[s], 1e-6)
    xr = np.ones(SHAPE, np.float32)
    for _ in range(2):
        for s in range(n_sub):
            xr = A.osem_step_subset(xr, y, cams, np.flatnonzero(sub == s), mu, psf)
    assert rel_l2(x.cpu().numpy(), xr) < 2 * RTOL
    if world == 1:
        rec = SH.ShardedOSEM(ops[0], counts[0], n_sub)
        x1 = rec.run(torch.ones(SHAPE, dtype=torch.float32, device="cuda"), 2)
        assert rec.collectives == 0
        assert rel_l2(x1.cpu().numpy(), xr) < 2 * RTOL


def test_plan_tall_volume_row_windows():
    """ny > 128: plans run the fused kernels in row windows (PSF halo 8 rows)."""
    from niftyrec_gb300.plan import Plan

    shape = (24, 260, 24)  # nz == nx: et_array_osem_step_subset's cubic-in-x volumes
    act = S.ellipsoid_phantom(shape, seed=61)
    mu = S.mu_map(shape, seed=61)
    psf = S.gaussian_psf(15, shape[2], 0.5, 0.05)
    cams = S.cameras_about_y(8, 2.0)
    y = S.poisson_counts(A.project(act, cams, psf, mu), 80, seed=10)
    p = Plan(shape, cams, psf, cuda(mu), subsets=2)
    assert p.fused
    order = p.subset_cameras(-1)
    s = p.project(cuda(act)).cpu().numpy()
    assert rel_l2(s, A.project(act, cams, psf, mu)[order]) < RTOL
    b = p.backproject(cuda(y[order])).cpu().numpy()
    assert rel_l2(b, A.backproject(y, cams, psf, mu, nz=shape[0])) < RTOL
    x = p.osem(cuda(y), iterations=1, layout="column", graph=True).cpu().numpy()
    xr = np.ones(shape, np.float32)
    for sub in range(2):
        xr = A.osem_step_subset(xr, y, cams, p.subset_cameras(sub), mu, psf)
    assert rel_l2(x, xr) < 2 * RTOL


@pytest.mark.parametrize("layout", ["nifti", "column"])
def test_plan_osmapem_matches_numpy_restatement(data, layout):
    """One-step-late MAP-EM with the quadratic MRF prior against a numpy
    restatement of et_osmapem_step (Python/NiftyRec/NiftyRec/NiftyRec.py:224-245,
    prior :400-404) on the oracle's projector and backprojector."""
    from scipy.signal import convolve

    from oracle.oracle import Restated

    act, mu, psf, cams, y = data
    p = make_plan(data, subsets=4)
    # small against sensitivity / gradient of counts-scaled activity, so that
    # max(sens - beta g, 0) + eps stays away from eps (where OSL diverges)
    beta = 1e-4
    x = p.osem(cuda(y), iterations=1, layout=layout, beta=beta).cpu().numpy()
    o = Restated("f32")
    kernel = -np.ones((3, 3, 3), np.float32)
    kernel[1, 1, 1] = 26
    xr = np.ones(SHAPE, np.float32)
    eps = np.float32(1e-6)
    for sub in range(4):
        idx = p.subset_cameras(sub)
        c = cams[:, idx]
        grad = convolve(xr, kernel, "same").astype(np.float32)
        norm = o.backproject(np.ones((len(idx),) + SHAPE[1:], np.float32), c, psf, mu, nz=SHAPE[0])
        norm = np.maximum(norm - np.float32(beta) * grad, 0) + eps
        pr = np.maximum(o.project(xr, c, psf, mu), 0) + eps
        upd = np.maximum(o.backproject(y[idx] / pr, c, psf, mu, nz=SHAPE[0]), 0)
        xr = (xr * upd / norm).astype(np.float32)
    assert np.isfinite(x).all() and x.max() < 1e4
    assert rel_l2(x, xr) < 2 * RTOL


def test_mrf_gradient_kernel():
    from scipy.signal import convolve

    from niftyrec_gb300 import _lib
    import ctypes

    L = _lib.load()
    x = np.random.default_rng(4).random((10, 12, 14)).astype(np.float32)
    g = torch.empty(x.shape, dtype=torch.float32, device="cuda")
    xt = cuda(x)
    st = L.nrgb_mrf_gradient_device(ctypes.c_void_p(xt.data_ptr()), ctypes.c_void_p(g.data_ptr()),
                                    (ctypes.c_int * 3)(14, 12, 10), None)
    assert st == 0
    kernel = -np.ones((3, 3, 3))
    kernel[1, 1, 1] = 26
    ref = convolve(x.astype(np.float64), kernel, "same")
    np.testing.assert_allclose(g.cpu().numpy(), ref, rtol=1e-5, atol=1e-5)


def test_plan_mirror_units_match_per_camera(data):
    """A plan whose subsets hold cameras at opposite angles (24 cameras at 15
    degrees, 4 interleaved subsets: camera k and k+12 share a subset) serves
    them as mirror units; a plan created with mirror pairs off computes every
    camera alone.  Both agree with each other and with the stateless call."""
    from niftyrec_gb300 import _lib

    act, mu, psf, cams, y = data
    L = _lib.load()
    p1 = make_plan(data)
    L.nrgb_set_mirror_pairs(0)
    try:
        p0 = make_plan(data)
    finally:
        L.nrgb_set_mirror_pairs(1)
    for sub in (-1, 0, 3):
        idx = p1.subset_cameras(sub)
        s1 = p1.project(cuda(act), subset=sub).cpu().numpy()
        s0 = p0.project(cuda(act), subset=sub).cpu().numpy()
        assert rel_l2(s1, s0) < RTOL
        b1 = p1.backproject(cuda(y[idx]), subset=sub).cpu().numpy()
        b0 = p0.backproject(cuda(y[idx]), subset=sub).cpu().numpy()
        assert rel_l2(b1, b0) < RTOL
        assert rel_l2(b1, A.backproject(y[idx], cams[:, idx], psf, mu)) < RTOL


def test_plan_osem_checkpoint_resume_bit_exact(tmp_path):
    """Plan.osem with a checkpoint: a run stopped after 1 of 3 iterations and
    resumed from its checkpoint to 3 iterations equals 3 uninterrupted
    iterations bit for bit; another problem's plan refuses the checkpoint."""
    import torch

    from niftyrec_gb300 import checkpoint as CK
    from niftyrec_gb300.plan import Plan

    shape = (32, 32, 32)
    act = S.ellipsoid_phantom(shape, seed=21)
    mu = torch.from_numpy(S.mu_map(shape, seed=21)).cuda()
    psf = S.gaussian_psf(5, 32, 0.5, 0.04)
    cams = S.cameras_about_y(12, 2.0)[1].copy()
    plan = Plan(shape, cams, psf, mu, subsets=3)
    y = torch.from_numpy(S.poisson_counts(plan.project(torch.from_numpy(act).cuda()).cpu().numpy(), 30, seed=3)).cuda()
    full = plan.osem(y, 3).cpu().numpy()
    ck = str(tmp_path / "p.npz")
    plan.osem(y, 1, checkpoint=ck)
    assert (CK.load(ck)["iteration"], CK.load(ck)["subset"]) == (1, 0)
    out = plan.osem(y, 3, checkpoint=ck, resume=True).cpu().numpy()
    np.testing.assert_array_equal(out, full)
    st = CK.load(ck)
    assert (st["iteration"], st["subset"]) == (3, 0)
    with pytest.raises(ValueError):
        Plan(shape, cams[:6].copy(), psf, mu, subsets=3).osem(y[:6], 3, checkpoint=ck, resume=True)


def test_truncated_backprojection_of_signed_data(data):
    """Backprojections of a sinogram with negative entries, truncated (the
    last gather of each row window stores max(value, 0)) and not, against the
    oracle: the plan in both layouts, the host-buffer call, and cameras about
    x (the gantry kernels on the caller's arrays)."""
    from oracle.oracle import Restated

    o = Restated("f32")
    act, mu, psf, cams, y = data
    ys = np.random.default_rng(12).uniform(-1.0, 1.0, y.shape).astype(np.float32)
    for trunc in (1, 0):
        bo = o.backproject(ys, cams, psf, mu, truncate=trunc, nz=SHAPE[0])
        if trunc:
            assert (bo == 0).any() and (bo > 0).any()
        b = A.backproject(ys, cams, psf, mu, truncate_negative_values=trunc)
        assert A.last_path() == 1
        assert rel_l2(b, bo) < RTOL
        p = make_plan(data, subsets=None)
        order = p.subset_cameras(-1)
        bn = p.backproject(cuda(ys[order]), truncate=bool(trunc)).cpu().numpy()
        assert rel_l2(bn, bo) < RTOL
        bc = p.from_column(p.backproject(p.to_column(cuda(ys)), layout="column", truncate=bool(trunc))).cpu().numpy()
        assert rel_l2(bc, bo) < RTOL
    cx = np.zeros((3, 10), np.float32)
    cx[0] = np.deg2rad(5.0 + 36.0 * np.arange(10))
    yx = np.random.default_rng(13).uniform(-1.0, 1.0, (10,) + SHAPE[1:]).astype(np.float32)
    bx = A.backproject(yx, cx, psf, mu, truncate_negative_values=1)
    assert A.last_path() == 1
    assert rel_l2(bx, o.backproject(yx, cx, psf, mu, truncate=1, nz=SHAPE[0])) < RTOL
