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
