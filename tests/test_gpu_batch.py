"""Batched OSEM (niftyrec_gb300.batch): volumes of uneven shape, camera and
subset counts, PSF widths and with / without mu in one batch must reconstruct
exactly what each plan's own OSEM gives (the batched kernels run the same
per-item arithmetic), eagerly and replayed from one CUDA graph."""
import numpy as np
import pytest

from conftest import rel_l2
from niftyrec_gb300 import array_api as A
from niftyrec_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

# (shape (nz, ny, nx), cameras, subsets, PSF width or 0, with mu)
VOLUMES = [((24, 24, 24), 12, 3, 5, True), ((20, 28, 32), 10, 2, 5, True), ((16, 140, 16), 8, 4, 5, True),
           ((24, 20, 24), 9, 3, 7, True), ((18, 18, 18), 6, 2, 5, False), ((12, 16, 20), 5, 1, 0, True)]


def make(i, shape, ncam, nsub, k, att):
    from niftyrec_gb300.plan import Plan

    act = S.ellipsoid_phantom(shape, seed=70 + i)
    mu = S.mu_map(shape, seed=70 + i) if att else None
    psf = S.gaussian_psf(k, shape[2], 0.5, 0.04) if k else None
    cams = S.cameras_about_y(ncam, 3.0)
    y = S.poisson_counts(A.project(act, cams, psf, mu), 60, seed=i)
    mu_t = torch.from_numpy(mu).cuda() if att else None
    return Plan(shape, cams, psf, mu_t, subsets=nsub), torch.from_numpy(y).cuda()


@pytest.fixture(scope="module")
def setup():
    plans, counts = zip(*[make(i, *v) for i, v in enumerate(VOLUMES)])
    return list(plans), list(counts)


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_each_plan(setup, graph):
    from niftyrec_gb300.batch import Batch

    plans, counts = setup
    ref = [p.osem(c, iterations=2, layout="column").cpu().numpy() for p, c in zip(plans, counts)]
    b = Batch(plans)
    out = b.osem(counts, iterations=2, graph=graph)
    for i, (x, r) in enumerate(zip(out, ref)):
        assert rel_l2(x.cpu().numpy(), r) < 1e-6, i


def test_batch_step_skips_finished_volumes(setup):
    """With iterations=1 a volume of 2 subsets stops after step 1 while one of
    4 subsets continues: its activity must not change at steps 2 and 3."""
    from niftyrec_gb300.batch import Batch

    plans, counts = setup
    b = Batch(plans)
    for v, c in enumerate(counts):
        b.set_counts(v, c)
        b.set_activity(v, torch.ones(plans[v].shape, dtype=torch.float32, device="cuda"))
    b.step(0, 1)
    b.step(1, 1)
    x2 = b.get_activity(1).clone()  # 2 subsets: done after step 1
    x4 = b.get_activity(2).clone()  # 4 subsets
    b.step(2, 1)
    b.step(3, 1)
    assert torch.equal(b.get_activity(1), x2)
    assert not torch.equal(b.get_activity(2), x4)
