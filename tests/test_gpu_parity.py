"""Parity of the CUDA path, called through the C-ABI, with the reference's own
outputs (golden fixtures from the compiled reference CPU path) and with the
oracle's C restatement on fresh seeded inputs.

Tolerance: relative L2 error <= 1e-5 per projection plane and per
backprojected volume (float32 arithmetic in a different order and CUDA's
__expf against the reference's expf)."""
import numpy as np
import pytest

from conftest import rel_l2
from niftyrec_gb300 import array_api as A
from niftyrec_gb300 import synthetic as S
from oracle.oracle import Restated

pytestmark = pytest.mark.gpu

RTOL = 1e-5
FUSED, GENERAL = 1, 2


def per_plane_rel(a, b):
    return max(rel_l2(a[i], b[i]) for i in range(b.shape[0]))


@pytest.fixture(scope="module")
def o32():
    return Restated("f32")


def test_golden_ygantry_psf_att(golden):
    g = golden("ygantry_psf_att_24")
    s = A.project(g["act"], g["cameras"], g["psf"], g["mu"])
    assert A.last_path() == FUSED
    assert per_plane_rel(s, g["sino"]) < RTOL
    b = A.backproject(g["counts"], g["cameras"], g["psf"], g["mu"])
    assert A.last_path() == FUSED
    assert rel_l2(b, g["bkpr"]) < RTOL


def test_golden_plain(golden):
    g = golden("ygantry_plain_20")
    for cams in (g["cameras"], g["cameras3"]):
        s = A.project(g["act"], cams)
        assert A.last_path() == FUSED
        assert per_plane_rel(s, g["sino"]) < RTOL
        b = A.backproject(g["sino"], cams)
        assert rel_l2(b, g["bkpr"]) < RTOL


def test_golden_noncubic(golden):
    g = golden("noncubic_24x20x16")
    s = A.project(g["act"], g["cameras"], g["psf"], g["mu"])
    assert A.last_path() == FUSED
    assert per_plane_rel(s, g["sino"]) < RTOL
    b = A.backproject(g["sino"], g["cameras"], g["psf"], g["mu"], nz=16)
    assert A.last_path() == FUSED
    assert rel_l2(b, g["bkpr"]) < RTOL


def test_golden_general_cameras(golden):
    g = golden("general_cams_18")
    bg, bga = float(g["bg"]), float(g["bg_att"])
    s = A.project(g["act"], g["cameras6"], None, g["mu"], bg, bga)
    assert A.last_path() == GENERAL
    assert per_plane_rel(s, g["sino_bg"]) < RTOL
    b = A.backproject(g["sino_bg"], g["cameras6"], None, g["mu"], bg, bga)
    assert rel_l2(b, g["bkpr_bg"]) < RTOL
    s = A.project(g["act"], g["cameras3"], None, g["mu"])
    assert A.last_path() == GENERAL
    assert per_plane_rel(s, g["sino"]) < RTOL
    b = A.backproject(g["sino"], g["cameras3"], None, g["mu"])
    assert rel_l2(b, g["bkpr"]) < RTOL


def test_golden_mlem_steps(golden):
    g = golden("mlem_16")
    x1 = A.mlem_step(np.ones_like(g["mu"]), g["counts"], g["cameras3"], g["mu"], g["psf"])
    assert A.last_path() == FUSED
    assert rel_l2(x1, g["x1"]) < RTOL
    x2 = A.mlem_step(x1, g["counts"], g["cameras3"], g["mu"], g["psf"])
    assert rel_l2(x2, g["x2"]) < 2 * RTOL


def test_golden_rotate(golden):
    g = golden("rotate_16x14x12")
    r = A.rotate(g["vol"], [0.3, -0.7, 0.2], [7.5, 6.5, 5.5], 0.0, 0)
    assert rel_l2(r, g["rot_xyz"]) < 1e-6
    r = A.rotate(g["vol"], [-0.3, 0.7, -0.2], [7.5, 6.5, 5.5], 0.0, 5)
    assert rel_l2(r, g["rot_zyx"]) < 1e-6


@pytest.mark.parametrize("shape", [(12, 14, 16), (33, 20, 27)])
def test_affine_matches_oracle_resampler(o32, shape):
    """et_array_affine applies its 4 x 4 matrix (column-major in the interface)
    with the reference's trilinear resampler: equal to the oracle's
    restatement of reg_affine_positionField + reg_resampleSourceImage
    (reg-lib/_reg_resampling.cpp:305-450) to 1e-6 (the rotation test's bound);
    the identity returns the input exactly; a rotation matrix gives
    et_array_rotate's result."""
    rng = np.random.default_rng(sum(shape))
    vol = rng.random(shape).astype(np.float32)
    M = np.array([[0.9, 0.2, -0.1, 1.5], [-0.15, 1.05, 0.05, -0.7], [0.1, -0.05, 0.95, 0.4], [0, 0, 0, 1]],
                 np.float32)
    out = A.affine(vol, M, background=0.25)
    ref = o32.affine_resample(vol, M, bg=0.25)
    assert (out == 0.25).any() and rel_l2(out, ref) < 1e-6
    assert np.array_equal(A.affine(vol, np.eye(4, dtype=np.float32)), vol)
    R = o32.rotation_matrix([0.3, -0.2, 0.5], [5.5, 6.5, 4.5], 0)
    assert rel_l2(A.affine(vol, R), A.rotate(vol, [0.3, -0.2, 0.5], [5.5, 6.5, 4.5], 0.0, 0)) < 1e-6


def test_affine_rejects_bad_matrix_size():
    import ctypes

    from niftyrec_gb300 import _lib

    L = _lib.load()
    vol = np.zeros((4, 4, 4), np.float32)
    out = np.zeros_like(vol)
    a = np.eye(4, dtype=np.float32)
    p = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    size = (ctypes.c_int * 3)(4, 4, 4)
    assert L.et_array_affine(p(vol), size, p(out), size, p(a), (ctypes.c_int * 2)(3, 4), 0.0, 1) == 2
    assert L.et_array_affine(p(vol), size, p(out), size, p(a), None, 0.0, 1) == 2


@pytest.mark.parametrize("shape,k", [((6, 20, 20), (7, 5)), ((3, 17, 29), (3, 9)), ((1, 32, 24), (11, 11))])
def test_convolve_matches_oracle(o32, shape, k):
    """et_array_convolve (per-slice 2D convolution, image clamped at its
    border) against the oracle's direct restatement, bit for bit (same term
    order, separate rounding); a centred delta kernel returns the image."""
    rng = np.random.default_rng(sum(shape))
    vol = rng.random(shape).astype(np.float32)
    ker = rng.random((shape[0],) + k).astype(np.float32)
    out = A.convolve(vol, ker)
    assert np.array_equal(out, o32.convolve2d(vol, ker))
    delta = np.zeros_like(ker)
    delta[:, (k[0] - 1) // 2, (k[1] - 1) // 2] = 1.0
    assert np.array_equal(A.convolve(vol, delta), vol)


def test_convolve_rejects_even_kernel():
    with pytest.raises(Exception):
        A.convolve(np.zeros((2, 8, 8), np.float32), np.zeros((2, 4, 3), np.float32))


# (nz, ny, nx): the PSF has nx planes (the reference's rule) and plane z serves
# depth z, so nz <= nx.
@pytest.mark.parametrize("shape,k,ncam", [((64, 64, 64), 11, 12), ((36, 52, 40), 7, 9), ((30, 18, 32), 15, 5),
                                          ((48, 128, 48), 3, 4), ((30, 30, 30), 1, 3)])
def test_oracle_fresh_inputs(o32, shape, k, ncam):
    act = S.ellipsoid_phantom(shape, seed=sum(shape))
    mu = S.mu_map(shape, seed=sum(shape))
    psf = S.gaussian_psf(k, shape[2], 0.5, 0.05)
    cams = S.cameras_about_y(ncam, 1.5)
    s = A.project(act, cams, psf, mu)
    assert A.last_path() == FUSED
    so = o32.project(act, cams, psf, mu)
    assert per_plane_rel(s, so) < RTOL
    b = A.backproject(so, cams, psf, mu, nz=shape[0])
    assert A.last_path() == FUSED
    bo = o32.backproject(so, cams, psf, mu, nz=shape[0])
    assert rel_l2(b, bo) < RTOL


@pytest.mark.parametrize("shape,k", [((20, 132, 20), 5), ((16, 300, 16), 15), ((12, 257, 14), 0),
                                     ((10, 250, 12), 1)])
def test_row_windows_large_ny(o32, shape, k):
    """ny > 128 runs on the fused kernels in row windows with a PSF halo;
    window seams must not show (checked per row against the oracle)."""
    act = S.ellipsoid_phantom(shape, seed=4)
    mu = S.mu_map(shape, seed=4)
    psf = S.gaussian_psf(k, shape[2]) if k else None
    cams = S.cameras_about_y(3, 10.0)
    s = A.project(act, cams, psf, mu)
    assert A.last_path() == FUSED
    so = o32.project(act, cams, psf, mu)
    assert per_plane_rel(s, so) < RTOL
    # every gantry-axis row, so a seam between windows cannot hide in the norm
    rows = np.linalg.norm(s - so, axis=(0, 2)) / np.maximum(np.linalg.norm(so, axis=(0, 2)), 1e-12)
    assert rows.max() < 1e-4, int(rows.argmax())
    b = A.backproject(so, cams, psf, mu, nz=shape[0])
    assert A.last_path() == FUSED
    assert rel_l2(b, o32.backproject(so, cams, psf, mu, nz=shape[0])) < RTOL
    torch = pytest.importorskip("torch")
    from niftyrec_gb300.autograd import backproject_raw

    bt = backproject_raw(torch.from_numpy(so).cuda(), torch.from_numpy(mu).cuda(), cams, psf, nz=shape[0], mode=1)
    bto = o32.backproject(so, cams, psf, mu, truncate=0, adjoint=True, nz=shape[0])
    assert rel_l2(bt.cpu().numpy(), bto) < RTOL


def test_general_path_with_background(o32):
    """A non-zero background leaves the fused kernels for the general path."""
    shape = (20, 132, 20)
    act = S.ellipsoid_phantom(shape, seed=4)
    mu = S.mu_map(shape, seed=4)
    psf = S.gaussian_psf(5, 20)
    cams = S.cameras_about_y(3, 10.0)
    s = A.project(act, cams, psf, mu, 0.5, 0.0)
    assert A.last_path() == GENERAL
    assert per_plane_rel(s, o32.project(act, cams, psf, mu, 0.5, 0.0)) < RTOL


def test_gradient_attenuation_matches_restated_reference(o32):
    shape = (24, 24, 24)
    act = S.ellipsoid_phantom(shape, seed=21)
    mu = S.mu_map(shape, seed=21)
    psf = S.gaussian_psf(5, 24)
    cams = S.cameras_about_y(6, 2.0)
    y = S.poisson_counts(o32.project(act, cams, psf, mu), 50)
    g = A.gradient_attenuation(y, act, mu, cams, psf)
    assert A.last_path() == FUSED
    go = o32.gradient_attenuation(y, act, mu, cams, psf)
    assert rel_l2(g, go) < RTOL


@pytest.mark.parametrize("shape,k,ncam,truncate", [
    ((20, 150, 20), 7, 5, 0),    # row windows (ny > 128)
    ((28, 36, 44), 15, 7, 1),    # radius 7, truncation of negative values
    ((16, 20, 24), 0, 4, 0),     # no PSF
    ((260, 8, 264), 15, 2, 0),   # PSF too large for the kernel-parameter table
])
def test_fused_gradient_attenuation(o32, shape, k, ncam, truncate):
    """The reference attenuation gradient on the gantry kernels (sampled
    activity and mu, suffix sums across depth slabs, PSF, inverse-rotation
    gather) against the oracle, with signed sinogram weights."""
    act = S.ellipsoid_phantom(shape, seed=71)
    mu = S.mu_map(shape, seed=71)
    psf = S.gaussian_psf(k, shape[2]) if k else None
    cams = S.cameras_about_y(ncam, 7.0)
    y = np.random.default_rng(71).uniform(-0.5, 1.5, (ncam, shape[1], shape[2])).astype(np.float32)
    g = A.gradient_attenuation(y, act, mu, cams, psf, truncate_negative_values=truncate)
    assert A.last_path() == FUSED
    go = o32.gradient_attenuation(y, act, mu, cams, psf, truncate=truncate)
    assert rel_l2(g, go) < RTOL


def test_fused_gradient_attenuation_x_gantry(o32):
    """Cameras rotating about x: the gradient runs on the gantry kernels with
    x and y exchanged."""
    shape = (20, 28, 24)
    act = S.ellipsoid_phantom(shape, seed=72)
    mu = S.mu_map(shape, seed=72)
    psf = S.gaussian_psf(5, shape[2], 0.5, 0.05)
    cams = np.zeros((3, 6), np.float32)
    cams[0] = np.deg2rad(3.0 + 60.0 * np.arange(6)).astype(np.float32)
    y = np.random.default_rng(72).uniform(0.0, 2.0, (6, shape[1], shape[2])).astype(np.float32)
    g = A.gradient_attenuation(y, act, mu, cams, psf)
    assert A.last_path() == FUSED
    assert rel_l2(g, o32.gradient_attenuation(y, act, mu, cams, psf)) < RTOL


def close(a, b, tol=RTOL):
    """Relative L2 error below tol, or both (near) zero."""
    nb = float(np.linalg.norm(np.asarray(b, np.float64)))
    if nb == 0.0:
        return float(np.abs(a).max(initial=0.0)) <= 1e-12
    return rel_l2(a, b) < tol


@pytest.mark.parametrize("shape,k,ncam", [((1, 1, 1), 0, 1), ((2, 3, 5), 3, 2), ((3, 12, 16), 3, 4),
                                          ((1, 7, 9), 5, 3), ((5, 1, 6), 0, 2), ((3, 5, 4), 5, 5)])
def test_tiny_and_ragged_volumes(o32, shape, k, ncam):
    """One-voxel, one-plane and one-row volumes, PSFs wider than the volume,
    odd sizes, more depth slabs than planes and an opposite-angle pair:
    projection, both backprojectors and the attenuation gradient against the
    oracle."""
    torch = pytest.importorskip("torch")
    from niftyrec_gb300.autograd import backproject_raw

    rng = np.random.default_rng(sum(shape) + k)
    act = rng.uniform(0.5, 2.0, shape).astype(np.float32)
    mu = rng.uniform(0.0, 0.1, shape).astype(np.float32)
    psf = S.gaussian_psf(k, shape[2]) if k else None
    cams = S.cameras_about_y(ncam, 7.0)
    nz = shape[0]
    s = A.project(act, cams, psf, mu)
    assert A.last_path() == FUSED
    so = o32.project(act, cams, psf, mu)
    assert close(s, so)
    b = A.backproject(so, cams, psf, mu, nz=nz)
    assert A.last_path() == FUSED
    assert close(b, o32.backproject(so, cams, psf, mu, nz=nz))
    bt = backproject_raw(torch.from_numpy(so).cuda(), torch.from_numpy(mu).cuda(), cams, psf, nz=nz, mode=1)
    assert close(bt.cpu().numpy(), o32.backproject(so, cams, psf, mu, truncate=0, adjoint=True, nz=nz))
    y = rng.uniform(-0.5, 1.5, so.shape).astype(np.float32)
    g = A.gradient_attenuation(y, act, mu, cams, psf)
    assert A.last_path() == FUSED
    assert close(g, o32.gradient_attenuation(y, act, mu, cams, psf))


def test_known_answer_angle0_is_depth_sum():
    vol = S.ellipsoid_phantom((32, 32, 32), seed=8)
    s = A.project(vol, np.zeros(1, np.float32))
    np.testing.assert_allclose(s[0], vol.sum(axis=0), rtol=1e-5, atol=1e-5)


def test_parameter_errors():
    act = np.ones((8, 8, 8), np.float32)
    cams = np.zeros(2, np.float32)
    with pytest.raises(Exception) as e:
        A.project(act, cams, np.ones((8, 4, 4), np.float32))  # even PSF
    assert getattr(e.value, "status", None) == 2
    with pytest.raises(Exception) as e:
        A.project(act, cams, np.ones((8, 3, 5), np.float32))  # non-square PSF
    assert getattr(e.value, "status", None) == 2
    with pytest.raises(Exception) as e:
        A.backproject(np.ones((3, 8, 8), np.float32), cams)  # n_cameras mismatch
    assert getattr(e.value, "status", None) == 2


@pytest.mark.parametrize("rotate,att,bgi", [(0, True, False), (1, True, True), (0, False, True), (1, False, False)])
def test_partial_sum_projector(o32, rotate, att, bgi):
    """et_array_project_partial against the oracle's restatement of
    et_project_partial_gpu: projections and partial-sum volumes."""
    shape = (20, 18, 24)
    act = S.ellipsoid_phantom(shape, seed=91)
    mu = S.mu_map(shape, seed=91) if att else None
    psf = S.gaussian_psf(5, shape[2], 0.5, 0.05)
    cams = S.cameras_about_y(5, 17.0)
    img = np.random.default_rng(2).uniform(0.5, 1.5, shape[1:]).astype(np.float32) if bgi else None
    s, part = A.project_partial(act, cams, psf, mu, 0.2, img, 0.0, 1, rotate)
    so, po = o32.project_partial(act, cams, psf, mu, bg=0.2, bg_image=img, truncate=1, rotate=rotate)
    assert per_plane_rel(s, so) < RTOL
    assert rel_l2(part, po) < RTOL


def test_fisher_grid_golden(golden, o32):
    """et_array_fisher_grid on the GPU against the compiled reference's
    (golden fixture) and, from the reference's own projection, exactly the
    reference's accumulation (et_array_fisher_grid_projection)."""
    g = golden("fisher_16")
    f, pr = A.fisher_grid(g["act"], g["cameras"], g["psf"], g["grid"], 24, g["mu"])
    assert rel_l2(f, g["fisher"]) < RTOL
    np.testing.assert_array_equal(pr, g["prior"])
    # from the oracle's projection (bit-exact to the reference's) the
    # accumulation is the reference's own order: bit-exact
    so = o32.project(g["act"], g["cameras"], g["psf"], g["mu"])
    f2, _ = A.fisher_grid_projection(so, g["cameras"], g["psf"], g["grid"], 24)
    np.testing.assert_array_equal(f2, g["fisher"])
    bad = g["grid"].copy()
    bad.flat[np.flatnonzero(bad)[:2]] = 1.0  # repeated index
    with pytest.raises(Exception) as e:
        A.fisher_grid(g["act"], g["cameras"], g["psf"], bad, 24, g["mu"])
    assert getattr(e.value, "status", None) == 2


@pytest.mark.parametrize("slabs", [2, 4, 8, 16])
def test_project_slab_counts(o32, slabs):
    """Every depth-slab count of the projector (cluster size, from the tuning
    table) gives the oracle's projection; the entry is removed afterwards."""
    from niftyrec_gb300 import _lib

    L = _lib.load()
    shape = (40, 36, 44)
    act = S.ellipsoid_phantom(shape, seed=33)
    mu = S.mu_map(shape, seed=33)
    psf = S.gaussian_psf(9, shape[2], 0.5, 0.05)
    cams = S.cameras_about_y(7, 3.0)
    key = (shape[2], shape[1], shape[0], 7)
    assert L.nrgb_set_project_slabs(*key, slabs) == 0
    try:
        s = A.project(act, cams, psf, mu)
        assert A.last_path() == FUSED
    finally:
        L.nrgb_set_project_slabs(*key, 0)
    assert per_plane_rel(s, o32.project(act, cams, psf, mu)) < RTOL


@pytest.mark.parametrize("shape,k,att_scale,angles", [
    ((40, 36, 40), 9, 1.0, None),            # 12 cameras: six mirror pairs
    ((40, 36, 40), 9, 400.0, None),          # slab mu sums above the mirror projector's bound
    ((24, 150, 24), 5, 1.0, [0, 33, 180, 213, 90, 17]),  # row windows, pairs and singles
    ((28, 20, 32), 0, 1.0, None),            # no PSF; nz != nx: backprojection centres unpaired
    ((36, 24, 44), 7, 1.0, None),            # nz != nx
])
def test_mirror_cameras(o32, shape, k, att_scale, angles):
    """Cameras at opposite angles served from shared samples (the default)
    match the oracle and the per-camera computation, in projection and in
    reference-mode backprojection."""
    from niftyrec_gb300 import _lib

    L = _lib.load()
    act = S.ellipsoid_phantom(shape, seed=12)
    mu = (S.mu_map(shape, seed=12) * att_scale).astype(np.float32)
    psf = S.gaussian_psf(k, shape[2], 0.5, 0.05) if k else None
    if angles is None:
        cams = S.cameras_about_y(12, 7.0)
    else:
        cams = np.zeros((3, len(angles)), np.float32)
        cams[1] = np.deg2rad(np.asarray(angles, np.float64)).astype(np.float32)
    assert L.nrgb_get_mirror_pairs() == 1
    s = A.project(act, cams, psf, mu)
    assert A.last_path() == FUSED
    so = o32.project(act, cams, psf, mu)
    assert per_plane_rel(s, so) < RTOL
    L.nrgb_set_mirror_pairs(0)
    try:
        s0 = A.project(act, cams, psf, mu)
    finally:
        L.nrgb_set_mirror_pairs(1)
    assert per_plane_rel(s0, so) < RTOL
    assert per_plane_rel(s, s0) < RTOL
    for m in (None, mu):  # without attenuation too
        assert per_plane_rel(A.project(act, cams, psf, m), o32.project(act, cams, psf, m)) < RTOL
    nz = shape[0]
    for m in (mu, None):
        b = A.backproject(so, cams, psf, m, nz=nz)
        assert A.last_path() == FUSED
        bo = o32.backproject(so, cams, psf, m, nz=nz)
        assert rel_l2(b, bo) < RTOL
        L.nrgb_set_mirror_pairs(0)
        try:
            b0 = A.backproject(so, cams, psf, m, nz=nz)
        finally:
            L.nrgb_set_mirror_pairs(1)
        assert rel_l2(b, b0) < RTOL
    # the exact-transpose backprojector (mode 1) serves mirror units too
    torch = pytest.importorskip("torch")
    from niftyrec_gb300.autograd import backproject_raw

    bt = backproject_raw(torch.from_numpy(so).cuda(), torch.from_numpy(mu).cuda(), cams, psf, nz=nz, mode=1)
    bto = o32.backproject(so, cams, psf, mu, truncate=0, adjoint=True, nz=nz)
    assert rel_l2(bt.cpu().numpy(), bto) < RTOL


@pytest.mark.parametrize("shape,k,ncam", [((24, 20, 24), 5, 12), ((20, 36, 28), 7, 9), ((20, 150, 24), 3, 6),
                                          ((20, 24, 132), 5, 8)])
def test_x_gantry_on_gantry_kernels(o32, shape, k, ncam):
    """Cameras rotating about x (nx a multiple of 4) run on the gantry kernels
    with x and y exchanged, reading the nifti arrays directly; projection,
    both backprojectors and d/dmu match the oracle / the general path."""
    torch = pytest.importorskip("torch")
    from niftyrec_gb300.autograd import attenuation_grad_raw, backproject_raw

    act = S.ellipsoid_phantom(shape, seed=61)
    mu = S.mu_map(shape, seed=61)
    psf = S.gaussian_psf(k, shape[2], 0.5, 0.05)
    cams = np.zeros((3, ncam), np.float32)
    cams[0] = np.deg2rad(3.0 + 360.0 / ncam * np.arange(ncam)).astype(np.float32)
    nz = shape[0]
    s = A.project(act, cams, psf, mu)
    assert A.last_path() == FUSED
    so = o32.project(act, cams, psf, mu)
    assert per_plane_rel(s, so) < RTOL
    b = A.backproject(so, cams, psf, mu, nz=nz)
    assert A.last_path() == FUSED
    assert rel_l2(b, o32.backproject(so, cams, psf, mu, nz=nz)) < RTOL
    bt = backproject_raw(torch.from_numpy(so).cuda(), torch.from_numpy(mu).cuda(), cams, psf, nz=nz, mode=1)
    bto = o32.backproject(so, cams, psf, mu, truncate=0, adjoint=True, nz=nz)
    assert rel_l2(bt.cpu().numpy(), bto) < RTOL
    g = torch.from_numpy(np.random.default_rng(5).uniform(0.5, 1.5, so.shape).astype(np.float32)).cuda()
    d = attenuation_grad_raw(g, torch.from_numpy(act).cuda(), torch.from_numpy(mu).cuda(), cams, psf)
    assert A.last_path() == FUSED
    tilted = cams.copy()
    tilted[2] = 1e-9
    dg = attenuation_grad_raw(g, torch.from_numpy(act).cuda(), torch.from_numpy(mu).cuda(), tilted, psf)
    assert A.last_path() == GENERAL
    assert rel_l2(d.cpu().numpy(), dg.cpu().numpy()) < RTOL


def test_x_gantry_odd_width_stays_general(o32):
    shape = (16, 18, 30)  # nx not a multiple of 4
    act = S.ellipsoid_phantom(shape, seed=62)
    cams = np.zeros((3, 6), np.float32)
    cams[0] = np.deg2rad(60.0 * np.arange(6)).astype(np.float32)
    s = A.project(act, cams, None, None)
    assert A.last_path() == GENERAL
    assert per_plane_rel(s, o32.project(act, cams, None, None)) < RTOL
