"""Pins the oracle's C restatement against the reference's own outputs (the
golden fixtures made by tests/golden/make_golden.py from the compiled
reference CPU path), and, where the compiled reference is present, against it
directly on fresh seeded inputs."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle.oracle import Reference, Restated
from niftyrec_gb300 import synthetic as S


@pytest.fixture(scope="module")
def o32():
    return Restated("f32")


@pytest.fixture(scope="module")
def o64():
    return Restated("f64")


def test_ygantry_psf_att_bitexact(o32, o64, golden):
    g = golden("ygantry_psf_att_24")
    sino = o32.project(g["act"], g["cameras"], g["psf"], g["mu"])
    assert np.array_equal(sino, g["sino"])
    bk = o32.backproject(g["counts"], g["cameras"], g["psf"], g["mu"])
    assert np.array_equal(bk, g["bkpr"])
    assert rel_l2(o64.project(g["act"], g["cameras"], g["psf"], g["mu"]), g["sino"]) < 1e-6
    assert rel_l2(o64.backproject(g["counts"], g["cameras"], g["psf"], g["mu"]), g["bkpr"]) < 1e-6


def test_plain_bitexact(o32, golden):
    g = golden("ygantry_plain_20")
    assert np.array_equal(o32.project(g["act"], g["cameras"]), g["sino"])
    assert np.array_equal(o32.backproject(g["sino"], g["cameras"]), g["bkpr"])
    assert np.array_equal(o32.project(g["act"], g["cameras3"]), g["sino"])


def test_noncubic_bitexact(o32, golden):
    g = golden("noncubic_24x20x16")
    assert np.array_equal(o32.project(g["act"], g["cameras"], g["psf"], g["mu"]), g["sino"])
    assert np.array_equal(o32.backproject(g["sino"], g["cameras"], g["psf"], g["mu"], nz=16), g["bkpr"])


def test_general_cameras_and_background_bitexact(o32, golden):
    g = golden("general_cams_18")
    bg, bga = float(g["bg"]), float(g["bg_att"])
    assert np.array_equal(o32.project(g["act"], g["cameras6"], None, g["mu"], bg, bga), g["sino_bg"])
    assert np.array_equal(o32.backproject(g["sino_bg"], g["cameras6"], None, g["mu"], bg, bga), g["bkpr_bg"])
    assert np.array_equal(o32.project(g["act"], g["cameras3"], None, g["mu"]), g["sino"])
    assert np.array_equal(o32.backproject(g["sino"], g["cameras3"], None, g["mu"]), g["bkpr"])


def test_mlem_step_bitexact(o32, golden):
    g = golden("mlem_16")
    n = g["cameras3"].shape[1]
    x1 = o32.osem_step(np.ones_like(g["mu"]), g["counts"], g["cameras3"], list(range(n)), g["mu"], g["psf"])
    assert np.array_equal(x1, g["x1"])
    x2 = o32.osem_step(x1, g["counts"], g["cameras3"], list(range(n)), g["mu"], g["psf"])
    assert np.array_equal(x2, g["x2"])


def test_rotation_bitexact(o32, golden):
    g = golden("rotate_16x14x12")
    M = o32.rotation_matrix([0.3, -0.7, 0.2], [7.5, 6.5, 5.5], 0)
    assert np.array_equal(o32.affine_resample(g["vol"], M), g["rot_xyz"])
    M = o32.rotation_matrix([-0.3, 0.7, -0.2], [7.5, 6.5, 5.5], 5)
    assert np.array_equal(o32.affine_resample(g["vol"], M), g["rot_zyx"])


def test_make_cameras_bitexact(o32, golden):
    g = golden("make_cameras")
    assert np.array_equal(o32.make_cameras(0.0, 354.0, 60, 1), g["c60"])
    assert np.array_equal(o32.make_cameras(-30.0, 45.0, 7, 0), g["c7x"])
    assert np.array_equal(o32.make_cameras(10.0, 100.0, 5, 2), g["c5z"])


def test_known_answers(o32):
    """Angle 0 is the plain z-sum; 90 degrees is the x-sum with x flipped."""
    vol = S.ellipsoid_phantom((12, 12, 12), seed=3)
    cams = np.array([0.0, np.pi / 2], dtype=np.float32)
    s = o32.project(vol, cams)
    np.testing.assert_allclose(s[0], vol.sum(axis=0), rtol=1e-5)
    # 90 degrees about y maps detector column x to the source plane z = 11 - x
    # (grid centre 5.5) and depth to source x: the projection is the x-sum.
    xsum = vol.sum(axis=2)  # (nz, ny)
    np.testing.assert_allclose(s[1], xsum.T[:, ::-1], rtol=2e-5, atol=1e-5)


def test_constant_mu_beer_lambert(o32):
    """Constant activity a and constant mu along depth: p = a * sum_z exp(-mu*(z+1))."""
    n = 10
    act = np.ones((n, n, n), np.float32)
    mu = np.full((n, n, n), 0.02, np.float32)
    s = o32.project(act, np.zeros(1, np.float32), None, mu)
    expect = np.sum(np.exp(-0.02 * np.arange(1, n + 1)))
    np.testing.assert_allclose(s[0], expect, rtol=1e-5)


def test_gradient_known_answer_angle0(o32):
    """The attenuation gradient at angle 0 without PSF is the sinogram times
    the depth suffix sum of a * exp(-T) (T the inclusive depth sum of mu),
    emission-lib_gpu/_et_attenuation_gradient_gpu_kernels.cu:24-39 with an
    identity rotation; with a PSF every plane of it is convolved (row, then
    column), and a camera at 90 degrees sees the same sums along x."""
    rng = np.random.default_rng(12)
    shape = (8, 7, 9)  # nz <= nx: the PSF has nx planes
    act = rng.uniform(0.5, 2.0, shape).astype(np.float32)
    mu = rng.uniform(0.0, 0.2, shape).astype(np.float32)
    s = rng.uniform(-1.0, 1.0, (1,) + shape[1:]).astype(np.float32)
    g = o32.gradient_attenuation(s, act, mu, np.zeros(1, np.float32))
    a, m = act.astype(np.float64), mu.astype(np.float64)
    w = a * np.exp(-np.cumsum(m, axis=0))
    expect = s[0].astype(np.float64) * np.cumsum(w[::-1], axis=0)[::-1]
    np.testing.assert_allclose(g, expect, rtol=2e-5, atol=1e-6)
    # separable PSF: each plane z of the suffix volume convolved with plane z's kernels
    psf = S.gaussian_psf(3, shape[2], 0.6, 0.1)
    gp = o32.gradient_attenuation(s, act, mu, np.zeros(1, np.float32), psf)
    conv = np.empty_like(expect)
    for z in range(shape[0]):
        k = psf[z].astype(np.float64)
        kr, kc = k[1, :], k[:, 1] / k[1, 1]
        row = np.zeros_like(expect[z])
        for d in (-1, 0, 1):  # true convolution along x: out[x] = sum_d in[x + d] * kr[1 - d]
            src = np.roll(expect[z], -d, axis=1)
            if d > 0:
                src[:, -d:] = 0
            if d < 0:
                src[:, :-d] = 0
            row += src * kr[1 - d]
        col = np.zeros_like(row)
        for d in (-1, 0, 1):
            src = np.roll(row, -d, axis=0)
            if d > 0:
                src[-d:, :] = 0
            if d < 0:
                src[:-d, :] = 0
            col += src * kc[1 - d]
        conv[z] = col
    np.testing.assert_allclose(gp, conv, rtol=5e-5, atol=1e-5)


@pytest.mark.skipif(not Reference.available, reason="compiled reference not present")
def test_against_compiled_reference_fresh_inputs(o32):
    R = Reference()
    rng = np.random.default_rng(99)
    for shape, k in [((14, 14, 14), 5), ((12, 10, 14), 3)]:
        act = S.ellipsoid_phantom(shape, seed=int(rng.integers(1000)))
        mu = S.mu_map(shape, seed=int(rng.integers(1000)))
        psf = S.gaussian_psf(k, shape[2])
        cams = rng.uniform(-3, 3, (3, 4)).astype(np.float32)
        cams[0] = 0
        cams[2] = 0
        assert np.array_equal(R.project(act, cams, psf, mu), o32.project(act, cams, psf, mu))
        s = R.project(act, cams, psf, mu)
        assert np.array_equal(R.backproject(s, cams, psf, mu, nz=shape[0]),
                              o32.backproject(s, cams, psf, mu, nz=shape[0]))


def test_partial_sum_projector_restatement():
    """The partial-sum projector (emission-lib/_et.cpp:2106-2436, GPU-only in
    the reference) sums the same terms as the projector in the opposite depth
    order: equal projections to float32 rounding; the farthest partial sum is
    the background (times the background image) and, without attenuation,
    partial sums fall monotonically toward the detector."""
    from oracle.oracle import Restated

    o = Restated("f32")
    shape = (14, 12, 16)
    act = S.ellipsoid_phantom(shape, seed=90)
    mu = S.mu_map(shape, seed=90)
    psf = S.gaussian_psf(5, shape[2], 0.5, 0.05)
    cams = S.cameras_about_y(4, 20.0)
    bgi = np.random.default_rng(1).uniform(0.5, 1.5, shape[1:]).astype(np.float32)
    s, part = o.project_partial(act, cams, psf, mu, bg=0.3, truncate=0)
    ref = o.project(act, cams, psf, mu, 0.3, truncate=0)
    assert np.linalg.norm(s - ref) / np.linalg.norm(ref) < 1e-5
    s2, part2 = o.project_partial(act, cams, psf, mu, bg=0.3, bg_image=bgi, truncate=0)
    np.testing.assert_array_equal(part2[:, -1], np.broadcast_to(np.float32(0.3) * bgi, part2[:, -1].shape))
    _, part3 = o.project_partial(act, cams, psf, None, truncate=0)
    assert np.all(np.diff(part3, axis=1) <= 0)
    sr, partr = o.project_partial(act, cams, psf, mu, bg=0.0, truncate=0, rotate=1)
    np.testing.assert_allclose(sr, o.project(act, cams, psf, mu, truncate=0), rtol=1e-4, atol=1e-5)
    assert partr.shape == (4,) + shape


def test_fisher_grid_restatement_matches_golden(golden):
    """et_fisher_grid (emission-lib/_et.cpp:531-746) restated: bit-exact to the
    compiled reference's et_array_fisher_grid on the committed fixture."""
    from oracle.oracle import Restated

    g = golden("fisher_16")
    f, pr = Restated("f32").fisher_grid(g["act"], g["cameras"], g["psf"], g["grid"], 24, g["mu"])
    np.testing.assert_array_equal(f, g["fisher"])
    np.testing.assert_array_equal(pr, g["prior"])
    assert np.allclose(f, f.T) and (np.diag(f) > 0).any()


@pytest.mark.parametrize("shape", [(12, 10, 16), (16, 10, 12), (10, 10, 10)])
def test_adjoint_is_transpose_of_projector(o64, shape):
    """The exact-adjoint backprojection (not in the reference) is the transpose
    of the projector, also when nz != nx (it takes the projector's rotation
    centre, not the reference backprojector's): <A x, y> = <x, A^T y>."""
    nz, ny, nx = shape
    rng = np.random.default_rng(nz * 7 + nx)
    cams = S.cameras_about_y(5, 11.0)
    # the reference takes a PSF of nx planes (indexed by depth z < nz)
    psf = S.gaussian_psf(3, nx, 0.6, 0.05) if nx >= nz else None
    mu = S.mu_map(shape, seed=2).astype(np.float64)
    x = rng.random(shape)
    y = rng.random((5, ny, nx))
    ax = o64.project(x, cams, psf, mu, truncate=0)
    aty = o64.backproject(y, cams, psf, mu, truncate=0, adjoint=True, nz=nz)
    lhs, rhs = float(np.sum(ax * y)), float(np.sum(x * aty))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs), (lhs, rhs)


def test_convolve2d_restatement_known_answers(o32):
    """The oracle's per-slice convolution: a constant image stays constant
    times the kernel sum (border clamping), a delta image returns the kernel
    centred on the delta (the impulse response of a true convolution), per
    slice."""
    rng = np.random.default_rng(3)
    ker = rng.random((2, 5, 3)).astype(np.float32)
    const = np.full((2, 9, 11), 2.0, np.float32)
    out = o32.convolve2d(const, ker)
    np.testing.assert_allclose(out, np.broadcast_to(2.0 * ker.sum(axis=(1, 2))[:, None, None], out.shape), rtol=1e-6)
    delta = np.zeros((2, 9, 11), np.float32)
    delta[:, 4, 5] = 1.0
    out = o32.convolve2d(delta, ker)
    for z in range(2):
        np.testing.assert_array_equal(out[z, 2:7, 4:7], ker[z])
