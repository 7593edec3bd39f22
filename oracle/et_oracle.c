/*
 * et_oracle.c -- CPU restatement of NiftyRec's rotation-based SPECT emission
 * path, used ONLY as test infrastructure: the oracle that the CUDA product
 * path is compared against, and the "port" CPU baseline of bench.py.  Nothing
 * in the shipped library links or calls this file.
 *
 * Parity of this restatement is pinned against the reference itself: the
 * reference CPU path compiled from its own sources (oracle/Makefile.ref ->
 * oracle/_ref/libref_et.so) and the golden fixtures generated from it
 * (tests/golden/make_golden.py).  The attenuation-gradient function has no
 * CPU implementation in the reference (its CPU entry point is a stub that
 * returns 1, emission-lib/_et.cpp:763-766); here it restates the GPU
 * orchestration emission-lib/_et.cpp:1787-1887 with the GPU kernel
 * emission-lib_gpu/_et_attenuation_gradient_gpu_kernels.cu:24-39, using the
 * CPU resampler and CPU separable convolution in place of tex3D and the GPU
 * convolution.
 *
 * The file is compiled twice: with REAL=float (suffix _f32, follows the
 * reference's float arithmetic operation by operation) and with REAL=double
 * (suffix _f64, the FP64 oracle).  Arrays are in nifti order: x fastest, then
 * y, then z; sinograms are [nx, ny, n_cameras] with x fastest.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL float
#endif
#ifndef SUFFIX
#define SUFFIX _f32
#endif
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define ORC(name) CAT(orc_##name, SUFFIX)

#if defined(ORACLE_DOUBLE)
#define R_SIN sin
#define R_COS cos
#define R_EXP exp
#define R_FLOOR floor
#else
#define R_SIN sinf
#define R_COS cosf
#define R_EXP expf
#define R_FLOOR floorf
#endif

/* Status codes of emission-lib/_et_common.h:40-48. */
#define ORC_OK 0
#define ORC_ERR_PARAMETERS 2
#define ORC_ERR_ALLOCCPU 5

/* 4x4 row-major matrix product, emission reference reg-lib/_reg_affineTransformation.cpp:18-29:
 * each entry is ((a0*b0 + a1*b1) + a2*b2) + a3*b3 evaluated left to right. */
static void mat_mul(const REAL *A, const REAL *B, REAL *C)
{
    REAL t[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            t[i * 4 + j] = A[i * 4 + 0] * B[0 * 4 + j] + A[i * 4 + 1] * B[1 * 4 + j]
                         + A[i * 4 + 2] * B[2 * 4 + j] + A[i * 4 + 3] * B[3 * 4 + j];
    memcpy(C, t, sizeof(t));
}

/* Rotation about a centre, emission-lib/_et_common.cpp:35-171.
 * axis_order 0..5 = XYZ, XZY, YXZ, YZX, ZXY, ZYX (emission-lib/_et_common.h:26-31).
 * The linear part is the product of the elementary rotations in the given
 * order (XYZ: Rz*(Ry*Rx)); the translation column is c - R*c. */
void ORC(rotation_matrix)(REAL *M, REAL tx, REAL ty, REAL tz, REAL cx, REAL cy, REAL cz, int axis_order)
{
    REAL sx = R_SIN(tx), cxs = R_COS(tx);
    REAL sy = R_SIN(ty), cys = R_COS(ty);
    REAL sz = R_SIN(tz), czs = R_COS(tz);
    REAL Rx[16] = {1, 0, 0, 0, 0, cxs, -sx, 0, 0, sx, cxs, 0, 0, 0, 0, 1};
    REAL Ry[16] = {cys, 0, sy, 0, 0, 1, 0, 0, -sy, 0, cys, 0, 0, 0, 0, 1};
    REAL Rz[16] = {czs, -sz, 0, 0, sz, czs, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    REAL T[16] = {0, 0, 0, cx, 0, 0, 0, cy, 0, 0, 0, cz, 0, 0, 0, 1};
    const REAL *first, *second, *third;
    switch (axis_order) {
    case 1: first = Rx; second = Rz; third = Ry; break;  /* XZY: Ry*(Rz*Rx) */
    case 2: first = Ry; second = Rx; third = Rz; break;  /* YXZ: Rz*(Rx*Ry) */
    case 3: first = Ry; second = Rz; third = Rx; break;  /* YZX: Rx*(Rz*Ry) */
    case 4: first = Rz; second = Rx; third = Ry; break;  /* ZXY: Ry*(Rx*Rz) */
    case 5: first = Rz; second = Ry; third = Rx; break;  /* ZYX: Rx*(Ry*Rz) */
    default: first = Rx; second = Ry; third = Rz; break; /* XYZ: Rz*(Ry*Rx) */
    }
    REAL P[16], RT[16];
    mat_mul(second, first, P);
    mat_mul(third, P, M);
    mat_mul(M, T, RT);
    M[3] = cx - RT[3];
    M[7] = cy - RT[7];
    M[11] = cz - RT[11];
}

/* Trilinear resampling of src at A*(x,y,z) for every voxel of dst (same
 * grid), reg-lib/_reg_affineTransformation.cpp:100-136 (position field, identity
 * voxel-to-world matrix) and reg-lib/_reg_resampling.cpp:334-450 (trilinear,
 * floor + "relative<0 => 0", out-of-grid neighbours skipped; with bg != 0 the
 * reference adds bg*xBasis[] for each skipped neighbour, reproduced here). */
void ORC(affine_resample)(const REAL *src, REAL *dst, int nx, int ny, int nz, const REAL *A, REAL bg)
{
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                REAL fx = (REAL)x, fy = (REAL)y, fz = (REAL)z;
                REAL pos[3];
                for (int i = 0; i < 3; i++)
                    pos[i] = A[i * 4 + 0] * fx + A[i * 4 + 1] * fy + A[i * 4 + 2] * fz + A[i * 4 + 3];
                int prev[3];
                REAL basis[3][2];
                for (int i = 0; i < 3; i++) {
                    prev[i] = (int)R_FLOOR(pos[i]);
                    REAL rel = pos[i] - (REAL)prev[i];
                    if (rel < 0) rel = 0;
                    basis[i][0] = (REAL)(1.0 - rel);
                    basis[i][1] = rel;
                }
                REAL val = 0;
                REAL bgw = 0;
                for (int c = 0; c < 2; c++) {
                    int Z = prev[2] + c;
                    if (Z >= 0 && Z < nz) {
                        REAL ysum = 0;
                        for (int b = 0; b < 2; b++) {
                            int Y = prev[1] + b;
                            if (Y >= 0 && Y < ny) {
                                REAL xsum = 0;
                                for (int a = 0; a < 2; a++) {
                                    int X = prev[0] + a;
                                    if (X >= 0 && X < nx)
                                        xsum += (REAL)(src[X + nx * (Y + (size_t)ny * Z)] * basis[0][a]);
                                    else if (bg != 0)
                                        bgw += (REAL)(bg * basis[0][a]);
                                }
                                ysum += xsum * basis[1][b];
                            } else if (bg != 0) {
                                bgw += (REAL)(bg * basis[0][b]);
                            }
                        }
                        val += ysum * basis[2][c];
                    } else if (bg != 0) {
                        bgw += (REAL)(bg * basis[0][c]);
                    }
                }
                if (bg != 0) val += bgw;
                dst[x + nx * (y + (size_t)ny * z)] = val;
            }
}

/* Separated depth-dependent PSF, emission-lib/_et.cpp:194-215: per plane n
 * the row kernel is the central row of the kx*ky plane and the column kernel
 * is the central column divided by the centre value.  Layout per plane:
 * [row (kx) | column (kx)], stride kx+ky as in the reference. */
void ORC(psf_separate)(const REAL *psf, int kx, int ky, int nplanes, REAL *sep)
{
    int stride = kx + ky;
    int c = (kx - 1) / 2;
    for (int n = 0; n < nplanes; n++) {
        const REAL *plane = psf + (size_t)kx * ky * n;
        REAL norm = plane[c * kx + c];
        for (int i = 0; i < kx; i++) {
            sep[stride * n + i] = plane[c * kx + i];
            sep[stride * n + kx + i] = plane[c + i * kx] / norm;
        }
    }
}

/* Per-plane separable convolution, emission-lib/_et_convolveSeparable2D.cpp:13-75:
 * a true convolution (kernel index R-k) along x with the row kernel, then
 * along y with the column kernel, zero outside the plane.  Plane z uses
 * kernel plane z.  In place. */
void ORC(convolve_separable)(REAL *vol, int nx, int ny, int nz, const REAL *sep, int klen_h, int klen_w)
{
    int rw = (klen_w - 1) / 2, rh = (klen_h - 1) / 2;
    int stride = klen_h + klen_w;
    REAL *buf = (REAL *)malloc(sizeof(REAL) * (size_t)nx * ny);
    for (int z = 0; z < nz; z++) {
        REAL *plane = vol + (size_t)nx * ny * z;
        const REAL *krow = sep + (size_t)stride * z;
        const REAL *kcol = krow + klen_w;
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                REAL s = 0;
                for (int k = -rw; k <= rw; k++) {
                    int d = x + k;
                    if (d >= 0 && d < nx) s += plane[y * nx + d] * krow[rw - k];
                }
                buf[y * nx + x] = s;
            }
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                REAL s = 0;
                for (int k = -rh; k <= rh; k++) {
                    int d = y + k;
                    if (d >= 0 && d < ny) s += buf[d * nx + x] * kcol[rh - k];
                }
                plane[y * nx + x] = s;
            }
    }
    free(buf);
}

/* Transpose of ORC(convolve_separable) (correlation, column pass first):
 * used by the exact-adjoint backprojector, which the reference does not have. */
static void convolve_separable_T(REAL *vol, int nx, int ny, int nz, const REAL *sep, int klen_h, int klen_w)
{
    int rw = (klen_w - 1) / 2, rh = (klen_h - 1) / 2;
    int stride = klen_h + klen_w;
    REAL *buf = (REAL *)malloc(sizeof(REAL) * (size_t)nx * ny);
    for (int z = 0; z < nz; z++) {
        REAL *plane = vol + (size_t)nx * ny * z;
        const REAL *krow = sep + (size_t)stride * z;
        const REAL *kcol = krow + klen_w;
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                REAL s = 0;
                for (int k = -rh; k <= rh; k++) {
                    int d = y + k;
                    if (d >= 0 && d < ny) s += plane[d * nx + x] * kcol[rh + k];
                }
                buf[y * nx + x] = s;
            }
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                REAL s = 0;
                for (int k = -rw; k <= rw; k++) {
                    int d = x + k;
                    if (d >= 0 && d < nx) s += buf[y * nx + d] * krow[rw + k];
                }
                plane[y * nx + x] = s;
            }
    }
    free(buf);
}

/* Attenuated line integral along z, emission-lib/_et_line_integral_attenuated.cpp:14-68.
 * The transmission includes the voxel's own mu: T += mu[z]; p += a[z]*exp(-T);
 * then p += bg*exp(-T_total).  act or att may be NULL (plain sum / mu only). */
void ORC(line_integral_attenuated)(const REAL *act, const REAL *att, REAL *plane_out, int nx, int ny, int nz, REAL bg)
{
    size_t nxy = (size_t)nx * ny;
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            size_t i0 = x + (size_t)nx * y;
            REAL p = 0, T = 0;
            if (act && att) {
                for (int z = 0; z < nz; z++) {
                    T += att[i0 + nxy * z];
                    p = p + act[i0 + nxy * z] * R_EXP(-T);
                }
                p = p + bg * R_EXP(-T);
            } else if (act) {
                for (int z = 0; z < nz; z++) p = p + act[i0 + nxy * z];
                p = p + bg;
            } else {
                for (int z = 0; z < nz; z++) T += att[i0 + nxy * z];
                p = bg * R_EXP(-T);
            }
            plane_out[i0] = p;
        }
}

/* Spread along z, emission-lib/_et_line_backproject_attenuated.cpp:17-36 and
 * emission-lib/_et_line_backproject.cpp:17-30: vol[x,y,z] = s[x,y]*exp(-T_z)
 * (T inclusive) or vol[x,y,z] = s[x,y]. */
static void line_backproject(const REAL *plane_in, const REAL *att, REAL *vol, int nx, int ny, int nz)
{
    size_t nxy = (size_t)nx * ny;
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            size_t i0 = x + (size_t)nx * y;
            REAL T = 0;
            for (int z = 0; z < nz; z++) {
                if (att) {
                    T += att[i0 + nxy * z];
                    vol[i0 + nxy * z] = plane_in[i0] * R_EXP(-T);
                } else {
                    vol[i0 + nxy * z] = plane_in[i0];
                }
            }
        }
}

/* Camera-column expansion of the array interface,
 * emission-lib/_et_array_interface.cpp:409-440: [n x 1] -> theta_y only,
 * [n x 3] -> angles, [n x 6] -> angles + per-camera centres; otherwise the
 * centre is (size-1)/2 computed in double and stored in the working type. */
static int expand_cameras(const REAL *cameras, int ncam, int ncols, const int center_size[3], REAL *angles, REAL *centers)
{
    if (!(ncols == 1 || ncols == 3 || ncols == 6)) return ORC_ERR_PARAMETERS;
    if (ncols == 1) {
        memset(angles, 0, sizeof(REAL) * 3 * ncam);
        for (int c = 0; c < ncam; c++) angles[ncam + c] = cameras[c];
    } else {
        memcpy(angles, cameras, sizeof(REAL) * 3 * ncam);
    }
    if (ncols == 6) {
        memcpy(centers, cameras + 3 * ncam, sizeof(REAL) * 3 * ncam);
    } else {
        for (int c = 0; c < ncam; c++)
            for (int a = 0; a < 3; a++) centers[a * ncam + c] = (REAL)((center_size[a] - 1) / 2.0);
    }
    return ORC_OK;
}

/* et_project, emission-lib/_et.cpp:122-296 (called through
 * SPECT_project_parallelholes, emission-lib/_et_array_interface.cpp:337-541).
 * act/att/psf may be NULL.  sino is [nx, ny, ncam]. */
int ORC(project)(const REAL *act, const REAL *att, const int size[3], REAL *sino,
                 const REAL *angles, const REAL *centers, int ncam,
                 const REAL *psf, const int psf_size[3], REAL bg, REAL bg_att, int truncate)
{
    int nx = size[0], ny = size[1], nz = size[2];
    size_t nvox = (size_t)nx * ny * nz, nxy = (size_t)nx * ny;
    if (!act && !att) return ORC_ERR_PARAMETERS;
    REAL *ract = act ? (REAL *)malloc(sizeof(REAL) * nvox) : NULL;
    REAL *ratt = att ? (REAL *)malloc(sizeof(REAL) * nvox) : NULL;
    REAL *sep = NULL;
    if (psf) {
        sep = (REAL *)malloc(sizeof(REAL) * (size_t)(psf_size[0] + psf_size[1]) * psf_size[2]);
        ORC(psf_separate)(psf, psf_size[0], psf_size[1], psf_size[2], sep);
    }
    REAL A[16];
    for (int cam = 0; cam < ncam; cam++) {
        ORC(rotation_matrix)(A, angles[cam], angles[ncam + cam], angles[2 * ncam + cam],
                             centers[cam], centers[ncam + cam], centers[2 * ncam + cam], 0);
        if (act) ORC(affine_resample)(act, ract, nx, ny, nz, A, bg);
        if (att) ORC(affine_resample)(att, ratt, nx, ny, nz, A, bg_att);
        if (psf && act) ORC(convolve_separable)(ract, nx, ny, nz, sep, psf_size[0], psf_size[1]);
        ORC(line_integral_attenuated)(ract, ratt, sino + nxy * cam, nx, ny, nz, bg);
    }
    if (truncate)
        for (size_t i = 0; i < nxy * ncam; i++)
            if (sino[i] < 0) sino[i] = 0;
    free(ract);
    free(ratt);
    free(sep);
    return ORC_OK;
}

/* et_backproject, emission-lib/_et.cpp:312-513: per camera rotate mu (+theta,
 * XYZ), spread (attenuated), PSF, rotate back (-theta, ZYX), accumulate.
 * adjoint != 0 replaces the inverse-rotation gather by the exact transpose of
 * the projector's trilinear gather and the PSF by its transpose (not in the
 * reference; used for adjoint tests). */
int ORC(backproject)(const REAL *sino, const REAL *att, const int size[3], REAL *bkpr,
                     const REAL *angles, const REAL *centers, int ncam,
                     const REAL *psf, const int psf_size[3], REAL bg, REAL bg_att, int truncate, int adjoint)
{
    int nx = size[0], ny = size[1], nz = size[2];
    size_t nvox = (size_t)nx * ny * nz, nxy = (size_t)nx * ny;
    REAL *ratt = att ? (REAL *)malloc(sizeof(REAL) * nvox) : NULL;
    REAL *tmp = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *rot = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *sep = NULL;
    if (psf) {
        sep = (REAL *)malloc(sizeof(REAL) * (size_t)(psf_size[0] + psf_size[1]) * psf_size[2]);
        ORC(psf_separate)(psf, psf_size[0], psf_size[1], psf_size[2], sep);
    }
    memset(bkpr, 0, sizeof(REAL) * nvox);
    REAL A[16];
    for (int cam = 0; cam < ncam; cam++) {
        REAL tx = angles[cam], ty = angles[ncam + cam], tz = angles[2 * ncam + cam];
        REAL cx = centers[cam], cy = centers[ncam + cam], cz = centers[2 * ncam + cam];
        ORC(rotation_matrix)(A, tx, ty, tz, cx, cy, cz, 0);
        if (att) ORC(affine_resample)(att, ratt, nx, ny, nz, A, bg_att);
        line_backproject(sino + nxy * cam, ratt, tmp, nx, ny, nz);
        if (!adjoint) {
            if (psf) ORC(convolve_separable)(tmp, nx, ny, nz, sep, psf_size[0], psf_size[1]);
            ORC(rotation_matrix)(A, -tx, -ty, -tz, cx, cy, cz, 5);
            ORC(affine_resample)(tmp, rot, nx, ny, nz, A, bg);
            for (size_t i = 0; i < nvox; i++) bkpr[i] += rot[i];
        } else {
            if (psf) convolve_separable_T(tmp, nx, ny, nz, sep, psf_size[0], psf_size[1]);
            /* scatter: transpose of ORC(affine_resample) with bg = 0 */
            for (int z = 0; z < nz; z++)
                for (int y = 0; y < ny; y++)
                    for (int x = 0; x < nx; x++) {
                        REAL v = tmp[x + nx * (y + (size_t)ny * z)];
                        REAL fx = (REAL)x, fy = (REAL)y, fz = (REAL)z;
                        REAL pos[3];
                        int prev[3];
                        REAL basis[3][2];
                        for (int i = 0; i < 3; i++) {
                            pos[i] = A[i * 4 + 0] * fx + A[i * 4 + 1] * fy + A[i * 4 + 2] * fz + A[i * 4 + 3];
                            prev[i] = (int)R_FLOOR(pos[i]);
                            REAL rel = pos[i] - (REAL)prev[i];
                            if (rel < 0) rel = 0;
                            basis[i][0] = (REAL)(1.0 - rel);
                            basis[i][1] = rel;
                        }
                        for (int c = 0; c < 2; c++) {
                            int Z = prev[2] + c;
                            if (Z < 0 || Z >= nz) continue;
                            for (int b = 0; b < 2; b++) {
                                int Y = prev[1] + b;
                                if (Y < 0 || Y >= ny) continue;
                                for (int a = 0; a < 2; a++) {
                                    int X = prev[0] + a;
                                    if (X < 0 || X >= nx) continue;
                                    bkpr[X + nx * (Y + (size_t)ny * Z)] += v * basis[0][a] * basis[1][b] * basis[2][c];
                                }
                            }
                        }
                    }
        }
    }
    if (truncate)
        for (size_t i = 0; i < nvox; i++)
            if (bkpr[i] < 0) bkpr[i] = 0;
    free(ratt);
    free(tmp);
    free(rot);
    free(sep);
    return ORC_OK;
}

/* Attenuation gradient, restating et_gradient_attenuation_gpu
 * (emission-lib/_et.cpp:1787-1887) on the CPU.  Per camera: rotate mu and
 * activity (+theta, XYZ; activity resampled with bg, mu with bg_att); run the
 * two-pass kernel of emission-lib_gpu/_et_attenuation_gradient_gpu_kernels.cu:24-39
 * (pass 1: inclusive prefix T_z; pass 2, far to near:
 * acc += a_z*exp(-T_z), g_z = s*acc); PSF; rotate back (-theta, ZYX, bg);
 * accumulate; truncate if asked. */
int ORC(gradient_attenuation)(const REAL *sino, const REAL *act, const REAL *att, const int size[3], REAL *grad,
                              const REAL *angles, const REAL *centers, int ncam,
                              const REAL *psf, const int psf_size[3], REAL bg, REAL bg_att, int truncate)
{
    int nx = size[0], ny = size[1], nz = size[2];
    size_t nvox = (size_t)nx * ny * nz, nxy = (size_t)nx * ny;
    REAL *ract = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *ratt = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *tmp = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *rot = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *sep = NULL;
    if (psf) {
        sep = (REAL *)malloc(sizeof(REAL) * (size_t)(psf_size[0] + psf_size[1]) * psf_size[2]);
        ORC(psf_separate)(psf, psf_size[0], psf_size[1], psf_size[2], sep);
    }
    memset(grad, 0, sizeof(REAL) * nvox);
    REAL A[16];
    for (int cam = 0; cam < ncam; cam++) {
        REAL tx = angles[cam], ty = angles[ncam + cam], tz = angles[2 * ncam + cam];
        REAL cx = centers[cam], cy = centers[ncam + cam], cz = centers[2 * ncam + cam];
        ORC(rotation_matrix)(A, tx, ty, tz, cx, cy, cz, 0);
        ORC(affine_resample)(att, ratt, nx, ny, nz, A, bg_att);
        ORC(affine_resample)(act, ract, nx, ny, nz, A, bg);
        const REAL *s = sino + nxy * cam;
        for (size_t i0 = 0; i0 < nxy; i0++) {
            REAL T = 0;
            for (int z = 0; z < nz; z++) {
                T += ratt[i0 + nxy * z];
                tmp[i0 + nxy * z] = T;
            }
            REAL acc = 0;
            for (int z = nz - 1; z >= 0; z--) {
                acc += ract[i0 + nxy * z] * R_EXP(-tmp[i0 + nxy * z]);
                tmp[i0 + nxy * z] = s[i0] * acc;
            }
        }
        if (psf) ORC(convolve_separable)(tmp, nx, ny, nz, sep, psf_size[0], psf_size[1]);
        ORC(rotation_matrix)(A, -tx, -ty, -tz, cx, cy, cz, 5);
        ORC(affine_resample)(tmp, rot, nx, ny, nz, A, bg);
        for (size_t i = 0; i < nvox; i++) grad[i] += rot[i];
    }
    if (truncate)
        for (size_t i = 0; i < nvox; i++)
            if (grad[i] < 0) grad[i] = 0;
    free(ract);
    free(ratt);
    free(tmp);
    free(rot);
    free(sep);
    return ORC_OK;
}

/* Array-interface wrappers with the reference's size and centre rules. */

/* SPECT_project_parallelholes, emission-lib/_et_array_interface.cpp:337-541. */
int ORC(spect_project)(const REAL *act, const int act_size[3], REAL *sino, const int sino_size[3],
                       const REAL *cameras, const int cam_size[2], const REAL *psf, const int psf_size[3],
                       const REAL *att, const int att_size[3], REAL bg, REAL bg_att, int truncate)
{
    int asz[3] = {act_size[0], act_size[1], act_size[2]};
    int no_act = (asz[0] == 0 && asz[1] == 0 && asz[2] == 0);
    int no_psf = (psf_size[0] == 0 && psf_size[1] == 0 && psf_size[2] == 0);
    int no_att = (att_size[0] == 0 && att_size[1] == 0 && att_size[2] == 0);
    if (no_act) { asz[0] = att_size[0]; asz[1] = att_size[1]; asz[2] = att_size[2]; }
    if (no_act && no_att) return ORC_ERR_PARAMETERS;
    int ncam = cam_size[0], ncols = cam_size[1];
    if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != asz[0])) return ORC_ERR_PARAMETERS;
    (void)sino_size;
    REAL *angles = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    REAL *centers = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    int st = expand_cameras(cameras, ncam, ncols, asz, angles, centers);
    if (st == ORC_OK)
        st = ORC(project)(no_act ? NULL : act, no_att ? NULL : att, asz, sino, angles, centers, ncam,
                          no_psf ? NULL : psf, psf_size, bg, bg_att, truncate);
    free(angles);
    free(centers);
    return st;
}

/* Partial-sum projector: et_project_partial_gpu, emission-lib/_et.cpp:2106-2436
 * (the CPU entry point et_project_partial is a stub returning 1,
 * emission-lib/_et.cpp:783-786), with the partial-sum branch of the line
 * integral kernel emission-lib_gpu/_et_line_integral_attenuated_gpu_kernels.cu:57-103
 * restated on the CPU pieces (resampler, separable PSF).  Per camera: rotate
 * activity (bg) and mu (bg_att), PSF, then walk depth from the far end:
 * partial[z] = s; s = (s + a[z]) * exp(-mu[z]) (mu only: s *= exp(-mu[z]);
 * activity only: s += a[z]), s starting at bg (times bg_image[x, y] if
 * given); the projection is the final s.  do_rotate: the partial-sum volume is
 * rotated back to the image frame (-theta, ZYX, background bg,
 * emission-lib/_et.cpp:2373-2404).  partial is [nx, ny, nz, ncam]. */
static void line_partial(const REAL *act, const REAL *att, const REAL *bg_image, REAL *plane_out, REAL *partial,
                         int nx, int ny, int nz, REAL bg)
{
    size_t nxy = (size_t)nx * ny;
    for (size_t i0 = 0; i0 < nxy; i0++) {
        REAL s = bg;
        if (bg_image) s = s * bg_image[i0];
        for (int z = nz - 1; z >= 0; z--) {
            size_t j = i0 + nxy * z;
            partial[j] = s;
            if (act && att)
                s = (s + act[j]) * R_EXP(-att[j]);
            else if (att)
                s = s * R_EXP(-att[j]);
            else
                s = s + act[j];
        }
        plane_out[i0] = s;
    }
}

int ORC(project_partial)(const REAL *act, const REAL *att, const int size[3], REAL *sino, REAL *partial,
                         const REAL *angles, const REAL *centers, int ncam, const REAL *psf, const int psf_size[3],
                         REAL bg, const REAL *bg_image, REAL bg_att, int truncate, int do_rotate)
{
    int nx = size[0], ny = size[1], nz = size[2];
    size_t nvox = (size_t)nx * ny * nz, nxy = (size_t)nx * ny;
    if (!act && !att) return ORC_ERR_PARAMETERS;
    REAL *ract = act ? (REAL *)malloc(sizeof(REAL) * nvox) : NULL;
    REAL *ratt = att ? (REAL *)malloc(sizeof(REAL) * nvox) : NULL;
    REAL *rpart = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *sep = NULL;
    if (psf) {
        sep = (REAL *)malloc(sizeof(REAL) * (size_t)(psf_size[0] + psf_size[1]) * psf_size[2]);
        ORC(psf_separate)(psf, psf_size[0], psf_size[1], psf_size[2], sep);
    }
    REAL A[16];
    for (int cam = 0; cam < ncam; cam++) {
        ORC(rotation_matrix)(A, angles[cam], angles[ncam + cam], angles[2 * ncam + cam],
                             centers[cam], centers[ncam + cam], centers[2 * ncam + cam], 0);
        if (act) ORC(affine_resample)(act, ract, nx, ny, nz, A, bg);
        if (att) ORC(affine_resample)(att, ratt, nx, ny, nz, A, bg_att);
        if (psf && act) ORC(convolve_separable)(ract, nx, ny, nz, sep, psf_size[0], psf_size[1]);
        REAL *dst = partial + nvox * cam;
        line_partial(ract, ratt, bg_image, sino + nxy * cam, do_rotate ? rpart : dst, nx, ny, nz, bg);
        if (do_rotate) {
            ORC(rotation_matrix)(A, -angles[cam], -angles[ncam + cam], -angles[2 * ncam + cam],
                                 centers[cam], centers[ncam + cam], centers[2 * ncam + cam], 5);
            ORC(affine_resample)(rpart, dst, nx, ny, nz, A, bg);
        }
    }
    if (truncate)
        for (size_t i = 0; i < nxy * ncam; i++)
            if (sino[i] < 0) sino[i] = 0;
    free(ract);
    free(ratt);
    free(rpart);
    free(sep);
    return ORC_OK;
}

/* et_array_project_partial, emission-lib/_et_array_interface.cpp:1561-1760:
 * argument rules of SPECT_project_parallelholes; bg_image [nx, ny] or NULL. */
int ORC(spect_project_partial)(const REAL *act, const int act_size[3], REAL *sino, REAL *partial,
                               const REAL *cameras, const int cam_size[2], const REAL *psf, const int psf_size[3],
                               const REAL *att, const int att_size[3], REAL bg, const REAL *bg_image, REAL bg_att,
                               int truncate, int do_rotate)
{
    int asz[3] = {act_size[0], act_size[1], act_size[2]};
    int no_act = (asz[0] == 0 && asz[1] == 0 && asz[2] == 0);
    int no_psf = (psf_size[0] == 0 && psf_size[1] == 0 && psf_size[2] == 0);
    int no_att = (att_size[0] == 0 && att_size[1] == 0 && att_size[2] == 0);
    if (no_act) { asz[0] = att_size[0]; asz[1] = att_size[1]; asz[2] = att_size[2]; }
    if (no_act && no_att) return ORC_ERR_PARAMETERS;
    int ncam = cam_size[0], ncols = cam_size[1];
    if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != asz[0])) return ORC_ERR_PARAMETERS;
    REAL *angles = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    REAL *centers = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    int st = expand_cameras(cameras, ncam, ncols, asz, angles, centers);
    if (st == ORC_OK)
        st = ORC(project_partial)(no_act ? NULL : act, no_att ? NULL : att, asz, sino, partial, angles, centers, ncam,
                                  no_psf ? NULL : psf, psf_size, bg, bg_image, bg_att, truncate, do_rotate);
    free(angles);
    free(centers);
    return st;
}

/* Fisher information of a grid of voxels, et_fisher_grid
 * (emission-lib/_et.cpp:531-746).  grid: volume [nx, ny, nz] holding 1..n at
 * the grid points, 0 elsewhere (scanned x outer, z inner, :580-598).  proj:
 * the projection [npx, npy, ncam] (the "inverse sinogram" of the reference,
 * whose inversion is commented out at :572-574, so it is the projection
 * itself).  Per camera the grid points are rotated (XYZ, +theta, about the
 * camera centre, reg_mat44_mul order, truncated to integers :619-623); for
 * every pair i <= j whose PSFs (plane = rotated depth) overlap, the products
 * of the two shifted PSFs times the projection are summed over the overlap
 * box (:626-700).  prior (optional): 1 where two points are 26-neighbours
 * (:703-721).  Both matrices symmetric [n, n].  Returns 2 for a malformed grid. */
int ORC(fisher_grid)(const REAL *proj, int npx, int npy, const REAL *grid, const int size[3], REAL *fisher,
                     REAL *prior, int n, const REAL *psf, int kx, int ky, const REAL *angles, const REAL *centers,
                     int ncam)
{
    int nx = size[0], ny = size[1], nz = size[2];
    int semi_x = (kx - 1) / 2, semi_y = (ky - 1) / 2;
    int *gc = (int *)malloc(sizeof(int) * 3 * (size_t)n);
    int *gr = (int *)malloc(sizeof(int) * 3 * (size_t)n);
    for (int i = 0; i < 3 * n; i++) gc[i] = -1;
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++)
            for (int z = 0; z < nz; z++) {
                REAL g = grid[(size_t)z * ny * nx + (size_t)y * nx + x];
                if (g != 0) {
                    int k = (int)g - 1;
                    if (k < 0 || k >= n || gc[3 * k] != -1) {
                        free(gc);
                        free(gr);
                        return ORC_ERR_PARAMETERS;
                    }
                    gc[3 * k] = x;
                    gc[3 * k + 1] = y;
                    gc[3 * k + 2] = z;
                }
            }
    for (size_t i = 0; i < (size_t)n * n; i++) fisher[i] = 0;
    if (prior)
        for (size_t i = 0; i < (size_t)n * n; i++) prior[i] = 0;
    REAL A[16];
    for (int cam = 0; cam < ncam; cam++) {
        const REAL *plane = proj + (size_t)npx * npy * cam;
        ORC(rotation_matrix)(A, angles[cam], angles[ncam + cam], angles[2 * ncam + cam],
                             centers[cam], centers[ncam + cam], centers[2 * ncam + cam], 0);
        for (int k = 0; k < n; k++) {
            REAL p0 = (REAL)gc[3 * k], p1 = (REAL)gc[3 * k + 1], p2 = (REAL)gc[3 * k + 2];
            for (int r = 0; r < 3; r++)
                gr[3 * k + r] = (int)(A[4 * r] * p0 + A[4 * r + 1] * p1 + A[4 * r + 2] * p2 + A[4 * r + 3]);
        }
        for (int i = 0; i < n; i++) {
            int ix = gr[3 * i], iy = gr[3 * i + 1], iz = gr[3 * i + 2];
            for (int j = i; j < n; j++) {
                int jx = gr[3 * j], jy = gr[3 * j + 1], jz = gr[3 * j + 2];
                int bx = kx - abs(jx - ix), by = ky - abs(jy - iy);
                int px = (ix > jx ? ix : jx) - semi_x, py = (iy > jy ? iy : jy) - semi_y;
                if (!(bx > 0 && by > 0 && iz >= 0 && jz >= 0 && iz < nz && jz < nz)) continue;
                int pix, piy, pjx, pjy;
                if (jx >= ix && jy > iy) { pix = jx - ix; piy = jy - iy; pjx = 0; pjy = 0; }
                else if (jx < ix && jy >= iy) { pix = 0; piy = jy - iy; pjx = ix - jx; pjy = 0; }
                else if (jx <= ix && jy < iy) { pix = 0; piy = 0; pjx = ix - jx; pjy = iy - jy; }
                else { pix = jx - ix; piy = 0; pjx = 0; pjy = iy - jy; }
                const REAL *Pi = psf + (size_t)iz * kx * ky, *Pj = psf + (size_t)jz * kx * ky;
                REAL f = fisher[(size_t)i * n + j];
                for (int x = 0; x < bx; x++)
                    for (int y = 0; y < by; y++) {
                        int qx = px + x, qy = py + y;
                        if (qx >= 0 && qy >= 0 && qx < npx && qy < npy)
                            f = f + Pj[(pjy + y) * kx + (pjx + x)] * Pi[(piy + y) * kx + (pix + x)] * plane[qy * npx + qx];
                    }
                fisher[(size_t)i * n + j] = f;
            }
        }
    }
    if (prior)
        for (int i = 0; i < n; i++)
            for (int j = i; j < n; j++)
                if (abs(gc[3 * i] - gc[3 * j]) <= 1 && abs(gc[3 * i + 1] - gc[3 * j + 1]) <= 1 &&
                    abs(gc[3 * i + 2] - gc[3 * j + 2]) <= 1)
                    prior[(size_t)i * n + j] = 1;
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            fisher[(size_t)j * n + i] = fisher[(size_t)i * n + j];
            if (prior) prior[(size_t)j * n + i] = prior[(size_t)i * n + j];
        }
    free(gc);
    free(gr);
    return ORC_OK;
}

/* et_array_fisher_grid (emission-lib/_et_array_interface.cpp:1135-1340):
 * project the activity (truncated, :557) and accumulate the Fisher matrix of
 * the grid; the projection planes are [nx, ny] (the reference sizes them
 * [nx, nz], equal for its cubic volumes). */
int ORC(spect_fisher_grid)(const REAL *act, const int act_size[3], const REAL *cameras, const int cam_size[2],
                           const REAL *psf, const int psf_size[3], const REAL *grid, REAL *fisher, REAL *prior, int n,
                           const REAL *att, const int att_size[3], REAL bg, REAL bg_att)
{
    int ncam = cam_size[0], ncols = cam_size[1];
    int no_att = (att_size[0] == 0 && att_size[1] == 0 && att_size[2] == 0);
    if (!psf || psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != act_size[0]) return ORC_ERR_PARAMETERS;
    REAL *angles = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    REAL *centers = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    REAL *proj = (REAL *)malloc(sizeof(REAL) * (size_t)act_size[0] * act_size[1] * ncam);
    int st = expand_cameras(cameras, ncam, ncols, act_size, angles, centers);
    if (st == ORC_OK)
        st = ORC(project)(act, no_att ? NULL : att, act_size, proj, angles, centers, ncam, psf, psf_size, bg, bg_att, 1);
    if (st == ORC_OK)
        st = ORC(fisher_grid)(proj, act_size[0], act_size[1], grid, act_size, fisher, prior, n, psf, psf_size[0],
                              psf_size[1], angles, centers, ncam);
    free(angles);
    free(centers);
    free(proj);
    return st;
}

/* SPECT_backproject_parallelholes, emission-lib/_et_array_interface.cpp:547-710:
 * the centre comes from (sino0, sino1, sino0), the volume grid from bkpr_size.
 * The exact adjoint (not in the reference) is the transpose of the projector
 * and takes the projector's centre, from (sino0, sino1, bkpr2). */
int ORC(spect_backproject)(const REAL *sino, const int sino_size[3], REAL *bkpr, const int bkpr_size[3],
                           const REAL *cameras, const int cam_size[2], const REAL *psf, const int psf_size[3],
                           const REAL *att, const int att_size[3], REAL bg, REAL bg_att, int truncate, int adjoint)
{
    int no_psf = (psf_size[0] == 0 && psf_size[1] == 0 && psf_size[2] == 0);
    int no_att = (att_size[0] == 0 && att_size[1] == 0 && att_size[2] == 0);
    int ncam = cam_size[0], ncols = cam_size[1];
    if (sino_size[2] != ncam) return ORC_ERR_PARAMETERS;
    if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != sino_size[0])) return ORC_ERR_PARAMETERS;
    int csz[3] = {sino_size[0], sino_size[1], adjoint ? bkpr_size[2] : sino_size[0]};
    REAL *angles = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    REAL *centers = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    int st = expand_cameras(cameras, ncam, ncols, csz, angles, centers);
    if (st == ORC_OK)
        st = ORC(backproject)(sino, no_att ? NULL : att, bkpr_size, bkpr, angles, centers, ncam,
                              no_psf ? NULL : psf, psf_size, bg, bg_att, truncate, adjoint);
    free(angles);
    free(centers);
    return st;
}

/* et_array_gradient_attenuation, emission-lib/_et_array_interface.cpp:714-892
 * (3-D sinograms): centres from activity_size, grids from gradient_size. */
int ORC(spect_gradient_attenuation)(const REAL *sino, const int sino_size[3], const REAL *act, const int act_size[3],
                                    REAL *grad, const int grad_size[3], const REAL *cameras, const int cam_size[2],
                                    const REAL *psf, const int psf_size[3], const REAL *att, REAL bg, REAL bg_att,
                                    int truncate)
{
    int no_psf = (psf_size[0] == 0 && psf_size[1] == 0 && psf_size[2] == 0);
    int ncam = cam_size[0], ncols = cam_size[1];
    if (sino_size[2] != ncam) return ORC_ERR_PARAMETERS;
    if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != sino_size[0])) return ORC_ERR_PARAMETERS;
    REAL *angles = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    REAL *centers = (REAL *)malloc(sizeof(REAL) * 3 * ncam);
    int st = expand_cameras(cameras, ncam, ncols, act_size, angles, centers);
    if (st == ORC_OK)
        st = ORC(gradient_attenuation)(sino, act, att, grad_size, grad, angles, centers, ncam,
                                       no_psf ? NULL : psf, psf_size, bg, bg_att, truncate);
    free(angles);
    free(centers);
    return st;
}

/* One OSEM step over an explicit camera subset, following
 * et_array_osem_step (emission-lib/_et_array_interface.cpp:972-1054) with the
 * random draw (:1001-1009) replaced by the given indexes; with all cameras it
 * is et_array_mlem_step (:1080-1131).  Volume [nx, ny, nx]; cameras [3 x n]
 * (axis-major); psf [kx, ky, nx] or NULL; att or NULL. */
int ORC(osem_step_subset)(REAL *act, int nx, int ny, const REAL *sino, int ncam, const REAL *cameras,
                          const int *idx, int nsub, const REAL *att, const REAL *psf, int kx, int ky,
                          REAL bg, REAL bg_att, REAL eps)
{
    int vsz[3] = {nx, ny, nx};
    size_t nvox = (size_t)nx * ny * nx, nxy = (size_t)nx * ny;
    int psz[3] = {kx, ky, nx};
    REAL *angles = (REAL *)malloc(sizeof(REAL) * 3 * nsub);
    REAL *centers = (REAL *)malloc(sizeof(REAL) * 3 * nsub);
    REAL *ysub = (REAL *)malloc(sizeof(REAL) * nxy * nsub);
    REAL *proj = (REAL *)malloc(sizeof(REAL) * nxy * nsub);
    REAL *ones = (REAL *)malloc(sizeof(REAL) * nxy * nsub);
    REAL *num = (REAL *)malloc(sizeof(REAL) * nvox);
    REAL *den = (REAL *)malloc(sizeof(REAL) * nvox);
    for (int c = 0; c < nsub; c++) {
        for (int a = 0; a < 3; a++) {
            angles[a * nsub + c] = cameras[idx[c] + a * ncam];
            centers[a * nsub + c] = (REAL)((vsz[a] - 1) / 2.0);
        }
        memcpy(ysub + nxy * c, sino + nxy * idx[c], sizeof(REAL) * nxy);
    }
    for (size_t i = 0; i < nxy * nsub; i++) ones[i] = 1;
    ORC(project)(act, att, vsz, proj, angles, centers, nsub, psf, psz, bg, bg_att, 1);
    for (size_t i = 0; i < nxy * nsub; i++)
        proj[i] = (proj[i] < eps) ? ysub[i] / eps : ysub[i] / proj[i];
    ORC(backproject)(proj, att, vsz, num, angles, centers, nsub, psf, psz, bg, bg_att, 1, 0);
    ORC(backproject)(ones, att, vsz, den, angles, centers, nsub, psf, psz, bg, bg_att, 1, 0);
    for (size_t i = 0; i < nvox; i++)
        if (den[i] < eps) den[i] = eps;
    for (size_t i = 0; i < nvox; i++) act[i] *= num[i] / den[i];
    free(angles);
    free(centers);
    free(ysub);
    free(proj);
    free(ones);
    free(num);
    free(den);
    return ORC_OK;
}

/* et_array_make_cameras, emission-lib/_et_array_interface.cpp:923-937:
 * angle_k = (first + (last-first)*k/(n-1)) / 180 * pi on rotation_axis,
 * layout [3 x n] axis-major. */
void ORC(make_cameras)(REAL *cams, REAL first_deg, REAL last_deg, int n, int axis)
{
    for (int c = 0; c < n; c++) {
        REAL angle = (REAL)((first_deg + (last_deg - first_deg) * c / (n - 1)) / (REAL)180.0 * (REAL)3.141592653589793);
        for (int a = 0; a < 3; a++) cams[c + a * n] = (a == axis) ? angle : (REAL)0;
    }
}

/* et_array_convolve, emission-lib/_et_array_interface.cpp:161-226 (per-slice
 * FFT convolution on the reference's GPU path, emission-lib_gpu/
 * _et_convolveFFT2D_gpu.cu:43-113; its CPU path is a stub, _et.cpp:776-780):
 * restated as the direct sum the FFT computes -- per slice z, a true 2D
 * convolution with kernel slice z, kernel centre ((kx-1)/2, (ky-1)/2), the
 * image clamped to its border outside (padDataClampToBorder).  Nifti order,
 * x fastest; kernel [kx][ky][nz] with kx fastest.  Terms in (j, i) order. */
void ORC(convolve2d)(const REAL *img, REAL *out, int nx, int ny, int nz, const REAL *psf, int kx, int ky)
{
    int cx = (kx - 1) / 2, cy = (ky - 1) / 2;
    for (int z = 0; z < nz; z++) {
        const REAL *k = psf + (size_t)z * kx * ky;
        const REAL *src = img + (size_t)z * nx * ny;
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                REAL acc = 0;
                for (int j = 0; j < ky; j++) {
                    int yy = y + cy - j;
                    yy = yy < 0 ? 0 : (yy >= ny ? ny - 1 : yy);
                    for (int i = 0; i < kx; i++) {
                        int xx = x + cx - i;
                        xx = xx < 0 ? 0 : (xx >= nx ? nx - 1 : xx);
                        REAL t = k[i + (size_t)kx * j] * src[xx + (size_t)nx * yy];
                        acc = acc + t;
                    }
                }
                out[x + (size_t)nx * (y + (size_t)ny * z)] = acc;
            }
    }
}
