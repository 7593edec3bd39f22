// General-orientation path: cameras with any (theta_x, theta_y, theta_z),
// any background values, any grid.  Volumes in nifti layout.  Each stage is a
// separate kernel following the reference's float operation order (products
// and sums rounded separately), so this path reproduces the reference CPU
// path up to the last bit of expf.  The fused kernels of et_yg_*.cu cover
// the common gantry case; this path covers everything else.
#include "et_kernels.h"
#include "et_profile.h"

namespace nrgb {

namespace {

template <class T>
struct Affine34T {
  T m[12];
};
using Affine34 = Affine34T<float>;

// Separately rounded arithmetic in the working type (float: the reference's
// type; double: the float64 reference path).
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double fm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double fa(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double fs(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float flo(float v) { return floorf(v); }
__device__ __forceinline__ double flo(double v) { return floor(v); }
__device__ __forceinline__ float ex(float v) { return expf(v); }
__device__ __forceinline__ double ex(double v) { return exp(v); }

// Trilinear resampling of one voxel, reg-lib/_reg_resampling.cpp:334-450
// (positions from reg-lib/_reg_affineTransformation.cpp:116-132 with an
// identity voxel-to-world matrix).  With bg != 0 every neighbour outside the
// grid adds bg * xBasis[.] to a separate background weight, as the reference
// does (:366-396).
template <class T>
__device__ __forceinline__ T trilinear_ref(const T* __restrict__ src, int nx, int ny, int nz, const Affine34T<T>& A,
                                           int x, int y, int z, T bg) {
  const T fx = static_cast<T>(x), fy = static_cast<T>(y), fz = static_cast<T>(z);
  T pos[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    pos[i] = fa(fa(fa(fm(A.m[4 * i + 0], fx), fm(A.m[4 * i + 1], fy)), fm(A.m[4 * i + 2], fz)), A.m[4 * i + 3]);
  int prev[3];
  T b0[3], b1[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    prev[i] = static_cast<int>(flo(pos[i]));
    T rel = fs(pos[i], static_cast<T>(prev[i]));
    if (rel < T(0)) rel = T(0);
    b0[i] = fs(T(1), rel);
    b1[i] = rel;
  }
  const T bx[2] = {b0[0], b1[0]};
  const T by[2] = {b0[1], b1[1]};
  const T bz[2] = {b0[2], b1[2]};
  T val = T(0), bgw = T(0);
  const bool use_bg = (bg != T(0));
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int Z = prev[2] + c;
    if (Z >= 0 && Z < nz) {
      T ysum = T(0);
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const int Y = prev[1] + b;
        if (Y >= 0 && Y < ny) {
          const T* row = src + (static_cast<size_t>(Z) * ny + Y) * nx;
          T xsum = T(0);
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            const int X = prev[0] + a;
            if (X >= 0 && X < nx)
              xsum = fa(xsum, fm(__ldg(row + X), bx[a]));
            else if (use_bg)
              bgw = fa(bgw, fm(bg, bx[a]));
          }
          ysum = fa(ysum, fm(xsum, by[b]));
        } else if (use_bg) {
          bgw = fa(bgw, fm(bg, bx[b]));
        }
      }
      val = fa(val, fm(ysum, bz[c]));
    } else if (use_bg) {
      bgw = fa(bgw, fm(bg, bx[c]));
    }
  }
  if (use_bg) val = fa(val, bgw);
  return val;
}

template <bool ACCUM, class T = float>
__global__ void k_resample(const T* __restrict__ src, T* __restrict__ dst, int nx, int ny, int nz, Affine34T<T> A,
                           T bg) {
  const size_t nvox = static_cast<size_t>(nx) * ny * nz;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < nvox;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % nx);
    const int y = static_cast<int>((i / nx) % ny);
    const int z = static_cast<int>(i / (static_cast<size_t>(nx) * ny));
    const T v = trilinear_ref<T>(src, nx, ny, nz, A, x, y, z, bg);
    if (ACCUM)
      dst[i] = fa(dst[i], v);
    else
      dst[i] = v;
  }
}

// Transpose of trilinear_ref with bg = 0: add v * weight to each in-grid
// corner of the footprint of (x, y, z) (atomics: footprints overlap).
__device__ __forceinline__ void trilinear_scatter(float* __restrict__ dst, int nx, int ny, int nz, const Affine34& A,
                                                  int x, int y, int z, float v) {
  const float fx = static_cast<float>(x), fy = static_cast<float>(y), fz = static_cast<float>(z);
  int prev[3];
  float b0[3], b1[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float pos =
        fa(fa(fa(fm(A.m[4 * i + 0], fx), fm(A.m[4 * i + 1], fy)), fm(A.m[4 * i + 2], fz)), A.m[4 * i + 3]);
    prev[i] = static_cast<int>(floorf(pos));
    float rel = __fsub_rn(pos, static_cast<float>(prev[i]));
    if (rel < 0.0f) rel = 0.0f;
    b0[i] = __fsub_rn(1.0f, rel);
    b1[i] = rel;
  }
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const int Z = prev[2] + c;
    if (Z < 0 || Z >= nz) continue;
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int Y = prev[1] + b;
      if (Y < 0 || Y >= ny) continue;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        const int X = prev[0] + a;
        if (X < 0 || X >= nx) continue;
        const float w = (a ? b1[0] : b0[0]) * (b ? b1[1] : b0[1]) * (c ? b1[2] : b0[2]);
        if (w != 0.0f) atomicAdd(dst + (static_cast<size_t>(Z) * ny + Y) * nx + X, v * w);
      }
    }
  }
}

__global__ void k_scatter(const float* __restrict__ src, float* __restrict__ dst, int nx, int ny, int nz, Affine34 A) {
  const size_t nvox = static_cast<size_t>(nx) * ny * nz;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < nvox;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const float v = src[i];
    if (v == 0.0f) continue;
    const int x = static_cast<int>(i % nx);
    const int y = static_cast<int>((i / nx) % ny);
    const int z = static_cast<int>(i / (static_cast<size_t>(nx) * ny));
    trilinear_scatter(dst, nx, ny, nz, A, x, y, z, v);
  }
}

// Row (x) then column (y) pass of emission-lib/_et_convolveSeparable2D.cpp:13-40:
// true convolution (kernel index R-k), zero outside the plane, plane z uses
// kernel plane z.  sep layout [plane][row k | column k].  FLIP: correlation
// (kernel index R+k), the transpose of the convolution.
template <bool ROWS, bool FLIP = false, class T = float>
__global__ void k_conv(const T* __restrict__ in, T* __restrict__ out, int nx, int ny, int nz, const T* __restrict__ sep,
                       int k) {
  const size_t nvox = static_cast<size_t>(nx) * ny * nz;
  const int R = (k - 1) / 2;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < nvox;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int x = static_cast<int>(i % nx);
    const int y = static_cast<int>((i / nx) % ny);
    const int z = static_cast<int>(i / (static_cast<size_t>(nx) * ny));
    const T* K = sep + static_cast<size_t>(2 * k) * z + (ROWS ? 0 : k);
    T s = T(0);
    for (int kk = -R; kk <= R; ++kk) {
      if (ROWS) {
        const int d = x + kk;
        if (d >= 0 && d < nx) s = fa(s, fm(__ldg(in + i + kk), __ldg(K + (FLIP ? R + kk : R - kk))));
      } else {
        const int d = y + kk;
        if (d >= 0 && d < ny)
          s = fa(s, fm(__ldg(in + i + static_cast<ptrdiff_t>(kk) * nx), __ldg(K + (FLIP ? R + kk : R - kk))));
      }
    }
    out[i] = s;
  }
}

// Attenuated line integral along z, emission-lib/_et_line_integral_attenuated.cpp:14-68.
template <class R = float>
__global__ void k_line_integral(const R* __restrict__ act, const R* __restrict__ att, R* __restrict__ out, int nx,
                                int ny, int nz, R bg) {
  const int nxy = nx * ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nxy) return;
  R p = R(0), T = R(0);
  if (act && att) {
    for (int z = 0; z < nz; ++z) {
      T = fa(T, __ldg(att + static_cast<size_t>(z) * nxy + i));
      p = fa(p, fm(__ldg(act + static_cast<size_t>(z) * nxy + i), ex(-T)));
    }
    p = fa(p, fm(bg, ex(-T)));
  } else if (act) {
    for (int z = 0; z < nz; ++z) p = fa(p, __ldg(act + static_cast<size_t>(z) * nxy + i));
    p = fa(p, bg);
  } else {
    for (int z = 0; z < nz; ++z) T = fa(T, __ldg(att + static_cast<size_t>(z) * nxy + i));
    p = fm(bg, ex(-T));
  }
  out[i] = p;
}

// Spread along z, emission-lib/_et_line_backproject_attenuated.cpp:17-36 and
// emission-lib/_et_line_backproject.cpp:17-30.
template <class R = float>
__global__ void k_spread(const R* __restrict__ plane, const R* __restrict__ att, R* __restrict__ vol, int nx, int ny,
                         int nz) {
  const int nxy = nx * ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nxy) return;
  const R s = __ldg(plane + i);
  R T = R(0);
  for (int z = 0; z < nz; ++z) {
    const size_t j = static_cast<size_t>(z) * nxy + i;
    if (att) {
      T = fa(T, __ldg(att + j));
      vol[j] = fm(s, ex(-T));
    } else {
      vol[j] = s;
    }
  }
}

// Partial-sum line integral, the partial-sum branch of
// emission-lib_gpu/_et_line_integral_attenuated_gpu_kernels.cu:57-103: walk
// depth from the far end, partial[z] = s before voxel z is added and
// attenuated; s starts at bg (times bg_image[x, y]); the projection is the
// final s.
__global__ void k_line_partial(const float* __restrict__ act, const float* __restrict__ att,
                               const float* __restrict__ bg_image, float* __restrict__ out,
                               float* __restrict__ partial, int nx, int ny, int nz, float bg) {
  const int nxy = nx * ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nxy) return;
  float s = bg;
  if (bg_image) s = fm(s, __ldg(bg_image + i));
  for (int z = nz - 1; z >= 0; --z) {
    const size_t j = static_cast<size_t>(z) * nxy + i;
    partial[j] = s;
    if (act && att)
      s = fm(fa(s, __ldg(act + j)), expf(-__ldg(att + j)));
    else if (att)
      s = fm(s, expf(-__ldg(att + j)));
    else
      s = fa(s, __ldg(act + j));
  }
  out[i] = s;
}

template <class R>
__global__ void k_truncate_t(R* __restrict__ buf, size_t n) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    if (buf[i] < R(0)) buf[i] = R(0);
}

// Attenuation-gradient scan, emission-lib_gpu/_et_attenuation_gradient_gpu_kernels.cu:24-39:
// pass 1 stores the inclusive prefix T_z, pass 2 (far to near) accumulates
// a_z * exp(-T_z) and stores s * acc.
__global__ void k_grad_scan(const float* __restrict__ act, const float* __restrict__ att,
                            const float* __restrict__ plane, float* __restrict__ vol, int nx, int ny, int nz) {
  const int nxy = nx * ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nxy) return;
  float T = 0.0f;
  for (int z = 0; z < nz; ++z) {
    const size_t j = static_cast<size_t>(z) * nxy + i;
    T = fa(T, __ldg(att + j));
    vol[j] = T;
  }
  const float s = __ldg(plane + i);
  float acc = 0.0f;
  for (int z = nz - 1; z >= 0; --z) {
    const size_t j = static_cast<size_t>(z) * nxy + i;
    acc = fa(acc, fm(__ldg(act + j), expf(-vol[j])));
    vol[j] = fm(s, acc);
  }
}

// Gradient of a projection plane with respect to the rotated mu.  With
// p = sum_z v_z exp(-T_z) + bg exp(-T_N) (v: PSF-convolved rotated activity,
// T inclusive prefix of the rotated mu m), dp/dm_z' = -(S_z' + bg exp(-T_N)),
// S_z' = sum_{z >= z'} v_z exp(-T_z) = P_v - (prefix of v exp(-T) before z').
// out[z'] = g * dp/dm_z'.  Not in the reference (whose gradient,
// emission-lib_gpu/_et_attenuation_gradient_gpu_kernels.cu:15-42, ignores the
// PSF coupling, the sign and the background).
__global__ void k_dmu_scan(const float* __restrict__ v, const float* __restrict__ m, const float* __restrict__ g_plane,
                           float* __restrict__ out, int nx, int ny, int nz, float bg) {
  const int nxy = nx * ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nxy) return;
  float T = 0.0f, Pv = 0.0f;
  for (int z = 0; z < nz; ++z) {
    const size_t j = static_cast<size_t>(z) * nxy + i;
    T += __ldg(m + j);
    Pv = fmaf(__ldg(v + j), __expf(-T), Pv);
  }
  const float tail = bg * __expf(-T);
  const float g = __ldg(g_plane + i);
  float prefix = 0.0f;
  T = 0.0f;
  for (int z = 0; z < nz; ++z) {
    const size_t j = static_cast<size_t>(z) * nxy + i;
    T += __ldg(m + j);
    const float e = __expf(-T);
    out[j] = -g * ((Pv - prefix) + tail);
    prefix = fmaf(__ldg(v + j), e, prefix);
  }
}

int grid_for(size_t n, int block) {
  const size_t g = (n + block - 1) / block;
  const int cap = sm_count() * 64;
  return static_cast<int>(g < cap ? g : cap);
}

template <class T>
Affine34T<T> affine_of(const T* m12) {
  Affine34T<T> a;
  for (int i = 0; i < 12; ++i) a.m[i] = m12[i];
  return a;
}

template <class T>
void launch_truncate_t(T* buf, size_t n, cudaStream_t st) {
  NRGB_LAUNCH_SCOPE("k_truncate", st);
  k_truncate_t<T><<<grid_for(n, 256), 256, 0, st>>>(buf, n);
}

// et_project (emission-lib/_et.cpp:218-281): per camera rotate activity and
// mu, PSF, attenuated line integral; truncation at the end (:283-292).
template <class T>
int general_project_t(const GeneralArgsT<T>& a, cudaStream_t st) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nxy = static_cast<size_t>(nx) * ny;
  const int B = 256;
  for (int cam = 0; cam < a.ncam; ++cam) {
    const Affine34T<T> F = affine_of<T>(a.geom_host[cam].fwd);
    if (a.act) { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false, T><<<grid_for(nvox, B), B, 0, st>>>(a.act, a.ws_act, nx, ny, nz, F, a.bg); }
    if (a.att) { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false, T><<<grid_for(nvox, B), B, 0, st>>>(a.att, a.ws_att, nx, ny, nz, F, a.bg_att); }
    if (a.psf_sep && a.act) {
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<true, false, T><<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.ws_tmp, nx, ny, nz, a.psf_sep, a.psf_k); }
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<false, false, T><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.ws_act, nx, ny, nz, a.psf_sep, a.psf_k); }
    }
    { NRGB_LAUNCH_SCOPE("k_line_integral", st); k_line_integral<T><<<static_cast<int>((nxy + B - 1) / B), B, 0, st>>>(a.act ? a.ws_act : nullptr,
                                                                      a.att ? a.ws_att : nullptr,
                                                                      a.out + nxy * cam, nx, ny, nz, a.bg); }
  }
  if (a.truncate) launch_truncate_t<T>(a.out, nxy * a.ncam, st);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

// et_backproject (emission-lib/_et.cpp:415-499): per camera rotate mu, spread
// the attenuated plane, PSF, rotate back with the inverse matrix, accumulate.
template <class T>
int general_backproject_t(const GeneralArgsT<T>& a, cudaStream_t st) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nxy = static_cast<size_t>(nx) * ny;
  const int B = 256;
  cudaMemsetAsync(a.out, 0, nvox * sizeof(T), st);
  for (int cam = 0; cam < a.ncam; ++cam) {
    const Affine34T<T> F = affine_of<T>(a.geom_host[cam].fwd);
    const Affine34T<T> Bk = affine_of<T>(a.geom_host[cam].bwd);
    if (a.att) { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false, T><<<grid_for(nvox, B), B, 0, st>>>(a.att, a.ws_att, nx, ny, nz, F, a.bg_att); }
    { NRGB_LAUNCH_SCOPE("k_spread", st); k_spread<T><<<static_cast<int>((nxy + B - 1) / B), B, 0, st>>>(a.sino + nxy * cam, a.att ? a.ws_att : nullptr,
                                                               a.ws_act, nx, ny, nz); }
    if (a.psf_sep) {
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<true, false, T><<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.ws_tmp, nx, ny, nz, a.psf_sep, a.psf_k); }
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<false, false, T><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.ws_act, nx, ny, nz, a.psf_sep, a.psf_k); }
    }
    { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<true, T><<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.out, nx, ny, nz, Bk, a.bg); }
  }
  if (a.truncate) launch_truncate_t<T>(a.out, nvox, st);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

}  // namespace

// et_project_partial_gpu (emission-lib/_et.cpp:2106-2436): per camera rotate
// activity (bg) and mu (bg_att), PSF, partial-sum line integral; with
// do_rotate the camera's partial-sum volume is rotated back to the image frame
// (-theta, ZYX, background bg, :2373-2404).  partial: [ncam][nz][ny][nx].
int general_project_partial(const GeneralArgs& a, const float* bg_image, float* partial, int do_rotate,
                            cudaStream_t st) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nxy = static_cast<size_t>(nx) * ny;
  const int B = 256;
  for (int cam = 0; cam < a.ncam; ++cam) {
    const Affine34 F = affine_of(a.geom_host[cam].fwd);
    if (a.act) { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.act, a.ws_act, nx, ny, nz, F, a.bg); }
    if (a.att) { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.att, a.ws_att, nx, ny, nz, F, a.bg_att); }
    if (a.psf_sep && a.act) {
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<true><<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.ws_tmp, nx, ny, nz, a.psf_sep, a.psf_k); }
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<false><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.ws_act, nx, ny, nz, a.psf_sep, a.psf_k); }
    }
    float* dst = partial + nvox * cam;
    {
      NRGB_LAUNCH_SCOPE("k_line_partial", st);
      k_line_partial<<<static_cast<int>((nxy + B - 1) / B), B, 0, st>>>(
          a.act ? a.ws_act : nullptr, a.att ? a.ws_att : nullptr, bg_image, a.out + nxy * cam,
          do_rotate ? a.ws_tmp : dst, nx, ny, nz, a.bg);
    }
    if (do_rotate) {
      NRGB_LAUNCH_SCOPE("k_resample", st);
      k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, dst, nx, ny, nz, affine_of(a.geom_host[cam].bwd),
                                                          a.bg);
    }
  }
  if (a.truncate) launch_truncate_t<float>(a.out, nxy * a.ncam, st);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int general_project(const GeneralArgs& a, cudaStream_t st) { return general_project_t<float>(a, st); }
int general_backproject(const GeneralArgs& a, cudaStream_t st) { return general_backproject_t<float>(a, st); }
int general_project64(const GeneralArgs64& a, cudaStream_t st) { return general_project_t<double>(a, st); }
int general_backproject64(const GeneralArgs64& a, cudaStream_t st) { return general_backproject_t<double>(a, st); }

// Exact transpose of general_project for fixed mu (bg terms dropped: the
// transpose of the projector's linear part): spread, transposed PSF
// (correlation, column pass first), transposed trilinear scatter.
int general_adjoint(const GeneralArgs& a, cudaStream_t st) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nxy = static_cast<size_t>(nx) * ny;
  const int B = 256;
  cudaMemsetAsync(a.out, 0, nvox * sizeof(float), st);
  for (int cam = 0; cam < a.ncam; ++cam) {
    const Affine34 F = affine_of(a.geom_host[cam].fwd);
    if (a.att) { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.att, a.ws_att, nx, ny, nz, F, a.bg_att); }
    { NRGB_LAUNCH_SCOPE("k_spread", st); k_spread<<<static_cast<int>((nxy + B - 1) / B), B, 0, st>>>(a.sino + nxy * cam, a.att ? a.ws_att : nullptr,
                                                               a.ws_act, nx, ny, nz); }
    if (a.psf_sep) {
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<false, true><<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.ws_tmp, nx, ny, nz, a.psf_sep, a.psf_k); }
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<true, true><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.ws_act, nx, ny, nz, a.psf_sep, a.psf_k); }
    }
    { NRGB_LAUNCH_SCOPE("k_scatter", st); k_scatter<<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.out, nx, ny, nz, F); }
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

// Gradient of sum(g * project(act, mu)) with respect to mu (a.sino = g),
// into a.out.  Per camera: rotate activity and mu, PSF on the activity,
// k_dmu_scan, transposed trilinear scatter of the rotated-frame gradient.
int general_dmu(const GeneralArgs& a, cudaStream_t st) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nxy = static_cast<size_t>(nx) * ny;
  const int B = 256;
  cudaMemsetAsync(a.out, 0, nvox * sizeof(float), st);
  for (int cam = 0; cam < a.ncam; ++cam) {
    const Affine34 F = affine_of(a.geom_host[cam].fwd);
    { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.act, a.ws_act, nx, ny, nz, F, a.bg); }
    { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.att, a.ws_att, nx, ny, nz, F, a.bg_att); }
    if (a.psf_sep) {
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<true><<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.ws_tmp, nx, ny, nz, a.psf_sep, a.psf_k); }
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<false><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.ws_act, nx, ny, nz, a.psf_sep, a.psf_k); }
    }
    { NRGB_LAUNCH_SCOPE("k_dmu_scan", st); k_dmu_scan<<<static_cast<int>((nxy + B - 1) / B), B, 0, st>>>(a.ws_act, a.ws_att, a.sino + nxy * cam, a.ws_tmp, nx, ny, nz, a.bg); }
    { NRGB_LAUNCH_SCOPE("k_scatter", st); k_scatter<<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.out, nx, ny, nz, F); }
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int general_gradient(const GeneralArgs& a, cudaStream_t st) {
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nxy = static_cast<size_t>(nx) * ny;
  const int B = 256;
  cudaMemsetAsync(a.out, 0, nvox * sizeof(float), st);
  for (int cam = 0; cam < a.ncam; ++cam) {
    const Affine34 F = affine_of(a.geom_host[cam].fwd);
    const Affine34 Bk = affine_of(a.geom_host[cam].bwd);
    { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.att, a.ws_att, nx, ny, nz, F, a.bg_att); }
    { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, B), B, 0, st>>>(a.act, a.ws_act, nx, ny, nz, F, a.bg); }
    { NRGB_LAUNCH_SCOPE("k_grad_scan", st); k_grad_scan<<<static_cast<int>((nxy + B - 1) / B), B, 0, st>>>(a.ws_act, a.ws_att, a.sino + nxy * cam,
                                                                  a.ws_tmp, nx, ny, nz); }
    if (a.psf_sep) {
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<true><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.ws_act, nx, ny, nz, a.psf_sep, a.psf_k); }
      { NRGB_LAUNCH_SCOPE("k_conv", st); k_conv<false><<<grid_for(nvox, B), B, 0, st>>>(a.ws_act, a.ws_tmp, nx, ny, nz, a.psf_sep, a.psf_k); }
    }
    { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<true><<<grid_for(nvox, B), B, 0, st>>>(a.ws_tmp, a.out, nx, ny, nz, Bk, a.bg); }
  }
  if (a.truncate) launch_truncate(a.out, nvox, st);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

namespace {

// Per-slice 2D true convolution with kernel slice z (centre ((kx-1)/2,
// (ky-1)/2)), the image clamped to its border outside; terms in (j, i) order,
// multiply and add rounded separately (the oracle's order and rounding).
__global__ void k_convolve2d(const float* __restrict__ src, float* __restrict__ dst, int nx, int ny,
                             const float* __restrict__ psf, int kx, int ky) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int z = blockIdx.z;
  if (x >= nx || y >= ny) return;
  const int cx = (kx - 1) / 2, cy = (ky - 1) / 2;
  const float* k = psf + static_cast<size_t>(z) * kx * ky;
  const float* img = src + static_cast<size_t>(z) * nx * ny;
  float acc = 0.0f;
  for (int j = 0; j < ky; ++j) {
    const int yy = min(max(y + cy - j, 0), ny - 1);
    const float* row = img + static_cast<size_t>(yy) * nx;
    for (int i = 0; i < kx; ++i) {
      const int xx = min(max(x + cx - i, 0), nx - 1);
      acc = __fadd_rn(acc, __fmul_rn(__ldg(k + i + kx * j), __ldg(row + xx)));
    }
  }
  dst[(static_cast<size_t>(z) * ny + y) * nx + x] = acc;
}

}  // namespace

int general_convolve2d(const float* src, float* dst, int nx, int ny, int nz, const float* psf, int kx, int ky,
                       cudaStream_t st) {
  const dim3 block(32, 8), grid((nx + 31) / 32, (ny + 7) / 8, nz);
  { NRGB_LAUNCH_SCOPE("k_convolve2d", st); k_convolve2d<<<grid, block, 0, st>>>(src, dst, nx, ny, psf, kx, ky); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int general_rotate(const float* src, float* dst, int nx, int ny, int nz, const float* m12, float bg, cudaStream_t st) {
  const size_t nvox = static_cast<size_t>(nx) * ny * nz;
  { NRGB_LAUNCH_SCOPE("k_resample", st); k_resample<false><<<grid_for(nvox, 256), 256, 0, st>>>(src, dst, nx, ny, nz, affine_of(m12), bg); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

}  // namespace nrgb
