// Elementwise kernels of the OSEM / MLEM step and small helpers.  All are
// HBM-streaming: float4 vectorised where the buffer allows it, grid-stride
// loops over a grid sized to a few waves of the SMs (152 on GB300).
#include "et_kernels.h"
#include "et_profile.h"

namespace nrgb {

namespace {

constexpr int kBlock = 256;

int grid_for(size_t n) {
  const size_t g = (n + kBlock - 1) / kBlock;
  const size_t cap = static_cast<size_t>(sm_count()) * 16;
  return static_cast<int>(g < cap ? (g == 0 ? 1 : g) : cap);
}

__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double dv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float ml(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double ml(double a, double b) { return __dmul_rn(a, b); }

// emission-lib/_et_array_interface.cpp:1022-1028: y/eps where p < eps, else y/p.
template <class T>
__global__ void k_ratio(const T* __restrict__ y, T* __restrict__ p, size_t n, T eps) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const T pv = p[i];
    p[i] = (pv < eps) ? dv(y[i], eps) : dv(y[i], pv);
  }
}

// emission-lib/_et_array_interface.cpp:1036-1044: den < eps -> eps; x *= num / den.
template <class T>
__global__ void k_update(T* __restrict__ x, const T* __restrict__ num, const T* __restrict__ den, size_t n, T eps) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    T d = den[i];
    if (d < eps) d = eps;
    x[i] = ml(x[i], dv(num[i], d));
  }
}

__global__ void k_truncate(float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    if (b[i] < 0.0f) b[i] = 0.0f;
}

__global__ void k_fill(float* __restrict__ b, size_t n, float v) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    b[i] = v;
}

// Deterministic FP64 totals: one partial per block (fixed order), then a
// single-block pass over the partials.
__global__ void k_sum_partial(const float* __restrict__ a, const float* __restrict__ b, size_t n,
                              double* __restrict__ part) {
  __shared__ double sa[kBlock], sb[kBlock];
  double va = 0.0, vb = 0.0;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    va += static_cast<double>(a[i]);
    if (b) vb += static_cast<double>(b[i]);
  }
  sa[threadIdx.x] = va;
  sb[threadIdx.x] = vb;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sa[threadIdx.x] += sa[threadIdx.x + s];
      sb[threadIdx.x] += sb[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sa[0];
    part[2 * blockIdx.x + 1] = sb[0];
  }
}

__global__ void k_sum_final(const double* __restrict__ part, int nparts, double* __restrict__ out) {
  __shared__ double sa[kBlock], sb[kBlock];
  double va = 0.0, vb = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    va += part[2 * i];
    vb += part[2 * i + 1];
  }
  sa[threadIdx.x] = va;
  sb[threadIdx.x] = vb;
  __syncthreads();
  for (int s = kBlock / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sa[threadIdx.x] += sa[threadIdx.x + s];
      sb[threadIdx.x] += sb[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sa[0];
    out[1] = sb[0];
  }
}

// The same two stages over a batch of volumes: a grid-stride loop over the
// concatenation of the selected volumes' elements (prefix in e.begin).
__device__ __forceinline__ int batch_volume(const BatchElems& e, long long i) {
  int v = 0;
  while (v + 1 < e.n && i >= e.begin[v + 1]) ++v;
  return v;
}

__global__ void k_ratio_batch(const BatchStepDesc* __restrict__ d, const BatchElems e, float eps) {
  const long long n = e.begin[e.n];
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int v = batch_volume(e, i);
    const BatchStepDesc& s = d[e.desc[v]];
    const long long j = i - e.begin[v];
    const float pv = s.proj.out[j];
    s.proj.out[j] = (pv < eps) ? __fdiv_rn(s.counts[j], eps) : __fdiv_rn(s.counts[j], pv);
  }
}

__global__ void k_update_batch(const BatchStepDesc* __restrict__ d, const BatchElems e, float eps) {
  const long long n = e.begin[e.n];
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int v = batch_volume(e, i);
    const BatchStepDesc& s = d[e.desc[v]];
    const long long j = i - e.begin[v];
    float den = s.sens[j];
    if (den < eps) den = eps;
    s.act[j] = __fmul_rn(s.act[j], __fdiv_rn(s.num[j], den));
  }
}

// One-step-late MAP-EM (et_osmapem_step, Python/NiftyRec/NiftyRec/NiftyRec.py:224-245).
// Ratio: y / (max(p, 0) + eps).
__global__ void k_ratio_osl(const float* __restrict__ y, float* __restrict__ p, size_t n, float eps) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const float pv = p[i];
    p[i] = __fdiv_rn(y[i], __fadd_rn(pv > 0.0f ? pv : 0.0f, eps));
  }
}

// x *= max(update, 0) / (max(sens - beta * grad, 0) + eps).
__global__ void k_update_osl(float* __restrict__ x, const float* __restrict__ upd, const float* __restrict__ sens,
                             const float* __restrict__ grad, size_t n, float beta, float eps) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    float norm = __fsub_rn(sens[i], __fmul_rn(beta, grad ? grad[i] : 0.0f));
    norm = __fadd_rn(norm > 0.0f ? norm : 0.0f, eps);
    const float u = upd[i] > 0.0f ? upd[i] : 0.0f;
    x[i] = __fdiv_rn(__fmul_rn(x[i], u), norm);
  }
}

// Gradient of the quadratic MRF prior (Python/NiftyRec/NiftyRec/NiftyRec.py:400-404):
// the 3x3x3 convolution with 26 at the centre and -1 elsewhere, zero outside
// the grid: g = 26 x - (sum of the in-grid neighbours).  Dimensions n0
// (fastest), n1, n2 of the buffer's own layout.
__global__ void k_mrf_gradient(const float* __restrict__ x, float* __restrict__ g, int n0, int n1, int n2) {
  const size_t n = static_cast<size_t>(n0) * n1 * n2;
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const int a = static_cast<int>(i % n0);
    const int b = static_cast<int>((i / n0) % n1);
    const int c = static_cast<int>(i / (static_cast<size_t>(n0) * n1));
    float nb = 0.0f;
    for (int dc = -1; dc <= 1; ++dc) {
      const int cc = c + dc;
      if (cc < 0 || cc >= n2) continue;
      for (int db = -1; db <= 1; ++db) {
        const int bb = b + db;
        if (bb < 0 || bb >= n1) continue;
        const float* row = x + (static_cast<size_t>(cc) * n1 + bb) * n0;
        for (int da = -1; da <= 1; ++da) {
          const int aa = a + da;
          if (aa < 0 || aa >= n0 || (da == 0 && db == 0 && dc == 0)) continue;
          nb = __fadd_rn(nb, __ldg(row + aa));
        }
      }
    }
    g[i] = __fsub_rn(__fmul_rn(26.0f, x[i]), nb);
  }
}

}  // namespace

int osem_ratio_osl(const float* y, float* p, size_t n, float eps, cudaStream_t st) {
  { NRGB_LAUNCH_SCOPE("k_ratio_osl", st); k_ratio_osl<<<grid_for(n), kBlock, 0, st>>>(y, p, n, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int osem_update_osl(float* x, const float* upd, const float* sens, const float* grad, size_t n, float beta, float eps,
                    cudaStream_t st) {
  { NRGB_LAUNCH_SCOPE("k_update_osl", st); k_update_osl<<<grid_for(n), kBlock, 0, st>>>(x, upd, sens, grad, n, beta, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int mrf_gradient(const float* x, float* g, int n0, int n1, int n2, cudaStream_t st) {
  const size_t n = static_cast<size_t>(n0) * n1 * n2;
  { NRGB_LAUNCH_SCOPE("k_mrf_gradient", st); k_mrf_gradient<<<grid_for(n), kBlock, 0, st>>>(x, g, n0, n1, n2); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int osem_ratio_batch(const BatchStepDesc* d_desc, const BatchElems& e, float eps, cudaStream_t st) {
  if (e.n <= 0) return kOk;
  { NRGB_LAUNCH_SCOPE("k_ratio_batch", st); k_ratio_batch<<<grid_for(static_cast<size_t>(e.begin[e.n])), kBlock, 0, st>>>(d_desc, e, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int osem_update_batch(const BatchStepDesc* d_desc, const BatchElems& e, float eps, cudaStream_t st) {
  if (e.n <= 0) return kOk;
  { NRGB_LAUNCH_SCOPE("k_update_batch", st); k_update_batch<<<grid_for(static_cast<size_t>(e.begin[e.n])), kBlock, 0, st>>>(d_desc, e, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int osem_ratio(const float* y, float* p, size_t n, float eps, cudaStream_t st) {
  { NRGB_LAUNCH_SCOPE("k_ratio", st); k_ratio<float><<<grid_for(n), kBlock, 0, st>>>(y, p, n, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int osem_update(float* x, const float* num, const float* den, size_t n, float eps, cudaStream_t st) {
  { NRGB_LAUNCH_SCOPE("k_update", st); k_update<float><<<grid_for(n), kBlock, 0, st>>>(x, num, den, n, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int osem_ratio64(const double* y, double* p, size_t n, double eps, cudaStream_t st) {
  { NRGB_LAUNCH_SCOPE("k_ratio", st); k_ratio<double><<<grid_for(n), kBlock, 0, st>>>(y, p, n, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int osem_update64(double* x, const double* num, const double* den, size_t n, double eps, cudaStream_t st) {
  { NRGB_LAUNCH_SCOPE("k_update", st); k_update<double><<<grid_for(n), kBlock, 0, st>>>(x, num, den, n, eps); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

void launch_truncate(float* buf, size_t n, cudaStream_t st) { { NRGB_LAUNCH_SCOPE("k_truncate", st); k_truncate<<<grid_for(n), kBlock, 0, st>>>(buf, n); } }

int fill(float* out, size_t n, float value, cudaStream_t st) {
  { NRGB_LAUNCH_SCOPE("k_fill", st); k_fill<<<grid_for(n), kBlock, 0, st>>>(out, n, value); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

// out must hold 2 + 2 * 256 doubles: [total_a, total_b, partials...].
int sum_fp64(const float* a, const float* b, size_t n, double* out, cudaStream_t st) {
  const int parts = 256;
  { NRGB_LAUNCH_SCOPE("k_sum_partial", st); k_sum_partial<<<parts, kBlock, 0, st>>>(a, b, n, out + 2); }
  { NRGB_LAUNCH_SCOPE("k_sum_final", st); k_sum_final<<<1, kBlock, 0, st>>>(out + 2, parts, out); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

}  // namespace nrgb
