// Layout kernels of the fused y-gantry path (nifti <-> column layout,
// bfloat16 conversions) and the fused path's support rules.
#include "et_yg_device.cuh"

namespace nrgb {
namespace {

// --------------------------------------------------------------- layouts
// dst[p][x][r] = src[p][row0 + r][x] for r < rows, zero pads up to cy.
// src planes have ny_src rows.
__global__ void k_to_col(const float* __restrict__ src, float* __restrict__ dst, int nx, int ny_src, int row0,
                         int rows, int cy) {
  __shared__ float tile[32][33];
  const int p = blockIdx.z;
  const int xb = blockIdx.x * 32, yb = blockIdx.y * 32;
  const int tx = threadIdx.x;
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int r = yb + dy, x = xb + tx;
    tile[dy][tx] = (r < rows && x < nx) ? src[(static_cast<size_t>(p) * ny_src + row0 + r) * nx + x] : 0.0f;
  }
  __syncthreads();
  for (int dx = threadIdx.y; dx < 32; dx += blockDim.y) {
    const int x = xb + dx, r = yb + tx;
    if (x < nx && r < cy) dst[(static_cast<size_t>(p) * nx + x) * cy + r] = tile[tx][dx];
  }
}

// k_to_col over 32 rows x 128 x per CTA with 16-byte reads along x (nx % 4 ==
// 0, src 16-byte aligned): each thread has four float4 loads in flight.  When
// src is host memory read over NVLink-C2C this reaches the link's read rate
// (the 32 x 32 form with 4-byte reads stays about 20% below it); on device
// memory both forms run at the same speed.
// With src2 (a second volume of the same shape) the planes past `planes`
// lay out src2 into dst2: two volumes in one launch.
__global__ void __launch_bounds__(256) k_to_col4(const float* __restrict__ src, float* __restrict__ dst, int nx,
                                                 int ny_src, int row0, int rows, int cy, const float* __restrict__ src2,
                                                 float* __restrict__ dst2, int planes) {
  __shared__ float tile[32][129];
  int p = blockIdx.z;
  if (p >= planes) {  // uniform over the CTA
    p -= planes;
    src = src2;
    dst = dst2;
  }
  const int xb = blockIdx.x * 128, yb = blockIdx.y * 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float4 v[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = yb + w + 8 * i, x = xb + 4 * lane;
    v[i] = (r < rows && x < nx)
               ? *reinterpret_cast<const float4*>(src + (static_cast<size_t>(p) * ny_src + row0 + r) * nx + x)
               : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float* t = &tile[w + 8 * i][4 * lane];
    t[0] = v[i].x;
    t[1] = v[i].y;
    t[2] = v[i].z;
    t[3] = v[i].w;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int dx = 16 * w + i, x = xb + dx, r = yb + lane;
    if (x < nx && r < cy) dst[(static_cast<size_t>(p) * nx + x) * cy + r] = tile[lane][dx];
  }
}

// bfloat16 variant of k_to_col: the source is float32 (rounded to nearest
// even) or already bfloat16 (copied).
template <class S>
__global__ void k_to_col_bf16(const S* __restrict__ src, __nv_bfloat16* __restrict__ dst, int nx, int ny_src,
                              int row0, int rows, int cy) {
  __shared__ float tile[32][33];
  const int p = blockIdx.z;
  const int xb = blockIdx.x * 32, yb = blockIdx.y * 32;
  const int tx = threadIdx.x;
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int r = yb + dy, x = xb + tx;
    float v = 0.0f;
    if (r < rows && x < nx) v = static_cast<float>(src[(static_cast<size_t>(p) * ny_src + row0 + r) * nx + x]);
    tile[dy][tx] = v;
  }
  __syncthreads();
  for (int dx = threadIdx.y; dx < 32; dx += blockDim.y) {
    const int x = xb + dx, r = yb + tx;
    if (x < nx && r < cy) dst[(static_cast<size_t>(p) * nx + x) * cy + r] = __float2bfloat16_rn(tile[tx][dx]);
  }
}

__global__ void k_to_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    dst[i] = __float2bfloat16_rn(src[i]);
}

__global__ void k_from_bf16(const __nv_bfloat16* __restrict__ src, float* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<size_t>(gridDim.x) * blockDim.x)
    dst[i] = __bfloat162float(src[i]);
}

// dst[p][row0 + r][x] = src[p][x][r] for r in [r_begin, r_end); dst planes
// have ny_dst rows; truncate clamps negatives to zero.
__global__ void k_from_col(const float* __restrict__ src, float* __restrict__ dst, int nx, int cy, int r_begin,
                           int r_end, int row0, int ny_dst, int truncate) {
  __shared__ float tile[32][33];
  const int p = blockIdx.z;
  const int xb = blockIdx.x * 32, yb = r_begin + blockIdx.y * 32;
  const int tx = threadIdx.x;
  for (int dx = threadIdx.y; dx < 32; dx += blockDim.y) {
    const int x = xb + dx, r = yb + tx;
    tile[dx][tx] = (x < nx && r < r_end) ? src[(static_cast<size_t>(p) * nx + x) * cy + r] : 0.0f;
  }
  __syncthreads();
  for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
    const int r = yb + dy, x = xb + tx;
    if (x < nx && r < r_end) {
      float v = tile[tx][dy];
      if (truncate && v < 0.0f) v = 0.0f;
      dst[(static_cast<size_t>(p) * ny_dst + row0 + r) * nx + x] = v;
    }
  }
}

// k_from_col over 128 x x 32 rows per CTA with 16-byte writes along x (nx % 4
// == 0, dst 16-byte aligned): host destinations written over NVLink-C2C reach
// the link's write rate (the 32 x 32 form with 4-byte writes about 25% below).
__global__ void __launch_bounds__(256) k_from_col4(const float* __restrict__ src, float* __restrict__ dst, int nx,
                                                   int cy, int r_begin, int r_end, int row0, int ny_dst,
                                                   int truncate) {
  __shared__ float tile[32][129];
  const int p = blockIdx.z;
  const int xb = blockIdx.x * 128, yb = r_begin + blockIdx.y * 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int x = xb + 16 * w + i, r = yb + lane;
    v[i] = (x < nx && r < r_end) ? src[(static_cast<size_t>(p) * nx + x) * cy + r] : 0.0f;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) tile[lane][16 * w + i] = v[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = yb + w + 8 * i, x = xb + 4 * lane;
    if (r < r_end && x < nx) {
      const float* t = &tile[w + 8 * i][4 * lane];
      float4 o = make_float4(t[0], t[1], t[2], t[3]);
      if (truncate) {
        o.x = o.x < 0.0f ? 0.0f : o.x;
        o.y = o.y < 0.0f ? 0.0f : o.y;
        o.z = o.z < 0.0f ? 0.0f : o.z;
        o.w = o.w < 0.0f ? 0.0f : o.w;
      }
      *reinterpret_cast<float4*>(dst + (static_cast<size_t>(p) * ny_dst + row0 + r) * nx + x) = o;
    }
  }
}

bool wide_rows(const void* p, int nx) { return nx % 4 == 0 && (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

int yg_row_windows(int ny, int psf_k, int* out, int max_windows) {
  const std::vector<Window> w = row_windows(ny, psf_k > 0 ? (psf_k - 1) / 2 : 0);
  if (static_cast<int>(w.size()) > max_windows) return -1;
  for (size_t i = 0; i < w.size(); ++i) {
    out[4 * i + 0] = w[i].row0;
    out[4 * i + 1] = w[i].rows;
    out[4 * i + 2] = w[i].lo;
    out[4 * i + 3] = w[i].hi;
  }
  return static_cast<int>(w.size());
}

bool yg_supported(int nx, int ny, int nz, int psf_k) {
  const int cy = round_up(ny, 4);
  if (nx < 1 || ny < 1 || nz < 1) return false;
  if (psf_k != 0 && (psf_k % 2 != 1 || psf_k > 15)) return false;
  // the PSF table of one CTA lives in shared memory next to the tile
  if (psf_k != 0 && tile_smem_bytes<7>(nz) > 110 * 1024) return false;
  // 32-bit element offsets inside one volume
  if (static_cast<size_t>(nz) * nx * cy >= (1u << 31)) return false;
  return true;
}

int to_column_rows(const float* src, float* dst, int nx, int ny_src, int row0, int rows, int cy, int planes,
                   cudaStream_t st) {
  if (wide_rows(src, nx)) {
    const dim3 grid((nx + 127) / 128, (cy + 31) / 32, planes);
    NRGB_LAUNCH_SCOPE("k_to_col4", st);
    k_to_col4<<<grid, 256, 0, st>>>(src, dst, nx, ny_src, row0, rows, cy, nullptr, nullptr, planes);
  } else {
    const dim3 grid((nx + 31) / 32, (cy + 31) / 32, planes), block(32, 8);
    NRGB_LAUNCH_SCOPE("k_to_col", st);
    k_to_col<<<grid, block, 0, st>>>(src, dst, nx, ny_src, row0, rows, cy);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int from_column_rows(const float* src, float* dst, int nx, int cy, int r_begin, int r_end, int row0, int ny_dst,
                     int planes, int truncate, cudaStream_t st) {
  if (r_end <= r_begin) return kOk;
  if (wide_rows(dst, nx)) {
    const dim3 grid((nx + 127) / 128, (r_end - r_begin + 31) / 32, planes);
    NRGB_LAUNCH_SCOPE("k_from_col4", st);
    k_from_col4<<<grid, 256, 0, st>>>(src, dst, nx, cy, r_begin, r_end, row0, ny_dst, truncate);
  } else {
    const dim3 grid((nx + 31) / 32, (r_end - r_begin + 31) / 32, planes), block(32, 8);
    NRGB_LAUNCH_SCOPE("k_from_col", st);
    k_from_col<<<grid, block, 0, st>>>(src, dst, nx, cy, r_begin, r_end, row0, ny_dst, truncate);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int to_column_rows_bf16(const float* src_f32, const void* src_bf16, void* dst, int nx, int ny_src, int row0, int rows,
                        int cy, int planes, cudaStream_t st) {
  const dim3 grid((nx + 31) / 32, (cy + 31) / 32, planes), block(32, 8);
  __nv_bfloat16* d = static_cast<__nv_bfloat16*>(dst);
  NRGB_LAUNCH_SCOPE("k_to_col_bf16", st);
  if (src_f32)
    k_to_col_bf16<float><<<grid, block, 0, st>>>(src_f32, d, nx, ny_src, row0, rows, cy);
  else
    k_to_col_bf16<__nv_bfloat16>
        <<<grid, block, 0, st>>>(static_cast<const __nv_bfloat16*>(src_bf16), d, nx, ny_src, row0, rows, cy);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int to_bf16(const float* src, void* dst, size_t n, cudaStream_t st) {
  if (n == 0) return kOk;
  const int grid = static_cast<int>(std::min<size_t>((n + 255) / 256, static_cast<size_t>(sm_count()) * 16));
  NRGB_LAUNCH_SCOPE("k_to_bf16", st);
  k_to_bf16<<<grid, 256, 0, st>>>(src, static_cast<__nv_bfloat16*>(dst), n);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int from_bf16(const void* src, float* dst, size_t n, cudaStream_t st) {
  if (n == 0) return kOk;
  const int grid = static_cast<int>(std::min<size_t>((n + 255) / 256, static_cast<size_t>(sm_count()) * 16));
  NRGB_LAUNCH_SCOPE("k_from_bf16", st);
  k_from_bf16<<<grid, 256, 0, st>>>(static_cast<const __nv_bfloat16*>(src), dst, n);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int to_column(const float* src, float* dst, int nx, int ny, int cy, int planes, cudaStream_t st) {
  return to_column_rows(src, dst, nx, ny, 0, ny, cy, planes, st);
}

int to_column2(const float* src_a, float* dst_a, const float* src_b, float* dst_b, int nx, int ny, int cy, int planes,
               cudaStream_t st) {
  if (!wide_rows(src_a, nx) || !wide_rows(src_b, nx) || 2 * static_cast<long long>(planes) > 65535) {
    const int s = to_column(src_a, dst_a, nx, ny, cy, planes, st);
    return s != kOk ? s : to_column(src_b, dst_b, nx, ny, cy, planes, st);
  }
  const dim3 grid((nx + 127) / 128, (cy + 31) / 32, 2 * planes);
  NRGB_LAUNCH_SCOPE("k_to_col4", st);
  k_to_col4<<<grid, 256, 0, st>>>(src_a, dst_a, nx, ny, 0, ny, cy, src_b, dst_b, planes);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int from_column(const float* src, float* dst, int nx, int ny, int cy, int planes, int truncate, cudaStream_t st) {
  return from_column_rows(src, dst, nx, cy, 0, ny, 0, ny, planes, truncate, st);
}

}  // namespace nrgb
