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
  const dim3 grid((nx + 31) / 32, (cy + 31) / 32, planes), block(32, 8);
  { NRGB_LAUNCH_SCOPE("k_to_col", st); k_to_col<<<grid, block, 0, st>>>(src, dst, nx, ny_src, row0, rows, cy); }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int from_column_rows(const float* src, float* dst, int nx, int cy, int r_begin, int r_end, int row0, int ny_dst,
                     int planes, int truncate, cudaStream_t st) {
  if (r_end <= r_begin) return kOk;
  const dim3 grid((nx + 31) / 32, (r_end - r_begin + 31) / 32, planes), block(32, 8);
  {
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

int from_column(const float* src, float* dst, int nx, int ny, int cy, int planes, int truncate, cudaStream_t st) {
  return from_column_rows(src, dst, nx, cy, 0, ny, 0, ny, planes, truncate, st);
}

}  // namespace nrgb
