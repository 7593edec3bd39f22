// Backprojection entry point that allocates nothing.
//
// Who needs it: callers that cannot call cudaMalloc -- a plug-in running
// inside a host application whose framework allocator has already reserved
// the GPU's memory (a cudaMalloc there fails or evicts the host's cache), or a
// real-time reconstruction loop that must not enter the driver's allocator
// (its latency is unbounded and it may synchronise the device).  They pass
// their own input and output buffers; every temporary lives in one file-scope
// __device__ array of fixed size (kNoAllocScratchBytes), which each GPU that
// loads this library holds until the process exits.
//
// It runs the same kernels as nrgb_backproject_device (the fused kernels for
// cameras about the gantry axis y, the general-orientation kernels for every
// other camera -- including cameras about x, which nrgb_backproject_device
// serves with the fused kernels), single-stream, with camera-group scratch
// sized to what fits in the array.  Camera matrices and the separated PSF are
// built on the host and stored into the array by small kernels that carry the
// values in their launch parameters, so no host memory is read after the call
// returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "et_array_interface.h"
#include "et_common.h"
#include "et_geometry.h"
#include "et_kernels.h"

namespace nrgb {
namespace {

constexpr size_t kNoAllocScratchBytes = static_cast<size_t>(64) << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;
constexpr int kMaxCams = 4096;
constexpr int kMaxPsfFloats = 2048 * 30;  // nz * 2k for nz <= 2048, k <= 15

// Words carried by value in one store launch (kernel parameters hold up to
// 32 KB).
constexpr int kWordsPerLaunch = 7936;
struct Words {
  unsigned int w[kWordsPerLaunch];
};

__global__ void k_store_words(unsigned int* __restrict__ dst, const __grid_constant__ Words src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src.w[i];
}

// Copies `bytes` (a multiple of 4) of host data into device memory through
// launch parameters.
int store_by_value(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  static thread_local Words chunk;
  const size_t n = bytes / sizeof(unsigned int);
  for (size_t i = 0; i < n; i += kWordsPerLaunch) {
    const int m = static_cast<int>(std::min<size_t>(kWordsPerLaunch, n - i));
    std::memcpy(chunk.w, static_cast<const unsigned int*>(src) + i, sizeof(unsigned int) * m);
    k_store_words<<<1, 256, 0, st>>>(static_cast<unsigned int*>(dst) + i, chunk, m);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrTransferGpu;
}

// The scratch.  In host code this name is only a handle: its device address
// comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;  // serialises host-side use of the fixed host arrays below
void* g_scratch_addr[kMaxDevices] = {};
CamGeom g_geom[kMaxCams];
float g_psf_sep[kMaxPsfFloats];

// Device address of the scratch on the current device (looked up on the first
// call per device).  Caller holds g_mu.
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return kErrNoGpuInstalled;
  }
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return kErrUnspecified;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return kOk;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace nrgb

using namespace nrgb;

extern "C" int nrgb_backproject_device_noalloc(const float* d_sinogram, const float* d_attenuation, const int* size,
                                               float* d_out, const float* cameras, const int* cameras_size,
                                               const float* psf, const int* psf_size, float background,
                                               float background_attenuation, int truncate, void* stream) {
  if (!size || !cameras || !cameras_size || !d_sinogram || !d_out) return kErrParameters;
  const int nx = size[0], ny = size[1], nz = size[2];
  const int ncam = cameras_size[0], ncols = cameras_size[1];
  if (nx <= 0 || ny <= 0 || nz <= 0 || ncam <= 0 || !(ncols == 1 || ncols == 3 || ncols == 6)) return kErrParameters;
  if (ncam > kMaxCams) return kErrScratchTooSmall;
  if (psf && !psf_size) return kErrParameters;
  int k = 0;
  if (psf && !(psf_size[0] == 0 && psf_size[1] == 0 && psf_size[2] == 0)) {
    k = psf_size[0];
    if (k % 2 != 1 || psf_size[1] != k || psf_size[2] < nz) return kErrParameters;
    if (static_cast<size_t>(nz) * 2 * k > static_cast<size_t>(kMaxPsfFloats)) return kErrScratchTooSmall;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lk(g_mu);
  void* base = nullptr;
  int s = scratch_address(&base);
  if (s != kOk) return s;

  // Camera matrices (rules of SPECT_backproject_parallelholes: theta_y-only
  // for one column, centre (size0-1)/2, (size1-1)/2, (size0-1)/2 unless given).
  bool ygantry = true;
  const float c0[3] = {static_cast<float>((nx - 1) / 2.0), static_cast<float>((ny - 1) / 2.0),
                       static_cast<float>((nx - 1) / 2.0)};
  for (int c = 0; c < ncam; ++c) {
    float ang[3], cen[3];
    for (int a = 0; a < 3; ++a) {
      ang[a] = (ncols == 1) ? (a == 1 ? cameras[c] : 0.0f) : cameras[a * ncam + c];
      cen[a] = (ncols == 6) ? cameras[(3 + a) * ncam + c] : c0[a];
    }
    if (ang[0] != 0.0f || ang[2] != 0.0f) ygantry = false;
    float M[16];
    rotation_matrix(M, ang[0], ang[1], ang[2], cen[0], cen[1], cen[2], 0);
    std::memcpy(g_geom[c].fwd, M, sizeof(float) * 12);
    rotation_matrix(M, -ang[0], -ang[1], -ang[2], cen[0], cen[1], cen[2], 5);
    std::memcpy(g_geom[c].bwd, M, sizeof(float) * 12);
  }
  if (k) {
    const int cc = (k - 1) / 2;
    for (int n = 0; n < nz; ++n) {
      const float* plane = psf + static_cast<size_t>(k) * k * n;
      const float norm = plane[cc * k + cc];
      for (int i = 0; i < k; ++i) {
        g_psf_sep[2 * k * n + i] = plane[cc * k + i];
        g_psf_sep[2 * k * n + k + i] = plane[cc + i * k] / norm;
      }
    }
  }

  // Scratch layout.
  const bool fused = ygantry && background == 0.0f && background_attenuation == 0.0f && yg_supported(nx, ny, nz, k);
  const int cy = round_up(ny, 4);
  const size_t geom_b = align256(sizeof(CamGeom) * ncam);
  const size_t psf_b = align256(sizeof(float) * static_cast<size_t>(nz) * 2 * k);
  size_t need = geom_b + psf_b;
  int group = 1;
  size_t col_b = 0, sino_b = 0, nvox_b = 0;
  if (fused) {
    col_b = align256(sizeof(float) * static_cast<size_t>(nz) * nx * cy);
    sino_b = align256(sizeof(float) * static_cast<size_t>(ncam) * nx * cy);
    const size_t fixed = need + sino_b + col_b * (d_attenuation ? 2 : 1);
    const size_t one = align256(yg_backproject_workspace(nx, ny, nz, ncam, 1, 1));
    if (fixed + one > kNoAllocScratchBytes) return kErrScratchTooSmall;
    for (group = 8; group > 1; --group)
      if (fixed + align256(yg_backproject_workspace(nx, ny, nz, ncam, group, 1)) <= kNoAllocScratchBytes) break;
    need = fixed + align256(yg_backproject_workspace(nx, ny, nz, ncam, group, 1));
  } else {
    nvox_b = align256(sizeof(float) * static_cast<size_t>(nx) * ny * nz);
    need += 3 * nvox_b;
  }
  if (need > kNoAllocScratchBytes) return kErrScratchTooSmall;

  char* p = static_cast<char*>(base);
  CamGeom* d_geom = reinterpret_cast<CamGeom*>(p);
  p += geom_b;
  float* d_psf = k ? reinterpret_cast<float*>(p) : nullptr;
  p += psf_b;
  if ((s = store_by_value(d_geom, g_geom, sizeof(CamGeom) * ncam, st)) != kOk) return s;
  if (k && (s = store_by_value(d_psf, g_psf_sep, sizeof(float) * static_cast<size_t>(nz) * 2 * k, st)) != kOk)
    return s;
  set_last_path(fused ? 1 : 2);

  if (fused) {
    float* sino_c = reinterpret_cast<float*>(p);
    p += sino_b;
    float* mu_c = nullptr;
    if (d_attenuation) {
      mu_c = reinterpret_cast<float*>(p);
      p += col_b;
    }
    float* out_c = reinterpret_cast<float*>(p);
    p += col_b;
    if ((s = to_column(d_sinogram, sino_c, nx, ny, cy, ncam, st)) != kOk) return s;
    if (d_attenuation && (s = to_column(d_attenuation, mu_c, nx, ny, cy, nz, st)) != kOk) return s;
    YgArgs a;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.cy = cy;
    a.ncam = ncam;
    a.geom = d_geom;
    a.mu = mu_c;
    a.sino = sino_c;
    a.out = out_c;
    a.psf = d_psf;
    a.psf_k = k;
    a.truncate = truncate;
    a.group = group;
    a.pipelined = 0;
    a.work = reinterpret_cast<float*>(p);
    if ((s = yg_backproject(a, st)) != kOk) return s;
    return from_column(out_c, d_out, nx, ny, cy, nz, truncate, st);
  }
  GeneralArgs g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.ncam = ncam;
  g.geom_host = g_geom;
  g.att = d_attenuation;
  g.sino = d_sinogram;
  g.out = d_out;
  g.psf_sep = d_psf;
  g.psf_k = k;
  g.bg = background;
  g.bg_att = background_attenuation;
  g.truncate = truncate;
  g.ws_act = reinterpret_cast<float*>(p);
  g.ws_att = reinterpret_cast<float*>(p + nvox_b);
  g.ws_tmp = reinterpret_cast<float*>(p + 2 * nvox_b);
  return general_backproject(g, st);
}
