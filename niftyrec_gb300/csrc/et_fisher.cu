// Fisher information of a grid of voxels (et_fisher_grid,
// emission-lib/_et.cpp:531-746): for every pair of grid points i <= j and
// every camera, the sum over the overlap of their two depth-dependent PSF
// footprints on the detector of PSF_i * PSF_j * projection.  One thread per
// pair walks the cameras and the overlap box in the reference's order
// (camera, x, y), so every matrix element is accumulated exactly as the
// reference does it; the projection comes from the fused projector on the
// device.  The rotated grid coordinates (integers, one per point and camera)
// are computed on the host with the reference's float operation order.
#include "et_kernels.h"
#include "et_profile.h"

namespace nrgb {

namespace {

__global__ void k_fisher_pairs(const float* __restrict__ proj, int npx, int npy, const int* __restrict__ coords,
                               const int* __restrict__ grid_xyz, int n, int ncam, const float* __restrict__ psf,
                               int kx, int ky, int nz, float* __restrict__ fisher, float* __restrict__ prior) {
  const int i = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || j >= n || j < i) return;
  const int semi_x = (kx - 1) / 2, semi_y = (ky - 1) / 2;
  float f = 0.0f;
  for (int cam = 0; cam < ncam; ++cam) {
    const int* c = coords + static_cast<size_t>(cam) * n * 3;
    const int ix = c[3 * i], iy = c[3 * i + 1], iz = c[3 * i + 2];
    const int jx = c[3 * j], jy = c[3 * j + 1], jz = c[3 * j + 2];
    const int bx = kx - abs(jx - ix), by = ky - abs(jy - iy);
    if (!(bx > 0 && by > 0 && iz >= 0 && jz >= 0 && iz < nz && jz < nz)) continue;
    const int px = max(ix, jx) - semi_x, py = max(iy, jy) - semi_y;
    // offsets of the overlap box inside each PSF (emission-lib/_et.cpp:650-676)
    int pix, piy, pjx, pjy;
    if (jx >= ix && jy > iy) {
      pix = jx - ix; piy = jy - iy; pjx = 0; pjy = 0;
    } else if (jx < ix && jy >= iy) {
      pix = 0; piy = jy - iy; pjx = ix - jx; pjy = 0;
    } else if (jx <= ix && jy < iy) {
      pix = 0; piy = 0; pjx = ix - jx; pjy = iy - jy;
    } else {
      pix = jx - ix; piy = 0; pjx = 0; pjy = iy - jy;
    }
    const float* Pi = psf + static_cast<size_t>(iz) * kx * ky;
    const float* Pj = psf + static_cast<size_t>(jz) * kx * ky;
    const float* plane = proj + static_cast<size_t>(cam) * npx * npy;
    for (int x = 0; x < bx; ++x)
      for (int y = 0; y < by; ++y) {
        const int qx = px + x, qy = py + y;
        if (qx >= 0 && qy >= 0 && qx < npx && qy < npy)
          f = __fadd_rn(f, __fmul_rn(__fmul_rn(__ldg(Pj + (pjy + y) * kx + (pjx + x)), __ldg(Pi + (piy + y) * kx + (pix + x))),
                                     __ldg(plane + qy * npx + qx)));
      }
  }
  fisher[static_cast<size_t>(i) * n + j] = f;
  fisher[static_cast<size_t>(j) * n + i] = f;
  if (prior) {
    // 26-neighbourhood of the unrotated grid points (emission-lib/_et.cpp:703-721)
    const int* a = grid_xyz + 3 * i;
    const int* b = grid_xyz + 3 * j;
    const float v = (abs(a[0] - b[0]) <= 1 && abs(a[1] - b[1]) <= 1 && abs(a[2] - b[2]) <= 1) ? 1.0f : 0.0f;
    prior[static_cast<size_t>(i) * n + j] = v;
    prior[static_cast<size_t>(j) * n + i] = v;
  }
}

}  // namespace

int fisher_pairs(const float* proj, int npx, int npy, const int* coords, const int* grid_xyz, int n, int ncam,
                 const float* psf, int kx, int ky, int nz, float* fisher, float* prior, cudaStream_t st) {
  if (n <= 0) return kOk;
  const dim3 block(128), grid((n + 127) / 128, n);
  {
    NRGB_LAUNCH_SCOPE("k_fisher_pairs", st);
    k_fisher_pairs<<<grid, block, 0, st>>>(proj, npx, npy, coords, grid_xyz, n, ncam, psf, kx, ky, nz, fisher, prior);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

}  // namespace nrgb
