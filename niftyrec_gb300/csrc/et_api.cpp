// The C-ABI: the entry points of NiftyRec's emission array interface
// (emission-lib/_et_array_interface.h), with the reference's argument meaning,
// size rules and status codes, implemented on the GB300 engine; plus
// device-pointer entry points for callers that keep data on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "et_array_interface.h"
#include "et_engine.h"
#include "et_trace.h"
#include "et_kernels.h"

using namespace nrgb;

namespace {

bool all_zero3(const int* s) { return s[0] == 0 && s[1] == 0 && s[2] == 0; }

// Diagnostics: which path the last call of this thread took.
thread_local int g_last_path = 0;  // 1 = fused gantry kernels (about y, or x with x and y exchanged), 2 = general path

size_t fbytes(size_t n) { return n * sizeof(float); }

}  // namespace

void nrgb::set_last_path(int path) { g_last_path = path; }

bool nrgb::log_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("NIFTYREC_LOG");
    return v && *v && std::strcmp(v, "0") != 0;
  }();
  return on;
}

void nrgb::log_call(const char* name, double host_ms) {
  std::fprintf(stderr, "{\"niftyrec\": \"%s\", \"host_ms\": %.3f, \"path\": %d}\n", name, host_ms, g_last_path);
}

namespace {

int finish(DeviceState& ds, int status) {
  cudaEventRecord(ds.last_use, ds.stream);
  const cudaError_t e = cudaStreamSynchronize(ds.stream);
  if (status != kOk) return status;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return kErrKernel;
  }
  return kOk;
}

int h2d(float* d, const float* h, size_t n, cudaStream_t st) {
  return cudaMemcpyAsync(d, h, fbytes(n), cudaMemcpyHostToDevice, st) == cudaSuccess ? kOk : kErrTransferGpu;
}

int d2h(float* h, const float* d, size_t n, cudaStream_t st) {
  return cudaMemcpyAsync(h, d, fbytes(n), cudaMemcpyDeviceToHost, st) == cudaSuccess ? kOk : kErrTransferGpu;
}

// Whether the current device reads pageable host memory through the host's
// page tables (address translation services, e.g. a Grace-Blackwell
// NVLink-C2C system): the fused path's layout kernels then read the caller's
// host arrays directly -- one pass over the link at the rate of a copy, no
// separate host-to-device copy and the transpose fused into it.
bool host_memory_readable() {
  static std::mutex mu;
  static std::map<int, bool> known;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lk(mu);
  auto it = known.find(dev);
  if (it != known.end()) return it->second;
  int pma = 0, ats = 0;
  if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
    cudaGetLastError();
    pma = ats = 0;
  }
  return known[dev] = (pma == 1 && ats == 1);
}

// Project with host buffers (activity and/or attenuation may be null).
int project_host(const Problem& pb, const float* act, const float* att, float* sino) {
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(pb.nx) * pb.ny * pb.nz;
  const size_t nsino = static_cast<size_t>(pb.nx) * pb.ny * pb.cams.n;
  const size_t ws = project_workspace(pb, act != nullptr, att != nullptr);
  if ((s = ensure_arena(ds, fbytes(2 * nvox + nsino) + 4 * 256 + ws)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_act = act ? cv.take<float>(nvox) : nullptr;
  float* d_att = att ? cv.take<float>(nvox) : nullptr;
  float* d_sino = cv.take<float>(nsino);
  char* w = cv.take<char>(ws);
  cudaStream_t st = ds.stream;
  g_last_path = ((use_fused(pb) || use_fused_x(pb)) && act) ? 1 : 2;
  const bool direct = use_fused(pb) && act && host_memory_readable();
  if (direct) {  // the layout kernels read the host arrays and write the host sinogram
    d_act = const_cast<float*>(act);
    d_att = const_cast<float*>(att);
    d_sino = sino;
  } else {
    if (act && (s = h2d(d_act, act, nvox, st)) != kOk) return finish(ds, s);
    if (att && (s = h2d(d_att, att, nvox, st)) != kOk) return finish(ds, s);
  }
  s = project_device(pb, d_act, d_att, d_sino, w, ws, &ds.staging, st);
  if (s == kOk && !direct) s = d2h(sino, d_sino, nsino, st);
  return finish(ds, s);
}

int backproject_host(const Problem& pb, const float* sino, const float* att, float* out) {
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(pb.nx) * pb.ny * pb.nz;
  const size_t nsino = static_cast<size_t>(pb.nx) * pb.ny * pb.cams.n;
  const size_t ws = backproject_workspace(pb, att != nullptr);
  if ((s = ensure_arena(ds, fbytes(2 * nvox + nsino) + 4 * 256 + ws)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_sino = cv.take<float>(nsino);
  float* d_att = att ? cv.take<float>(nvox) : nullptr;
  float* d_out = cv.take<float>(nvox);
  char* w = cv.take<char>(ws);
  cudaStream_t st = ds.stream;
  g_last_path = (use_fused(pb) || use_fused_x(pb)) ? 1 : 2;
  const bool direct = use_fused(pb) && host_memory_readable();
  if (direct) {  // the layout kernels read the host arrays and write the host volume
    d_sino = const_cast<float*>(sino);
    d_att = const_cast<float*>(att);
    d_out = out;
  } else {
    if ((s = h2d(d_sino, sino, nsino, st)) != kOk) return finish(ds, s);
    if (att && (s = h2d(d_att, att, nvox, st)) != kOk) return finish(ds, s);
  }
  s = backproject_device(pb, d_sino, d_att, d_out, w, ws, &ds.staging, st);
  if (s == kOk && !direct) s = d2h(out, d_out, nvox, st);
  return finish(ds, s);
}

int gradient_host(const Problem& pb, const float* sino, const float* act, const float* att, float* out) {
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(pb.nx) * pb.ny * pb.nz;
  const size_t nsino = static_cast<size_t>(pb.nx) * pb.ny * pb.cams.n;
  const size_t ws = gradient_workspace(pb);
  if ((s = ensure_arena(ds, fbytes(3 * nvox + nsino) + 5 * 256 + ws)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_sino = cv.take<float>(nsino);
  float* d_act = cv.take<float>(nvox);
  float* d_att = cv.take<float>(nvox);
  float* d_out = cv.take<float>(nvox);
  char* w = cv.take<char>(ws);
  cudaStream_t st = ds.stream;
  const bool fused = (use_fused(pb) || use_fused_x(pb)) && pb.storage == kStorageF32;
  g_last_path = fused ? 1 : 2;
  if (fused && use_fused(pb) && host_memory_readable()) {  // the layout kernels read the host arrays
    d_sino = const_cast<float*>(sino);
    d_act = const_cast<float*>(act);
    d_att = const_cast<float*>(att);
  } else {
    if ((s = h2d(d_sino, sino, nsino, st)) != kOk) return finish(ds, s);
    if ((s = h2d(d_act, act, nvox, st)) != kOk) return finish(ds, s);
    if ((s = h2d(d_att, att, nvox, st)) != kOk) return finish(ds, s);
  }
  s = gradient_device(pb, d_sino, d_act, d_att, d_out, w, ws, &ds.staging, st);
  if (s == kOk) s = d2h(out, d_out, nvox, st);
  return finish(ds, s);
}

// One OSEM step over the given camera subset on the device:
// project (truncate) -> ratio -> backproject ratio and ones (truncate) -> update,
// emission-lib/_et_array_interface.cpp:1017-1044.
int osem_step_host(const Problem& pb, float* act, const float* ysub, const float* att, float eps) {
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(pb.nx) * pb.ny * pb.nz;
  const size_t nsino = static_cast<size_t>(pb.nx) * pb.ny * pb.cams.n;
  const size_t ws = std::max(project_workspace(pb, true, att != nullptr), backproject_workspace(pb, att != nullptr));
  if ((s = ensure_arena(ds, fbytes(4 * nvox + 3 * nsino) + 8 * 256 + ws)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_act = cv.take<float>(nvox);
  float* d_att = att ? cv.take<float>(nvox) : nullptr;
  float* d_num = cv.take<float>(nvox);
  float* d_den = cv.take<float>(nvox);
  float* d_y = cv.take<float>(nsino);
  float* d_p = cv.take<float>(nsino);
  float* d_ones = cv.take<float>(nsino);
  char* w = cv.take<char>(ws);
  cudaStream_t st = ds.stream;
  if ((s = h2d(d_act, act, nvox, st)) != kOk) return finish(ds, s);
  if (att && (s = h2d(d_att, att, nvox, st)) != kOk) return finish(ds, s);
  if ((s = h2d(d_y, ysub, nsino, st)) != kOk) return finish(ds, s);
  Problem p1 = pb;
  p1.truncate = 1;
  g_last_path = (use_fused(p1) || use_fused_x(p1)) ? 1 : 2;
  if ((s = project_device(p1, d_act, d_att, d_p, w, ws, &ds.staging, st)) != kOk) return finish(ds, s);
  if ((s = osem_ratio(d_y, d_p, nsino, eps, st)) != kOk) return finish(ds, s);
  if ((s = backproject_device(p1, d_p, d_att, d_num, w, ws, &ds.staging, st)) != kOk) return finish(ds, s);
  if ((s = fill(d_ones, nsino, 1.0f, st)) != kOk) return finish(ds, s);
  if ((s = backproject_device(p1, d_ones, d_att, d_den, w, ws, &ds.staging, st)) != kOk) return finish(ds, s);
  if ((s = osem_update(d_act, d_num, d_den, nvox, eps, st)) != kOk) return finish(ds, s);
  s = d2h(act, d_act, nvox, st);
  return finish(ds, s);
}

// Grid points of a Fisher-information grid volume (values 1..n at the points,
// 0 elsewhere), scanned x outer, z inner as emission-lib/_et.cpp:580-598;
// kErrParameters (the reference's ET_ERROR_BADGRID) for a repeated or
// out-of-range index.
int grid_points(const float* grid, int nx, int ny, int nz, int n, std::vector<int>* xyz) {
  xyz->assign(3 * static_cast<size_t>(n), -1);
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y)
      for (int z = 0; z < nz; ++z) {
        const float g = grid[(static_cast<size_t>(z) * ny + y) * nx + x];
        if (g == 0.0f) continue;
        const int k = static_cast<int>(g) - 1;
        if (k < 0 || k >= n || (*xyz)[3 * k] != -1) return kErrParameters;
        (*xyz)[3 * k] = x;
        (*xyz)[3 * k + 1] = y;
        (*xyz)[3 * k + 2] = z;
      }
  return kOk;
}

// Grid points rotated into every camera's frame (XYZ, +theta), with
// reg_mat44_mul's float order (reg-lib/_reg_affineTransformation.cpp:44-51)
// and the implicit truncation to integers of emission-lib/_et.cpp:619-623.
std::vector<int> rotated_grid(const Cameras& cc, const std::vector<int>& xyz, int n) {
  std::vector<int> out(static_cast<size_t>(cc.n) * n * 3);
  const int nc = cc.n;
  for (int cam = 0; cam < nc; ++cam) {
    float M[16];
    rotation_matrix(M, cc.angles[cam], cc.angles[nc + cam], cc.angles[2 * nc + cam], cc.centers[cam],
                    cc.centers[nc + cam], cc.centers[2 * nc + cam], 0);
    for (int k = 0; k < n; ++k) {
      const float p0 = static_cast<float>(xyz[3 * k]), p1 = static_cast<float>(xyz[3 * k + 1]),
                  p2 = static_cast<float>(xyz[3 * k + 2]);
      for (int r = 0; r < 3; ++r) {
        const float v = M[4 * r] * p0 + M[4 * r + 1] * p1 + M[4 * r + 2] * p2 + M[4 * r + 3];
        out[(static_cast<size_t>(cam) * n + k) * 3 + r] = static_cast<int>(v);
      }
    }
  }
  return out;
}

// Fisher matrix on the device from a projection (device, [ncam][npy][npx]),
// grid points and PSF planes (host); fisher / prior are host [n][n].
int fisher_from_projection(DeviceState& ds, Carver& cv, const float* d_proj, int npx, int npy, int nz,
                           const Cameras& cc, const std::vector<int>& xyz, int n, const float* psf, int kx, int ky,
                           int psf_planes, float* fisher, float* prior, cudaStream_t st) {
  const std::vector<int> coords = rotated_grid(cc, xyz, n);
  int* d_coords = cv.take<int>(coords.size());
  int* d_xyz = cv.take<int>(xyz.size());
  float* d_psf = cv.take<float>(static_cast<size_t>(kx) * ky * psf_planes);
  float* d_f = cv.take<float>(static_cast<size_t>(n) * n);
  float* d_p = prior ? cv.take<float>(static_cast<size_t>(n) * n) : nullptr;
  if (!d_coords || !d_xyz || !d_psf || !d_f || (prior && !d_p)) return kErrAllocGpu;
  if (cudaMemcpyAsync(d_coords, coords.data(), sizeof(int) * coords.size(), cudaMemcpyHostToDevice, st) !=
          cudaSuccess ||
      cudaMemcpyAsync(d_xyz, xyz.data(), sizeof(int) * xyz.size(), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(d_psf, psf, sizeof(float) * kx * ky * psf_planes, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return kErrTransferGpu;
  int s = fisher_pairs(d_proj, npx, npy, d_coords, d_xyz, n, cc.n, d_psf, kx, ky, nz, d_f, d_p, st);
  if (s == kOk) s = d2h(fisher, d_f, static_cast<size_t>(n) * n, st);
  if (s == kOk && prior) s = d2h(prior, d_p, static_cast<size_t>(n) * n, st);
  (void)ds;
  return s;
}

int project_partial_host(const Problem& pb, const float* act, const float* att, const float* bg_image, float* sino,
                         float* partial, int do_rotate) {
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(pb.nx) * pb.ny * pb.nz;
  const size_t nxy = static_cast<size_t>(pb.nx) * pb.ny;
  const size_t nsino = nxy * pb.cams.n;
  const size_t npart = nvox * pb.cams.n;
  const size_t ws = partial_workspace(pb);
  if ((s = ensure_arena(ds, fbytes(2 * nvox + nxy + nsino + npart) + 6 * 256 + ws)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_act = act ? cv.take<float>(nvox) : nullptr;
  float* d_att = att ? cv.take<float>(nvox) : nullptr;
  float* d_bgi = bg_image ? cv.take<float>(nxy) : nullptr;
  float* d_sino = cv.take<float>(nsino);
  float* d_part = cv.take<float>(npart);
  char* w = cv.take<char>(ws);
  cudaStream_t st = ds.stream;
  if (act && (s = h2d(d_act, act, nvox, st)) != kOk) return finish(ds, s);
  if (att && (s = h2d(d_att, att, nvox, st)) != kOk) return finish(ds, s);
  if (bg_image && (s = h2d(d_bgi, bg_image, nxy, st)) != kOk) return finish(ds, s);
  g_last_path = 2;
  s = project_partial_device(pb, d_act, d_att, d_bgi, d_sino, d_part, do_rotate, w, ws, &ds.staging, st);
  if (s == kOk) s = d2h(sino, d_sino, nsino, st);
  if (s == kOk) s = d2h(partial, d_part, npart, st);
  return finish(ds, s);
}

// random_0_1 of emission-lib/_et_array_interface.cpp:961-967 (two rand() draws).
float random_0_1() {
  const float scale = RAND_MAX + 1.;
  const float base = rand() / scale;
  const float fine = rand() / scale;
  return base + fine / scale;
}

int subset_step(float* activity_data, int size_x, int size_y, const float* sinogram_data, int n_cameras,
                const float* cameras_data, const std::vector<int>& idx, int use_attenuation,
                const float* attenuation_data, int use_psf, const float* psf_data, unsigned psf_size_x,
                unsigned psf_size_y, float background, float background_attenuation, float epsilon) {
  const int nsub = static_cast<int>(idx.size());
  if (size_x <= 0 || size_y <= 0 || n_cameras <= 0 || nsub <= 0) return kErrParameters;
  for (int i : idx)
    if (i < 0 || i >= n_cameras) return kErrParameters;
  std::vector<float> cams(3 * static_cast<size_t>(nsub));
  for (int c = 0; c < nsub; ++c)
    for (int a = 0; a < 3; ++a) cams[a * nsub + c] = cameras_data[idx[c] + a * static_cast<size_t>(n_cameras)];
  const size_t nxy = static_cast<size_t>(size_x) * size_y;
  std::vector<float> ysub(nxy * nsub);
  for (int c = 0; c < nsub; ++c) std::memcpy(&ysub[nxy * c], sinogram_data + nxy * idx[c], fbytes(nxy));
  const int vsize[3] = {size_x, size_y, size_x};
  Cameras cc;
  int s = expand_cameras(cams.data(), nsub, 3, vsize, &cc);
  if (s != kOk) return s;
  const int psz[3] = {static_cast<int>(psf_size_x), static_cast<int>(psf_size_y), size_x};
  Problem pb;
  s = make_problem(size_x, size_y, size_x, cc, use_psf ? psf_data : nullptr, psz, background, background_attenuation,
                   1, &pb);
  if (s != kOk) return s;
  return osem_step_host(pb, activity_data, ysub.data(), use_attenuation ? attenuation_data : nullptr, epsilon);
}

int spect_project(float* activity, int* activity_size, float* sinogram, int* sinogram_size, float* cameras,
                  int* cameras_size, float* psf, int* psf_size, float* attenuation, int* attenuation_size,
                  float background, float background_attenuation, int truncate) {
  if (!activity_size || !cameras_size || !psf_size || !attenuation_size) return kErrParameters;
  int asz[3] = {activity_size[0], activity_size[1], activity_size[2]};
  const bool no_act = all_zero3(asz);
  const bool no_psf = all_zero3(psf_size);
  const bool no_att = all_zero3(attenuation_size);
  if (no_act && no_att) return kErrParameters;
  if (no_act) std::memcpy(asz, attenuation_size, sizeof(asz));
  if (!no_act && !no_att &&
      (attenuation_size[0] != asz[0] || attenuation_size[1] != asz[1] || attenuation_size[2] != asz[2]))
    return kErrParameters;
  const int ncam = cameras_size[0], ncols = cameras_size[1];
  if (!(ncols == 1 || ncols == 3 || ncols == 6)) return kErrParameters;
  if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != asz[0])) return kErrParameters;
  if (sinogram_size &&
      static_cast<long long>(sinogram_size[0]) * sinogram_size[1] * sinogram_size[2] <
          static_cast<long long>(asz[0]) * asz[1] * ncam)
    return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, ncam, ncols, asz, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(asz[0], asz[1], asz[2], cc, no_psf ? nullptr : psf, psf_size, background, background_attenuation,
                   truncate, &pb);
  if (s != kOk) return s;
  return project_host(pb, no_act ? nullptr : activity, no_att ? nullptr : attenuation, sinogram);
}

int spect_backproject(float* sino, int* sino_size, float* bkpr, int* bkpr_size, float* cameras, int* cameras_size,
                      float* psf, int* psf_size, float* attenuation, int* attenuation_size, float background,
                      float background_attenuation, int truncate) {
  if (!sino_size || !bkpr_size || !cameras_size || !psf_size || !attenuation_size) return kErrParameters;
  const bool no_psf = all_zero3(psf_size);
  const bool no_att = all_zero3(attenuation_size);
  const int ncam = cameras_size[0], ncols = cameras_size[1];
  if (!(ncols == 1 || ncols == 3 || ncols == 6)) return kErrParameters;
  if (sino_size[2] != ncam) return kErrParameters;
  if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != sino_size[0])) return kErrParameters;
  // The spread writes sinogram plane (x, y) into the volume grid, so they must agree.
  if (bkpr_size[0] != sino_size[0] || bkpr_size[1] != sino_size[1]) return kErrParameters;
  if (!no_att && (attenuation_size[0] != bkpr_size[0] || attenuation_size[1] != bkpr_size[1] ||
                  attenuation_size[2] != bkpr_size[2]))
    return kErrParameters;
  // Centre of rotation from (sino0, sino1, sino0), emission-lib/_et_array_interface.cpp:598-630.
  const int csz[3] = {sino_size[0], sino_size[1], sino_size[0]};
  Cameras cc;
  int s = expand_cameras(cameras, ncam, ncols, csz, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(bkpr_size[0], bkpr_size[1], bkpr_size[2], cc, no_psf ? nullptr : psf, psf_size, background,
                   background_attenuation, truncate, &pb);
  if (s != kOk) return s;
  return backproject_host(pb, sino, no_att ? nullptr : attenuation, bkpr);
}

const char* kMessages[] = {
    "niftyrec: success",
    "niftyrec: unspecified error",
    "niftyrec: wrong parameters",
    "niftyrec: CUDA kernel failed",
    "niftyrec: GPU memory allocation failed",
    "niftyrec: host memory allocation failed",
    "niftyrec: host/GPU transfer failed",
    "niftyrec: built without GPU support",
    "niftyrec: no GPU installed",
    "niftyrec: status 9 is not used",
    "niftyrec: the problem needs more work space than the 64 MiB fixed scratch of "
    "nrgb_backproject_device_noalloc (use nrgb_backproject_device, or fewer cameras / a smaller grid)",
};

}  // namespace

extern "C" {

// ---------------------------------------------------------------- status
// emission-lib/_et_array_interface.cpp:21-52
int status_success(int* status) { *status = 0; return 0; }
int status_io_error(int* status) { *status = 101; return 0; }
int status_initialisation_error(int* status) { *status = 103; return 0; }
int status_parameter_error(int* status) { *status = 104; return 0; }
int status_unhandled_error(int* status) { *status = 105; return 0; }
int echo(int* in, int* out) { *out = *in; return 0; }

// emission-lib/_et_common.cpp:269-306
char* niftyrec_error_msg(int status) {
  if (status >= 0 && status <= kErrScratchTooSmall) return const_cast<char*>(kMessages[status]);
  return const_cast<char*>("niftyrec: unknown status");
}

// --------------------------------------------------------------- devices
// emission-lib/_et_array_interface.cpp:269-272 returns 0; here 1 when a GPU is usable.
int et_array_isinstalled() {
  NRGB_API("et_array_isinstalled");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n > 0 ? 1 : 0;
}

// emission-lib/_et.cpp:1988-2022: five ints per device
// {id, SMs * clock_kHz, SMs, clock_kHz, global memory in MB}.
int et_array_list_gpus(int* gpu_count, int* gpus_info_array) {
  NRGB_API("et_array_list_gpus");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    gpu_count[0] = 0;
    return kErrNoGpuInstalled;
  }
  const int nmax = std::min(n, 16);
  for (int d = 0; d < nmax; ++d) {
    int sms = 0, clk = 0;
    size_t mem = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, d);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, d) == cudaSuccess) mem = prop.totalGlobalMem;
    gpus_info_array[5 * d + 0] = d;
    gpus_info_array[5 * d + 1] = sms * clk;
    gpus_info_array[5 * d + 2] = sms;
    gpus_info_array[5 * d + 3] = clk;
    gpus_info_array[5 * d + 4] = static_cast<int>(std::floor(mem / 1000000.0));
  }
  gpu_count[0] = n;
  return kOk;
}

// emission-lib/_et.cpp:2029-2044
int et_array_set_gpu(int id) {
  NRGB_API("et_array_set_gpu");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || id < 0 || id >= n) {
    cudaGetLastError();
    return kErrUnspecified;
  }
  return cudaSetDevice(id) == cudaSuccess ? kOk : kErrUnspecified;
}

int et_array_set_gpu_pointer(int* id) { return et_array_set_gpu(id[0]); }

// emission-lib/_et.cpp:2445-2451.  Frees this library's work space on the
// current device; the CUDA context itself is left to its other users.
// Fault injection for tests of callers' error handling (no counterpart in
// the reference): the next n work-space allocations fail with status 4.
int nrgb_debug_fail_allocations(int n) {
  fail_next_allocations(n);
  return kOk;
}

int et_array_reset_gpu() {
  NRGB_API("et_array_reset_gpu");
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  cudaStreamSynchronize(ds.stream);
  if (ds.arena) cudaFree(ds.arena);
  ds.arena = nullptr;
  ds.arena_bytes = 0;
  return kOk;
}

// emission-lib/_et.cpp:27-36.  The fused kernels take any size: every size is
// a "block multiple" and the block size is 1.
unsigned short et_array_is_block_multiple(unsigned short size) { return size > 0 ? 1 : 0; }
unsigned short et_array_get_block_size(void) { return 1; }

// ------------------------------------------------------------ projection
// emission-lib/_et_array_interface.h:44 (scalars by pointer), impl .cpp:337-541.
int SPECT_project_parallelholes(float* activity, int* activity_size, float* sinogram, int* sinogram_size,
                                float* cameras, int* cameras_size, float* psf, int* psf_size, float* attenuation,
                                int* attenuation_size, float* Background, float* Background_attenuation, int* Gpu,
                                int* Truncate_negative_values) {
  NRGB_API("SPECT_project_parallelholes");
  (void)Gpu;
  return spect_project(activity, activity_size, sinogram, sinogram_size, cameras, cameras_size, psf, psf_size,
                       attenuation, attenuation_size, *Background, *Background_attenuation,
                       *Truncate_negative_values);
}

// The by-value spelling bound by Python/NiftyRec/NiftyRec/NiftyRec.py:83-84.
int et_array_project(float* activity, int* activity_size, float* sinogram, int* sinogram_size, float* cameras,
                     int* cameras_size, float* psf, int* psf_size, float* attenuation, int* attenuation_size,
                     float background, float background_attenuation, int gpu, int truncate_negative_values) {
  NRGB_API("et_array_project");
  (void)gpu;
  return spect_project(activity, activity_size, sinogram, sinogram_size, cameras, cameras_size, psf, psf_size,
                       attenuation, attenuation_size, background, background_attenuation, truncate_negative_values);
}

// --------------------------------------------------------- backprojection
// emission-lib/_et_array_interface.h:45, impl .cpp:547-710.
int SPECT_backproject_parallelholes(float* sino, int* sino_size, float* bkpr, int* bkpr_size, float* cameras,
                                    int* cameras_size, float* psf, int* psf_size, float* attenuation,
                                    int* attenuation_size, float* Background, float* Background_attenuation,
                                    int* Gpu, int* Truncate_negative_values) {
  NRGB_API("SPECT_backproject_parallelholes");
  (void)Gpu;
  return spect_backproject(sino, sino_size, bkpr, bkpr_size, cameras, cameras_size, psf, psf_size, attenuation,
                           attenuation_size, *Background, *Background_attenuation, *Truncate_negative_values);
}

// By-value spelling bound by Python/NiftyRec/NiftyRec/NiftyRec.py:145-146.
int et_array_backproject(float* sino, int* sino_size, float* bkpr, int* bkpr_size, float* cameras, int* cameras_size,
                         float* psf, int* psf_size, float* attenuation, int* attenuation_size, float background,
                         float background_attenuation, int gpu, int truncate_negative_values) {
  NRGB_API("et_array_backproject");
  (void)gpu;
  return spect_backproject(sino, sino_size, bkpr, bkpr_size, cameras, cameras_size, psf, psf_size, attenuation,
                           attenuation_size, background, background_attenuation, truncate_negative_values);
}

// ---------------------------------------------------- attenuation gradient
// emission-lib/_et_array_interface.h:48, impl .cpp:714-892 (3-D sinograms),
// computed as et_gradient_attenuation_gpu, emission-lib/_et.cpp:1679-1924.
int et_array_gradient_attenuation(float* sino, int* sino_size, float* activity, int* activity_size, float* gradient,
                                  int* gradient_size, float* cameras, int* cameras_size, float* psf, int* psf_size,
                                  float* attenuation, int* attenuation_size, float background,
                                  float background_attenuation, int GPU, int truncate_negative_values) {
  NRGB_API("et_array_gradient_attenuation");
  (void)GPU;
  (void)attenuation_size;
  if (!sino_size || !activity_size || !gradient_size || !cameras_size || !psf_size) return kErrParameters;
  const bool no_psf = all_zero3(psf_size);
  const int ncam = cameras_size[0], ncols = cameras_size[1];
  if (!(ncols == 1 || ncols == 3 || ncols == 6)) return kErrParameters;
  if (sino_size[2] != ncam) return kErrParameters;
  if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != sino_size[0])) return kErrParameters;
  if (gradient_size[0] != sino_size[0] || gradient_size[1] != sino_size[1]) return kErrParameters;
  if (!activity || !attenuation || !gradient) return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, ncam, ncols, activity_size, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(gradient_size[0], gradient_size[1], gradient_size[2], cc, no_psf ? nullptr : psf, psf_size,
                   background, background_attenuation, truncate_negative_values, &pb);
  if (s != kOk) return s;
  return gradient_host(pb, sino, activity, attenuation, gradient);
}

// Alias with the words in the other order (et_array_attenuation_gradient).
int et_array_attenuation_gradient(float* sino, int* sino_size, float* activity, int* activity_size, float* gradient,
                                  int* gradient_size, float* cameras, int* cameras_size, float* psf, int* psf_size,
                                  float* attenuation, int* attenuation_size, float background,
                                  float background_attenuation, int GPU, int truncate_negative_values) {
  NRGB_API("et_array_attenuation_gradient");
  return et_array_gradient_attenuation(sino, sino_size, activity, activity_size, gradient, gradient_size, cameras,
                                       cameras_size, psf, psf_size, attenuation, attenuation_size, background,
                                       background_attenuation, GPU, truncate_negative_values);
}

// ------------------------------------------------------------ utilities
// emission-lib/_et_array_interface.cpp:896-920: the reference's PSF builder is a
// fixed 5 x 5 stub filled with ones; kept as is for drop-in behaviour.
int et_array_calculate_size_psf(unsigned int* psf_size_x, unsigned int* psf_size_y, float, float, float, float,
                                float, float) {
  NRGB_API("et_array_calculate_size_psf");
  *psf_size_x = 5;
  *psf_size_y = 5;
  return 0;
}

int et_array_make_psf(float* psf_data, unsigned int psf_size_x, unsigned int psf_size_y, float, float, float, float,
                      float, float, unsigned int N_psf_planes) {
  NRGB_API("et_array_make_psf");
  if (psf_size_x != 5 || psf_size_y != 5) {
    std::fprintf(stderr, "et_array_make_psf: PSF size mismatch. \n");
    return 1;
  }
  for (unsigned i = 0; i < psf_size_x * psf_size_y * N_psf_planes; ++i) psf_data[i] = 1.0f;
  return 0;
}

// emission-lib/_et_array_interface.cpp:923-937, same float arithmetic; a single
// camera gets the first angle (the reference divides by n-1 = 0 there).
int et_array_make_cameras(float* cameras_data, float firstcamera_deg, float lastcamera_deg, unsigned int n_cameras,
                          unsigned int rotation_axis) {
  NRGB_API("et_array_make_cameras");
  const float kPi = 3.141592653589793f;
  for (unsigned cam = 0; cam < n_cameras; ++cam) {
    float angle;
    if (n_cameras > 1)
      angle = (firstcamera_deg + (lastcamera_deg - firstcamera_deg) * static_cast<int>(cam) /
                                     static_cast<float>(n_cameras - 1)) /
              180.0f * kPi;
    else
      angle = firstcamera_deg / 180.0f * kPi;
    for (unsigned axis = 0; axis < 3; ++axis)
      cameras_data[cam + axis * n_cameras] = (axis == rotation_axis) ? angle : 0.0f;
  }
  return 0;
}

// emission-lib/_et_array_interface.cpp:112-156: rotate a volume about a centre.
int et_array_rotate(float* image, int* size, float* rotated_image, float* angles, float* centers, float background,
                    int axis_order, int GPU) {
  NRGB_API("et_array_rotate");
  (void)GPU;
  if (!size || size[0] <= 0 || size[1] <= 0 || size[2] <= 0) return kErrParameters;
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(size[0]) * size[1] * size[2];
  if ((s = ensure_arena(ds, fbytes(2 * nvox) + 512)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_in = cv.take<float>(nvox);
  float* d_out = cv.take<float>(nvox);
  float M[16];
  rotation_matrix(M, angles[0], angles[1], angles[2], centers[0], centers[1], centers[2], axis_order);
  if ((s = h2d(d_in, image, nvox, ds.stream)) != kOk) return finish(ds, s);
  s = general_rotate(d_in, d_out, size[0], size[1], size[2], M, background, ds.stream);
  if (s == kOk) s = d2h(rotated_image, d_out, nvox, ds.stream);
  return finish(ds, s);
}

// emission-lib/_et_array_interface.cpp:58-108: affine transformation of a
// volume, out(x) = trilinear(image, A x) with `background` outside, A the 4 x 4
// matrix affine_ptr in the interface's column-major order (affine_size {4, 4};
// the Matlab caller _et_affine_mex.cpp:110-118 passes it so).  The output has
// the image's size (the reference sizes it from the source and does not read
// transformed_image_size).  The reference itself never reads affine_ptr (a
// zeroed mat44 marked FIXME, so every voxel took the value of voxel 0); this
// applies the matrix, as its documentation states, with the same resampler as
// et_array_rotate.
int et_array_affine(float* image_ptr, int* image_size, float* transformed_image_ptr, int* transformed_image_size,
                    float* affine_ptr, int* affine_size, float background, int GPU) {
  NRGB_API("et_array_affine");
  (void)GPU;
  (void)transformed_image_size;
  if (!image_ptr || !image_size || !transformed_image_ptr || !affine_ptr || !affine_size) return kErrParameters;
  if (image_size[0] <= 0 || image_size[1] <= 0 || image_size[2] <= 0) return kErrParameters;
  if (affine_size[0] != 4 || affine_size[1] != 4) return kErrParameters;
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(image_size[0]) * image_size[1] * image_size[2];
  if ((s = ensure_arena(ds, fbytes(2 * nvox) + 512)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_in = cv.take<float>(nvox);
  float* d_out = cv.take<float>(nvox);
  float M[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) M[4 * i + j] = affine_ptr[i + 4 * j];
  if ((s = h2d(d_in, image_ptr, nvox, ds.stream)) != kOk) return finish(ds, s);
  s = general_rotate(d_in, d_out, image_size[0], image_size[1], image_size[2], M, background, ds.stream);
  if (s == kOk) s = d2h(transformed_image_ptr, d_out, nvox, ds.stream);
  return finish(ds, s);
}

// emission-lib/_et_array_interface.cpp:161-226: per-slice 2D convolution of
// an image [nx, ny, nz] with kernel slices [kx, ky, nz] (kx, ky odd), as the
// reference's GPU path computes it by FFT (emission-lib_gpu/
// _et_convolveFFT2D_gpu.cu:43-113: kernel centred at ((kx-1)/2, (ky-1)/2),
// image clamped to its border); here summed directly.  The output has the
// image's size (out_size is not read, as in the reference).  The reference's
// CPU path is a stub that returns 1 (_et.cpp:776-780) and its GPU path passes
// the nifti dim array shifted by one (dim[0] = 3 taken as the height).
int et_array_convolve(float* image, int* image_size, float* out, int* out_size, float* psf, int* psf_size, int GPU) {
  NRGB_API("et_array_convolve");
  (void)GPU;
  (void)out_size;
  if (!image || !image_size || !out || !psf || !psf_size) return kErrParameters;
  const int nx = image_size[0], ny = image_size[1], nz = image_size[2];
  const int kx = psf_size[0], ky = psf_size[1];
  if (nx <= 0 || ny <= 0 || nz <= 0 || kx <= 0 || ky <= 0 || kx % 2 != 1 || ky % 2 != 1 || psf_size[2] != nz)
    return kErrParameters;
  int s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nk = static_cast<size_t>(kx) * ky * nz;
  if ((s = ensure_arena(ds, fbytes(2 * nvox + nk) + 768)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_in = cv.take<float>(nvox);
  float* d_out = cv.take<float>(nvox);
  float* d_k = cv.take<float>(nk);
  if ((s = h2d(d_in, image, nvox, ds.stream)) != kOk) return finish(ds, s);
  if ((s = h2d(d_k, psf, nk, ds.stream)) != kOk) return finish(ds, s);
  s = general_convolve2d(d_in, d_out, nx, ny, nz, d_k, kx, ky, ds.stream);
  if (s == kOk) s = d2h(out, d_out, nvox, ds.stream);
  return finish(ds, s);
}

// ---------------------------------------------------------- OSEM / MLEM
// emission-lib/_et_array_interface.cpp:972-1054.  Subset of n_cameras /
// subset_order cameras drawn with rand() as the reference does; an index that
// rounds up to n_cameras is clamped to n_cameras - 1 (the reference reads one
// past the end there, :1006).
int et_array_osem_step(float* activity_data, int size_x, int size_y, unsigned int subset_order, float* sinogram_data,
                       int n_cameras, float* cameras_data, int use_attenuation, float* attenuation_data, int use_psf,
                       float* psf_data, unsigned int psf_size_x, unsigned int psf_size_y, float background,
                       float background_attenuation, float epsilon, int use_gpu) {
  NRGB_API("et_array_osem_step");
  (void)use_gpu;
  if (subset_order == 0 || n_cameras <= 0) return kErrParameters;
  const int nsub = n_cameras / static_cast<int>(subset_order);
  if (nsub <= 0) return kErrParameters;
  std::vector<int> idx(nsub);
  for (int c = 0; c < nsub; ++c) {
    const float R = random_0_1();
    unsigned v = static_cast<unsigned>(n_cameras * R);
    if (v >= static_cast<unsigned>(n_cameras)) v = n_cameras - 1;
    idx[c] = static_cast<int>(v);
  }
  return subset_step(activity_data, size_x, size_y, sinogram_data, n_cameras, cameras_data, idx, use_attenuation,
                     attenuation_data, use_psf, psf_data, psf_size_x, psf_size_y, background, background_attenuation,
                     epsilon);
}

// Deterministic variant of et_array_osem_step: the subset is given as camera
// indexes (the reference draws it from unseeded rand()).
int et_array_osem_step_subset(float* activity_data, int size_x, int size_y, float* sinogram_data, int n_cameras,
                              float* cameras_data, const int* camera_indexes, int n_subset, int use_attenuation,
                              float* attenuation_data, int use_psf, float* psf_data, unsigned int psf_size_x,
                              unsigned int psf_size_y, float background, float background_attenuation, float epsilon) {
  NRGB_API("et_array_osem_step_subset");
  if (!camera_indexes || n_subset <= 0) return kErrParameters;
  std::vector<int> idx(camera_indexes, camera_indexes + n_subset);
  return subset_step(activity_data, size_x, size_y, sinogram_data, n_cameras, cameras_data, idx, use_attenuation,
                     attenuation_data, use_psf, psf_data, psf_size_x, psf_size_y, background, background_attenuation,
                     epsilon);
}

// emission-lib/_et_array_interface.cpp:1561-1760 (GPU semantics of
// et_project_partial_gpu, emission-lib/_et.cpp:2106-2436; the reference's CPU
// path is a stub).  partialsum is [nx, ny, nz, n_cameras]; background_image
// [nx, ny] or NULL.
int et_array_project_partial(float* activity, int* activity_size, float* sinogram, int* sinogram_size,
                             float* partialsum, int* partialsum_size, float* cameras, int* cameras_size, float* psf,
                             int* psf_size, float* attenuation, int* attenuation_size, float background,
                             float* background_image, float background_attenuation, int GPU,
                             int truncate_negative_values, int do_rotate_partial) {
  NRGB_API("et_array_project_partial");
  (void)GPU;
  if (!activity_size || !cameras_size || !psf_size || !attenuation_size || !sinogram || !partialsum ||
      !partialsum_size)
    return kErrParameters;
  int asz[3] = {activity_size[0], activity_size[1], activity_size[2]};
  const bool no_act = all_zero3(asz);
  const bool no_psf = all_zero3(psf_size);
  const bool no_att = all_zero3(attenuation_size);
  if (no_act && no_att) return kErrParameters;
  if (no_act) std::memcpy(asz, attenuation_size, sizeof(asz));
  const int ncam = cameras_size[0], ncols = cameras_size[1];
  if (!(ncols == 1 || ncols == 3 || ncols == 6)) return kErrParameters;
  if (!no_psf && (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != asz[0])) return kErrParameters;
  const long long nvox = static_cast<long long>(asz[0]) * asz[1] * asz[2];
  if (static_cast<long long>(partialsum_size[0]) * partialsum_size[1] * partialsum_size[2] * partialsum_size[3] <
      nvox * ncam)
    return kErrParameters;
  if (sinogram_size &&
      static_cast<long long>(sinogram_size[0]) * sinogram_size[1] * sinogram_size[2] <
          static_cast<long long>(asz[0]) * asz[1] * ncam)
    return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, ncam, ncols, asz, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(asz[0], asz[1], asz[2], cc, no_psf ? nullptr : psf, psf_size, background, background_attenuation,
                   truncate_negative_values, &pb);
  if (s != kOk) return s;
  return project_partial_host(pb, no_act ? nullptr : activity, no_att ? nullptr : attenuation, background_image,
                              sinogram, partialsum, do_rotate_partial);
}

// emission-lib/_et_array_interface.cpp:1135-1340 (et_fisher_grid,
// emission-lib/_et.cpp:531-746): Fisher information of the grid points of
// grid_ptr (values 1..n, n = fisher_size[0]) for the projection of the
// activity (truncated).  fisher_prior_ptr may be NULL.  A PSF is required
// (the reference dereferences it unconditionally).
int et_array_fisher_grid(float* activity_ptr, int* activity_size, float* cameras, int* cameras_size, float* psf,
                         int* psf_size, float* grid_ptr, float* fisher_ptr, float* fisher_prior_ptr, int* fisher_size,
                         float* attenuation, int* attenuation_size, float epsilon, float background,
                         float background_attenuation, int GPU) {
  NRGB_API("et_array_fisher_grid");
  (void)epsilon;
  (void)GPU;
  if (!activity_ptr || !activity_size || !cameras || !cameras_size || !psf || !psf_size || !grid_ptr ||
      !fisher_ptr || !fisher_size || !attenuation_size)
    return kErrParameters;
  const int nx = activity_size[0], ny = activity_size[1], nz = activity_size[2];
  const int ncam = cameras_size[0], ncols = cameras_size[1], n = fisher_size[0];
  if (!(ncols == 1 || ncols == 3 || ncols == 6) || n <= 0 || nx <= 0 || ny <= 0 || nz <= 0) return kErrParameters;
  if (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != nx) return kErrParameters;
  const bool no_att = all_zero3(attenuation_size);
  std::vector<int> xyz;
  int s = grid_points(grid_ptr, nx, ny, nz, n, &xyz);
  if (s != kOk) return s;
  Cameras cc;
  const int asz[3] = {nx, ny, nz};
  if ((s = expand_cameras(cameras, ncam, ncols, asz, &cc)) != kOk) return s;
  Problem pb;
  if ((s = make_problem(nx, ny, nz, cc, psf, psf_size, background, background_attenuation, 1, &pb)) != kOk) return s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nvox = static_cast<size_t>(nx) * ny * nz, nsino = static_cast<size_t>(nx) * ny * ncam;
  const size_t extra = sizeof(int) * (3 * static_cast<size_t>(n) * (ncam + 1)) +
                       sizeof(float) * (static_cast<size_t>(psf_size[0]) * psf_size[1] * psf_size[2] +
                                        2 * static_cast<size_t>(n) * n) + 8 * 256;
  const size_t ws = project_workspace(pb, true, !no_att);
  if ((s = ensure_arena(ds, fbytes(2 * nvox + nsino) + 4 * 256 + ws + extra)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_act = cv.take<float>(nvox);
  float* d_att = no_att ? nullptr : cv.take<float>(nvox);
  float* d_sino = cv.take<float>(nsino);
  char* w = cv.take<char>(ws);
  cudaStream_t st = ds.stream;
  if ((s = h2d(d_act, activity_ptr, nvox, st)) != kOk) return finish(ds, s);
  if (d_att && (s = h2d(d_att, attenuation, nvox, st)) != kOk) return finish(ds, s);
  g_last_path = (use_fused(pb) || use_fused_x(pb)) ? 1 : 2;
  if ((s = project_device(pb, d_act, d_att, d_sino, w, ws, &ds.staging, st)) != kOk) return finish(ds, s);
  s = fisher_from_projection(ds, cv, d_sino, nx, ny, nz, cc, xyz, n, psf, psf_size[0], psf_size[1], psf_size[2],
                             fisher_ptr, fisher_prior_ptr, st);
  return finish(ds, s);
}

// emission-lib/_et_array_interface.cpp:1344-1540: the same from a given
// projection (sinogram_size = {nx, ny, n_cameras}); the grid volume has
// bkpr_size and the camera centres follow (nx, ny, nx).
int et_array_fisher_grid_projection(float* sinogram_ptr, int* sinogram_size, int* bkpr_size, float* cameras,
                                    int* cameras_size, float* psf, int* psf_size, float* grid_ptr, float* fisher_ptr,
                                    float* fisher_prior_ptr, int* fisher_size, float* attenuation,
                                    int* attenuation_size, float epsilon, float background,
                                    float background_attenuation, int GPU) {
  NRGB_API("et_array_fisher_grid_projection");
  (void)epsilon;
  (void)GPU;
  (void)attenuation;
  (void)attenuation_size;
  (void)background;
  (void)background_attenuation;
  if (!sinogram_ptr || !sinogram_size || !bkpr_size || !cameras || !cameras_size || !psf || !psf_size || !grid_ptr ||
      !fisher_ptr || !fisher_size)
    return kErrParameters;
  const int npx = sinogram_size[0], npy = sinogram_size[1], ncam = cameras_size[0], ncols = cameras_size[1];
  const int n = fisher_size[0];
  if (!(ncols == 1 || ncols == 3 || ncols == 6) || n <= 0 || npx <= 0 || npy <= 0 || sinogram_size[2] < ncam)
    return kErrParameters;
  if (psf_size[0] % 2 != 1 || psf_size[1] % 2 != 1 || psf_size[2] != bkpr_size[0]) return kErrParameters;
  std::vector<int> xyz;
  int s = grid_points(grid_ptr, bkpr_size[0], bkpr_size[1], bkpr_size[2], n, &xyz);
  if (s != kOk) return s;
  Cameras cc;
  const int csz[3] = {npx, npy, npx};
  if ((s = expand_cameras(cameras, ncam, ncols, csz, &cc)) != kOk) return s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t nsino = static_cast<size_t>(npx) * npy * ncam;
  const size_t extra = sizeof(int) * (3 * static_cast<size_t>(n) * (ncam + 1)) +
                       sizeof(float) * (static_cast<size_t>(psf_size[0]) * psf_size[1] * psf_size[2] +
                                        2 * static_cast<size_t>(n) * n) + 8 * 256;
  if ((s = ensure_arena(ds, fbytes(nsino) + 256 + extra)) != kOk) return s;
  Carver cv(ds.arena, ds.arena_bytes);
  float* d_sino = cv.take<float>(nsino);
  cudaStream_t st = ds.stream;
  g_last_path = 2;
  if ((s = h2d(d_sino, sinogram_ptr, nsino, st)) != kOk) return finish(ds, s);
  s = fisher_from_projection(ds, cv, d_sino, npx, npy, bkpr_size[2], cc, xyz, n, psf, psf_size[0], psf_size[1],
                             psf_size[2], fisher_ptr, fisher_prior_ptr, st);
  return finish(ds, s);
}

// emission-lib/_et_array_interface.cpp:1080-1131.
int et_array_mlem_step(float* activity_data, int size_x, int size_y, float* sinogram_data, int n_cameras,
                       float* cameras_data, int use_attenuation, float* attenuation_data, int use_psf,
                       float* psf_data, unsigned int psf_size_x, unsigned int psf_size_y, float background,
                       float background_attenuation, float epsilon, int use_gpu) {
  NRGB_API("et_array_mlem_step");
  (void)use_gpu;
  if (n_cameras <= 0) return kErrParameters;
  std::vector<int> idx(n_cameras);
  for (int c = 0; c < n_cameras; ++c) idx[c] = c;
  return subset_step(activity_data, size_x, size_y, sinogram_data, n_cameras, cameras_data, idx, use_attenuation,
                     attenuation_data, use_psf, psf_data, psf_size_x, psf_size_y, background, background_attenuation,
                     epsilon);
}

// emission-lib/_et_array_interface.cpp:940-957.
int et_array_osem(float* activity_data, unsigned int size_x, unsigned int size_y, unsigned int subset_order,
                  float* sinogram_data, int n_cameras, float firstcamera, float lastcamera, unsigned int rotation_axis,
                  int iterations, int use_attenuation, float* attenuation_data, int use_psf, float* psf_data,
                  unsigned int psf_size_x, unsigned int psf_size_y, float background, float background_attenuation,
                  float epsilon, int use_gpu) {
  NRGB_API("et_array_osem");
  const size_t n = static_cast<size_t>(size_x) * size_y * size_x;
  for (size_t i = 0; i < n; ++i) activity_data[i] = 1.0f;
  std::vector<float> cams(3 * static_cast<size_t>(n_cameras));
  int status = et_array_make_cameras(cams.data(), firstcamera, lastcamera, n_cameras, rotation_axis);
  for (int it = 0; it < iterations; ++it)
    status += et_array_osem_step(activity_data, size_x, size_y, subset_order, sinogram_data, n_cameras, cams.data(),
                                 use_attenuation, attenuation_data, use_psf, psf_data, psf_size_x, psf_size_y,
                                 background, background_attenuation, epsilon, use_gpu);
  return status;
}

// emission-lib/_et_array_interface.cpp:1058-1076.
int et_array_mlem(float* activity_data, unsigned int size_x, unsigned int size_y, float* sinogram_data, int n_cameras,
                  float firstcamera, float lastcamera, unsigned int rotation_axis, int iterations, int use_attenuation,
                  float* attenuation_data, int use_psf, float* psf_data, unsigned int psf_size_x,
                  unsigned int psf_size_y, float background, float background_attenuation, float epsilon,
                  int use_gpu) {
  NRGB_API("et_array_mlem");
  const size_t n = static_cast<size_t>(size_x) * size_y * size_x;
  for (size_t i = 0; i < n; ++i) activity_data[i] = 1.0f;
  std::vector<float> cams(3 * static_cast<size_t>(n_cameras));
  int status = et_array_make_cameras(cams.data(), firstcamera, lastcamera, n_cameras, rotation_axis);
  for (int it = 0; it < iterations; ++it)
    status += et_array_mlem_step(activity_data, size_x, size_y, sinogram_data, n_cameras, cams.data(),
                                 use_attenuation, attenuation_data, use_psf, psf_data, psf_size_x, psf_size_y,
                                 background, background_attenuation, epsilon, use_gpu);
  return status;
}

}  // extern "C"

// ------------------------------------------------ device-pointer additions
// Same operations on device buffers (nifti layout) on the caller's stream;
// cameras and PSF stay host arrays.  The call returns once the work is
// enqueued.  No counterpart in the reference (its GPU path copies host
// buffers in and out on every call).
namespace {

int project_device_call(const float* d_activity, const float* d_attenuation, const int* size, float* d_sinogram,
                        const float* cameras, const int* cameras_size, const float* psf, const int* psf_size,
                        float background, float background_attenuation, int truncate, bool bf16, void* stream) {
  if (!size || !cameras || !cameras_size || (!d_activity && !d_attenuation) || !d_sinogram) return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], size, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(size[0], size[1], size[2], cc, psf, psf_size, background, background_attenuation, truncate, &pb);
  if (s != kOk) return s;
  if (bf16) {
    pb.storage = kStorageBF16;
    pb.input_bf16 = true;
  }
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t ws = project_workspace(pb, d_activity != nullptr, d_attenuation != nullptr);
  if ((s = ensure_arena(ds, ws)) != kOk) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamWaitEvent(st, ds.last_use, 0);
  g_last_path = ((use_fused(pb) || use_fused_x(pb)) && d_activity) ? 1 : 2;
  s = project_device(pb, d_activity, d_attenuation, d_sinogram, ds.arena, ds.arena_bytes, &ds.staging, st);
  cudaEventRecord(ds.last_use, st);
  return s;
}

int backproject_device_call(const float* d_sinogram, const float* d_attenuation, const int* size, float* d_out,
                            const float* cameras, const int* cameras_size, const float* psf, const int* psf_size,
                            float background, float background_attenuation, int truncate, int mode, bool bf16,
                            void* stream) {
  if (!size || !cameras || !cameras_size || !d_sinogram || !d_out || (mode != kBackReference && mode != kBackAdjoint))
    return kErrParameters;
  Cameras cc;
  // camera centres: the reference backprojector's {size0, size1, size0} rule;
  // the exact transpose of the projector takes the projector's (the volume
  // size), which differ when nz != nx
  const int csz[3] = {size[0], size[1], mode == kBackAdjoint ? size[2] : size[0]};
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], csz, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(size[0], size[1], size[2], cc, psf, psf_size, background, background_attenuation, truncate, &pb);
  if (s != kOk) return s;
  pb.back_mode = mode;
  if (bf16) {
    pb.storage = kStorageBF16;
    pb.input_bf16 = true;
  }
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t ws = backproject_workspace(pb, d_attenuation != nullptr);
  if ((s = ensure_arena(ds, ws)) != kOk) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamWaitEvent(st, ds.last_use, 0);
  g_last_path = (use_fused(pb) || use_fused_x(pb)) ? 1 : 2;
  s = backproject_device(pb, d_sinogram, d_attenuation, d_out, ds.arena, ds.arena_bytes, &ds.staging, st);
  cudaEventRecord(ds.last_use, st);
  return s;
}

int pair_device_call(const float* d_activity, const float* d_attenuation, const int* size, float* d_sinogram,
                     const float* d_backproject_input, float* d_backprojection, const float* cameras,
                     const int* cameras_size, const float* psf, const int* psf_size, float background,
                     float background_attenuation, int truncate, int mode, bool bf16, void* stream) {
  if (!size || !cameras || !cameras_size || !d_activity || !d_sinogram || !d_backprojection ||
      (mode != kBackReference && mode != kBackAdjoint))
    return kErrParameters;
  // camera centres: the projector's from the volume size, the
  // backprojector's with the reference's {size0, size1, size0} rule (the
  // exact transpose: the projector's)
  Cameras cc, cb;
  const int csz[3] = {size[0], size[1], mode == kBackAdjoint ? size[2] : size[0]};
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], size, &cc);
  if (s != kOk) return s;
  if ((s = expand_cameras(cameras, cameras_size[0], cameras_size[1], csz, &cb)) != kOk) return s;
  Problem pb, pbb;
  s = make_problem(size[0], size[1], size[2], cc, psf, psf_size, background, background_attenuation, truncate, &pb);
  if (s != kOk) return s;
  s = make_problem(size[0], size[1], size[2], cb, psf, psf_size, background, background_attenuation, truncate, &pbb);
  if (s != kOk) return s;
  pb.back_mode = pbb.back_mode = mode;
  if (bf16) {
    pb.storage = pbb.storage = kStorageBF16;
    pb.input_bf16 = pbb.input_bf16 = true;
  }
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t ws = std::max(pair_workspace(pb, d_attenuation != nullptr, d_backproject_input != nullptr),
                             backproject_workspace(pbb, d_attenuation != nullptr));
  if ((s = ensure_arena(ds, ws)) != kOk) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamWaitEvent(st, ds.last_use, 0);
  g_last_path = (use_fused(pb) || use_fused_x(pb)) ? 1 : 2;
  s = pair_device(pb, pbb, d_activity, d_attenuation, d_sinogram, d_backproject_input, d_backprojection, ds.arena,
                  ds.arena_bytes, &ds.staging, st);
  cudaEventRecord(ds.last_use, st);
  return s;
}

}  // namespace

extern "C" {

// Projection and backprojection in one call (see the header).
int nrgb_project_backproject_device(const float* d_activity, const float* d_attenuation, const int* size,
                                    float* d_sinogram, const float* d_backproject_input, float* d_backprojection,
                                    const float* cameras, const int* cameras_size, const float* psf,
                                    const int* psf_size, float background, float background_attenuation,
                                    int truncate, int mode, void* stream) {
  NRGB_API("nrgb_project_backproject_device");
  return pair_device_call(d_activity, d_attenuation, size, d_sinogram, d_backproject_input, d_backprojection,
                          cameras, cameras_size, psf, psf_size, background, background_attenuation, truncate, mode,
                          false, stream);
}

// The same with bfloat16 activity / mu (see the header).
int nrgb_project_backproject_device_bf16(const void* d_activity, const void* d_attenuation, const int* size,
                                         float* d_sinogram, const float* d_backproject_input, float* d_backprojection,
                                         const float* cameras, const int* cameras_size, const float* psf,
                                         const int* psf_size, float background, float background_attenuation,
                                         int truncate, int mode, void* stream) {
  NRGB_API("nrgb_project_backproject_device_bf16");
  return pair_device_call(static_cast<const float*>(d_activity), static_cast<const float*>(d_attenuation), size,
                          d_sinogram, d_backproject_input, d_backprojection, cameras, cameras_size, psf, psf_size,
                          background, background_attenuation, truncate, mode, true, stream);
}

int nrgb_project_device(const float* d_activity, const float* d_attenuation, const int* size, float* d_sinogram,
                        const float* cameras, const int* cameras_size, const float* psf, const int* psf_size,
                        float background, float background_attenuation, int truncate, void* stream) {
  NRGB_API("nrgb_project_device");
  return project_device_call(d_activity, d_attenuation, size, d_sinogram, cameras, cameras_size, psf, psf_size,
                             background, background_attenuation, truncate, false, stream);
}

// mode: 0 = the reference's inverse-rotation backprojector; 1 = the exact
// transpose of the projector (for gradients).
int nrgb_backproject_device(const float* d_sinogram, const float* d_attenuation, const int* size, float* d_out,
                            const float* cameras, const int* cameras_size, const float* psf, const int* psf_size,
                            float background, float background_attenuation, int truncate, int mode, void* stream) {
  NRGB_API("nrgb_backproject_device");
  return backproject_device_call(d_sinogram, d_attenuation, size, d_out, cameras, cameras_size, psf, psf_size,
                                 background, background_attenuation, truncate, mode, false, stream);
}

// bfloat16 activity / mu (nifti order) with float32 arithmetic and
// Kahan-compensated depth sums; sinograms and backprojections stay float32.
int nrgb_project_device_bf16(const void* d_activity, const void* d_attenuation, const int* size, float* d_sinogram,
                             const float* cameras, const int* cameras_size, const float* psf, const int* psf_size,
                             float background, float background_attenuation, int truncate, void* stream) {
  NRGB_API("nrgb_project_device_bf16");
  return project_device_call(static_cast<const float*>(d_activity), static_cast<const float*>(d_attenuation), size,
                             d_sinogram, cameras, cameras_size, psf, psf_size, background, background_attenuation,
                             truncate, true, stream);
}

int nrgb_backproject_device_bf16(const float* d_sinogram, const void* d_attenuation, const int* size, float* d_out,
                                 const float* cameras, const int* cameras_size, const float* psf, const int* psf_size,
                                 float background, float background_attenuation, int truncate, int mode,
                                 void* stream) {
  NRGB_API("nrgb_backproject_device_bf16");
  return backproject_device_call(d_sinogram, static_cast<const float*>(d_attenuation), size, d_out, cameras,
                                 cameras_size, psf, psf_size, background, background_attenuation, truncate, mode, true,
                                 stream);
}

// float64 reference run: the general-orientation projector and the reference
// backprojector with geometry, PSF and all arithmetic in double.
int nrgb_project_device_f64(const double* d_activity, const double* d_attenuation, const int* size,
                            double* d_sinogram, const float* cameras, const int* cameras_size, const float* psf,
                            const int* psf_size, double background, double background_attenuation, int truncate,
                            void* stream) {
  NRGB_API("nrgb_project_device_f64");
  if (!size || !cameras || !cameras_size || (!d_activity && !d_attenuation) || !d_sinogram) return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], size, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(size[0], size[1], size[2], cc, psf, psf_size, static_cast<float>(background),
                   static_cast<float>(background_attenuation), truncate, &pb);
  if (s != kOk) return s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  if ((s = ensure_arena(ds, workspace64(pb))) != kOk) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamWaitEvent(st, ds.last_use, 0);
  g_last_path = 2;
  s = project_device64(pb, d_activity, d_attenuation, d_sinogram, ds.arena, ds.arena_bytes, st);
  cudaEventRecord(ds.last_use, st);
  return s;
}

int nrgb_backproject_device_f64(const double* d_sinogram, const double* d_attenuation, const int* size,
                                double* d_out, const float* cameras, const int* cameras_size, const float* psf,
                                const int* psf_size, double background, double background_attenuation, int truncate,
                                void* stream) {
  NRGB_API("nrgb_backproject_device_f64");
  if (!size || !cameras || !cameras_size || !d_sinogram || !d_out) return kErrParameters;
  Cameras cc;
  const int csz[3] = {size[0], size[1], size[0]};
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], csz, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(size[0], size[1], size[2], cc, psf, psf_size, static_cast<float>(background),
                   static_cast<float>(background_attenuation), truncate, &pb);
  if (s != kOk) return s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  if ((s = ensure_arena(ds, workspace64(pb))) != kOk) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamWaitEvent(st, ds.last_use, 0);
  g_last_path = 2;
  s = backproject_device64(pb, d_sinogram, d_attenuation, d_out, ds.arena, ds.arena_bytes, st);
  cudaEventRecord(ds.last_use, st);
  return s;
}

int nrgb_osem_ratio_device_f64(const double* d_counts, double* d_projection, long long n, double epsilon,
                               void* stream) {
  NRGB_API("nrgb_osem_ratio_device_f64");
  if (!d_counts || !d_projection || n < 0) return kErrParameters;
  if (n == 0) return kOk;
  return osem_ratio64(d_counts, d_projection, static_cast<size_t>(n), epsilon, static_cast<cudaStream_t>(stream));
}

int nrgb_osem_update_device_f64(double* d_activity, const double* d_numerator, const double* d_denominator,
                                long long n, double epsilon, void* stream) {
  NRGB_API("nrgb_osem_update_device_f64");
  if (!d_activity || !d_numerator || !d_denominator || n < 0) return kErrParameters;
  if (n == 0) return kOk;
  return osem_update64(d_activity, d_numerator, d_denominator, static_cast<size_t>(n), epsilon,
                       static_cast<cudaStream_t>(stream));
}

// Exact gradient with respect to mu of sum(g * P(activity, mu)) where P is the
// projector (no truncation) and g = d_grad_sinogram, all device buffers.
int nrgb_attenuation_grad_device(const float* d_grad_sinogram, const float* d_activity, const float* d_attenuation,
                                 const int* size, float* d_out, const float* cameras, const int* cameras_size,
                                 const float* psf, const int* psf_size, float background,
                                 float background_attenuation, void* stream) {
  NRGB_API("nrgb_attenuation_grad_device");
  if (!size || !cameras || !cameras_size || !d_grad_sinogram || !d_activity || !d_attenuation || !d_out)
    return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], size, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(size[0], size[1], size[2], cc, psf, psf_size, background, background_attenuation, 0, &pb);
  if (s != kOk) return s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t ws = dmu_workspace(pb);
  if ((s = ensure_arena(ds, ws)) != kOk) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamWaitEvent(st, ds.last_use, 0);
  g_last_path = (use_fused(pb) || use_fused_x(pb)) ? 1 : 2;
  s = dmu_device(pb, d_grad_sinogram, d_activity, d_attenuation, d_out, ds.arena, ds.arena_bytes, &ds.staging, st);
  cudaEventRecord(ds.last_use, st);
  return s;
}

// et_array_gradient_attenuation on device buffers (nifti order, float32),
// enqueued on `stream`.
int nrgb_gradient_attenuation_device(const float* d_sinogram, const float* d_activity, const float* d_attenuation,
                                     const int* size, float* d_out, const float* cameras, const int* cameras_size,
                                     const float* psf, const int* psf_size, float background,
                                     float background_attenuation, int truncate, void* stream) {
  NRGB_API("nrgb_gradient_attenuation_device");
  if (!size || !cameras || !cameras_size || !d_sinogram || !d_activity || !d_attenuation || !d_out)
    return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], size, &cc);
  if (s != kOk) return s;
  Problem pb;
  s = make_problem(size[0], size[1], size[2], cc, psf, psf_size, background, background_attenuation, truncate, &pb);
  if (s != kOk) return s;
  DeviceState& ds = current_device_state(&s);
  if (s != kOk) return s;
  std::lock_guard<std::mutex> lk(ds.mu);
  const size_t ws = gradient_workspace(pb);
  if ((s = ensure_arena(ds, ws)) != kOk) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamWaitEvent(st, ds.last_use, 0);
  g_last_path = (use_fused(pb) || use_fused_x(pb)) && pb.storage == kStorageF32 ? 1 : 2;
  s = gradient_device(pb, d_sinogram, d_activity, d_attenuation, d_out, ds.arena, ds.arena_bytes, &ds.staging, st);
  cudaEventRecord(ds.last_use, st);
  return s;
}

// The two elementwise stages of et_array_osem_step on device buffers, for
// callers that assemble the step themselves (e.g. with partial
// backprojections summed across processes in between):
// ratio (emission-lib/_et_array_interface.cpp:1022-1028) overwrites the
// projection with y / p (y / eps where p < eps); update (:1036-1044) does
// x *= num / max(den, eps).
int nrgb_osem_ratio_device(const float* d_counts, float* d_projection, long long n, float epsilon, void* stream) {
  NRGB_API("nrgb_osem_ratio_device");
  if (!d_counts || !d_projection || n < 0) return kErrParameters;
  if (n == 0) return kOk;
  return osem_ratio(d_counts, d_projection, static_cast<size_t>(n), epsilon, static_cast<cudaStream_t>(stream));
}

int nrgb_osem_update_device(float* d_activity, const float* d_numerator, const float* d_denominator, long long n,
                            float epsilon, void* stream) {
  NRGB_API("nrgb_osem_update_device");
  if (!d_activity || !d_numerator || !d_denominator || n < 0) return kErrParameters;
  if (n == 0) return kOk;
  return osem_update(d_activity, d_numerator, d_denominator, static_cast<size_t>(n), epsilon,
                     static_cast<cudaStream_t>(stream));
}

// Tuning table of the fused backprojector: cameras per scratch group for the
// shape (nx, ny, nz, n_cameras); an all-zero shape sets the default.
int nrgb_set_backproject_group(int nx, int ny, int nz, int ncam, int group) {
  NRGB_API("nrgb_set_backproject_group");
  if (group < 0 || group > 64) return kErrParameters;
  set_tuned_group(nx, ny, nz, ncam, group);
  return kOk;
}

int nrgb_get_backproject_group(int nx, int ny, int nz, int ncam) { return tuned_group(nx, ny, nz, ncam); }

// Tuning table of the fused projector: depth slabs (cluster size 2, 4, 8,
// 16; 0 removes the entry) for the shape (nx, ny, nz, n_cameras).
int nrgb_set_project_slabs(int nx, int ny, int nz, int ncam, int slabs) {
  NRGB_API("nrgb_set_project_slabs");
  if (slabs != 0 && slabs != 2 && slabs != 4 && slabs != 8 && slabs != 16) return kErrParameters;
  set_tuned_project_slabs(nx, ny, nz, ncam, slabs);
  return kOk;
}

int nrgb_get_project_slabs(int nx, int ny, int nz, int ncam) { return tuned_project_slabs(nx, ny, nz, ncam); }

// Mirror cameras: 1 (default) serves a camera at the opposite angle about the
// grid centre from the same bilinear samples; 0 computes every camera from
// its own matrix.  Applies to calls made afterwards.
int nrgb_set_mirror_pairs(int on) {
  NRGB_API("nrgb_set_mirror_pairs");
  set_mirror_pairs(on);
  return kOk;
}

int nrgb_get_mirror_pairs(void) { return mirror_pairs(); }

// Deterministic exact-transpose backprojection and d/dmu on the fused kernels
// (group scratch + transposed gather): 1 on, 0 (default) vector reductions.
int nrgb_set_deterministic(int on) {
  NRGB_API("nrgb_set_deterministic");
  set_deterministic(on);
  return kOk;
}

int nrgb_get_deterministic(void) { return deterministic(); }

// The mirror units the fused kernels would form for these cameras and this
// volume (host only): {camera, mate} pairs, mate -1 when unpaired, in the
// cameras' order; *n_units = 0 when every camera runs on its own (no
// opposite-angle pairs about the grid centre, cameras off the gantry forms,
// or nrgb_set_mirror_pairs(0)).
int nrgb_mirror_units(const float* cameras, const int* cameras_size, const int* size, int* out_units, int max_units,
                      int* n_units) {
  NRGB_API("nrgb_mirror_units");
  if (!cameras || !cameras_size || !size || !n_units || max_units < 0 || (max_units > 0 && !out_units))
    return kErrParameters;
  Cameras cc;
  int s = expand_cameras(cameras, cameras_size[0], cameras_size[1], size, &cc);
  if (s != kOk) return s;
  Problem pb;
  if ((s = make_problem(size[0], size[1], size[2], cc, nullptr, nullptr, 0.0f, 0.0f, 0, &pb)) != kOk) return s;
  const std::vector<int>& u = pb.xgantry ? pb.units_x : pb.units;
  const int n = static_cast<int>(u.size() / 2);
  *n_units = n;
  if (n > max_units) return kErrParameters;
  std::copy(u.begin(), u.end(), out_units);
  return kOk;
}

// Row windows of the fused kernels for ny rows and a PSF of width psf_k (0:
// none), host only: {first row, rows, first valid row, end of valid rows}
// per window (valid rows relative to the first row).
int nrgb_row_windows(int ny, int psf_k, int* out, int max_windows, int* n_windows) {
  NRGB_API("nrgb_row_windows");
  if (ny < 1 || psf_k < 0 || !n_windows || max_windows < 0 || (max_windows > 0 && !out)) return kErrParameters;
  std::vector<int> w(4 * static_cast<size_t>(ny + 1));
  const int n = yg_row_windows(ny, psf_k, w.data(), ny + 1);
  if (n < 0) return kErrParameters;
  *n_windows = n;
  if (n > max_windows) return kErrParameters;
  std::copy(w.begin(), w.begin() + 4 * n, out);
  return kOk;
}

// 1 when the last call of this thread ran the fused y-gantry kernels, 2 when
// it ran the general-orientation path, 0 before any call.
int nrgb_last_path(void) { return g_last_path; }

}  // extern "C"
