// Engine: problem description, per-device work space and the device-pointer
// implementations behind the C-ABI.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "et_common.h"
#include "et_geometry.h"

namespace nrgb {

// One projection / backprojection problem: grid, cameras, PSF, backgrounds.
struct Problem {
  int nx = 0, ny = 0, nz = 0;
  Cameras cams;
  std::vector<CamGeom> geom;
  std::vector<int> units;  // mirror-camera units of the fused projector (mirror_units), or empty
  bool ygantry = false;
  // Cameras rotating about x with nx a multiple of 4: the gantry kernels run
  // on the nifti arrays directly with x and y exchanged (engine geometry,
  // separated PSF with row and column kernels exchanged, mirror units).
  bool xgantry = false;
  std::vector<CamGeom> geom_x;
  std::vector<float> psf_sep_x;
  std::vector<int> units_x;
  int psf_k = 0;               // 0: no PSF
  std::vector<float> psf_sep;  // [nz][2k]
  const float* psf_host = nullptr;  // the caller's PSF, valid during the call only
  float bg = 0.0f, bg_att = 0.0f;
  int truncate = 0;
  int back_mode = kBackReference;
  int group = 16;  // cameras per backprojection scratch group (set from the tuning table)
  int pslabs = 0;  // projector depth slabs (tuning table; 0: the launcher's choice)
  // Storage of the sampled volumes inside the fused kernels, and whether the
  // caller's activity / mu buffers are bfloat16 (nifti order) rather than
  // float32.  bfloat16 inputs imply bfloat16 storage; the general-orientation
  // path widens them to float32 first.
  int storage = kStorageF32;
  bool input_bf16 = false;
  // Deterministic exact-transpose backprojection and d/dmu on the fused
  // kernels (scratch + transposed gather instead of vector reductions); set
  // from the library-wide switch when the problem is made.
  int det = 0;
};

// Build a Problem; psf may be null.  psf_size = {kx, ky, planes}.  Returns
// kErrParameters for shapes the engine does not support (non-square or even
// PSF, fewer PSF planes than nz).
int make_problem(int nx, int ny, int nz, const Cameras& cams, const float* psf, const int* psf_size, float bg,
                 float bg_att, int truncate, Problem* out);

// Whether the fused y-gantry kernels handle this problem (any ny: volumes
// taller than 128 rows run in row windows inside the kernels' launchers).
bool use_fused(const Problem& pb);
// Whether the gantry kernels handle this problem with x and y exchanged
// (cameras about x; the direct device and host-buffer entry points).
bool use_fused_x(const Problem& pb);

// Cameras per backprojection scratch group for a problem shape (tuning table;
// all-zero shape = default for shapes without an entry).
int tuned_group(int nx, int ny, int nz, int ncam);
void set_tuned_group(int nx, int ny, int nz, int ncam, int group);
// Projector depth slabs (cluster size 2, 4 or 8) for a shape; 0 = none
// recorded (the launcher then chooses).
int tuned_project_slabs(int nx, int ny, int nz, int ncam);
void set_tuned_project_slabs(int nx, int ny, int nz, int ncam, int slabs);
// Whether new problems serve mirror cameras (opposite angles) from shared
// samples (1, the default) or every camera from its own matrix (0).
void set_mirror_pairs(int on);
int mirror_pairs();
void set_deterministic(int on);
int deterministic();

// Pinned, double-buffered staging of the per-call parameters (camera
// matrices, separated PSF): copies from pinned memory stay asynchronous,
// where a copy from pageable memory would synchronise the stream.
struct Staging {
  char* pinned[2] = {nullptr, nullptr};
  size_t bytes[2] = {0, 0};
  cudaEvent_t done[2] = {nullptr, nullptr};
  int slot = 0;
};

// Per-device state: a library-owned stream, a growing device arena, an event
// that orders successive users of the arena on any stream, and the staging.
struct DeviceState {
  std::mutex mu;
  int device = 0;
  cudaStream_t stream = nullptr;
  char* arena = nullptr;
  size_t arena_bytes = 0;
  cudaEvent_t last_use = nullptr;
  Staging staging;
};

// Host-side fault injection: the next n work-space allocations that would
// grow a device arena fail with kErrAllocGpu instead (no CUDA call is made).
void fail_next_allocations(int n);

// Lock the current device's state (created on first use) for the caller.
DeviceState& current_device_state(int* status);

// Carves 256-byte aligned pieces out of the arena.
class Carver {
 public:
  Carver(char* base, size_t cap) : base_(base), cap_(cap) {}
  template <class T>
  T* take(size_t count) {
    const size_t bytes = (count * sizeof(T) + 255) / 256 * 256;
    if (off_ + bytes > cap_) return nullptr;
    T* p = reinterpret_cast<T*>(base_ + off_);
    off_ += bytes;
    return p;
  }
  size_t used() const { return off_; }

 private:
  char* base_;
  size_t cap_;
  size_t off_ = 0;
};

// Ensure the arena holds at least `bytes`.
int ensure_arena(DeviceState& ds, size_t bytes);

// Device-pointer operations (nifti layout in and out, stream-ordered).
size_t project_workspace(const Problem& pb, bool has_act, bool has_att);
size_t backproject_workspace(const Problem& pb, bool has_att);
size_t gradient_workspace(const Problem& pb);
int project_device(const Problem& pb, const float* d_act, const float* d_att, float* d_sino, char* ws, size_t ws_bytes,
                   Staging* stg, cudaStream_t st);
int backproject_device(const Problem& pb, const float* d_sino, const float* d_att, float* d_out, char* ws,
                       size_t ws_bytes, Staging* stg, cudaStream_t st);
int gradient_device(const Problem& pb, const float* d_sino, const float* d_act, const float* d_att, float* d_out,
                    char* ws, size_t ws_bytes, Staging* stg, cudaStream_t st);
// Projection followed by a backprojection with the same cameras, PSF and mu
// (d_bk_in, or the projection itself when null), in one sequence: for
// cameras about the gantry axis the volumes are laid out once, the projector
// leaves the backprojector's transmission carries, and the projection feeds
// the backprojector in its column layout.
size_t pair_workspace(const Problem& pb, bool has_att, bool has_input);
// pb: the projection's problem; pb_back: the backprojection's (camera
// centres from its own size rule).
int pair_device(const Problem& pb, const Problem& pb_back, const float* d_act, const float* d_att, float* d_sino,
                const float* d_bk_in, float* d_bk, char* ws, size_t ws_bytes, Staging* stg, cudaStream_t st);
// Projection with partial sums (et_project_partial): d_partial receives
// [ncam][nz][ny][nx]; d_bg_image [ny][nx] or null.
size_t partial_workspace(const Problem& pb);
int project_partial_device(const Problem& pb, const float* d_act, const float* d_att, const float* d_bg_image,
                           float* d_sino, float* d_partial, int do_rotate, char* ws, size_t ws_bytes, Staging* stg,
                           cudaStream_t st);
// float64 reference run of the general-orientation projector and the
// reference backprojector (geometry, PSF and every operation in double);
// device buffers are double, nifti order.
size_t workspace64(const Problem& pb);
int project_device64(const Problem& pb, const double* d_act, const double* d_att, double* d_sino, char* ws,
                     size_t ws_bytes, cudaStream_t st);
int backproject_device64(const Problem& pb, const double* d_sino, const double* d_att, double* d_out, char* ws,
                         size_t ws_bytes, cudaStream_t st);
// Exact d/dmu of sum(g * project(act, mu)) (g = d_sino); work space
// dmu_workspace.  Gantry cameras without backgrounds run the fused kernel.
size_t dmu_workspace(const Problem& pb);
int dmu_device(const Problem& pb, const float* d_g, const float* d_act, const float* d_att, float* d_out, char* ws,
               size_t ws_bytes, Staging* stg, cudaStream_t st);

}  // namespace nrgb
