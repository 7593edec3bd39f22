// Engine implementation: dispatch between the fused y-gantry kernels and the
// general-orientation path, work-space layout, per-device state.
#include "et_engine.h"

#include <algorithm>
#include <cstdint>
#include <initializer_list>
#include <atomic>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>

#include "et_kernels.h"

namespace nrgb {

int sm_count() {
  static std::mutex mu;
  static std::map<int, int> counts;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 152;
  std::lock_guard<std::mutex> lk(mu);
  auto it = counts.find(dev);
  if (it != counts.end()) return it->second;
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
    cudaGetLastError();
    n = 152;
  }
  return counts[dev] = n;
}

// ------------------------------------------------------------ tuning table
// Cameras per backprojection scratch group, keyed by (nx, ny, nz, ncam); a
// key of zeros is the default.  Filled by nrgb_tune_set (the autotuner in
// niftyrec_gb300/autotune.py measures candidates and records the fastest).
namespace {
// Cameras per group without a table entry: groups of at most 48 cameras, as
// even as possible (larger launches fill the GPU better; measured on GB300:
// 128^3 x 120 cameras 1.23 ms per backprojection with 40, 1.42 ms with one
// group of 120, 1.60 ms with 16; 256^3 x 180: 22.8 ms with 45; 15 or 45
// cameras: one group is fastest), and at most 2 GiB of scratch per slot.
int default_group(int nx, int ny, int nz, int ncam) {
  const int groups = (ncam + 47) / 48;
  const int g = (ncam + groups - 1) / groups;
  const size_t per_cam = sizeof(float) * static_cast<size_t>(nz) * nx * round_up(std::min(ny, 128), 4);
  const size_t cap = std::max<size_t>(1, (static_cast<size_t>(2) << 30) / per_cam);
  return std::max(1, static_cast<int>(std::min<size_t>(g, cap)));
}
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, int> g_tune_group;
}  // namespace

int tuned_group(int nx, int ny, int nz, int ncam) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune_group.find(std::make_tuple(nx, ny, nz, ncam));
  if (it != g_tune_group.end()) return it->second;
  it = g_tune_group.find(std::make_tuple(0, 0, 0, 0));
  return it != g_tune_group.end() ? it->second : default_group(nx, ny, nz, ncam);
}

void set_tuned_group(int nx, int ny, int nz, int ncam, int group) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (group > 0)
    g_tune_group[std::make_tuple(nx, ny, nz, ncam)] = group;
  else
    g_tune_group.erase(std::make_tuple(nx, ny, nz, ncam));
}

namespace {
std::map<std::tuple<int, int, int, int>, int> g_tune_slabs;
}  // namespace

int tuned_project_slabs(int nx, int ny, int nz, int ncam) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune_slabs.find(std::make_tuple(nx, ny, nz, ncam));
  return it != g_tune_slabs.end() ? it->second : 0;
}

void set_tuned_project_slabs(int nx, int ny, int nz, int ncam, int slabs) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (slabs > 0)
    g_tune_slabs[std::make_tuple(nx, ny, nz, ncam)] = slabs;
  else
    g_tune_slabs.erase(std::make_tuple(nx, ny, nz, ncam));
}

namespace {
std::atomic<int> g_mirror_pairs{1};
std::atomic<int> g_deterministic{0};
}  // namespace

void set_mirror_pairs(int on) { g_mirror_pairs.store(on ? 1 : 0); }
int mirror_pairs() { return g_mirror_pairs.load(); }
void set_deterministic(int on) { g_deterministic.store(on ? 1 : 0); }
int deterministic() { return g_deterministic.load(); }

int make_problem(int nx, int ny, int nz, const Cameras& cams, const float* psf, const int* psf_size, float bg,
                 float bg_att, int truncate, Problem* out) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || cams.n <= 0) return kErrParameters;
  Problem pb;
  pb.nx = nx;
  pb.ny = ny;
  pb.nz = nz;
  pb.cams = cams;
  pb.geom = camera_geometry(cams);
  pb.ygantry = is_y_gantry(cams);
  if (pb.ygantry && mirror_pairs()) pb.units = mirror_units(cams, nx, nz);
  if (!pb.ygantry && nx % 4 == 0 && is_x_gantry(cams)) {
    pb.xgantry = true;
    pb.geom_x.resize(pb.geom.size());
    for (size_t c = 0; c < pb.geom.size(); ++c) pb.geom_x[c] = swap_xy(pb.geom[c]);
    if (mirror_pairs()) pb.units_x = mirror_units(cams, ny, nz, 0);
  }
  pb.bg = bg;
  pb.bg_att = bg_att;
  pb.truncate = truncate;
  pb.det = deterministic();
  pb.group = tuned_group(nx, ny, nz, cams.n);
  pb.pslabs = tuned_project_slabs(nx, ny, nz, cams.n);
  if (psf) {
    const int kx = psf_size[0], ky = psf_size[1], planes = psf_size[2];
    // The reference separates the PSF assuming kx == ky (emission-lib/_et.cpp:199-213
    // indexes both kernels with psf_size[0]) and reads plane z for every depth z.
    if (kx % 2 != 1 || ky % 2 != 1 || kx != ky || planes < nz) return kErrParameters;
    pb.psf_k = kx;
    pb.psf_sep = separate_psf(psf, kx, nz);
    pb.psf_host = psf;
    if (pb.xgantry) {  // row and column kernels exchanged
      pb.psf_sep_x.resize(pb.psf_sep.size());
      for (int n = 0; n < nz; ++n)
        for (int i = 0; i < kx; ++i) {
          pb.psf_sep_x[static_cast<size_t>(2 * kx) * n + i] = pb.psf_sep[static_cast<size_t>(2 * kx) * n + kx + i];
          pb.psf_sep_x[static_cast<size_t>(2 * kx) * n + kx + i] = pb.psf_sep[static_cast<size_t>(2 * kx) * n + i];
        }
    }
  }
  *out = std::move(pb);
  return kOk;
}

bool use_fused(const Problem& pb) {
  return pb.ygantry && pb.bg == 0.0f && pb.bg_att == 0.0f && yg_supported(pb.nx, pb.ny, pb.nz, pb.psf_k);
}

bool use_fused_x(const Problem& pb) {
  return pb.xgantry && pb.bg == 0.0f && pb.bg_att == 0.0f && yg_supported(pb.ny, pb.nx, pb.nz, pb.psf_k);
}

namespace {

size_t vol_n(const Problem& pb) { return static_cast<size_t>(pb.nx) * pb.ny * pb.nz; }
size_t col_n(const Problem& pb) { return static_cast<size_t>(pb.nx) * round_up(pb.ny, 4) * pb.nz; }
size_t sino_col_n(const Problem& pb) { return static_cast<size_t>(pb.nx) * round_up(pb.ny, 4) * pb.cams.n; }
constexpr size_t kSlack = 8 * 256;

size_t common_bytes(const Problem& pb) {
  return sizeof(CamGeom) * pb.cams.n + sizeof(float) * pb.psf_sep.size() +
         sizeof(int) * std::max(pb.units.size(), pb.units_x.size()) + kSlack;
}

// The x-gantry form reads and writes the caller's nifti buffers directly with
// vector loads: 16-byte aligned float32 (8-byte bfloat16) buffers only.
bool aligned_for_x(const Problem& pb, std::initializer_list<const void*> ptrs) {
  const uintptr_t mask = pb.storage == kStorageBF16 ? 7 : 15;
  for (const void* p : ptrs)
    if (p && (reinterpret_cast<uintptr_t>(p) & mask)) return false;
  return true;
}

// Gantry-kernel arguments of an x-gantry problem on nifti buffers: engine x
// is nifti y, engine rows are nifti x (column stride nx).
YgArgs x_args(const Problem& pb, const CamGeom* d_geom, const float* d_psf, const int2* d_units) {
  YgArgs a;
  a.storage = pb.storage;
  a.pslabs = pb.pslabs;
  a.nx = pb.ny;
  a.ny = pb.nx;
  a.nz = pb.nz;
  a.cy = pb.nx;
  a.ncam = pb.cams.n;
  a.geom = d_geom;
  a.units = d_units;
  a.nunits = static_cast<int>(pb.units_x.size() / 2);
  a.psf = d_psf;
  a.psf_host = pb.psf_k ? pb.psf_sep_x.data() : nullptr;
  a.psf_k = pb.psf_k;
  a.truncate = pb.truncate;
  return a;
}

// Uploads camera matrices, the separated PSF and the mirror-camera units
// through the pinned staging slot that is not in flight (waiting for its
// previous copy if needed).
// engine_x: the x-gantry forms (geom_x, psf_sep_x, units_x).
int upload_common(const Problem& pb, Carver& cv, CamGeom** d_geom, float** d_psf, Staging* stg, cudaStream_t st,
                  int2** d_units = nullptr, bool engine_x = false) {
  const std::vector<CamGeom>& geom = engine_x ? pb.geom_x : pb.geom;
  const std::vector<float>& psf_sep = engine_x ? pb.psf_sep_x : pb.psf_sep;
  const std::vector<int>& units = engine_x ? pb.units_x : pb.units;
  *d_geom = cv.take<CamGeom>(pb.cams.n);
  *d_psf = nullptr;
  if (!*d_geom) return kErrAllocGpu;
  if (pb.psf_k) {
    *d_psf = cv.take<float>(psf_sep.size());
    if (!*d_psf) return kErrAllocGpu;
  }
  const size_t ubytes = d_units ? sizeof(int) * units.size() : 0;
  if (d_units) {
    *d_units = nullptr;
    if (ubytes && !(*d_units = cv.take<int2>(units.size() / 2))) return kErrAllocGpu;
  }
  const size_t gbytes = sizeof(CamGeom) * pb.cams.n;
  const size_t pbytes = sizeof(float) * psf_sep.size();
  const int slot = stg->slot;
  stg->slot ^= 1;
  if (stg->done[slot]) {
    cudaEventSynchronize(stg->done[slot]);
  } else if (cudaEventCreateWithFlags(&stg->done[slot], cudaEventDisableTiming) != cudaSuccess) {
    return kErrUnspecified;
  }
  if (stg->bytes[slot] < gbytes + pbytes + ubytes) {
    if (stg->pinned[slot]) cudaFreeHost(stg->pinned[slot]);
    stg->pinned[slot] = nullptr;
    stg->bytes[slot] = 0;
    const size_t want = std::max(gbytes + pbytes + ubytes, static_cast<size_t>(1) << 20);
    if (cudaMallocHost(&stg->pinned[slot], want) != cudaSuccess) {
      cudaGetLastError();
      return kErrAllocCpu;
    }
    stg->bytes[slot] = want;
  }
  char* h = stg->pinned[slot];
  std::memcpy(h, geom.data(), gbytes);
  if (pbytes) std::memcpy(h + gbytes, psf_sep.data(), pbytes);
  if (cudaMemcpyAsync(*d_geom, h, gbytes, cudaMemcpyHostToDevice, st) != cudaSuccess) return kErrTransferGpu;
  if (pbytes && cudaMemcpyAsync(*d_psf, h + gbytes, pbytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return kErrTransferGpu;
  if (ubytes) {
    std::memcpy(h + gbytes + pbytes, units.data(), ubytes);
    if (cudaMemcpyAsync(*d_units, h + gbytes + pbytes, ubytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return kErrTransferGpu;
  }
  cudaEventRecord(stg->done[slot], st);
  return kOk;
}

int check(int status) {
  if (status != kOk) return status;
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

// float32 copies of bfloat16 inputs for the general-orientation path
size_t widen_bytes(const Problem& pb) { return pb.input_bf16 ? 2 * (sizeof(float) * vol_n(pb) + 256) : 0; }

// Widen the caller's bfloat16 activity / mu (nifti order) into float32 work
// volumes; the pointers are replaced by the copies.
int widen_inputs(const Problem& pb, Carver& cv, const float** act, const float** att, cudaStream_t st) {
  const float** ps[2] = {act, att};
  for (const float** p : ps) {
    if (!p || !*p) continue;
    float* w = cv.take<float>(vol_n(pb));
    if (!w) return kErrAllocGpu;
    int s = from_bf16(*p, w, vol_n(pb), st);
    if (s != kOk) return s;
    *p = w;
  }
  return kOk;
}

}  // namespace

size_t project_workspace(const Problem& pb, bool has_act, bool has_att) {
  size_t b = common_bytes(pb);
  if (use_fused_x(pb) && has_act) return b + vol_n(pb) * 3 * sizeof(float) + widen_bytes(pb);  // or general
  if (use_fused(pb) && has_act)
    b += sizeof(float) * (col_n(pb) * (has_att ? 2 : 1) + sino_col_n(pb));
  else
    b += sizeof(float) * vol_n(pb) * 3 + widen_bytes(pb);
  return b;
}

size_t backproject_workspace(const Problem& pb, bool has_att) {
  size_t b = common_bytes(pb);
  if (use_fused_x(pb))  // the fused form's scratch, or the general path's volumes
    return b + std::max(yg_backproject_workspace(pb.ny, pb.nx, pb.nz, pb.cams.n, pb.group) + kSlack,
                        sizeof(float) * vol_n(pb) * 3 + widen_bytes(pb));
  if (use_fused(pb))
    b += sizeof(float) * (col_n(pb) * (has_att ? 2 : 1) + sino_col_n(pb)) +
         yg_backproject_workspace(pb.nx, pb.ny, pb.nz, pb.cams.n, pb.group) + kSlack;
  else
    b += sizeof(float) * vol_n(pb) * 3 + widen_bytes(pb);
  return b;
}

namespace {
// The general-orientation path's three work volumes.
size_t general3_workspace(const Problem& pb) { return common_bytes(pb) + sizeof(float) * vol_n(pb) * 3; }
int grad_group(const Problem& pb) { return std::max(1, std::min(pb.group, pb.cams.n)); }
}  // namespace

size_t gradient_workspace(const Problem& pb) {
  if (pb.storage != kStorageF32) return general3_workspace(pb);
  if (use_fused_x(pb))  // the fused form's scratch, or the general path's volumes
    return std::max(general3_workspace(pb),
                    common_bytes(pb) + yg_gradient_workspace(pb.ny, pb.nx, pb.nz, pb.cams.n, grad_group(pb)) + kSlack);
  if (use_fused(pb))
    return common_bytes(pb) + sizeof(float) * (3 * col_n(pb) + sino_col_n(pb)) +
           yg_gradient_workspace(pb.nx, pb.ny, pb.nz, pb.cams.n, grad_group(pb)) + kSlack;
  return general3_workspace(pb);
}

namespace {

// A caller volume (nifti, float32 or bfloat16) into the fused kernels'
// column buffer in the problem's storage type.
int stage_column(const Problem& pb, const float* src, float* dst, int cy, int planes, cudaStream_t st) {
  if (pb.storage == kStorageBF16)
    return to_column_rows_bf16(pb.input_bf16 ? nullptr : src, pb.input_bf16 ? src : nullptr, dst, pb.nx, pb.ny, 0,
                               pb.ny, cy, planes, st);
  return to_column(src, dst, pb.nx, pb.ny, cy, planes, st);
}

}  // namespace

int project_device(const Problem& pb, const float* d_act, const float* d_att, float* d_sino, char* ws,
                   size_t ws_bytes, Staging* stg, cudaStream_t st) {
  if (use_fused_x(pb) && d_act && aligned_for_x(pb, {d_act, d_att, d_sino})) {
    Carver cx(ws, ws_bytes);
    CamGeom* d_geom;
    float* d_psf;
    int2* d_units;
    int s = upload_common(pb, cx, &d_geom, &d_psf, stg, st, &d_units, true);
    if (s != kOk) return s;
    YgArgs a = x_args(pb, d_geom, d_psf, d_units);
    a.act = d_act;
    a.mu = d_att;
    a.out = d_sino;
    return check(yg_project(a, st));
  }
  Carver cv(ws, ws_bytes);
  CamGeom* d_geom;
  float* d_psf;
  int2* d_units;
  int s = upload_common(pb, cv, &d_geom, &d_psf, stg, st, &d_units);
  if (s != kOk) return s;
  if (use_fused(pb) && d_act) {
    float* act_c = cv.take<float>(col_n(pb));
    float* mu_c = d_att ? cv.take<float>(col_n(pb)) : nullptr;
    float* sino_c = cv.take<float>(sino_col_n(pb));
    if (!act_c || !sino_c || (d_att && !mu_c)) return kErrAllocGpu;
    const int cy = round_up(pb.ny, 4);
    if (pb.storage == kStorageF32 && d_att) {  // activity and mu in one launch
      if ((s = to_column2(d_act, act_c, d_att, mu_c, pb.nx, pb.ny, cy, pb.nz, st)) != kOk) return s;
    } else {
      if ((s = stage_column(pb, d_act, act_c, cy, pb.nz, st)) != kOk) return s;
      if (d_att && (s = stage_column(pb, d_att, mu_c, cy, pb.nz, st)) != kOk) return s;
    }
    YgArgs a;
    a.storage = pb.storage;
    a.pslabs = pb.pslabs;
    a.nx = pb.nx;
    a.ny = pb.ny;
    a.nz = pb.nz;
    a.cy = cy;
    a.ncam = pb.cams.n;
    a.geom = d_geom;
    a.units = d_units;
    a.nunits = static_cast<int>(pb.units.size() / 2);
    a.act = act_c;
    a.mu = mu_c;
    a.out = sino_c;
    a.psf = d_psf;
    a.psf_host = pb.psf_k ? pb.psf_sep.data() : nullptr;
    a.psf_k = pb.psf_k;
    a.truncate = pb.truncate;
    if ((s = yg_project(a, st)) != kOk) return s;
    return check(from_column(sino_c, d_sino, pb.nx, pb.ny, cy, pb.cams.n, 0, st));
  }
  if (pb.input_bf16 && (s = widen_inputs(pb, cv, &d_act, &d_att, st)) != kOk) return s;
  GeneralArgs g;
  g.nx = pb.nx;
  g.ny = pb.ny;
  g.nz = pb.nz;
  g.ncam = pb.cams.n;
  g.geom_host = pb.geom.data();
  g.act = d_act;
  g.att = d_att;
  g.out = d_sino;
  g.psf_sep = d_psf;
  g.psf_k = pb.psf_k;
  g.bg = pb.bg;
  g.bg_att = pb.bg_att;
  g.truncate = pb.truncate;
  g.ws_act = cv.take<float>(vol_n(pb));
  g.ws_att = cv.take<float>(vol_n(pb));
  g.ws_tmp = cv.take<float>(vol_n(pb));
  if (!g.ws_act || !g.ws_att || !g.ws_tmp) return kErrAllocGpu;
  return check(general_project(g, st));
}

namespace {

// A second stream per device on which a backprojection converts its
// sinogram while the transmission carries run on the caller's stream.
struct SideStream {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
};

SideStream* side_for_current_device() {
  static std::mutex mu;
  static std::map<int, std::unique_ptr<SideStream>> sides;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  std::unique_ptr<SideStream>& p = sides[dev];
  if (!p) {
    auto q = std::make_unique<SideStream>();
    if (cudaStreamCreateWithFlags(&q->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&q->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&q->done, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    p = std::move(q);
  }
  return p.get();
}

}  // namespace

int backproject_device(const Problem& pb, const float* d_sino, const float* d_att, float* d_out, char* ws,
                       size_t ws_bytes, Staging* stg, cudaStream_t st) {
  if (use_fused_x(pb) && aligned_for_x(pb, {d_sino, d_att, d_out})) {
    Carver cx(ws, ws_bytes);
    CamGeom* d_geom;
    float* d_psf;
    int2* d_units;
    int s = upload_common(pb, cx, &d_geom, &d_psf, stg, st, &d_units, true);
    if (s != kOk) return s;
    YgArgs a = x_args(pb, d_geom, d_psf, d_units);
    a.mu = d_att;
    a.sino = d_sino;
    a.out = d_out;
    a.back_mode = pb.back_mode;
    a.det = pb.det;
    a.group = std::max(1, std::min(pb.group, pb.cams.n));
    a.work = cx.take<float>(yg_backproject_workspace(pb.ny, pb.nx, pb.nz, pb.cams.n, a.group) / sizeof(float));
    if (!a.work) return kErrAllocGpu;
    if ((s = yg_backproject(a, st)) != kOk) return s;
    // the gathers clamp as they store; the vector-reduction transpose does not
    if (pb.truncate && pb.back_mode == kBackAdjoint && !pb.det) launch_truncate(d_out, vol_n(pb), st);
    return check(kOk);
  }
  Carver cv(ws, ws_bytes);
  CamGeom* d_geom;
  float* d_psf;
  int2* d_units;
  int s = upload_common(pb, cv, &d_geom, &d_psf, stg, st, &d_units);
  if (s != kOk) return s;
  if (use_fused(pb)) {
    float* sino_c = cv.take<float>(sino_col_n(pb));
    float* mu_c = d_att ? cv.take<float>(col_n(pb)) : nullptr;
    float* out_c = cv.take<float>(col_n(pb));
    const int group = std::max(1, std::min(pb.group, pb.cams.n));
    float* slab = cv.take<float>(yg_backproject_workspace(pb.nx, pb.ny, pb.nz, pb.cams.n, group) / sizeof(float));
    if (!sino_c || !out_c || !slab || (d_att && !mu_c)) return kErrAllocGpu;
    const int cy = round_up(pb.ny, 4);
    // with attenuation the sinogram is converted on a side stream while the
    // carries (which need only mu) run on st
    SideStream* side = d_att ? side_for_current_device() : nullptr;
    std::unique_lock<std::mutex> side_lock;
    if (side) {
      side_lock = std::unique_lock<std::mutex>(side->mu);
      if ((s = stage_column(pb, d_att, mu_c, cy, pb.nz, st)) != kOk) return s;
      cudaEventRecord(side->fork, st);
      cudaStreamWaitEvent(side->stream, side->fork, 0);
      if ((s = to_column(d_sino, sino_c, pb.nx, pb.ny, cy, pb.cams.n, side->stream)) != kOk) return s;
      cudaEventRecord(side->done, side->stream);
    } else {
      if ((s = to_column(d_sino, sino_c, pb.nx, pb.ny, cy, pb.cams.n, st)) != kOk) return s;
      if (d_att && (s = stage_column(pb, d_att, mu_c, cy, pb.nz, st)) != kOk) return s;
    }
    YgArgs a;
    a.sino_ready = side ? side->done : nullptr;
    a.storage = pb.storage;
    a.nx = pb.nx;
    a.ny = pb.ny;
    a.nz = pb.nz;
    a.cy = cy;
    a.ncam = pb.cams.n;
    a.geom = d_geom;
    a.units = d_units;
    a.nunits = static_cast<int>(pb.units.size() / 2);
    a.mu = mu_c;
    a.sino = sino_c;
    a.out = out_c;
    a.psf = d_psf;
    a.psf_host = pb.psf_k ? pb.psf_sep.data() : nullptr;
    a.psf_k = pb.psf_k;
    a.truncate = pb.truncate;
    a.back_mode = pb.back_mode;
    a.det = pb.det;
    a.group = group;
    a.work = slab;
    if ((s = yg_backproject(a, st)) != kOk) return s;
    return check(from_column(out_c, d_out, pb.nx, pb.ny, cy, pb.nz, pb.truncate, st));
  }
  if (pb.input_bf16 && (s = widen_inputs(pb, cv, nullptr, &d_att, st)) != kOk) return s;
  GeneralArgs g;
  g.nx = pb.nx;
  g.ny = pb.ny;
  g.nz = pb.nz;
  g.ncam = pb.cams.n;
  g.geom_host = pb.geom.data();
  g.att = d_att;
  g.sino = d_sino;
  g.out = d_out;
  g.psf_sep = d_psf;
  g.psf_k = pb.psf_k;
  g.bg = pb.bg;
  g.bg_att = pb.bg_att;
  g.truncate = pb.truncate;
  g.ws_act = cv.take<float>(vol_n(pb));
  g.ws_att = cv.take<float>(vol_n(pb));
  g.ws_tmp = cv.take<float>(vol_n(pb));
  if (!g.ws_act || !g.ws_att || !g.ws_tmp) return kErrAllocGpu;
  return check(pb.back_mode == kBackAdjoint ? general_adjoint(g, st) : general_backproject(g, st));
}

size_t pair_workspace(const Problem& pb, bool has_att, bool has_input) {
  const size_t seq = std::max(project_workspace(pb, true, has_att), backproject_workspace(pb, has_att));
  if (!use_fused(pb)) return seq;
  const int group = std::max(1, std::min(pb.group, pb.cams.n));
  return common_bytes(pb) +
         sizeof(float) * (col_n(pb) * (has_att ? 3 : 2) + sino_col_n(pb) * (has_input ? 2 : 1)) +
         yg_backproject_workspace(pb.nx, pb.ny, pb.nz, pb.cams.n, group) + kSlack;
}

bool same_geometry(const Problem& a, const Problem& b) {
  return a.geom.size() == b.geom.size() &&
         std::memcmp(a.geom.data(), b.geom.data(), sizeof(CamGeom) * a.geom.size()) == 0 && a.units == b.units;
}

int pair_device(const Problem& pb, const Problem& pb_back, const float* d_act, const float* d_att, float* d_sino,
                const float* d_bk_in, float* d_bk, char* ws, size_t ws_bytes, Staging* stg, cudaStream_t st) {
  // The two calls in sequence (stream-ordered reuse of the work space) where
  // the fused kernels do not apply or the backprojector's cameras sit
  // elsewhere (the reference centres them at (nx-1)/2 in z, the projector's
  // at (nz-1)/2).
  if (!use_fused(pb) || !d_act || !use_fused(pb_back) || !same_geometry(pb, pb_back)) {
    int s = project_device(pb, d_act, d_att, d_sino, ws, ws_bytes, stg, st);
    if (s != kOk) return s;
    return backproject_device(pb_back, d_bk_in ? d_bk_in : d_sino, d_att, d_bk, ws, ws_bytes, stg, st);
  }
  Carver cv(ws, ws_bytes);
  CamGeom* d_geom;
  float* d_psf;
  int2* d_units;
  int s = upload_common(pb, cv, &d_geom, &d_psf, stg, st, &d_units);
  if (s != kOk) return s;
  const int cy = round_up(pb.ny, 4);
  const int group = std::max(1, std::min(pb.group, pb.cams.n));
  float* act_c = cv.take<float>(col_n(pb));
  float* mu_c = d_att ? cv.take<float>(col_n(pb)) : nullptr;
  float* sino_c = cv.take<float>(sino_col_n(pb));
  float* in_c = d_bk_in ? cv.take<float>(sino_col_n(pb)) : sino_c;
  float* out_c = cv.take<float>(col_n(pb));
  // carries (at most kSlabsB + 1 slots per camera) then the scratch slots
  float* work = cv.take<float>(yg_backproject_workspace(pb.nx, pb.ny, pb.nz, pb.cams.n, group) / sizeof(float));
  if (!act_c || !sino_c || !in_c || !out_c || !work || (d_att && !mu_c)) return kErrAllocGpu;
  const size_t carry_n = static_cast<size_t>(pb.cams.n) * yg_carry_slabs() * pb.nx * cy;
  if (pb.storage == kStorageF32 && d_att) {  // activity and mu in one launch
    if ((s = to_column2(d_act, act_c, d_att, mu_c, pb.nx, pb.ny, cy, pb.nz, st)) != kOk) return s;
  } else {
    if ((s = stage_column(pb, d_act, act_c, cy, pb.nz, st)) != kOk) return s;
    if (d_att && (s = stage_column(pb, d_att, mu_c, cy, pb.nz, st)) != kOk) return s;
  }
  YgArgs a;
  a.storage = pb.storage;
  a.pslabs = pb.pslabs;
  a.nx = pb.nx;
  a.ny = pb.ny;
  a.nz = pb.nz;
  a.cy = cy;
  a.ncam = pb.cams.n;
  a.geom = d_geom;
  a.units = d_units;
  a.nunits = static_cast<int>(pb.units.size() / 2);
  a.act = act_c;
  a.mu = mu_c;
  a.out = sino_c;
  a.psf = d_psf;
  a.psf_host = pb.psf_k ? pb.psf_sep.data() : nullptr;
  a.psf_k = pb.psf_k;
  a.truncate = pb.truncate;
  // the projector leaves the carries of its depth slabs for the backprojector
  // (split at mid-slab where that gives the backprojector its preferred
  // twice-as-many slabs: 128^3 x 120 projects with 4 slabs, spreads with 8)
  a.carry_out = d_att ? work : nullptr;
  a.carry_split = 1;
  YgArgs b = a;
  b.carry_out = nullptr;
  b.act = nullptr;
  b.sino = in_c;
  b.out = out_c;
  b.back_mode = pb.back_mode;
  b.det = pb.det;
  b.group = group;
  b.carry = d_att ? work : nullptr;
  b.work = work + (d_att ? carry_n : 0);
  int slabs = 0;
  if ((s = yg_project(a, st, &slabs)) != kOk) return s;
  if (d_att && (slabs < 1 || slabs + 1 > yg_carry_slabs())) return kErrKernel;
  // the caller's projection (nifti order) is written on a side stream while
  // the backprojector reads the column-layout copy
  SideStream* side = side_for_current_device();
  std::unique_lock<std::mutex> side_lock;
  if (side) {
    side_lock = std::unique_lock<std::mutex>(side->mu);
    cudaEventRecord(side->fork, st);
    cudaStreamWaitEvent(side->stream, side->fork, 0);
    if ((s = from_column(sino_c, d_sino, pb.nx, pb.ny, cy, pb.cams.n, 0, side->stream)) != kOk) return s;
    cudaEventRecord(side->done, side->stream);
  } else if ((s = from_column(sino_c, d_sino, pb.nx, pb.ny, cy, pb.cams.n, 0, st)) != kOk) {
    return s;
  }
  if (d_bk_in && (s = to_column(d_bk_in, in_c, pb.nx, pb.ny, cy, pb.cams.n, st)) != kOk) return s;
  b.bslabs = d_att ? slabs : b.bslabs;
  s = yg_backproject(b, st);
  if (side) cudaStreamWaitEvent(st, side->done, 0);
  if (s != kOk) return s;
  return check(from_column(out_c, d_bk, pb.nx, pb.ny, cy, pb.nz, pb.truncate, st));
}

size_t partial_workspace(const Problem& pb) { return common_bytes(pb) + sizeof(float) * vol_n(pb) * 3 + 3 * 256; }

int project_partial_device(const Problem& pb, const float* d_act, const float* d_att, const float* d_bg_image,
                           float* d_sino, float* d_partial, int do_rotate, char* ws, size_t ws_bytes, Staging* stg,
                           cudaStream_t st) {
  Carver cv(ws, ws_bytes);
  CamGeom* d_geom;
  float* d_psf;
  int s = upload_common(pb, cv, &d_geom, &d_psf, stg, st);
  if (s != kOk) return s;
  GeneralArgs g;
  g.nx = pb.nx;
  g.ny = pb.ny;
  g.nz = pb.nz;
  g.ncam = pb.cams.n;
  g.geom_host = pb.geom.data();
  g.act = d_act;
  g.att = d_att;
  g.out = d_sino;
  g.psf_sep = d_psf;
  g.psf_k = pb.psf_k;
  g.bg = pb.bg;
  g.bg_att = pb.bg_att;
  g.truncate = pb.truncate;
  g.ws_act = cv.take<float>(vol_n(pb));
  g.ws_att = cv.take<float>(vol_n(pb));
  g.ws_tmp = cv.take<float>(vol_n(pb));
  if (!g.ws_act || !g.ws_att || !g.ws_tmp) return kErrAllocGpu;
  return check(general_project_partial(g, d_bg_image, d_partial, do_rotate, st));
}

size_t dmu_workspace(const Problem& pb) {
  if (use_fused_x(pb) && pb.storage == kStorageF32)  // the fused form's scratch, or the general path's volumes
    return std::max(general3_workspace(pb),
                    common_bytes(pb) + (pb.det ? yg_dmu_det_workspace(pb.ny, pb.nx, pb.nz, pb.cams.n, pb.group) : 0) +
                        kSlack);
  if (use_fused(pb) && pb.storage == kStorageF32)
    return common_bytes(pb) + sizeof(float) * (3 * col_n(pb) + sino_col_n(pb)) + 4 * 256 +
           (pb.det ? yg_dmu_det_workspace(pb.nx, pb.ny, pb.nz, pb.cams.n, pb.group) + kSlack : 0);
  return general3_workspace(pb);
}

int dmu_device(const Problem& pb, const float* d_g, const float* d_act, const float* d_att, float* d_out, char* ws,
               size_t ws_bytes, Staging* stg, cudaStream_t st) {
  if (use_fused_x(pb) && pb.storage == kStorageF32 && aligned_for_x(pb, {d_g, d_act, d_att, d_out})) {
    Carver cx(ws, ws_bytes);
    CamGeom* d_geom;
    float* d_psf;
    int s = upload_common(pb, cx, &d_geom, &d_psf, stg, st, nullptr, true);
    if (s != kOk) return s;
    YgArgs a = x_args(pb, d_geom, d_psf, nullptr);
    a.units = nullptr;
    a.nunits = 0;
    a.act = d_act;
    a.mu = d_att;
    a.sino = d_g;
    a.out = d_out;
    if (pb.det) {
      a.det = 1;
      a.group = pb.group;
      a.work = cx.take<float>(yg_dmu_det_workspace(a.nx, a.ny, a.nz, a.ncam, a.group) / sizeof(float));
      if (!a.work) return kErrAllocGpu;
    }
    return check(yg_dmu(a, st));
  }
  Carver cv(ws, ws_bytes);
  CamGeom* d_geom;
  float* d_psf;
  int s = upload_common(pb, cv, &d_geom, &d_psf, stg, st);
  if (s != kOk) return s;
  if (use_fused(pb) && pb.storage == kStorageF32) {
    const int cy = round_up(pb.ny, 4);
    float* act_c = cv.take<float>(col_n(pb));
    float* mu_c = cv.take<float>(col_n(pb));
    float* out_c = cv.take<float>(col_n(pb));
    float* g_c = cv.take<float>(sino_col_n(pb));
    if (!act_c || !mu_c || !out_c || !g_c) return kErrAllocGpu;
    if ((s = to_column(d_act, act_c, pb.nx, pb.ny, cy, pb.nz, st)) != kOk) return s;
    if ((s = to_column(d_att, mu_c, pb.nx, pb.ny, cy, pb.nz, st)) != kOk) return s;
    if ((s = to_column(d_g, g_c, pb.nx, pb.ny, cy, pb.cams.n, st)) != kOk) return s;
    YgArgs a;
    a.nx = pb.nx;
    a.ny = pb.ny;
    a.nz = pb.nz;
    a.cy = cy;
    a.ncam = pb.cams.n;
    a.geom = d_geom;
    a.act = act_c;
    a.mu = mu_c;
    a.sino = g_c;
    a.out = out_c;
    a.psf = d_psf;
    a.psf_host = pb.psf_k ? pb.psf_sep.data() : nullptr;
    a.psf_k = pb.psf_k;
    if (pb.det) {
      a.det = 1;
      a.group = pb.group;
      a.work = cv.take<float>(yg_dmu_det_workspace(a.nx, a.ny, a.nz, a.ncam, a.group) / sizeof(float));
      if (!a.work) return kErrAllocGpu;
    }
    if ((s = yg_dmu(a, st)) != kOk) return s;
    return check(from_column(out_c, d_out, pb.nx, pb.ny, cy, pb.nz, 0, st));
  }
  GeneralArgs g;
  g.nx = pb.nx;
  g.ny = pb.ny;
  g.nz = pb.nz;
  g.ncam = pb.cams.n;
  g.geom_host = pb.geom.data();
  g.act = d_act;
  g.att = d_att;
  g.sino = d_g;
  g.out = d_out;
  g.psf_sep = d_psf;
  g.psf_k = pb.psf_k;
  g.bg = pb.bg;
  g.bg_att = pb.bg_att;
  g.ws_act = cv.take<float>(vol_n(pb));
  g.ws_att = cv.take<float>(vol_n(pb));
  g.ws_tmp = cv.take<float>(vol_n(pb));
  if (!g.ws_act || !g.ws_att || !g.ws_tmp) return kErrAllocGpu;
  return check(general_dmu(g, st));
}

int gradient_device(const Problem& pb, const float* d_sino, const float* d_act, const float* d_att, float* d_out,
                    char* ws, size_t ws_bytes, Staging* stg, cudaStream_t st) {
  if (use_fused_x(pb) && pb.storage == kStorageF32 && aligned_for_x(pb, {d_sino, d_act, d_att, d_out})) {
    Carver cx(ws, ws_bytes);
    CamGeom* d_geom;
    float* d_psf;
    int s = upload_common(pb, cx, &d_geom, &d_psf, stg, st, nullptr, true);
    if (s != kOk) return s;
    YgArgs a = x_args(pb, d_geom, d_psf, nullptr);
    a.units = nullptr;
    a.nunits = 0;
    a.gradient = 1;
    a.act = d_act;
    a.mu = d_att;
    a.sino = d_sino;
    a.out = d_out;
    a.group = grad_group(pb);
    a.work = cx.take<float>(yg_gradient_workspace(pb.ny, pb.nx, pb.nz, pb.cams.n, a.group) / sizeof(float));
    if (!a.work) return kErrAllocGpu;
    return check(yg_backproject(a, st));  // the last gathers clamp when truncating
  }
  Carver cv(ws, ws_bytes);
  CamGeom* d_geom;
  float* d_psf;
  int s = upload_common(pb, cv, &d_geom, &d_psf, stg, st);
  if (s != kOk) return s;
  if (use_fused(pb) && pb.storage == kStorageF32) {
    const int cy = round_up(pb.ny, 4);
    float* act_c = cv.take<float>(col_n(pb));
    float* mu_c = cv.take<float>(col_n(pb));
    float* out_c = cv.take<float>(col_n(pb));
    float* sino_c = cv.take<float>(sino_col_n(pb));
    const int group = grad_group(pb);
    float* work = cv.take<float>(yg_gradient_workspace(pb.nx, pb.ny, pb.nz, pb.cams.n, group) / sizeof(float));
    if (!act_c || !mu_c || !out_c || !sino_c || !work) return kErrAllocGpu;
    if ((s = to_column(d_act, act_c, pb.nx, pb.ny, cy, pb.nz, st)) != kOk) return s;
    if ((s = to_column(d_att, mu_c, pb.nx, pb.ny, cy, pb.nz, st)) != kOk) return s;
    if ((s = to_column(d_sino, sino_c, pb.nx, pb.ny, cy, pb.cams.n, st)) != kOk) return s;
    YgArgs a;
    a.nx = pb.nx;
    a.ny = pb.ny;
    a.nz = pb.nz;
    a.cy = cy;
    a.ncam = pb.cams.n;
    a.geom = d_geom;
    a.act = act_c;
    a.mu = mu_c;
    a.sino = sino_c;
    a.out = out_c;
    a.psf = d_psf;
    a.psf_host = pb.psf_k ? pb.psf_sep.data() : nullptr;
    a.psf_k = pb.psf_k;
    a.pslabs = pb.pslabs;
    a.gradient = 1;
    a.group = group;
    a.work = work;
    if ((s = yg_backproject(a, st)) != kOk) return s;
    return check(from_column(out_c, d_out, pb.nx, pb.ny, cy, pb.nz, pb.truncate, st));
  }
  GeneralArgs g;
  g.nx = pb.nx;
  g.ny = pb.ny;
  g.nz = pb.nz;
  g.ncam = pb.cams.n;
  g.geom_host = pb.geom.data();
  g.act = d_act;
  g.att = d_att;
  g.sino = d_sino;
  g.out = d_out;
  g.psf_sep = d_psf;
  g.psf_k = pb.psf_k;
  g.bg = pb.bg;
  g.bg_att = pb.bg_att;
  g.truncate = pb.truncate;
  g.ws_act = cv.take<float>(vol_n(pb));
  g.ws_att = cv.take<float>(vol_n(pb));
  g.ws_tmp = cv.take<float>(vol_n(pb));
  if (!g.ws_act || !g.ws_att || !g.ws_tmp) return kErrAllocGpu;
  return check(general_gradient(g, st));
}

// ------------------------------------------------------------ float64 run
size_t workspace64(const Problem& pb) {
  return sizeof(double) * (3 * vol_n(pb) + static_cast<size_t>(2 * pb.psf_k) * pb.nz) + kSlack;
}

namespace {

// Fills the float64 arguments: double geometry and separated PSF (uploaded
// from a host vector that the synchronous pageable copy has consumed when
// cudaMemcpyAsync returns), three work volumes.
int setup64(const Problem& pb, const float* psf_host, Carver& cv, std::vector<CamGeom64>* geom, GeneralArgs64* g,
            cudaStream_t st) {
  *geom = camera_geometry64(pb.cams);
  g->nx = pb.nx;
  g->ny = pb.ny;
  g->nz = pb.nz;
  g->ncam = pb.cams.n;
  g->geom_host = geom->data();
  g->psf_k = pb.psf_k;
  g->bg = pb.bg;
  g->bg_att = pb.bg_att;
  g->truncate = pb.truncate;
  if (pb.psf_k) {
    const std::vector<double> sep = separate_psf64(psf_host, pb.psf_k, pb.nz);
    double* d = cv.take<double>(sep.size());
    if (!d) return kErrAllocGpu;
    if (cudaMemcpyAsync(d, sep.data(), sizeof(double) * sep.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
      return kErrTransferGpu;
    g->psf_sep = d;
  }
  g->ws_act = cv.take<double>(vol_n(pb));
  g->ws_att = cv.take<double>(vol_n(pb));
  g->ws_tmp = cv.take<double>(vol_n(pb));
  return (g->ws_act && g->ws_att && g->ws_tmp) ? kOk : kErrAllocGpu;
}

}  // namespace

int project_device64(const Problem& pb, const double* d_act, const double* d_att, double* d_sino, char* ws,
                     size_t ws_bytes, cudaStream_t st) {
  Carver cv(ws, ws_bytes);
  std::vector<CamGeom64> geom;
  GeneralArgs64 g;
  int s = setup64(pb, pb.psf_host, cv, &geom, &g, st);
  if (s != kOk) return s;
  g.act = d_act;
  g.att = d_att;
  g.out = d_sino;
  return check(general_project64(g, st));
}

int backproject_device64(const Problem& pb, const double* d_sino, const double* d_att, double* d_out, char* ws,
                         size_t ws_bytes, cudaStream_t st) {
  Carver cv(ws, ws_bytes);
  std::vector<CamGeom64> geom;
  GeneralArgs64 g;
  int s = setup64(pb, pb.psf_host, cv, &geom, &g, st);
  if (s != kOk) return s;
  g.att = d_att;
  g.sino = d_sino;
  g.out = d_out;
  return check(general_backproject64(g, st));
}

// ------------------------------------------------------------ device state
namespace {
std::mutex g_states_mu;
std::map<int, std::unique_ptr<DeviceState>> g_states;
}  // namespace

DeviceState& current_device_state(int* status) {
  int dev = 0;
  *status = kOk;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    *status = kErrNoGpuInstalled;
  }
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_states_mu);
  auto& p = g_states[dev];
  if (!p) {
    p.reset(new DeviceState());
    p->device = dev;
    if (*status == kOk) {
      if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&p->last_use, cudaEventDisableTiming) != cudaSuccess)
        *status = kErrUnspecified;
    }
  }
  return *p;
}

namespace {
std::atomic<int> g_fail_allocs{0};  // host-side fault injection (nrgb_debug_fail_allocations)
}  // namespace

void fail_next_allocations(int n) { g_fail_allocs.store(n > 0 ? n : 0); }

int ensure_arena(DeviceState& ds, size_t bytes) {
  if (ds.arena_bytes >= bytes) return kOk;
  for (int n = g_fail_allocs.load(); n > 0; n = g_fail_allocs.load())
    if (g_fail_allocs.compare_exchange_weak(n, n - 1)) return kErrAllocGpu;  // injected, before any CUDA call
  if (ds.arena) {
    cudaStreamSynchronize(ds.stream);
    cudaDeviceSynchronize();
    cudaFree(ds.arena);
    ds.arena = nullptr;
    ds.arena_bytes = 0;
  }
  // grow geometrically so repeated slightly-larger calls do not reallocate
  const size_t want = std::max(bytes, static_cast<size_t>(64) << 20);
  if (cudaMalloc(&ds.arena, want) != cudaSuccess) {
    cudaGetLastError();
    ds.arena = nullptr;
    return kErrAllocGpu;
  }
  ds.arena_bytes = want;
  return kOk;
}

}  // namespace nrgb
