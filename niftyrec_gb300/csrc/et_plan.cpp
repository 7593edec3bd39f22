// Plans: device state precomputed once for repeated projections and
// backprojections with the same grid, cameras, PSF and attenuation map -- the
// OSEM pattern of emission-lib/_et_array_interface.cpp:972-1131, where every
// subset step projects and backprojects with unchanged mu.  A plan owns its
// device memory (allocated at creation), keeps mu in column layout, holds the
// transmission carries of every camera and the per-subset sensitivity images,
// so its execute calls allocate nothing, copy nothing from the host and can be
// captured in CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "et_trace.h"
#include "et_array_interface.h"
#include "et_engine.h"
#include "et_kernels.h"

namespace nrgb {
namespace {

struct Plan {
  int device = 0;
  Problem proj;  // cameras in subset order, centres of SPECT_project_parallelholes
  Problem back;  // same cameras, centres of SPECT_backproject_parallelholes
  bool fused = false;
  bool has_att = false;
  int cy = 0;
  int n_subsets = 1;
  std::vector<int> sub_begin;  // n_subsets + 1 offsets into the reordered cameras
  std::vector<int> order;      // reordered position -> original camera index
  char* mem = nullptr;
  size_t bytes = 0;
  CamGeom* geom_p = nullptr;
  CamGeom* geom_b = nullptr;
  float* psf = nullptr;
  float* mu = nullptr;     // column layout (fused) or nifti copy (general)
  float* carry = nullptr;  // [ncam][slots][nx][cy] (fused with attenuation)
  float* act_c = nullptr;  // column staging for nifti-layout calls (fused)
  float* sino_c = nullptr;
  float* out_c = nullptr;
  float* work = nullptr;
  size_t work_bytes = 0;
  // OSEM state
  int osem_layout = -1;
  float* osem_p = nullptr;
  float* osem_num = nullptr;
  float* sens = nullptr;  // [n_subsets][volume]
  float* prior_grad = nullptr;  // MRF prior gradient (one volume)
  size_t vol_elems = 0, plane_elems = 0;  // per layout of the OSEM buffers
  // mirror-camera units of every subset (index n_subsets: all cameras), camera
  // indexes relative to the subset's first camera; projector and backprojector
  // geometry each
  int2* units_p = nullptr;
  int2* units_b = nullptr;
  std::vector<int> uoff_p, ucnt_p, uoff_b, ucnt_b;
};

size_t al(size_t b) { return (b + 255) / 256 * 256; }

int check() { return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel; }

void range(const Plan& p, int subset, int* b, int* e) {
  if (subset < 0) {
    *b = 0;
    *e = p.proj.cams.n;
  } else {
    *b = p.sub_begin[subset];
    *e = p.sub_begin[subset + 1];
  }
}

// Units of a subset (-1: all cameras) or null.
void subset_units(const Plan& p, int subset, bool back, YgArgs* a) {
  const int i = subset < 0 ? p.n_subsets : subset;
  const std::vector<int>& cnt = back ? p.ucnt_b : p.ucnt_p;
  if (cnt.empty() || cnt[i] == 0) return;
  a->units = (back ? p.units_b : p.units_p) + (back ? p.uoff_b : p.uoff_p)[i];
  a->nunits = cnt[i];
}

int plan_project(Plan& p, int subset, const float* d_act, float* d_sino, int layout, int truncate, cudaStream_t st) {
  int b, e;
  range(p, subset, &b, &e);
  const int n = e - b;
  if (n <= 0) return kOk;
  const Problem& pb = p.proj;
  if (p.fused) {
    const float* act = d_act;
    if (layout == kLayoutNifti) {
      int s = to_column(d_act, p.act_c, pb.nx, pb.ny, p.cy, pb.nz, st);
      if (s != kOk) return s;
      act = p.act_c;
    }
    YgArgs a;
    a.pslabs = tuned_project_slabs(pb.nx, pb.ny, pb.nz, n);  // by the subset's camera count
    a.nx = pb.nx;
    a.ny = pb.ny;
    a.nz = pb.nz;
    a.cy = p.cy;
    a.ncam = n;
    a.geom = p.geom_p + b;
    subset_units(p, subset, false, &a);
    a.act = act;
    a.mu = p.has_att ? p.mu : nullptr;
    a.out = layout == kLayoutNifti ? p.sino_c : d_sino;
    a.psf = p.psf;
    a.psf_host = pb.psf_k ? pb.psf_sep.data() : nullptr;
    a.psf_k = pb.psf_k;
    a.truncate = truncate;
    int s = yg_project(a, st);
    if (s != kOk) return s;
    if (layout == kLayoutNifti) return from_column(p.sino_c, d_sino, pb.nx, pb.ny, p.cy, n, 0, st);
    return kOk;
  }
  if (layout != kLayoutNifti) return kErrParameters;
  GeneralArgs g;
  g.nx = pb.nx;
  g.ny = pb.ny;
  g.nz = pb.nz;
  g.ncam = n;
  g.geom_host = pb.geom.data() + b;
  g.act = d_act;
  g.att = p.has_att ? p.mu : nullptr;
  g.out = d_sino;
  g.psf_sep = p.psf;
  g.psf_k = pb.psf_k;
  g.bg = pb.bg;
  g.bg_att = pb.bg_att;
  g.truncate = truncate;
  const size_t nv = static_cast<size_t>(pb.nx) * pb.ny * pb.nz;
  g.ws_act = p.work;
  g.ws_att = p.work + nv;
  g.ws_tmp = p.work + 2 * nv;
  int s = general_project(g, st);
  return s != kOk ? s : check();
}

int plan_backproject(Plan& p, int subset, const float* d_sino, float* d_out, int layout, int truncate,
                     cudaStream_t st, int pipelined = 1) {
  int b, e;
  range(p, subset, &b, &e);
  const int n = e - b;
  if (n <= 0) return kErrParameters;
  const Problem& pb = p.back;
  if (p.fused) {
    const float* sino = d_sino;
    if (layout == kLayoutNifti) {
      int s = to_column(d_sino, p.sino_c, pb.nx, pb.ny, p.cy, n, st);
      if (s != kOk) return s;
      sino = p.sino_c;
    }
    float* out = layout == kLayoutNifti ? p.out_c : d_out;
    YgArgs a;
    a.nx = pb.nx;
    a.ny = pb.ny;
    a.nz = pb.nz;
    a.cy = p.cy;
    a.ncam = n;
    a.geom = p.geom_b + b;
    subset_units(p, subset, true, &a);
    a.mu = p.has_att ? p.mu : nullptr;
    a.sino = sino;
    a.out = out;
    a.psf = p.psf;
    a.psf_host = pb.psf_k ? pb.psf_sep.data() : nullptr;
    a.psf_k = pb.psf_k;
    a.truncate = truncate;
    a.group = std::min(pb.group, tuned_group(pb.nx, pb.ny, pb.nz, n));  // by the subset's camera count
    a.work = p.work;
    a.carry = p.carry ? p.carry + static_cast<size_t>(b) * yg_carry_slabs() * pb.nx * p.cy : nullptr;
    a.pipelined = pipelined;
    int s = yg_backproject(a, st);
    if (s != kOk) return s;
    // the last gather of every row window already stored max(result, 0) when truncating
    if (layout == kLayoutNifti) return from_column(p.out_c, d_out, pb.nx, pb.ny, p.cy, pb.nz, truncate, st);
    return check();
  }
  if (layout != kLayoutNifti) return kErrParameters;
  GeneralArgs g;
  g.nx = pb.nx;
  g.ny = pb.ny;
  g.nz = pb.nz;
  g.ncam = n;
  g.geom_host = pb.geom.data() + b;
  g.att = p.has_att ? p.mu : nullptr;
  g.sino = d_sino;
  g.out = d_out;
  g.psf_sep = p.psf;
  g.psf_k = pb.psf_k;
  g.bg = pb.bg;
  g.bg_att = pb.bg_att;
  g.truncate = truncate;
  const size_t nv = static_cast<size_t>(pb.nx) * pb.ny * pb.nz;
  g.ws_act = p.work;
  g.ws_att = p.work + nv;
  g.ws_tmp = p.work + 2 * nv;
  int s = general_backproject(g, st);
  return s != kOk ? s : check();
}

}  // namespace
}  // namespace nrgb

using namespace nrgb;

extern "C" {

// Create a plan.  size = {nx, ny, nz}; cameras as for SPECT_project_parallelholes
// ([n x 1|3|6], axis-major); psf host [k, k, >= nz] or null; d_attenuation a
// device volume (nifti order) or null; subset_of_camera: per camera its subset
// in [0, n_subsets), or null for a single subset.
int nrgb_plan_create(void** out_plan, const int* size, const float* cameras, const int* cameras_size,
                     const float* psf, const int* psf_size, const float* d_attenuation, float background,
                     float background_attenuation, const int* subset_of_camera, int n_subsets, void* stream) {
  NRGB_API("nrgb_plan_create");
  if (!out_plan || !size || !cameras || !cameras_size || n_subsets < 1) return kErrParameters;
  *out_plan = nullptr;
  const int nx = size[0], ny = size[1], nz = size[2], ncam = cameras_size[0], ncols = cameras_size[1];
  if (nx <= 0 || ny <= 0 || nz <= 0 || ncam <= 0) return kErrParameters;
  // subset order: cameras of subset 0, then subset 1, ...; stable inside a subset
  std::vector<int> order;
  std::vector<int> begin(n_subsets + 1, 0);
  for (int s = 0; s < n_subsets; ++s) {
    begin[s] = static_cast<int>(order.size());
    for (int c = 0; c < ncam; ++c) {
      const int sc = subset_of_camera ? subset_of_camera[c] : 0;
      if (sc < 0 || sc >= n_subsets) return kErrParameters;
      if (sc == s) order.push_back(c);
    }
  }
  begin[n_subsets] = ncam;
  // reorder the camera table (all 6 columns' meaning kept)
  Cameras cp, cb;
  const int psz[3] = {size[0], size[1], size[2]};
  const int bsz[3] = {size[0], size[1], size[0]};
  int s = expand_cameras(cameras, ncam, ncols, psz, &cp);
  if (s != kOk) return s;
  s = expand_cameras(cameras, ncam, ncols, bsz, &cb);
  if (s != kOk) return s;
  auto reorder = [&](Cameras& c) {
    Cameras r = c;
    for (int i = 0; i < ncam; ++i)
      for (int a = 0; a < 3; ++a) {
        r.angles[a * ncam + i] = c.angles[a * ncam + order[i]];
        r.centers[a * ncam + i] = c.centers[a * ncam + order[i]];
      }
    c = r;
  };
  reorder(cp);
  reorder(cb);
  Plan* p = new (std::nothrow) Plan();
  if (!p) return kErrAllocCpu;
  cudaGetDevice(&p->device);
  s = make_problem(nx, ny, nz, cp, psf, psf_size, background, background_attenuation, 0, &p->proj);
  if (s == kOk) s = make_problem(nx, ny, nz, cb, psf, psf_size, background, background_attenuation, 0, &p->back);
  if (s != kOk) {
    delete p;
    return s;
  }
  p->fused = use_fused(p->proj);
  p->has_att = d_attenuation != nullptr;
  p->cy = round_up(ny, 4);
  p->n_subsets = n_subsets;
  p->sub_begin = begin;
  p->order = order;
  int max_sub = 0;
  for (int i = 0; i < n_subsets; ++i) max_sub = std::max(max_sub, begin[i + 1] - begin[i]);
  // mirror units per subset and for all cameras (fused path, mirror pairs on)
  std::vector<int> hu_p, hu_b;
  if (p->fused && mirror_pairs()) {
    auto units_of = [&](const Cameras& all, std::vector<int>& host, std::vector<int>& off, std::vector<int>& cnt) {
      off.assign(n_subsets + 1, 0);
      cnt.assign(n_subsets + 1, 0);
      for (int i = 0; i <= n_subsets; ++i) {
        const int b = i < n_subsets ? begin[i] : 0, e = i < n_subsets ? begin[i + 1] : ncam;
        if (e <= b) continue;
        Cameras sub;
        sub.n = e - b;
        sub.angles.resize(3 * static_cast<size_t>(sub.n));
        sub.centers.resize(3 * static_cast<size_t>(sub.n));
        for (int a = 0; a < 3; ++a)
          for (int c = 0; c < sub.n; ++c) {
            sub.angles[a * sub.n + c] = all.angles[a * ncam + b + c];
            sub.centers[a * sub.n + c] = all.centers[a * ncam + b + c];
          }
        const std::vector<int> u = mirror_units(sub, nx, nz);
        off[i] = static_cast<int>(host.size() / 2);
        cnt[i] = static_cast<int>(u.size() / 2);
        host.insert(host.end(), u.begin(), u.end());
      }
    };
    units_of(p->proj.cams, hu_p, p->uoff_p, p->ucnt_p);
    units_of(p->back.cams, hu_b, p->uoff_b, p->ucnt_b);
  }

  const size_t nv = static_cast<size_t>(nx) * ny * nz;
  const size_t ncv = static_cast<size_t>(nx) * p->cy * nz;
  const size_t nsc = static_cast<size_t>(nx) * p->cy * ncam;
  size_t bytes = al(sizeof(CamGeom) * ncam) * 2 + al(sizeof(float) * p->proj.psf_sep.size()) +
                 al(sizeof(int) * hu_p.size()) + al(sizeof(int) * hu_b.size());
  if (p->fused) {
    bytes += al(sizeof(float) * ncv) * (p->has_att ? 4 : 3) + al(sizeof(float) * nsc);
    if (p->has_att) bytes += al(sizeof(float) * static_cast<size_t>(ncam) * yg_carry_slabs() * nx * p->cy);
    p->work_bytes = yg_backproject_workspace(nx, ny, nz, ncam, p->back.group, 2) -
                    sizeof(float) * static_cast<size_t>(ncam) * yg_carry_slabs() * nx * p->cy;
  } else {
    bytes += al(sizeof(float) * nv) * (p->has_att ? 1 : 0);
    p->work_bytes = sizeof(float) * nv * 3;
  }
  bytes += al(p->work_bytes);
  if (cudaMalloc(&p->mem, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    return kErrAllocGpu;
  }
  p->bytes = bytes;
  Carver cv(p->mem, bytes);
  p->geom_p = cv.take<CamGeom>(ncam);
  p->geom_b = cv.take<CamGeom>(ncam);
  if (!p->proj.psf_sep.empty()) p->psf = cv.take<float>(p->proj.psf_sep.size());
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaMemcpyAsync(p->geom_p, p->proj.geom.data(), sizeof(CamGeom) * ncam, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(p->geom_b, p->back.geom.data(), sizeof(CamGeom) * ncam, cudaMemcpyHostToDevice, st);
  if (p->psf)
    cudaMemcpyAsync(p->psf, p->proj.psf_sep.data(), sizeof(float) * p->proj.psf_sep.size(), cudaMemcpyHostToDevice,
                    st);
  // the host vectors live until the copies have consumed them: pageable
  // copies return after staging the source
  if (!hu_p.empty()) {
    p->units_p = cv.take<int2>(hu_p.size() / 2);
    cudaMemcpyAsync(p->units_p, hu_p.data(), sizeof(int) * hu_p.size(), cudaMemcpyHostToDevice, st);
  }
  if (!hu_b.empty()) {
    p->units_b = cv.take<int2>(hu_b.size() / 2);
    cudaMemcpyAsync(p->units_b, hu_b.data(), sizeof(int) * hu_b.size(), cudaMemcpyHostToDevice, st);
  }
  if (p->fused) {
    if (p->has_att) p->mu = cv.take<float>(ncv);
    p->act_c = cv.take<float>(ncv);
    p->out_c = cv.take<float>(ncv);
    p->sino_c = cv.take<float>(nsc);
    if (p->has_att) {
      p->carry = cv.take<float>(static_cast<size_t>(ncam) * yg_carry_slabs() * nx * p->cy);
      s = to_column(d_attenuation, p->mu, nx, ny, p->cy, nz, st);
      YgArgs a;
      a.nx = nx;
      a.ny = ny;
      a.nz = nz;
      a.cy = p->cy;
      a.ncam = ncam;
      a.geom = p->geom_b;
      a.mu = p->mu;
      if (s == kOk) s = yg_mu_carry(a, p->carry, st);
    }
  } else if (p->has_att) {
    p->mu = cv.take<float>(nv);
    cudaMemcpyAsync(p->mu, d_attenuation, sizeof(float) * nv, cudaMemcpyDeviceToDevice, st);
  }
  p->work = cv.take<float>((p->work_bytes + sizeof(float) - 1) / sizeof(float));
  if (s == kOk) s = check();
  if (s != kOk || !p->work) {
    cudaFree(p->mem);
    delete p;
    return s != kOk ? s : kErrAllocGpu;
  }
  *out_plan = p;
  return kOk;
}

int nrgb_plan_destroy(void* plan) {
  NRGB_API("nrgb_plan_destroy");
  Plan* p = static_cast<Plan*>(plan);
  if (!p) return kErrParameters;
  cudaDeviceSynchronize();
  cudaFree(p->mem);
  if (p->osem_p) cudaFree(p->osem_p);
  delete p;
  return kOk;
}

// out[0..6] = {nx, ny, nz, cy, n_cameras, n_subsets, fused}
int nrgb_plan_shape(void* plan, int* out) {
  NRGB_API("nrgb_plan_shape");
  Plan* p = static_cast<Plan*>(plan);
  if (!p || !out) return kErrParameters;
  out[0] = p->proj.nx;
  out[1] = p->proj.ny;
  out[2] = p->proj.nz;
  out[3] = p->cy;
  out[4] = p->proj.cams.n;
  out[5] = p->n_subsets;
  out[6] = p->fused ? 1 : 0;
  return kOk;
}

// Original camera indexes of a subset, in the order its sinogram planes use;
// returns the subset size (subset -1: all cameras).
int nrgb_plan_subset_cameras(void* plan, int subset, int* idx_out) {
  NRGB_API("nrgb_plan_subset_cameras");
  Plan* p = static_cast<Plan*>(plan);
  if (!p || subset < -1 || subset >= p->n_subsets) return -1;
  int b, e;
  range(*p, subset, &b, &e);
  if (idx_out)
    for (int i = b; i < e; ++i) idx_out[i - b] = p->order[i];
  return e - b;
}

// Project the cameras of `subset` (-1: all) of d_activity into d_sinogram
// ([n_subset][ny][nx] nifti or [n_subset][nx][cy] column layout).
int nrgb_plan_project(void* plan, int subset, const float* d_activity, float* d_sinogram, int layout, int truncate,
                      void* stream) {
  NRGB_API("nrgb_plan_project");
  Plan* p = static_cast<Plan*>(plan);
  if (!p || subset < -1 || subset >= p->n_subsets || !d_activity || !d_sinogram) return kErrParameters;
  return plan_project(*p, subset, d_activity, d_sinogram, layout, truncate, static_cast<cudaStream_t>(stream));
}

// Backproject d_sinogram (cameras of `subset`) into d_out (reference semantics).
int nrgb_plan_backproject(void* plan, int subset, const float* d_sinogram, float* d_out, int layout, int truncate,
                          void* stream) {
  NRGB_API("nrgb_plan_backproject");
  Plan* p = static_cast<Plan*>(plan);
  if (!p || subset < -1 || subset >= p->n_subsets || !d_sinogram || !d_out) return kErrParameters;
  return plan_backproject(*p, subset, d_sinogram, d_out, layout, truncate, static_cast<cudaStream_t>(stream));
}

// Allocate the OSEM buffers for `layout` and compute every subset's
// sensitivity image (backprojection of ones, truncated; floored at epsilon in
// the update) once.  Call before capturing OSEM steps in a graph.
int nrgb_plan_osem_prepare(void* plan, int layout, void* stream) {
  NRGB_API("nrgb_plan_osem_prepare");
  Plan* p = static_cast<Plan*>(plan);
  if (!p || (layout != kLayoutNifti && layout != kLayoutColumn)) return kErrParameters;
  if (layout == kLayoutColumn && !p->fused) return kErrParameters;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Problem& pb = p->proj;
  const int ny_l = layout == kLayoutColumn ? p->cy : pb.ny;
  p->vol_elems = static_cast<size_t>(pb.nx) * ny_l * pb.nz;
  p->plane_elems = static_cast<size_t>(pb.nx) * ny_l;
  int max_sub = 0;
  for (int i = 0; i < p->n_subsets; ++i) max_sub = std::max(max_sub, p->sub_begin[i + 1] - p->sub_begin[i]);
  if (p->osem_p) cudaFree(p->osem_p);
  p->osem_p = nullptr;
  const size_t n_p = al(sizeof(float) * p->plane_elems * max_sub);
  const size_t n_v = al(sizeof(float) * p->vol_elems);
  if (cudaMalloc(&p->osem_p, n_p + n_v * (2 + p->n_subsets)) != cudaSuccess) {
    cudaGetLastError();
    p->osem_p = nullptr;
    return kErrAllocGpu;
  }
  char* base = reinterpret_cast<char*>(p->osem_p);
  p->osem_num = reinterpret_cast<float*>(base + n_p);
  p->sens = reinterpret_cast<float*>(base + n_p + n_v);
  p->prior_grad = reinterpret_cast<float*>(base + n_p + n_v * (1 + p->n_subsets));
  p->osem_layout = layout;
  cudaMemsetAsync(p->osem_p, 0, n_p + n_v * (2 + p->n_subsets), st);
  for (int sidx = 0; sidx < p->n_subsets; ++sidx) {
    const int n = p->sub_begin[sidx + 1] - p->sub_begin[sidx];
    if (n <= 0) continue;
    int s = fill(p->osem_p, p->plane_elems * n, 1.0f, st);
    if (s == kOk && layout == kLayoutColumn) {
      // column pads stay zero
      s = to_column(p->osem_p, p->sino_c, pb.nx, pb.ny, p->cy, n, st);
      if (s == kOk) s = cudaMemcpyAsync(p->osem_p, p->sino_c, sizeof(float) * p->plane_elems * n,
                                        cudaMemcpyDeviceToDevice, st) == cudaSuccess ? kOk : kErrTransferGpu;
    }
    if (s == kOk)
      s = plan_backproject(*p, sidx, p->osem_p, p->sens + p->vol_elems * sidx, layout, 1, st);
    if (s != kOk) return s;
  }
  return check();
}

// One OSEM step over `subset` with the reference's update
// (emission-lib/_et_array_interface.cpp:1017-1044): p = A x (truncated),
// r = y / max-rule(p), x *= (A^T r, truncated) / max(sensitivity, eps).
// d_activity and d_counts use the layout given to nrgb_plan_osem_prepare;
// d_counts holds the subset's planes in nrgb_plan_subset_cameras order.
int nrgb_plan_osem_step(void* plan, int subset, float* d_activity, const float* d_counts, float epsilon,
                        void* stream) {
  NRGB_API("nrgb_plan_osem_step");
  Plan* p = static_cast<Plan*>(plan);
  if (!p || subset < 0 || subset >= p->n_subsets || !d_activity || !d_counts || p->osem_layout < 0)
    return kErrParameters;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int n = p->sub_begin[subset + 1] - p->sub_begin[subset];
  if (n <= 0) return kOk;
  const float* sens = p->sens + p->vol_elems * subset;
  int s = plan_project(*p, subset, d_activity, p->osem_p, p->osem_layout, 1, st);
  if (s == kOk) s = osem_ratio(d_counts, p->osem_p, p->plane_elems * n, epsilon, st);
  if (s == kOk) s = plan_backproject(*p, subset, p->osem_p, p->osem_num, p->osem_layout, 1, st);
  if (s == kOk) s = osem_update(d_activity, p->osem_num, sens, p->vol_elems, epsilon, st);
  return s;
}

// One-step-late MAP-EM step with the quadratic MRF prior
// (et_osmapem_step, Python/NiftyRec/NiftyRec/NiftyRec.py:224-245, prior
// gradient of :400-404 computed from the current activity): p = A x
// (truncated), r = y / (max(p, 0) + eps), u = A^T r (truncated),
// x *= max(u, 0) / (max(sens - beta * g, 0) + eps).  beta = 0 is OSEM with the
// OSL ratio rule.  Same layouts as nrgb_plan_osem_step.
int nrgb_plan_osmapem_step(void* plan, int subset, float* d_activity, const float* d_counts, float beta,
                           float epsilon, void* stream) {
  NRGB_API("nrgb_plan_osmapem_step");
  Plan* p = static_cast<Plan*>(plan);
  if (!p || subset < 0 || subset >= p->n_subsets || !d_activity || !d_counts || p->osem_layout < 0)
    return kErrParameters;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int n = p->sub_begin[subset + 1] - p->sub_begin[subset];
  if (n <= 0) return kOk;
  const Problem& pb = p->proj;
  const bool col = p->osem_layout == kLayoutColumn;
  int s = kOk;
  if (beta != 0.0f)
    s = mrf_gradient(d_activity, p->prior_grad, col ? p->cy : pb.nx, col ? pb.nx : pb.ny, pb.nz, st);
  if (s == kOk) s = plan_project(*p, subset, d_activity, p->osem_p, p->osem_layout, 1, st);
  if (s == kOk) s = osem_ratio_osl(d_counts, p->osem_p, p->plane_elems * n, epsilon, st);
  if (s == kOk) s = plan_backproject(*p, subset, p->osem_p, p->osem_num, p->osem_layout, 1, st);
  if (s == kOk)
    s = osem_update_osl(d_activity, p->osem_num, p->sens + p->vol_elems * subset, beta != 0.0f ? p->prior_grad : nullptr,
                        p->vol_elems, beta, epsilon, st);
  return s;
}

// Quadratic MRF prior gradient of a device volume in nifti order (nx fastest).
int nrgb_mrf_gradient_device(const float* d_activity, float* d_gradient, const int* size, void* stream) {
  NRGB_API("nrgb_mrf_gradient_device");
  if (!d_activity || !d_gradient || !size || size[0] <= 0 || size[1] <= 0 || size[2] <= 0) return kErrParameters;
  return mrf_gradient(d_activity, d_gradient, size[0], size[1], size[2], static_cast<cudaStream_t>(stream));
}

// Layout conversion for callers of the column-layout entry points:
// direction 0: nifti [planes][ny][nx] -> column [planes][nx][cy];
// direction 1: column -> nifti (truncate: clamp negatives to 0).
int nrgb_layout_convert(const float* src, float* dst, int nx, int ny, int planes, int direction, int truncate,
                        void* stream) {
  NRGB_API("nrgb_layout_convert");
  if (!src || !dst || nx <= 0 || ny <= 0 || planes <= 0) return kErrParameters;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int cy = round_up(ny, 4);
  return direction == 0 ? to_column(src, dst, nx, ny, cy, planes, st)
                        : from_column(src, dst, nx, ny, cy, planes, truncate, st);
}

}  // extern "C"

// ------------------------------------------------------------------ batches
// A batch runs one OSEM subset step of many plans at once: one persistent
// projector launch over every volume's subset cameras (per PSF width and
// attenuation kind), one ratio launch, the plans' reference backprojections
// concurrently on side streams, one update launch.  The batch owns each volume's activity and counts in
// column layout; its descriptors are built once, so a step allocates nothing,
// copies nothing from the host and can be captured in a CUDA graph.
namespace nrgb {
namespace {

// Side streams of a batch step: the volumes' backprojections run
// concurrently on them (each volume on its own scratch), forked from and
// joined back into the caller's stream with events (capturable in a CUDA
// graph).
constexpr int kBatchStreams = 4;

struct Batch {
  int device = 0;
  cudaStream_t side[kBatchStreams] = {};
  cudaEvent_t fork = nullptr, join[kBatchStreams] = {};
  std::vector<Plan*> plans;
  std::vector<int> order;      // volumes by decreasing work per item (large first)
  char* mem = nullptr;
  std::vector<float*> act;     // per volume: [nz][nx][cy]
  std::vector<float*> counts;  // per volume: [ncam][nx][cy], plan camera order
  std::vector<int> desc_base;  // per volume: descriptor index of subset 0
  std::vector<BatchStepDesc> h_desc;
  BatchStepDesc* d_desc = nullptr;
  int* d_counter = nullptr;    // one per projector launch of a step
};

void destroy_batch_streams(Batch* b) {
  if (b->fork) cudaEventDestroy(b->fork);
  for (int k = 0; k < kBatchStreams; ++k) {
    if (b->join[k]) cudaEventDestroy(b->join[k]);
    if (b->side[k]) cudaStreamDestroy(b->side[k]);
  }
  b->fork = nullptr;
}

}  // namespace
}  // namespace nrgb

extern "C" {

// Build a batch over fused plans prepared for OSEM in column layout
// (nrgb_plan_osem_prepare(plan, 1, ...)).  At most 64 plans, one device.
int nrgb_batch_create(void** out_batch, void* const* plans, int n_plans, void* stream) {
  NRGB_API("nrgb_batch_create");
  if (!out_batch || !plans || n_plans < 1 || n_plans > kMaxBatch) return kErrParameters;
  *out_batch = nullptr;
  Batch* b = new (std::nothrow) Batch();
  if (!b) return kErrAllocCpu;
  cudaGetDevice(&b->device);
  bool ok = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < kBatchStreams && ok; ++k)
    ok = cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    destroy_batch_streams(b);
    delete b;
    return kErrUnspecified;
  }
  size_t bytes = al(sizeof(int) * kMaxBatch);
  int ndesc = 0;
  for (int v = 0; v < n_plans; ++v) {
    Plan* p = static_cast<Plan*>(plans[v]);
    if (!p || !p->fused || p->osem_layout != kLayoutColumn || p->device != b->device) {
      destroy_batch_streams(b);
      delete b;
      return kErrParameters;
    }
    b->plans.push_back(p);
    const Problem& pb = p->proj;
    bytes += al(sizeof(float) * static_cast<size_t>(pb.nz) * pb.nx * p->cy);
    bytes += al(sizeof(float) * static_cast<size_t>(pb.cams.n) * pb.nx * p->cy);
    b->desc_base.push_back(ndesc);
    ndesc += p->n_subsets;
  }
  bytes += al(sizeof(BatchStepDesc) * ndesc);
  if (cudaMalloc(&b->mem, bytes) != cudaSuccess) {
    cudaGetLastError();
    destroy_batch_streams(b);
    delete b;
    return kErrAllocGpu;
  }
  Carver cv(b->mem, bytes);
  b->d_counter = cv.take<int>(kMaxBatch);
  b->h_desc.resize(ndesc);
  for (int v = 0; v < n_plans; ++v) {
    Plan* p = b->plans[v];
    const Problem& pb = p->proj;
    b->act.push_back(cv.take<float>(static_cast<size_t>(pb.nz) * pb.nx * p->cy));
    b->counts.push_back(cv.take<float>(static_cast<size_t>(pb.cams.n) * pb.nx * p->cy));
    for (int s = 0; s < p->n_subsets; ++s) {
      BatchStepDesc& d = b->h_desc[b->desc_base[v] + s];
      const int c0 = p->sub_begin[s], n = p->sub_begin[s + 1] - c0;
      const size_t plane = static_cast<size_t>(pb.nx) * p->cy;
      YgArgs& a = d.proj;
      a.nx = pb.nx;
      a.ny = pb.ny;
      a.nz = pb.nz;
      a.cy = p->cy;
      a.ncam = n;
      a.geom = p->geom_p + c0;
      a.act = b->act[v];
      a.mu = p->has_att ? p->mu : nullptr;
      a.out = p->osem_p;
      a.psf = p->psf;
      a.psf_k = pb.psf_k;
      a.truncate = 1;
      d.nwin = yg_row_windows(pb.ny, pb.psf_k, &d.win[0][0], kMaxWindows);
      if (d.nwin < 0) {
        cudaFree(b->mem);
        destroy_batch_streams(b);
        delete b;
        return kErrParameters;
      }
      d.counts = b->counts[v] + plane * c0;
      d.act = b->act[v];
      d.num = p->osem_num;
      d.sens = p->sens + p->vol_elems * s;
      d.sino_elems = static_cast<long long>(plane) * n;
      d.vol_elems = static_cast<long long>(p->vol_elems);
    }
  }
  b->d_desc = cv.take<BatchStepDesc>(ndesc);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(b->d_desc, b->h_desc.data(), sizeof(BatchStepDesc) * ndesc, cudaMemcpyHostToDevice, st) !=
      cudaSuccess) {
    cudaFree(b->mem);
    destroy_batch_streams(b);
    delete b;
    return kErrTransferGpu;
  }
  cudaStreamSynchronize(st);  // the host descriptors are pageable
  // large items first: the persistent projector then ends on small items
  b->order.resize(n_plans);
  for (int v = 0; v < n_plans; ++v) b->order[v] = v;
  std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
    const Problem& px = b->plans[x]->proj;
    const Problem& py = b->plans[y]->proj;
    return static_cast<long long>(px.nz) * b->plans[x]->cy > static_cast<long long>(py.nz) * b->plans[y]->cy;
  });
  *out_batch = b;
  return kOk;
}

int nrgb_batch_destroy(void* batch) {
  NRGB_API("nrgb_batch_destroy");
  Batch* b = static_cast<Batch*>(batch);
  if (!b) return kErrParameters;
  cudaDeviceSynchronize();
  destroy_batch_streams(b);
  cudaFree(b->mem);
  delete b;
  return kOk;
}

// Counts of volume v: device (n_cameras, ny, nx) nifti, original camera order.
int nrgb_batch_set_counts(void* batch, int v, const float* d_counts, void* stream) {
  NRGB_API("nrgb_batch_set_counts");
  Batch* b = static_cast<Batch*>(batch);
  if (!b || v < 0 || v >= static_cast<int>(b->plans.size()) || !d_counts) return kErrParameters;
  const Plan& p = *b->plans[v];
  const Problem& pb = p.proj;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t in_plane = static_cast<size_t>(pb.nx) * pb.ny, out_plane = static_cast<size_t>(pb.nx) * p.cy;
  for (int i = 0; i < pb.cams.n; ++i) {
    const int s = to_column(d_counts + in_plane * p.order[i], b->counts[v] + out_plane * i, pb.nx, pb.ny, p.cy, 1, st);
    if (s != kOk) return s;
  }
  return kOk;
}

// Activity of volume v in and out, device (nz, ny, nx) nifti.
int nrgb_batch_set_activity(void* batch, int v, const float* d_activity, void* stream) {
  NRGB_API("nrgb_batch_set_activity");
  Batch* b = static_cast<Batch*>(batch);
  if (!b || v < 0 || v >= static_cast<int>(b->plans.size()) || !d_activity) return kErrParameters;
  const Plan& p = *b->plans[v];
  return to_column(d_activity, b->act[v], p.proj.nx, p.proj.ny, p.cy, p.proj.nz, static_cast<cudaStream_t>(stream));
}

int nrgb_batch_get_activity(void* batch, int v, float* d_activity, void* stream) {
  NRGB_API("nrgb_batch_get_activity");
  Batch* b = static_cast<Batch*>(batch);
  if (!b || v < 0 || v >= static_cast<int>(b->plans.size()) || !d_activity) return kErrParameters;
  const Plan& p = *b->plans[v];
  return from_column(b->act[v], d_activity, p.proj.nx, p.proj.ny, p.cy, p.proj.nz, 0,
                     static_cast<cudaStream_t>(stream));
}

// One OSEM subset step of every volume: volume v runs its subset
// (step mod n_subsets_v) with the update of nrgb_plan_osem_step.  With
// iterations > 0, volumes that have completed that many passes over their
// subsets (step >= iterations * n_subsets_v) sit the step out, so volumes with
// different subset counts all end after `iterations` iterations.
int nrgb_batch_osem_step(void* batch, int step, int iterations, float epsilon, void* stream) {
  NRGB_API("nrgb_batch_osem_step");
  Batch* b = static_cast<Batch*>(batch);
  if (!b || step < 0) return kErrParameters;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  BatchElems ratio_e, vol_e;
  // projector launches: one per (PSF width, attenuation) among the volumes
  std::vector<std::pair<int, int>> kinds;
  std::vector<int> sub(b->plans.size(), -1);
  for (int v : b->order) {
    Plan& p = *b->plans[v];
    if (iterations > 0 && step >= iterations * p.n_subsets) continue;
    const int s = step % p.n_subsets;
    if (p.sub_begin[s + 1] - p.sub_begin[s] <= 0) continue;
    sub[v] = s;
    const std::pair<int, int> kind(p.proj.psf_k, p.has_att ? 1 : 0);
    if (std::find(kinds.begin(), kinds.end(), kind) == kinds.end()) kinds.push_back(kind);
    const BatchStepDesc& d = b->h_desc[b->desc_base[v] + s];
    ratio_e.desc[ratio_e.n] = vol_e.desc[vol_e.n] = b->desc_base[v] + s;
    ratio_e.begin[ratio_e.n + 1] = ratio_e.begin[ratio_e.n] + d.sino_elems;
    vol_e.begin[vol_e.n + 1] = vol_e.begin[vol_e.n] + d.vol_elems;
    ++ratio_e.n;
    ++vol_e.n;
  }
  if (static_cast<int>(kinds.size()) > kMaxBatch) return kErrParameters;
  if (cudaMemsetAsync(b->d_counter, 0, sizeof(int) * kinds.size(), st) != cudaSuccess) return kErrKernel;
  for (size_t k = 0; k < kinds.size(); ++k) {
    BatchSel sel;
    int max_nz = 0;
    for (int v : b->order) {
      const Plan& p = *b->plans[v];
      if (sub[v] < 0 || p.proj.psf_k != kinds[k].first || (p.has_att ? 1 : 0) != kinds[k].second) continue;
      const BatchStepDesc& d = b->h_desc[b->desc_base[v] + sub[v]];
      const int ntile = (d.proj.nx + 31) / 32;
      sel.desc[sel.n] = b->desc_base[v] + sub[v];
      sel.begin[sel.n + 1] = sel.begin[sel.n] + d.nwin * d.proj.ncam * ntile;
      ++sel.n;
      max_nz = std::max(max_nz, d.proj.nz);
    }
    sel.total = sel.begin[sel.n];
    const int s = yg_project_batch(b->d_desc, sel, kinds[k].first, kinds[k].second != 0, max_nz, b->d_counter + k, st);
    if (s != kOk) return s;
  }
  int s = osem_ratio_batch(b->d_desc, ratio_e, epsilon, st);
  if (s != kOk) return s;
  // the backprojections, volume by volume (largest first) on the least loaded
  // side stream, each spread and gather in sequence on its stream
  if (cudaEventRecord(b->fork, st) != cudaSuccess) return kErrKernel;
  for (int k = 0; k < kBatchStreams; ++k) cudaStreamWaitEvent(b->side[k], b->fork, 0);
  double load[kBatchStreams] = {};
  for (int v : b->order) {
    if (sub[v] < 0 || s != kOk) continue;
    Plan& p = *b->plans[v];
    const int k = static_cast<int>(std::min_element(load, load + kBatchStreams) - load);
    load[k] += static_cast<double>(p.back.nz) * p.back.nx * p.cy * (p.sub_begin[sub[v] + 1] - p.sub_begin[sub[v]]);
    s = plan_backproject(p, sub[v], p.osem_p, p.osem_num, kLayoutColumn, 1, b->side[k], 0);
  }
  for (int k = 0; k < kBatchStreams; ++k) {
    cudaEventRecord(b->join[k], b->side[k]);
    cudaStreamWaitEvent(st, b->join[k], 0);
  }
  if (s == kOk) s = osem_update_batch(b->d_desc, vol_e, epsilon, st);
  return s;
}

}  // extern "C"
