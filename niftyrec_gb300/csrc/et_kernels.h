// Launch-side declarations of the CUDA kernels (device code in et_general.cu,
// et_yg_*.cu / et_yg_*.cuh and et_ygantry.cu, et_update.cu, et_fisher.cu).
#pragma once

#include <cuda_runtime.h>

#include "et_common.h"

namespace nrgb {

// ---- general-orientation path (nifti layout) ----
template <class T>
struct GeneralArgsT {
  int nx = 0, ny = 0, nz = 0, ncam = 0;
  const CamGeomT<T>* geom_host = nullptr;  // host array; matrices go to kernels by value
  const T* act = nullptr;                  // device volume or null
  const T* att = nullptr;                  // device volume or null
  const T* sino = nullptr;                 // device sinogram input (backprojection, gradient)
  T* out = nullptr;                        // device output
  const T* psf_sep = nullptr;              // device [nz][2k] or null
  int psf_k = 0;
  T bg = 0, bg_att = 0;
  int truncate = 0;
  T* ws_act = nullptr;  // three nvox work volumes
  T* ws_att = nullptr;
  T* ws_tmp = nullptr;
};
using GeneralArgs = GeneralArgsT<float>;
// The same projector / backprojector evaluated in float64 (every product,
// sum, position and exp in double): the float64 reference run that the
// float32 and bfloat16-storage results are measured against.
using GeneralArgs64 = GeneralArgsT<double>;
int general_project64(const GeneralArgs64& a, cudaStream_t st);
int general_backproject64(const GeneralArgs64& a, cudaStream_t st);
int general_project(const GeneralArgs& a, cudaStream_t st);
// Projection with partial sums (et_project_partial): a.out the sinogram,
// partial [ncam][nz][ny][nx] the emission reaching each depth from behind,
// in the rotated frame or (do_rotate) rotated back; bg_image [ny][nx] or null.
int general_project_partial(const GeneralArgs& a, const float* bg_image, float* partial, int do_rotate,
                            cudaStream_t st);
int general_backproject(const GeneralArgs& a, cudaStream_t st);
int general_gradient(const GeneralArgs& a, cudaStream_t st);
// Exact transpose of general_project's linear part (backprojector mode 1).
int general_adjoint(const GeneralArgs& a, cudaStream_t st);
// d/dmu of sum(g * project(act, mu)); a.sino = g (sinogram), a.out = gradient.
int general_dmu(const GeneralArgs& a, cudaStream_t st);
int general_rotate(const float* src, float* dst, int nx, int ny, int nz, const float* m12, float bg, cudaStream_t st);
// Per-slice 2D convolution of nz slices (nx x ny, x fastest) with kernel slices
// [nz][ky][kx], centre ((kx-1)/2, (ky-1)/2), image clamped at its border.
int general_convolve2d(const float* src, float* dst, int nx, int ny, int nz, const float* psf, int kx, int ky,
                       cudaStream_t st);

// ---- y-gantry fused path (column layout) ----
// Callers describe whole volumes (ny rows, column stride cy = round_up(ny, 4));
// yg_project / yg_backproject split them into row windows of at most 128
// rows and fill row0 / out_lo / out_hi / cs per launch (ny then counts the
// window's rows).
struct YgArgs {
  int nx = 0, ny = 0, nz = 0, cy = 0, ncam = 0;
  int row0 = 0;                   // first row of the window (multiple of 4)
  int out_lo = 0, out_hi = 1 << 30;  // valid output rows of the window, relative to row0
  int cs = 0;                     // column stride of the backprojector's scratch
  const CamGeom* geom = nullptr;  // device [ncam]
  const float* act = nullptr;     // [nz][nx][cy] (bfloat16 data when storage == kStorageBF16)
  const float* mu = nullptr;      // [nz][nx][cy] or null (same storage as act)
  const float* sino = nullptr;    // [ncam][nx][cy] (backprojection input)
  float* out = nullptr;           // projector: [ncam][nx][cy]; backprojector: [nz][nx][cy]
  const float* psf = nullptr;     // device [nz][2k] or null
  const float* psf_host = nullptr;  // host copy of psf (valid during the launching call) or null
  int psf_k = 0;
  int truncate = 0;
  int back_mode = kBackReference;
  int storage = kStorageF32;  // type of act and mu
  int pslabs = 0;  // projector depth slabs = cluster size (2, 4, 8; 0: chosen by the launcher)
  // Units (device [nunits]): {camera, mirror camera or -1}; a mirror camera
  // sits at the opposite angle about the grid centre and is served from the
  // same samples by the projector and the reference-mode backprojector
  // (float32 storage).  Null: unit u = camera u.
  const int2* units = nullptr;
  int nunits = 0;
  // backprojector work space (yg_backproject_workspace bytes); the kernels
  // see it as carries [ncam][slots][nx][cy] then scratch [group][nz][nx][cy]
  float* work = nullptr;
  float* slab_T = nullptr;
  float* temp = nullptr;
  int group = 16;
  // Backprojector depth slabs (1..16): carries hold bslabs + 1 slots per
  // camera (every slab's exclusive prefix, then the column total).
  int bslabs = 16;
  // Projector: non-null -> also write the transmission carries of its own
  // depth slabs ([ncam][pslabs + 1][nx][cy], the layout above with bslabs =
  // the projector's slab count; with units, at each unit's first camera).
  float* carry_out = nullptr;
  // Projector with carry_out: 1 -> also record the transmission at the middle
  // of every depth slab, so the carries serve twice as many backprojector
  // slabs (the launcher applies it where the halves line up and the result
  // has at most 8 slabs; slabs_used reports the carries' slab count).
  int carry_split = 0;
  // 1: spread on the caller's stream, gather on a second stream, two scratch
  // slots; 0: both on the caller's stream with one slot (creates no stream
  // or event).
  int pipelined = 1;
  // Backprojector: non-null when the caller produces a.sino on another
  // stream; this event (a cudaEvent_t) marks its completion and is waited
  // for after the transmission carries are launched, which overlap it.
  void* sino_ready = nullptr;
  // Non-null: transmission carries [ncam][slots][nx][cy] computed beforehand
  // (yg_mu_carry) for exactly these cameras; the backprojector then skips
  // that pass and the work space holds only the scratch slot(s).
  const float* carry = nullptr;
  // yg_backproject (reference form, deterministic transpose): the window's
  // last gather stores max(result, 0) when a.truncate is set.
  // Non-zero: yg_backproject spreads the reference's attenuation gradient
  // instead (a.act and a.mu sampled, a.sino the camera planes; no carries,
  // no mirror units), then gathers it like the reference-mode backprojection.
  int gradient = 0;
  // Non-zero (exact-transpose backprojector, d/dmu): deterministic form --
  // the rotated-frame values go into the group scratch instead of vector
  // reductions into a.out, and a transposed gather (fixed order) sums them.
  int det = 0;
  // d/dmu: first camera of the launch (scratch volume g = camera - cam0).
  int cam0 = 0;
};
// Carry slots per camera of the backprojector's transmission carries (the
// exclusive prefix of every depth slab, then the column total).
int yg_carry_slabs();
// Transmission carries of the rotated mu for a.ncam cameras into out
// ([ncam][slots][nx][cy]); with a.units only the units' first cameras.
int yg_mu_carry(const YgArgs& a, float* out, cudaStream_t st);
// True when the fused kernels support this grid / PSF size.
bool yg_supported(int nx, int ny, int nz, int psf_k);
// Bytes of work space yg_backproject needs (slab carries + `slots` camera-group
// scratch volumes of `group` cameras each).
size_t yg_backproject_workspace(int nx, int ny, int nz, int ncam, int group, int slots = 2);
// Camera-group size the backprojector uses for n units and a requested group
// (groups as even as possible, at most `group` units each).
int yg_even_group(int n, int group);
// Depth slabs the per-call projector chooses for nunits mirror units (or
// cameras) of an nx-wide volume with nz planes, two CTAs per SM.
int yg_pair_project_slabs(int nunits, int nx, int nz);
// slabs_used (if non-null): the slab count of the carries written to
// a.carry_out (the projector's depth slabs, twice that with a carry split).
int yg_project(const YgArgs& a, cudaStream_t st, int* slabs_used = nullptr);
// Gradient of sum(g * project(act, mu)) with respect to mu for gantry cameras
// (column layouts: a.act, a.mu; a.sino = g [ncam][nx][cy]; a.out = the
// gradient [nz][nx][cy], zeroed here); no backgrounds.
int yg_dmu(const YgArgs& a, cudaStream_t st);
// Work space of yg_dmu with a.det (one scratch slot of a camera group).
size_t yg_dmu_det_workspace(int nx, int ny, int nz, int ncam, int group);
// Deterministic transposed gather of scratch volumes a.temp[0 .. gcount) of
// units (or cameras) c0 .. c0 + gcount - 1 into a.out (assigned when c0 == 0,
// else added; clamp: negative results stored as zero), rows of the window a
// describes.
void yg_tgather(const YgArgs& a, int c0, int gcount, int clamp, cudaStream_t st);
int yg_backproject(const YgArgs& a, cudaStream_t st);
// Spread of the reference attenuation gradient for cameras [c0, c0 + gcount)
// into the scratch volumes a.temp (one row window: a.row0, a.ny, a.cs).
int yg_grad_spread(const YgArgs& a, int c0, int gcount, cudaStream_t st);
// Bytes of work space of the fused attenuation gradient (`slots` scratch
// volumes of `group` cameras each; no carries).
size_t yg_gradient_workspace(int nx, int ny, int nz, int ncam, int group, int slots = 2);

// ---- batches of volumes (one OSEM subset step of many plans at once) ----
constexpr int kMaxBatch = 64;    // volumes per batched launch
constexpr int kMaxWindows = 8;   // row windows per volume (ny up to ~900)
// Device descriptor of one (volume, subset): the projector arguments for the
// whole volume and the subset's cameras, its row windows, and the OSEM
// buffers of that subset step.
struct BatchStepDesc {
  YgArgs proj;
  int nwin = 0;
  int win[kMaxWindows][4] = {};  // row0, rows, lo, hi (as the launchers' windows)
  const float* counts = nullptr;   // subset counts, column layout
  float* act = nullptr;            // activity (column layout; proj.act), written by the update
  float* num = nullptr;            // backprojected ratio
  const float* sens = nullptr;     // sensitivity of the subset
  long long sino_elems = 0, vol_elems = 0;
};
// Selection of one batched projector launch, passed by value: descriptor per
// volume and the prefix of its work items (window x camera x x-tile).
struct BatchSel {
  int n = 0, total = 0;
  int desc[kMaxBatch] = {};
  int begin[kMaxBatch + 1] = {};
};
// Selection of a batched elementwise launch: descriptor per volume and the
// prefix of its elements.
struct BatchElems {
  int n = 0;
  int desc[kMaxBatch] = {};
  long long begin[kMaxBatch + 1] = {};
};
// Row windows the fused launchers use for ny rows and PSF width psf_k (0: no
// PSF); writes 4 ints per window (row0, rows, lo, hi), returns the count or
// -1 if more than max_windows.
int yg_row_windows(int ny, int psf_k, int* out, int max_windows);
// Persistent projector over all selected volumes: clusters take work items
// from the counter (zeroed by the caller) until none are left.  Volumes of
// one launch share psf_k and whether they have mu; max_nz sizes the PSF table.
int yg_project_batch(const BatchStepDesc* d_desc, const BatchSel& sel, int psf_k, bool att, int max_nz,
                     int* d_counter, cudaStream_t st);
// ratio (desc.proj.out <- counts / max-rule(proj.out)) and update
// (proj.act *= num / max(sens, eps)) over all selected volumes in one launch.
int osem_ratio_batch(const BatchStepDesc* d_desc, const BatchElems& e, float eps, cudaStream_t st);
int osem_update_batch(const BatchStepDesc* d_desc, const BatchElems& e, float eps, cudaStream_t st);

// ---- Fisher information of a grid of points ----
// fisher[i][j] (and [j][i]) = sum over cameras and the overlap of the two
// points' PSF footprints of PSF_i * PSF_j * proj, in the order of
// emission-lib/_et.cpp:626-700; proj [ncam][npy][npx]; coords [ncam][n][3]
// rotated integer coordinates; grid_xyz [n][3]; psf planes [plane][ky][kx];
// prior (optional) 1 for 26-neighbour pairs.
int fisher_pairs(const float* proj, int npx, int npy, const int* coords, const int* grid_xyz, int n, int ncam,
                 const float* psf, int kx, int ky, int nz, float* fisher, float* prior, cudaStream_t st);

// ---- layout conversion and elementwise helpers ----
// planes x [ny][nx] (nifti) <-> planes x [nx][cy] (column), zero pads.
int to_column(const float* src, float* dst, int nx, int ny, int cy, int planes, cudaStream_t st);
// Two volumes of the same shape laid out in one launch (two launches where
// the 16-byte form does not apply).
int to_column2(const float* src_a, float* dst_a, const float* src_b, float* dst_b, int nx, int ny, int cy, int planes,
               cudaStream_t st);
int from_column(const float* src, float* dst, int nx, int ny, int cy, int planes, int truncate, cudaStream_t st);
// Row windows: dst column [planes][nx][cy] <- src nifti rows [row0, row0+rows)
// (planes of ny_src rows); and nifti rows [row0+r_begin, row0+r_end) of dst
// (planes of ny_dst rows) <- column rows [r_begin, r_end) of src.
int to_column_rows(const float* src, float* dst, int nx, int ny_src, int row0, int rows, int cy, int planes,
                   cudaStream_t st);
int from_column_rows(const float* src, float* dst, int nx, int cy, int r_begin, int r_end, int row0, int ny_dst,
                     int planes, int truncate, cudaStream_t st);
// bfloat16 column layout (round to nearest even) from float32 or bfloat16
// nifti rows [row0, row0 + rows); and elementwise float32 -> bfloat16.
int to_column_rows_bf16(const float* src_f32, const void* src_bf16, void* dst, int nx, int ny_src, int row0, int rows,
                        int cy, int planes, cudaStream_t st);
int to_bf16(const float* src, void* dst, size_t n, cudaStream_t st);
int from_bf16(const void* src, float* dst, size_t n, cudaStream_t st);
void launch_truncate(float* buf, size_t n, cudaStream_t st);

// ---- OSEM / MLEM update kernels ----
// ratio[i] = y[i] / (p[i] < eps ? eps : p[i])   (emission-lib/_et_array_interface.cpp:1022-1028)
int osem_ratio(const float* y, float* p_to_ratio, size_t n, float eps, cudaStream_t st);
// x[i] *= num[i] / max(den[i], eps)            (:1036-1044)
int osem_update(float* x, const float* num, const float* den, size_t n, float eps, cudaStream_t st);
// One-step-late MAP-EM (et_osmapem_step, Python/NiftyRec/NiftyRec/NiftyRec.py:224-245):
// ratio y / (max(p, 0) + eps); update x *= max(upd, 0) / (max(sens - beta g, 0) + eps)
// (g may be null: no prior).
int osem_ratio_osl(const float* y, float* p_to_ratio, size_t n, float eps, cudaStream_t st);
int osem_update_osl(float* x, const float* upd, const float* sens, const float* grad, size_t n, float beta, float eps,
                    cudaStream_t st);
// Quadratic MRF prior gradient: 26 x - sum of the in-grid 3x3x3 neighbours
// (n0 fastest).
int mrf_gradient(const float* x, float* g, int n0, int n1, int n2, cudaStream_t st);
// float64 variants of the two, for the float64 reference run.
int osem_ratio64(const double* y, double* p_to_ratio, size_t n, double eps, cudaStream_t st);
int osem_update64(double* x, const double* num, const double* den, size_t n, double eps, cudaStream_t st);
// FP64 totals: out[0] = sum(a), out[1] = sum(b) (b may be null), device doubles.
int sum_fp64(const float* a, const float* b, size_t n, double* out, cudaStream_t st);
// out[i] = value
int fill(float* out, size_t n, float value, cudaStream_t st);

// Records which path the calling thread's last call took (read back by
// nrgb_last_path; defined in et_api.cpp): 1 fused gantry kernels, 2 general.
void set_last_path(int path);

}  // namespace nrgb
