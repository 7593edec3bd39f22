// Fused kernels for cameras that rotate about the gantry axis (nifti y):
// theta_x = theta_z = 0, so the resampling matrix is an exact rotation in the
// (x, z) plane and y maps to itself.  Every detector row y then samples the
// SAME bilinear footprint in the (x, z) plane, so the device layout puts y
// fastest ("column layout" [z][x][cy]) and one warp handles whole columns:
// lane l owns y = 4l..4l+3 (float4), the footprint of an (x, z) column is
// computed once and every gather is a coalesced 16-byte-per-lane column load.
//
// Projector (emission-lib/_et.cpp:218-281): per camera and depth plane z,
//   rotate (bilinear gather of activity and mu), per-plane separable PSF
//   (row pass along x in a register sliding window over a shared tile, column
//   pass along y with warp shuffles), attenuated depth scan T += mu;
//   p += v * exp(-T).  No rotated volume is written anywhere: a thread-block
//   cluster owns (camera, 32-column x-tile), its CTAs own depth slabs and
//   merge (T, p) through distributed shared memory.
// Backprojector, reference mode (emission-lib/_et.cpp:415-499):
//   (1) per-slab transmission carries of the rotated mu, (2) per camera
//   group: spread s*exp(-T) + PSF in the rotated frame into an L2-sized
//   scratch, (3) inverse-rotation gather of the group into the accumulator.
#include "et_kernels.h"
#include "et_profile.h"

#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <type_traits>
#include <vector>

namespace nrgb {

namespace {

namespace cg = cooperative_groups;

constexpr int kW = 8;             // warps per CTA of the tile engine
constexpr int kTXW = 4;           // output columns per warp
constexpr int kTXC = kW * kTXW;   // output columns per CTA
constexpr int kSlabsP = 4;        // depth slabs (= cluster size) of the batched projector
constexpr int kSlabsB = 16;       // backprojector depth slabs
constexpr int kCarrySlots = kSlabsB + 1;  // carries per camera: slab prefixes, column total
constexpr int kCarryCols = 64 / kSlabsB;  // columns per CTA of the carry pass (32 KB of slab sums)
constexpr int kGatherWarps = 4;   // warps per CTA of the inverse-rotation gather
constexpr int kGatherCols = 2;    // accumulator columns per warp in the gather
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }

// Bilinear footprint of one sampled column.  Corner (a, c) sits at
// off + a*dx + c*dz; corners outside the grid get weight 0 and a clamped
// (valid) address, so loads never leave the volume.
struct __align__(16) Tap {
  int off, dx, dz, any;
  float w00, w10, w01, w11;
};

// Footprint of rotated column (xp, zp) under rows (m00, m02, m03) -> x and
// (m20, m22, m23) -> z.  Position arithmetic follows
// reg-lib/_reg_affineTransformation.cpp:116-132 (the y terms are exact zeros
// for a y-gantry), floor/relative/basis follow reg-lib/_reg_resampling.cpp:347-364.
__device__ __forceinline__ Tap make_tap(int xp, int zp, float m00, float m02, float m03, float m20, float m22,
                                        float m23, int nx, int nz, int cy, bool col_valid) {
  const float fx = static_cast<float>(xp), fz = static_cast<float>(zp);
  const float px = fa(fa(fm(m00, fx), fm(m02, fz)), m03);
  const float pz = fa(fa(fm(m20, fx), fm(m22, fz)), m23);
  const int xs = static_cast<int>(floorf(px));
  const int zs = static_cast<int>(floorf(pz));
  float rx = __fsub_rn(px, static_cast<float>(xs));
  float rz = __fsub_rn(pz, static_cast<float>(zs));
  if (rx < 0.0f) rx = 0.0f;
  if (rz < 0.0f) rz = 0.0f;
  const float wx0 = __fsub_rn(1.0f, rx), wx1 = rx, wz0 = __fsub_rn(1.0f, rz), wz1 = rz;
  const bool x0 = col_valid && xs >= 0 && xs < nx;
  const bool x1 = col_valid && xs + 1 >= 0 && xs + 1 < nx;
  const bool z0 = col_valid && zs >= 0 && zs < nz;
  const bool z1 = col_valid && zs + 1 >= 0 && zs + 1 < nz;
  Tap t;
  const int xb = x0 ? xs : (x1 ? xs + 1 : 0);
  const int zb = z0 ? zs : (z1 ? zs + 1 : 0);
  t.off = (zb * nx + xb) * cy;
  t.dx = (x0 && x1) ? cy : 0;
  t.dz = (z0 && z1) ? nx * cy : 0;
  t.w00 = (x0 && z0) ? wx0 * wz0 : 0.0f;
  t.w10 = (x1 && z0) ? wx1 * wz0 : 0.0f;
  t.w01 = (x0 && z1) ? wx0 * wz1 : 0.0f;
  t.w11 = (x1 && z1) ? wx1 * wz1 : 0.0f;
  t.any = (x0 || x1) && (z0 || z1);
  return t;
}

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// Four consecutive rows of a bfloat16 column (8 bytes, 8-byte aligned since
// cy and the lane's first row are multiples of 4), widened to float32: a
// bfloat16 is the high half of the float32 with the same value.
__device__ __forceinline__ float4 ldg4(const __nv_bfloat16* p) {
  const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
  return make_float4(__uint_as_float(u.x << 16), __uint_as_float(u.x & 0xffff0000u), __uint_as_float(u.y << 16),
                     __uint_as_float(u.y & 0xffff0000u));
}

template <class V>
__device__ __forceinline__ float4 sample4(const V* __restrict__ base, const Tap& t, int yb, bool yok) {
  float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!t.any || !yok) return r;
  const V* p = base + t.off + yb;
  const float4 a = ldg4(p), b = ldg4(p + t.dx), c = ldg4(p + t.dz), d = ldg4(p + t.dx + t.dz);
  r.x = fmaf(d.x, t.w11, fmaf(c.x, t.w01, fmaf(b.x, t.w10, a.x * t.w00)));
  r.y = fmaf(d.y, t.w11, fmaf(c.y, t.w01, fmaf(b.y, t.w10, a.y * t.w00)));
  r.z = fmaf(d.z, t.w11, fmaf(c.z, t.w01, fmaf(b.z, t.w10, a.z * t.w00)));
  r.w = fmaf(d.w, t.w11, fmaf(c.w, t.w01, fmaf(b.w, t.w10, a.w * t.w00)));
  return r;
}

__device__ __forceinline__ float comp(const float4& v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }

__device__ __forceinline__ void axpy4(float4& acc, float k, const float4& v) {
  acc.x = fmaf(k, v.x, acc.x);
  acc.y = fmaf(k, v.y, acc.y);
  acc.z = fmaf(k, v.z, acc.z);
  acc.w = fmaf(k, v.w, acc.w);
}

// Rows y >= ny are zero pads of the column layout; the column pass must not
// leak into them (the reference's column pass only produces rows < ny).
__device__ __forceinline__ float4 mask_rows(float4 v, int yb, int ny) {
  if (yb + 0 >= ny) v.x = 0.0f;
  if (yb + 1 >= ny) v.y = 0.0f;
  if (yb + 2 >= ny) v.z = 0.0f;
  if (yb + 3 >= ny) v.w = 0.0f;
  return v;
}

// Column (y) pass of the per-plane convolution for the 4 rows a lane owns:
// out[y] = sum_k in[y+k] * kc[R-k], zero outside [0, ny) (rows >= ny are zero
// pads, rows < 0 come from lanes below 0 and are masked).  Neighbour rows come
// from lanes l-1, l-2 and l+1, l+2 by shuffles.
template <int R, class KC>
__device__ __forceinline__ float4 yconv4(const float4& u, KC kc, int lane) {
  float w[2 * R + 4];
  w[R + 0] = u.x;
  w[R + 1] = u.y;
  w[R + 2] = u.z;
  w[R + 3] = u.w;
#pragma unroll
  for (int t = 1; t <= R; ++t) {
    const int dl = (t + 3) / 4;
    const float s = __shfl_up_sync(kFull, comp(u, 4 * dl - t), dl);
    w[R - t] = (lane >= dl) ? s : 0.0f;
  }
#pragma unroll
  for (int t = 1; t <= R; ++t) {
    const int dl = (t + 3) / 4;
    const float s = __shfl_down_sync(kFull, comp(u, t + 3 - 4 * dl), dl);
    w[R + 3 + t] = (lane + dl < 32) ? s : 0.0f;
  }
  float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int k = -R; k <= R; ++k) {
    const float kk = kc[R - k];
    o.x = fmaf(w[R + 0 + k], kk, o.x);
    o.y = fmaf(w[R + 1 + k], kk, o.y);
    o.z = fmaf(w[R + 2 + k], kk, o.z);
    o.w = fmaf(w[R + 3 + k], kk, o.w);
  }
  return o;
}

__device__ __forceinline__ float4 exp_neg4(const float4& t) {
  return make_float4(__expf(-t.x), __expf(-t.y), __expf(-t.z), __expf(-t.w));
}

__device__ __forceinline__ void add4(float4& a, const float4& b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  a.w += b.w;
}

__device__ __forceinline__ void fma4(float4& acc, const float4& a, const float4& b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.y = fmaf(a.y, b.y, acc.y);
  acc.z = fmaf(a.z, b.z, acc.z);
  acc.w = fmaf(a.w, b.w, acc.w);
}

__device__ __forceinline__ float4 mul4(const float4& a, const float4& b) {
  return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w);
}

// Compensated summation (Kahan, CACM 8(1):40, 1965): s + (-c) tracks the
// exact sum of the added terms far better than s alone; c holds the rounding
// excess of the previous additions.  Each operation rounds separately.
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

__device__ __forceinline__ void kahan_add4(float4& s, float4& c, const float4& v) {
  kahan_add(s.x, c.x, v.x);
  kahan_add(s.y, c.y, v.y);
  kahan_add(s.z, c.z, v.z);
  kahan_add(s.w, c.w, v.w);
}

// Compensated value of a Kahan pair.
__device__ __forceinline__ float4 kahan_value4(const float4& s, const float4& c) {
  return make_float4(__fsub_rn(s.x, c.x), __fsub_rn(s.y, c.y), __fsub_rn(s.z, c.z), __fsub_rn(s.w, c.w));
}

// Depth sum s += v: plain float32 (the reference's order) or compensated.
template <bool KAHAN>
__device__ __forceinline__ void depth_add4(float4& s, float4& c, const float4& v) {
  if (KAHAN)
    kahan_add4(s, c, v);
  else
    add4(s, v);
}

template <bool KAHAN>
__device__ __forceinline__ float4 depth_value4(const float4& s, const float4& c) {
  return KAHAN ? kahan_value4(s, c) : s;
}

// Storage type of the sampled volumes; bfloat16 storage sums with Kahan.
template <class V>
struct StorageTraits {
  static constexpr bool kKahan = false;
};
template <>
struct StorageTraits<__nv_bfloat16> {
  static constexpr bool kKahan = true;
};

struct CamRows {
  float m00, m02, m03, m20, m22, m23;
};

__device__ __forceinline__ CamRows cam_rows(const float* m) {
  CamRows c;
  c.m00 = __ldg(m + 0);
  c.m02 = __ldg(m + 2);
  c.m03 = __ldg(m + 3);
  c.m20 = __ldg(m + 8);
  c.m22 = __ldg(m + 10);
  c.m23 = __ldg(m + 11);
  return c;
}

// Separated PSF of every plane ([nz][2K]: row kernel, then column kernel)
// passed as a kernel parameter: the coefficients are read from the constant
// bank with uniform addresses (no shared-memory copy, no load instruction per
// use in the row and column passes).  Tables larger than this use the shared
// memory copy.
constexpr int kPsfTableFloats = 7680;
struct PsfTable {
  float c[kPsfTableFloats];
};

// A row kernel read backwards (k -> p[2R - k]): a mirror camera's row pass.
template <int R>
struct Reversed {
  const float* p;
  __device__ __forceinline__ float operator[](int k) const { return p[2 * R - k]; }
};

// ------------------------------------------------------------ tile engine
// A CTA of kW warps owns kTXC = kW * kTXW consecutive output columns of one
// camera and walks one depth slab.  At every depth step the NS = kTXC + 2R
// sampled columns (outputs plus the PSF row halo) are produced once per CTA
// -- column c by warp c % kW -- into a double-buffered shared tile; after one
// barrier each warp runs the row pass (register sliding window over its
// kTXW + 2R tile columns), the column pass and its consumer for its kTXW
// outputs.  Writes of step z+1 go to the other buffer, so one barrier per
// step suffices.
template <int R>
struct TileShape {
  static constexpr int NS = kTXC + 2 * R;            // sampled columns per CTA
  static constexpr int kOwn = (NS + kW - 1) / kW;    // sampled columns per warp (max)
  static constexpr int kTapSlots = kW * kOwn;         // footprint slots per stage (see tap_slot)
  static constexpr size_t kSbBytes = sizeof(float4) * 2 * NS * 32;
  static constexpr size_t kTapBytes = sizeof(Tap) * 2 * kTapSlots;
  // Projector with a mirror camera: the tile region also holds the three
  // slab-merge buffers (T, P and the mirror camera's P per output column).
  static constexpr size_t kSbBytesPair = sizeof(float4) * 32 * (2 * NS > 3 * kTXC ? 2 * NS : 3 * kTXC);
  __host__ __device__ static constexpr size_t sb_bytes(bool pair) { return pair ? kSbBytesPair : kSbBytes; }
};

// Footprint slot of sampled column c in the tap buffer: the columns one warp
// computes (c = warp + kW * k) sit next to each other, so the footprint
// stores of a warp do not collide in shared-memory banks.
template <int R>
__device__ __forceinline__ int tap_slot(int c) {
  return (c % kW) * TileShape<R>::kOwn + c / kW;
}

// Tile, footprints and the separated PSF of nz planes (twice with a mirror
// camera: its kernels are the mirrored planes, row kernels reversed).
template <int R>
__host__ __device__ constexpr size_t tile_smem_bytes(int nz, bool pair = false) {
  return TileShape<R>::sb_bytes(pair) + TileShape<R>::kTapBytes +
         sizeof(float) * static_cast<size_t>(nz) * 2 * (2 * R + 1) * (pair ? 2 : 1);
}

// Row pass from the shared tile: outputs i = 0..kTXW-1 of this warp use tile
// columns base + i .. base + i + 2R (base = warp * kTXW).
template <int R, class EmitFn, class KR, class KC>
__device__ __forceinline__ void rowpass_from_tile(const float4* __restrict__ sbuf, int base, EmitFn emit, KR kr, KC kc,
                                                  int lane, int ny) {
  constexpr int K = 2 * R + 1;
  constexpr int NJ = kTXW + 2 * R;
  float4 u[K];
#pragma unroll
  for (int q = 0; q < K; ++q) u[q] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const float4 r = sbuf[(base + j) * 32 + lane];
#pragma unroll
    for (int d = 0; d < K; ++d) {
      const int i = j - d;
      if (i >= 0 && i < kTXW) axpy4(u[i % K], kr[2 * R - d], r);
    }
    const int i = j - 2 * R;
    if (i >= 0 && i < kTXW) {
      emit(i, mask_rows(yconv4<R>(u[i % K], kc, lane), 4 * lane, ny));
      u[i % K] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

// Row passes of two cameras over the same tile (a camera and its mirror
// camera): each tile column is read once and feeds both sliding windows;
// output i of camera b is emitted before output i of camera a.
template <int R, class EmitA, class EmitB, class KRA, class KCA, class KRB, class KCB>
__device__ __forceinline__ void rowpass2_from_tile(const float4* __restrict__ sbuf, int base, EmitA emit_a, KRA kra,
                                                   KCA kca, EmitB emit_b, KRB krb, KCB kcb, int lane, int ny) {
  constexpr int NJ = kTXW + 2 * R;
  float4 ua[kTXW], ub[kTXW];
#pragma unroll
  for (int q = 0; q < kTXW; ++q) {
    ua[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    ub[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const float4 r = sbuf[(base + j) * 32 + lane];
#pragma unroll
    for (int d = 0; d <= 2 * R; ++d) {
      const int i = j - d;
      if (i >= 0 && i < kTXW) {
        axpy4(ua[i], kra[2 * R - d], r);
        axpy4(ub[i], krb[2 * R - d], r);
      }
    }
    const int i = j - 2 * R;
    if (i >= 0 && i < kTXW) {
      emit_b(i, mask_rows(yconv4<R>(ub[i], kcb, lane), 4 * lane, ny));
      emit_a(i, mask_rows(yconv4<R>(ua[i], kca, lane), 4 * lane, ny));
    }
  }
}

// ---------------------------------------------------------------- projector
// Row windows: a column holds cy >= ny rows, the kernels see one window of at
// most 128 rows at a time: rows [row0, row0 + ny) of the columns (row0 a
// multiple of 4, so lane loads stay aligned), valid output rows [out_lo,
// out_hi) relative to row0.  Rows past a window's end read as zero (lanes past
// round_up(ny, 4) sample nothing; the rows inside the last lane are the zero
// pads of the column layout at the volume's end, the only place a window
// ends off a multiple of 4).
__device__ __forceinline__ bool lane_rows_ok(const YgArgs& a, int yb) { return yb < ((a.ny + 3) & ~3); }
__device__ __forceinline__ bool lane_writes(const YgArgs& a, int yb) { return yb >= a.out_lo && yb < a.out_hi; }

// One projector work item: camera `cam`, output columns x0 .. x0 + kTXC - 1;
// the CTAs of the cluster walk the depth slabs and merge (T, p) through
// distributed shared memory: p = p0 + exp(-T0) p1 + exp(-T0-T1) p2 + ...
// V: storage type of activity and mu (float or bfloat16; bfloat16 sums with
// Kahan).  Ends with a cluster barrier, after which the shared memory may be
// reused.
//
// Mirror camera (PAIR, mate >= 0): a camera at the opposite angle (theta + pi)
// about the grid centre samples the same points: its rotated volume is this
// camera's mirrored in x and z (column x of depth z is its column nx-1-x of
// depth nz-1-z).  The CTA then serves both from one set of bilinear samples:
// the mate's row pass uses the PSF plane nz-1-z with the row kernel reversed,
// its depth sum runs towards this camera, and its slab partial
//   q = sum_z v'_z exp(-(S - E_z)) = exp(-S) sum_z v'_z exp(E_z)
// (S the slab's mu sum, E_z the sum before plane z) is accumulated in the
// forward walk as sum v' exp(E).  A slab whose mu sum exceeds kMateMaxT (or
// whose sum overflows) is redone for the mate alone by a descending walk with
// the direct weights.  The mate's slabs merge in the opposite order.
constexpr float kMateMaxT = 40.0f;

template <int R, bool PSF, bool ATT, class V, bool PAIR = false, bool PTAB = false>
__device__ __forceinline__ void project_item(const YgArgs& a, int cam, int mate, int x0, unsigned char* smem,
                                             const float* ptab = nullptr) {
  using TS = TileShape<R>;
  constexpr bool KAHAN = StorageTraits<V>::kKahan;
  static_assert(!(PAIR && KAHAN), "mirror cameras are served by the float32 projector");
  const V* __restrict__ act = reinterpret_cast<const V*>(a.act) + a.row0;
  const V* __restrict__ mu = reinterpret_cast<const V*>(a.mu) + a.row0;
  constexpr int NS = TS::NS;
  constexpr int K = 2 * R + 1;
  constexpr size_t kSb = TS::sb_bytes(PAIR);
  float4* sb = reinterpret_cast<float4*>(smem);                    // [2][NS][32]
  Tap* taps = reinterpret_cast<Tap*>(smem + kSb);                   // [2][kTapSlots]
  float* s_psf = reinterpret_cast<float*>(smem + kSb + TS::kTapBytes);  // [nz][2K]
  float* s_psf_m = s_psf + static_cast<size_t>(a.nz) * 2 * K;       // [nz][2K] (mate)

  cg::cluster_group cluster = cg::this_cluster();
  const int slab = static_cast<int>(cluster.block_rank());
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const bool paired = PAIR && mate >= 0;  // uniform over the cluster

  const int nslabs = static_cast<int>(cluster.num_blocks());  // depth slabs = cluster size (2, 4 or 8)
  const int zper = (a.nz + nslabs - 1) / nslabs;
  const int zbeg = slab * zper, zend = min(a.nz, zbeg + zper);
  if (PSF && !PTAB) {  // this slab's planes only
    for (int i = zbeg * 2 * K + threadIdx.x; i < zend * 2 * K; i += blockDim.x) s_psf[i] = __ldg(a.psf + i);
    if (paired) {
      for (int i = zbeg * 2 * K + threadIdx.x; i < zend * 2 * K; i += blockDim.x) {
        const int z = i / (2 * K), j = i % (2 * K);
        s_psf_m[i] = __ldg(a.psf + (a.nz - 1 - z) * 2 * K + (j < K ? K - 1 - j : j));
      }
    }
  }
  // row and column kernels of plane z for this camera and for the mate
  // (plane nz-1-z, row kernel reversed)
  auto mate_pass = [&](const float4* sbuf, int z, auto emit_m) {
    if constexpr (PTAB) {
      const float* m = ptab + (a.nz - 1 - z) * 2 * K;
      rowpass_from_tile<R>(sbuf, warp * kTXW, emit_m, Reversed<R>{m}, m + K, lane, a.ny);
    } else {
      const float* m = s_psf_m + z * 2 * K;
      rowpass_from_tile<R>(sbuf, warp * kTXW, emit_m, m, m + K, lane, a.ny);
    }
  };
  auto both_pass = [&](const float4* sbuf, int z, auto emit, auto emit_m) {
    const float* kr = (PTAB ? ptab : s_psf) + z * 2 * K;
    if constexpr (PTAB) {
      const float* m = ptab + (a.nz - 1 - z) * 2 * K;
      rowpass2_from_tile<R>(sbuf, warp * kTXW, emit, kr, kr + K, emit_m, Reversed<R>{m}, m + K, lane, a.ny);
    } else {
      const float* m = s_psf_m + z * 2 * K;
      rowpass2_from_tile<R>(sbuf, warp * kTXW, emit, kr, kr + K, emit_m, m, m + K, lane, a.ny);
    }
  };
  const CamRows cr = cam_rows(a.geom[cam].fwd);

  float4 T[kTXW], P[kTXW], cT[kTXW], cP[kTXW];  // c*: Kahan compensations (KAHAN only)
  float4 Q[PAIR ? kTXW : 1];                    // mate's slab partial
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    T[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    cT[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    cP[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (PAIR) Q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  __syncthreads();

  // One depth step at plane z into tile buffer b.  MODE 0: this camera (and
  // the mate's forward form); MODE 1: the mate alone, direct weights (walked
  // from the slab's far end).
  auto step = [&](int z, int b, auto mode) {
    constexpr int MODE = decltype(mode)::value;
    float4* sbuf = sb + b * NS * 32;
    Tap* tb = taps + b * TS::kTapSlots;
    // footprints of the columns this warp samples (c = warp + kW * k)
    if (lane < TS::kOwn) {
      const int c = warp + kW * lane;
      if (c < NS) {
        const int xp = x0 - R + c;
        tb[tap_slot<R>(c)] = make_tap(xp, z, cr.m00, cr.m02, cr.m03, cr.m20, cr.m22, cr.m23, a.nx, a.nz, a.cy,
                                      xp >= 0 && xp < a.nx);
      }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < TS::kOwn; ++k) {
      const int c = warp + kW * k;
      if (c < NS) sbuf[c * 32 + lane] = sample4(act, tb[tap_slot<R>(c)], yb, yok);
    }
    __syncthreads();
    auto emit_m = [&](int i, const float4& v) {
      if (!ATT) {
        add4(Q[i], v);
      } else if (MODE == 0) {  // weight exp(E_z): T holds the sum before plane z
        fma4(Q[i], v, exp_neg4(make_float4(-T[i].x, -T[i].y, -T[i].z, -T[i].w)));
      } else {  // T runs from the slab's far end, inclusive
        add4(T[i], sample4(mu, tb[tap_slot<R>(warp * kTXW + i + R)], yb, yok));
        fma4(Q[i], v, exp_neg4(T[i]));
      }
    };
    if (MODE == 1) {
      if (PSF) {
        mate_pass(sbuf, z, emit_m);
      } else {
#pragma unroll
        for (int i = 0; i < kTXW; ++i) emit_m(i, sbuf[(warp * kTXW + i) * 32 + lane]);
      }
      return;
    }
    auto emit = [&](int i, const float4& v) {
      if (ATT) {
        const float4 m = sample4(mu, tb[tap_slot<R>(warp * kTXW + i + R)], yb, yok);
        if (KAHAN) {
          kahan_add4(T[i], cT[i], m);
          kahan_add4(P[i], cP[i], mul4(v, exp_neg4(kahan_value4(T[i], cT[i]))));
        } else {
          add4(T[i], m);
          fma4(P[i], v, exp_neg4(T[i]));
        }
      } else {
        depth_add4<KAHAN>(P[i], cP[i], v);
      }
    };
    if (PSF) {
      if (PAIR && paired) {
        both_pass(sbuf, z, emit, emit_m);
      } else {
        const float* kr = (PTAB ? ptab : s_psf) + z * 2 * K;
        rowpass_from_tile<R>(sbuf, warp * kTXW, emit, kr, kr + K, lane, a.ny);
      }
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) {
        const float4 v = sbuf[(warp * kTXW + i) * 32 + lane];
        if (PAIR && paired) emit_m(i, v);
        emit(i, v);
      }
    }
  };

  for (int z = zbeg; z < zend; ++z) step(z, z & 1, std::integral_constant<int, 0>());

  if (PAIR && paired && ATT) {
    bool redo = false;
#pragma unroll
    for (int i = 0; i < kTXW; ++i) {
      redo |= !(T[i].x <= kMateMaxT && T[i].y <= kMateMaxT && T[i].z <= kMateMaxT && T[i].w <= kMateMaxT);
      redo |= !(isfinite(Q[i].x) && isfinite(Q[i].y) && isfinite(Q[i].z) && isfinite(Q[i].w));
    }
    if (__syncthreads_or(redo)) {  // uniform over the CTA
#pragma unroll
      for (int i = 0; i < kTXW; ++i) {
        Q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        T[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // ends at the slab sum again
      }
      for (int k = 0; k < zend - zbeg; ++k) step(zend - 1 - k, k & 1, std::integral_constant<int, 1>());
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) Q[i] = mul4(Q[i], exp_neg4(T[i]));
    }
  }

  // cluster merge of the depth slabs (the shared tile is free after this barrier)
  __syncthreads();
  float4* sT = sb;                // [kTXC][32]
  float4* sP = sb + kTXC * 32;    // [kTXC][32]
  float4* sQ = sb + 2 * kTXC * 32;  // [kTXC][32] (PAIR)
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    sT[(warp * kTXW + i) * 32 + lane] = depth_value4<KAHAN>(T[i], cT[i]);
    sP[(warp * kTXW + i) * 32 + lane] = depth_value4<KAHAN>(P[i], cP[i]);
    if (PAIR && paired) sQ[(warp * kTXW + i) * 32 + lane] = Q[i];
  }
  cluster.sync();
  const int per_rank = kTXC / nslabs;  // outputs merged by each CTA of the cluster
  auto store = [&](int c, int x, float4 Pt) {
    if (a.truncate) {
      Pt.x = fmaxf(Pt.x, 0.f);
      Pt.y = fmaxf(Pt.y, 0.f);
      Pt.z = fmaxf(Pt.z, 0.f);
      Pt.w = fmaxf(Pt.w, 0.f);
    }
    *reinterpret_cast<float4*>(a.out + (static_cast<size_t>(c) * a.nx + x) * a.cy + a.row0 + yb) = Pt;
  };
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    const int o = warp * kTXW + i;
    const int x = x0 + o;
    if (o / per_rank != slab || x >= a.nx || !yok || !lane_writes(a, yb)) continue;
    float4 Pt = make_float4(0.f, 0.f, 0.f, 0.f), Tt = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int s = 0; s < nslabs; ++s) {
      const float4* rT = cluster.map_shared_rank(sT, s);
      const float4* rP = cluster.map_shared_rank(sP, s);
      const float4 ps = rP[o * 32 + lane];
      if (ATT) {
        fma4(Pt, exp_neg4(Tt), ps);
        add4(Tt, rT[o * 32 + lane]);
      } else {
        add4(Pt, ps);
      }
    }
    store(cam, x, Pt);
    if (PAIR && paired) {  // the mate's slabs from the far end: its column nx-1-x
      Pt = make_float4(0.f, 0.f, 0.f, 0.f);
      Tt = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int s = nslabs - 1; s >= 0; --s) {
        const float4 qs = cluster.map_shared_rank(sQ, s)[o * 32 + lane];
        if (ATT) {
          fma4(Pt, exp_neg4(Tt), qs);
          add4(Tt, cluster.map_shared_rank(sT, s)[o * 32 + lane]);
        } else {
          add4(Pt, qs);
        }
      }
      store(mate, a.nx - 1 - x, Pt);
    }
  }
  cluster.sync();  // keep this CTA's shared memory alive until the others have read it
}

// One work item per cluster of a.pslabs CTAs (the cluster size is set at
// launch): blockIdx.x / a.pslabs = (unit, x-tile); a unit is a camera and,
// with a.units, its mirror camera.  CTAS: CTAs per SM the kernel is compiled
// for -- 3 (80 registers, more warps to hide the gathers' latency) where
// three tiles fit in shared memory and the storage is float32, else 2 (128
// registers; bfloat16 needs them for its Kahan compensations).
template <int R, bool PSF, bool ATT, class V, int CTAS, bool PAIR>
__global__ void __launch_bounds__(32 * kW, CTAS) k_project_yg(const YgArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int item = blockIdx.x / a.pslabs;
  const int u = item / ntile;
  const int2 uc = PAIR ? a.units[u] : make_int2(u, -1);
  project_item<R, PSF, ATT, V, PAIR>(a, uc.x, uc.y, (item % ntile) * kTXC, smem);
}

// The same with the separated PSF in the kernel parameters (PsfTable).
template <int R, bool ATT, class V, int CTAS, bool PAIR>
__global__ void __launch_bounds__(32 * kW, CTAS) k_project_ptab_yg(const YgArgs a, const __grid_constant__ PsfTable t) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int item = blockIdx.x / a.pslabs;
  const int u = item / ntile;
  const int2 uc = PAIR ? a.units[u] : make_int2(u, -1);
  project_item<R, true, ATT, V, PAIR, true>(a, uc.x, uc.y, (item % ntile) * kTXC, smem, t.c);
}

// Persistent projector over a batch of volumes: each cluster takes work items
// (volume, row window, camera, x-tile) from a global counter until none are
// left, so volumes of any size share the GPU in one launch.  The item number
// is drawn by the cluster's first thread and read by the other CTAs from its
// shared memory (double-buffered: the slot of item i is rewritten at item i+2,
// after the barriers of item i+1).
template <int R, bool PSF, bool ATT>
__global__ void __cluster_dims__(kSlabsP, 1, 1) __launch_bounds__(32 * kW, 2)
    k_project_batch_yg(const BatchStepDesc* __restrict__ descs, const BatchSel sel, int* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_item[2];
  cg::cluster_group cluster = cg::this_cluster();
  const bool leader = cluster.block_rank() == 0 && threadIdx.x == 0;
  for (int it = 0;; ++it) {
    int* slot = &s_item[it & 1];
    if (leader) *slot = atomicAdd(counter, 1);
    cluster.sync();
    const int item = *cluster.map_shared_rank(slot, 0);
    if (item >= sel.total) {
      cluster.sync();  // rank 0's shared memory stays alive until every CTA has read it
      return;
    }
    int v = 0;
    while (v + 1 < sel.n && item >= sel.begin[v + 1]) ++v;
    const BatchStepDesc& d = descs[sel.desc[v]];
    const int ntile = (d.proj.nx + kTXC - 1) / kTXC;
    const int per_win = d.proj.ncam * ntile;
    const int local = item - sel.begin[v];
    const int w = local / per_win, r = local % per_win;
    YgArgs a = d.proj;
    a.row0 = d.win[w][0];
    a.ny = d.win[w][1];
    a.out_lo = d.win[w][2];
    a.out_hi = d.win[w][3];
    project_item<R, PSF, ATT, float>(a, r / ntile, -1, (r % ntile) * kTXC, smem);
  }
}

// ------------------------------------------------ backprojector: slab carry
// carry[c][s][x][y] (s < kSlabsB) = sum of the rotated mu over the depth
// slabs before s (exclusive prefix): the transmission a depth slab starts
// from; carry[c][kSlabsB][x][y] = the whole column's sum.  One block row per
// camera c, or with a.units per unit (its first camera c; a mirror camera's
// transmissions are c's read from the other end).
template <class V>
__global__ void __launch_bounds__(32 * kSlabsB) k_mu_carry_yg(const YgArgs a) {
  constexpr int C = kCarryCols;
  constexpr bool KAHAN = StorageTraits<V>::kKahan;
  const V* __restrict__ mu = reinterpret_cast<const V*>(a.mu) + a.row0;
  __shared__ Tap s_tap[kSlabsB][C];
  __shared__ float4 s_sum[kSlabsB][C][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunk = (a.nx + C - 1) / C;
  const int unit = blockIdx.x / nchunk;
  const int cam = a.units ? a.units[unit].x : unit;
  const int x0 = (blockIdx.x % nchunk) * C;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const CamRows cr = cam_rows(a.geom[cam].fwd);
  const int zper = (a.nz + kSlabsB - 1) / kSlabsB;
  const int zbeg = warp * zper, zend = min(a.nz, zbeg + zper);
  float4 S[C], cS[C];
#pragma unroll
  for (int i = 0; i < C; ++i) {
    S[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    cS[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int z = zbeg; z < zend; ++z) {
    if (lane < C) {
      const int xp = x0 + lane;
      s_tap[warp][lane] = make_tap(xp, z, cr.m00, cr.m02, cr.m03, cr.m20, cr.m22, cr.m23, a.nx, a.nz, a.cy, xp < a.nx);
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < C; ++i) depth_add4<KAHAN>(S[i], cS[i], sample4(mu, s_tap[warp][i], yb, yok));
    __syncwarp();
  }
#pragma unroll
  for (int i = 0; i < C; ++i) s_sum[warp][i][lane] = depth_value4<KAHAN>(S[i], cS[i]);
  __syncthreads();
  if (!yok || !lane_writes(a, yb)) return;
#pragma unroll
  for (int i = 0; i < C; ++i) {
    const int x = x0 + i;
    if (x >= a.nx) continue;
    float4 pre = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int s = 0; s < warp; ++s) add4(pre, s_sum[s][i][lane]);
    float* dst = a.slab_T + ((static_cast<size_t>(cam) * kCarrySlots + warp) * a.nx + x) * a.cy + a.row0 + yb;
    *reinterpret_cast<float4*>(dst) = pre;
    if (warp == kSlabsB - 1) {  // the column total, one slot further
      add4(pre, s_sum[warp][i][lane]);
      *reinterpret_cast<float4*>(dst + static_cast<size_t>(a.nx) * a.cy) = pre;
    }
  }
}

// Vector reduction of 4 floats into global memory (sm_90+).
__device__ __forceinline__ void red4(float* p, const float4& v) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
               : "memory");
}

__device__ __forceinline__ float4 scale4(const float4& v, float w) {
  return make_float4(v.x * w, v.y * w, v.z * w, v.w * w);
}

// Transposed bilinear interpolation: add w * v to each corner of footprint t
// (corners outside the grid have weight 0 and are skipped).
__device__ __forceinline__ void scatter4(float* __restrict__ base, const Tap& t, int yb, const float4& v) {
  if (!t.any) return;
  float* p = base + t.off + yb;
  if (t.w00 != 0.0f) red4(p, scale4(v, t.w00));
  if (t.w10 != 0.0f) red4(p + t.dx, scale4(v, t.w10));
  if (t.w01 != 0.0f) red4(p + t.dz, scale4(v, t.w01));
  if (t.w11 != 0.0f) red4(p + t.dx + t.dz, scale4(v, t.w11));
}

// ---------------------------------------- backprojector: spread + PSF
// temp[g][z][x][y] = PSF_z( s(x', y) * exp(-T_z(x', y)) ) for camera c0+g,
// T inclusive (emission-lib/_et_line_backproject_attenuated.cpp:24-34), PSF
// as in the projector.  CTA = (camera, x-tile, depth slab); every sampled
// column starts its transmission from the slab carry.
// ADJ: the exact transpose of the projector instead (not in the reference):
// the PSF taps are flipped (correlation) and each output column is scattered
// with the projector's own bilinear weights into the accumulator a.out
// (vector reductions; all cameras in one launch, no scratch).
// CTAS: CTAs per SM the kernel is compiled for (3 where three tiles fit in
// shared memory, for the float32 reference spread; else 2).
template <int R, bool PSF, bool ATT, bool ADJ, class V, int CTAS = 2>
__global__ void __launch_bounds__(32 * kW, CTAS) k_spread_yg(const YgArgs a, int c0) {
  using TS = TileShape<R>;
  constexpr bool KAHAN = StorageTraits<V>::kKahan;
  const V* __restrict__ mu = reinterpret_cast<const V*>(a.mu) + a.row0;
  constexpr int NS = TS::NS;
  constexpr int K = 2 * R + 1;
  extern __shared__ __align__(16) unsigned char smem[];
  float4* sb = reinterpret_cast<float4*>(smem);
  Tap* taps = reinterpret_cast<Tap*>(smem + TS::kSbBytes);
  float* s_psf = reinterpret_cast<float*>(smem + TS::kSbBytes + TS::kTapBytes);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int slab = blockIdx.x % kSlabsB;
  const int item = blockIdx.x / kSlabsB;
  const int g = item / ntile;
  const int cam = c0 + g;
  const int x0 = (item % ntile) * kTXC;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const int zper = (a.nz + kSlabsB - 1) / kSlabsB;
  const int zbeg = slab * zper, zend = min(a.nz, zbeg + zper);
  if (zbeg >= zend) return;  // uniform over the CTA
  if (PSF) {  // this slab's planes only
    for (int i = zbeg * 2 * K + threadIdx.x; i < zend * 2 * K; i += blockDim.x) {
      const int j = i % (2 * K), base = i - j;
      // transpose of a convolution = correlation: reverse each kernel
      const int src = !ADJ ? i : (j < K ? base + (K - 1 - j) : base + K + (2 * K - 1 - j));
      s_psf[i] = __ldg(a.psf + src);
    }
  }
  const CamRows cr = cam_rows(a.geom[cam].fwd);
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * a.cs;  // one scratch volume
  float* __restrict__ tmp = ADJ ? a.out + a.row0 : a.temp + vol * g;
  const float* __restrict__ srow = a.sino + static_cast<size_t>(cam) * a.nx * a.cy + a.row0;

  float4 Tc[TS::kOwn], cTc[TS::kOwn];  // transmission per sampled column (+ Kahan compensation)
#pragma unroll
  for (int k = 0; k < TS::kOwn; ++k) {
    Tc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    cTc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int xp = x0 - R + warp + kW * k;
    if (ATT && warp + kW * k < NS && xp >= 0 && xp < a.nx && yok)
      Tc[k] = ldg4(a.slab_T + ((static_cast<size_t>(cam) * kCarrySlots + slab) * a.nx + xp) * a.cy + a.row0 + yb);
  }
  __syncthreads();

  for (int z = zbeg; z < zend; ++z) {
    const int b = z & 1;
    float4* sbuf = sb + b * NS * 32;
    Tap* tb = taps + b * TS::kTapSlots;
    if ((ATT || ADJ) && lane < TS::kOwn) {
      const int c = warp + kW * lane;
      if (c < NS) {
        const int xp = x0 - R + c;
        tb[tap_slot<R>(c)] = make_tap(xp, z, cr.m00, cr.m02, cr.m03, cr.m20, cr.m22, cr.m23, a.nx, a.nz, a.cy,
                         xp >= 0 && xp < a.nx);
      }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < TS::kOwn; ++k) {
      const int c = warp + kW * k;
      if (c < NS) {
        const int xp = x0 - R + c;
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        if (xp >= 0 && xp < a.nx && yok) s = ldg4(srow + static_cast<size_t>(xp) * a.cy + yb);
        if (ATT) {
          depth_add4<KAHAN>(Tc[k], cTc[k], sample4(mu, tb[tap_slot<R>(c)], yb, yok));
          s = mul4(s, exp_neg4(depth_value4<KAHAN>(Tc[k], cTc[k])));
        }
        sbuf[c * 32 + lane] = s;
      }
    }
    __syncthreads();
    auto emit = [&](int i, const float4& v) {
      const int x = x0 + warp * kTXW + i;
      if (x >= a.nx || !yok) return;
      if (ADJ) {
        // halo rows lack part of their PSF support: their owner window adds them
        if (lane_writes(a, yb)) scatter4(tmp, tb[tap_slot<R>(warp * kTXW + i + R)], yb, v);
      } else {
        *reinterpret_cast<float4*>(tmp + (static_cast<size_t>(z) * a.nx + x) * a.cs + yb) = v;
      }
    };
    if (PSF) {
      const float* kr = s_psf + z * 2 * K;
      rowpass_from_tile<R>(sbuf, warp * kTXW, emit, kr, kr + K, lane, a.ny);
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) emit(i, sbuf[(warp * kTXW + i) * 32 + lane]);
    }
  }
}

// Reference-mode spread of a mirror unit -- camera c and its mate m at the
// opposite angle about the grid centre -- into ONE scratch volume in c's
// rotated frame:
//   U(x', y, z') = PSF_z'[s_c e^{-T}](x') + PSF'_{nz-1-z'}[s_m(nx-1-x') e^{-T'}](x')
// with T the inclusive mu sum along c's column from its detector side, T'
// the inclusive sum from the other end (the mate's detector side), and PSF'
// the mate's plane nz-1-z' with the row kernel reversed.  The mate's inverse
// matrix is c's mirrored in x and z, so gathering U with c's inverse matrix
// adds both cameras' terms: one mu scan, one scratch volume and one gather
// per pair.  A unit without a mate spreads its camera alone.  CTA = (unit,
// x-tile, depth slab); the PSF planes of the slab only sit in shared memory.
template <int R, bool PSF, bool ATT>
__global__ void __launch_bounds__(32 * kW, 2) k_spread_pair_yg(const YgArgs a, int u0) {
  using TS = TileShape<R>;
  constexpr int NS = TS::NS;
  constexpr int K = 2 * R + 1;
  const float* __restrict__ mu = a.mu + a.row0;
  extern __shared__ __align__(16) unsigned char smem[];
  float4* sb = reinterpret_cast<float4*>(smem);                              // [2 stages][2][NS][32]
  Tap* taps = reinterpret_cast<Tap*>(smem + 2 * TS::kSbBytes);                // [2][kTapSlots]
  float* s_psf = reinterpret_cast<float*>(smem + 2 * TS::kSbBytes + TS::kTapBytes);  // [zper][2K], mate's next

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int slab = blockIdx.x % kSlabsB;
  const int item = blockIdx.x / kSlabsB;
  const int g = item / ntile;
  const int unit = u0 + g;
  const int2 uc = a.units[unit];
  const int cam = uc.x, mate = uc.y;
  const bool paired = mate >= 0;  // uniform over the CTA
  const int x0 = (item % ntile) * kTXC;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const int zper = (a.nz + kSlabsB - 1) / kSlabsB;
  const int zbeg = slab * zper, zend = min(a.nz, zbeg + zper);
  if (zbeg >= zend) return;  // uniform over the CTA
  float* s_psf_m = s_psf + zper * 2 * K;
  if (PSF) {
    for (int i = threadIdx.x; i < (zend - zbeg) * 2 * K; i += blockDim.x) {
      s_psf[i] = __ldg(a.psf + zbeg * 2 * K + i);
      if (paired) {
        const int z = zbeg + i / (2 * K), j = i % (2 * K);
        s_psf_m[i] = __ldg(a.psf + (a.nz - 1 - z) * 2 * K + (j < K ? K - 1 - j : j));
      }
    }
  }
  const CamRows cr = cam_rows(a.geom[cam].fwd);
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * a.cs;  // one scratch volume
  float* __restrict__ tmp = a.temp + vol * g;
  const float* __restrict__ srow = a.sino + static_cast<size_t>(cam) * a.nx * a.cy + a.row0;
  const float* __restrict__ mrow = a.sino + static_cast<size_t>(paired ? mate : cam) * a.nx * a.cy + a.row0;

  // transmissions per sampled column: forward (from the slab carry) and, for
  // the mate, from the far end (column total minus the carry)
  float4 Tc[TS::kOwn], Tr[TS::kOwn];
#pragma unroll
  for (int k = 0; k < TS::kOwn; ++k) {
    Tc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    Tr[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int xp = x0 - R + warp + kW * k;
    if (ATT && warp + kW * k < NS && xp >= 0 && xp < a.nx && yok) {
      const float* cp = a.slab_T + ((static_cast<size_t>(cam) * kCarrySlots + slab) * a.nx + xp) * a.cy + a.row0 + yb;
      Tc[k] = ldg4(cp);
      if (paired) {
        const float4 tot = ldg4(cp + static_cast<size_t>(kSlabsB - slab) * a.nx * a.cy);
        Tr[k] = make_float4(tot.x - Tc[k].x, tot.y - Tc[k].y, tot.z - Tc[k].z, tot.w - Tc[k].w);
      }
    }
  }
  __syncthreads();

  for (int z = zbeg; z < zend; ++z) {
    const int b = z & 1;
    float4* sc = sb + b * 2 * NS * 32;
    float4* sm = sc + NS * 32;
    Tap* tb = taps + b * TS::kTapSlots;
    if (ATT && lane < TS::kOwn) {
      const int c = warp + kW * lane;
      if (c < NS) {
        const int xp = x0 - R + c;
        tb[tap_slot<R>(c)] = make_tap(xp, z, cr.m00, cr.m02, cr.m03, cr.m20, cr.m22, cr.m23, a.nx, a.nz, a.cy,
                                      xp >= 0 && xp < a.nx);
      }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < TS::kOwn; ++k) {
      const int c = warp + kW * k;
      if (c < NS) {
        const int xp = x0 - R + c;
        const bool ok = xp >= 0 && xp < a.nx && yok;
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f), q = s;
        if (ok) s = ldg4(srow + static_cast<size_t>(xp) * a.cy + yb);
        if (paired && ok) q = ldg4(mrow + static_cast<size_t>(a.nx - 1 - xp) * a.cy + yb);
        if (ATT) {
          const float4 m = sample4(mu, tb[tap_slot<R>(c)], yb, yok);
          add4(Tc[k], m);
          s = mul4(s, exp_neg4(Tc[k]));
          if (paired) {
            q = mul4(q, exp_neg4(Tr[k]));
            Tr[k] = make_float4(Tr[k].x - m.x, Tr[k].y - m.y, Tr[k].z - m.z, Tr[k].w - m.w);
          }
        }
        sc[c * 32 + lane] = s;
        if (paired) sm[c * 32 + lane] = q;
      }
    }
    __syncthreads();
    float4 acc[kTXW];
#pragma unroll
    for (int i = 0; i < kTXW; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    auto write = [&](int i, float4 v) {
      const int x = x0 + warp * kTXW + i;
      if (x >= a.nx || !yok) return;
      if (paired) add4(v, acc[i]);
      *reinterpret_cast<float4*>(tmp + (static_cast<size_t>(z) * a.nx + x) * a.cs + yb) = v;
    };
    if (PSF) {
      if (paired) {
        const float* km = s_psf_m + (z - zbeg) * 2 * K;
        rowpass_from_tile<R>(sm, warp * kTXW, [&](int i, const float4& v) { acc[i] = v; }, km, km + K, lane,
                             a.ny);
      }
      const float* kr = s_psf + (z - zbeg) * 2 * K;
      rowpass_from_tile<R>(sc, warp * kTXW, write, kr, kr + K, lane, a.ny);
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) {
        if (paired) acc[i] = sm[(warp * kTXW + i) * 32 + lane];
        write(i, sc[(warp * kTXW + i) * 32 + lane]);
      }
    }
  }
}

// ------------------------------------ backprojector: inverse-rotation gather
// out[Z][X][y] (+)= sum_g bilinear(temp[g], B_g * (X, y, Z)) with B_g the
// camera's inverse matrix (ZYX order, -theta), emission-lib/_et.cpp:474-497.
// With a.units, g runs over units and B_g is the unit's first camera's.
__global__ void __launch_bounds__(32 * kGatherWarps) k_gather_yg(const YgArgs a, int c0, int gcount, int first) {
  constexpr int C = kGatherCols;
  extern __shared__ Tap s_gtap[];  // [kGatherWarps][C * group]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunk = (a.nx + C - 1) / C;
  const int item = blockIdx.x * kGatherWarps + warp;
  if (item >= nchunk * a.nz) return;
  const int Z = item / nchunk;
  const int X0 = (item % nchunk) * C;
  const int yb = lane * 4;
  Tap* tap = s_gtap + warp * C * a.group;
  for (int e = lane; e < C * gcount; e += 32) {
    const int g = e / C, X = X0 + e % C;
    const CamRows cr = cam_rows(a.geom[a.units ? a.units[c0 + g].x : c0 + g].bwd);
    // footprints in the scratch (column stride cs)
    tap[e] = make_tap(X, Z, cr.m00, cr.m02, cr.m03, cr.m20, cr.m22, cr.m23, a.nx, a.nz, a.cs, X < a.nx);
  }
  __syncwarp();
  if (!lane_rows_ok(a, yb) || !lane_writes(a, yb)) return;
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * a.cs;
  // camera outer, columns inner: neighbouring accumulator columns of one
  // camera share footprint columns, which then hit in L1
  float4 acc[C];
#pragma unroll
  for (int i = 0; i < C; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int g = 0; g < gcount; ++g) {
    const float* src = a.temp + vol * g;
#pragma unroll
    for (int i = 0; i < C; ++i) add4(acc[i], sample4(src, tap[g * C + i], yb, true));
  }
#pragma unroll
  for (int i = 0; i < C; ++i) {
    const int X = X0 + i;
    if (X >= a.nx) continue;
    float4* dst = reinterpret_cast<float4*>(a.out + (static_cast<size_t>(Z) * a.nx + X) * a.cy + a.row0 + yb);
    if (!first) add4(acc[i], *dst);
    *dst = acc[i];
  }
}

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

// ------------------------------------------------------------- dispatch
// Depth slabs (cluster size) of the projector: the fewest of 2, 4, 8 that
// give at least four waves of CTAs (fewer slabs merge less; more slabs fill
// the GPU for small problems).  Measured on GB300: 128^3 x 120 cameras 4
// (0.84 ms; 2: 0.87, 8: 0.87), 256^3 x 180: 2 (15.9 ms; 4: 16.7),
// 64^3 x 60: 8 (0.149 ms; 4: 0.158).
int project_slabs(int items, int ctas_per_sm) {
  const int slots = 152 * ctas_per_sm;
  for (int s = 2; s < 8; s *= 2)
    if (items * s >= 4 * slots) return s;
  return 8;
}

template <int R>
int launch_project_R(const YgArgs& a_in, cudaStream_t st) {
  YgArgs a = a_in;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const bool psf = a.psf != nullptr;
  const bool bf16 = a.storage == kStorageBF16;
  // mirror cameras are served by the float32 kernels only
  const bool pair = a.units != nullptr && a.nunits > 0 && !bf16;
  const int nunits = pair ? a.nunits : a.ncam;
  // the PSF in the kernel parameters when the host copy is given and fits
  const bool ptab = psf && a.psf_host && static_cast<size_t>(a.nz) * 2 * (2 * R + 1) <= kPsfTableFloats;
  const size_t smem = tile_smem_bytes<R>(psf && !ptab ? a.nz : 0, pair);
  // three CTAs per SM need three tiles (plus 1 KB reserved each) in the 228 KB
  const bool three = 3 * (smem + 1024) <= 228 * 1024;
  if (a.pslabs != 2 && a.pslabs != 4 && a.pslabs != 8)
    a.pslabs = project_slabs(nunits * ntile, three && !bf16 && !pair ? 3 : 2);
  auto go = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nunits * ntile * a.pslabs);
    cfg.blockDim = dim3(32 * kW);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = a.pslabs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NRGB_LAUNCH_SCOPE("k_project_yg", st);
    cudaLaunchKernelEx(&cfg, k, a);
  };
  auto go_tab = [&](auto k) {
    static thread_local PsfTable table;
    std::memcpy(table.c, a.psf_host, sizeof(float) * a.nz * 2 * (2 * R + 1));
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nunits * ntile * a.pslabs);
    cfg.blockDim = dim3(32 * kW);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = a.pslabs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    NRGB_LAUNCH_SCOPE("k_project_yg", st);
    cudaLaunchKernelEx(&cfg, k, a, table);
  };
  auto pick = [&](auto v, auto ctas, auto paired) {
    using V = decltype(v);
    constexpr int C = decltype(ctas)::value;
    constexpr bool P = decltype(paired)::value;
    if (psf && ptab) {
      if (a.mu) go_tab(k_project_ptab_yg<R, true, V, C, P>);
      else go_tab(k_project_ptab_yg<R, false, V, C, P>);
    } else if (psf) {
      if (a.mu) go(k_project_yg<R, true, true, V, C, P>);
      else go(k_project_yg<R, true, false, V, C, P>);
    } else {
      if (a.mu) go(k_project_yg<0, false, true, V, C, P>);
      else go(k_project_yg<0, false, false, V, C, P>);
    }
  };
  using Off = std::false_type;
  using On = std::true_type;
  // the mirror-camera item needs the 128-register budget of two CTAs per SM
  if (bf16)
    pick(__nv_bfloat16(), std::integral_constant<int, 2>(), Off());
  else if (pair)
    pick(0.0f, std::integral_constant<int, 2>(), On());
  else if (three)
    pick(0.0f, std::integral_constant<int, 3>(), Off());
  else
    pick(0.0f, std::integral_constant<int, 2>(), Off());
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

template <int R, bool ADJ>
int launch_spread_R(const YgArgs& a, int c0, int gcount, cudaStream_t st) {
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const dim3 grid(gcount * ntile * kSlabsB), block(32 * kW);
  const bool psf = a.psf != nullptr;
  const size_t smem = tile_smem_bytes<R>(psf ? a.nz : 0);
  auto go = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE(ADJ ? "k_adjoint_yg" : "k_spread_yg", st);
    k<<<grid, block, smem, st>>>(a, c0);
  };
  // only mu is sampled from storage here (the sinogram is float32)
  const bool bf16 = a.storage == kStorageBF16;
  const bool three = 3 * (smem + 1024) <= 228 * 1024;
  if (psf) {
    if (a.mu && bf16) {
      go(k_spread_yg<R, true, true, ADJ, __nv_bfloat16>);
    } else if (a.mu) {
      if constexpr (!ADJ) {
        if (three)
          go(k_spread_yg<R, true, true, false, float, 3>);
        else
          go(k_spread_yg<R, true, true, false, float>);
      } else {
        go(k_spread_yg<R, true, true, true, float>);
      }
    } else {
      go(k_spread_yg<R, true, false, ADJ, float>);
    }
  } else {
    if (a.mu && bf16) go(k_spread_yg<0, false, true, ADJ, __nv_bfloat16>);
    else if (a.mu) go(k_spread_yg<0, false, true, ADJ, float>);
    else go(k_spread_yg<0, false, false, ADJ, float>);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

template <int R>
int launch_spread_pair_R(const YgArgs& a, int u0, int gcount, cudaStream_t st) {
  using TS = TileShape<R>;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const dim3 grid(gcount * ntile * kSlabsB), block(32 * kW);
  const bool psf = a.psf != nullptr;
  const int zper = (a.nz + kSlabsB - 1) / kSlabsB;
  const size_t smem = 2 * TS::kSbBytes + TS::kTapBytes + (psf ? sizeof(float) * 2 * zper * 2 * (2 * R + 1) : 0);
  auto go = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE("k_spread_pair_yg", st);
    k<<<grid, block, smem, st>>>(a, u0);
  };
  if (psf) {
    if (a.mu) go(k_spread_pair_yg<R, true, true>);
    else go(k_spread_pair_yg<R, true, false>);
  } else {
    if (a.mu) go(k_spread_pair_yg<0, false, true>);
    else go(k_spread_pair_yg<0, false, false>);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int spread_pair_by_radius(int R, const YgArgs& a, int u0, int gcount, cudaStream_t st) {
  switch (R) {
    case 0: return launch_spread_pair_R<0>(a, u0, gcount, st);
    case 1: return launch_spread_pair_R<1>(a, u0, gcount, st);
    case 2: return launch_spread_pair_R<2>(a, u0, gcount, st);
    case 3: return launch_spread_pair_R<3>(a, u0, gcount, st);
    case 4: return launch_spread_pair_R<4>(a, u0, gcount, st);
    case 5: return launch_spread_pair_R<5>(a, u0, gcount, st);
    case 6: return launch_spread_pair_R<6>(a, u0, gcount, st);
    case 7: return launch_spread_pair_R<7>(a, u0, gcount, st);
    default: return kErrParameters;
  }
}

int project_by_radius(int R, const YgArgs& a, cudaStream_t st) {
  switch (R) {
    case 0: return launch_project_R<0>(a, st);
    case 1: return launch_project_R<1>(a, st);
    case 2: return launch_project_R<2>(a, st);
    case 3: return launch_project_R<3>(a, st);
    case 4: return launch_project_R<4>(a, st);
    case 5: return launch_project_R<5>(a, st);
    case 6: return launch_project_R<6>(a, st);
    case 7: return launch_project_R<7>(a, st);
    default: return kErrParameters;
  }
}

// Persistent grid: two CTAs per SM, whole clusters.
constexpr int kBatchClusters = 152 * 2 / kSlabsP;

template <int R, bool PSF>
int launch_project_batch_R(const BatchStepDesc* d, const BatchSel& sel, bool att, int max_nz, int* counter,
                           cudaStream_t st) {
  const size_t smem = tile_smem_bytes<R>(PSF ? max_nz : 0);
  auto go = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE("k_project_batch_yg", st);
    k<<<kBatchClusters * kSlabsP, 32 * kW, smem, st>>>(d, sel, counter);
  };
  if (att)
    go(k_project_batch_yg<R, PSF, true>);
  else
    go(k_project_batch_yg<R, PSF, false>);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int project_batch_by_radius(int psf_k, const BatchStepDesc* d, const BatchSel& sel, bool att, int max_nz,
                            int* counter, cudaStream_t st) {
  if (psf_k == 0) return launch_project_batch_R<0, false>(d, sel, att, max_nz, counter, st);
  switch ((psf_k - 1) / 2) {
    case 0: return launch_project_batch_R<0, true>(d, sel, att, max_nz, counter, st);
    case 1: return launch_project_batch_R<1, true>(d, sel, att, max_nz, counter, st);
    case 2: return launch_project_batch_R<2, true>(d, sel, att, max_nz, counter, st);
    case 3: return launch_project_batch_R<3, true>(d, sel, att, max_nz, counter, st);
    case 4: return launch_project_batch_R<4, true>(d, sel, att, max_nz, counter, st);
    case 5: return launch_project_batch_R<5, true>(d, sel, att, max_nz, counter, st);
    case 6: return launch_project_batch_R<6, true>(d, sel, att, max_nz, counter, st);
    case 7: return launch_project_batch_R<7, true>(d, sel, att, max_nz, counter, st);
    default: return kErrParameters;
  }
}

template <bool ADJ>
int spread_by_radius_t(int R, const YgArgs& a, int c0, int gcount, cudaStream_t st) {
  switch (R) {
    case 0: return launch_spread_R<0, ADJ>(a, c0, gcount, st);
    case 1: return launch_spread_R<1, ADJ>(a, c0, gcount, st);
    case 2: return launch_spread_R<2, ADJ>(a, c0, gcount, st);
    case 3: return launch_spread_R<3, ADJ>(a, c0, gcount, st);
    case 4: return launch_spread_R<4, ADJ>(a, c0, gcount, st);
    case 5: return launch_spread_R<5, ADJ>(a, c0, gcount, st);
    case 6: return launch_spread_R<6, ADJ>(a, c0, gcount, st);
    case 7: return launch_spread_R<7, ADJ>(a, c0, gcount, st);
    default: return kErrParameters;
  }
}

int spread_by_radius(int R, const YgArgs& a, int c0, int gcount, cudaStream_t st) {
  return spread_by_radius_t<false>(R, a, c0, gcount, st);
}

}  // namespace

namespace {

constexpr int kWindowRows = 128;  // rows one warp covers (32 lanes x 4)

// Row windows of a volume for a PSF halo: window starts and valid ranges are
// multiples of 4 (the halo is rounded up), every row is valid in exactly one
// window, and a valid row's whole PSF support lies inside its window or past
// the volume's edge.  Y-gantry rotations keep y, so a window computes its
// valid rows with exactly the arithmetic of a single pass.
struct Window {
  int row0, rows, lo, hi;  // rows [row0, row0 + rows); valid [row0 + lo, row0 + hi)
};

std::vector<Window> row_windows(int ny, int halo) {
  const int h = (halo + 3) & ~3;
  std::vector<Window> w;
  if (ny <= kWindowRows) {
    w.push_back({0, ny, 0, ny});
    return w;
  }
  int out0 = 0;
  while (out0 < ny) {
    const int in0 = std::max(0, out0 - h);
    if (in0 + kWindowRows >= ny) {
      w.push_back({in0, ny - in0, out0 - in0, ny - in0});
      break;
    }
    const int out1 = in0 + kWindowRows - h;
    w.push_back({in0, kWindowRows, out0 - in0, out1 - in0});
    out0 = out1;
  }
  return w;
}

YgArgs windowed(const YgArgs& a, const Window& w) {
  YgArgs b = a;
  b.row0 = w.row0;
  b.ny = w.rows;
  b.out_lo = w.lo;
  b.out_hi = w.hi;
  b.cs = round_up(w.rows, 4);
  return b;
}

int scratch_rows(int ny) { return round_up(std::min(ny, kWindowRows), 4); }

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

int yg_project_batch(const BatchStepDesc* d_desc, const BatchSel& sel, int psf_k, bool att, int max_nz,
                     int* d_counter, cudaStream_t st) {
  if (sel.n <= 0 || sel.total <= 0) return kOk;
  return project_batch_by_radius(psf_k, d_desc, sel, att, max_nz, d_counter, st);
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

size_t yg_backproject_workspace(int nx, int ny, int nz, int ncam, int group, int slots) {
  const size_t cy = round_up(ny, 4);
  const size_t vol = static_cast<size_t>(nz) * nx * scratch_rows(ny);  // one window's scratch volume
  const size_t slabs = static_cast<size_t>(ncam) * kCarrySlots * nx * cy;
  // with two slots the spread of group g+1 overlaps the gather of group g
  return sizeof(float) * (slabs + static_cast<size_t>(slots) * vol * std::max(1, std::min(group, ncam)));
}

int yg_carry_slabs() { return kCarrySlots; }

int yg_mu_carry(const YgArgs& a_in, float* out, cudaStream_t st) {
  const int nchunk = (a_in.nx + kCarryCols - 1) / kCarryCols;
  const int n = a_in.units ? a_in.nunits : a_in.ncam;
  for (const Window& w : row_windows(a_in.ny, 0)) {  // carries need no halo
    YgArgs a = windowed(a_in, w);
    a.slab_T = out;
    NRGB_LAUNCH_SCOPE("k_mu_carry_yg", st);
    if (a.storage == kStorageBF16)
      k_mu_carry_yg<__nv_bfloat16><<<n * nchunk, 32 * kSlabsB, 0, st>>>(a);
    else
      k_mu_carry_yg<float><<<n * nchunk, 32 * kSlabsB, 0, st>>>(a);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int yg_project(const YgArgs& a, cudaStream_t st) {
  const int R = a.psf ? (a.psf_k - 1) / 2 : 0;
  for (const Window& w : row_windows(a.ny, R)) {
    const int s = project_by_radius(R, windowed(a, w), st);
    if (s != kOk) return s;
  }
  return kOk;
}

namespace {

// Second stream and events of the backprojection pipeline, one set per device.
struct Pipe {
  cudaStream_t aux = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr, spread_done[2] = {nullptr, nullptr},
              gather_done[2] = {nullptr, nullptr};
};

Pipe* pipe_for_current_device() {
  static std::mutex mu;
  static std::map<int, Pipe> pipes;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  Pipe& p = pipes[dev];
  if (!p.aux) {
    if (cudaStreamCreateWithFlags(&p.aux, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    cudaEvent_t* evs[] = {&p.fork, &p.join, &p.spread_done[0], &p.spread_done[1], &p.gather_done[0],
                          &p.gather_done[1]};
    for (cudaEvent_t* e : evs)
      if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
  }
  return &p;
}

}  // namespace

// Per row window and camera group: spread on the caller's stream, gather on
// a second stream; step g (over all windows' groups) uses scratch slot g % 2,
// so the spread of step g+1 runs while the gather of step g reads the other
// slot.
int yg_backproject(const YgArgs& a_in, cudaStream_t st) {
  YgArgs a = a_in;
  const int R = a.psf ? (a.psf_k - 1) / 2 : 0;
  // mirror units: reference mode, float32 mu
  const bool pair = a.units && a.nunits > 0 && a.back_mode == kBackReference && a.storage != kStorageBF16;
  if (!pair) {
    a.units = nullptr;
    a.nunits = 0;
  }
  const int nunits = pair ? a.nunits : a.ncam;  // scratch volumes to spread and gather
  // even groups of at most a.group units
  int group = std::max(1, std::min(a.group, nunits));
  const int ngroups = (nunits + group - 1) / group;
  group = (nunits + ngroups - 1) / ngroups;
  // work space: slab carries first (unless given), then the scratch slot(s)
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * scratch_rows(a.ny);
  float* slot0;
  if (a.carry || !a.mu) {  // carries given, or not needed without attenuation
    a.slab_T = const_cast<float*>(a.carry);
    slot0 = a.work;
  } else {
    a.slab_T = a.work;
    slot0 = a.work + static_cast<size_t>(a.ncam) * kCarrySlots * a.nx * a.cy;
    int s = yg_mu_carry(a, a.slab_T, st);
    if (s != kOk) return s;
  }
  a.group = group;
  auto spread = [&](const YgArgs& b, int c0, int gcount) {
    return pair ? spread_pair_by_radius(R, b, c0, gcount, st) : spread_by_radius(R, b, c0, gcount, st);
  };
  const std::vector<Window> wins = row_windows(a.ny, R);
  if (a.back_mode == kBackAdjoint) {
    // transpose of the projector: one launch per window over all cameras,
    // scattered straight into the zeroed accumulator
    const size_t full = static_cast<size_t>(a.nz) * a.nx * a.cy;
    if (cudaMemsetAsync(a.out, 0, sizeof(float) * full, st) != cudaSuccess) return kErrKernel;
    for (const Window& w : wins) {
      const int s = spread_by_radius_t<true>(R, windowed(a, w), 0, a.ncam, st);
      if (s != kOk) return s;
    }
    return kOk;
  }
  const int nchunk = (a.nx + kGatherCols - 1) / kGatherCols;
  const int gblocks = (nchunk * a.nz + kGatherWarps - 1) / kGatherWarps;
  const size_t gsmem = sizeof(Tap) * kGatherWarps * kGatherCols * group;
  cudaFuncSetAttribute(k_gather_yg, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(gsmem));
  if (!a.pipelined) {
    for (const Window& w : wins) {
      YgArgs b = windowed(a, w);
      b.temp = slot0;
      for (int c0 = 0; c0 < nunits; c0 += group) {
        const int gcount = std::min(group, nunits - c0);
        int st_ = spread(b, c0, gcount);
        if (st_ != kOk) return st_;
        NRGB_LAUNCH_SCOPE("k_gather_yg", st);
        k_gather_yg<<<gblocks, 32 * kGatherWarps, gsmem, st>>>(b, c0, gcount, c0 == 0 ? 1 : 0);
      }
    }
    return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
  }
  Pipe* pp = pipe_for_current_device();
  if (!pp) return kErrUnspecified;
  cudaEventRecord(pp->fork, st);
  cudaStreamWaitEvent(pp->aux, pp->fork, 0);
  int gi = 0;
  for (const Window& w : wins) {
    YgArgs b = windowed(a, w);
    for (int c0 = 0; c0 < nunits; c0 += group, ++gi) {
      const int gcount = std::min(group, nunits - c0);
      const int slot = gi & 1;
      b.temp = slot0 + vol * group * slot;
      if (gi >= 2) cudaStreamWaitEvent(st, pp->gather_done[slot], 0);
      int st_ = spread(b, c0, gcount);
      if (st_ != kOk) return st_;
      cudaEventRecord(pp->spread_done[slot], st);
      cudaStreamWaitEvent(pp->aux, pp->spread_done[slot], 0);
      {
        NRGB_LAUNCH_SCOPE("k_gather_yg", pp->aux);
        k_gather_yg<<<gblocks, 32 * kGatherWarps, gsmem, pp->aux>>>(b, c0, gcount, c0 == 0 ? 1 : 0);
      }
      cudaEventRecord(pp->gather_done[slot], pp->aux);
    }
  }
  cudaEventRecord(pp->join, pp->aux);
  cudaStreamWaitEvent(st, pp->join, 0);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
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
  const int grid = static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 16));
  NRGB_LAUNCH_SCOPE("k_to_bf16", st);
  k_to_bf16<<<grid, 256, 0, st>>>(src, static_cast<__nv_bfloat16*>(dst), n);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

int from_bf16(const void* src, float* dst, size_t n, cudaStream_t st) {
  if (n == 0) return kOk;
  const int grid = static_cast<int>(std::min<size_t>((n + 255) / 256, 152 * 16));
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
