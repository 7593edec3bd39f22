// Device building blocks of the fused y-gantry kernels (shared by the
// projector, backprojector and layout translation units): the column layout,
// bilinear footprints, the tile engine with its row and column passes, the
// projector's work item, and the row windows of tall volumes.
//
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
//   pass along y through a per-warp shared row buffer), attenuated depth scan
//   T += mu;
//   p += v * exp(-T).  No rotated volume is written anywhere: a thread-block
//   cluster owns (camera, 32-column x-tile), its CTAs own depth slabs and
//   merge (T, p) through distributed shared memory.
// Backprojector, reference mode (emission-lib/_et.cpp:415-499):
//   (1) per-slab transmission carries of the rotated mu, (2) per camera
//   group: spread s*exp(-T) + PSF in the rotated frame into an L2-sized
//   scratch, (3) inverse-rotation gather of the group into the accumulator.
#pragma once

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
constexpr int kGatherUnits = 2;   // scratch volumes whose loads a gather warp has in flight at once
constexpr unsigned kFull = 0xffffffffu;

__host__ __device__ constexpr size_t round_up16(size_t b) { return (b + 15) / 16 * 16; }

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

// sample4 for a lane whose rows are inside the column (yok) without the
// branch on t.any: the four corner loads are always issued (a footprint's
// offsets stay inside the volume: clamped corners have zero weight and
// offset deltas), so loads of several footprints can be in flight together;
// the value is zero without any valid corner, as in sample4.
__device__ __forceinline__ float4 sample4_loaded(const float* __restrict__ base, const Tap& t, int yb) {
  const float* p = base + t.off + yb;
  const float4 a = ldg4(p), b = ldg4(p + t.dx), c = ldg4(p + t.dz), d = ldg4(p + t.dx + t.dz);
  float4 r;
  r.x = fmaf(d.x, t.w11, fmaf(c.x, t.w01, fmaf(b.x, t.w10, a.x * t.w00)));
  r.y = fmaf(d.y, t.w11, fmaf(c.y, t.w01, fmaf(b.y, t.w10, a.y * t.w00)));
  r.z = fmaf(d.z, t.w11, fmaf(c.z, t.w01, fmaf(b.z, t.w10, a.z * t.w00)));
  r.w = fmaf(d.w, t.w11, fmaf(c.w, t.w01, fmaf(b.w, t.w10, a.w * t.w00)));
  return t.any ? r : make_float4(0.f, 0.f, 0.f, 0.f);
}

// Negative values to zero (NaN kept), as the truncation of the reference.
__device__ __forceinline__ float4 clamp0(float4 v) {
  v.x = v.x < 0.0f ? 0.0f : v.x;
  v.y = v.y < 0.0f ? 0.0f : v.y;
  v.z = v.z < 0.0f ? 0.0f : v.z;
  v.w = v.w < 0.0f ? 0.0f : v.w;
  return v;
}

__device__ __forceinline__ float comp(const float4& v, int c) { return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w; }

// Packed float32 pairs (sm_100 and later): two lanes in one 64-bit register
// pair, multiplied and added by one fma.rn.f32x2 instruction; each lane rounds
// exactly like fmaf.  The row passes keep their accumulators as pairs (rows
// 4l, 4l+1 and 4l+2, 4l+3 of a lane), which halves their FMA instructions.
typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 pk2(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}

__device__ __forceinline__ float2 upk2(f32x2 v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}

// acc = a * b + acc, lane by lane
__device__ __forceinline__ void ffma2(f32x2& acc, f32x2 a, f32x2 b) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(a), "l"(b));
}

// Four rows as two pairs.
struct Pair4 {
  f32x2 lo, hi;
};

__device__ __forceinline__ Pair4 pair4(const float4& v) { return {pk2(v.x, v.y), pk2(v.z, v.w)}; }

__device__ __forceinline__ float4 unpair4(const Pair4& p) {
  const float2 a = upk2(p.lo), b = upk2(p.hi);
  return make_float4(a.x, a.y, b.x, b.y);
}

// acc += k * v for the 4 rows (k broadcast to both lanes of a pair)
__device__ __forceinline__ void axpy4p(Pair4& acc, f32x2 kk, const Pair4& v) {
  ffma2(acc.lo, v.lo, kk);
  ffma2(acc.hi, v.hi, kk);
}

// Elementwise float4 operations as two packed pair instructions each (the
// same roundings as the scalar forms, lane by lane): the projector's depth
// sums and their Kahan steps.
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ void add4p(float4& a, const float4& b) {
  const Pair4 x = pair4(a), y = pair4(b);
  a = unpair4({add2(x.lo, y.lo), add2(x.hi, y.hi)});
}
__device__ __forceinline__ float4 mul4p(const float4& a, const float4& b) {
  const Pair4 x = pair4(a), y = pair4(b);
  return unpair4({mul2(x.lo, y.lo), mul2(x.hi, y.hi)});
}
__device__ __forceinline__ void fma4p(float4& acc, const float4& a, const float4& b) {
  Pair4 c = pair4(acc);
  const Pair4 x = pair4(a), y = pair4(b);
  ffma2(c.lo, x.lo, y.lo);
  ffma2(c.hi, x.hi, y.hi);
  acc = unpair4(c);
}
// Kahan step (kahan_add below) on pairs: y = v - c; t = s + y; c = (t - s) - y; s = t
__device__ __forceinline__ void kahan_add4p(float4& s, float4& c, const float4& v) {
  const Pair4 S = pair4(s), C = pair4(c), V = pair4(v);
  const f32x2 ylo = sub2(V.lo, C.lo), yhi = sub2(V.hi, C.hi);
  const f32x2 tlo = add2(S.lo, ylo), thi = add2(S.hi, yhi);
  c = unpair4({sub2(sub2(tlo, S.lo), ylo), sub2(sub2(thi, S.hi), yhi)});
  s = unpair4({tlo, thi});
}
__device__ __forceinline__ float4 kahan_value4p(const float4& s, const float4& c) {
  const Pair4 S = pair4(s), C = pair4(c);
  return unpair4({sub2(S.lo, C.lo), sub2(S.hi, C.hi)});
}

__device__ __forceinline__ void axpy4(float4& acc, float k, const float4& v) {
  acc.x = fmaf(k, v.x, acc.x);
  acc.y = fmaf(k, v.y, acc.y);
  acc.z = fmaf(k, v.z, acc.z);
  acc.w = fmaf(k, v.w, acc.w);
}

// Rows y >= ny are zero pads of the column layout; the column pass must not
// leak into them (the reference's column pass only produces rows < ny).
__device__ __forceinline__ float4 mask_rows(float4 v, int yb, int ny) {
  if (yb + 3 < ny) return v;  // every lane of a full window
  if (yb + 0 >= ny) v.x = 0.0f;
  if (yb + 1 >= ny) v.y = 0.0f;
  if (yb + 2 >= ny) v.z = 0.0f;
  if (yb + 3 >= ny) v.w = 0.0f;
  return v;
}

// Column (y) pass of the per-plane convolution for the 4 rows a lane owns:
// out[y] = sum_k in[y+k] * kc[R-k], zero outside [0, ny) (rows >= ny are zero
// pads, rows < 0 come from lanes below 0 and are masked).  Neighbour rows come
// from lanes l-1, l-2 and l+1, l+2 by shuffles (the form for R = 0; larger
// radii use yconv4s below).
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

// Column pass through shared memory: each lane stores its 4 rows in its
// warp's row buffer and reads the neighbour rows back with 16-byte loads (one
// store and 2 ceil(R/4) loads in place of 2R shuffles and 2R selects).  Two
// buffers per warp alternate, so one warp barrier per call orders a store
// after the loads of the call before the previous one.  Rows outside the
// warp's 128 read zero pads, written by ybuf_zero_pads before a kernel's
// first row pass.
constexpr int kYPad = 2;  // pad chunks (4 rows each) on either side: R <= 8
__shared__ __align__(16) float4 s_ybuf[kW][2][32 + 2 * kYPad];
constexpr size_t kYBufBytes = sizeof(float4) * kW * 2 * (32 + 2 * kYPad);  // static, per CTA

__device__ __forceinline__ void ybuf_zero_pads() {
  for (int i = threadIdx.x; i < kW * 2 * 2 * kYPad; i += blockDim.x) {
    const int w = i / (4 * kYPad), r = i % (4 * kYPad);
    const int b = r / (2 * kYPad), q = r % (2 * kYPad);
    s_ybuf[w][b][q < kYPad ? q : 32 + q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

template <int R, class KC>
__device__ __forceinline__ float4 yconv4s(const float4& u, KC kc, int lane, int b) {
  if constexpr (R == 0) {
    return yconv4<0>(u, kc, lane);
  } else {
    constexpr int C = (R + 3) / 4;
    static_assert(C <= kYPad, "row-buffer pads");
    float4* row = &s_ybuf[threadIdx.x >> 5][b][kYPad];
    row[lane] = u;
    __syncwarp();
    float w[2 * R + 4];
#pragma unroll
    for (int c = -C; c <= C; ++c) {
      const float4 v = c == 0 ? u : row[lane + c];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int rel = 4 * c + q;
        if (rel >= -R && rel <= 3 + R) w[R + rel] = comp(v, q);
      }
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
  // Projector: 2 x steps tile buffers (steps depth planes sampled per
  // barrier); the region also holds the slab-merge buffers after the walk (T
  // and P per output column, and with a mirror camera its P).
  __host__ __device__ static constexpr size_t sb_bytes(bool pair, int steps = 1) {
    return sizeof(float4) * 32 * (2 * steps * NS > (pair ? 3 : 2) * kTXC ? 2 * steps * NS : (pair ? 3 : 2) * kTXC);
  }
  __host__ __device__ static constexpr size_t tap_bytes(int steps = 1) { return sizeof(Tap) * 2 * steps * kTapSlots; }
  // Projector serving mirror cameras from bfloat16 storage: the Kahan
  // compensations of T, P and the mate's Q, one float4 per thread and output
  // column each, in shared memory ([3][kTXC][32]) -- registers hold the sums.
  __host__ __device__ static constexpr size_t comp_bytes(bool on) { return on ? sizeof(float4) * 3 * kTXC * 32 : 0; }
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
__host__ __device__ constexpr size_t tile_smem_bytes(int nz, bool pair = false, int steps = 1) {
  return TileShape<R>::sb_bytes(pair, steps) + TileShape<R>::tap_bytes(steps) +
         sizeof(float) * static_cast<size_t>(nz) * 2 * (2 * R + 1) * (pair ? 2 : 1);
}

// The projector's: the tile above plus, for mirror cameras from bfloat16
// storage, the shared-memory Kahan compensations.
template <int R>
__host__ __device__ constexpr size_t project_smem_bytes(int nz, bool pair, bool kahan, int steps = 1) {
  return tile_smem_bytes<R>(nz, pair, steps) + TileShape<R>::comp_bytes(pair && kahan);
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
      emit(i, mask_rows(yconv4s<R>(u[i % K], kc, lane, i & 1), 4 * lane, ny));
      u[i % K] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
}

// Packed forms of the two row passes below (accumulators as float32 pairs,
// one fma.rn.f32x2 per two rows; the same roundings in the same order), used
// by the projector.  The spread keeps the scalar forms: its two transmission
// arrays leave no registers for the broadcast coefficient pairs.
template <int R, class EmitFn, class KR, class KC>
__device__ __forceinline__ void rowpass_from_tile_p(const float4* __restrict__ sbuf, int base, EmitFn emit, KR kr, KC kc,
                                                  int lane, int ny) {
  constexpr int K = 2 * R + 1;
  constexpr int NJ = kTXW + 2 * R;
  Pair4 u[kTXW];
  const f32x2 zero = pk2(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < kTXW; ++q) u[q] = {zero, zero};
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const Pair4 r = pair4(sbuf[(base + j) * 32 + lane]);
#pragma unroll
    for (int d = 0; d < K; ++d) {
      const int i = j - d;
      if (i >= 0 && i < kTXW) {
        const float k = kr[2 * R - d];
        axpy4p(u[i], pk2(k, k), r);
      }
    }
    const int i = j - 2 * R;
    if (i >= 0 && i < kTXW) emit(i, mask_rows(yconv4s<R>(unpair4(u[i]), kc, lane, i & 1), 4 * lane, ny));
  }
}

// Row passes of two cameras in one sweep: over the same tile (a camera and
// its mirror camera in the projector: each tile column is read once and feeds
// both sliding windows) or over two tiles (the mirror-unit spread); output i
// of camera b is emitted before output i of camera a.
template <int R, class EmitA, class EmitB, class KRA, class KCA, class KRB, class KCB>
__device__ __forceinline__ void rowpass2_from_tiles(const float4* __restrict__ sa, const float4* __restrict__ sbt,
                                                    int base, EmitA emit_a, KRA kra, KCA kca, EmitB emit_b, KRB krb,
                                                    KCB kcb, int lane, int ny) {
  constexpr int NJ = kTXW + 2 * R;
  float4 ua[kTXW], ub[kTXW];
#pragma unroll
  for (int q = 0; q < kTXW; ++q) {
    ua[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    ub[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const float4 r = sa[(base + j) * 32 + lane];
    const float4 rb = sbt == sa ? r : sbt[(base + j) * 32 + lane];
#pragma unroll
    for (int d = 0; d <= 2 * R; ++d) {
      const int i = j - d;
      if (i >= 0 && i < kTXW) {
        axpy4(ua[i], kra[2 * R - d], r);
        axpy4(ub[i], krb[2 * R - d], rb);
      }
    }
    const int i = j - 2 * R;
    if (i >= 0 && i < kTXW) {
      emit_b(i, mask_rows(yconv4s<R>(ub[i], kcb, lane, 0), 4 * lane, ny));
      emit_a(i, mask_rows(yconv4s<R>(ua[i], kca, lane, 1), 4 * lane, ny));
    }
  }
}

template <int R, class EmitA, class EmitB, class KRA, class KCA, class KRB, class KCB>
__device__ __forceinline__ void rowpass2_from_tiles_p(const float4* __restrict__ sa, const float4* __restrict__ sbt,
                                                    int base, EmitA emit_a, KRA kra, KCA kca, EmitB emit_b, KRB krb,
                                                    KCB kcb, int lane, int ny) {
  constexpr int NJ = kTXW + 2 * R;
  Pair4 ua[kTXW], ub[kTXW];
  const f32x2 zero = pk2(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < kTXW; ++q) {
    ua[q] = {zero, zero};
    ub[q] = {zero, zero};
  }
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const float4 rf = sa[(base + j) * 32 + lane];
    const Pair4 r = pair4(rf);
    const Pair4 rb = sbt == sa ? r : pair4(sbt[(base + j) * 32 + lane]);
#pragma unroll
    for (int d = 0; d <= 2 * R; ++d) {
      const int i = j - d;
      if (i >= 0 && i < kTXW) {
        const float ka = kra[2 * R - d], kb = krb[2 * R - d];
        axpy4p(ua[i], pk2(ka, ka), r);
        axpy4p(ub[i], pk2(kb, kb), rb);
      }
    }
    const int i = j - 2 * R;
    if (i >= 0 && i < kTXW) {
      emit_b(i, mask_rows(yconv4s<R>(unpair4(ub[i]), kcb, lane, 0), 4 * lane, ny));
      emit_a(i, mask_rows(yconv4s<R>(unpair4(ua[i]), kca, lane, 1), 4 * lane, ny));
    }
  }
}

template <int R, class EmitA, class EmitB, class KRA, class KCA, class KRB, class KCB>
__device__ __forceinline__ void rowpass2_from_tile(const float4* __restrict__ sbuf, int base, EmitA emit_a, KRA kra,
                                                   KCA kca, EmitB emit_b, KRB krb, KCB kcb, int lane, int ny) {
  rowpass2_from_tiles<R>(sbuf, sbuf, base, emit_a, kra, kca, emit_b, krb, kcb, lane, ny);
}

template <int R, class EmitA, class EmitB, class KRA, class KCA, class KRB, class KCB>
__device__ __forceinline__ void rowpass2_from_tile_p(const float4* __restrict__ sbuf, int base, EmitA emit_a, KRA kra,
                                                     KCA kca, EmitB emit_b, KRB krb, KCB kcb, int lane, int ny) {
  rowpass2_from_tiles_p<R>(sbuf, sbuf, base, emit_a, kra, kca, emit_b, krb, kcb, lane, ny);
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

//
// STEPS: depth planes sampled per barrier (2 x STEPS tile buffers).  Two
// planes per barrier measured no faster on GB300 (128^3 x 120: 0.676 against
// 0.674 ms; 256^3 x 180: 11.9 against 11.2 ms), so the kernels use one.
template <int R, bool PSF, bool ATT, class V, bool PAIR = false, bool PTAB = false, int STEPS = 1>
__device__ __forceinline__ void project_item(const YgArgs& a, int cam, int mate, int x0, unsigned char* smem,
                                             const float* ptab = nullptr) {
  using TS = TileShape<R>;
  constexpr bool KAHAN = StorageTraits<V>::kKahan;
  // mirror cameras from bfloat16 storage: compensations in shared memory
  constexpr bool SCOMP = PAIR && KAHAN;
  const V* __restrict__ act = reinterpret_cast<const V*>(a.act) + a.row0;
  const V* __restrict__ mu = reinterpret_cast<const V*>(a.mu) + a.row0;
  constexpr int NS = TS::NS;
  constexpr int K = 2 * R + 1;
  constexpr size_t kSb = TS::sb_bytes(PAIR, STEPS);
  float4* sb = reinterpret_cast<float4*>(smem);                    // [2 * STEPS][NS][32]
  Tap* taps = reinterpret_cast<Tap*>(smem + kSb);                   // [2 * STEPS][kTapSlots]
  float4* scomp = reinterpret_cast<float4*>(smem + kSb + TS::tap_bytes(STEPS));  // [3][kTXC][32] (SCOMP)
  float* s_psf = reinterpret_cast<float*>(smem + kSb + TS::tap_bytes(STEPS) + TS::comp_bytes(SCOMP));  // [nz][2K]
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
      rowpass_from_tile_p<R>(sbuf, warp * kTXW, emit_m, Reversed<R>{m}, m + K, lane, a.ny);
    } else {
      const float* m = s_psf_m + z * 2 * K;
      rowpass_from_tile_p<R>(sbuf, warp * kTXW, emit_m, m, m + K, lane, a.ny);
    }
  };
  auto both_pass = [&](const float4* sbuf, int z, auto emit, auto emit_m) {
    const float* kr = (PTAB ? ptab : s_psf) + z * 2 * K;
    if constexpr (PTAB) {
      const float* m = ptab + (a.nz - 1 - z) * 2 * K;
      rowpass2_from_tile_p<R>(sbuf, warp * kTXW, emit, kr, kr + K, emit_m, Reversed<R>{m}, m + K, lane, a.ny);
    } else {
      const float* m = s_psf_m + z * 2 * K;
      rowpass2_from_tile_p<R>(sbuf, warp * kTXW, emit, kr, kr + K, emit_m, m, m + K, lane, a.ny);
    }
  };
  const CamRows cr = cam_rows(a.geom[cam].fwd);

  constexpr int NC = SCOMP ? 1 : kTXW;
  float4 T[kTXW], P[kTXW], cT[NC], cP[NC];  // c*: Kahan compensations (KAHAN without SCOMP)
  float4 Q[PAIR ? kTXW : 1];                // mate's slab partial
  // compensation slot of quantity q (0 T, 1 P, 2 Q) of output i (SCOMP)
  auto cslot = [&](int q, int i) { return scomp + (q * kTXC + warp * kTXW + i) * 32 + lane; };
  // s += v, Kahan-compensated (KAHAN) or plain; value of a compensated sum
  auto kadd = [&](float4& s, float4* creg, int q, int i, const float4& v) {
    if constexpr (SCOMP) {
      float4 c = *cslot(q, i);
      kahan_add4p(s, c, v);
      *cslot(q, i) = c;
    } else if constexpr (KAHAN) {
      kahan_add4p(s, *creg, v);
    } else {
      add4p(s, v);
    }
  };
  auto kval = [&](const float4& s, const float4* creg, int q, int i) -> float4 {
    if constexpr (SCOMP) return kahan_value4p(s, *cslot(q, i));
    else if constexpr (KAHAN) return kahan_value4p(s, *creg);
    else return s;
  };
  auto kclear = [&](int q, int i) {
    if constexpr (SCOMP) *cslot(q, i) = make_float4(0.f, 0.f, 0.f, 0.f);
  };
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    T[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!SCOMP) {
      cT[SCOMP ? 0 : i] = make_float4(0.f, 0.f, 0.f, 0.f);
      cP[SCOMP ? 0 : i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (PAIR) Q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int q = 0; q < 3; ++q) kclear(q, i);
  }
  ybuf_zero_pads();
  __syncthreads();

  // A depth step at plane z through tile buffer b: produce (footprints and
  // samples of the NS columns), then, after a barrier, consume (row and
  // column passes, depth sums).  MODE 0: this camera (and the mate's forward
  // form); MODE 1: the mate alone, direct weights (walked from the slab's
  // far end).
  auto produce = [&](int z, int b) {
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
  };
  auto consume = [&](int z, int b, auto mode) {
    constexpr int MODE = decltype(mode)::value;
    const float4* sbuf = sb + b * NS * 32;
    const Tap* tb = taps + b * TS::kTapSlots;
    auto emit_m = [&](int i, const float4& v) {
      if (!ATT) {
        if (KAHAN) kadd(Q[i], nullptr, 2, i, v);
        else add4(Q[i], v);
      } else if (MODE == 0) {  // weight exp(E_z): T holds the sum before plane z
        if (KAHAN) {
          const float4 e = kval(T[i], &cT[SCOMP ? 0 : i], 0, i);
          kadd(Q[i], nullptr, 2, i, mul4p(v, exp_neg4(make_float4(-e.x, -e.y, -e.z, -e.w))));
        } else {
          fma4p(Q[i], v, exp_neg4(make_float4(-T[i].x, -T[i].y, -T[i].z, -T[i].w)));
        }
      } else {  // T runs from the slab's far end, inclusive
        const float4 m = sample4(mu, tb[tap_slot<R>(warp * kTXW + i + R)], yb, yok);
        if (KAHAN) {
          kadd(T[i], &cT[SCOMP ? 0 : i], 0, i, m);
          kadd(Q[i], nullptr, 2, i, mul4p(v, exp_neg4(kval(T[i], &cT[SCOMP ? 0 : i], 0, i))));
        } else {
          add4p(T[i], m);
          fma4p(Q[i], v, exp_neg4(T[i]));
        }
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
    // float32, PSF radius <= 5: mu of the warp's output columns sampled
    // before the row pass, so that the gathers' latency overlaps the PSF
    // arithmetic (128^3 x 120, PSF 11: projector 0.608 -> 0.586 ms); wider
    // PSFs would spill registers (radius 7: slower)
    constexpr bool kEarlyMu = ATT && !KAHAN && R <= 5;
    float4 mv[kTXW];
    if constexpr (kEarlyMu) {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) mv[i] = sample4(mu, tb[tap_slot<R>(warp * kTXW + i + R)], yb, yok);
    }
    auto emit = [&](int i, const float4& v) {
      if (ATT) {
        const float4 m = kEarlyMu ? mv[i] : sample4(mu, tb[tap_slot<R>(warp * kTXW + i + R)], yb, yok);
        if (KAHAN) {
          kadd(T[i], &cT[SCOMP ? 0 : i], 0, i, m);
          kadd(P[i], &cP[SCOMP ? 0 : i], 1, i, mul4p(v, exp_neg4(kval(T[i], &cT[SCOMP ? 0 : i], 0, i))));
        } else {
          add4p(T[i], m);
          fma4p(P[i], v, exp_neg4(T[i]));
        }
      } else {
        kadd(P[i], &cP[SCOMP ? 0 : i], 1, i, v);
      }
    };
    if (PSF) {
      if (PAIR && paired) {
        both_pass(sbuf, z, emit, emit_m);
      } else {
        const float* kr = (PTAB ? ptab : s_psf) + z * 2 * K;
        rowpass_from_tile_p<R>(sbuf, warp * kTXW, emit, kr, kr + K, lane, a.ny);
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

  // walk: STEPS planes per barrier; iteration j uses buffers (j & 1) * STEPS + s,
  // rewritten at iteration j + 2 after the barrier of iteration j + 1
  // carry split: planes of the slab's first half (the backprojector's slab
  // of twice the count that starts at zbeg); the slab-local transmission at
  // the middle goes straight into its carry slot, where the merge adds the
  // transmission of the slabs before (after the cluster barrier, which
  // orders these writes before the merge's reads)
  const bool split = ATT && a.carry_out && a.carry_split;
  const int zhalf = (a.nz + 2 * nslabs - 1) / (2 * nslabs);
  const int cslabs = split ? 2 * nslabs : nslabs;  // slabs of the carries
  const size_t cstride = static_cast<size_t>(a.nx) * a.cy;
  auto carry_at = [&](int o, int slot) {  // carry of output column o in `slot`
    return a.carry_out + a.row0 + yb + (static_cast<size_t>(cam) * (cslabs + 1) * a.nx + x0 + o) * a.cy +
           static_cast<size_t>(slot) * cstride;
  };
  auto stash_mid = [&]() {
#pragma unroll
    for (int i = 0; i < kTXW; ++i) {
      const int o = warp * kTXW + i;
      if (x0 + o < a.nx && yok && lane_writes(a, yb))
        *reinterpret_cast<float4*>(carry_at(o, 2 * slab + 1)) = kval(T[i], &cT[SCOMP ? 0 : i], 0, i);
    }
  };
  auto walk = [&](auto mode) {
    constexpr int MODE = decltype(mode)::value;
    const int n = zend - zbeg;
    for (int k = 0; k < n; k += STEPS) {
      const int base = ((k / STEPS) & 1) * STEPS;
#pragma unroll
      for (int s = 0; s < STEPS; ++s)
        if (k + s < n) produce(MODE == 0 ? zbeg + k + s : zend - 1 - k - s, base + s);
      __syncthreads();
#pragma unroll
      for (int s = 0; s < STEPS; ++s) {
        if (k + s < n) consume(MODE == 0 ? zbeg + k + s : zend - 1 - k - s, base + s, mode);
        if (MODE == 0 && split && k + s + 1 == zhalf) stash_mid();
      }
    }
    if (MODE == 0 && split && n < zhalf) stash_mid();  // the half ends past the volume
  };
  walk(std::integral_constant<int, 0>());

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
        if (KAHAN) cT[SCOMP ? 0 : i] = make_float4(0.f, 0.f, 0.f, 0.f);
        kclear(0, i);
        kclear(2, i);
      }
      walk(std::integral_constant<int, 1>());
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) {
        Q[i] = mul4(kval(Q[i], nullptr, 2, i), exp_neg4(kval(T[i], &cT[SCOMP ? 0 : i], 0, i)));
        kclear(2, i);
      }
    }
  }

  // cluster merge of the depth slabs (the shared tile is free after this barrier)
  __syncthreads();
  float4* sT = sb;                // [kTXC][32]
  float4* sP = sb + kTXC * 32;    // [kTXC][32]
  float4* sQ = sb + 2 * kTXC * 32;  // [kTXC][32] (PAIR)
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    sT[(warp * kTXW + i) * 32 + lane] = kval(T[i], &cT[SCOMP ? 0 : i], 0, i);
    sP[(warp * kTXW + i) * 32 + lane] = kval(P[i], &cP[SCOMP ? 0 : i], 1, i);
    if (PAIR && paired) sQ[(warp * kTXW + i) * 32 + lane] = kval(Q[i], nullptr, 2, i);
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
  // transmission carries for the backprojector (a.carry_out): the exclusive
  // prefix of the slab sums at every slab, then the column total
  const bool carry = ATT && a.carry_out;
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
        if (carry) {
          *reinterpret_cast<float4*>(carry_at(o, split ? 2 * s : s)) = Tt;
          if (split) {  // slab s's mid-slab transmission, from its CTA
            float4* m = reinterpret_cast<float4*>(carry_at(o, 2 * s + 1));
            float4 mid = Tt;
            add4(mid, __ldcg(m));
            *m = mid;
          }
        }
        fma4(Pt, exp_neg4(Tt), ps);
        add4(Tt, rT[o * 32 + lane]);
      } else {
        add4(Pt, ps);
      }
    }
    if (carry) *reinterpret_cast<float4*>(carry_at(o, cslabs)) = Tt;
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
}  // namespace nrgb
