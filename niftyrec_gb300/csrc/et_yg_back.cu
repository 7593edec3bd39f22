// Fused y-gantry backprojector: transmission carries, spread (reference and
// exact-transpose forms, mirror units), inverse-rotation gather and the
// two-stream pipeline over camera groups.
#include "et_yg_device.cuh"

namespace nrgb {
namespace {

// ------------------------------------------------ backprojector: slab carry
// carry[c][s][x][y] (s < a.bslabs) = sum of the rotated mu over the depth
// slabs before s (exclusive prefix): the transmission a depth slab starts
// from; carry[c][a.bslabs][x][y] = the whole column's sum.  One block row per
// camera c, or with a.units per unit (its first camera c; a mirror camera's
// transmissions are c's read from the other end); one warp per depth slab.
template <class V>
__global__ void __launch_bounds__(32 * kSlabsB) k_mu_carry_yg(const YgArgs a, int u0) {
  constexpr int C = kCarryCols;
  constexpr bool KAHAN = StorageTraits<V>::kKahan;
  const V* __restrict__ mu = reinterpret_cast<const V*>(a.mu) + a.row0;
  __shared__ Tap s_tap[kSlabsB][C];
  __shared__ float4 s_sum[kSlabsB][C][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunk = (a.nx + C - 1) / C;
  const int unit = u0 + blockIdx.x / nchunk;
  const int cam = a.units ? a.units[unit].x : unit;
  const int x0 = (blockIdx.x % nchunk) * C;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const CamRows cr = cam_rows(a.geom[cam].fwd);
  const int nsl = a.bslabs, slots = nsl + 1;
  const int zper = (a.nz + nsl - 1) / nsl;
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
    float* dst = a.slab_T + ((static_cast<size_t>(cam) * slots + warp) * a.nx + x) * a.cy + a.row0 + yb;
    *reinterpret_cast<float4*>(dst) = pre;
    if (warp == nsl - 1) {  // the column total, one slot further
      add4(pre, s_sum[warp][i][lane]);
      *reinterpret_cast<float4*>(dst + static_cast<size_t>(a.nx) * a.cy) = pre;
    }
  }
}

// ---------------------------------------- backprojector: spread + PSF
// temp[g][z][x][y] = PSF_z( s(x', y) * exp(-T_z(x', y)) ) for camera c0+g,
// T inclusive (emission-lib/_et_line_backproject_attenuated.cpp:24-34), PSF
// as in the projector.  CTA = (camera, x-tile, depth slab); every sampled
// column starts its transmission from the slab carry.
// ADJ: the exact transpose of the projector instead (not in the reference):
// the PSF taps are flipped (correlation) and each output column is scattered
// with the projector's own bilinear weights into the accumulator a.out
// (vector reductions; all cameras in one launch, no scratch), or, with
// a.det, written to the group scratch like the reference form for the
// transposed gather k_tgather_yg (a fixed summation order).
// CTAS: CTAs per SM the kernel is compiled for (3 where three tiles fit in
// shared memory, for the float32 reference spread; else 2).
// PTAB: the separated PSF comes from the kernel-parameter table `ptab`
// ([nz][2K]) instead of a shared-memory copy of the slab's planes.
template <int R, bool PSF, bool ATT, bool ADJ, class V, bool PTAB>
__device__ __forceinline__ void spread_body(const YgArgs& a, int c0, const float* ptab) {
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
  const int nsl = a.bslabs, slots = nsl + 1;
  const int slab = blockIdx.x % nsl;
  const int item = blockIdx.x / nsl;
  const int g = item / ntile;
  const int cam = c0 + g;
  const int x0 = (item % ntile) * kTXC;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const int zper = (a.nz + nsl - 1) / nsl;
  const int zbeg = slab * zper, zend = min(a.nz, zbeg + zper);
  if (zbeg >= zend) return;  // uniform over the CTA
  if (PSF && !PTAB) {  // this slab's planes only
    for (int i = zbeg * 2 * K + threadIdx.x; i < zend * 2 * K; i += blockDim.x) {
      const int j = i % (2 * K), base = i - j;
      // transpose of a convolution = correlation: reverse each kernel
      const int src = !ADJ ? i : (j < K ? base + (K - 1 - j) : base + K + (2 * K - 1 - j));
      s_psf[i] = __ldg(a.psf + src);
    }
  }
  const CamRows cr = cam_rows(a.geom[cam].fwd);
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * a.cs;  // one scratch volume
  const bool scatter = ADJ && !a.det;  // uniform over the launch
  float* __restrict__ tmp = scatter ? a.out + a.row0 : a.temp + vol * g;
  const float* __restrict__ srow = a.sino + static_cast<size_t>(cam) * a.nx * a.cy + a.row0;

  float4 Tc[TS::kOwn], cTc[TS::kOwn];  // transmission per sampled column (+ Kahan compensation)
#pragma unroll
  for (int k = 0; k < TS::kOwn; ++k) {
    Tc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    cTc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int xp = x0 - R + warp + kW * k;
    if (ATT && warp + kW * k < NS && xp >= 0 && xp < a.nx && yok)
      Tc[k] = ldg4(a.slab_T + ((static_cast<size_t>(cam) * slots + slab) * a.nx + xp) * a.cy + a.row0 + yb);
  }
  ybuf_zero_pads();
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
      if (scatter) {
        // halo rows lack part of their PSF support: their owner window adds them
        if (lane_writes(a, yb)) scatter4(tmp, tb[tap_slot<R>(warp * kTXW + i + R)], yb, v);
      } else {
        *reinterpret_cast<float4*>(tmp + (static_cast<size_t>(z) * a.nx + x) * a.cs + yb) = v;
      }
    };
    if (PSF) {
      if constexpr (PTAB && ADJ) {  // transpose of a convolution = correlation: both kernels reversed
        const float* kr = ptab + z * 2 * K;
        rowpass_from_tile<R>(sbuf, warp * kTXW, emit, Reversed<R>{kr}, Reversed<R>{kr + K}, lane, a.ny);
      } else {
        const float* kr = (PTAB ? ptab : s_psf) + z * 2 * K;
        rowpass_from_tile<R>(sbuf, warp * kTXW, emit, kr, kr + K, lane, a.ny);
      }
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) emit(i, sbuf[(warp * kTXW + i) * 32 + lane]);
    }
  }
}

template <int R, bool PSF, bool ATT, bool ADJ, class V, int CTAS = 2>
__global__ void __launch_bounds__(32 * kW, CTAS) k_spread_yg(const YgArgs a, int c0) {
  spread_body<R, PSF, ATT, ADJ, V, false>(a, c0, nullptr);
}

template <int R, bool ATT, bool ADJ, class V, int CTAS = 2>
__global__ void __launch_bounds__(32 * kW, CTAS)
    k_spread_ptab_yg(const YgArgs a, int c0, const __grid_constant__ PsfTable t) {
  spread_body<R, true, ATT, ADJ, V, true>(a, c0, t.c);
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
//
// ADJ: the exact transpose of the mirror-unit projector instead: both terms in
// c's frame go through the transposed PSF (camera: both kernels reversed;
// mate: row kernel forward, column kernel reversed) and, summed, are
// scattered with c's bilinear weights into the accumulator a.out (the mate's
// footprint of its mirrored column is c's), or with a.det written to the
// group scratch for k_tgather_yg.
//
// V = bfloat16 (mu stored in bfloat16): the forward transmission is summed
// with Kahan compensation (the compensation of each sampled column in shared
// memory), the mate's transmission is the column total minus the compensated
// forward sum (no second running sum), and the tiles are single-buffered (a
// second barrier per plane) so that two CTAs per SM still fit.
template <int R, class V>
__host__ __device__ constexpr size_t spread_pair_fixed_smem() {
  using TS = TileShape<R>;
  constexpr bool KAHAN = StorageTraits<V>::kKahan;
  return (KAHAN ? 1 : 2) * TS::kSbBytes + TS::kTapBytes + (KAHAN ? sizeof(float4) * TS::kOwn * 32 * kW : 0);
}

template <int R, bool PSF, bool ATT, bool ADJ, bool PTAB, class V = float>
__device__ __forceinline__ void spread_pair_body(const YgArgs& a, int u0, const float* ptab) {
  using TS = TileShape<R>;
  constexpr bool KAHAN = StorageTraits<V>::kKahan;
  constexpr int NB = KAHAN ? 1 : 2;  // tile buffers
  constexpr int NS = TS::NS;
  constexpr int K = 2 * R + 1;
  const V* __restrict__ mu = reinterpret_cast<const V*>(a.mu) + a.row0;
  extern __shared__ __align__(16) unsigned char smem[];
  float4* sb = reinterpret_cast<float4*>(smem);                              // [NB stages][2][NS][32]
  Tap* taps = reinterpret_cast<Tap*>(smem + NB * TS::kSbBytes);               // [2][kTapSlots]
  float4* scomp = reinterpret_cast<float4*>(smem + NB * TS::kSbBytes + TS::kTapBytes);  // [kOwn][256] (KAHAN)
  float* s_psf = reinterpret_cast<float*>(smem + spread_pair_fixed_smem<R, V>());  // [zper][2K], mate's next

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int nsl = a.bslabs, slots = nsl + 1;
  const int slab = blockIdx.x % nsl;
  const int item = blockIdx.x / nsl;
  const int g = item / ntile;
  const int unit = u0 + g;
  const int2 uc = a.units[unit];
  const int cam = uc.x, mate = uc.y;
  const bool paired = mate >= 0;  // uniform over the CTA
  const int x0 = (item % ntile) * kTXC;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const int zper = (a.nz + nsl - 1) / nsl;
  const int zbeg = slab * zper, zend = min(a.nz, zbeg + zper);
  if (zbeg >= zend) return;  // uniform over the CTA
  float* s_psf_m = s_psf + zper * 2 * K;
  if (PSF && !PTAB) {
    // reversed index of a row (j < K) or column (j >= K) kernel entry
    auto rev = [&](int j) { return j < K ? K - 1 - j : 3 * K - 1 - j; };
    for (int i = threadIdx.x; i < (zend - zbeg) * 2 * K; i += blockDim.x) {
      const int z = zbeg + i / (2 * K), j = i % (2 * K);
      s_psf[i] = __ldg(a.psf + z * 2 * K + (ADJ ? rev(j) : j));
      if (paired) {  // mate: reference row reversed; transpose column reversed
        const int jm = (j < K) != ADJ ? rev(j) : j;
        s_psf_m[i] = __ldg(a.psf + (a.nz - 1 - z) * 2 * K + jm);
      }
    }
  }
  const CamRows cr = cam_rows(a.geom[cam].fwd);
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * a.cs;  // one scratch volume
  const bool scatter = ADJ && !a.det;  // uniform over the launch
  float* __restrict__ tmp = scatter ? a.out + a.row0 : a.temp + vol * g;
  const float* __restrict__ srow = a.sino + static_cast<size_t>(cam) * a.nx * a.cy + a.row0;
  const float* __restrict__ mrow = a.sino + static_cast<size_t>(paired ? mate : cam) * a.nx * a.cy + a.row0;

  // transmissions per sampled column: forward (from the slab carry) and, for
  // the mate, from the far end (column total minus the carry; with KAHAN Tr
  // holds the column total)
  float4 Tc[TS::kOwn], Tr[TS::kOwn];
#pragma unroll
  for (int k = 0; k < TS::kOwn; ++k) {
    Tc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    Tr[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (KAHAN) scomp[k * 32 * kW + threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int xp = x0 - R + warp + kW * k;
    if (ATT && warp + kW * k < NS && xp >= 0 && xp < a.nx && yok) {
      const float* cp = a.slab_T + ((static_cast<size_t>(cam) * slots + slab) * a.nx + xp) * a.cy + a.row0 + yb;
      Tc[k] = ldg4(cp);
      if (paired) {
        const float4 tot = ldg4(cp + static_cast<size_t>(nsl - slab) * a.nx * a.cy);
        Tr[k] = KAHAN ? tot : make_float4(tot.x - Tc[k].x, tot.y - Tc[k].y, tot.z - Tc[k].z, tot.w - Tc[k].w);
      }
    }
  }
  ybuf_zero_pads();
  __syncthreads();

  for (int z = zbeg; z < zend; ++z) {
    const int b = z & 1;
    float4* sc = sb + (NB == 2 ? b : 0) * 2 * NS * 32;
    float4* sm = sc + NS * 32;
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
        const bool ok = xp >= 0 && xp < a.nx && yok;
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f), q = s;
        if (ok) s = ldg4(srow + static_cast<size_t>(xp) * a.cy + yb);
        if (paired && ok) q = ldg4(mrow + static_cast<size_t>(a.nx - 1 - xp) * a.cy + yb);
        if (ATT) {
          const float4 m = sample4(mu, tb[tap_slot<R>(c)], yb, yok);
          if constexpr (KAHAN) {
            float4 cc = scomp[k * 32 * kW + threadIdx.x];
            kahan_add4p(Tc[k], cc, m);
            scomp[k * 32 * kW + threadIdx.x] = cc;
            const float4 tv = kahan_value4p(Tc[k], cc);
            s = mul4p(s, exp_neg4(tv));
            if (paired) {  // sum from the far end, inclusive: total - forward sum + this plane
              const Pair4 tot = pair4(Tr[k]), v = pair4(tv), mm = pair4(m);
              q = mul4p(q, exp_neg4(unpair4({add2(sub2(tot.lo, v.lo), mm.lo), add2(sub2(tot.hi, v.hi), mm.hi)})));
            }
          } else {
            add4p(Tc[k], m);
            s = mul4p(s, exp_neg4(Tc[k]));
            if (paired) {
              q = mul4p(q, exp_neg4(Tr[k]));
              const Pair4 tr = pair4(Tr[k]), mm = pair4(m);
              Tr[k] = unpair4({sub2(tr.lo, mm.lo), sub2(tr.hi, mm.hi)});
            }
          }
        }
        sc[c * 32 + lane] = s;
        if (paired) sm[c * 32 + lane] = q;
      }
    }
    __syncthreads();
    auto write = [&](int i, const float4& v) {
      const int x = x0 + warp * kTXW + i;
      if (x >= a.nx || !yok) return;
      if (scatter) {
        // halo rows lack part of their PSF support: their owner window adds them
        if (lane_writes(a, yb)) scatter4(tmp, tb[tap_slot<R>(warp * kTXW + i + R)], yb, v);
      } else {
        *reinterpret_cast<float4*>(tmp + (static_cast<size_t>(z) * a.nx + x) * a.cs + yb) = v;
      }
    };
    float4 pend;  // the mate's term of the output being written
    auto keep = [&](int i, const float4& v) { pend = v; };
    auto write_sum = [&](int i, float4 v) {
      add4p(v, pend);
      write(i, v);
    };
    if (PSF) {
      const float* kr = PTAB ? ptab + z * 2 * K : s_psf + (z - zbeg) * 2 * K;
      if (paired) {  // both row passes in one sweep over the two tiles
        if constexpr (PTAB && ADJ) {
          const float* km = ptab + (a.nz - 1 - z) * 2 * K;
          rowpass2_from_tiles<R>(sc, sm, warp * kTXW, write_sum, Reversed<R>{kr}, Reversed<R>{kr + K}, keep, km,
                                 Reversed<R>{km + K}, lane, a.ny);
        } else if constexpr (PTAB) {
          const float* km = ptab + (a.nz - 1 - z) * 2 * K;
          rowpass2_from_tiles<R>(sc, sm, warp * kTXW, write_sum, kr, kr + K, keep, Reversed<R>{km}, km + K, lane,
                                 a.ny);
        } else {
          const float* km = s_psf_m + (z - zbeg) * 2 * K;
          rowpass2_from_tiles<R>(sc, sm, warp * kTXW, write_sum, kr, kr + K, keep, km, km + K, lane, a.ny);
        }
      } else if constexpr (PTAB && ADJ) {
        rowpass_from_tile<R>(sc, warp * kTXW, write, Reversed<R>{kr}, Reversed<R>{kr + K}, lane, a.ny);
      } else {
        rowpass_from_tile<R>(sc, warp * kTXW, write, kr, kr + K, lane, a.ny);
      }
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) {
        float4 v = sc[(warp * kTXW + i) * 32 + lane];
        if (paired) add4(v, sm[(warp * kTXW + i) * 32 + lane]);
        write(i, v);
      }
    }
    if (NB == 1) __syncthreads();  // the single tile buffer is rewritten next plane
  }
}

template <int R, bool PSF, bool ATT, bool ADJ, class V = float>
__global__ void __launch_bounds__(32 * kW, 2) k_spread_pair_yg(const YgArgs a, int u0) {
  spread_pair_body<R, PSF, ATT, ADJ, false, V>(a, u0, nullptr);
}

template <int R, bool ATT, bool ADJ, class V = float>
__global__ void __launch_bounds__(32 * kW, 2)
    k_spread_pair_ptab_yg(const YgArgs a, int u0, const __grid_constant__ PsfTable t) {
  spread_pair_body<R, true, ATT, ADJ, true, V>(a, u0, t.c);
}

// ------------------------------------ backprojector: inverse-rotation gather
// out[Z][X][y] (+)= sum_g bilinear(temp[g], B_g * (X, y, Z)) with B_g the
// camera's inverse matrix (ZYX order, -theta), emission-lib/_et.cpp:474-497.
// With a.units, g runs over units and B_g is the unit's first camera's.
// first: assign instead of adding to a.out; clamp: the last group of the
// window with a.truncate -- negative sums become zero as they are stored.
template <int U>
__global__ void __launch_bounds__(32 * kGatherWarps) k_gather_yg(const YgArgs a, int c0, int gcount, int first,
                                                                int clamp) {
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
  // camera share footprint columns, which then hit in L1; the loads of U
  // units' volumes in flight at once (every footprint offset is inside its
  // volume, see make_tap), added in unit order
  float4 acc[C];
#pragma unroll
  for (int i = 0; i < C; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  int g = 0;
  for (; g + U <= gcount; g += U) {
    float4 v[U][C];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int i = 0; i < C; ++i) v[u][i] = sample4_loaded(a.temp + vol * (g + u), tap[(g + u) * C + i], yb);
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int i = 0; i < C; ++i) add4(acc[i], v[u][i]);
  }
  for (; g < gcount; ++g) {
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
    if (clamp) acc[i] = clamp0(acc[i]);
    *dst = acc[i];
  }
}

// Forward bilinear weight of corner (X, Z) in the footprint of rotated column
// (xp, zp) (0 when (X, Z) is not one of its corners): make_tap's position,
// floor, relative and basis arithmetic, and its product for that corner, so
// the weight equals the one the scatter of the atomic form applies.
__device__ __forceinline__ float corner_weight(int xp, int zp, const CamRows& cr, int X, int Z) {
  const float fx = static_cast<float>(xp), fz = static_cast<float>(zp);
  const float px = fa(fa(fm(cr.m00, fx), fm(cr.m02, fz)), cr.m03);
  const float pz = fa(fa(fm(cr.m20, fx), fm(cr.m22, fz)), cr.m23);
  const int xs = static_cast<int>(floorf(px));
  const int zs = static_cast<int>(floorf(pz));
  if ((X != xs && X != xs + 1) || (Z != zs && Z != zs + 1)) return 0.0f;
  float rx = __fsub_rn(px, static_cast<float>(xs));
  float rz = __fsub_rn(pz, static_cast<float>(zs));
  if (rx < 0.0f) rx = 0.0f;
  if (rz < 0.0f) rz = 0.0f;
  const float wx = X == xs ? __fsub_rn(1.0f, rx) : rx;
  const float wz = Z == zs ? __fsub_rn(1.0f, rz) : rz;
  return wx * wz;
}

// Deterministic transposed gather: out[Z][X][y] (+)= sum over the group's
// units g (camera order) and over the rotated columns (x', z') whose forward
// footprint has (X, Z) as a corner, of that corner's weight times
// scratch_g[z'][x'][y] -- the transpose of the projector's bilinear sampling
// without vector reductions.  The forward rows are a rotation, so those
// columns lie within sqrt(2) of the inverse image of (X, Z): inside the 4 x 4
// integer box around it.  Lane l evaluates box candidate l % 16 of output
// column X0 + l / 16; the nonzero weights are then added in lane order.
__global__ void __launch_bounds__(32 * kGatherWarps) k_tgather_yg(const YgArgs a, int c0, int gcount, int first,
                                                                  int clamp) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunk = (a.nx + 1) / 2;
  const int item = blockIdx.x * kGatherWarps + warp;
  if (item >= nchunk * a.nz) return;
  const int Z = item / nchunk;
  const int X0 = (item % nchunk) * 2;
  const int yb = lane * 4;
  const bool rows = lane_rows_ok(a, yb) && lane_writes(a, yb);
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * a.cs;
  const int X = X0 + (lane >> 4);
  const int bx = (lane & 3) - 1, bz = ((lane >> 2) & 3) - 1;
  float4 acc[2] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
  for (int g = 0; g < gcount; ++g) {
    const CamRows cr = cam_rows(a.geom[a.units ? a.units[c0 + g].x : c0 + g].fwd);
    float w = 0.0f;
    int off = 0;
    if (X < a.nx) {
      const float det = cr.m00 * cr.m22 - cr.m02 * cr.m20;
      const float dx = static_cast<float>(X) - cr.m03, dz = static_cast<float>(Z) - cr.m23;
      const int xp = static_cast<int>(floorf((cr.m22 * dx - cr.m02 * dz) / det)) + bx;
      const int zp = static_cast<int>(floorf((cr.m00 * dz - cr.m20 * dx) / det)) + bz;
      if (xp >= 0 && xp < a.nx && zp >= 0 && zp < a.nz) {
        w = corner_weight(xp, zp, cr, X, Z);
        off = (zp * a.nx + xp) * a.cs;
      }
    }
    const float* src = a.temp + vol * g + (rows ? yb : 0);
    // the nonzero weights four at a time: their loads in flight together,
    // then the terms added in lane order
    for (unsigned m = __ballot_sync(kFull, w != 0.0f); m;) {
      int l[4];
      float wl[4];
      float4 v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        l[q] = m ? __ffs(m) - 1 : -1;  // uniform: from the ballot
        m &= m ? m - 1 : 0u;
        const int src_lane = l[q] < 0 ? 0 : l[q];
        wl[q] = __shfl_sync(kFull, w, src_lane);
        const int ol = __shfl_sync(kFull, off, src_lane);  // an offset inside the volume
        v[q] = ldg4(src + ol);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (l[q] < 0) break;
        const float4 wv = make_float4(wl[q] * v[q].x, wl[q] * v[q].y, wl[q] * v[q].z, wl[q] * v[q].w);
        if (l[q] < 16)
          add4(acc[0], wv);
        else
          add4(acc[1], wv);
      }
    }
  }
  if (!rows) return;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int Xo = X0 + i;
    if (Xo >= a.nx) continue;
    float4* dst = reinterpret_cast<float4*>(a.out + (static_cast<size_t>(Z) * a.nx + Xo) * a.cy + a.row0 + yb);
    if (!first) add4(acc[i], *dst);
    if (clamp) acc[i] = clamp0(acc[i]);
    *dst = acc[i];
  }
}

// clamp: this is the window's last group and the result is truncated
void launch_tgather(const YgArgs& b, int c0, int gcount, int clamp, cudaStream_t st) {
  const int blocks = ((b.nx + 1) / 2 * b.nz + kGatherWarps - 1) / kGatherWarps;
  NRGB_LAUNCH_SCOPE("k_tgather_yg", st);
  k_tgather_yg<<<blocks, 32 * kGatherWarps, 0, st>>>(b, c0, gcount, c0 == 0 ? 1 : 0, clamp);
}

void launch_gather(const YgArgs& b, int c0, int gcount, int clamp, int blocks, size_t smem, cudaStream_t st) {
  NRGB_LAUNCH_SCOPE("k_gather_yg", st);
  k_gather_yg<kGatherUnits><<<blocks, 32 * kGatherWarps, smem, st>>>(b, c0, gcount, c0 == 0 ? 1 : 0, clamp);
}

// The separated PSF of a.nz planes as a kernel-parameter table, or null when
// it is not available on the host or does not fit.
template <int R>
const PsfTable* psf_table(const YgArgs& a) {
  if (!a.psf || !a.psf_host || static_cast<size_t>(a.nz) * 2 * (2 * R + 1) > kPsfTableFloats) return nullptr;
  static thread_local PsfTable table;
  std::memcpy(table.c, a.psf_host, sizeof(float) * a.nz * 2 * (2 * R + 1));
  return &table;
}

template <int R, bool ADJ>
int launch_spread_R(const YgArgs& a, int c0, int gcount, cudaStream_t st) {
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const dim3 grid(gcount * ntile * a.bslabs), block(32 * kW);
  const bool psf = a.psf != nullptr;
  const PsfTable* tab = psf_table<R>(a);
  const size_t smem = tile_smem_bytes<R>(psf && !tab ? a.nz : 0);
  auto go = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE(ADJ ? "k_adjoint_yg" : "k_spread_yg", st);
    k<<<grid, block, smem, st>>>(a, c0);
  };
  auto go_tab = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE(ADJ ? "k_adjoint_yg" : "k_spread_yg", st);
    k<<<grid, block, smem, st>>>(a, c0, *tab);
  };
  // only mu is sampled from storage here (the sinogram is float32)
  const bool bf16 = a.storage == kStorageBF16;
  const bool three = 3 * (smem + kYBufBytes + 1024) <= 228 * 1024;
  if (psf && tab) {
    if (a.mu && bf16) {
      go_tab(k_spread_ptab_yg<R, true, ADJ, __nv_bfloat16>);
    } else if (a.mu) {
      if constexpr (!ADJ) {
        if (three)
          go_tab(k_spread_ptab_yg<R, true, false, float, 3>);
        else
          go_tab(k_spread_ptab_yg<R, true, false, float>);
      } else {
        go_tab(k_spread_ptab_yg<R, true, true, float>);
      }
    } else {
      go_tab(k_spread_ptab_yg<R, false, ADJ, float>);
    }
  } else if (psf) {
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

template <int R, bool ADJ>
int launch_spread_pair_R(const YgArgs& a, int u0, int gcount, cudaStream_t st) {
  using TS = TileShape<R>;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const dim3 grid(gcount * ntile * a.bslabs), block(32 * kW);
  const bool psf = a.psf != nullptr;
  const int zper = (a.nz + a.bslabs - 1) / a.bslabs;
  const PsfTable* tab = psf_table<R>(a);
  // bfloat16 mu: the Kahan form (reference mode only)
  const bool bf16 = a.storage == kStorageBF16 && a.mu && !ADJ;
  const size_t smem = (bf16 ? spread_pair_fixed_smem<R, __nv_bfloat16>() : spread_pair_fixed_smem<R, float>()) +
                      (psf && !tab ? sizeof(float) * 2 * zper * 2 * (2 * R + 1) : 0);
  auto go = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE(ADJ ? "k_adjoint_pair_yg" : "k_spread_pair_yg", st);
    k<<<grid, block, smem, st>>>(a, u0);
  };
  auto go_tab = [&](auto k) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE(ADJ ? "k_adjoint_pair_yg" : "k_spread_pair_yg", st);
    k<<<grid, block, smem, st>>>(a, u0, *tab);
  };
  if constexpr (!ADJ) {
    if (bf16) {
      if (psf && tab) go_tab(k_spread_pair_ptab_yg<R, true, false, __nv_bfloat16>);
      else if (psf) go(k_spread_pair_yg<R, true, true, false, __nv_bfloat16>);
      else go(k_spread_pair_yg<0, false, true, false, __nv_bfloat16>);
      return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
    }
  }
  if (psf && tab) {
    if (a.mu) go_tab(k_spread_pair_ptab_yg<R, true, ADJ>);
    else go_tab(k_spread_pair_ptab_yg<R, false, ADJ>);
  } else if (psf) {
    if (a.mu) go(k_spread_pair_yg<R, true, true, ADJ>);
    else go(k_spread_pair_yg<R, true, false, ADJ>);
  } else {
    if (a.mu) go(k_spread_pair_yg<0, false, true, ADJ>);
    else go(k_spread_pair_yg<0, false, false, ADJ>);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

template <bool ADJ>
int spread_pair_by_radius(int R, const YgArgs& a, int u0, int gcount, cudaStream_t st) {
  switch (R) {
    case 0: return launch_spread_pair_R<0, ADJ>(a, u0, gcount, st);
    case 1: return launch_spread_pair_R<1, ADJ>(a, u0, gcount, st);
    case 2: return launch_spread_pair_R<2, ADJ>(a, u0, gcount, st);
    case 3: return launch_spread_pair_R<3, ADJ>(a, u0, gcount, st);
    case 4: return launch_spread_pair_R<4, ADJ>(a, u0, gcount, st);
    case 5: return launch_spread_pair_R<5, ADJ>(a, u0, gcount, st);
    case 6: return launch_spread_pair_R<6, ADJ>(a, u0, gcount, st);
    case 7: return launch_spread_pair_R<7, ADJ>(a, u0, gcount, st);
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

int yg_even_group(int n, int group) {
  group = std::max(1, std::min(group, n));
  const int ngroups = (n + group - 1) / group;
  return (n + ngroups - 1) / ngroups;
}

size_t yg_backproject_workspace(int nx, int ny, int nz, int ncam, int group, int slots) {
  const size_t cy = round_up(ny, 4);
  const size_t vol = static_cast<size_t>(nz) * nx * scratch_rows(ny);  // one window's scratch volume
  const size_t slabs = static_cast<size_t>(ncam) * kCarrySlots * nx * cy;  // at most kSlabsB slabs
  // with two slots the spread of group g+1 overlaps the gather of group g
  return sizeof(float) * (slabs + static_cast<size_t>(slots) * vol * std::max(1, std::min(group, ncam)));
}

size_t yg_gradient_workspace(int nx, int ny, int nz, int ncam, int group, int slots) {
  const size_t vol = static_cast<size_t>(nz) * nx * scratch_rows(ny);
  return sizeof(float) * static_cast<size_t>(slots) * vol * std::max(1, std::min(group, ncam));
}

int yg_carry_slabs() { return kCarrySlots; }

namespace {

// Carries of units (or cameras) [u0, u0 + n).
int mu_carry_range(const YgArgs& a_in, float* out, int u0, int n, cudaStream_t st) {
  const int nchunk = (a_in.nx + kCarryCols - 1) / kCarryCols;
  for (const Window& w : row_windows(a_in.ny, 0)) {  // carries need no halo
    YgArgs a = windowed(a_in, w);
    a.slab_T = out;
    NRGB_LAUNCH_SCOPE("k_mu_carry_yg", st);
    if (a.storage == kStorageBF16)
      k_mu_carry_yg<__nv_bfloat16><<<n * nchunk, 32 * a.bslabs, 0, st>>>(a, u0);
    else
      k_mu_carry_yg<float><<<n * nchunk, 32 * a.bslabs, 0, st>>>(a, u0);
  }
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

}  // namespace

int yg_mu_carry(const YgArgs& a, float* out, cudaStream_t st) {
  return mu_carry_range(a, out, 0, a.units ? a.nunits : a.ncam, st);
}

namespace {

// Second stream and events of the backprojection pipeline, one set per
// device; `mu` makes each call's event records and waits one sequence (calls
// from several host threads, e.g. plans on their own streams).
struct Pipe {
  std::mutex mu;
  cudaStream_t aux = nullptr, aux2 = nullptr;
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
    if (cudaStreamCreateWithFlags(&p.aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p.aux2, cudaStreamNonBlocking) != cudaSuccess)
      return nullptr;
    cudaEvent_t* evs[] = {&p.fork, &p.join, &p.spread_done[0], &p.spread_done[1], &p.gather_done[0],
                          &p.gather_done[1]};
    for (cudaEvent_t* e : evs)
      if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
  }
  return &p;
}

}  // namespace

void yg_tgather(const YgArgs& a, int c0, int gcount, int clamp, cudaStream_t st) {
  launch_tgather(a, c0, gcount, clamp, st);
}

// Per row window and camera group: step g (over all windows' groups) uses
// scratch slot g % 2 and spreads on the caller's stream (even g) or a second
// spread stream (odd g), its gather following on a gather stream.  The
// spread of step g+1 thus starts while step g's last wave of CTAs drains (a
// 30-unit spread at 128^3 is 3.2 waves on 152 SMs) and runs beside the
// gather of step g; a slot is spread again only after its gather.
int yg_backproject(const YgArgs& a_in, cudaStream_t st) {
  YgArgs a = a_in;
  if (a.bslabs < 1 || a.bslabs > kSlabsB) return kErrParameters;
  const int R = a.psf ? (a.psf_k - 1) / 2 : 0;
  // mirror units: float32 mu, or bfloat16 mu in reference mode
  const bool pair = !a.gradient && a.units && a.nunits > 0 &&
                    (a.storage != kStorageBF16 || a.back_mode != kBackAdjoint);
  if (!pair) {
    a.units = nullptr;
    a.nunits = 0;
  }
  const int nunits = pair ? a.nunits : a.ncam;  // scratch volumes to spread and gather
  // even groups of at most a.group units
  int group = yg_even_group(nunits, a.group);
  const std::vector<Window> wins = row_windows(a.ny, R);
  // work space: slab carries first (unless given), then the scratch slot(s)
  const size_t vol = static_cast<size_t>(a.nz) * a.nx * scratch_rows(a.ny);
  float* slot0;
  // carries of every unit first (computing group g+1's carries on the gather
  // stream while group g spreads measured no faster on GB300)
  if (a.gradient || a.carry || !a.mu) {  // carries given, or not needed
    a.slab_T = const_cast<float*>(a.carry);
    slot0 = a.work;
  } else {
    a.slab_T = a.work;
    slot0 = a.work + static_cast<size_t>(a.ncam) * (a.bslabs + 1) * a.nx * a.cy;
    int s = yg_mu_carry(a, a.slab_T, st);
    if (s != kOk) return s;
  }
  if (a.sino_ready) cudaStreamWaitEvent(st, static_cast<cudaEvent_t>(a.sino_ready), 0);
  a.group = group;
  // the exact transpose in its deterministic form: group scratch + transposed gather
  const bool tgather = a.back_mode == kBackAdjoint && !a.gradient && a.det;
  auto spread_on = [&](const YgArgs& b, int c0, int gcount, cudaStream_t ss) {
    if (a.gradient) return yg_grad_spread(b, c0, gcount, ss);
    if (tgather)
      return pair ? spread_pair_by_radius<true>(R, b, c0, gcount, ss) : spread_by_radius_t<true>(R, b, c0, gcount, ss);
    return pair ? spread_pair_by_radius<false>(R, b, c0, gcount, ss) : spread_by_radius(R, b, c0, gcount, ss);
  };
  // with a.truncate the window's last group clamps the result as it stores it
  auto gather_on = [&](const YgArgs& b, int c0, int gcount, int blocks, size_t smem, cudaStream_t gs) {
    const int clamp = a.truncate && c0 + gcount == nunits ? 1 : 0;
    if (tgather)
      launch_tgather(b, c0, gcount, clamp, gs);
    else
      launch_gather(b, c0, gcount, clamp, blocks, smem, gs);
  };
  auto spread = [&](const YgArgs& b, int c0, int gcount) { return spread_on(b, c0, gcount, st); };
  if (a.back_mode == kBackAdjoint && !a.gradient && !a.det) {
    // transpose of the projector: one launch per window over all cameras,
    // scattered straight into the zeroed accumulator
    const size_t full = static_cast<size_t>(a.nz) * a.nx * a.cy;
    if (cudaMemsetAsync(a.out, 0, sizeof(float) * full, st) != cudaSuccess) return kErrKernel;
    for (const Window& w : wins) {
      const int s = pair ? spread_pair_by_radius<true>(R, windowed(a, w), 0, nunits, st)
                         : spread_by_radius_t<true>(R, windowed(a, w), 0, a.ncam, st);
      if (s != kOk) return s;
    }
    return kOk;
  }
  const int nchunk = (a.nx + kGatherCols - 1) / kGatherCols;
  const int gblocks = (nchunk * a.nz + kGatherWarps - 1) / kGatherWarps;
  const size_t gsmem = sizeof(Tap) * kGatherWarps * kGatherCols * group;
  cudaFuncSetAttribute(k_gather_yg<kGatherUnits>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       static_cast<int>(gsmem));
  if (!a.pipelined) {
    for (const Window& w : wins) {
      YgArgs b = windowed(a, w);
      b.temp = slot0;
      for (int c0 = 0; c0 < nunits; c0 += group) {
        const int gcount = std::min(group, nunits - c0);
        int st_ = spread(b, c0, gcount);
        if (st_ != kOk) return st_;
        gather_on(b, c0, gcount, gblocks, gsmem, st);
      }
    }
    return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
  }
  Pipe* pp = pipe_for_current_device();
  if (!pp) return kErrUnspecified;
  std::lock_guard<std::mutex> pipe_lock(pp->mu);
  cudaEventRecord(pp->fork, st);
  cudaStreamWaitEvent(pp->aux, pp->fork, 0);
  cudaStreamWaitEvent(pp->aux2, pp->fork, 0);
  int gi = 0;
  for (const Window& w : wins) {
    YgArgs b = windowed(a, w);
    for (int c0 = 0; c0 < nunits; c0 += group, ++gi) {
      const int gcount = std::min(group, nunits - c0);
      const int slot = gi & 1;
      cudaStream_t ss = slot ? pp->aux2 : st;
      b.temp = slot0 + vol * group * slot;
      if (gi >= 2) cudaStreamWaitEvent(ss, pp->gather_done[slot], 0);
      int st_ = spread_on(b, c0, gcount, ss);
      if (st_ != kOk) return st_;
      cudaEventRecord(pp->spread_done[slot], ss);
      cudaStreamWaitEvent(pp->aux, pp->spread_done[slot], 0);
      gather_on(b, c0, gcount, gblocks, gsmem, pp->aux);
      cudaEventRecord(pp->gather_done[slot], pp->aux);
    }
  }
  cudaEventRecord(pp->join, pp->aux);
  cudaStreamWaitEvent(st, pp->join, 0);
  return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
}

}  // namespace nrgb
