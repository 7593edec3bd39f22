// Fused y-gantry form of the reference's attenuation gradient
// (et_array_gradient_attenuation; emission-lib/_et.cpp:1679-1924 with the
// scan of emission-lib_gpu/_et_attenuation_gradient_gpu_kernels.cu:15-42).
// Per camera, in the rotated frame (a, m: rotated activity and mu, T_z the
// inclusive depth sum of m, s the sinogram plane):
//   w(x, y, z) = s(x, y) * sum_{z' >= z} a_z' exp(-T_z'),
// then the per-plane PSF (as in the projector) and the inverse-rotation
// gather into the accumulator.  The gather and the camera-group pipeline are
// the reference-mode backprojector's; this file holds the spread that writes
// PSF(w) of a camera group into the scratch volumes.
//
// Work item as the projector's: a cluster of depth-slab CTAs per (camera,
// 32-column tile), every CTA owning the NS = 32 + 2R sampled columns its PSF
// needs.  Walk 1 sums the slab's local transmission T_s and partial
// P_s = sum a exp(-T_local) per sampled column; the cluster exchanges them
// through distributed shared memory, so slab s knows the transmission before
// it (Tb) and the weighted partials of the slabs after it
// (later = sum_{r > s} exp(-Tb_r) P_r).  Walk 2 runs from the slab's far end
// with the global transmission V = Tb + T_s (decremented by each plane's mu)
// and the suffix W = later + sum a exp(-V), so every term is added, none
// cancelled; s * W goes into the shared tile and the row / column passes of
// the plane write PSF(w) to the scratch.
#include "et_yg_device.cuh"

namespace nrgb {
namespace {

template <int R, bool PSF, bool PTAB>
__device__ __forceinline__ void grad_item(const YgArgs& a, int cam, int g, int x0, unsigned char* smem,
                                          const float* ptab) {
  using TS = TileShape<R>;
  constexpr int NS = TS::NS;
  constexpr int OWN = TS::kOwn;
  constexpr int K = 2 * R + 1;
  constexpr size_t kSb = TS::sb_bytes(false);
  static_assert(kSb >= sizeof(float4) * 2 * NS * 32, "the exchange needs two NS x 32 arrays");
  const float* __restrict__ act = a.act + a.row0;
  const float* __restrict__ mu = a.mu + a.row0;
  float4* sb = reinterpret_cast<float4*>(smem);                         // [2][NS][32]
  Tap* taps = reinterpret_cast<Tap*>(smem + kSb);                        // [2][kTapSlots]
  float* s_psf = reinterpret_cast<float*>(smem + kSb + TS::kTapBytes);   // [nz][2K]

  cg::cluster_group cluster = cg::this_cluster();
  const int slab = static_cast<int>(cluster.block_rank());
  const int nslabs = static_cast<int>(cluster.num_blocks());
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int yb = lane * 4;
  const bool yok = lane_rows_ok(a, yb);
  const int zper = (a.nz + nslabs - 1) / nslabs;
  const int zbeg = slab * zper, zend = min(a.nz, zbeg + zper);
  if (PSF && !PTAB)
    for (int i = zbeg * 2 * K + threadIdx.x; i < zend * 2 * K; i += blockDim.x) s_psf[i] = __ldg(a.psf + i);
  const CamRows cr = cam_rows(a.geom[cam].fwd);
  const float* __restrict__ srow = a.sino + static_cast<size_t>(cam) * a.nx * a.cy + a.row0;
  float* __restrict__ tmp = a.temp + static_cast<size_t>(a.nz) * a.nx * a.cs * g;

  // footprints of the columns this warp samples (c = warp + kW * k), shared
  // within the warp through buffer b of the tap slots
  auto footprints = [&](int z, int b) {
    Tap* tb = taps + b * TS::kTapSlots;
    if (lane < OWN) {
      const int c = warp + kW * lane;
      if (c < NS) {
        const int xp = x0 - R + c;
        tb[tap_slot<R>(c)] = make_tap(xp, z, cr.m00, cr.m02, cr.m03, cr.m20, cr.m22, cr.m23, a.nx, a.nz, a.cy,
                                      xp >= 0 && xp < a.nx);
      }
    }
    __syncwarp();
    return tb;
  };

  ybuf_zero_pads();  // ordered before walk 2 by the cluster barriers

  // walk 1: the slab's transmission and partial per sampled column
  float4 T[OWN], P[OWN];
#pragma unroll
  for (int k = 0; k < OWN; ++k) {
    T[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    P[k] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int z = zbeg; z < zend; ++z) {
    const Tap* tb = footprints(z, z & 1);
#pragma unroll
    for (int k = 0; k < OWN; ++k) {
      const int c = warp + kW * k;
      if (c < NS) {
        const Tap& t = tb[tap_slot<R>(c)];
        add4(T[k], sample4(mu, t, yb, yok));
        fma4(P[k], sample4(act, t, yb, yok), exp_neg4(T[k]));
      }
    }
  }

  // exchange through distributed shared memory (the tile region is unused so far)
  float4* sT = sb;
  float4* sP = sb + NS * 32;
#pragma unroll
  for (int k = 0; k < OWN; ++k) {
    const int c = warp + kW * k;
    if (c < NS) {
      sT[c * 32 + lane] = T[k];
      sP[c * 32 + lane] = P[k];
    }
  }
  cluster.sync();
  // V: global transmission at the slab's last plane; W: the suffix from the
  // slabs after this one
#pragma unroll
  for (int k = 0; k < OWN; ++k) {
    const int c = warp + kW * k;
    if (c >= NS) continue;
    float4 tacc = make_float4(0.f, 0.f, 0.f, 0.f), later = tacc, before = tacc;
    for (int s = 0; s < nslabs; ++s) {
      if (s == slab) before = tacc;
      if (s > slab) fma4(later, exp_neg4(tacc), cluster.map_shared_rank(sP, s)[c * 32 + lane]);
      add4(tacc, cluster.map_shared_rank(sT, s)[c * 32 + lane]);
    }
    add4(before, T[k]);
    T[k] = before;  // V
    P[k] = later;   // W
  }
  cluster.sync();  // every CTA's exchange reads are done before the tiles are rewritten

  // walk 2, from the slab's far end
  const int n = zend - zbeg;
  for (int j = 0; j < n; ++j) {
    const int z = zend - 1 - j;
    const int b = j & 1;
    float4* sbuf = sb + b * NS * 32;
    const Tap* tb = footprints(z, b);
#pragma unroll
    for (int k = 0; k < OWN; ++k) {
      const int c = warp + kW * k;
      if (c < NS) {
        const Tap& t = tb[tap_slot<R>(c)];
        const float4 m = sample4(mu, t, yb, yok);
        fma4(P[k], sample4(act, t, yb, yok), exp_neg4(T[k]));
        T[k] = make_float4(T[k].x - m.x, T[k].y - m.y, T[k].z - m.z, T[k].w - m.w);
        const int xp = x0 - R + c;
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        if (xp >= 0 && xp < a.nx && yok) s = ldg4(srow + static_cast<size_t>(xp) * a.cy + yb);
        sbuf[c * 32 + lane] = mul4(s, P[k]);
      }
    }
    __syncthreads();
    auto emit = [&](int i, const float4& v) {
      const int x = x0 + warp * kTXW + i;
      if (x < a.nx && yok) *reinterpret_cast<float4*>(tmp + (static_cast<size_t>(z) * a.nx + x) * a.cs + yb) = v;
    };
    if (PSF) {
      const float* kr = (PTAB ? ptab : s_psf) + z * 2 * K;
      rowpass_from_tile<R>(sbuf, warp * kTXW, emit, kr, kr + K, lane, a.ny);
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) emit(i, sbuf[(warp * kTXW + i) * 32 + lane]);
    }
  }
}

// Grid: (camera g of the group, x-tile) items x depth slabs (the cluster).
template <int R, bool PSF>
__global__ void __launch_bounds__(32 * kW, 2) k_grad_spread_yg(const YgArgs a, int c0) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int item = blockIdx.x / a.pslabs;
  const int g = item / ntile;
  grad_item<R, PSF, false>(a, c0 + g, g, (item % ntile) * kTXC, smem, nullptr);
}

template <int R>
__global__ void __launch_bounds__(32 * kW, 2)
    k_grad_spread_ptab_yg(const YgArgs a, int c0, const __grid_constant__ PsfTable t) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int item = blockIdx.x / a.pslabs;
  const int g = item / ntile;
  grad_item<R, true, true>(a, c0 + g, g, (item % ntile) * kTXC, smem, t.c);
}

template <int R>
int launch_grad_R(const YgArgs& a_in, int c0, int gcount, cudaStream_t st) {
  YgArgs a = a_in;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const bool psf = a.psf != nullptr;
  const bool ptab = psf && a.psf_host && static_cast<size_t>(a.nz) * 2 * (2 * R + 1) <= kPsfTableFloats;
  const size_t smem = tile_smem_bytes<R>(psf && !ptab ? a.nz : 0);
  // depth slabs: the fewest of 2, 4, 8 giving four waves of two CTAs per SM
  if (a.pslabs != 2 && a.pslabs != 4 && a.pslabs != 8) {
    a.pslabs = 8;
    for (int s = 2; s < 8; s *= 2)
      if (gcount * ntile * s >= 4 * 2 * sm_count()) {
        a.pslabs = s;
        break;
      }
  }
  bool launch_err = false;
  auto launch = [&](auto k, auto&&... extra) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(gcount * ntile * a.pslabs);
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
    NRGB_LAUNCH_SCOPE("k_grad_spread_yg", st);
    if (cudaLaunchKernelEx(&cfg, k, a, c0, extra...) != cudaSuccess) launch_err = true;
  };
  if (ptab) {
    static thread_local PsfTable table;
    std::memcpy(table.c, a.psf_host, sizeof(float) * a.nz * 2 * (2 * R + 1));
    launch(k_grad_spread_ptab_yg<R>, table);
  } else if (psf) {
    launch(k_grad_spread_yg<R, true>);
  } else {
    launch(k_grad_spread_yg<0, false>);
  }
  return cudaGetLastError() == cudaSuccess && !launch_err ? kOk : kErrKernel;
}

}  // namespace

int yg_grad_spread(const YgArgs& a, int c0, int gcount, cudaStream_t st) {
  if (!a.mu || !a.act || !a.sino || !a.temp) return kErrParameters;
  const int R = a.psf ? (a.psf_k - 1) / 2 : 0;
  switch (R) {
    case 0: return launch_grad_R<0>(a, c0, gcount, st);
    case 1: return launch_grad_R<1>(a, c0, gcount, st);
    case 2: return launch_grad_R<2>(a, c0, gcount, st);
    case 3: return launch_grad_R<3>(a, c0, gcount, st);
    case 4: return launch_grad_R<4>(a, c0, gcount, st);
    case 5: return launch_grad_R<5>(a, c0, gcount, st);
    case 6: return launch_grad_R<6>(a, c0, gcount, st);
    case 7: return launch_grad_R<7>(a, c0, gcount, st);
    default: return kErrParameters;
  }
}

}  // namespace nrgb
