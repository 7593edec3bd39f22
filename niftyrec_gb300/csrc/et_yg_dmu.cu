// Fused y-gantry gradient of L = sum(g * project(activity, mu)) with respect
// to mu (the d/dmu of the differentiable projector; the reference's own
// attenuation gradient, emission-lib/_et.cpp:1679-1924, is a different
// quantity and stays on the general path).
//
// For one ray of camera c, p = sum_z v_z exp(-T_z) with v the PSF-convolved
// rotated activity and T_z the inclusive sum of the rotated mu, so
//   dL/dmu_rot(z) = -g * S(z),  S(z) = sum_{z' >= z} v_z' exp(-T_z'),
// and dL/dmu is its transposed bilinear scatter into the volume.  Work item as
// the projector's: a cluster of depth-slab CTAs per (camera, 32-column tile).
// Walk 1 forms each slab's local transmission and partial; the cluster
// exchanges them (slab s needs exp(-T before s) and the weighted partials of
// the slabs after it); walk 2 recomputes the samples and row / column passes
// (nothing per depth is stored) and scatters -g S(z) with vector reductions,
// or with a.det writes it to the rotated-frame scratch of its camera (volume
// camera - a.cam0 at a.temp) for the transposed gather (fixed summation order).
#include "et_yg_device.cuh"

namespace nrgb {
namespace {

template <int R, bool PSF, bool PTAB>
__device__ __forceinline__ void dmu_item(const YgArgs& a, int cam, int x0, unsigned char* smem, const float* ptab) {
  using TS = TileShape<R>;
  const float* __restrict__ act = a.act + a.row0;
  const float* __restrict__ mu = a.mu + a.row0;
  float* __restrict__ out = a.out + a.row0;
  float* __restrict__ scratch = a.det ? a.temp + static_cast<size_t>(cam - a.cam0) * a.nz * a.nx * a.cs : nullptr;
  constexpr int NS = TS::NS;
  constexpr int K = 2 * R + 1;
  constexpr size_t kSb = TS::sb_bytes(false);
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

  float4 T[kTXW], P[kTXW];
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    T[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  ybuf_zero_pads();
  __syncthreads();

  auto produce = [&](int z, int b) {
    float4* sbuf = sb + b * NS * 32;
    Tap* tb = taps + b * TS::kTapSlots;
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
  // the PSF-convolved activity of this warp's output columns at plane z
  auto pass = [&](int z, int b, auto emit) {
    const float4* sbuf = sb + b * NS * 32;
    if (PSF) {
      const float* kr = (PTAB ? ptab : s_psf) + z * 2 * K;
      rowpass_from_tile<R>(sbuf, warp * kTXW, emit, kr, kr + K, lane, a.ny);
    } else {
#pragma unroll
      for (int i = 0; i < kTXW; ++i) emit(i, sbuf[(warp * kTXW + i) * 32 + lane]);
    }
  };
  auto walk = [&](auto consume) {
    for (int z = zbeg; z < zend; ++z) {
      produce(z, z & 1);
      __syncthreads();
      consume(z, z & 1);
    }
  };

  // walk 1: local transmission T and partial P of the slab
  walk([&](int z, int b) {
    const Tap* tb = taps + b * TS::kTapSlots;
    pass(z, b, [&](int i, const float4& v) {
      add4(T[i], sample4(mu, tb[tap_slot<R>(warp * kTXW + i + R)], yb, yok));
      fma4(P[i], v, exp_neg4(T[i]));
    });
  });

  // exchange through distributed shared memory (the tile region is free)
  __syncthreads();
  float4* sT = sb;
  float4* sP = sb + kTXC * 32;
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    sT[(warp * kTXW + i) * 32 + lane] = T[i];
    sP[(warp * kTXW + i) * 32 + lane] = P[i];
  }
  cluster.sync();
  // per output column: contribution -g S(z) = A + B * Pre(z), Pre(z) the local
  // partial before plane z; A = -g (exp(-Tb) P_slab + later), B = g exp(-Tb)
  float4 A[kTXW], Bq[kTXW];
#pragma unroll
  for (int i = 0; i < kTXW; ++i) {
    const int o = warp * kTXW + i;
    const int x = x0 + o;
    float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
    if (x < a.nx && yok) g = ldg4(a.sino + (static_cast<size_t>(cam) * a.nx + x) * a.cy + a.row0 + yb);
    float4 tacc = make_float4(0.f, 0.f, 0.f, 0.f), later = tacc, wscale = tacc;
    for (int s = 0; s < nslabs; ++s) {
      const float4 ts = cluster.map_shared_rank(sT, s)[o * 32 + lane];
      if (s == slab) wscale = exp_neg4(tacc);
      if (s > slab) fma4(later, exp_neg4(tacc), cluster.map_shared_rank(sP, s)[o * 32 + lane]);
      add4(tacc, ts);
    }
    const float4 total = make_float4(fmaf(wscale.x, P[i].x, later.x), fmaf(wscale.y, P[i].y, later.y),
                                     fmaf(wscale.z, P[i].z, later.z), fmaf(wscale.w, P[i].w, later.w));
    A[i] = make_float4(-g.x * total.x, -g.y * total.y, -g.z * total.z, -g.w * total.w);
    Bq[i] = mul4(g, wscale);
    T[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P[i] = make_float4(0.f, 0.f, 0.f, 0.f);  // Pre from here on
  }
  cluster.sync();  // every CTA's exchange reads are done before the tiles are rewritten

  // walk 2: recompute and scatter
  walk([&](int z, int b) {
    const Tap* tb = taps + b * TS::kTapSlots;
    pass(z, b, [&](int i, const float4& v) {
      const Tap& t = tb[tap_slot<R>(warp * kTXW + i + R)];
      add4(T[i], sample4(mu, t, yb, yok));
      const float4 d = make_float4(fmaf(Bq[i].x, P[i].x, A[i].x), fmaf(Bq[i].y, P[i].y, A[i].y),
                                   fmaf(Bq[i].z, P[i].z, A[i].z), fmaf(Bq[i].w, P[i].w, A[i].w));
      const int x = x0 + warp * kTXW + i;
      if (a.det) {  // uniform over the launch
        if (x < a.nx && yok) *reinterpret_cast<float4*>(scratch + (static_cast<size_t>(z) * a.nx + x) * a.cs + yb) = d;
      } else if (x < a.nx && yok && lane_writes(a, yb)) {
        scatter4(out, t, yb, d);
      }
      fma4(P[i], v, exp_neg4(T[i]));
    });
  });
}

template <int R, bool PSF>
__global__ void __launch_bounds__(32 * kW, 2) k_dmu_yg(const YgArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int item = blockIdx.x / a.pslabs;
  dmu_item<R, PSF, false>(a, a.cam0 + item / ntile, (item % ntile) * kTXC, smem, nullptr);
}

template <int R>
__global__ void __launch_bounds__(32 * kW, 2) k_dmu_ptab_yg(const YgArgs a, const __grid_constant__ PsfTable t) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const int item = blockIdx.x / a.pslabs;
  dmu_item<R, true, true>(a, a.cam0 + item / ntile, (item % ntile) * kTXC, smem, t.c);
}

template <int R>
int launch_dmu_R(const YgArgs& a_in, cudaStream_t st) {
  YgArgs a = a_in;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const bool psf = a.psf != nullptr;
  const bool ptab = psf && a.psf_host && static_cast<size_t>(a.nz) * 2 * (2 * R + 1) <= kPsfTableFloats;
  const size_t smem = tile_smem_bytes<R>(psf && !ptab ? a.nz : 0);
  // depth slabs: the fewest of 2, 4, 8 giving four waves of two CTAs per SM
  if (a.pslabs != 2 && a.pslabs != 4 && a.pslabs != 8) {
    a.pslabs = 8;
    for (int s = 2; s < 8; s *= 2)
      if (a.ncam * ntile * s >= 4 * 2 * sm_count()) {
        a.pslabs = s;
        break;
      }
  }
  bool launch_err = false;
  auto launch = [&](auto k, auto&&... extra) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(a.ncam * ntile * a.pslabs);
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
    NRGB_LAUNCH_SCOPE("k_dmu_yg", st);
    if (cudaLaunchKernelEx(&cfg, k, a, extra...) != cudaSuccess) launch_err = true;
  };
  if (ptab) {
    static thread_local PsfTable table;
    std::memcpy(table.c, a.psf_host, sizeof(float) * a.nz * 2 * (2 * R + 1));
    launch(k_dmu_ptab_yg<R>, table);
  } else if (psf) {
    launch(k_dmu_yg<R, true>);
  } else {
    launch(k_dmu_yg<0, false>);
  }
  return cudaGetLastError() == cudaSuccess && !launch_err ? kOk : kErrKernel;
}

int dmu_by_radius(int R, const YgArgs& a, cudaStream_t st) {
  switch (R) {
    case 0: return launch_dmu_R<0>(a, st);
    case 1: return launch_dmu_R<1>(a, st);
    case 2: return launch_dmu_R<2>(a, st);
    case 3: return launch_dmu_R<3>(a, st);
    case 4: return launch_dmu_R<4>(a, st);
    case 5: return launch_dmu_R<5>(a, st);
    case 6: return launch_dmu_R<6>(a, st);
    case 7: return launch_dmu_R<7>(a, st);
    default: return kErrParameters;
  }
}

}  // namespace

int yg_dmu(const YgArgs& a, cudaStream_t st) {
  if (!a.mu || !a.act || !a.sino || !a.out) return kErrParameters;
  const int R = a.psf ? (a.psf_k - 1) / 2 : 0;
  if (a.det) {
    // camera groups into the scratch (a.work, yg_dmu_det_workspace bytes),
    // each followed by the transposed gather on the same stream
    if (!a.work) return kErrParameters;
    const int group = yg_even_group(a.ncam, a.group);
    for (const Window& w : row_windows(a.ny, R)) {
      YgArgs b = windowed(a, w);
      b.temp = a.work;
      b.units = nullptr;
      for (int c0 = 0; c0 < a.ncam; c0 += group) {
        YgArgs d = b;
        d.cam0 = c0;
        d.ncam = std::min(group, a.ncam - c0);
        const int s = dmu_by_radius(R, d, st);
        if (s != kOk) return s;
        yg_tgather(b, c0, d.ncam, 0, st);
      }
    }
    return cudaGetLastError() == cudaSuccess ? kOk : kErrKernel;
  }
  const size_t full = static_cast<size_t>(a.nz) * a.nx * a.cy;
  if (cudaMemsetAsync(a.out, 0, sizeof(float) * full, st) != cudaSuccess) return kErrKernel;
  for (const Window& w : row_windows(a.ny, R)) {
    const int s = dmu_by_radius(R, windowed(a, w), st);
    if (s != kOk) return s;
  }
  return kOk;
}

size_t yg_dmu_det_workspace(int nx, int ny, int nz, int ncam, int group) {
  return yg_gradient_workspace(nx, ny, nz, ncam, yg_even_group(ncam, group), 1);
}

}  // namespace nrgb
