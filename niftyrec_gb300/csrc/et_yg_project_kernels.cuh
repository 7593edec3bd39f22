// Per-call projector kernels and their launcher, instantiated per PSF
// radius in separate translation units (et_yg_proj_r*.cu) so that the
// projector's many instantiations compile in parallel.
#pragma once

#include "et_yg_device.cuh"

namespace nrgb {

// Depth slabs (cluster size) of the projector for `items` cluster work items
// at `ctas_per_sm` CTAs per SM and nz depth planes (et_yg_project.cu).
int project_slabs(int items, int ctas_per_sm, int nz);

namespace {

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

}  // namespace

// Launch the per-call projector of PSF radius R (R = 0: no PSF) for one row
// window; explicitly instantiated in et_yg_proj_r*.cu.  slabs_used (if
// non-null) receives the depth-slab count of the launch (the slabs of the
// carries written to a.carry_out).
template <int R>
int launch_project_R(const YgArgs& a_in, cudaStream_t st, int* slabs_used) {
  YgArgs a = a_in;
  const int ntile = (a.nx + kTXC - 1) / kTXC;
  const bool psf = a.psf != nullptr;
  const bool bf16 = a.storage == kStorageBF16;
  // the PSF in the kernel parameters when the host copy is given and fits
  const bool ptab = psf && a.psf_host && static_cast<size_t>(a.nz) * 2 * (2 * R + 1) <= kPsfTableFloats;
  // mirror cameras: float32 always; bfloat16 (Kahan compensations in shared
  // memory) where two CTAs per SM still fit
  bool pair = a.units != nullptr && a.nunits > 0;
  size_t smem = project_smem_bytes<R>(psf && !ptab ? a.nz : 0, pair, bf16);
  if (pair && bf16 && 2 * (smem + kYBufBytes + 1024) > 228 * 1024) {
    pair = false;
    smem = project_smem_bytes<R>(psf && !ptab ? a.nz : 0, false, true);
  }
  const int nunits = pair ? a.nunits : a.ncam;
  // three CTAs per SM need three tiles (plus 1 KB reserved each) in the 228 KB
  const bool three = 3 * (smem + kYBufBytes + 1024) <= 228 * 1024;
  if (a.pslabs != 2 && a.pslabs != 4 && a.pslabs != 8 && a.pslabs != 16)
    a.pslabs = project_slabs(nunits * ntile, three && !bf16 && !pair ? 3 : 2, a.nz);
  // carry split: the slab's halves must be the backprojector's slabs of twice
  // the count, with at most 8 of them
  auto split_ok = [&](int p) {
    return a.carry_out && a.mu && a.carry_split && 2 * p <= 8 &&
           (a.nz + p - 1) / p == 2 * ((a.nz + 2 * p - 1) / (2 * p));
  };
  a.carry_split = split_ok(a.pslabs) ? 1 : 0;
  // one cluster of a.pslabs CTAs per (unit, x-tile); 16 is a non-portable
  // cluster size: it falls back to 8 where the kernel cannot be resident so
  bool launch_err = false;
  auto launch = [&](auto k, auto&&... extra) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(32 * kW);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (a.pslabs == 16) {
      int clusters = 0;
      cfg.gridDim = dim3(nunits * ntile * 16);
      attr[0].val.clusterDim.x = 16;
      if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
          cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess || clusters < 1) {
        cudaGetLastError();
        a.pslabs = 8;
        a.carry_split = split_ok(8) ? 1 : 0;
      }
    }
    cfg.gridDim = dim3(nunits * ntile * a.pslabs);
    attr[0].val.clusterDim.x = a.pslabs;
    if (slabs_used) *slabs_used = a.carry_split ? 2 * a.pslabs : a.pslabs;
    NRGB_LAUNCH_SCOPE("k_project_yg", st);
    if (cudaLaunchKernelEx(&cfg, k, a, extra...) != cudaSuccess) launch_err = true;
  };
  auto go = [&](auto k) { launch(k); };
  auto go_tab = [&](auto k) {
    static thread_local PsfTable table;
    std::memcpy(table.c, a.psf_host, sizeof(float) * a.nz * 2 * (2 * R + 1));
    launch(k, table);
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
  if (bf16 && pair)
    pick(__nv_bfloat16(), std::integral_constant<int, 2>(), On());
  else if (bf16)
    pick(__nv_bfloat16(), std::integral_constant<int, 2>(), Off());
  else if (pair)
    pick(0.0f, std::integral_constant<int, 2>(), On());
  else if (three)
    pick(0.0f, std::integral_constant<int, 3>(), Off());
  else
    pick(0.0f, std::integral_constant<int, 2>(), Off());
  return cudaGetLastError() == cudaSuccess && !launch_err ? kOk : kErrKernel;
}

}  // namespace nrgb
