// Fused y-gantry projector: dispatch of the per-call kernels by PSF radius,
// the persistent batched projector, and the public entry points.
#include "et_yg_device.cuh"

namespace nrgb {

template <int R>
int launch_project_R(const YgArgs& a, cudaStream_t st, int* slabs_used);  // et_yg_project_kernels.cuh

// ------------------------------------------------------------- dispatch
// Depth slabs (cluster size) of the projector: the fewest of 2, 4, 8 (16
// with at least 8 planes per slab) that give at least three waves of CTAs
// (fewer slabs merge less; more slabs fill the GPU for small problems, e.g.
// the 15-camera subsets of an OSEM step).  Measured on GB300 without mirror
// units: 128^3 x 120 cameras 4 (0.84 ms; 2: 0.87, 8: 0.87), 256^3 x 180: 2
// (15.9 ms; 4: 16.7), 64^3 x 60: 8 (0.149 ms; 4: 0.158); with mirror units
// (60 units at 128^3 x 120): 4 (0.612 ms; 8: 0.640, 16: 0.858).
int project_slabs(int items, int ctas_per_sm, int nz) {
  const int slots = sm_count() * ctas_per_sm;
  // few items (an OSEM subset: 15 cameras x 4 tiles at 128^3): one round of
  // 4-slab clusters beats several rounds of shorter slabs (8 subsets at
  // 128^3 x 120: 2.42 against 2.49 ms per iteration with 16 slabs)
  if (items * 4 <= slots) return 4;
  const int most = nz >= 128 ? 16 : 8;
  for (int s = 2; s < most; s *= 2)
    if (items * s >= 3 * slots) return s;
  return most;
}

int yg_pair_project_slabs(int nunits, int nx, int nz) {
  return project_slabs(nunits * ((nx + kTXC - 1) / kTXC), 2, nz);
}

namespace {

// Persistent projector over a batch of volumes: each cluster takes work items
// (volume, row window, camera, x-tile) from a global counter until none are
// left, so volumes of any size share the GPU in one launch.  The item number
// is drawn by the cluster's first thread and read by the other CTAs from its
// shared memory (double-buffered: the slot of item i is rewritten at item i+2,
// after the barriers of item i+1).
// CTAS: CTAs per SM the kernel is built for (3: 80 registers and more warps to
// hide the gathers' latency, where three tiles fit in shared memory; else 2).
template <int R, bool PSF, bool ATT, int CTAS>
__global__ void __cluster_dims__(kSlabsP, 1, 1) __launch_bounds__(32 * kW, CTAS)
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

int project_by_radius(int R, const YgArgs& a, cudaStream_t st, int* slabs_used) {
  switch (R) {
    case 0: return launch_project_R<0>(a, st, slabs_used);
    case 1: return launch_project_R<1>(a, st, slabs_used);
    case 2: return launch_project_R<2>(a, st, slabs_used);
    case 3: return launch_project_R<3>(a, st, slabs_used);
    case 4: return launch_project_R<4>(a, st, slabs_used);
    case 5: return launch_project_R<5>(a, st, slabs_used);
    case 6: return launch_project_R<6>(a, st, slabs_used);
    case 7: return launch_project_R<7>(a, st, slabs_used);
    default: return kErrParameters;
  }
}

// Persistent grid: `ctas` CTAs per SM, whole clusters.
int batch_clusters(int ctas) { return sm_count() * ctas / kSlabsP; }

template <int R, bool PSF>
int launch_project_batch_R(const BatchStepDesc* d, const BatchSel& sel, bool att, int max_nz, int* counter,
                           cudaStream_t st) {
  const size_t smem = tile_smem_bytes<R>(PSF ? max_nz : 0);
  const bool three = 3 * (smem + kYBufBytes + 1024) <= 228 * 1024;
  auto go = [&](auto k, int ctas) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    NRGB_LAUNCH_SCOPE("k_project_batch_yg", st);
    k<<<batch_clusters(ctas) * kSlabsP, 32 * kW, smem, st>>>(d, sel, counter);
  };
  if (att) {
    if (three) go(k_project_batch_yg<R, PSF, true, 3>, 3);
    else go(k_project_batch_yg<R, PSF, true, 2>, 2);
  } else {
    if (three) go(k_project_batch_yg<R, PSF, false, 3>, 3);
    else go(k_project_batch_yg<R, PSF, false, 2>, 2);
  }
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

}  // namespace

int yg_project_batch(const BatchStepDesc* d_desc, const BatchSel& sel, int psf_k, bool att, int max_nz,
                     int* d_counter, cudaStream_t st) {
  if (sel.n <= 0 || sel.total <= 0) return kOk;
  return project_batch_by_radius(psf_k, d_desc, sel, att, max_nz, d_counter, st);
}

int yg_project(const YgArgs& a, cudaStream_t st, int* slabs_used) {
  const int R = a.psf ? (a.psf_k - 1) / 2 : 0;
  int used = 0;
  for (const Window& w : row_windows(a.ny, R)) {
    const int s = project_by_radius(R, windowed(a, w), st, &used);
    if (s != kOk) return s;
    // every window launches with the same slab count (same sizes, same kernel)
    if (slabs_used) *slabs_used = used;
  }
  return kOk;
}

}  // namespace nrgb
