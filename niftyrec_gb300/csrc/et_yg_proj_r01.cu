// Per-call projector kernels for PSF radii 0 and 1.
#include "et_yg_project_kernels.cuh"

namespace nrgb {

template int launch_project_R<0>(const YgArgs& a, cudaStream_t st, int* slabs_used);
template int launch_project_R<1>(const YgArgs& a, cudaStream_t st, int* slabs_used);

}  // namespace nrgb
