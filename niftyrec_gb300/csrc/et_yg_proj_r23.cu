// Per-call projector kernels for PSF radii 2 and 3.
#include "et_yg_project_kernels.cuh"

namespace nrgb {

template int launch_project_R<2>(const YgArgs& a, cudaStream_t st, int* slabs_used);
template int launch_project_R<3>(const YgArgs& a, cudaStream_t st, int* slabs_used);

}  // namespace nrgb
