// Per-call projector kernels for PSF radii 4 and 5.
#include "et_yg_project_kernels.cuh"

namespace nrgb {

template int launch_project_R<4>(const YgArgs& a, cudaStream_t st, int* slabs_used);
template int launch_project_R<5>(const YgArgs& a, cudaStream_t st, int* slabs_used);

}  // namespace nrgb
