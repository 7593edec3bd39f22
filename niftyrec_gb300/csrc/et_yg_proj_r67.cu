// Per-call projector kernels for PSF radii 6 and 7.
#include "et_yg_project_kernels.cuh"

namespace nrgb {

template int launch_project_R<6>(const YgArgs& a, cudaStream_t st, int* slabs_used);
template int launch_project_R<7>(const YgArgs& a, cudaStream_t st, int* slabs_used);

}  // namespace nrgb
