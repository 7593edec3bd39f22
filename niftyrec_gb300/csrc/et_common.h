// Shared definitions of the GB300 SPECT projector library: status codes,
// per-camera geometry, problem description and device layouts.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace nrgb {

// Status codes.  0..8 keep the values of the reference
// (emission-lib/_et_common.h:40-48); 10 is new: the problem does not fit the
// fixed scratch of the no-allocation backprojection entry point.  9 is not
// used (no kernel of this library waits on another block or device).
enum Status : int {
  kOk = 0,
  kErrUnspecified = 1,
  kErrParameters = 2,
  kErrKernel = 3,
  kErrAllocGpu = 4,
  kErrAllocCpu = 5,
  kErrTransferGpu = 6,
  kErrNoGpuBuilt = 7,
  kErrNoGpuInstalled = 8,
  kErrScratchTooSmall = 10,
};

// Memory layouts of device volumes and sinograms.
//  kLayoutNifti : x fastest, then y, then z (cameras for sinograms) -- the
//                 reference's nifti order.
//  kLayoutColumn: y fastest ("columns" along the gantry axis), then x, then z;
//                 each column padded to cy = round_up(ny, 4) floats with zero
//                 pads.  Native layout of the fused y-gantry kernels.
enum Layout : int { kLayoutNifti = 0, kLayoutColumn = 1 };

// Affine rows of one camera.  fwd: the projector's resampling matrix (XYZ
// order, +theta, about the centre); bwd: the backprojector's inverse
// resampling matrix (ZYX order, -theta).  Row-major 3x4: p_i = m[4i+0]*x +
// m[4i+1]*y + m[4i+2]*z + m[4i+3].
template <class T>
struct CamGeomT {
  T fwd[12];
  T bwd[12];
};
using CamGeom = CamGeomT<float>;
using CamGeom64 = CamGeomT<double>;  // geometry of the float64 reference path

// Backprojector variants.
//  kBackReference: the reference's inverse-rotation gather
//                  (emission-lib/_et.cpp:474-494).
//  kBackAdjoint  : exact transpose of the projector (transposed PSF and
//                  transposed trilinear interpolation); not in the reference.
enum BackMode : int { kBackReference = 0, kBackAdjoint = 1 };

// Storage type of the volumes the fused kernels sample (activity, mu).
//  kStorageF32 : float32, the reference's type.
//  kStorageBF16: bfloat16 (half the bytes), widened exactly to float32 on
//                load; all arithmetic stays float32 and the depth sums (the
//                transmission prefix and the projection) are
//                Kahan-compensated.
enum Storage : int { kStorageF32 = 0, kStorageBF16 = 1 };

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// Streaming multiprocessors of the current device (queried once per device;
// 152 on GB300), for grids sized in waves.
int sm_count();

}  // namespace nrgb
