// Host-side geometry: rotation matrices, camera expansion and PSF separation,
// each following the reference's float arithmetic so that the device sees the
// same sampling positions as the reference CPU path.
#pragma once

#include <vector>

#include "et_common.h"

namespace nrgb {

// 4x4 row-major rotation about a centre; axis_order 0..5 = XYZ, XZY, YXZ, YZX,
// ZXY, ZYX.  Follows emission-lib/_et_common.cpp:35-171 (products evaluated
// left to right in float, translation column c - R*c).
void rotation_matrix(float M[16], float tx, float ty, float tz, float cx, float cy, float cz, int axis_order);

// Expanded camera set: angles[a*n + c] and centres[a*n + c] for axis a.
struct Cameras {
  int n = 0;
  std::vector<float> angles;
  std::vector<float> centers;
};

// Camera-column rules of emission-lib/_et_array_interface.cpp:409-440:
// [n x 1] -> theta_y only; [n x 3] -> angles; [n x 6] -> angles + centres;
// otherwise the centre is (center_size - 1) / 2.  Returns kErrParameters for
// other column counts.
int expand_cameras(const float* cameras, int n, int ncols, const int center_size[3], Cameras* out);

// Forward/backward matrices per camera (see CamGeom); the float64 variant
// evaluates the same formulas in double from the float angles and centres.
std::vector<CamGeom> camera_geometry(const Cameras& cams);
std::vector<CamGeom64> camera_geometry64(const Cameras& cams);

// True when every camera rotates about the gantry axis only (theta_x ==
// theta_z == 0), so that the resampling matrices are exact rotations about y.
bool is_y_gantry(const Cameras& cams);

// Mirror pairs of y-gantry cameras on an nx x nz grid: cameras i < j whose
// angles differ by pi (within kMirrorTolerance radians, modulo 2 pi) and
// whose centres are both the grid centre ((nx-1)/2, (nz-1)/2) sample the
// same points (camera j's rotated volume is camera i's mirrored in x and z).
// Returns units {i, j} and {i, -1} (unpaired cameras) in the order of their
// first camera, two ints per unit; empty when no pair exists.
// axis 1 (gantry about y, the default) or 0 (gantry about x: nx is then the
// y extent and the angles and centres are the x-rotation's and y's).
constexpr double kMirrorTolerance = 1e-6;
std::vector<int> mirror_units(const Cameras& cams, int nx, int nz, int axis = 1);

// True when every camera rotates about the x axis only (theta_y == theta_z ==
// 0).  Such cameras run on the gantry kernels with x and y exchanged: the
// nifti volume [z][y][x] is then their column layout (x fastest), and
// swap_xy gives the matrices in those coordinates (rows and columns of x and
// y exchanged: the same float values, so the same sampling positions).
bool is_x_gantry(const Cameras& cams);
CamGeom swap_xy(const CamGeom& g);

// Separated depth-dependent PSF (emission-lib/_et.cpp:194-215): for plane n,
// row kernel = central row, column kernel = central column / centre value.
// Device layout: sep[n*2k + i] = row[i], sep[n*2k + k + i] = col[i], the
// kernels stored as given (the convolution reverses them).  Square kernels
// only (k = kx = ky).
std::vector<float> separate_psf(const float* psf, int k, int nplanes);
std::vector<double> separate_psf64(const float* psf, int k, int nplanes);

}  // namespace nrgb
