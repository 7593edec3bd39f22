// Host geometry.  Compiled with -ffp-contract=off: every product and sum is
// rounded separately, as in the reference's x86-64 float code.
#include "et_geometry.h"

#include <cmath>
#include <cstring>

namespace nrgb {

namespace {

// C = A * B, 4x4 row-major, each entry ((a0*b0 + a1*b1) + a2*b2) + a3*b3.
void mul44(const float* A, const float* B, float* C) {
  float t[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float s = A[4 * i + 0] * B[j];
      s = s + A[4 * i + 1] * B[4 + j];
      s = s + A[4 * i + 2] * B[8 + j];
      s = s + A[4 * i + 3] * B[12 + j];
      t[4 * i + j] = s;
    }
  std::memcpy(C, t, sizeof(t));
}

}  // namespace

void rotation_matrix(float M[16], float tx, float ty, float tz, float cx, float cy, float cz, int axis_order) {
  const float sx = std::sin(tx), cxs = std::cos(tx);
  const float sy = std::sin(ty), cys = std::cos(ty);
  const float sz = std::sin(tz), czs = std::cos(tz);
  const float Rx[16] = {1, 0, 0, 0, 0, cxs, -sx, 0, 0, sx, cxs, 0, 0, 0, 0, 1};
  const float Ry[16] = {cys, 0, sy, 0, 0, 1, 0, 0, -sy, 0, cys, 0, 0, 0, 0, 1};
  const float Rz[16] = {czs, -sz, 0, 0, sz, czs, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  const float T[16] = {0, 0, 0, cx, 0, 0, 0, cy, 0, 0, 0, cz, 0, 0, 0, 1};
  // The first-applied rotation is the innermost factor: order "ABC" = C*(B*A).
  const float* order[6][3] = {{Rx, Ry, Rz}, {Rx, Rz, Ry}, {Ry, Rx, Rz},
                              {Ry, Rz, Rx}, {Rz, Rx, Ry}, {Rz, Ry, Rx}};
  const int o = (axis_order >= 0 && axis_order < 6) ? axis_order : 0;
  float P[16], RT[16];
  mul44(order[o][1], order[o][0], P);
  mul44(order[o][2], P, M);
  mul44(M, T, RT);
  M[3] = cx - RT[3];
  M[7] = cy - RT[7];
  M[11] = cz - RT[11];
}

int expand_cameras(const float* cameras, int n, int ncols, const int center_size[3], Cameras* out) {
  if (!(ncols == 1 || ncols == 3 || ncols == 6) || n <= 0) return kErrParameters;
  out->n = n;
  out->angles.assign(3 * static_cast<size_t>(n), 0.0f);
  out->centers.assign(3 * static_cast<size_t>(n), 0.0f);
  if (ncols == 1) {
    for (int c = 0; c < n; ++c) out->angles[n + c] = cameras[c];
  } else {
    std::memcpy(out->angles.data(), cameras, sizeof(float) * 3 * n);
  }
  if (ncols == 6) {
    std::memcpy(out->centers.data(), cameras + 3 * static_cast<size_t>(n), sizeof(float) * 3 * n);
  } else {
    for (int a = 0; a < 3; ++a) {
      const float c0 = static_cast<float>((center_size[a] - 1) / 2.0);
      for (int c = 0; c < n; ++c) out->centers[a * n + c] = c0;
    }
  }
  return kOk;
}

std::vector<CamGeom> camera_geometry(const Cameras& cams) {
  std::vector<CamGeom> g(cams.n);
  const int n = cams.n;
  for (int c = 0; c < n; ++c) {
    const float tx = cams.angles[c], ty = cams.angles[n + c], tz = cams.angles[2 * n + c];
    const float cx = cams.centers[c], cy = cams.centers[n + c], cz = cams.centers[2 * n + c];
    float M[16];
    rotation_matrix(M, tx, ty, tz, cx, cy, cz, 0);
    std::memcpy(g[c].fwd, M, sizeof(float) * 12);
    rotation_matrix(M, -tx, -ty, -tz, cx, cy, cz, 5);
    std::memcpy(g[c].bwd, M, sizeof(float) * 12);
  }
  return g;
}

bool is_y_gantry(const Cameras& cams) {
  for (int c = 0; c < cams.n; ++c)
    if (cams.angles[c] != 0.0f || cams.angles[2 * cams.n + c] != 0.0f) return false;
  return true;
}

std::vector<float> separate_psf(const float* psf, int k, int nplanes) {
  std::vector<float> sep(static_cast<size_t>(2 * k) * nplanes);
  const int c = (k - 1) / 2;
  for (int n = 0; n < nplanes; ++n) {
    const float* plane = psf + static_cast<size_t>(k) * k * n;
    const float norm = plane[c * k + c];
    for (int i = 0; i < k; ++i) {
      sep[static_cast<size_t>(2 * k) * n + i] = plane[c * k + i];
      sep[static_cast<size_t>(2 * k) * n + k + i] = plane[c + i * k] / norm;
    }
  }
  return sep;
}

}  // namespace nrgb
