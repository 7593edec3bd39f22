// Host geometry.  Compiled with -ffp-contract=off: every product and sum is
// rounded separately, as in the reference's x86-64 float code.
#include "et_geometry.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace nrgb {

namespace {

// C = A * B, 4x4 row-major, each entry ((a0*b0 + a1*b1) + a2*b2) + a3*b3.
template <class T>
void mul44(const T* A, const T* B, T* C) {
  T t[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      T s = A[4 * i + 0] * B[j];
      s = s + A[4 * i + 1] * B[4 + j];
      s = s + A[4 * i + 2] * B[8 + j];
      s = s + A[4 * i + 3] * B[12 + j];
      t[4 * i + j] = s;
    }
  std::memcpy(C, t, sizeof(t));
}

}  // namespace

template <class T>
void rotation_matrix_t(T M[16], T tx, T ty, T tz, T cx, T cy, T cz, int axis_order) {
  const T sx = std::sin(tx), cxs = std::cos(tx);
  const T sy = std::sin(ty), cys = std::cos(ty);
  const T sz = std::sin(tz), czs = std::cos(tz);
  const T Rx[16] = {1, 0, 0, 0, 0, cxs, -sx, 0, 0, sx, cxs, 0, 0, 0, 0, 1};
  const T Ry[16] = {cys, 0, sy, 0, 0, 1, 0, 0, -sy, 0, cys, 0, 0, 0, 0, 1};
  const T Rz[16] = {czs, -sz, 0, 0, sz, czs, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  const T Tr[16] = {0, 0, 0, cx, 0, 0, 0, cy, 0, 0, 0, cz, 0, 0, 0, 1};
  // The first-applied rotation is the innermost factor: order "ABC" = C*(B*A).
  const T* order[6][3] = {{Rx, Ry, Rz}, {Rx, Rz, Ry}, {Ry, Rx, Rz},
                          {Ry, Rz, Rx}, {Rz, Rx, Ry}, {Rz, Ry, Rx}};
  const int o = (axis_order >= 0 && axis_order < 6) ? axis_order : 0;
  T P[16], RT[16];
  mul44(order[o][1], order[o][0], P);
  mul44(order[o][2], P, M);
  mul44(M, Tr, RT);
  M[3] = cx - RT[3];
  M[7] = cy - RT[7];
  M[11] = cz - RT[11];
}

void rotation_matrix(float M[16], float tx, float ty, float tz, float cx, float cy, float cz, int axis_order) {
  rotation_matrix_t<float>(M, tx, ty, tz, cx, cy, cz, axis_order);
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

template <class T>
std::vector<CamGeomT<T>> camera_geometry_t(const Cameras& cams) {
  std::vector<CamGeomT<T>> g(cams.n);
  const int n = cams.n;
  for (int c = 0; c < n; ++c) {
    const T tx = cams.angles[c], ty = cams.angles[n + c], tz = cams.angles[2 * n + c];
    const T cx = cams.centers[c], cy = cams.centers[n + c], cz = cams.centers[2 * n + c];
    T M[16];
    rotation_matrix_t<T>(M, tx, ty, tz, cx, cy, cz, 0);
    std::memcpy(g[c].fwd, M, sizeof(T) * 12);
    rotation_matrix_t<T>(M, -tx, -ty, -tz, cx, cy, cz, 5);
    std::memcpy(g[c].bwd, M, sizeof(T) * 12);
  }
  return g;
}

std::vector<CamGeom> camera_geometry(const Cameras& cams) { return camera_geometry_t<float>(cams); }
std::vector<CamGeom64> camera_geometry64(const Cameras& cams) { return camera_geometry_t<double>(cams); }

bool is_y_gantry(const Cameras& cams) {
  for (int c = 0; c < cams.n; ++c)
    if (cams.angles[c] != 0.0f || cams.angles[2 * cams.n + c] != 0.0f) return false;
  return true;
}

bool is_x_gantry(const Cameras& cams) {
  for (int c = 0; c < cams.n; ++c)
    if (cams.angles[cams.n + c] != 0.0f || cams.angles[2 * cams.n + c] != 0.0f) return false;
  return true;
}

CamGeom swap_xy(const CamGeom& g) {
  static const int sigma[3] = {1, 0, 2};
  CamGeom o;
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) {
      o.fwd[4 * r + c] = g.fwd[4 * sigma[r] + sigma[c]];
      o.bwd[4 * r + c] = g.bwd[4 * sigma[r] + sigma[c]];
    }
    o.fwd[4 * r + 3] = g.fwd[4 * sigma[r] + 3];
    o.bwd[4 * r + 3] = g.bwd[4 * sigma[r] + 3];
  }
  return o;
}

std::vector<int> mirror_units(const Cameras& cams, int nx, int nz, int axis) {
  const int n = cams.n;
  const int lateral = axis == 0 ? 1 : 0;  // the rotated in-plane axis other than z
  const float cx = static_cast<float>((nx - 1) / 2.0), cz = static_cast<float>((nz - 1) / 2.0);
  std::vector<int> mate(n, -1);
  std::vector<char> taken(n, 0);
  bool any = false;
  const double two_pi = 2.0 * M_PI;
  auto centred = [&](int c) { return cams.centers[lateral * n + c] == cx && cams.centers[2 * n + c] == cz; };
  const float* theta = cams.angles.data() + static_cast<size_t>(axis) * n;
  auto opposite = [&](int i, int j) {
    const double d = static_cast<double>(theta[j]) - static_cast<double>(theta[i]) - M_PI;
    return std::fabs(d - two_pi * std::nearbyint(d / two_pi)) <= kMirrorTolerance;
  };
  auto reduce = [&](double a) { return a - two_pi * std::floor(a / two_pi); };
  // centred cameras by angle in [0, 2 pi): each camera looks up the cameras
  // near its opposite angle instead of testing every later camera
  std::vector<std::pair<double, int>> by_angle;
  for (int c = 0; c < n; ++c)
    if (centred(c)) by_angle.emplace_back(reduce(theta[c]), c);
  std::sort(by_angle.begin(), by_angle.end());
  const double reach = kMirrorTolerance + 1e-9;  // covers the rounding of the reduction
  for (int i = 0; i < n; ++i) {
    if (taken[i] || !centred(i)) continue;
    // the first later camera (by index) that is free and opposite, as a scan
    // over all later cameras would find it
    int best = -1;
    auto scan = [&](double lo, double hi) {
      for (auto it = std::lower_bound(by_angle.begin(), by_angle.end(), std::make_pair(lo, -1));
           it != by_angle.end() && it->first <= hi; ++it) {
        const int j = it->second;
        if (j > i && !taken[j] && (best < 0 || j < best) && opposite(i, j)) best = j;
      }
    };
    const double target = reduce(static_cast<double>(theta[i]) + M_PI);
    scan(target - reach, target + reach);
    if (target - reach < 0.0) scan(target - reach + two_pi, two_pi);
    if (target + reach >= two_pi) scan(0.0, target + reach - two_pi);
    if (best >= 0) {
      mate[i] = best;
      taken[i] = taken[best] = 1;
      any = true;
    }
  }
  std::vector<int> units;
  if (!any || !(axis == 0 ? is_x_gantry(cams) : is_y_gantry(cams))) return units;
  for (int i = 0; i < n; ++i) {
    if (taken[i] && mate[i] < 0) continue;  // the second camera of a pair
    units.push_back(i);
    units.push_back(mate[i]);
  }
  return units;
}

template <class T>
std::vector<T> separate_psf_t(const float* psf, int k, int nplanes) {
  std::vector<T> sep(static_cast<size_t>(2 * k) * nplanes);
  const int c = (k - 1) / 2;
  for (int n = 0; n < nplanes; ++n) {
    const float* plane = psf + static_cast<size_t>(k) * k * n;
    const T norm = plane[c * k + c];
    for (int i = 0; i < k; ++i) {
      sep[static_cast<size_t>(2 * k) * n + i] = plane[c * k + i];
      sep[static_cast<size_t>(2 * k) * n + k + i] = static_cast<T>(plane[c + i * k]) / norm;
    }
  }
  return sep;
}

std::vector<float> separate_psf(const float* psf, int k, int nplanes) { return separate_psf_t<float>(psf, k, nplanes); }
std::vector<double> separate_psf64(const float* psf, int k, int nplanes) {
  return separate_psf_t<double>(psf, k, nplanes);
}

}  // namespace nrgb
