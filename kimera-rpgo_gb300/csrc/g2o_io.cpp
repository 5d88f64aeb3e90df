// Native g2o reader (rpgo_g2o_read, include/rpgo_gb300.h).
//
// Reads the file format of every Kimera-RPGO fixture and result the way
// GTSAM's readG2o / load3D / load2D (called at examples/RpgoReadG2o.cpp:129-143)
// build the graph that RobustSolver::update receives:
//   VERTEX_SE3:QUAT id x y z qx qy qz qw  -> Pose3(Rot3::Quaternion(qw, qx,
//     qy, qz) of the normalised quaternion, (x, y, z));
//   EDGE_SE3:QUAT id1 id2 x y z qx qy qz qw I11 I12 .. I66 (upper triangle,
//     g2o's [t; R] order) -> BetweenFactor<Pose3> with the information
//     reordered to GTSAM's [R; t] (the inverse of src/Logger.cpp:148-152);
//   VERTEX_SE2 id x y theta; EDGE_SE2 id1 id2 dx dy dtheta I11 I12 I13 I22
//     I23 I33 (Pose2 tangent order x, y, theta).
// Noise models follow noiseModel::Gaussian::Information(I, smart = true): a
// diagonal I becomes Diagonal::Precisions (sigma_k = sqrt(1 / I_kk),
// covariance sigma_k^2, square-root information 1 / sigma_k); otherwise the
// covariance is I^-1 and the square-root information the upper-triangular R
// with R^T R = I. Other lines are skipped.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/rpgo_gb300.h"

struct rpgo_g2o {
  int dim = 3;
  std::vector<int32_t> kind;
  std::vector<uint64_t> k1, k2, vkeys;
  std::vector<double> meas, cov, sqrt_info, poses;
};

namespace {

void rot_from_quaternion(double w, double x, double y, double z, double* R) {
  const double f = 1.0 / std::sqrt(w * w + x * x + y * y + z * z);
  w *= f, x *= f, y *= f, z *= f;
  const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
  const double twx = tx * w, twy = ty * w, twz = tz * w;
  const double txx = tx * x, txy = ty * x, txz = tz * x;
  const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
  R[0] = 1.0 - (tyy + tzz), R[1] = txy - twz, R[2] = txz + twy;
  R[3] = txy + twz, R[4] = 1.0 - (txx + tzz), R[5] = tyz - twx;
  R[6] = txz - twy, R[7] = tyz + twx, R[8] = 1.0 - (txx + tyy);
}

// Gaussian::Information(I, smart): covariance and upper-triangular R (d x d,
// row-major). Returns false when I is not positive definite.
bool noise_from_information(int d, const double* I, double* cov, double* R) {
  bool diagonal = true;
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j)
      if (i != j && I[d * i + j] != 0.0) diagonal = false;
  std::memset(cov, 0, sizeof(double) * d * d);
  std::memset(R, 0, sizeof(double) * d * d);
  if (diagonal) {
    for (int i = 0; i < d; ++i) {
      if (!(I[d * i + i] > 0.0)) return false;
      const double s = std::sqrt(1.0 / I[d * i + i]);
      cov[d * i + i] = s * s;
      R[d * i + i] = 1.0 / s;
    }
    return true;
  }
  // I = L L^T (lower L), R = L^T
  double L[36] = {0};
  for (int j = 0; j < d; ++j) {
    double s = I[d * j + j];
    for (int k = 0; k < j; ++k) s -= L[d * j + k] * L[d * j + k];
    if (!(s > 0.0)) return false;
    L[d * j + j] = std::sqrt(s);
    for (int i = j + 1; i < d; ++i) {
      double t = I[d * i + j];
      for (int k = 0; k < j; ++k) t -= L[d * i + k] * L[d * j + k];
      L[d * i + j] = t / L[d * j + j];
    }
  }
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < d; ++j) R[d * i + j] = L[d * j + i];
  // covariance = I^-1 = L^-T L^-1, column by column
  for (int c = 0; c < d; ++c) {
    double y[6], x[6];
    for (int i = 0; i < d; ++i) {
      double t = (i == c) ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) t -= L[d * i + k] * y[k];
      y[i] = t / L[d * i + i];
    }
    for (int i = d - 1; i >= 0; --i) {
      double t = y[i];
      for (int k = i + 1; k < d; ++k) t -= L[d * k + i] * x[k];
      x[i] = t / L[d * i + i];
    }
    for (int i = 0; i < d; ++i) cov[d * i + c] = x[i];
  }
  return true;
}

bool read_doubles(const char*& p, double* out, int n) {
  for (int k = 0; k < n; ++k) {
    char* end = nullptr;
    out[k] = std::strtod(p, &end);
    if (end == p) return false;
    p = end;
  }
  return true;
}

bool read_key(const char*& p, uint64_t* out) {
  char* end = nullptr;
  const unsigned long long v = std::strtoull(p, &end, 10);
  if (end == p) return false;
  p = end;
  *out = (uint64_t)v;
  return true;
}

bool parse_line(rpgo_g2o* g, const char* line) {
  while (*line == ' ' || *line == '\t') ++line;
  const char* p = line;
  const char* tag_end = p;
  while (*tag_end && *tag_end != ' ' && *tag_end != '\t' && *tag_end != '\r' && *tag_end != '\n') ++tag_end;
  const std::string tag(p, tag_end);
  p = tag_end;
  if (g->dim == 3 && tag == "VERTEX_SE3:QUAT") {
    uint64_t k;
    double v[7];
    if (!read_key(p, &k) || !read_doubles(p, v, 7)) return false;
    double pose[12];
    rot_from_quaternion(v[6], v[3], v[4], v[5], pose);
    pose[9] = v[0], pose[10] = v[1], pose[11] = v[2];
    g->vkeys.push_back(k);
    g->poses.insert(g->poses.end(), pose, pose + 12);
  } else if (g->dim == 3 && tag == "EDGE_SE3:QUAT") {
    uint64_t a, b;
    double v[28];
    if (!read_key(p, &a) || !read_key(p, &b) || !read_doubles(p, v, 28)) return false;
    double pose[12];
    rot_from_quaternion(v[6], v[3], v[4], v[5], pose);
    pose[9] = v[0], pose[10] = v[1], pose[11] = v[2];
    double Ig[36];
    int k = 7;
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j) Ig[6 * i + j] = Ig[6 * j + i] = v[k++];
    static const int swap[6] = {3, 4, 5, 0, 1, 2};  // g2o [t; R] -> GTSAM [R; t]
    double I[36], cov[36], R[36];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) I[6 * i + j] = Ig[6 * swap[i] + swap[j]];
    if (!noise_from_information(6, I, cov, R)) return false;
    g->kind.push_back(RPGO_FACTOR_BETWEEN);
    g->k1.push_back(a);
    g->k2.push_back(b);
    g->meas.insert(g->meas.end(), pose, pose + 12);
    g->cov.insert(g->cov.end(), cov, cov + 36);
    g->sqrt_info.insert(g->sqrt_info.end(), R, R + 36);
  } else if (g->dim == 2 && tag == "VERTEX_SE2") {
    uint64_t k;
    double v[3];
    if (!read_key(p, &k) || !read_doubles(p, v, 3)) return false;
    const double pose[4] = {std::cos(v[2]), std::sin(v[2]), v[0], v[1]};
    g->vkeys.push_back(k);
    g->poses.insert(g->poses.end(), pose, pose + 4);
  } else if (g->dim == 2 && tag == "EDGE_SE2") {
    uint64_t a, b;
    double v[9];
    if (!read_key(p, &a) || !read_key(p, &b) || !read_doubles(p, v, 9)) return false;
    const double pose[4] = {std::cos(v[2]), std::sin(v[2]), v[0], v[1]};
    const double I[9] = {v[3], v[4], v[5], v[4], v[6], v[7], v[5], v[7], v[8]};
    double cov[9], R[9];
    if (!noise_from_information(3, I, cov, R)) return false;
    g->kind.push_back(RPGO_FACTOR_BETWEEN);
    g->k1.push_back(a);
    g->k2.push_back(b);
    g->meas.insert(g->meas.end(), pose, pose + 4);
    g->cov.insert(g->cov.end(), cov, cov + 9);
    g->sqrt_info.insert(g->sqrt_info.end(), R, R + 9);
  }
  return true;
}

}  // namespace

extern "C" {

rpgo_g2o* rpgo_g2o_read(const char* path, int32_t dim, int32_t* status) {
  int32_t dummy;
  if (!status) status = &dummy;
  if (!path || (dim != 2 && dim != 3)) {
    *status = RPGO_ERR_ARG;
    return nullptr;
  }
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    *status = RPGO_ERR_ARG;
    return nullptr;
  }
  auto* g = new rpgo_g2o;
  g->dim = dim;
  std::string line;
  std::vector<char> buf(1 << 16);
  size_t lineno = 0;
  bool ok = true;
  while (ok && std::fgets(buf.data(), (int)buf.size(), f)) {
    line.assign(buf.data());
    while (!line.empty() && line.back() != '\n' && std::fgets(buf.data(), (int)buf.size(), f)) line += buf.data();
    ++lineno;
    if (!parse_line(g, line.c_str())) {
      std::fprintf(stderr, "rpgo_gb300: %s:%zu: malformed g2o line\n", path, lineno);
      ok = false;
    }
  }
  std::fclose(f);
  if (!ok) {
    delete g;
    *status = RPGO_ERR_ARG;
    return nullptr;
  }
  *status = RPGO_OK;
  return g;
}

int rpgo_g2o_view(const rpgo_g2o* g, rpgo_factor_batch* factors, rpgo_value_batch* values) {
  if (!g) return RPGO_ERR_ARG;
  if (factors)
    *factors = rpgo_factor_batch{(int64_t)g->kind.size(), g->kind.data(), g->k1.data(), g->k2.data(),
                                 g->meas.data(), g->cov.data(), g->sqrt_info.data()};
  if (values) *values = rpgo_value_batch{(int64_t)g->vkeys.size(), g->vkeys.data(), g->poses.data()};
  return RPGO_OK;
}

void rpgo_g2o_free(rpgo_g2o* g) { delete g; }

}  // extern "C"
