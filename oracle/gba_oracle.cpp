// gba_oracle.cpp -- CPU FP64 oracle (TEST INFRASTRUCTURE ONLY; see
// gba_oracle.h).  A restatement of the reference's camera-shared bundle
// adjustment path in plain C++ (no Eigen).  Every function names the
// reference file:line it follows; paths are relative to
// include/hs_sfm/ of the reference project.
#include "gba_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <utility>
#include <vector>

namespace {

typedef std::vector<double> Vec;

// ---------------------------------------------------------------------------
// Problem view: sizes, x layout and constraint rows.
// x layout: sfm bundle_adjustment/camera_shared_vector_function.hpp:349-410.
// ---------------------------------------------------------------------------
struct ConstraintRow {
  int group;        // 0 point, 1 image, 2 camera
  int64_t block;    // point / image / camera id
  int param;        // parameter index inside that block
};

struct Model {
  const gba_problem* p = nullptr;
  int64_t P = 0, I = 0, C = 0, K = 0, cps = 0;
  bool fixP = false, fixI = false, fixC = false;
  bool radial = false, decent = false, intr = false;
  int64_t x_image_begin = 0, x_camera_begin = 0, x_size = 0;
  std::vector<ConstraintRow> rows;  // constraint rows in y order
  int64_t n_priors = 0;             // point priors: 3 rows each after the constraint rows
  int64_t prior_y_begin = 0;
  int64_t y_size = 0;
  std::vector<int32_t> key_image, key_point, key_camera;

  int init(const gba_problem* prob) {
    p = prob;
    if (!p) return GBA_ERR_INVALID;
    P = p->number_of_points; I = p->number_of_images;
    C = p->number_of_cameras; K = p->number_of_keys;
    if (P < 0 || I < 0 || C < 0 || K < 0) return GBA_ERR_INVALID;
    if (K > 0 && !p->feature_maps) return GBA_ERR_INVALID;
    if (I > 0 && !p->image_camera_map) return GBA_ERR_INVALID;
    uint32_t m = p->intrinsic_computations_mask;
    radial = m & GBA_COMPUTE_RADIAL_DISTORTION;
    decent = m & GBA_COMPUTE_DECENTERING_DISTORTION;
    intr = m & GBA_COMPUTE_INTRINSIC_PARAMS;
    cps = (radial ? 3 : 0) + (decent ? 2 : 0) + (intr ? 5 : 0);
    fixP = p->fix_mask & GBA_FIX_POINTS;
    fixI = p->fix_mask & GBA_FIX_IMAGES;
    fixC = p->fix_mask & GBA_FIX_CAMERAS;
    if (fixP && !p->fix_points && P > 0) return GBA_ERR_INVALID;
    if (fixI && !p->fix_images && I > 0) return GBA_ERR_INVALID;
    if (fixC && !p->fix_cameras && C > 0 && cps > 0) return GBA_ERR_INVALID;
    x_image_begin = fixP ? 0 : 3 * P;
    x_camera_begin = x_image_begin + (fixI ? 0 : 6 * I);
    x_size = x_camera_begin + (fixC ? 0 : cps * C);
    key_image.resize(K); key_point.resize(K); key_camera.resize(K);
    for (int64_t i = 0; i < I; ++i) {
      int64_t c = p->image_camera_map[i];
      if (c < 0 || c >= C) return GBA_ERR_BAD_INDEX;
    }
    for (int64_t k = 0; k < K; ++k) {
      int64_t im = p->feature_maps[2 * k], pt = p->feature_maps[2 * k + 1];
      if (im < 0 || im >= I || pt < 0 || pt >= P) return GBA_ERR_BAD_INDEX;
      key_image[k] = int32_t(im); key_point[k] = int32_t(pt);
      key_camera[k] = int32_t(p->image_camera_map[im]);
    }
    // Duplicate (point, image) keys: the reference's point-image block map
    // (camera_shared_normal_equation_builder.hpp:141-155) assumes unique
    // pairs, so they are rejected up front.
    {
      std::vector<std::pair<int32_t, int32_t>> pairs(K);
      for (int64_t k = 0; k < K; ++k) pairs[k] = {key_point[k], key_image[k]};
      std::sort(pairs.begin(), pairs.end());
      for (int64_t k = 1; k < K; ++k)
        if (pairs[k] == pairs[k - 1]) return GBA_ERR_DUPLICATE;
    }
    // Constraint rows in y order (camera_shared_vector_function.hpp:483-629;
    // camera_shared_jacobian_matrix.hpp SetPoint/Image/CameraConstraints).
    rows.clear();
    if (!fixP) {
      for (int64_t c = 0; c < p->number_of_point_constraints; ++c) {
        const gba_point_constraint& pc = p->point_constraints[c];
        if (pc.point_id < 0 || pc.point_id >= P) return GBA_ERR_BAD_INDEX;
        for (int b = 0; b < 3; ++b)
          if (pc.mask & (1u << b)) rows.push_back({0, pc.point_id, b});
      }
    }
    if (!fixI) {
      for (int64_t c = 0; c < p->number_of_image_constraints; ++c) {
        const gba_image_constraint& ic = p->image_constraints[c];
        if (ic.image_id < 0 || ic.image_id >= I) return GBA_ERR_BAD_INDEX;
        if (ic.mask & GBA_IMAGE_CONSTRAIN_ROTATION)
          for (int b = 0; b < 3; ++b) rows.push_back({1, ic.image_id, b});
        if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_X) rows.push_back({1, ic.image_id, 3});
        if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_Y) rows.push_back({1, ic.image_id, 4});
        if (ic.mask & GBA_IMAGE_CONSTRAIN_POSITION_Z) rows.push_back({1, ic.image_id, 5});
      }
    }
    if (!fixC) {
      for (int64_t c = 0; c < p->number_of_camera_constraints; ++c) {
        const gba_camera_constraint& cc = p->camera_constraints[c];
        if (cc.camera_id < 0 || cc.camera_id >= C) return GBA_ERR_BAD_INDEX;
        // :549-557 -- a constraint on a group that is not computed fails.
        if ((cc.radial_mask && !radial) || (cc.decentering_mask && !decent) ||
            (cc.intrinsic_mask && !intr))
          return GBA_ERR;
        int off = 0;
        for (int b = 0; b < 3; ++b)
          if (cc.radial_mask & (1u << b)) rows.push_back({2, cc.camera_id, off + b});
        if (radial) off += 3;
        for (int b = 0; b < 2; ++b)
          if (cc.decentering_mask & (1u << b)) rows.push_back({2, cc.camera_id, off + b});
        if (decent) off += 2;
        for (int b = 0; b < 5; ++b)
          if (cc.intrinsic_mask & (1u << b)) rows.push_back({2, cc.camera_id, off + b});
      }
    }
    // Point priors (ba_gcp_constrained_vector_function.hpp:60-110): copies
    // of the prior points' coordinates, weighted by a 3x3 block each.
    n_priors = p->number_of_point_priors;
    if (n_priors < 0 || (n_priors > 0 && (!p->point_prior_ids || fixP))) return GBA_ERR_INVALID;
    for (int64_t i = 0; i < n_priors; ++i)
      if (p->point_prior_ids[i] < 0 || p->point_prior_ids[i] >= P) return GBA_ERR_BAD_INDEX;
    prior_y_begin = 2 * K + int64_t(rows.size());
    y_size = prior_y_begin + 3 * n_priors;
    return GBA_OK;
  }

  // Inverse covariance of prior i (ba_gcp_constrained_y_covariance_inverse.hpp:18-25).
  void prior_weight(int64_t i, double L[9]) const {
    for (int j = 0; j < 9; ++j)
      L[j] = p->point_prior_information ? p->point_prior_information[9 * i + j] : (j % 4 == 0);
  }

  const double* point(int64_t id, const double* x) const {
    return fixP ? p->fix_points + 3 * id : x + 3 * id;
  }
  const double* image(int64_t id, const double* x) const {
    return fixI ? p->fix_images + 6 * id : x + x_image_begin + 6 * id;
  }
  const double* camera(int64_t id, const double* x) const {
    return fixC ? p->fix_cameras + cps * id : x + x_camera_begin + cps * id;
  }
  int64_t row_x_index(const ConstraintRow& r) const {
    if (r.group == 0) return 3 * r.block + r.param;
    if (r.group == 1) return x_image_begin + 6 * r.block + r.param;
    return x_camera_begin + cps * r.block + r.param;
  }
  void key_weight(int64_t k, double L[4]) const {
    if (p->key_covariance_inverse) {
      for (int j = 0; j < 4; ++j) L[j] = p->key_covariance_inverse[4 * k + j];
    } else {
      L[0] = 1; L[1] = 0; L[2] = 0; L[3] = 1;
    }
  }
  double row_weight(int64_t r) const {
    return p->constraint_weights ? p->constraint_weights[r] : 1.0;
  }
};

// ---------------------------------------------------------------------------
// Projection: camera_shared_vector_function.hpp:634-744,
// sfm_utility/radial_distortor.hpp:14-28, decentering_distortor.hpp:14-24.
// ---------------------------------------------------------------------------
void normalized_key(const double X[3], const double r[3], const double t[3],
                    double n[2]) {  // :688-710
  double theta = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  double c[3];
  if (theta == 0.0) {
    for (int i = 0; i < 3; ++i) c[i] = X[i] + t[i];
  } else {
    double nr[3] = {r[0] / theta, r[1] / theta, r[2] / theta};
    double ct = std::cos(theta), st = std::sin(theta);
    double cr[3] = {nr[1] * X[2] - nr[2] * X[1], nr[2] * X[0] - nr[0] * X[2],
                    nr[0] * X[1] - nr[1] * X[0]};
    double d = X[0] * nr[0] + X[1] * nr[1] + X[2] * nr[2];
    for (int i = 0; i < 3; ++i)
      c[i] = ct * X[i] + st * cr[i] + (1 - ct) * d * nr[i] + t[i];
  }
  n[0] = c[0] / c[2];
  n[1] = c[1] / c[2];
}

void radial_delta(double k1, double k2, double k3, double x, double y,
                  double& dx, double& dy) {  // radial_distortor.hpp:14-28
  double r2 = x * x + y * y, r4 = r2 * r2, r6 = r2 * r4;
  double coeff = k1 * r2 + k2 * r4 + k3 * r6;
  dx = coeff * x;
  dy = coeff * y;
}

void decentering_delta(double d1, double d2, double x, double y, double& dx,
                       double& dy) {  // decentering_distortor.hpp:14-24
  double r2 = x * x + y * y;
  dx = 2 * d1 * x * y + d2 * (r2 + 2 * x * x);
  dy = 2 * d2 * x * y + d1 * (r2 + 2 * y * y);
}

void image_key(const Model& m, const double X[3], const double* im,
               const double* cam, double out[2]) {  // :634-686
  double n[2];
  normalized_key(X, im, im + 3, n);
  int off = 0;
  double rd[2] = {0, 0}, dd[2] = {0, 0};
  if (m.radial) {
    radial_delta(cam[0], cam[1], cam[2], n[0], n[1], rd[0], rd[1]);
    off += 3;
  }
  if (m.decent) {
    decentering_delta(cam[off], cam[off + 1], n[0], n[1], dd[0], dd[1]);
    off += 2;
  }
  n[0] += rd[0] + dd[0];
  n[1] += rd[1] + dd[1];
  if (m.intr) {  // NormalizedKeyToImageKey :731-744
    double f = cam[off], s = cam[off + 1], cx = cam[off + 2],
           cy = cam[off + 3], a = cam[off + 4];
    out[0] = f * n[0] + s * n[1] + cx;
    out[1] = f * a * n[1] + cy;
  } else {
    out[0] = n[0];
    out[1] = n[1];
  }
}

// ---------------------------------------------------------------------------
// Analytical derivatives:
// camera_shared_analytical_jacobian_matrix_calculator.hpp:334-557.
// Matrices are row-major: A[r][c].
// ---------------------------------------------------------------------------
void normalized_point_derivation(const double p[3], const double r[3],
                                 const double t[3], double pnpe[2][6],
                                 double pnpp[2][3]) {  // :334-429
  double theta = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  double theta2 = theta * theta, theta4 = theta2 * theta2;
  double d = r[0] * p[0] + r[1] * p[1] + r[2] * p[2];
  double st = std::sin(theta), ct = std::cos(theta);
  double f[3] = {ct * p[0], ct * p[1], ct * p[2]};
  double pfpr[3][3], pfpp[3][3] = {{ct, 0, 0}, {0, ct, 0}, {0, 0, ct}};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) pfpr[i][j] = p[i] * (-st / theta * r[j]);
  double s = st / theta;
  double pspr[3];
  for (int i = 0; i < 3; ++i) pspr[i] = (ct * theta - st) / theta2 / theta * r[i];
  double v[3] = {r[1] * p[2] - r[2] * p[1], r[2] * p[0] - r[0] * p[2],
                 r[0] * p[1] - r[1] * p[0]};
  double pvpr[3][3] = {{0, p[2], -p[1]}, {-p[2], 0, p[0]}, {p[1], -p[0], 0}};
  double pvpp[3][3] = {{0, -r[2], r[1]}, {r[2], 0, -r[0]}, {-r[1], r[0], 0}};
  double c = (1 - ct) / theta2;
  double pcpr[3];
  for (int i = 0; i < 3; ++i) pcpr[i] = (st * theta - 2 * (1 - ct)) / theta4 * r[i];
  double u[3] = {d * r[0], d * r[1], d * r[2]};
  double pupr[3][3], pupp[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      pupr[i][j] = (i == j ? d : 0.0) + r[i] * p[j];
      pupp[i][j] = r[i] * r[j];
    }
  double y[3];
  for (int i = 0; i < 3; ++i) y[i] = f[i] + s * v[i] + c * u[i] + t[i];
  double pypr[3][3], pypp[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      pypr[i][j] = pfpr[i][j] + v[i] * pspr[j] + s * pvpr[i][j] +
                   u[i] * pcpr[j] + c * pupr[i][j];
      pypp[i][j] = pfpp[i][j] + s * pvpp[i][j] + c * pupp[i][j];
    }
  for (int m = 0; m < 3; ++m) {
    pnpe[0][m] = (pypr[0][m] * y[2] - y[0] * pypr[2][m]) / y[2] / y[2];
    pnpe[1][m] = (pypr[1][m] * y[2] - y[1] * pypr[2][m]) / y[2] / y[2];
    double e0 = (m == 0), e1 = (m == 1), e2 = (m == 2);  // pypt = I
    pnpe[0][3 + m] = (e0 * y[2] - y[0] * e2) / y[2] / y[2];
    pnpe[1][3 + m] = (e1 * y[2] - y[1] * e2) / y[2] / y[2];
  }
  for (int m = 0; m < 3; ++m) {
    pnpp[0][m] = (pypp[0][m] * y[2] - y[0] * pypp[2][m]) / y[2] / y[2];
    pnpp[1][m] = (pypp[1][m] * y[2] - y[1] * pypp[2][m]) / y[2] / y[2];
  }
}

void radial_derivation(const double n[2], const double pnpp[2][3],
                       const double pnpe[2][6], double k1, double k2,
                       double k3, double prdpp[2][3], double prdpe[2][6],
                       double prdpr[2][3]) {  // :431-470
  double r2 = n[0] * n[0] + n[1] * n[1], r4 = r2 * r2, r6 = r2 * r4;
  double coeff = k1 * r2 + k2 * r4 + k3 * r6;
  for (int j = 0; j < 3; ++j) {
    double pr2 = 2 * n[0] * pnpp[0][j] + 2 * n[1] * pnpp[1][j];
    double pr4 = 2 * r2 * pr2, pr6 = 3 * r4 * pr2;
    double cd = k1 * pr2 + k2 * pr4 + k3 * pr6;
    prdpp[0][j] = cd * n[0] + coeff * pnpp[0][j];
    prdpp[1][j] = cd * n[1] + coeff * pnpp[1][j];
  }
  for (int j = 0; j < 6; ++j) {
    double pr2 = 2 * n[0] * pnpe[0][j] + 2 * n[1] * pnpe[1][j];
    double pr4 = 2 * r2 * pr2, pr6 = 3 * r4 * pr2;
    double cd = k1 * pr2 + k2 * pr4 + k3 * pr6;
    prdpe[0][j] = cd * n[0] + coeff * pnpe[0][j];
    prdpe[1][j] = cd * n[1] + coeff * pnpe[1][j];
  }
  prdpr[0][0] = r2 * n[0]; prdpr[0][1] = r4 * n[0]; prdpr[0][2] = r6 * n[0];
  prdpr[1][0] = r2 * n[1]; prdpr[1][1] = r4 * n[1]; prdpr[1][2] = r6 * n[1];
}

void decentering_derivation(const double n[2], const double pnpp[2][3],
                            const double pnpe[2][6], double d1, double d2,
                            double pddpp[2][3], double pddpe[2][6],
                            double pddpd[2][2]) {  // :472-503
  double r2 = n[0] * n[0] + n[1] * n[1];
  for (int j = 0; j < 3; ++j) {
    double pr2 = 2 * n[0] * pnpp[0][j] + 2 * n[1] * pnpp[1][j];
    double cross = pnpp[0][j] * n[1] + pnpp[1][j] * n[0];
    pddpp[0][j] = 2 * d1 * cross + d2 * (pr2 + 4 * n[0] * pnpp[0][j]);
    pddpp[1][j] = 2 * d2 * cross + d1 * (pr2 + 4 * n[1] * pnpp[1][j]);
  }
  for (int j = 0; j < 6; ++j) {
    double pr2 = 2 * n[0] * pnpe[0][j] + 2 * n[1] * pnpe[1][j];
    double cross = pnpe[0][j] * n[1] + pnpe[1][j] * n[0];
    pddpe[0][j] = 2 * d1 * cross + d2 * (pr2 + 4 * n[0] * pnpe[0][j]);
    pddpe[1][j] = 2 * d2 * cross + d1 * (pr2 + 4 * n[1] * pnpe[1][j]);
  }
  pddpd[0][0] = 2 * n[0] * n[1]; pddpd[0][1] = r2 + 2 * n[0] * n[0];
  pddpd[1][0] = r2 + 2 * n[1] * n[1]; pddpd[1][1] = 2 * n[0] * n[1];
}

// One key's Jacobian blocks (the loop body of :94-321).  jp 2x3, ji 2x6,
// jc 2xcps, all row-major.
void key_jacobian(const Model& m, const double X[3], const double* im,
                  const double* cam, double jp[6], double ji[12],
                  double* jc) {
  double n[2];
  normalized_key(X, im, im + 3, n);
  double pnpp[2][3], pnpe[2][6];
  normalized_point_derivation(X, im, im + 3, pnpe, pnpp);
  int off = 0;
  double prdpr[2][3] = {}, prdpp[2][3] = {}, prdpe[2][6] = {}, rd[2] = {0, 0};
  if (m.radial) {
    radial_delta(cam[0], cam[1], cam[2], n[0], n[1], rd[0], rd[1]);
    radial_derivation(n, pnpp, pnpe, cam[0], cam[1], cam[2], prdpp, prdpe, prdpr);
    off += 3;
  }
  double pddpd[2][2] = {}, pddpp[2][3] = {}, pddpe[2][6] = {}, dd[2] = {0, 0};
  if (m.decent) {
    decentering_delta(cam[off], cam[off + 1], n[0], n[1], dd[0], dd[1]);
    decentering_derivation(n, pnpp, pnpe, cam[off], cam[off + 1], pddpp, pddpe, pddpd);
    off += 2;
  }
  if (m.radial) {
    n[0] += rd[0]; n[1] += rd[1];
    for (int r = 0; r < 2; ++r) {
      for (int j = 0; j < 3; ++j) pnpp[r][j] += prdpp[r][j];
      for (int j = 0; j < 6; ++j) pnpe[r][j] += prdpe[r][j];
    }
  }
  if (m.decent) {
    n[0] += dd[0]; n[1] += dd[1];
    for (int r = 0; r < 2; ++r) {
      for (int j = 0; j < 3; ++j) pnpp[r][j] += pddpp[r][j];
      for (int j = 0; j < 6; ++j) pnpe[r][j] += pddpe[r][j];
    }
  }
  int cps = int(m.cps);
  if (m.intr) {
    double f = cam[off], s = cam[off + 1], cx = cam[off + 2],
           cy = cam[off + 3], a = cam[off + 4];
    (void)cx; (void)cy;
    for (int j = 0; j < 3; ++j) {  // IntrinsicPointDerivation :505-513
      jp[j] = f * pnpp[0][j] + s * pnpp[1][j];
      jp[3 + j] = f * a * pnpp[1][j];
    }
    for (int j = 0; j < 6; ++j) {  // IntrinsicExtrinsicDerivation :515-524
      ji[j] = f * pnpe[0][j] + s * pnpe[1][j];
      ji[6 + j] = f * a * pnpe[1][j];
    }
    if (jc) {
      int o = 0;
      if (m.radial) {  // IntrinsicRadialDerivation :526-534
        for (int j = 0; j < 3; ++j) {
          jc[o + j] = f * prdpr[0][j] + s * prdpr[1][j];
          jc[cps + o + j] = f * a * prdpr[1][j];
        }
        o += 3;
      }
      if (m.decent) {  // IntrinsicDecenteringDerivation :536-544
        for (int j = 0; j < 2; ++j) {
          jc[o + j] = f * pddpd[0][j] + s * pddpd[1][j];
          jc[cps + o + j] = f * a * pddpd[1][j];
        }
        o += 2;
      }
      // IntrinsicIntrinsicDerivation :546-557
      jc[o + 0] = n[0]; jc[o + 1] = n[1]; jc[o + 2] = 1; jc[o + 3] = 0; jc[o + 4] = 0;
      jc[cps + o + 0] = a * n[1]; jc[cps + o + 1] = 0; jc[cps + o + 2] = 0;
      jc[cps + o + 3] = 1; jc[cps + o + 4] = f * n[1];
    }
  } else {
    for (int j = 0; j < 3; ++j) { jp[j] = pnpp[0][j]; jp[3 + j] = pnpp[1][j]; }
    for (int j = 0; j < 6; ++j) { ji[j] = pnpe[0][j]; ji[6 + j] = pnpe[1][j]; }
    if (jc) {
      int o = 0;
      if (m.radial) {
        for (int j = 0; j < 3; ++j) { jc[o + j] = prdpr[0][j]; jc[cps + o + j] = prdpr[1][j]; }
        o += 3;
      }
      if (m.decent) {
        for (int j = 0; j < 2; ++j) { jc[o + j] = pddpd[0][j]; jc[cps + o + j] = pddpd[1][j]; }
        o += 2;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Residuals, weights and cost.
// camera_shared_mahalanobis_distance_calculator.hpp:28-58 (F = sum r^T L r);
// Huber as restated from the reference's Ceres path
// (camera_shared_ceres_optimizor.hpp:253): rho(s) = s for s <= d^2, else
// 2 d sqrt(s) - d^2, IRLS weight rho'(s).
// ---------------------------------------------------------------------------
struct Loss {
  int32_t kind = GBA_LOSS_TRIVIAL;
  double delta = 1.0;
  double rho(double s) const {
    if (kind == GBA_LOSS_HUBER && s > delta * delta)
      return 2 * delta * std::sqrt(s) - delta * delta;
    return s;
  }
  double weight(double s) const {
    if (kind == GBA_LOSS_HUBER && s > delta * delta) return delta / std::sqrt(s);
    return 1.0;
  }
};

int residuals(const Model& m, const double* x, const double* near_y, Vec& r) {
  r.assign(m.y_size, 0.0);
  for (int64_t k = 0; k < m.K; ++k) {
    double key[2];
    image_key(m, m.point(m.key_point[k], x), m.image(m.key_image[k], x),
              m.camera(m.key_camera[k], x), key);
    r[2 * k] = key[0] - near_y[2 * k];  // r = f(x) - y
    r[2 * k + 1] = key[1] - near_y[2 * k + 1];
  }
  for (size_t c = 0; c < m.rows.size(); ++c) {
    int64_t yi = 2 * m.K + int64_t(c);
    r[yi] = x[m.row_x_index(m.rows[c])] - near_y[yi];
  }
  for (int64_t i = 0; i < m.n_priors; ++i)
    for (int a = 0; a < 3; ++a) {
      const int64_t yi = m.prior_y_begin + 3 * i + a;
      r[yi] = x[3 * m.p->point_prior_ids[i] + a] - near_y[yi];
    }
  return GBA_OK;
}

// r^T L r of prior i (ba_gcp_constrained_mahalanobis_distance_calculator.hpp:55-62).
double prior_sq(const Model& m, int64_t i, const double* r) {
  double L[9];
  m.prior_weight(i, L);
  const double* v = r + m.prior_y_begin + 3 * i;
  double s = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) s += v[a] * L[3 * a + b] * v[b];
  return s;
}

double key_sq(const Model& m, int64_t k, const double* r) {
  double L[4];
  m.key_weight(k, L);
  double a = r[2 * k], b = r[2 * k + 1];
  return a * (L[0] * a + L[1] * b) + b * (L[2] * a + L[3] * b);
}

double cost_of(const Model& m, const Vec& r, const Loss& loss) {
  double F = 0;
  for (int64_t k = 0; k < m.K; ++k) F += loss.rho(key_sq(m, k, r.data()));
  for (size_t c = 0; c < m.rows.size(); ++c) {
    double v = r[2 * m.K + c];
    F += v * m.row_weight(int64_t(c)) * v;
  }
  for (int64_t i = 0; i < m.n_priors; ++i) F += prior_sq(m, i, r.data());
  return F;
}

// ---------------------------------------------------------------------------
// Block normal equations:
// camera_shared_normal_equation_builder.hpp:111-462.
// ---------------------------------------------------------------------------
struct Blocks {
  int64_t cps = 0;
  Vec V;       // P x 9   point blocks
  Vec U;       // I x 36  image blocks
  Vec Cb;      // C x cps^2 camera blocks
  Vec W;       // K x 18  point-image blocks (one per key; unique pairs)
  // point-camera and image-camera blocks: unique pairs, summed over keys.
  std::vector<std::pair<int32_t, int32_t>> pc_pairs, ic_pairs;  // (p,c), (i,c)
  std::vector<int64_t> key_pc, key_ic;                          // key -> pair
  Vec Wc;      // npc x 3*cps
  Vec E;       // nic x 6*cps
  Vec gp, gi, gc;
};

// out += A^T L B with A 2xa, B 2xb (row-major), out a x b.
inline void add_atlb(const double* A, int a, const double* B, int b,
                     const double L[4], double* out, double scale = 1.0) {
  for (int i = 0; i < a; ++i) {
    double l0 = (A[i] * L[0] + A[a + i] * L[2]) * scale;
    double l1 = (A[i] * L[1] + A[a + i] * L[3]) * scale;
    for (int j = 0; j < b; ++j) out[i * b + j] += l0 * B[j] + l1 * B[b + j];
  }
}

int build_blocks(const Model& m, const double* x, const Vec& r,
                 const Loss& loss, Blocks& B) {
  const int64_t cps = m.cps;
  B.cps = cps;
  B.V.assign(m.fixP ? 0 : m.P * 9, 0.0);
  B.U.assign(m.fixI ? 0 : m.I * 36, 0.0);
  B.Cb.assign(m.fixC ? 0 : m.C * cps * cps, 0.0);
  B.W.assign((m.fixP || m.fixI) ? 0 : m.K * 18, 0.0);
  B.gp.assign(m.fixP ? 0 : m.P * 3, 0.0);
  B.gi.assign(m.fixI ? 0 : m.I * 6, 0.0);
  B.gc.assign(m.fixC ? 0 : m.C * cps, 0.0);
  B.pc_pairs.clear(); B.ic_pairs.clear();
  B.key_pc.assign(m.K, -1); B.key_ic.assign(m.K, -1);
  if (!m.fixP && !m.fixC) {  // std::set of (point, camera) :157-181
    std::vector<std::pair<std::pair<int32_t, int32_t>, int64_t>> t(m.K);
    for (int64_t k = 0; k < m.K; ++k) t[k] = {{m.key_point[k], m.key_camera[k]}, k};
    std::sort(t.begin(), t.end());
    for (int64_t k = 0; k < m.K; ++k) {
      if (k == 0 || t[k].first != t[k - 1].first) B.pc_pairs.push_back(t[k].first);
      B.key_pc[t[k].second] = int64_t(B.pc_pairs.size()) - 1;
    }
  }
  if (!m.fixI && !m.fixC) {  // std::set of (image, camera) :182-205
    std::vector<std::pair<std::pair<int32_t, int32_t>, int64_t>> t(m.K);
    for (int64_t k = 0; k < m.K; ++k) t[k] = {{m.key_image[k], m.key_camera[k]}, k};
    std::sort(t.begin(), t.end());
    for (int64_t k = 0; k < m.K; ++k) {
      if (k == 0 || t[k].first != t[k - 1].first) B.ic_pairs.push_back(t[k].first);
      B.key_ic[t[k].second] = int64_t(B.ic_pairs.size()) - 1;
    }
  }
  B.Wc.assign(B.pc_pairs.size() * 3 * cps, 0.0);
  B.E.assign(B.ic_pairs.size() * 6 * cps, 0.0);

  std::vector<double> jc(2 * std::max<int64_t>(cps, 1));
  for (int64_t k = 0; k < m.K; ++k) {
    double jp[6], ji[12];
    key_jacobian(m, m.point(m.key_point[k], x), m.image(m.key_image[k], x),
                 m.camera(m.key_camera[k], x), jp, ji, jc.data());
    double L[4];
    m.key_weight(k, L);
    double w = loss.weight(key_sq(m, k, r.data()));
    const double* rk = &r[2 * k];
    int32_t pt = m.key_point[k], im = m.key_image[k], cam = m.key_camera[k];
    if (!m.fixP) {
      add_atlb(jp, 3, jp, 3, L, &B.V[9 * pt], w);
      add_atlb(jp, 3, rk, 1, L, &B.gp[3 * pt], w);
    }
    if (!m.fixI) {
      add_atlb(ji, 6, ji, 6, L, &B.U[36 * im], w);
      add_atlb(ji, 6, rk, 1, L, &B.gi[6 * im], w);
    }
    if (!m.fixC) {
      add_atlb(jc.data(), int(cps), jc.data(), int(cps), L, &B.Cb[cps * cps * cam], w);
      add_atlb(jc.data(), int(cps), rk, 1, L, &B.gc[cps * cam], w);
    }
    if (!m.fixP && !m.fixI) add_atlb(jp, 3, ji, 6, L, &B.W[18 * k], w);
    if (!m.fixP && !m.fixC)
      add_atlb(jp, 3, jc.data(), int(cps), L, &B.Wc[3 * cps * B.key_pc[k]], w);
    if (!m.fixI && !m.fixC)
      add_atlb(ji, 6, jc.data(), int(cps), L, &B.E[6 * cps * B.key_ic[k]], w);
  }
  // Constraint rows: diagonal weight and weighted residual (:309-349, :418-459).
  for (size_t c = 0; c < m.rows.size(); ++c) {
    const ConstraintRow& row = m.rows[c];
    double wgt = m.row_weight(int64_t(c));
    double rv = r[2 * m.K + c];
    if (row.group == 0) {
      B.V[9 * row.block + 4 * row.param] += wgt;
      B.gp[3 * row.block + row.param] += wgt * rv;
    } else if (row.group == 1) {
      B.U[36 * row.block + 7 * row.param] += wgt;
      B.gi[6 * row.block + row.param] += wgt * rv;
    } else {
      B.Cb[cps * cps * row.block + (cps + 1) * row.param] += wgt;
      B.gc[cps * row.block + row.param] += wgt * rv;
    }
  }
  // Point priors: V_p += L, g_p += L r (ba_gcp_constrained_normal_equation_builder.hpp:59-72).
  for (int64_t i = 0; i < m.n_priors; ++i) {
    double L[9];
    m.prior_weight(i, L);
    const int64_t pt = m.p->point_prior_ids[i];
    const double* v = &r[m.prior_y_begin + 3 * i];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        B.V[9 * pt + 3 * a + b] += L[3 * a + b];
        B.gp[3 * pt + a] += L[3 * a + b] * v[b];
      }
  }
  return GBA_OK;
}

void blocks_to_dense(const Model& m, const Blocks& B, double* N, double* g) {
  const int64_t n = m.x_size, cps = m.cps;
  std::fill(N, N + n * n, 0.0);
  auto put = [&](int64_t r0, int64_t c0, const double* blk, int rows, int cols, bool sym) {
    for (int i = 0; i < rows; ++i)
      for (int j = 0; j < cols; ++j) {
        N[(r0 + i) * n + c0 + j] += blk[i * cols + j];
        if (sym) N[(c0 + j) * n + r0 + i] += blk[i * cols + j];
      }
  };
  if (!m.fixP) for (int64_t p = 0; p < m.P; ++p) put(3 * p, 3 * p, &B.V[9 * p], 3, 3, false);
  if (!m.fixI) for (int64_t i = 0; i < m.I; ++i)
    put(m.x_image_begin + 6 * i, m.x_image_begin + 6 * i, &B.U[36 * i], 6, 6, false);
  if (!m.fixC) for (int64_t c = 0; c < m.C; ++c)
    put(m.x_camera_begin + cps * c, m.x_camera_begin + cps * c, &B.Cb[cps * cps * c], int(cps), int(cps), false);
  if (!m.fixP && !m.fixI) for (int64_t k = 0; k < m.K; ++k)
    put(3 * m.key_point[k], m.x_image_begin + 6 * m.key_image[k], &B.W[18 * k], 3, 6, true);
  for (size_t q = 0; q < B.pc_pairs.size(); ++q)
    put(3 * B.pc_pairs[q].first, m.x_camera_begin + cps * B.pc_pairs[q].second,
        &B.Wc[3 * cps * q], 3, int(cps), true);
  for (size_t q = 0; q < B.ic_pairs.size(); ++q)
    put(m.x_image_begin + 6 * B.ic_pairs[q].first, m.x_camera_begin + cps * B.ic_pairs[q].second,
        &B.E[6 * cps * q], 6, int(cps), true);
  if (g) {
    int64_t o = 0;
    for (double v : B.gp) g[o++] = v;
    for (double v : B.gi) g[o++] = v;
    for (double v : B.gc) g[o++] = v;
  }
}

// ---------------------------------------------------------------------------
// Small dense helpers.
// ---------------------------------------------------------------------------
// 3x3 inverse by cofactors (the closed form Eigen uses for fixed 3x3,
// camera_shared_normal_equation_solver.hpp:148 calls .inverse()).
void inverse3(const double A[9], double R[9]) {
  double c00 = A[4] * A[8] - A[5] * A[7];
  double c01 = A[5] * A[6] - A[3] * A[8];
  double c02 = A[3] * A[7] - A[4] * A[6];
  double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
  double id = 1.0 / det;
  R[0] = c00 * id; R[1] = (A[2] * A[7] - A[1] * A[8]) * id; R[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  R[3] = c01 * id; R[4] = (A[0] * A[8] - A[2] * A[6]) * id; R[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  R[6] = c02 * id; R[7] = (A[1] * A[6] - A[0] * A[7]) * id; R[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

// Dense LDL^T (no pivoting): the restatement of Eigen::SimplicialLDLT used
// at camera_shared_normal_equation_solver.hpp:448-466.  It fails, as
// SimplicialLDLT does, on a zero (or non-finite) pivot.  A is n x n
// row-major, overwritten by L (strict lower) and D (diagonal).
int ldlt_factor(std::vector<double>& A, int64_t n) {
  std::vector<double> t(n);
  for (int64_t j = 0; j < n; ++j) {
    double* Aj = &A[j * n];
    for (int64_t k = 0; k < j; ++k) t[k] = Aj[k] * A[k * n + k];  // L_jk d_k
    double d = Aj[j];
    for (int64_t k = 0; k < j; ++k) d -= Aj[k] * t[k];
    if (d == 0.0 || !std::isfinite(d)) return GBA_ERR_NOT_SPD;
    Aj[j] = d;
    for (int64_t i = j + 1; i < n; ++i) {
      double* Ai = &A[i * n];
      double s = Ai[j];
      for (int64_t k = 0; k < j; ++k) s -= Ai[k] * t[k];
      Ai[j] = s / d;
    }
  }
  return GBA_OK;
}

void ldlt_solve(const std::vector<double>& A, int64_t n, double* b) {
  for (int64_t i = 0; i < n; ++i) {
    double s = b[i];
    for (int64_t k = 0; k < i; ++k) s -= A[i * n + k] * b[k];
    b[i] = s;
  }
  for (int64_t i = 0; i < n; ++i) b[i] /= A[i * n + i];
  for (int64_t i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int64_t k = i + 1; k < n; ++k) s -= A[k * n + i] * b[k];
    b[i] = s;
  }
}

// C (r x c) = A (r x k) * B (k x c), accumulate with sign.
inline void gemm_acc(const double* A, const double* Bm, double* Cm, int r,
                     int k, int c, double sign) {
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j) {
      double s = 0;
      for (int q = 0; q < k; ++q) s += A[i * k + q] * Bm[q * c + j];
      Cm[i * c + j] += sign * s;
    }
}

// ---------------------------------------------------------------------------
// Sparse block maps with the lookup cost of Eigen::SparseMatrix::coeff
// (a binary search over the inner indices of one outer vector).
// ---------------------------------------------------------------------------
struct Csc {
  std::vector<int64_t> outer;   // size n_outer + 1
  std::vector<int32_t> inner;   // sorted per outer
  std::vector<int64_t> value;   // block index + 1 (0 = absent)
  void build(int64_t n_outer, const std::vector<std::pair<int32_t, int32_t>>& outer_inner,
             const std::vector<int64_t>& vals) {
    outer.assign(n_outer + 1, 0);
    for (auto& oi : outer_inner) outer[oi.first + 1]++;
    for (int64_t i = 0; i < n_outer; ++i) outer[i + 1] += outer[i];
    std::vector<std::pair<int32_t, int64_t>> tmp(outer_inner.size());
    std::vector<int64_t> cur(outer.begin(), outer.end() - 1);
    for (size_t e = 0; e < outer_inner.size(); ++e)
      tmp[cur[outer_inner[e].first]++] = {outer_inner[e].second, vals[e]};
    inner.resize(tmp.size()); value.resize(tmp.size());
    for (int64_t o = 0; o < n_outer; ++o) {
      std::sort(tmp.begin() + outer[o], tmp.begin() + outer[o + 1]);
      for (int64_t e = outer[o]; e < outer[o + 1]; ++e) {
        inner[e] = tmp[e].first;
        value[e] = tmp[e].second;
      }
    }
  }
  int64_t coeff(int32_t in, int64_t out) const {
    auto b = inner.begin() + outer[out], e = inner.begin() + outer[out + 1];
    auto it = std::lower_bound(b, e, in);
    if (it == e || *it != in) return 0;
    return value[it - inner.begin()];
  }
};

// ---------------------------------------------------------------------------
// Schur-complement solve:
// camera_shared_normal_equation_solver.hpp:75-706.
// ---------------------------------------------------------------------------
struct SchurTiming {
  double reduce = 0, factor = 0, backsub = 0;
  int row_stride = 1;
};

int solve_points_only(const Model& m, const Blocks& B, double mu, double* dx) {  // :540-569
  for (int64_t p = 0; p < m.P; ++p) {
    double V[9], Vi[9];
    std::memcpy(V, &B.V[9 * p], sizeof V);
    V[0] += mu; V[4] += mu; V[8] += mu;
    inverse3(V, Vi);
    for (int i = 0; i < 3; ++i)
      dx[3 * p + i] = Vi[3 * i] * B.gp[3 * p] + Vi[3 * i + 1] * B.gp[3 * p + 1] +
                      Vi[3 * i + 2] * B.gp[3 * p + 2];
  }
  return GBA_OK;
}

int solve_images_cameras_only(const Model& m, const Blocks& B, double mu,
                              double* dx) {  // :571-706
  const int64_t cps = m.cps;
  const int64_t ib = m.fixI ? 0 : 6 * m.I;
  const int64_t n = ib + (m.fixC ? 0 : cps * m.C);
  std::vector<double> S(n * n, 0.0);
  if (!m.fixI)
    for (int64_t i = 0; i < m.I; ++i)
      for (int a = 0; a < 6; ++a)
        for (int b = 0; b < 6; ++b)
          S[(6 * i + a) * n + 6 * i + b] = B.U[36 * i + 6 * a + b] + (a == b ? mu : 0.0);
  if (!m.fixC)
    for (int64_t c = 0; c < m.C; ++c)
      for (int a = 0; a < cps; ++a)
        for (int b = 0; b < cps; ++b)
          S[(ib + cps * c + a) * n + ib + cps * c + b] =
              B.Cb[cps * cps * c + cps * a + b] + (a == b ? mu : 0.0);
  for (size_t q = 0; q < B.ic_pairs.size(); ++q) {
    int64_t i = B.ic_pairs[q].first, c = B.ic_pairs[q].second;
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < cps; ++b) {
        double v = B.E[6 * cps * q + cps * a + b];
        S[(6 * i + a) * n + ib + cps * c + b] += v;
        S[(ib + cps * c + b) * n + 6 * i + a] += v;
      }
  }
  std::vector<double> rhs(n);
  for (int64_t j = 0; j < int64_t(B.gi.size()); ++j) rhs[j] = B.gi[j];
  for (int64_t j = 0; j < int64_t(B.gc.size()); ++j) rhs[ib + j] = B.gc[j];
  int err = ldlt_factor(S, n);
  if (err) return err;
  ldlt_solve(S, n, rhs.data());
  std::copy(rhs.begin(), rhs.end(), dx);
  return GBA_OK;
}

// The reduced camera system S, rhs b for points eliminated.  faithful keeps
// the reference's loop nest (:138-420); otherwise point-major accumulation.
int reduced_system(const Model& m, const Blocks& B, double mu, bool faithful,
                   int row_stride, std::vector<double>& S, std::vector<double>& b,
                   std::vector<double>& Vinv) {
  const int64_t P = m.P, I = m.I, C = m.C, cps = m.cps;
  const int64_t cb = m.fixI ? 0 : 6 * I;           // cameras_begin
  const int64_t n = cb + (m.fixC ? 0 : cps * C);   // reduced_size
  S.assign(n * n, 0.0);
  b.assign(n, 0.0);
  Vinv.assign(P * 9, 0.0);
  for (int64_t p = 0; p < P; ++p) {  // :141-148
    double V[9];
    std::memcpy(V, &B.V[9 * p], sizeof V);
    V[0] += mu; V[4] += mu; V[8] += mu;
    inverse3(V, &Vinv[9 * p]);
  }
  // Per-key weighted blocks Y = W^T Vinv (6x3) and Yc = Wc^T Vinv (cps x 3).
  std::vector<double> Y((m.fixI ? 0 : m.K) * 18), Yc(B.pc_pairs.size() * 3 * cps);
  auto make_y = [&](int64_t k) {
    const double* W = &B.W[18 * k];
    const double* Vi = &Vinv[9 * m.key_point[k]];
    for (int a = 0; a < 6; ++a)
      for (int c = 0; c < 3; ++c)
        Y[18 * k + 3 * a + c] = W[a] * Vi[c] + W[6 + a] * Vi[3 + c] + W[12 + a] * Vi[6 + c];
  };
  auto make_yc = [&](int64_t q) {
    const double* Wc = &B.Wc[3 * cps * q];
    const double* Vi = &Vinv[9 * B.pc_pairs[q].first];
    for (int a = 0; a < cps; ++a)
      for (int c = 0; c < 3; ++c)
        Yc[3 * cps * q + 3 * a + c] =
            Wc[a] * Vi[c] + Wc[cps + a] * Vi[3 + c] + Wc[2 * cps + a] * Vi[6 + c];
  };
  if (!faithful) {
    for (int64_t k = 0; k < (m.fixI ? 0 : m.K); ++k) make_y(k);
    for (size_t q = 0; q < B.pc_pairs.size(); ++q) make_yc(int64_t(q));
    // Point-major: keys grouped by point.
    std::vector<std::vector<int64_t>> pk(P);
    for (int64_t k = 0; k < m.K; ++k) pk[m.key_point[k]].push_back(k);
    std::vector<std::vector<int64_t>> pq(P);
    for (size_t q = 0; q < B.pc_pairs.size(); ++q) pq[B.pc_pairs[q].first].push_back(int64_t(q));
    double blk[36];
    std::vector<double> cblk(cps * cps), icblk(6 * cps);
    if (!m.fixI) {
      for (int64_t i = 0; i < I; ++i)
        for (int a = 0; a < 6; ++a)
          for (int c = 0; c < 6; ++c)
            S[(6 * i + a) * n + 6 * i + c] = B.U[36 * i + 6 * a + c] + (a == c ? mu : 0.0);
    }
    if (!m.fixC) {
      for (int64_t c = 0; c < C; ++c)
        for (int a = 0; a < cps; ++a)
          for (int d = 0; d < cps; ++d)
            S[(cb + cps * c + a) * n + cb + cps * c + d] =
                B.Cb[cps * cps * c + cps * a + d] + (a == d ? mu : 0.0);
      if (!m.fixI)
        for (size_t q = 0; q < B.ic_pairs.size(); ++q) {
          int64_t i = B.ic_pairs[q].first, c = B.ic_pairs[q].second;
          for (int a = 0; a < 6; ++a)
            for (int d = 0; d < cps; ++d) {
              double v = B.E[6 * cps * q + cps * a + d];
              S[(6 * i + a) * n + cb + cps * c + d] += v;
              S[(cb + cps * c + d) * n + 6 * i + a] += v;
            }
        }
    }
    for (int64_t p = 0; p < P; ++p) {
      if (!m.fixI) {
        for (int64_t ka : pk[p]) {
          int64_t i = m.key_image[ka];
          for (int64_t kb : pk[p]) {
            int64_t j = m.key_image[kb];
            if (j < i) continue;
            std::fill(blk, blk + 36, 0.0);
            gemm_acc(&Y[18 * ka], &B.W[18 * kb], blk, 6, 3, 6, 1.0);
            for (int a = 0; a < 6; ++a)
              for (int c = 0; c < 6; ++c) {
                S[(6 * i + a) * n + 6 * j + c] -= blk[6 * a + c];
                if (j != i) S[(6 * j + c) * n + 6 * i + a] -= blk[6 * a + c];
              }
          }
          // rhs: b_i -= Y g_p
          for (int a = 0; a < 6; ++a)
            b[6 * i + a] -= Y[18 * ka + 3 * a] * B.gp[3 * p] +
                            Y[18 * ka + 3 * a + 1] * B.gp[3 * p + 1] +
                            Y[18 * ka + 3 * a + 2] * B.gp[3 * p + 2];
          if (!m.fixC) {  // image-camera coupling: -Y_i Wc_pc
            for (int64_t q : pq[p]) {
              int64_t c = B.pc_pairs[q].second;
              std::fill(icblk.begin(), icblk.end(), 0.0);
              gemm_acc(&Y[18 * ka], &B.Wc[3 * cps * q], icblk.data(), 6, 3, int(cps), 1.0);
              for (int a = 0; a < 6; ++a)
                for (int d = 0; d < cps; ++d) {
                  S[(6 * i + a) * n + cb + cps * c + d] -= icblk[cps * a + d];
                  S[(cb + cps * c + d) * n + 6 * i + a] -= icblk[cps * a + d];
                }
            }
          }
        }
      }
      if (!m.fixC) {
        for (int64_t qa : pq[p]) {
          int64_t c = B.pc_pairs[qa].second;
          for (int64_t qb : pq[p]) {
            int64_t d = B.pc_pairs[qb].second;
            if (d < c) continue;
            std::fill(cblk.begin(), cblk.end(), 0.0);
            gemm_acc(&Yc[3 * cps * qa], &B.Wc[3 * cps * qb], cblk.data(), int(cps), 3, int(cps), 1.0);
            for (int a = 0; a < cps; ++a)
              for (int e = 0; e < cps; ++e) {
                S[(cb + cps * c + a) * n + cb + cps * d + e] -= cblk[cps * a + e];
                if (d != c) S[(cb + cps * d + e) * n + cb + cps * c + a] -= cblk[cps * a + e];
              }
          }
          for (int a = 0; a < cps; ++a)
            b[cb + cps * c + a] -= Yc[3 * cps * qa + 3 * a] * B.gp[3 * p] +
                                   Yc[3 * cps * qa + 3 * a + 1] * B.gp[3 * p + 1] +
                                   Yc[3 * cps * qa + 3 * a + 2] * B.gp[3 * p + 2];
        }
      }
    }
    for (int64_t j = 0; j < int64_t(B.gi.size()); ++j) b[j] += B.gi[j];
    for (int64_t j = 0; j < int64_t(B.gc.size()); ++j) b[cb + j] += B.gc[j];
    return GBA_OK;
  }

  // ---- faithful loop nest --------------------------------------------------
  // Block maps: point_image_map_ (P x I, column = image), point_camera_map_
  // (P x C, column = camera), image_camera_map_ (I x C, column = camera).
  Csc point_image, point_camera, image_camera;
  {
    std::vector<std::pair<int32_t, int32_t>> oi(m.K);
    std::vector<int64_t> v(m.K);
    for (int64_t k = 0; k < m.K; ++k) { oi[k] = {m.key_image[k], m.key_point[k]}; v[k] = k + 1; }
    if (!m.fixI) point_image.build(I, oi, v);
    std::vector<std::pair<int32_t, int32_t>> oc(B.pc_pairs.size());
    std::vector<int64_t> vc(B.pc_pairs.size());
    for (size_t q = 0; q < B.pc_pairs.size(); ++q) { oc[q] = {B.pc_pairs[q].second, B.pc_pairs[q].first}; vc[q] = int64_t(q) + 1; }
    if (!m.fixC) point_camera.build(C, oc, vc);
    std::vector<std::pair<int32_t, int32_t>> ic(B.ic_pairs.size());
    std::vector<int64_t> vi(B.ic_pairs.size());
    for (size_t q = 0; q < B.ic_pairs.size(); ++q) { ic[q] = {B.ic_pairs[q].second, B.ic_pairs[q].first}; vi[q] = int64_t(q) + 1; }
    if (!m.fixI && !m.fixC) image_camera.build(C, ic, vi);
  }
  // :141-184 -- weighted blocks in point order, image order.
  std::vector<double> WY, WYc;  // weighted image-point / camera-point blocks
  std::vector<std::pair<int32_t, int32_t>> ip_trip, cp_trip;
  std::vector<int64_t> ip_val, cp_val;
  for (int64_t p = 0; p < P; ++p) {
    const double* Vi = &Vinv[9 * p];
    if (!m.fixI) {
      for (int64_t i = 0; i < I; ++i) {
        int64_t kk = point_image.coeff(int32_t(p), i);
        if (kk > 0) {
          const double* W = &B.W[18 * (kk - 1)];
          size_t base = WY.size();
          WY.resize(base + 18);
          for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 3; ++c)
              WY[base + 3 * a + c] = W[a] * Vi[c] + W[6 + a] * Vi[3 + c] + W[12 + a] * Vi[6 + c];
          ip_trip.push_back({int32_t(p), int32_t(i)});  // column = point
          ip_val.push_back(int64_t(WY.size() / 18));
        }
      }
    }
    if (!m.fixC) {
      for (int64_t c = 0; c < C; ++c) {
        int64_t qq = point_camera.coeff(int32_t(p), c);
        if (qq > 0) {
          const double* Wc = &B.Wc[3 * cps * (qq - 1)];
          size_t base = WYc.size();
          WYc.resize(base + 3 * cps);
          for (int a = 0; a < cps; ++a)
            for (int cc = 0; cc < 3; ++cc)
              WYc[base + 3 * a + cc] =
                  Wc[a] * Vi[cc] + Wc[cps + a] * Vi[3 + cc] + Wc[2 * cps + a] * Vi[6 + cc];
          cp_trip.push_back({int32_t(p), int32_t(c)});
          cp_val.push_back(int64_t(WYc.size() / (3 * cps)));
        }
      }
    }
  }
  Csc image_point, camera_point;  // (I x P) and (C x P), column = point
  if (!m.fixI) image_point.build(P, ip_trip, ip_val);
  if (!m.fixC) camera_point.build(P, cp_trip, cp_val);

  // :190-267 -- image-image blocks.
  if (!m.fixI) {
    double blk[36];
    for (int64_t wi = 0; wi < I; wi += row_stride) {
      for (int64_t i = wi; i < I; ++i) {
        std::fill(blk, blk + 36, 0.0);
        if (wi == i)
          for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 6; ++c)
              blk[6 * a + c] = B.U[36 * i + 6 * a + c] + (a == c ? mu : 0.0);
        bool exist = false;
        for (int64_t p = 0; p < P; ++p) {
          int64_t wid = image_point.coeff(int32_t(wi), p);
          int64_t kk = point_image.coeff(int32_t(p), i);
          if (wid > 0 && kk > 0) {
            gemm_acc(&WY[18 * (wid - 1)], &B.W[18 * (kk - 1)], blk, 6, 3, 6, -1.0);
            exist = true;
          }
        }
        if (exist) {
          for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 6; ++c) {
              S[(6 * wi + a) * n + 6 * i + c] += blk[6 * a + c];
              if (wi != i) S[(6 * i + c) * n + 6 * wi + a] += blk[6 * a + c];
            }
        }
      }
    }
  }
  // :270-343 -- camera-camera blocks.
  if (!m.fixC) {
    std::vector<double> blk(cps * cps);
    for (int64_t wc = 0; wc < C; ++wc) {
      for (int64_t c = wc; c < C; ++c) {
        std::fill(blk.begin(), blk.end(), 0.0);
        if (wc == c)
          for (int a = 0; a < cps; ++a)
            for (int d = 0; d < cps; ++d)
              blk[cps * a + d] = B.Cb[cps * cps * c + cps * a + d] + (a == d ? mu : 0.0);
        bool exist = false;
        for (int64_t p = 0; p < P; ++p) {
          int64_t wid = camera_point.coeff(int32_t(wc), p);
          int64_t qq = point_camera.coeff(int32_t(p), c);
          if (wid > 0 && qq > 0) {
            gemm_acc(&WYc[3 * cps * (wid - 1)], &B.Wc[3 * cps * (qq - 1)], blk.data(),
                     int(cps), 3, int(cps), -1.0);
            exist = true;
          }
        }
        if (exist)
          for (int a = 0; a < cps; ++a)
            for (int d = 0; d < cps; ++d) {
              S[(cb + cps * wc + a) * n + cb + cps * c + d] += blk[cps * a + d];
              if (wc != c) S[(cb + cps * c + d) * n + cb + cps * wc + a] += blk[cps * a + d];
            }
      }
    }
  }
  // :345-392 -- image-camera blocks.
  if (!m.fixC && !m.fixI) {
    std::vector<double> blk(6 * cps);
    for (int64_t i = 0; i < I; ++i) {
      for (int64_t c = 0; c < C; ++c) {
        std::fill(blk.begin(), blk.end(), 0.0);
        int64_t qe = image_camera.coeff(int32_t(i), c);
        if (qe > 0) std::copy(&B.E[6 * cps * (qe - 1)], &B.E[6 * cps * qe], blk.begin());
        bool exist = false;
        for (int64_t p = 0; p < P; ++p) {
          int64_t qq = point_camera.coeff(int32_t(p), c);
          int64_t wid = image_point.coeff(int32_t(i), p);
          if (wid > 0 && qq > 0) {
            gemm_acc(&WY[18 * (wid - 1)], &B.Wc[3 * cps * (qq - 1)], blk.data(), 6, 3, int(cps), -1.0);
            exist = true;
          }
        }
        if (exist)
          for (int a = 0; a < 6; ++a)
            for (int d = 0; d < cps; ++d) {
              S[(6 * i + a) * n + cb + cps * c + d] += blk[cps * a + d];
              S[(cb + cps * c + d) * n + 6 * i + a] += blk[cps * a + d];
            }
      }
    }
  }
  // :398-443 -- reduced rhs.  The reference's camera loop leaves point_id
  // uninitialised (:429); the restatement starts it at 0.
  if (!m.fixI) {
    for (int64_t i = 0; i < I; ++i) {
      for (int a = 0; a < 6; ++a) b[6 * i + a] = B.gi[6 * i + a];
      for (int64_t p = 0; p < P; ++p) {
        int64_t wid = image_point.coeff(int32_t(i), p);
        if (wid > 0) {
          const double* Yb = &WY[18 * (wid - 1)];
          for (int a = 0; a < 6; ++a)
            b[6 * i + a] -= Yb[3 * a] * B.gp[3 * p] + Yb[3 * a + 1] * B.gp[3 * p + 1] +
                            Yb[3 * a + 2] * B.gp[3 * p + 2];
        }
      }
    }
  }
  if (!m.fixC) {
    for (int64_t c = 0; c < C; ++c) {
      for (int a = 0; a < cps; ++a) b[cb + cps * c + a] = B.gc[cps * c + a];
      for (int64_t p = 0; p < P; ++p) {
        int64_t wid = camera_point.coeff(int32_t(c), p);
        if (wid > 0) {
          const double* Yb = &WYc[3 * cps * (wid - 1)];
          for (int a = 0; a < cps; ++a)
            b[cb + cps * c + a] -= Yb[3 * a] * B.gp[3 * p] + Yb[3 * a + 1] * B.gp[3 * p + 1] +
                                   Yb[3 * a + 2] * B.gp[3 * p + 2];
        }
      }
    }
  }
  return GBA_OK;
}

// :468-538 -- point back-substitution.
void back_substitution(const Model& m, const Blocks& B, const std::vector<double>& Vinv,
                       bool faithful, double* dx) {
  const int64_t P = m.P, cps = m.cps;
  const int64_t pb = 3 * P, cb = m.fixI ? 0 : 6 * m.I;
  std::vector<std::vector<int64_t>> pk, pq;
  if (!faithful) {
    pk.resize(P); pq.resize(P);
    for (int64_t k = 0; k < m.K; ++k) pk[m.key_point[k]].push_back(k);
    for (size_t q = 0; q < B.pc_pairs.size(); ++q) pq[B.pc_pairs[q].first].push_back(int64_t(q));
  }
  Csc point_image, point_camera;
  if (faithful) {
    std::vector<std::pair<int32_t, int32_t>> oi(m.K);
    std::vector<int64_t> v(m.K);
    for (int64_t k = 0; k < m.K; ++k) { oi[k] = {m.key_image[k], m.key_point[k]}; v[k] = k + 1; }
    if (!m.fixI) point_image.build(m.I, oi, v);
    std::vector<std::pair<int32_t, int32_t>> oc(B.pc_pairs.size());
    std::vector<int64_t> vc(B.pc_pairs.size());
    for (size_t q = 0; q < B.pc_pairs.size(); ++q) { oc[q] = {B.pc_pairs[q].second, B.pc_pairs[q].first}; vc[q] = int64_t(q) + 1; }
    if (!m.fixC) point_camera.build(m.C, oc, vc);
  }
  for (int64_t p = 0; p < P; ++p) {
    const double* Vi = &Vinv[9 * p];
    double t[3] = {B.gp[3 * p], B.gp[3 * p + 1], B.gp[3 * p + 2]};
    auto sub_image = [&](int64_t k) {
      const double* W = &B.W[18 * k];
      const double* d = &dx[pb + 6 * m.key_image[k]];
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 6; ++c) t[a] -= W[6 * a + c] * d[c];
    };
    auto sub_camera = [&](int64_t q) {
      const double* Wc = &B.Wc[3 * cps * q];
      const double* d = &dx[pb + cb + cps * B.pc_pairs[q].second];
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < cps; ++c) t[a] -= Wc[cps * a + c] * d[c];
    };
    if (faithful) {
      if (!m.fixI)
        for (int64_t i = 0; i < m.I; ++i) {
          int64_t kk = point_image.coeff(int32_t(p), i);
          if (kk > 0) sub_image(kk - 1);
        }
      if (!m.fixC)
        for (int64_t c = 0; c < m.C; ++c) {
          int64_t qq = point_camera.coeff(int32_t(p), c);
          if (qq > 0) sub_camera(qq - 1);
        }
    } else {
      if (!m.fixI) for (int64_t k : pk[p]) sub_image(k);
      if (!m.fixC) for (int64_t q : pq[p]) sub_camera(q);
    }
    for (int a = 0; a < 3; ++a)
      dx[3 * p + a] = Vi[3 * a] * t[0] + Vi[3 * a + 1] * t[1] + Vi[3 * a + 2] * t[2];
  }
}

// :75-114 dispatch.  dx [x_size].
int schur_solve(const Model& m, const Blocks& B, double mu, bool faithful,
                double* dx, SchurTiming* timing = nullptr) {
  if (!m.fixP) {
    if (!m.fixI || !m.fixC) {
      std::vector<double> S, b, Vinv;
      auto t0 = std::chrono::steady_clock::now();
      int row_stride = timing ? timing->row_stride : 1;
      int err = reduced_system(m, B, mu, faithful, row_stride, S, b, Vinv);
      auto t1 = std::chrono::steady_clock::now();
      if (err) return err;
      if (timing && row_stride > 1) {
        // The sampled loop left S incomplete; time the factorization on the
        // full reduced system (the point-major restatement gives the same S).
        reduced_system(m, B, mu, false, 1, S, b, Vinv);
      }
      const int64_t n = int64_t(b.size());
      auto t2 = std::chrono::steady_clock::now();
      err = ldlt_factor(S, n);
      if (err) return err;
      ldlt_solve(S, n, b.data());
      auto t3 = std::chrono::steady_clock::now();
      std::copy(b.begin(), b.end(), dx + 3 * m.P);
      back_substitution(m, B, Vinv, faithful, dx);
      auto t4 = std::chrono::steady_clock::now();
      if (timing) {
        timing->reduce = std::chrono::duration<double>(t1 - t0).count() * row_stride;
        timing->factor = std::chrono::duration<double>(t3 - t2).count();
        timing->backsub = std::chrono::duration<double>(t4 - t3).count();
      }
      return GBA_OK;
    }
    return solve_points_only(m, B, mu, dx);
  }
  return solve_images_cameras_only(m, B, mu, dx);
}

double max_diagonal(const Model& m, const Blocks& B) {  // ..._max_diagonal_value_calculator.hpp:26-36
  double v = -std::numeric_limits<double>::max();
  if (!m.fixP) for (int64_t p = 0; p < m.P; ++p) for (int a = 0; a < 3; ++a) v = std::max(v, B.V[9 * p + 4 * a]);
  if (!m.fixI) for (int64_t i = 0; i < m.I; ++i) for (int a = 0; a < 6; ++a) v = std::max(v, B.U[36 * i + 7 * a]);
  if (!m.fixC) for (int64_t c = 0; c < m.C; ++c) for (int a = 0; a < m.cps; ++a) v = std::max(v, B.Cb[m.cps * m.cps * c + (m.cps + 1) * a]);
  return v;
}

double gradient_inf_norm(const Blocks& B) {  // ..._gradient_infinite_norm_calculator.hpp:27-37
  double v = -std::numeric_limits<double>::max();
  for (double g : B.gp) v = std::max(v, std::abs(g));
  for (double g : B.gi) v = std::max(v, std::abs(g));
  for (double g : B.gc) v = std::max(v, std::abs(g));
  return v;
}

double gradient_dot(const Blocks& B, const double* dx) {  // ..._dot_product_calculator.hpp:26-36
  double s = 0;
  int64_t o = 0;
  for (double g : B.gp) s += g * dx[o++];
  for (double g : B.gi) s += g * dx[o++];
  for (double g : B.gc) s += g * dx[o++];
  return s;
}

double rmse_of(const Model& m, const Vec& r) {
  if (m.K == 0) return 0;
  double s = 0;
  for (int64_t k = 0; k < 2 * m.K; ++k) s += r[k] * r[k];
  return std::sqrt(s / double(m.K));
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int oracle_vector_function(const gba_problem* problem, const double* x, double* y) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  for (int64_t k = 0; k < m.K; ++k)
    image_key(m, m.point(m.key_point[k], x), m.image(m.key_image[k], x),
              m.camera(m.key_camera[k], x), &y[2 * k]);
  for (size_t c = 0; c < m.rows.size(); ++c) y[2 * m.K + c] = x[m.row_x_index(m.rows[c])];
  for (int64_t i = 0; i < m.n_priors; ++i)
    for (int a = 0; a < 3; ++a) y[m.prior_y_begin + 3 * i + a] = x[3 * problem->point_prior_ids[i] + a];
  return GBA_OK;
}

int oracle_jacobian(const gba_problem* problem, const double* x, double* pb,
                    double* ib, double* cb) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  std::vector<double> jc(2 * std::max<int64_t>(m.cps, 1));
  for (int64_t k = 0; k < m.K; ++k) {
    double jp[6], ji[12];
    key_jacobian(m, m.point(m.key_point[k], x), m.image(m.key_image[k], x),
                 m.camera(m.key_camera[k], x), jp, ji, jc.data());
    if (pb && !m.fixP) std::copy(jp, jp + 6, pb + 6 * k);
    if (ib && !m.fixI) std::copy(ji, ji + 12, ib + 12 * k);
    if (cb && !m.fixC) std::copy(jc.begin(), jc.begin() + 2 * m.cps, cb + 2 * m.cps * k);
  }
  return GBA_OK;
}

int oracle_ffd_jacobian(const gba_problem* problem, const double* x, double delta,
                        double min_delta, double* pb, double* ib, double* cb) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  for (int64_t k = 0; k < m.K; ++k) {
    double X[3], im[6];
    std::vector<double> cam(m.cps);
    std::copy(m.point(m.key_point[k], x), m.point(m.key_point[k], x) + 3, X);
    std::copy(m.image(m.key_image[k], x), m.image(m.key_image[k], x) + 6, im);
    std::copy(m.camera(m.key_camera[k], x), m.camera(m.key_camera[k], x) + m.cps, cam.begin());
    double base[2], pert[2];
    image_key(m, X, im, cam.data(), base);
    auto column = [&](double& v, double* out, int ncols, int col) {
      double orig = v;
      double d = std::max(std::abs(delta * orig), min_delta);
      v += d;
      image_key(m, X, im, cam.data(), pert);
      v = orig;
      out[col] = (pert[0] - base[0]) / d;
      out[ncols + col] = (pert[1] - base[1]) / d;
    };
    if (pb && !m.fixP) for (int j = 0; j < 3; ++j) column(X[j], pb + 6 * k, 3, j);
    if (ib && !m.fixI) for (int j = 0; j < 6; ++j) column(im[j], ib + 12 * k, 6, j);
    if (cb && !m.fixC) for (int j = 0; j < m.cps; ++j) column(cam[j], cb + 2 * m.cps * k, int(m.cps), j);
  }
  return GBA_OK;
}

int oracle_dense_jacobian(const gba_problem* problem, const double* x, double* J) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  const int64_t n = m.x_size;
  std::fill(J, J + m.y_size * n, 0.0);
  std::vector<double> jc(2 * std::max<int64_t>(m.cps, 1));
  for (int64_t k = 0; k < m.K; ++k) {
    double jp[6], ji[12];
    key_jacobian(m, m.point(m.key_point[k], x), m.image(m.key_image[k], x),
                 m.camera(m.key_camera[k], x), jp, ji, jc.data());
    for (int r = 0; r < 2; ++r) {
      double* row = J + (2 * k + r) * n;
      if (!m.fixP) for (int j = 0; j < 3; ++j) row[3 * m.key_point[k] + j] = jp[3 * r + j];
      if (!m.fixI) for (int j = 0; j < 6; ++j) row[m.x_image_begin + 6 * m.key_image[k] + j] = ji[6 * r + j];
      if (!m.fixC) for (int j = 0; j < m.cps; ++j)
        row[m.x_camera_begin + m.cps * m.key_camera[k] + j] = jc[m.cps * r + j];
    }
  }
  for (size_t c = 0; c < m.rows.size(); ++c) J[(2 * m.K + c) * n + m.row_x_index(m.rows[c])] = 1.0;
  for (int64_t i = 0; i < m.n_priors; ++i)
    for (int a = 0; a < 3; ++a)
      J[(m.prior_y_begin + 3 * i + a) * n + 3 * problem->point_prior_ids[i] + a] = 1.0;
  return GBA_OK;
}

int oracle_normal_equation_dense(const gba_problem* problem, const double* x,
                                 const double* near_y, double* N, double* g) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  Vec r;
  residuals(m, x, near_y, r);
  Blocks B;
  build_blocks(m, x, r, Loss(), B);
  blocks_to_dense(m, B, N, g);
  return GBA_OK;
}

int oracle_cost(const gba_problem* problem, const double* x, const double* near_y,
                int32_t loss, double huber_delta, double* cost) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  Vec r;
  residuals(m, x, near_y, r);
  Loss L;
  L.kind = loss;
  L.delta = huber_delta;
  *cost = cost_of(m, r, L);
  return std::isfinite(*cost) ? GBA_OK : GBA_ERR_NAN;
}

int oracle_schur_step(const gba_problem* problem, const double* x, const double* near_y,
                      double mu, int32_t faithful, int32_t loss, double huber_delta,
                      double* dx) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  Vec r;
  residuals(m, x, near_y, r);
  Loss L;
  L.kind = loss;
  L.delta = huber_delta;
  Blocks B;
  build_blocks(m, x, r, L, B);
  return schur_solve(m, B, mu, faithful != 0, dx);
}

// LM driver restated from Madsen, Nielsen & Tingleff (2004), Alg. 3.16, with
// the quantities supplied by the reference's trait classes
// (camera_shared_nllso_meta_levenberg_marquardt.hpp:33-106):
//   mu0 = tau * max diag(N);  stop when ||g||inf <= eps1 or
//   ||delta|| <= eps2 (||x|| + eps2);  x_new = x - delta where
//   (N + mu I) delta = g, g = J^T Lambda r, r = f(x) - y;
//   gain rho = (F(x) - F(x_new)) / (mu ||delta||^2 + g^T delta) for
//   F = sum r^T Lambda r (the predicted reduction of that F);
//   accepted: mu *= max(1/3, 1 - (2 rho - 1)^3), nu = 2;
//   rejected (or the reduced system fails to factor): mu *= nu, nu *= 2.
int oracle_lm_solve(const gba_problem* problem, const double* near_y,
                    const gba_options* opt, int32_t faithful, double* x,
                    gba_report* rep) {
  Model m;
  int err = m.init(problem);
  gba_report local{};
  gba_report& R = rep ? *rep : local;
  std::memset(&R, 0, sizeof(R));
  if (err) { R.status = err; return err; }
  Loss L;
  L.kind = opt->loss;
  L.delta = opt->huber_delta;
  const int64_t n = m.x_size;
  Vec r, r_new, x_new(n), dx(n);
  residuals(m, x, near_y, r);
  double F = cost_of(m, r, L);
  R.initial_cost = F;
  Blocks B;
  build_blocks(m, x, r, L, B);
  double ginf = gradient_inf_norm(B);
  bool found = ginf <= opt->eps1;
  double mu = opt->tau * max_diagonal(m, B);
  double nu = 2.0;
  int k = 0;
  R.stop_reason = found ? GBA_STOP_SMALL_GRADIENT : GBA_STOP_MAX_ITERATIONS;
  while (!found && k < opt->max_iterations) {
    ++k;
    int serr = schur_solve(m, B, mu, faithful != 0, dx.data());
    if (serr != GBA_OK) {
      R.factor_failures++;
      R.rejected++;
      mu *= nu;
      nu *= 2;
      continue;
    }
    double dn = 0, xn = 0;
    for (int64_t i = 0; i < n; ++i) { dn += dx[i] * dx[i]; xn += x[i] * x[i]; }
    dn = std::sqrt(dn);
    xn = std::sqrt(xn);
    if (dn <= opt->eps2 * (xn + opt->eps2)) {
      found = true;
      R.stop_reason = GBA_STOP_SMALL_STEP;
      break;
    }
    for (int64_t i = 0; i < n; ++i) x_new[i] = x[i] - dx[i];
    residuals(m, x_new.data(), near_y, r_new);
    double F_new = cost_of(m, r_new, L);
    double denom = mu * dn * dn + gradient_dot(B, dx.data());
    double rho = (F - F_new) / denom;
    if (std::isfinite(F_new) && rho > 0) {
      // Ceres' function tolerance (camera_shared_ceres_optimizor.hpp:478):
      // stop once an accepted step lowers F by at most ftol F
      const bool small_change = opt->function_tolerance > 0 && F - F_new <= opt->function_tolerance * F;
      std::copy(x_new.begin(), x_new.end(), x);
      r.swap(r_new);
      F = F_new;
      if (small_change) {
        R.accepted++;
        R.stop_reason = GBA_STOP_SMALL_COST_CHANGE;
        double t = 2 * rho - 1;
        mu *= std::max(1.0 / 3.0, 1 - t * t * t);
        break;
      }
      build_blocks(m, x, r, L, B);
      ginf = gradient_inf_norm(B);
      found = ginf <= opt->eps1;
      if (found) R.stop_reason = GBA_STOP_SMALL_GRADIENT;
      double t = 2 * rho - 1;
      mu *= std::max(1.0 / 3.0, 1 - t * t * t);
      nu = 2;
      R.accepted++;
    } else {
      mu *= nu;
      nu *= 2;
      R.rejected++;
    }
  }
  R.iterations = k;
  R.final_cost = F;
  R.final_rmse = rmse_of(m, r);
  R.final_mu = mu;
  R.final_gradient_inf_norm = ginf;
  R.status = std::isfinite(F) ? GBA_OK : GBA_ERR_NAN;
  return R.status;
}

int oracle_time_faithful_iteration(const gba_problem* problem, const double* near_y,
                                   const double* x, double mu, int32_t row_stride,
                                   double* seconds) {
  Model m;
  int err = m.init(problem);
  if (err) return err;
  using clk = std::chrono::steady_clock;
  auto t0 = clk::now();
  Vec r;
  residuals(m, x, near_y, r);
  Loss L;
  Blocks B;
  build_blocks(m, x, r, L, B);
  double ginf = gradient_inf_norm(B);
  (void)ginf;
  auto t1 = clk::now();
  Vec dx(m.x_size);
  SchurTiming T;
  T.row_stride = std::max(1, int(row_stride));
  err = schur_solve(m, B, mu, true, dx.data(), &T);
  if (err) return err;
  auto t2 = clk::now();
  Vec xn(m.x_size), rn;
  for (int64_t i = 0; i < m.x_size; ++i) xn[i] = x[i] - dx[i];
  residuals(m, xn.data(), near_y, rn);
  double Fn = cost_of(m, rn, L);
  (void)Fn;
  double gd = gradient_dot(B, dx.data());
  (void)gd;
  auto t3 = clk::now();
  double lin = std::chrono::duration<double>(t1 - t0).count();
  double cost = std::chrono::duration<double>(t3 - t2).count();
  (void)t2;
  seconds[1] = lin;
  seconds[2] = T.reduce;
  seconds[3] = T.factor;
  seconds[4] = T.backsub;
  seconds[5] = cost;
  seconds[0] = lin + T.reduce + T.factor + T.backsub + cost;
  return GBA_OK;
}

}  // extern "C"
