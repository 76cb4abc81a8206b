// gba/triangulate.hpp -- header-only C++ facade of gba_triangulate() with the
// names and call operator of the reference's multi-view triangulation
// (hs_sfm include/hs_sfm/triangulate/, sfm_utility/camera_type.hpp):
//
//   CameraIntrinsicParams<S>                    sfm_utility/camera_type.hpp:15-231
//   CameraExtrinsicParams<S>                    sfm_utility/camera_type.hpp:233-333
//   MultipleViewMaximumLikelihoodEstimator<S>   multiple_view_maximum_likelihood_estimator.hpp:14-84
//
// plus MultipleViewTriangulator<S>, which solves many tracks in one call (one
// GPU thread per point).  Rotations are angle-axis vectors (world to camera),
// positions are camera centres; keys are the observed, distorted pixel keys.
// Errors come back as the reference's Err: 0 on success, -1 otherwise.
#ifndef GBA_TRIANGULATE_HPP_
#define GBA_TRIANGULATE_HPP_

#include <array>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "../gba.h"

namespace gba {

template <typename _Scalar>
class CameraIntrinsicParams {
 public:
  typedef _Scalar Scalar;
  CameraIntrinsicParams() {}
  CameraIntrinsicParams(Scalar focal_length, Scalar skew = 0, Scalar principal_point_x = 0,
                        Scalar principal_point_y = 0, Scalar pixel_ratio = 1, Scalar k1 = 0,
                        Scalar k2 = 0, Scalar k3 = 0, Scalar d1 = 0, Scalar d2 = 0)
      : v_{{focal_length, skew, principal_point_x, principal_point_y, pixel_ratio, k1, k2, k3, d1,
            d2}} {}
  Scalar focal_length() const { return v_[0]; }
  void set_focal_length(Scalar v) { v_[0] = v; }
  Scalar skew() const { return v_[1]; }
  void set_skew(Scalar v) { v_[1] = v; }
  Scalar principal_point_x() const { return v_[2]; }
  void set_principal_point_x(Scalar v) { v_[2] = v; }
  Scalar principal_point_y() const { return v_[3]; }
  void set_principal_point_y(Scalar v) { v_[3] = v; }
  Scalar pixel_ratio() const { return v_[4]; }
  void set_pixel_ratio(Scalar v) { v_[4] = v; }
  Scalar k1() const { return v_[5]; }
  void set_k1(Scalar v) { v_[5] = v; }
  Scalar k2() const { return v_[6]; }
  void set_k2(Scalar v) { v_[6] = v; }
  Scalar k3() const { return v_[7]; }
  void set_k3(Scalar v) { v_[7] = v; }
  Scalar d1() const { return v_[8]; }
  void set_d1(Scalar v) { v_[8] = v; }
  Scalar d2() const { return v_[9]; }
  void set_d2(Scalar v) { v_[9] = v; }
  // [f skew cx cy pixel_ratio k1 k2 k3 d1 d2], the layout gba_triangulate reads
  const std::array<Scalar, 10>& values() const { return v_; }

 private:
  std::array<Scalar, 10> v_{{1, 0, 0, 0, 1, 0, 0, 0, 0, 0}};
};

template <typename _Scalar>
class CameraExtrinsicParams {
 public:
  typedef _Scalar Scalar;
  typedef std::array<Scalar, 3> Rotation;   // angle-axis, world to camera
  typedef std::array<Scalar, 3> Position;   // camera centre
  CameraExtrinsicParams() : rotation_{{0, 0, 0}}, position_{{0, 0, 0}} {}
  CameraExtrinsicParams(const Rotation& rotation, const Position& position)
      : rotation_(rotation), position_(position) {}
  const Rotation& rotation() const { return rotation_; }
  Rotation& rotation() { return rotation_; }
  const Position& position() const { return position_; }
  Position& position() { return position_; }

 private:
  Rotation rotation_;
  Position position_;
};

// Many tracks over one set of views in one gba_triangulate call.
template <typename _Scalar>
class MultipleViewTriangulator {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  typedef CameraIntrinsicParams<Scalar> IntrinsicParams;
  typedef CameraExtrinsicParams<Scalar> ExtrinsicParams;

  MultipleViewTriangulator() { gba_default_options(&options_); }
  gba_options& options() { return options_; }

  // track_offsets [n + 1], track_views [m], track_keys [2m]; points [3n],
  // status [n] (GBA_OK, GBA_ERR_INVALID for fewer than 2 views, GBA_ERR_NAN).
  Err operator()(const std::vector<IntrinsicParams>& intrinsics,
                 const std::vector<ExtrinsicParams>& extrinsics,
                 const std::vector<int64_t>& track_offsets, const std::vector<int64_t>& track_views,
                 const std::vector<Scalar>& track_keys, std::vector<Scalar>& points,
                 std::vector<int32_t>& status) const {
    if (intrinsics.size() != extrinsics.size() || track_offsets.empty()) return -1;
    const size_t n = track_offsets.size() - 1;
    std::vector<double> intr(10 * intrinsics.size()), extr(6 * extrinsics.size());
    for (size_t v = 0; v < intrinsics.size(); ++v) {
      for (int j = 0; j < 10; ++j) intr[10 * v + j] = double(intrinsics[v].values()[j]);
      for (int j = 0; j < 3; ++j) {
        extr[6 * v + j] = double(extrinsics[v].rotation()[j]);
        extr[6 * v + 3 + j] = double(extrinsics[v].position()[j]);
      }
    }
    std::vector<double> keys(track_keys.begin(), track_keys.end()), pts(3 * n);
    gba_triangulation p = {};
    p.number_of_views = int64_t(intrinsics.size());
    p.intrinsics = intr.data();
    p.extrinsics = extr.data();
    p.number_of_points = int64_t(n);
    p.track_offsets = track_offsets.data();
    p.track_views = track_views.data();
    p.track_keys = keys.data();
    status.assign(n, GBA_OK);
    last_status_ = gba_triangulate(&p, &options_, pts.data(), status.data());
    points.assign(pts.begin(), pts.end());
    return last_status_ == GBA_OK ? 0 : -1;
  }
  int last_status() const { return last_status_; }

 private:
  gba_options options_;
  mutable int last_status_ = GBA_OK;
};

// multiple_view_maximum_likelihood_estimator.hpp:49-84: one point from its
// views and keys (at least two), -1 on failure.  Point is any type with
// operator[] (Eigen::Vector3d, std::array<double, 3>, ...).
template <typename _Scalar>
class MultipleViewMaximumLikelihoodEstimator {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  typedef CameraIntrinsicParams<Scalar> IntrinsicParams;
  typedef std::vector<IntrinsicParams> IntrinsicParamsContainer;
  typedef CameraExtrinsicParams<Scalar> ExtrinsicParams;
  typedef std::vector<ExtrinsicParams> ExtrinsicParamsContainer;
  typedef std::array<Scalar, 2> Key;
  typedef std::vector<Key> KeyContainer;

  template <typename Point>
  Err operator()(const IntrinsicParamsContainer& intrinsic_params_set,
                 const ExtrinsicParamsContainer& extrinsic_params_set, const KeyContainer& keys,
                 Point& point) const {
    const size_t nv = intrinsic_params_set.size();
    if (extrinsic_params_set.size() != nv || keys.size() != nv || nv < 2) return -1;
    std::vector<int64_t> off = {0, int64_t(nv)}, views(nv);
    std::vector<Scalar> k(2 * nv), pts;
    for (size_t i = 0; i < nv; ++i) {
      views[i] = int64_t(i);
      k[2 * i] = keys[i][0];
      k[2 * i + 1] = keys[i][1];
    }
    std::vector<int32_t> st;
    MultipleViewTriangulator<Scalar> tri;
    if (tri(intrinsic_params_set, extrinsic_params_set, off, views, k, pts, st) != 0 ||
        st[0] != GBA_OK)
      return -1;
    for (int i = 0; i < 3; ++i) point[i] = pts[size_t(i)];
    return 0;
  }
};

}  // namespace gba

#endif  // GBA_TRIANGULATE_HPP_
