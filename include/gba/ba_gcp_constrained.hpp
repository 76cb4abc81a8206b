// gba/ba_gcp_constrained.hpp -- header-only C++ facade of libgba.so with the
// class names, constructors and call operators of the reference's
// GCP-constrained bundle adjustment (hs_sfm include/hs_sfm/bundle_adjustment/):
//
//   BAGCPConstrainedVectorFunction<S>          ba_gcp_constrained_vector_function.hpp:14-115
//   BAGCPConstrainedYCovarianceInverse<S>      ba_gcp_constrained_y_covariance_inverse.hpp:14-25
//   BAGCPConstrainedLevenbergMarquardtOptimizor ba_gcp_constrained_levenberg_marquardt_optimizor.hpp:15-70
//
// The model is the naive one (ba_naive_vector_function.hpp:14-205): x holds
// 6 parameters (axis-angle rotation, translation) per camera and then 3 per
// point, keys are normalized image coordinates (no intrinsics), and the last
// number_of_gcps points are ground control points whose coordinates are
// observed after the keys in y, each with a 3x3 inverse covariance.  The
// optimizer maps it onto the camera-shared device path: naive cameras become
// images, one camera without parameters, the control points point priors.
#ifndef GBA_BA_GCP_CONSTRAINED_HPP_
#define GBA_BA_GCP_CONSTRAINED_HPP_

#include <cstddef>
#include <cstdint>
#include <utility>
#include <vector>

#include "camera_shared.hpp"

namespace gba {

template <typename _Scalar>
class BAGCPConstrainedVectorFunction {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  typedef std::ptrdiff_t Index;
  typedef VectorX<Scalar> XVector;
  typedef VectorX<Scalar> YVector;
  static const Index params_per_camera_ = 6;
  static const Index params_per_point_ = 3;
  static const Index params_per_feature_ = 2;
  typedef std::pair<Index, Index> FeatureMap;   // (camera_id, point_id)
  typedef std::vector<FeatureMap> FeatureMapContainer;

  BAGCPConstrainedVectorFunction() {}
  BAGCPConstrainedVectorFunction(Index number_of_cameras, Index number_of_points,
                                 Index number_of_features, const FeatureMapContainer& feature_maps,
                                 Index number_of_gcps)
      : number_of_cameras_(number_of_cameras), number_of_points_(number_of_points),
        number_of_features_(number_of_features), feature_maps_(feature_maps),
        number_of_gcps_(number_of_gcps) {}

  Index number_of_cameras() const { return number_of_cameras_; }
  void set_number_of_cameras(Index n) { number_of_cameras_ = n; }
  Index number_of_points() const { return number_of_points_; }
  void set_number_of_points(Index n) { number_of_points_ = n; }
  Index number_of_features() const { return number_of_features_; }
  void set_number_of_features(Index n) { number_of_features_ = n; }
  const FeatureMapContainer& feature_maps() const { return feature_maps_; }
  void set_feature_maps(const FeatureMapContainer& f) { feature_maps_ = f; }
  Index number_of_gcps() const { return number_of_gcps_; }
  void set_number_of_gcps(Index n) { number_of_gcps_ = n; }

  Index GetCameraParamsSize() const { return number_of_cameras_ * params_per_camera_; }
  Index GetPointParamsSize() const { return number_of_points_ * params_per_point_; }
  Index GetXSize() const { return GetCameraParamsSize() + GetPointParamsSize(); }
  Index GetYFeatureSize() const { return number_of_features_ * params_per_feature_; }
  Index GetYSize() const { return GetYFeatureSize() + number_of_gcps_ * params_per_point_; }

  // The problem on the device path's layout: images = the naive cameras,
  // one camera without parameters, point priors = the last number_of_gcps
  // points.  gcp_ids is filled and must outlive the returned struct.
  gba_problem to_c(std::vector<int64_t>& image_camera_map, std::vector<int64_t>& gcp_ids) const {
    static_assert(sizeof(FeatureMap) == 2 * sizeof(int64_t), "pair<Index, Index> is two int64");
    gba_problem p = {};
    p.number_of_points = number_of_points_;
    p.number_of_images = number_of_cameras_;
    p.number_of_cameras = 1;
    p.number_of_keys = number_of_features_;
    p.feature_maps = reinterpret_cast<const int64_t*>(feature_maps_.data());
    image_camera_map.assign(size_t(number_of_cameras_), 0);
    p.image_camera_map = image_camera_map.data();
    p.intrinsic_computations_mask = 0;
    p.fix_mask = GBA_FIX_CAMERAS;
    gcp_ids.resize(size_t(number_of_gcps_ > 0 ? number_of_gcps_ : 0));
    for (size_t i = 0; i < gcp_ids.size(); ++i)
      gcp_ids[i] = int64_t(number_of_points_ - number_of_gcps_) + int64_t(i);
    p.number_of_point_priors = int64_t(gcp_ids.size());
    p.point_prior_ids = gcp_ids.empty() ? nullptr : gcp_ids.data();
    return p;
  }

  // x [cameras 6C][points 3P] <-> the device path's [points 3P][images 6C]
  template <typename XV>
  void to_device_x(const XV& x, std::vector<double>& out) const {
    const Index c6 = GetCameraParamsSize(), p3 = GetPointParamsSize();
    out.resize(size_t(c6 + p3));
    for (Index i = 0; i < p3; ++i) out[size_t(i)] = double(x.data()[c6 + i]);
    for (Index i = 0; i < c6; ++i) out[size_t(p3 + i)] = double(x.data()[i]);
  }
  template <typename XV>
  void from_device_x(const std::vector<double>& in, XV& x) const {
    const Index c6 = GetCameraParamsSize(), p3 = GetPointParamsSize();
    x.resize(c6 + p3);
    for (Index i = 0; i < p3; ++i) x.data()[c6 + i] = Scalar(in[size_t(i)]);
    for (Index i = 0; i < c6; ++i) x.data()[i] = Scalar(in[size_t(p3 + i)]);
  }

  // ba_gcp_constrained_vector_function.hpp:73-110: y = [keys 2F][gcp points 3G].
  template <typename XV, typename YV>
  Err operator()(const XV& x, YV& y) const {
    if (detail::vec_len(x) != GetXSize()) return -1;
    if (number_of_features_ != Index(feature_maps_.size())) return -1;
    std::vector<int64_t> icm, gcp;
    gba_problem p = to_c(icm, gcp);
    std::vector<double> xd;
    std::vector<double> yd(static_cast<size_t>(GetYSize()));
    to_device_x(x, xd);
    if (gba_vector_function(&p, xd.data(), yd.data(), GBA_PRECISION_FP64) != GBA_OK) return -1;
    y.resize(GetYSize());
    for (size_t i = 0; i < yd.size(); ++i) y.data()[i] = Scalar(yd[i]);
    return 0;
  }

 private:
  Index number_of_cameras_ = 0, number_of_points_ = 0, number_of_features_ = 0;
  FeatureMapContainer feature_maps_;
  Index number_of_gcps_ = 0;
};

// ba_gcp_constrained_y_covariance_inverse.hpp:14-25 with the naive key
// blocks (ba_naive_feature_covariance_inverse.hpp:17-25); blocks row-major.
template <typename _Scalar>
struct BAGCPConstrainedYCovarianceInverse {
  typedef _Scalar Scalar;
  struct GCPBlock {
    Scalar m[9];
    Scalar operator()(int r, int c) const { return m[3 * r + c]; }
    Scalar& operator()(int r, int c) { return m[3 * r + c]; }
  };
  struct NaiveYCovarianceInverse {
    struct Block {
      Scalar m[4];
      Scalar operator()(int r, int c) const { return m[2 * r + c]; }
      Scalar& operator()(int r, int c) { return m[2 * r + c]; }
    };
    std::vector<Block> blocks;
  };
  std::vector<GCPBlock> gcp_blocks;
  NaiveYCovarianceInverse naive_y_covariance_inverse;
};

template <typename _VectorFunction>
class BAGCPConstrainedLevenbergMarquardtOptimizor;

template <typename _Scalar>
class BAGCPConstrainedLevenbergMarquardtOptimizor<BAGCPConstrainedVectorFunction<_Scalar> > {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  typedef BAGCPConstrainedVectorFunction<Scalar> VectorFunction;
  typedef typename VectorFunction::Index Index;
  typedef typename VectorFunction::XVector XVector;
  typedef typename VectorFunction::YVector YVector;
  typedef BAGCPConstrainedYCovarianceInverse<Scalar> YCovarianceInverse;

  template <typename XV>
  explicit BAGCPConstrainedLevenbergMarquardtOptimizor(const XV& initial_x) {
    copy_in(initial_x);
    gba_default_options(&options_);
  }
  template <typename XV>
  BAGCPConstrainedLevenbergMarquardtOptimizor(const XV& initial_x, size_t max_itr_num, Scalar tau,
                                              Scalar eps1, Scalar eps2) {
    copy_in(initial_x);
    gba_default_options(&options_);
    options_.max_iterations = int32_t(max_itr_num);
    options_.tau = double(tau);
    options_.eps1 = double(eps1);
    options_.eps2 = double(eps2);
  }

  gba_options& options() { return options_; }
  int last_status() const { return last_status_; }
  const gba_report& last_report() const { return last_report_; }

  // ba_gcp_constrained_levenberg_marquardt_optimizor.hpp:45-60
  template <typename YV, typename XV>
  Err operator()(const VectorFunction& vf, const YV& near_y, const YCovarianceInverse& cov,
                 XV& optimized_x) const {
    if (std::ptrdiff_t(initial_x_.size()) != vf.GetXSize() ||
        detail::vec_len(near_y) != vf.GetYSize()) {
      last_status_ = GBA_ERR_INVALID;
      return -1;
    }
    std::vector<int64_t> icm, gcp;
    gba_problem p = vf.to_c(icm, gcp);
    std::vector<double> kci, info;
    const auto& kb = cov.naive_y_covariance_inverse.blocks;
    if (!kb.empty()) {
      if (std::ptrdiff_t(kb.size()) != vf.number_of_features()) {
        last_status_ = GBA_ERR_INVALID;
        return -1;
      }
      kci.resize(4 * kb.size());
      for (size_t k = 0; k < kb.size(); ++k)
        for (int j = 0; j < 4; ++j) kci[4 * k + j] = double(kb[k].m[j]);
      p.key_covariance_inverse = kci.data();
    }
    if (!cov.gcp_blocks.empty()) {
      if (cov.gcp_blocks.size() != gcp.size()) {
        last_status_ = GBA_ERR_INVALID;
        return -1;
      }
      info.resize(9 * gcp.size());
      for (size_t i = 0; i < gcp.size(); ++i)
        for (int j = 0; j < 9; ++j) info[9 * i + j] = double(cov.gcp_blocks[i].m[j]);
      p.point_prior_information = info.data();
    }
    std::vector<double> y(size_t(detail::vec_len(near_y)));
    for (size_t i = 0; i < y.size(); ++i) y[i] = double(near_y.data()[i]);
    std::vector<double> x;
    vf.to_device_x(initial_x_, x);
    last_status_ = gba_solve(&p, y.data(), &options_, x.data(), &last_report_);
    vf.from_device_x(x, optimized_x);
    return last_status_ == GBA_OK ? 0 : -1;
  }

 private:
  template <typename XV>
  void copy_in(const XV& v) {
    initial_x_.resize(size_t(detail::vec_len(v)));
    for (size_t i = 0; i < initial_x_.size(); ++i) initial_x_[i] = double(v.data()[i]);
  }
  std::vector<double> initial_x_;
  gba_options options_;
  mutable int last_status_ = GBA_OK;
  mutable gba_report last_report_ = {};
};

}  // namespace gba

#endif  // GBA_BA_GCP_CONSTRAINED_HPP_
