// gba/camera_shared.hpp -- header-only C++ facade of libgba.so with the class
// names, constructors and call operators of the reference's camera-shared
// bundle-adjustment path (hs_sfm include/hs_sfm/bundle_adjustment/):
//
//   CameraSharedVectorFunction<S>            camera_shared_vector_function.hpp:20-764
//   CameraSharedYCovarianceInverse<S>        camera_shared_y_covariance_inverse.hpp:18-149
//   CameraSharedLevenbergMarquardtOptimizor  camera_shared_levenberg_marquardt_optimizor.hpp:19-63
//   CameraSharedCeresOptimizor               camera_shared_ceres_optimizor.hpp:163-500
//
// The optimizer's operator() marshals the problem into a gba_problem (the
// feature maps and the image-camera map are passed without copying: they
// have the layout of the reference's std::pair<Index, Index> /
// std::vector<Index> containers) and calls gba_solve().  Vectors are any
// type with rows() or size(), data() and resize(); gba::VectorX is a minimal
// one for callers without Eigen, and Eigen::VectorXd works as well.
// Errors come back as the reference's Err: 0 on success, -1 otherwise (the
// detailed status is kept in last_status()).
#ifndef GBA_CAMERA_SHARED_HPP_
#define GBA_CAMERA_SHARED_HPP_

#include <bitset>
#include <cstddef>
#include <cstdint>
#include <utility>
#include <vector>

#include "../gba.h"

namespace gba {

// ---------------------------------------------------------------------------
// masks and constraints (camera_shared_common_types.hpp:14-104)
// ---------------------------------------------------------------------------
enum { COMPUTE_RADIAL_DISTORTION = 0, COMPUTE_DECENTERING_DISTORTION, COMPUTE_INTRINSIC_PARAMS,
       NUMBER_OF_INTRINSIC_COMPUTATIONS };
typedef std::bitset<NUMBER_OF_INTRINSIC_COMPUTATIONS> IntrinsicComputationsMask;
enum { POINT_CONSTRAIN_X = 0, POINT_CONSTRAIN_Y, POINT_CONSTRAIN_Z, NUMBER_OF_POINT_CONSTRAINTS };
typedef std::bitset<NUMBER_OF_POINT_CONSTRAINTS> PointConstraintsMask;
struct PointConstraint {
  size_t point_id;
  PointConstraintsMask mask;
};
typedef std::vector<PointConstraint> PointConstraintContainer;
enum { IMAGE_CONSTRAIN_ROTATION = 0, IMAGE_CONSTRAIN_POSITION_X, IMAGE_CONSTRAIN_POSITION_Y,
       IMAGE_CONSTRAIN_POSITION_Z, NUMBER_OF_IMAGE_CONSTRAINTS };
typedef std::bitset<NUMBER_OF_IMAGE_CONSTRAINTS> ImageConstraintsMask;
struct ImageConstraint {
  size_t image_id;
  ImageConstraintsMask mask;
};
typedef std::vector<ImageConstraint> ImageConstraintContainer;
typedef std::bitset<3> RadialConstraintsMask;
typedef std::bitset<2> DecenteringConstraintsMask;
typedef std::bitset<5> IntrinsicConstraintsMask;
struct CameraConstraint {
  size_t camera_id;
  RadialConstraintsMask radial_mask;
  DecenteringConstraintsMask decentering_mask;
  IntrinsicConstraintsMask intrinsic_mask;
};
typedef std::vector<CameraConstraint> CameraConstraintContainer;
enum { FIX_POINTS = 0, FIX_IMAGES, FIX_CAMERAS, NUMBER_OF_FIX_PARAMS };
typedef std::bitset<NUMBER_OF_FIX_PARAMS> FixMask;

// ---------------------------------------------------------------------------
// A minimal dense vector for callers without Eigen.
// ---------------------------------------------------------------------------
template <typename Scalar>
class VectorX {
 public:
  typedef std::ptrdiff_t Index;
  VectorX() {}
  explicit VectorX(Index n) : v_(size_t(n), Scalar(0)) {}
  Index rows() const { return Index(v_.size()); }
  Index size() const { return Index(v_.size()); }
  void resize(Index n) { v_.resize(size_t(n)); }
  Scalar* data() { return v_.data(); }
  const Scalar* data() const { return v_.data(); }
  Scalar& operator[](Index i) { return v_[size_t(i)]; }
  const Scalar& operator[](Index i) const { return v_[size_t(i)]; }
  Scalar& operator()(Index i) { return v_[size_t(i)]; }
  const Scalar& operator()(Index i) const { return v_[size_t(i)]; }

 private:
  std::vector<Scalar> v_;
};

namespace detail {
template <typename V>
auto vec_rows(const V& v) -> decltype(v.rows()) { return v.rows(); }
template <typename V>
inline std::ptrdiff_t vec_len(const V& v) { return std::ptrdiff_t(vec_rows(v)); }
}  // namespace detail

// ---------------------------------------------------------------------------
// CameraSharedVectorFunction: the problem description
// (camera_shared_vector_function.hpp:20-764).  Fixed blocks are stored as
// flat vectors [3P], [6I], [cC].
// ---------------------------------------------------------------------------
template <typename _Scalar>
class CameraSharedVectorFunction {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  typedef std::ptrdiff_t Index;
  typedef VectorX<Scalar> XVector;
  typedef VectorX<Scalar> YVector;
  static const Index extrinsic_params_per_image_ = 6;
  static const Index params_per_point_ = 3;
  static const Index params_per_key_ = 2;
  typedef std::pair<Index, Index> FeatureMap;   // (image_id, point_id)
  typedef std::vector<FeatureMap> FeatureMapContainer;
  typedef std::vector<Index> ImageCameraMap;

  Index number_of_cameras() const { return number_of_cameras_; }
  void set_number_of_cameras(Index n) { number_of_cameras_ = n; }
  Index number_of_images() const { return number_of_images_; }
  void set_number_of_images(Index n) { number_of_images_ = n; }
  Index number_of_points() const { return number_of_points_; }
  void set_number_of_points(Index n) { number_of_points_ = n; }
  Index number_of_keys() const { return number_of_keys_; }
  void set_number_of_keys(Index n) { number_of_keys_ = n; }
  const FeatureMapContainer& feature_maps() const { return feature_maps_; }
  void set_feature_maps(const FeatureMapContainer& f) { feature_maps_ = f; }
  const ImageCameraMap& image_camera_map() const { return image_camera_map_; }
  void set_image_camera_map(const ImageCameraMap& m) { image_camera_map_ = m; }
  const IntrinsicComputationsMask& intrinsic_computations_mask() const { return intrinsic_mask_; }
  IntrinsicComputationsMask& intrinsic_computations_mask() { return intrinsic_mask_; }
  const PointConstraintContainer& point_constraints() const { return point_constraints_; }
  PointConstraintContainer& point_constraints() { return point_constraints_; }
  const ImageConstraintContainer& image_constraints() const { return image_constraints_; }
  ImageConstraintContainer& image_constraints() { return image_constraints_; }
  const CameraConstraintContainer& camera_constraints() const { return camera_constraints_; }
  CameraConstraintContainer& camera_constraints() { return camera_constraints_; }

  // :156-235 -- size checks as in the reference
  Err set_fix_points(const std::vector<Scalar>& pts) {
    if (Index(pts.size()) != number_of_points_ * params_per_point_) return -1;
    fix_mask_.set(FIX_POINTS);
    fix_points_ = pts;
    return 0;
  }
  Err set_fix_images(const std::vector<Scalar>& imgs) {
    if (Index(imgs.size()) != number_of_images_ * extrinsic_params_per_image_) return -1;
    fix_mask_.set(FIX_IMAGES);
    fix_images_ = imgs;
    return 0;
  }
  Err set_fix_cameras(const std::vector<Scalar>& cams) {
    if (Index(cams.size()) != number_of_cameras_ * GetIntrinsicParamsSizePerCamera()) return -1;
    fix_mask_.set(FIX_CAMERAS);
    fix_cameras_ = cams;
    return 0;
  }
  void unset_fix_points() { fix_mask_.reset(FIX_POINTS); fix_points_.clear(); }
  void unset_fix_images() { fix_mask_.reset(FIX_IMAGES); fix_images_.clear(); }
  void unset_fix_cameras() { fix_mask_.reset(FIX_CAMERAS); fix_cameras_.clear(); }
  bool is_fix_points() const { return fix_mask_[FIX_POINTS]; }
  bool is_fix_images() const { return fix_mask_[FIX_IMAGES]; }
  bool is_fix_cameras() const { return fix_mask_[FIX_CAMERAS]; }
  const std::vector<Scalar>& fix_points() const { return fix_points_; }
  const std::vector<Scalar>& fix_images() const { return fix_images_; }
  const std::vector<Scalar>& fix_cameras() const { return fix_cameras_; }

  Index GetIntrinsicParamsSizePerCamera() const {   // :247-263
    return Index(gba_params_per_camera(uint32_t(intrinsic_mask_.to_ulong())));
  }

  // The C view of this problem; valid while *this and the extra arrays live.
  gba_problem to_c(std::vector<gba_point_constraint>& pc, std::vector<gba_image_constraint>& ic,
                   std::vector<gba_camera_constraint>& cc) const {
    static_assert(sizeof(FeatureMap) == 2 * sizeof(int64_t), "pair<Index, Index> is two int64");
    static_assert(sizeof(Index) == sizeof(int64_t), "Index is int64");
    gba_problem p = {};
    p.number_of_points = number_of_points_;
    p.number_of_images = number_of_images_;
    p.number_of_cameras = number_of_cameras_;
    p.number_of_keys = number_of_keys_;
    p.feature_maps = reinterpret_cast<const int64_t*>(feature_maps_.data());
    p.image_camera_map = reinterpret_cast<const int64_t*>(image_camera_map_.data());
    p.intrinsic_computations_mask = uint32_t(intrinsic_mask_.to_ulong());
    p.fix_mask = (is_fix_points() ? GBA_FIX_POINTS : 0u) | (is_fix_images() ? GBA_FIX_IMAGES : 0u) |
                 (is_fix_cameras() ? GBA_FIX_CAMERAS : 0u);
    p.fix_points = is_fix_points() ? fix_points_.data() : nullptr;
    p.fix_images = is_fix_images() ? fix_images_.data() : nullptr;
    p.fix_cameras = is_fix_cameras() ? fix_cameras_.data() : nullptr;
    pc.clear();
    for (const PointConstraint& c : point_constraints_)
      pc.push_back({int64_t(c.point_id), uint32_t(c.mask.to_ulong()), 0u});
    ic.clear();
    for (const ImageConstraint& c : image_constraints_)
      ic.push_back({int64_t(c.image_id), uint32_t(c.mask.to_ulong()), 0u});
    cc.clear();
    for (const CameraConstraint& c : camera_constraints_)
      cc.push_back({int64_t(c.camera_id), uint32_t(c.radial_mask.to_ulong()),
                    uint32_t(c.decentering_mask.to_ulong()), uint32_t(c.intrinsic_mask.to_ulong()), 0u});
    p.number_of_point_constraints = int64_t(pc.size());
    p.point_constraints = pc.empty() ? nullptr : pc.data();
    p.number_of_image_constraints = int64_t(ic.size());
    p.image_constraints = ic.empty() ? nullptr : ic.data();
    p.number_of_camera_constraints = int64_t(cc.size());
    p.camera_constraints = cc.empty() ? nullptr : cc.data();
    return p;
  }

  Index GetXSize() const {
    std::vector<gba_point_constraint> pc;
    std::vector<gba_image_constraint> ic;
    std::vector<gba_camera_constraint> cc;
    gba_problem p = to_c(pc, ic, cc);
    return Index(gba_x_size(&p));
  }
  Index GetYSize() const {
    std::vector<gba_point_constraint> pc;
    std::vector<gba_image_constraint> ic;
    std::vector<gba_camera_constraint> cc;
    gba_problem p = to_c(pc, ic, cc);
    return Index(gba_y_size(&p));
  }

 private:
  Index number_of_images_ = 0, number_of_points_ = 0, number_of_keys_ = 0, number_of_cameras_ = 0;
  FeatureMapContainer feature_maps_;
  ImageCameraMap image_camera_map_;
  IntrinsicComputationsMask intrinsic_mask_;
  PointConstraintContainer point_constraints_;
  ImageConstraintContainer image_constraints_;
  CameraConstraintContainer camera_constraints_;
  FixMask fix_mask_;
  std::vector<Scalar> fix_points_, fix_images_, fix_cameras_;
};

// ---------------------------------------------------------------------------
// CameraSharedYCovarianceInverse (camera_shared_y_covariance_inverse.hpp:18-149)
// ---------------------------------------------------------------------------
template <typename _Scalar>
class CameraSharedYCovarianceInverse {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  struct KeyBlock {   // row-major 2x2
    Scalar m[4];
    Scalar operator()(int r, int c) const { return m[2 * r + c]; }
  };

  void Clear() { key_blocks_.clear(); constraints_.clear(); }
  // :43-50 -- as in the reference, the block stored for each key is the
  // inverse of I / sigma^2, i.e. sigma^2 I (identical at sigma = 1).
  Err SetKeysUniformStdDev(Scalar key_std_dev, size_t number_of_keys) {
    if (key_std_dev == Scalar(0)) return -1;
    const Scalar v = Scalar(1) / (key_std_dev * key_std_dev);
    KeyBlock cov = {{v, 0, 0, v}};
    return SetKeysUniformCovariance(cov, number_of_keys);
  }
  Err SetKeysUniformCovariance(const KeyBlock& cov, size_t number_of_keys) {
    KeyBlock inv;
    if (!invert(cov, inv)) return -1;
    key_blocks_.assign(number_of_keys, inv);
    return 0;
  }
  Err AddKeyCovariance(const KeyBlock& cov) {
    KeyBlock inv;
    if (!invert(cov, inv)) return -1;
    key_blocks_.push_back(inv);
    return 0;
  }
  const KeyBlock& GetKeyBlock(size_t key_id) const { return key_blocks_[key_id]; }
  void AddConstraint(Scalar c) { constraints_.push_back(c); }
  Scalar GetConstraint(size_t i) const { return constraints_[i]; }
  size_t NumberOfKeys() const { return key_blocks_.size(); }
  const std::vector<KeyBlock>& key_blocks() const { return key_blocks_; }
  const std::vector<Scalar>& constraints() const { return constraints_; }

 private:
  static bool invert(const KeyBlock& a, KeyBlock& out) {
    const Scalar det = a.m[0] * a.m[3] - a.m[1] * a.m[2];
    if (det == Scalar(0)) return false;
    out.m[0] = a.m[3] / det;
    out.m[1] = -a.m[1] / det;
    out.m[2] = -a.m[2] / det;
    out.m[3] = a.m[0] / det;
    return true;
  }
  std::vector<KeyBlock> key_blocks_;
  std::vector<Scalar> constraints_;
};

// ---------------------------------------------------------------------------
// CameraSharedLevenbergMarquardtOptimizor
// (camera_shared_levenberg_marquardt_optimizor.hpp:19-63).
// ---------------------------------------------------------------------------
template <typename _VectorFunction>
class CameraSharedLevenbergMarquardtOptimizor;

template <typename _Scalar>
class CameraSharedLevenbergMarquardtOptimizor<CameraSharedVectorFunction<_Scalar> > {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  typedef CameraSharedVectorFunction<Scalar> VectorFunction;
  typedef typename VectorFunction::XVector XVector;
  typedef typename VectorFunction::YVector YVector;
  typedef CameraSharedYCovarianceInverse<Scalar> YCovarianceInverse;

  template <typename XV>
  explicit CameraSharedLevenbergMarquardtOptimizor(const XV& initial_x) {
    copy_in(initial_x);
    gba_default_options(&options_);
  }
  template <typename XV>
  CameraSharedLevenbergMarquardtOptimizor(const XV& initial_x, size_t max_itr_num, Scalar tau,
                                          Scalar eps1, Scalar eps2) {
    copy_in(initial_x);
    gba_default_options(&options_);
    options_.max_iterations = int32_t(max_itr_num);
    options_.tau = double(tau);
    options_.eps1 = double(eps1);
    options_.eps2 = double(eps2);
  }

  // Solver choices beyond the reference's constructor (precision, loss, device).
  gba_options& options() { return options_; }
  int last_status() const { return last_status_; }
  const gba_report& last_report() const { return last_report_; }

  template <typename YV, typename XV>
  Err operator()(const VectorFunction& vf, const YV& near_y, const YCovarianceInverse& cov,
                 XV& optimized_x) const {
    const std::ptrdiff_t x_size = vf.GetXSize();
    if (std::ptrdiff_t(initial_x_.size()) != x_size) {   // :48-51
      last_status_ = GBA_ERR_INVALID;
      return -1;
    }
    if (detail::vec_len(near_y) != vf.GetYSize()) {
      last_status_ = GBA_ERR_INVALID;
      return -1;
    }
    std::vector<gba_point_constraint> pc;
    std::vector<gba_image_constraint> ic;
    std::vector<gba_camera_constraint> cc;
    gba_problem p = vf.to_c(pc, ic, cc);
    std::vector<double> kci;
    if (cov.NumberOfKeys() > 0) {
      if (std::ptrdiff_t(cov.NumberOfKeys()) != vf.number_of_keys()) {
        last_status_ = GBA_ERR_INVALID;
        return -1;
      }
      kci.resize(4 * cov.NumberOfKeys());
      for (size_t k = 0; k < cov.NumberOfKeys(); ++k)
        for (int j = 0; j < 4; ++j) kci[4 * k + j] = double(cov.GetKeyBlock(k).m[j]);
      p.key_covariance_inverse = kci.data();
    }
    std::vector<double> cw(cov.constraints().begin(), cov.constraints().end());
    if (!cw.empty()) p.constraint_weights = cw.data();
    std::vector<double> y(size_t(detail::vec_len(near_y)));
    for (size_t i = 0; i < y.size(); ++i) y[i] = double(near_y.data()[i]);
    std::vector<double> x(initial_x_.begin(), initial_x_.end());
    last_status_ = gba_solve(&p, y.data(), &options_, x.data(), &last_report_);
    optimized_x.resize(x_size);
    for (std::ptrdiff_t i = 0; i < x_size; ++i) optimized_x.data()[i] = Scalar(x[size_t(i)]);
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

// ---------------------------------------------------------------------------
// CameraSharedCeresOptimizor (camera_shared_ceres_optimizor.hpp:163-500), the
// optimizer of the production pipeline (sfm_pipeline/bundle_adjustment_optimizor.hpp:48-49),
// with its constructor: (initial_x, number_of_threads = 1,
// max_num_iterations = 50, function_tolerance = 1e-6,
// parameter_tolerance = 1e-8).  The same model is solved by the device LM
// with the reference's robust loss, Huber(1.0) on every key (:253), and its
// stops: max_num_iterations iterations, an accepted step lowering the cost
// by at most function_tolerance of it, a step with
// ||delta|| <= parameter_tolerance (||x|| + parameter_tolerance), and
// Ceres' default gradient tolerance 1e-10 on ||g||inf.  number_of_threads
// is kept and not used (one GPU solves).  As in the reference, every group
// must be free and all three intrinsic groups computed (:193-202), else -1.
// ---------------------------------------------------------------------------
template <typename _VectorFunction>
class CameraSharedCeresOptimizor;

template <typename _Scalar>
class CameraSharedCeresOptimizor<CameraSharedVectorFunction<_Scalar> > {
 public:
  typedef _Scalar Scalar;
  typedef int Err;
  typedef CameraSharedVectorFunction<Scalar> VectorFunction;
  typedef typename VectorFunction::Index Index;
  typedef typename VectorFunction::XVector XVector;
  typedef typename VectorFunction::YVector YVector;
  typedef CameraSharedYCovarianceInverse<Scalar> YCovarianceInverse;

  template <typename XV>
  explicit CameraSharedCeresOptimizor(const XV& initial_x, int number_of_threads = 1,
                                      int max_num_iterations = 50,
                                      double function_tolerance = 1e-6,
                                      double parameter_tolerance = 1e-8)
      : lm_(initial_x, size_t(max_num_iterations > 0 ? max_num_iterations : 0), Scalar(1e-3),
            Scalar(1e-10), Scalar(parameter_tolerance)),
        number_of_threads_(number_of_threads) {
    gba_options& o = lm_.options();
    o.loss = GBA_LOSS_HUBER;
    o.huber_delta = 1.0;
    o.function_tolerance = function_tolerance;
  }

  // Solver choices beyond the reference's constructor (precision, device).
  gba_options& options() { return lm_.options(); }
  int number_of_threads() const { return number_of_threads_; }
  int last_status() const { return lm_.last_status(); }
  const gba_report& last_report() const { return lm_.last_report(); }

  template <typename YV, typename XV>
  Err operator()(const VectorFunction& vf, const YV& near_y, const YCovarianceInverse& cov,
                 XV& optimized_x) const {
    const IntrinsicComputationsMask& m = vf.intrinsic_computations_mask();
    if (vf.is_fix_points() || vf.is_fix_images() || vf.is_fix_cameras() ||
        !m[COMPUTE_RADIAL_DISTORTION] || !m[COMPUTE_DECENTERING_DISTORTION] ||
        !m[COMPUTE_INTRINSIC_PARAMS])
      return -1;
    return lm_(vf, near_y, cov, optimized_x);
  }

 private:
  CameraSharedLevenbergMarquardtOptimizor<VectorFunction> lm_;
  int number_of_threads_;
};

}  // namespace gba

#endif  // GBA_CAMERA_SHARED_HPP_
