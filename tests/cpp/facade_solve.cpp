// Drives the header-only facade (include/gba/camera_shared.hpp) the way the
// reference's callers drive CameraSharedLevenbergMarquardtOptimizor
// (test_camera_shared_relative_pair.cpp:976-984): build the vector function,
// the inverse covariance and the optimizer, call it, read x back.
//
// usage: facade_solve <problem.bin> <x_out.bin> [--bad-size]
// problem.bin: int64 P I C K mask iters mode; int64 feature_maps[2K];
//              int64 image_camera_map[I]; double cameras[cC];
//              double near_y[2K]; double x0[3P + 6I (+ cC)]
// mode 0: cameras fixed, CameraSharedLevenbergMarquardtOptimizor
//         (max_itr_num = iters, tau 1e-3, eps1 = eps2 = 0);
// mode 1: cameras free (x0 carries them), CameraSharedCeresOptimizor
//         (threads 1, max_num_iterations = iters, ftol 1e-6, ptol 1e-8), as
//         sfm_pipeline/bundle_adjustment_optimizor.hpp:200-224 calls it;
// mode 2: as 1 with the cameras fixed (the Ceres optimizer refuses it);
// mode 3: points and cameras fixed (an images-only solve), the LM optimizer:
//         x0 holds the images [6I] and double points[3P] follows it.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gba/camera_shared.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int64_t hdr[7];
  if (std::fread(hdr, sizeof(int64_t), 7, f) != 7) return 2;
  const int64_t P = hdr[0], I = hdr[1], C = hdr[2], K = hdr[3], mask = hdr[4], iters = hdr[5],
                mode = hdr[6];
  typedef gba::CameraSharedVectorFunction<double> VF;
  VF vf;
  vf.set_number_of_points(P);
  vf.set_number_of_images(I);
  vf.set_number_of_cameras(C);
  vf.set_number_of_keys(K);
  vf.intrinsic_computations_mask() = gba::IntrinsicComputationsMask((unsigned long)mask);
  VF::FeatureMapContainer fm(static_cast<size_t>(K));
  std::vector<int64_t> raw(2 * K);
  if (std::fread(raw.data(), sizeof(int64_t), raw.size(), f) != raw.size()) return 2;
  for (int64_t k = 0; k < K; ++k) fm[k] = VF::FeatureMap(raw[2 * k], raw[2 * k + 1]);
  vf.set_feature_maps(fm);
  VF::ImageCameraMap icm(static_cast<size_t>(I));
  if (std::fread(icm.data(), sizeof(int64_t), icm.size(), f) != icm.size()) return 2;
  vf.set_image_camera_map(icm);
  std::vector<double> cams(size_t(C * vf.GetIntrinsicParamsSizePerCamera()));
  if (std::fread(cams.data(), sizeof(double), cams.size(), f) != cams.size()) return 2;
  if (mode != 1 && vf.set_fix_cameras(cams) != 0) return 3;
  gba::VectorX<double> y(2 * K);
  if (std::fread(y.data(), sizeof(double), size_t(y.size()), f) != size_t(y.size())) return 2;
  gba::VectorX<double> x0((mode == 3 ? 0 : 3 * P) + 6 * I + (mode == 1 ? int64_t(cams.size()) : 0));
  if (std::fread(x0.data(), sizeof(double), size_t(x0.size()), f) != size_t(x0.size())) return 2;
  if (mode == 3) {
    std::vector<double> pts(size_t(3 * P));
    if (std::fread(pts.data(), sizeof(double), pts.size(), f) != pts.size()) return 2;
    if (vf.set_fix_points(pts) != 0) return 3;
  }
  std::fclose(f);
  if (argc > 3 && std::strcmp(argv[3], "--bad-size") == 0) x0.resize(x0.size() - 1);

  gba::CameraSharedYCovarianceInverse<double> cov;
  cov.SetKeysUniformStdDev(1.0, size_t(K));
  gba::VectorX<double> x;
  int err = 0;
  if (mode == 0 || mode == 3) {
    // (max_itr_num, tau, eps1, eps2) as the reference's relative-pair test
    gba::CameraSharedLevenbergMarquardtOptimizor<VF> optimizor(x0, size_t(iters), 1e-3, 0.0, 0.0);
    err = optimizor(vf, y, cov, x);
    std::printf("err %d status %d iterations %d final_cost %.17g\n", err, optimizor.last_status(),
                optimizor.last_report().iterations, optimizor.last_report().final_cost);
  } else {
    gba::CameraSharedCeresOptimizor<VF> optimizor(x0, 1, int(iters), 1e-6, 1e-8);
    err = optimizor(vf, y, cov, x);
    std::printf("err %d status %d iterations %d final_cost %.17g stop %d\n", err,
                optimizor.last_status(), optimizor.last_report().iterations,
                optimizor.last_report().final_cost, optimizor.last_report().stop_reason);
  }
  if (err != 0) return 1;
  FILE* g = std::fopen(argv[2], "wb");
  std::fwrite(x.data(), sizeof(double), size_t(x.size()), g);
  std::fclose(g);
  return 0;
}
