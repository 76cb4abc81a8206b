// Drives the GCP-constrained facade (include/gba/ba_gcp_constrained.hpp) the
// way the reference's scene expandor drives its optimizer
// (sfm_pipeline/scene_expandor_gcp_constrained.hpp:518-520): vector
// function, inverse covariance with 2x2 key blocks and 3x3 control-point
// blocks, optimizer, x back in the naive layout.
//
// usage: gcp_solve <problem.bin> <x_out.bin> [--bad-size]
// problem.bin: int64 C P F G iters; int64 feature_maps[2F] (camera, point);
//              double near_y[2F + 3G]; double key_blocks[4F];
//              double gcp_blocks[9G]; double x0[6C + 3P]
#include <cstdio>
#include <cstring>
#include <vector>

#include "gba/ba_gcp_constrained.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int64_t hdr[5];
  if (std::fread(hdr, sizeof(int64_t), 5, f) != 5) return 2;
  const int64_t C = hdr[0], P = hdr[1], F = hdr[2], G = hdr[3], iters = hdr[4];
  typedef gba::BAGCPConstrainedVectorFunction<double> VF;
  std::vector<int64_t> raw(2 * F);
  if (std::fread(raw.data(), sizeof(int64_t), raw.size(), f) != raw.size()) return 2;
  VF::FeatureMapContainer fm(static_cast<size_t>(F));
  for (int64_t k = 0; k < F; ++k) fm[k] = VF::FeatureMap(raw[2 * k], raw[2 * k + 1]);
  VF vf(C, P, F, fm, G);
  gba::VectorX<double> y(2 * F + 3 * G);
  if (std::fread(y.data(), sizeof(double), size_t(y.size()), f) != size_t(y.size())) return 2;
  gba::BAGCPConstrainedYCovarianceInverse<double> cov;
  cov.naive_y_covariance_inverse.blocks.resize(size_t(F));
  for (auto& b : cov.naive_y_covariance_inverse.blocks)
    if (std::fread(b.m, sizeof(double), 4, f) != 4) return 2;
  cov.gcp_blocks.resize(size_t(G));
  for (auto& b : cov.gcp_blocks)
    if (std::fread(b.m, sizeof(double), 9, f) != 9) return 2;
  gba::VectorX<double> x0(6 * C + 3 * P);
  if (std::fread(x0.data(), sizeof(double), size_t(x0.size()), f) != size_t(x0.size())) return 2;
  std::fclose(f);
  if (argc > 3 && std::strcmp(argv[3], "--bad-size") == 0) x0.resize(x0.size() - 1);

  gba::VectorX<double> y0;
  if (argc <= 3 && vf(x0, y0) != 0) return 4;   // the vector function at x0
  gba::BAGCPConstrainedLevenbergMarquardtOptimizor<VF> optimizor(x0, size_t(iters), 1e-3, 1e-8,
                                                                 1e-8);
  gba::VectorX<double> x;
  const int err = optimizor(vf, y, cov, x);
  std::printf("err %d status %d iterations %d final_cost %.17g stop %d\n", err,
              optimizor.last_status(), optimizor.last_report().iterations,
              optimizor.last_report().final_cost, optimizor.last_report().stop_reason);
  if (err != 0) return 1;
  FILE* g = std::fopen(argv[2], "wb");
  std::fwrite(x.data(), sizeof(double), size_t(x.size()), g);
  std::fwrite(y0.data(), sizeof(double), size_t(y0.size()), g);
  std::fclose(g);
  return 0;
}
