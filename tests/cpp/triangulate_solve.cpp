// Drives the triangulation facade (include/gba/triangulate.hpp): the batch
// triangulator over every track, and MultipleViewMaximumLikelihoodEstimator
// (triangulate/multiple_view_maximum_likelihood_estimator.hpp:49-84) on the
// first track alone.
//
// usage: triangulate_solve <batch.bin> <out.bin> [--one-view]
// batch.bin: int64 V n m; double intrinsics[10V]; double extrinsics[6V];
//            int64 offsets[n + 1]; int64 views[m]; double keys[2m]
// out.bin:   double points[3n]; int32 status[n]; double first_point[3]
#include <array>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gba/triangulate.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int64_t hdr[3];
  if (std::fread(hdr, sizeof(int64_t), 3, f) != 3) return 2;
  const int64_t V = hdr[0], n = hdr[1], m = hdr[2];
  typedef gba::CameraIntrinsicParams<double> Intr;
  typedef gba::CameraExtrinsicParams<double> Extr;
  std::vector<Intr> intr;
  std::vector<Extr> extr;
  for (int64_t v = 0; v < V; ++v) {
    double a[10];
    if (std::fread(a, sizeof(double), 10, f) != 10) return 2;
    intr.push_back(Intr(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9]));
  }
  for (int64_t v = 0; v < V; ++v) {
    double a[6];
    if (std::fread(a, sizeof(double), 6, f) != 6) return 2;
    extr.push_back(Extr({{a[0], a[1], a[2]}}, {{a[3], a[4], a[5]}}));
  }
  std::vector<int64_t> off(n + 1), views(m);
  std::vector<double> keys(2 * m);
  if (std::fread(off.data(), sizeof(int64_t), off.size(), f) != off.size()) return 2;
  if (std::fread(views.data(), sizeof(int64_t), views.size(), f) != views.size()) return 2;
  if (std::fread(keys.data(), sizeof(double), keys.size(), f) != keys.size()) return 2;
  std::fclose(f);

  // the first track through the single-point estimator
  gba::MultipleViewMaximumLikelihoodEstimator<double> mle;
  gba::MultipleViewMaximumLikelihoodEstimator<double>::IntrinsicParamsContainer i0;
  gba::MultipleViewMaximumLikelihoodEstimator<double>::ExtrinsicParamsContainer e0;
  gba::MultipleViewMaximumLikelihoodEstimator<double>::KeyContainer k0;
  const int64_t last = (argc > 3 && std::strcmp(argv[3], "--one-view") == 0) ? off[0] + 1 : off[1];
  for (int64_t t = off[0]; t < last; ++t) {
    i0.push_back(intr[size_t(views[t])]);
    e0.push_back(extr[size_t(views[t])]);
    k0.push_back({{keys[2 * t], keys[2 * t + 1]}});
  }
  std::array<double, 3> p0 = {{0, 0, 0}};
  const int err0 = mle(i0, e0, k0, p0);
  std::printf("mle %d\n", err0);
  if (err0 != 0) return 1;

  gba::MultipleViewTriangulator<double> tri;
  std::vector<double> pts;
  std::vector<int32_t> st;
  const int err = tri(intr, extr, off, views, keys, pts, st);
  std::printf("batch %d\n", err);
  if (err != 0) return 1;
  FILE* g = std::fopen(argv[2], "wb");
  std::fwrite(pts.data(), sizeof(double), pts.size(), g);
  std::fwrite(st.data(), sizeof(int32_t), st.size(), g);
  std::fwrite(p0.data(), sizeof(double), 3, g);
  std::fclose(g);
  return 0;
}
