// gba_oracle_triangulate.cpp -- CPU FP64 oracle of the batched multi-view
// triangulation.  TEST INFRASTRUCTURE ONLY (see gba_oracle.h): a plain
// restatement of hs_sfm's triangulate/ path, used by the tests as the checker
// and by the benchmark as the timed CPU baseline.
//
//   projection      sfm_utility/projective_functions.hpp:22-52 (rotation of
//                   X - position, divide by z, radial + decentering deltas of
//                   the undistorted normalized key, K)
//   undistortion    sfm_utility/undistortor.hpp:24-80 (normalize by K^-1,
//                   five fixed-point iterations, denormalize)
//   initialisation  triangulate/multiple_view_dlt.hpp:27-52 (rows
//                   u P3 - P1, v P3 - P2 of P = K [R | -R C]; the right
//                   singular vector of the smallest singular value)
//   refinement      triangulate/multiple_view_levenberg_marquardt_optimizor.hpp:50-99
//                   with the LM driver of the absent hs_optimizor restated
//                   from Madsen, Nielsen & Tingleff (2004) Alg. 3.16, the
//                   same restatement as oracle_lm_solve, identity weights.
// Deviations, both deliberate: the smallest right singular vector of A is
// taken as the eigenvector of A^T A for its smallest eigenvalue (cyclic
// Jacobi, Golub & Van Loan 8.5), which is the same vector; the refinement
// uses the analytical point Jacobian where the reference's generic driver
// may use finite differences -- both converge to the same minimum.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "gba_oracle.h"

namespace {

struct View {
  double f, s, cx, cy, a, k1, k2, k3, d1, d2;
  double R[9];
  double C[3];
};

void view_of(const double* intr, const double* extr, View& v) {
  v.f = intr[0]; v.s = intr[1]; v.cx = intr[2]; v.cy = intr[3]; v.a = intr[4];
  v.k1 = intr[5]; v.k2 = intr[6]; v.k3 = intr[7]; v.d1 = intr[8]; v.d2 = intr[9];
  const double* r = extr;
  const double th = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  if (th == 0.0) {
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::memcpy(v.R, I, sizeof(I));
  } else {   // R = cos I + sin [k]x + (1 - cos) k k^T
    const double k[3] = {r[0] / th, r[1] / th, r[2] / th};
    const double c = std::cos(th), s = std::sin(th), t = 1 - c;
    v.R[0] = c + t * k[0] * k[0];        v.R[1] = t * k[0] * k[1] - s * k[2]; v.R[2] = t * k[0] * k[2] + s * k[1];
    v.R[3] = t * k[1] * k[0] + s * k[2]; v.R[4] = c + t * k[1] * k[1];        v.R[5] = t * k[1] * k[2] - s * k[0];
    v.R[6] = t * k[2] * k[0] - s * k[1]; v.R[7] = t * k[2] * k[1] + s * k[0]; v.R[8] = c + t * k[2] * k[2];
  }
  for (int i = 0; i < 3; ++i) v.C[i] = extr[3 + i];
}

// Key of X and (if J) its 2x3 derivative.
void project(const View& v, const double X[3], double key[2], double* J) {
  const double d[3] = {X[0] - v.C[0], X[1] - v.C[1], X[2] - v.C[2]};
  double c[3];
  for (int i = 0; i < 3; ++i) c[i] = v.R[3 * i] * d[0] + v.R[3 * i + 1] * d[1] + v.R[3 * i + 2] * d[2];
  const double x = c[0] / c[2], y = c[1] / c[2];
  const double r2 = x * x + y * y;
  const double coeff = v.k1 * r2 + v.k2 * r2 * r2 + v.k3 * r2 * r2 * r2;
  const double ex = x + coeff * x + 2 * v.d1 * x * y + v.d2 * (r2 + 2 * x * x);
  const double ey = y + coeff * y + 2 * v.d2 * x * y + v.d1 * (r2 + 2 * y * y);
  key[0] = v.f * ex + v.s * ey + v.cx;
  key[1] = v.f * v.a * ey + v.cy;
  if (!J) return;
  // de/dn
  const double dc = 2 * (v.k1 + 2 * v.k2 * r2 + 3 * v.k3 * r2 * r2);   // d coeff / d r2 * 2
  const double exx = 1 + coeff + dc * x * x + 2 * v.d1 * y + 6 * v.d2 * x;
  const double exy = dc * x * y + 2 * v.d1 * x + 2 * v.d2 * y;
  const double eyx = dc * x * y + 2 * v.d2 * y + 2 * v.d1 * x;
  const double eyy = 1 + coeff + dc * y * y + 2 * v.d2 * x + 6 * v.d1 * y;
  // dk/dn = K2 de/dn, K2 = [f s; 0 f a]
  const double kxx = v.f * exx + v.s * eyx, kxy = v.f * exy + v.s * eyy;
  const double kyx = v.f * v.a * eyx, kyy = v.f * v.a * eyy;
  // dn/dX = (1/c2) [1 0 -x; 0 1 -y] R
  for (int j = 0; j < 3; ++j) {
    const double nx = (v.R[j] - x * v.R[6 + j]) / c[2];
    const double ny = (v.R[3 + j] - y * v.R[6 + j]) / c[2];
    J[j] = kxx * nx + kxy * ny;
    J[3 + j] = kyx * nx + kyy * ny;
  }
}

// Undistorted pixel key (sfm_utility/undistortor.hpp:24-80).
void undistort(const View& v, const double in[2], double out[2]) {
  // K^-1 of [f s cx; 0 f a cy; 0 0 1]
  const double fa = v.f * v.a;
  const double y0 = (in[1] - v.cy) / fa;
  const double x0 = (in[0] - v.cx - v.s * y0) / v.f;
  double x = x0, y = y0;
  for (int i = 0; i < 5; ++i) {
    const double r2 = x * x + y * y;
    const double rc = 1.0 / (1 + r2 * (v.k1 + r2 * (v.k2 + r2 * v.k3)));
    const double dx = 2.0 * v.d1 * x * y + v.d2 * (r2 + 2.0 * x * x);
    const double dy = 2.0 * v.d2 * x * y + v.d1 * (r2 + 2.0 * y * y);
    x = (x0 - dx) * rc;
    y = (y0 - dy) * rc;
  }
  out[0] = v.f * x + v.s * y + v.cx;
  out[1] = fa * y + v.cy;
}

// Eigenvector of the smallest eigenvalue of a symmetric 4x4 matrix by
// cyclic Jacobi rotations (Golub & Van Loan, Matrix Computations, 8.5).
void smallest_eigenvector(double A[16], double out[4]) {
  double V[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0, tot = 0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        tot += A[4 * i + j] * A[4 * i + j];
        if (i != j) off += A[4 * i + j] * A[4 * i + j];
      }
    if (off <= 1e-30 * tot) break;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 4; ++q) {
        const double apq = A[4 * p + q];
        if (apq == 0.0) continue;
        const double theta = (A[4 * q + q] - A[4 * p + p]) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < 4; ++k) {   // A <- J^T A J, columns then rows
          const double akp = A[4 * k + p], akq = A[4 * k + q];
          A[4 * k + p] = c * akp - s * akq;
          A[4 * k + q] = s * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          const double apk = A[4 * p + k], aqk = A[4 * q + k];
          A[4 * p + k] = c * apk - s * aqk;
          A[4 * q + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 4; ++k) {
          const double vkp = V[4 * k + p], vkq = V[4 * k + q];
          V[4 * k + p] = c * vkp - s * vkq;
          V[4 * k + q] = s * vkp + c * vkq;
        }
      }
  }
  int m = 0;
  for (int i = 1; i < 4; ++i)
    if (A[5 * i] < A[5 * m]) m = i;
  for (int i = 0; i < 4; ++i) out[i] = V[4 * i + m];
}

struct Track {
  const View* views;
  const int64_t* vid;
  const double* keys;
  int64_t m;
};

double cost_at(const Track& t, const double X[3]) {
  double F = 0;
  for (int64_t i = 0; i < t.m; ++i) {
    double k[2];
    project(t.views[t.vid[i]], X, k, nullptr);
    const double a = k[0] - t.keys[2 * i], b = k[1] - t.keys[2 * i + 1];
    F += a * a + b * b;
  }
  return F;
}

// N = J^T J (upper 6), g = J^T r at X.
void normal_at(const Track& t, const double X[3], double N[6], double g[3]) {
  std::fill(N, N + 6, 0.0);
  std::fill(g, g + 3, 0.0);
  for (int64_t i = 0; i < t.m; ++i) {
    double k[2], J[6];
    project(t.views[t.vid[i]], X, k, J);
    const double r0 = k[0] - t.keys[2 * i], r1 = k[1] - t.keys[2 * i + 1];
    int e = 0;
    for (int a = 0; a < 3; ++a) {
      for (int b = a; b < 3; ++b) N[e++] += J[a] * J[b] + J[3 + a] * J[3 + b];
      g[a] += J[a] * r0 + J[3 + a] * r1;
    }
  }
}

// (N + mu I) d = g by Cholesky; false when not positive definite.
bool solve3(const double N[6], double mu, const double g[3], double d[3]) {
  const double a00 = N[0] + mu, a01 = N[1], a02 = N[2], a11 = N[3] + mu, a12 = N[4], a22 = N[5] + mu;
  if (!(a00 > 0)) return false;
  const double l00 = std::sqrt(a00), l10 = a01 / l00, l20 = a02 / l00;
  const double s11 = a11 - l10 * l10;
  if (!(s11 > 0)) return false;
  const double l11 = std::sqrt(s11), l21 = (a12 - l20 * l10) / l11;
  const double s22 = a22 - l20 * l20 - l21 * l21;
  if (!(s22 > 0)) return false;
  const double l22 = std::sqrt(s22);
  const double y0 = g[0] / l00, y1 = (g[1] - l10 * y0) / l11, y2 = (g[2] - l20 * y0 - l21 * y1) / l22;
  d[2] = y2 / l22;
  d[1] = (y1 - l21 * d[2]) / l11;
  d[0] = (y0 - l10 * d[1] - l20 * d[2]) / l00;
  return true;
}

int triangulate_one(const Track& t, const gba_options& o, double X[3]) {
  if (t.m < 2) return GBA_ERR_INVALID;   // multiple_view_levenberg_marquardt_optimizor.hpp:66-70
  // DLT on undistorted keys
  double M[16] = {0};
  for (int64_t i = 0; i < t.m; ++i) {
    const View& v = t.views[t.vid[i]];
    double u[2];
    undistort(v, t.keys + 2 * i, u);
    // P = K [R | -R C]
    double Rt[12];
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c) Rt[4 * r + c] = v.R[3 * r + c];
      Rt[4 * r + 3] = -(v.R[3 * r] * v.C[0] + v.R[3 * r + 1] * v.C[1] + v.R[3 * r + 2] * v.C[2]);
    }
    double P[12];
    for (int c = 0; c < 4; ++c) {
      P[c] = v.f * Rt[c] + v.s * Rt[4 + c] + v.cx * Rt[8 + c];
      P[4 + c] = v.f * v.a * Rt[4 + c] + v.cy * Rt[8 + c];
      P[8 + c] = Rt[8 + c];
    }
    double row[2][4];
    for (int c = 0; c < 4; ++c) {
      row[0][c] = u[0] * P[8 + c] - P[c];
      row[1][c] = u[1] * P[8 + c] - P[4 + c];
    }
    for (int r = 0; r < 2; ++r)
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) M[4 * a + b] += row[r][a] * row[r][b];
  }
  double h[4];
  smallest_eigenvector(M, h);
  if (h[3] == 0.0) return GBA_ERR_NAN;
  for (int i = 0; i < 3; ++i) X[i] = h[i] / h[3];
  if (!(std::isfinite(X[0]) && std::isfinite(X[1]) && std::isfinite(X[2]))) return GBA_ERR_NAN;
  // LM (MNT Alg. 3.16, as oracle_lm_solve)
  double F = cost_at(t, X), N[6], g[3];
  normal_at(t, X, N, g);
  double ginf = std::max(std::fabs(g[0]), std::max(std::fabs(g[1]), std::fabs(g[2])));
  bool found = ginf <= o.eps1;
  double mu = o.tau * std::max(N[0], std::max(N[3], N[5]));
  double nu = 2.0;
  for (int k = 0; !found && k < o.max_iterations; ++k) {
    double d[3];
    if (!solve3(N, mu, g, d)) {
      mu *= nu;
      nu *= 2;
      continue;
    }
    const double dn = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double xn = std::sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
    if (dn <= o.eps2 * (xn + o.eps2)) break;
    const double Xn[3] = {X[0] - d[0], X[1] - d[1], X[2] - d[2]};
    const double Fn = cost_at(t, Xn);
    const double denom = mu * dn * dn + (g[0] * d[0] + g[1] * d[1] + g[2] * d[2]);
    const double rho = (F - Fn) / denom;
    if (std::isfinite(Fn) && rho > 0) {
      std::copy(Xn, Xn + 3, X);
      F = Fn;
      normal_at(t, X, N, g);
      ginf = std::max(std::fabs(g[0]), std::max(std::fabs(g[1]), std::fabs(g[2])));
      found = ginf <= o.eps1;
      const double tt = 2 * rho - 1;
      mu *= std::max(1.0 / 3.0, 1 - tt * tt * tt);
      nu = 2;
    } else {
      mu *= nu;
      nu *= 2;
    }
  }
  return std::isfinite(F) ? GBA_OK : GBA_ERR_NAN;
}

}  // namespace

extern "C" int oracle_triangulate(const gba_triangulation* p, const gba_options* o, double* points,
                                  int32_t* status) {
  if (!p || !o || !points || p->number_of_views < 0 || p->number_of_points < 0)
    return GBA_ERR_INVALID;
  const int64_t V = p->number_of_views, n = p->number_of_points;
  if (n > 0 && !p->track_offsets) return GBA_ERR_INVALID;
  View* views = new View[size_t(std::max<int64_t>(V, 1))];
  for (int64_t v = 0; v < V; ++v) view_of(p->intrinsics + 10 * v, p->extrinsics + 6 * v, views[v]);
  int err = GBA_OK;
  for (int64_t j = 0; j < n && !err; ++j)
    for (int64_t t = p->track_offsets[j]; t < p->track_offsets[j + 1]; ++t)
      if (p->track_views[t] < 0 || p->track_views[t] >= V) err = GBA_ERR_BAD_INDEX;
  for (int64_t j = 0; j < n && !err; ++j) {
    Track t{views, p->track_views + p->track_offsets[j], p->track_keys + 2 * p->track_offsets[j],
            p->track_offsets[j + 1] - p->track_offsets[j]};
    double X[3] = {0, 0, 0};
    const int st = triangulate_one(t, *o, X);
    for (int i = 0; i < 3; ++i) points[3 * j + i] = X[i];
    if (status) status[j] = st;
  }
  delete[] views;
  return err;
}
