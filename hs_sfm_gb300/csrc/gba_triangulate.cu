// gba_triangulate.cu -- gba_triangulate(): batched multi-view triangulation
// (hs_sfm triangulate/multiple_view_*), one thread per point, FP64.
//
// Each point: undistort its keys (sfm_utility/undistortor.hpp:24-80), build
// the DLT system rows u P3 - P1, v P3 - P2 of P = K [R | -R C]
// (triangulate/multiple_view_dlt.hpp:27-52) as the 4x4 normal matrix
// A^T A, take the eigenvector of its smallest eigenvalue (the smallest right
// singular vector of A) by cyclic Jacobi rotations, then refine the point by
// Levenberg-Marquardt (Madsen, Nielsen & Tingleff 2004, Alg. 3.16: the
// driver the reference's MultipleViewLevenbergMarquardtOptimizor binds,
// multiple_view_levenberg_marquardt_optimizor.hpp:50-99) on its keys with
// identity weights and the analytical 2x3 point Jacobian of the projection
// (sfm_utility/projective_functions.hpp:22-52).  Tracks are independent, so
// one launch covers the whole batch; the views (22 doubles each) are
// expanded once by a small kernel and read through the L1.
#include "gba_internal.h"

#include <cmath>
#include <cstdio>
#include <vector>

namespace gba {
namespace {

#define TRI_CUDA(call)                                                          \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      std::fprintf(stderr, "gba: %s failed: %s\n", #call, cudaGetErrorString(e_)); \
      throw CudaError{e_ == cudaErrorMemoryAllocation ? GBA_ERR_OOM : GBA_ERR_CUDA}; \
    }                                                                           \
  } while (0)

constexpr int kViewDoubles = 22;   // f s cx cy a k1 k2 k3 d1 d2, R (9), C (3)

thread_local double g_tri_last_ms = 0.0;   // the calling thread's last kernel time (profile)

__global__ void k_tri_views(int V, const double* __restrict__ intr, const double* __restrict__ extr,
                            double* __restrict__ views) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  double* o = views + (long long)kViewDoubles * v;
  for (int j = 0; j < 10; ++j) o[j] = intr[10LL * v + j];
  const double r0 = extr[6LL * v], r1 = extr[6LL * v + 1], r2 = extr[6LL * v + 2];
  const double th = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
  double* R = o + 10;
  if (th == 0.0) {
    for (int j = 0; j < 9; ++j) R[j] = (j % 4 == 0) ? 1.0 : 0.0;
  } else {   // world to camera: cos I + sin [k]x + (1 - cos) k k^T
    const double k0 = r0 / th, k1 = r1 / th, k2 = r2 / th;
    const double c = cos(th), s = sin(th), t = 1.0 - c;
    R[0] = c + t * k0 * k0;      R[1] = t * k0 * k1 - s * k2; R[2] = t * k0 * k2 + s * k1;
    R[3] = t * k1 * k0 + s * k2; R[4] = c + t * k1 * k1;      R[5] = t * k1 * k2 - s * k0;
    R[6] = t * k2 * k0 - s * k1; R[7] = t * k2 * k1 + s * k0; R[8] = c + t * k2 * k2;
  }
  for (int j = 0; j < 3; ++j) o[19 + j] = extr[6LL * v + 3 + j];
}

struct TriView {
  double f, s, cx, cy, a, k1, k2, k3, d1, d2;
  double R[9], C[3];
};

__device__ __forceinline__ void load_view(const double* __restrict__ views, long long v, TriView& w) {
  const double* p = views + kViewDoubles * v;
  w.f = __ldg(p); w.s = __ldg(p + 1); w.cx = __ldg(p + 2); w.cy = __ldg(p + 3); w.a = __ldg(p + 4);
  w.k1 = __ldg(p + 5); w.k2 = __ldg(p + 6); w.k3 = __ldg(p + 7); w.d1 = __ldg(p + 8); w.d2 = __ldg(p + 9);
#pragma unroll
  for (int j = 0; j < 9; ++j) w.R[j] = __ldg(p + 10 + j);
#pragma unroll
  for (int j = 0; j < 3; ++j) w.C[j] = __ldg(p + 19 + j);
}

// Key of X in view w; with J, also d key / d X (2 x 3, row-major).
template <bool kJac>
__device__ __forceinline__ void tri_project(const TriView& w, const double X[3], double key[2], double* J) {
  const double d0 = X[0] - w.C[0], d1v = X[1] - w.C[1], d2v = X[2] - w.C[2];
  const double c0 = w.R[0] * d0 + w.R[1] * d1v + w.R[2] * d2v;
  const double c1 = w.R[3] * d0 + w.R[4] * d1v + w.R[5] * d2v;
  const double c2 = w.R[6] * d0 + w.R[7] * d1v + w.R[8] * d2v;
  const double iz = 1.0 / c2;
  const double x = c0 * iz, y = c1 * iz;
  const double r2 = x * x + y * y;
  const double coeff = w.k1 * r2 + w.k2 * r2 * r2 + w.k3 * r2 * r2 * r2;
  const double ex = x + coeff * x + 2.0 * w.d1 * x * y + w.d2 * (r2 + 2.0 * x * x);
  const double ey = y + coeff * y + 2.0 * w.d2 * x * y + w.d1 * (r2 + 2.0 * y * y);
  key[0] = w.f * ex + w.s * ey + w.cx;
  key[1] = w.f * w.a * ey + w.cy;
  if (kJac) {
    const double dc = 2.0 * (w.k1 + 2.0 * w.k2 * r2 + 3.0 * w.k3 * r2 * r2);
    const double exx = 1.0 + coeff + dc * x * x + 2.0 * w.d1 * y + 6.0 * w.d2 * x;
    const double exy = dc * x * y + 2.0 * w.d1 * x + 2.0 * w.d2 * y;
    const double eyx = dc * x * y + 2.0 * w.d2 * y + 2.0 * w.d1 * x;
    const double eyy = 1.0 + coeff + dc * y * y + 2.0 * w.d2 * x + 6.0 * w.d1 * y;
    const double kxx = w.f * exx + w.s * eyx, kxy = w.f * exy + w.s * eyy;
    const double kyx = w.f * w.a * eyx, kyy = w.f * w.a * eyy;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double nx = (w.R[j] - x * w.R[6 + j]) * iz;
      const double ny = (w.R[3 + j] - y * w.R[6 + j]) * iz;
      J[j] = kxx * nx + kxy * ny;
      J[3 + j] = kyx * nx + kyy * ny;
    }
  }
}

__device__ double tri_cost(const double* views, const long long* tv, const double* keys, int m,
                           const double X[3]) {
  double F = 0.0;
  for (int i = 0; i < m; ++i) {
    TriView w;
    load_view(views, tv[i], w);
    double k[2];
    tri_project<false>(w, X, k, nullptr);
    const double a = k[0] - keys[2 * i], b = k[1] - keys[2 * i + 1];
    F += a * a + b * b;
  }
  return F;
}

__device__ void tri_normal(const double* views, const long long* tv, const double* keys, int m,
                           const double X[3], double N[6], double g[3]) {
#pragma unroll
  for (int e = 0; e < 6; ++e) N[e] = 0.0;
  g[0] = g[1] = g[2] = 0.0;
  for (int i = 0; i < m; ++i) {
    TriView w;
    load_view(views, tv[i], w);
    double k[2], J[6];
    tri_project<true>(w, X, k, J);
    const double r0 = k[0] - keys[2 * i], r1 = k[1] - keys[2 * i + 1];
    N[0] += J[0] * J[0] + J[3] * J[3];
    N[1] += J[0] * J[1] + J[3] * J[4];
    N[2] += J[0] * J[2] + J[3] * J[5];
    N[3] += J[1] * J[1] + J[4] * J[4];
    N[4] += J[1] * J[2] + J[4] * J[5];
    N[5] += J[2] * J[2] + J[5] * J[5];
    g[0] += J[0] * r0 + J[3] * r1;
    g[1] += J[1] * r0 + J[4] * r1;
    g[2] += J[2] * r0 + J[5] * r1;
  }
}

// (N + mu I) d = g by a 3x3 Cholesky; false when not positive definite.
__device__ bool tri_solve(const double N[6], double mu, const double g[3], double d[3]) {
  const double a00 = N[0] + mu, a11 = N[3] + mu, a22 = N[5] + mu;
  if (!(a00 > 0.0)) return false;
  const double l00 = sqrt(a00), l10 = N[1] / l00, l20 = N[2] / l00;
  const double s11 = a11 - l10 * l10;
  if (!(s11 > 0.0)) return false;
  const double l11 = sqrt(s11), l21 = (N[4] - l20 * l10) / l11;
  const double s22 = a22 - l20 * l20 - l21 * l21;
  if (!(s22 > 0.0)) return false;
  const double l22 = sqrt(s22);
  const double y0 = g[0] / l00, y1 = (g[1] - l10 * y0) / l11, y2 = (g[2] - l20 * y0 - l21 * y1) / l22;
  d[2] = y2 / l22;
  d[1] = (y1 - l21 * d[2]) / l11;
  d[0] = (y0 - l10 * d[1] - l20 * d[2]) / l00;
  return true;
}

// Eigenvector of the smallest eigenvalue of the symmetric 4x4 A (row-major),
// cyclic Jacobi (Golub & Van Loan 8.5), at most 30 sweeps.
__device__ void tri_smallest_eigenvector(double A[16], double out[4]) {
  double V[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) V[e] = (e % 5 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0.0, tot = 0.0;
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      tot += A[e] * A[e];
      if (e % 5 != 0) off += A[e] * A[e];
    }
    if (off <= 1e-30 * tot) break;
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll
      for (int q = p + 1; q < 4; ++q) {
        const double apq = A[4 * p + q];
        if (apq != 0.0) {
          const double theta = (A[4 * q + q] - A[4 * p + p]) / (2.0 * apq);
          const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const double akp = A[4 * k + p], akq = A[4 * k + q];
            A[4 * k + p] = c * akp - s * akq;
            A[4 * k + q] = s * akp + c * akq;
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const double apk = A[4 * p + k], aqk = A[4 * q + k];
            A[4 * p + k] = c * apk - s * aqk;
            A[4 * q + k] = s * apk + c * aqk;
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const double vkp = V[4 * k + p], vkq = V[4 * k + q];
            V[4 * k + p] = c * vkp - s * vkq;
            V[4 * k + q] = s * vkp + c * vkq;
          }
        }
      }
    }
  }
  double best = A[0];
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = V[4 * k];
#pragma unroll
  for (int i = 1; i < 4; ++i)
    if (A[5 * i] < best) {
      best = A[5 * i];
#pragma unroll
      for (int k = 0; k < 4; ++k) out[k] = V[4 * k + i];
    }
}

struct TriParams {
  int max_iterations;
  double tau, eps1, eps2;
};

__global__ void __launch_bounds__(128) k_triangulate(long long n, const long long* __restrict__ off,
                                                     const long long* __restrict__ track_views,
                                                     const double* __restrict__ track_keys,
                                                     const double* __restrict__ views, TriParams prm,
                                                     double* __restrict__ points, int* __restrict__ status) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j >= n) return;
  const long long t0 = off[j];
  const int m = int(off[j + 1] - t0);
  const long long* tv = track_views + t0;
  const double* keys = track_keys + 2 * t0;
  double X[3] = {0.0, 0.0, 0.0};
  int st = GBA_OK;
  if (m < 2) {
    st = GBA_ERR_INVALID;
  } else {
    // DLT normal matrix A^T A of the undistorted keys
    double M[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) M[e] = 0.0;
    for (int i = 0; i < m; ++i) {
      TriView w;
      load_view(views, tv[i], w);
      const double fa = w.f * w.a;
      const double y0 = (keys[2 * i + 1] - w.cy) / fa;
      const double x0 = (keys[2 * i] - w.cx - w.s * y0) / w.f;
      double x = x0, y = y0;
      for (int it = 0; it < 5; ++it) {
        const double r2 = x * x + y * y;
        const double rc = 1.0 / (1.0 + r2 * (w.k1 + r2 * (w.k2 + r2 * w.k3)));
        const double dx = 2.0 * w.d1 * x * y + w.d2 * (r2 + 2.0 * x * x);
        const double dy = 2.0 * w.d2 * x * y + w.d1 * (r2 + 2.0 * y * y);
        x = (x0 - dx) * rc;
        y = (y0 - dy) * rc;
      }
      const double u = w.f * x + w.s * y + w.cx, v = fa * y + w.cy;
      // P = K [R | -R C]
      double Rt[12];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) Rt[4 * r + c] = w.R[3 * r + c];
        Rt[4 * r + 3] = -(w.R[3 * r] * w.C[0] + w.R[3 * r + 1] * w.C[1] + w.R[3 * r + 2] * w.C[2]);
      }
      double row0[4], row1[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double p0 = w.f * Rt[c] + w.s * Rt[4 + c] + w.cx * Rt[8 + c];
        const double p1 = fa * Rt[4 + c] + w.cy * Rt[8 + c];
        const double p2 = Rt[8 + c];
        row0[c] = u * p2 - p0;
        row1[c] = v * p2 - p1;
      }
#pragma unroll
      for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int b = 0; b < 4; ++b) M[4 * a + b] += row0[a] * row0[b] + row1[a] * row1[b];
      }
    }
    double h[4];
    tri_smallest_eigenvector(M, h);
    if (h[3] == 0.0) {
      st = GBA_ERR_NAN;
    } else {
      X[0] = h[0] / h[3];
      X[1] = h[1] / h[3];
      X[2] = h[2] / h[3];
      if (!(isfinite(X[0]) && isfinite(X[1]) && isfinite(X[2]))) st = GBA_ERR_NAN;
    }
    if (st == GBA_OK) {   // LM refinement
      double F = tri_cost(views, tv, keys, m, X), N[6], g[3];
      tri_normal(views, tv, keys, m, X, N, g);
      double ginf = fmax(fabs(g[0]), fmax(fabs(g[1]), fabs(g[2])));
      bool found = ginf <= prm.eps1;
      double mu = prm.tau * fmax(N[0], fmax(N[3], N[5]));
      double nu = 2.0;
      for (int k = 0; !found && k < prm.max_iterations; ++k) {
        double d[3];
        if (!tri_solve(N, mu, g, d)) {
          mu *= nu;
          nu *= 2.0;
          continue;
        }
        const double dn = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        const double xn = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
        if (dn <= prm.eps2 * (xn + prm.eps2)) break;
        const double Xn[3] = {X[0] - d[0], X[1] - d[1], X[2] - d[2]};
        const double Fn = tri_cost(views, tv, keys, m, Xn);
        const double denom = mu * dn * dn + (g[0] * d[0] + g[1] * d[1] + g[2] * d[2]);
        const double rho = (F - Fn) / denom;
        if (isfinite(Fn) && rho > 0.0) {
          X[0] = Xn[0];
          X[1] = Xn[1];
          X[2] = Xn[2];
          F = Fn;
          tri_normal(views, tv, keys, m, X, N, g);
          ginf = fmax(fabs(g[0]), fmax(fabs(g[1]), fabs(g[2])));
          found = ginf <= prm.eps1;
          const double tt = 2.0 * rho - 1.0;
          mu *= fmax(1.0 / 3.0, 1.0 - tt * tt * tt);
          nu = 2.0;
        } else {
          mu *= nu;
          nu *= 2.0;
        }
      }
      if (!isfinite(F)) st = GBA_ERR_NAN;
    }
  }
  points[3 * j] = X[0];
  points[3 * j + 1] = X[1];
  points[3 * j + 2] = X[2];
  status[j] = st;
}

}  // namespace
}  // namespace gba

extern "C" int gba_triangulate(const gba_triangulation* p, const gba_options* o, double* points,
                               int32_t* point_status) {
  using namespace gba;
  if (!p || !o || !points || p->number_of_views < 0 || p->number_of_points < 0 ||
      o->max_iterations < 0)
    return GBA_ERR_INVALID;
  const long long V = p->number_of_views, n = p->number_of_points;
  if (n == 0) return GBA_OK;
  if (!p->track_offsets || (V > 0 && (!p->intrinsics || !p->extrinsics))) return GBA_ERR_INVALID;
  if (p->track_offsets[0] != 0) return GBA_ERR_INVALID;
  for (long long j = 0; j < n; ++j)
    if (p->track_offsets[j + 1] < p->track_offsets[j]) return GBA_ERR_INVALID;
  const long long m = p->track_offsets[n];
  if (m > 0 && (!p->track_views || !p->track_keys)) return GBA_ERR_INVALID;
  for (long long t = 0; t < m; ++t)
    if (p->track_views[t] < 0 || p->track_views[t] >= V) return GBA_ERR_BAD_INDEX;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return GBA_ERR_NO_DEVICE;
  }
  cudaStream_t s = nullptr;
  std::vector<void*> bufs;
  int err = GBA_OK;
  try {
    TRI_CUDA(cudaSetDevice(o->device));
    TRI_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    auto dev = [&](size_t bytes) {
      void* d = nullptr;
      TRI_CUDA(cudaMallocAsync(&d, bytes > 0 ? bytes : 1, s));
      bufs.push_back(d);
      return d;
    };
    auto up = [&](const void* h, size_t bytes) {
      void* d = dev(bytes);
      if (bytes) TRI_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s));
      return d;
    };
    const double* d_intr = static_cast<const double*>(up(p->intrinsics, sizeof(double) * 10 * V));
    const double* d_extr = static_cast<const double*>(up(p->extrinsics, sizeof(double) * 6 * V));
    double* d_views = static_cast<double*>(dev(sizeof(double) * kViewDoubles * (V > 0 ? V : 1)));
    const long long* d_off = static_cast<const long long*>(up(p->track_offsets, sizeof(int64_t) * (n + 1)));
    const long long* d_tv = static_cast<const long long*>(up(p->track_views, sizeof(int64_t) * m));
    const double* d_keys = static_cast<const double*>(up(p->track_keys, sizeof(double) * 2 * m));
    double* d_pts = static_cast<double*>(dev(sizeof(double) * 3 * n));
    int* d_st = static_cast<int*>(dev(sizeof(int) * n));
    int launches = 0;
    if (V > 0) {
      k_tri_views<<<unsigned((V + 127) / 128), 128, 0, s>>>(int(V), d_intr, d_extr, d_views);
      ++launches;
    }
    TriParams prm{o->max_iterations, o->tau, o->eps1, o->eps2};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    if (o->profile) {
      TRI_CUDA(cudaEventCreate(&ev[0]));
      TRI_CUDA(cudaEventCreate(&ev[1]));
      TRI_CUDA(cudaEventRecord(ev[0], s));
    }
    k_triangulate<<<unsigned((n + 127) / 128), 128, 0, s>>>(n, d_off, d_tv, d_keys, d_views, prm,
                                                             d_pts, d_st);
    ++launches;
    TRI_CUDA(cudaGetLastError());
    g_tri_last_ms = 0.0;
    if (o->profile) {
      TRI_CUDA(cudaEventRecord(ev[1], s));
      TRI_CUDA(cudaEventSynchronize(ev[1]));
      float ms = 0.0f;
      TRI_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      g_tri_last_ms = ms;
      cudaEventDestroy(ev[0]);
      cudaEventDestroy(ev[1]);
    }
    count_launches(launches);
    TRI_CUDA(cudaMemcpyAsync(points, d_pts, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    std::vector<int> st(static_cast<size_t>(n));
    TRI_CUDA(cudaMemcpyAsync(st.data(), d_st, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
    TRI_CUDA(cudaStreamSynchronize(s));
    if (point_status)
      for (long long j = 0; j < n; ++j) point_status[j] = st[size_t(j)];
  } catch (const CudaError& e) {
    err = e.status;
  }
  for (void* b : bufs) cudaFreeAsync(b, s);
  if (s) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  return err;
}

extern "C" double gba_triangulate_last_kernel_ms(void) { return gba::g_tri_last_ms; }
