// gba_kernels.cu -- the sm_103a kernels of one Levenberg-Marquardt iteration
// over a batch of bundle-adjustment problems, and their launchers.
//
// Stage map (reference: include/hs_sfm/bundle_adjustment/):
//   k_image_prep     rotation of each image: Rodrigues matrix (FP64) and the
//                    coefficients of the analytical rotation derivative
//                    (camera_shared_analytical_jacobian_matrix_calculator.hpp:341-380)
//   k_cost           r = f(x) - y in FP64, whitening by the key weight, Huber
//                    rho and IRLS weight, per-chunk FP64 cost sums
//                    (camera_shared_vector_function.hpp:634-744,
//                     camera_shared_mahalanobis_distance_calculator.hpp:28-58)
//   k_linearize      per point: analytical Jacobian of each key (T), whitened
//                    blocks J_p, J_i, V_p = sum J_p^T J_p, g_p = sum J_p^T r
//                    (analytical_jacobian_matrix_calculator.hpp:66-557,
//                     normal_equation_builder.hpp:207-220,377-391)
//   k_image_reduce   per image: U_i = sum J_i^T J_i, g_i = sum J_i^T r with
//                    compensated (Kahan) lane sums (normal_equation_builder.hpp:221-234)
//   k_point_schur    per point: C C^T = V_p + mu I, Z_a = C^-1 J_p^T J_i,
//                    h_p = C^-1 g_p (normal_equation_solver.hpp:141-184)
//   k_assemble_items per block (i<=j) of the reduced system: -sum Z_a^T Z_b
//                    over the points seen by both images, rhs terms
//                    (normal_equation_solver.hpp:190-267,398-420)
//   k_assemble_S     dense FP64 reduced system S and rhs b
//   k_chol_*         tiled FP64 Cholesky with the forward solve folded in,
//                    then the backward solve (normal_equation_solver.hpp:448-466)
//   k_backsub        delta_p = C^-T (h_p - sum Z_a delta_i), x_new = x - delta
//                    (normal_equation_solver.hpp:468-538)
//   k_ctrl_*         the LM decisions per problem on the device (Madsen,
//                    Nielsen & Tingleff 2004, Alg. 3.16 as bound by
//                    camera_shared_nllso_meta_levenberg_marquardt.hpp:33-106)
#include "gba_internal.h"

#include <cmath>
#include <cstdio>

namespace gba {
namespace {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dbits(double v) {
  return static_cast<unsigned long long>(__double_as_longlong(v));
}
__device__ __forceinline__ double bitsd(unsigned long long b) {
  return __longlong_as_double(static_cast<long long>(b));
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

// Load N consecutive T (N even for double, multiple of 4 for float) from a
// 16-byte aligned address with vector loads.
template <int N>
__device__ __forceinline__ void load_vec(const float* __restrict__ p, float* out) {
  static_assert(N % 4 == 0, "float vectors of 4");
#pragma unroll
  for (int i = 0; i < N / 4; ++i) {
    float4 v = __ldg(reinterpret_cast<const float4*>(p) + i);
    out[4 * i] = v.x; out[4 * i + 1] = v.y; out[4 * i + 2] = v.z; out[4 * i + 3] = v.w;
  }
}
template <int N>
__device__ __forceinline__ void load_vec(const double* __restrict__ p, double* out) {
  static_assert(N % 2 == 0, "double vectors of 2");
#pragma unroll
  for (int i = 0; i < N / 2; ++i) {
    double2 v = __ldg(reinterpret_cast<const double2*>(p) + i);
    out[2 * i] = v.x; out[2 * i + 1] = v.y;
  }
}
template <int N>
__device__ __forceinline__ void store_vec(float* p, const float* in) {
#pragma unroll
  for (int i = 0; i < N / 4; ++i)
    reinterpret_cast<float4*>(p)[i] = make_float4(in[4 * i], in[4 * i + 1], in[4 * i + 2], in[4 * i + 3]);
}
template <int N>
__device__ __forceinline__ void store_vec(double* p, const double* in) {
#pragma unroll
  for (int i = 0; i < N / 2; ++i)
    reinterpret_cast<double2*>(p)[i] = make_double2(in[2 * i], in[2 * i + 1]);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Deterministic block sum of one double per thread (blockDim multiple of 32,
// at most 1024).  Result valid in thread 0.
__device__ double block_sum(double v, double* smem) {
  v = warp_sum(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) smem[w] = v;
  __syncthreads();
  double r = 0;
  if (w == 0) {
    int nw = blockDim.x >> 5;
    r = (l < nw) ? smem[l] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

__device__ double block_max(double v, double* smem) {
  v = warp_max(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) smem[w] = v;
  __syncthreads();
  double r = 0;
  if (w == 0) {
    int nw = blockDim.x >> 5;
    r = (l < nw) ? smem[l] : 0.0;
    r = warp_max(r);
  }
  __syncthreads();
  return r;
}

// Huber rho and IRLS weight of a squared whitened residual s (Ceres'
// HuberLoss semantics, restated from camera_shared_ceres_optimizor.hpp:253).
__device__ __forceinline__ void loss_eval(int loss, double delta, double s, double& rho, double& w) {
  if (loss == GBA_LOSS_HUBER && s > delta * delta) {
    double r = sqrt(s);
    rho = 2.0 * delta * r - delta * delta;
    w = delta / r;
  } else {
    rho = s;
    w = 1.0;
  }
}

// Rodrigues coefficients of an angle-axis vector.  Near theta = 0 the
// reference formulas divide by zero (analytical_jacobian_matrix_calculator.hpp
// :359-380); series of sin and cos are used below theta = 1e-2.
//   s  = sin(t)/t, c = (1 - cos t)/t^2,
//   a1 = (t cos t - sin t)/t^3, a2 = (t sin t - 2(1 - cos t))/t^4.
__device__ void rodrigues_coeffs(double theta, double& ct, double& s, double& c, double& a1,
                                 double& a2) {
  double t2 = theta * theta;
  if (theta < 1e-2) {
    double t4 = t2 * t2;
    ct = 1.0 - t2 / 2.0 + t4 / 24.0;
    s = 1.0 - t2 / 6.0 + t4 / 120.0;
    c = 0.5 - t2 / 24.0 + t4 / 720.0;
    a1 = -1.0 / 3.0 + t2 / 30.0 - t4 / 840.0;
    a2 = -1.0 / 12.0 + t2 / 180.0 - t4 / 6720.0;
  } else {
    double st;
    sincos(theta, &st, &ct);
    s = st / theta;
    c = (1.0 - ct) / t2;
    a1 = (theta * ct - st) / (t2 * theta);
    a2 = (theta * st - 2.0 * (1.0 - ct)) / (t2 * t2);
  }
}

// ---------------------------------------------------------------------------
// Device projection in FP64 (camera_shared_vector_function.hpp:634-744 with
// radial_distortor.hpp:14-28, decentering_distortor.hpp:14-24).  The camera
// is the full 10-parameter model [k1 k2 k3 d1 d2 f s cx cy a]; groups absent
// from the intrinsic mask hold the identity values (0 / f=1 s=0 c=0 a=1),
// which reproduce the reference's per-mask projection exactly.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void project64(const double* R, const double* X, const double* cam,
                                          double& u, double& v) {
  double y0 = R[0] * X[0] + R[1] * X[1] + R[2] * X[2] + R[9];
  double y1 = R[3] * X[0] + R[4] * X[1] + R[5] * X[2] + R[10];
  double y2 = R[6] * X[0] + R[7] * X[1] + R[8] * X[2] + R[11];
  double n0 = y0 / y2, n1 = y1 / y2;
  double r2 = n0 * n0 + n1 * n1;
  double coeff = cam[0] * r2 + cam[1] * (r2 * r2) + cam[2] * (r2 * r2 * r2);
  double dx = coeff * n0 + (2.0 * cam[3] * n0 * n1 + cam[4] * (r2 + 2.0 * n0 * n0));
  double dy = coeff * n1 + (2.0 * cam[4] * n0 * n1 + cam[3] * (r2 + 2.0 * n1 * n1));
  n0 += dx;
  n1 += dy;
  u = cam[5] * n0 + cam[6] * n1 + cam[7];
  v = cam[5] * cam[9] * n1 + cam[8];
}

// Analytical Jacobian of one key in precision T: jp 2x3, ji 2x6 (row-major).
// IL = [r0 r1 r2 t0 t1 t2 ct s c a1 a2 pad] of the image.  Follows
// WorldPointToNormalizedPointDerivation (:334-429), RadialDistortDerivation
// (:431-470), DecenteringDistortDerivation (:472-503) and the intrinsic
// chains (:505-524).
template <typename T>
__device__ __forceinline__ void key_jacobian(const T* X, const T* IL, const T* cam, T* jp, T* ji) {
  const T r0 = IL[0], r1 = IL[1], r2 = IL[2];
  const T ct = IL[6], s = IL[7], c = IL[8], a1 = IL[9], a2 = IL[10];
  const T d = r0 * X[0] + r1 * X[1] + r2 * X[2];
  const T v0 = r1 * X[2] - r2 * X[1], v1 = r2 * X[0] - r0 * X[2], v2 = r0 * X[1] - r1 * X[0];
  const T y0 = ct * X[0] + s * v0 + c * d * r0 + IL[3];
  const T y1 = ct * X[1] + s * v1 + c * d * r1 + IL[4];
  const T y2 = ct * X[2] + s * v2 + c * d * r2 + IL[5];
  // pypr = w r^T + s [pvpr] + c (d I + r X^T),  w = -s X + a1 v + a2 d r
  const T w0 = -s * X[0] + a1 * v0 + a2 * d * r0;
  const T w1 = -s * X[1] + a1 * v1 + a2 * d * r1;
  const T w2 = -s * X[2] + a1 * v2 + a2 * d * r2;
  T pr[3][3];
  pr[0][0] = w0 * r0 + c * (d + r0 * X[0]);
  pr[0][1] = w0 * r1 + s * X[2] + c * r0 * X[1];
  pr[0][2] = w0 * r2 - s * X[1] + c * r0 * X[2];
  pr[1][0] = w1 * r0 - s * X[2] + c * r1 * X[0];
  pr[1][1] = w1 * r1 + c * (d + r1 * X[1]);
  pr[1][2] = w1 * r2 + s * X[0] + c * r1 * X[2];
  pr[2][0] = w2 * r0 + s * X[1] + c * r2 * X[0];
  pr[2][1] = w2 * r1 - s * X[0] + c * r2 * X[1];
  pr[2][2] = w2 * r2 + c * (d + r2 * X[2]);
  // pypp = ct I + s [r]x + c r r^T
  T pp[3][3];
  pp[0][0] = ct + c * r0 * r0; pp[0][1] = -s * r2 + c * r0 * r1; pp[0][2] = s * r1 + c * r0 * r2;
  pp[1][0] = s * r2 + c * r1 * r0; pp[1][1] = ct + c * r1 * r1; pp[1][2] = -s * r0 + c * r1 * r2;
  pp[2][0] = -s * r1 + c * r2 * r0; pp[2][1] = s * r0 + c * r2 * r1; pp[2][2] = ct + c * r2 * r2;
  const T iz = T(1) / y2;
  const T n0 = y0 * iz, n1 = y1 * iz;
  // normalized-key derivatives A (2 x 9): columns 0..2 point, 3..8 image
  T A0[9], A1[9];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    A0[m] = (pp[0][m] - n0 * pp[2][m]) * iz;
    A1[m] = (pp[1][m] - n1 * pp[2][m]) * iz;
    A0[3 + m] = (pr[0][m] - n0 * pr[2][m]) * iz;
    A1[3 + m] = (pr[1][m] - n1 * pr[2][m]) * iz;
  }
  A0[6] = iz; A0[7] = T(0); A0[8] = -n0 * iz;
  A1[6] = T(0); A1[7] = iz; A1[8] = -n1 * iz;
  // distortion chains (both from the undistorted key and A)
  const T rr2 = n0 * n0 + n1 * n1, rr4 = rr2 * rr2;
  const T coeff = cam[0] * rr2 + cam[1] * rr4 + cam[2] * rr4 * rr2;
  const T dcoef = cam[0] + T(2) * cam[1] * rr2 + T(3) * cam[2] * rr4;
  const T d1 = cam[3], d2 = cam[4];
  const T f = cam[5], sk = cam[6], fa = cam[5] * cam[9];
  T out0[9], out1[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    const T pr2 = T(2) * (n0 * A0[j] + n1 * A1[j]);
    const T cd = dcoef * pr2;
    const T cross = A0[j] * n1 + A1[j] * n0;
    const T e0 = A0[j] + (cd * n0 + coeff * A0[j]) +
                 (T(2) * d1 * cross + d2 * (pr2 + T(4) * n0 * A0[j]));
    const T e1 = A1[j] + (cd * n1 + coeff * A1[j]) +
                 (T(2) * d2 * cross + d1 * (pr2 + T(4) * n1 * A1[j]));
    out0[j] = f * e0 + sk * e1;
    out1[j] = fa * e1;
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) { jp[m] = out0[m]; jp[3 + m] = out1[m]; }
#pragma unroll
  for (int m = 0; m < 6; ++m) { ji[m] = out0[3 + m]; ji[6 + m] = out1[3 + m]; }
}

template <typename T>
__device__ __forceinline__ const T* tptr(const void* p) { return static_cast<const T*>(p); }
template <typename T>
__device__ __forceinline__ T* tptr_mut(void* p) { return static_cast<T*>(p); }

template <typename T>
__device__ __forceinline__ void load_cam(const DevPlan& d, int cam, T* out);
template <>
__device__ __forceinline__ void load_cam<float>(const DevPlan& d, int cam, float* out) {
#pragma unroll
  for (int j = 0; j < 10; ++j) out[j] = __ldg(d.cam32 + 10 * cam + j);
}
template <>
__device__ __forceinline__ void load_cam<double>(const DevPlan& d, int cam, double* out) {
#pragma unroll
  for (int j = 0; j < 10; ++j) out[j] = __ldg(d.cam64 + 10 * cam + j);
}

// ---------------------------------------------------------------------------
// init / copy x0
// ---------------------------------------------------------------------------
__global__ void k_init(DevPlan d) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < d.B) {
    LMState st = {};
    st.nu = 2.0;
    st.active = 1;
    st.relin = 1;
    st.first = 1;
    st.factor_ok = 1;
    st.stop = GBA_STOP_MAX_ITERATIONS;
    st.status = GBA_OK;
    d.state[p] = st;
    d.factor_flag[p] = 0;
  }
}

__global__ void k_copy_x0(DevPlan d) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long np = 3LL * d.P, ni = 6LL * d.I;
  if (i < np) d.x_pt[0][i] = d.x0_pt[i];
  else if (i < np + ni) d.x_img[0][i - np] = d.x0_img[i - np];
}

// ---------------------------------------------------------------------------
// image prep: which = 0 current x (at init), 1 candidate x (when evaluating)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_image_prep(DevPlan d, int which) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.I) return;
  const LMState& st = d.state[d.img_prob[i]];
  if (which == 0 ? !st.active : !st.evaluate) return;
  int par = which ? 1 - st.parity : st.parity;
  const double* x = d.x_img[par] + 6LL * i;
  double r0 = x[0], r1 = x[1], r2 = x[2];
  double theta = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
  double ct, s, c, a1, a2;
  rodrigues_coeffs(theta, ct, s, c, a1, a2);
  double* R = d.img_rot[par] + 12LL * i;
  if (theta == 0.0) {  // :695-698 -- camera point = X + t
    R[0] = 1; R[1] = 0; R[2] = 0; R[3] = 0; R[4] = 1; R[5] = 0; R[6] = 0; R[7] = 0; R[8] = 1;
  } else {
    // R = cos I + sin [k]x + (1 - cos) k k^T, k = r / theta
    double st_ = s * theta, omc = c * theta * theta;
    double k0 = r0 / theta, k1 = r1 / theta, k2 = r2 / theta;
    R[0] = ct + omc * k0 * k0; R[1] = -st_ * k2 + omc * k0 * k1; R[2] = st_ * k1 + omc * k0 * k2;
    R[3] = st_ * k2 + omc * k1 * k0; R[4] = ct + omc * k1 * k1; R[5] = -st_ * k0 + omc * k1 * k2;
    R[6] = -st_ * k1 + omc * k2 * k0; R[7] = st_ * k0 + omc * k2 * k1; R[8] = ct + omc * k2 * k2;
  }
  R[9] = x[3]; R[10] = x[4]; R[11] = x[5];
  T* IL = tptr_mut<T>(d.img_lin[par]) + 12LL * i;
  IL[0] = T(r0); IL[1] = T(r1); IL[2] = T(r2);
  IL[3] = T(x[3]); IL[4] = T(x[4]); IL[5] = T(x[5]);
  IL[6] = T(ct); IL[7] = T(s); IL[8] = T(c); IL[9] = T(a1); IL[10] = T(a2); IL[11] = T(0);
}

// ---------------------------------------------------------------------------
// cost: FP64 residual per key, whitened and weighted residual stored in T
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_cost(DevPlan d, int which) {
  __shared__ double red[32];
  const Chunk ch = d.key_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (which == 0 ? !st.active : !st.evaluate) return;
  const int par = which ? 1 - st.parity : st.parity;
  const double* __restrict__ xp = d.x_pt[par];
  const double* __restrict__ rot = d.img_rot[par];
  T* __restrict__ rw = tptr_mut<T>(d.RW[par]);
  double acc = 0.0;
  for (int k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    const int img = __ldg(d.key_img + k), pt = __ldg(d.key_pt + k);
    double R[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) R[j] = rot[12LL * img + j];
    double X[3] = {xp[3LL * pt], xp[3LL * pt + 1], xp[3LL * pt + 2]};
    double cam[10];
    const int ci = __ldg(d.img_cam + img);
#pragma unroll
    for (int j = 0; j < 10; ++j) cam[j] = __ldg(d.cam64 + 10 * ci + j);
    double u, v;
    project64(R, X, cam, u, v);
    const double2 ob = __ldg(d.key_obs + k);
    double e0 = u - ob.x, e1 = v - ob.y;   // r = f(x) - y
    if (d.key_wl) {
      const double l00 = __ldg(d.key_wl + 3LL * k), l10 = __ldg(d.key_wl + 3LL * k + 1),
                   l11 = __ldg(d.key_wl + 3LL * k + 2);
      double w0 = l00 * e0 + l10 * e1;
      e1 = l11 * e1;
      e0 = w0;
    }
    const double sq = e0 * e0 + e1 * e1;
    double rho, w;
    loss_eval(d.loss, d.huber_delta, sq, rho, w);
    acc += rho;
    const double sw = sqrt(w);
    T out[4] = {T(e0 * sw), T(e1 * sw), T(sw), T(0)};
    store_vec<4>(rw + 4LL * k, out);
  }
  double tot = block_sum(acc, red);
  if (threadIdx.x == 0) d.key_chunk_sum[blockIdx.x] = tot;
}

// ---------------------------------------------------------------------------
// linearize: per point (thread), its keys' Jacobians, V_p, g_p
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPointChunk) k_linearize(DevPlan d) {
  __shared__ double red[32];
  const Chunk ch = d.pt_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.relin || !st.active) return;
  const int par = st.parity;
  const int pt = ch.begin + threadIdx.x;
  double vmax = 0.0, gmax = 0.0;
  if (pt < ch.end) {
    const double* xp = d.x_pt[par] + 3LL * pt;
    const T X[3] = {T(xp[0]), T(xp[1]), T(xp[2])};
    const T* __restrict__ IL = tptr<T>(d.img_lin[par]);
    const T* __restrict__ rwb = tptr<T>(d.RW[par]);
    T* __restrict__ JR = tptr_mut<T>(d.JR);
    T V[6] = {0, 0, 0, 0, 0, 0}, g[3] = {0, 0, 0};
    const int kb = __ldg(d.pt_key_off + pt), ke = __ldg(d.pt_key_off + pt + 1);
    for (int k = kb; k < ke; ++k) {
      const int img = __ldg(d.key_img + k);
      T il[12];
      load_vec<12>(IL + 12LL * img, il);
      T cam[10];
      load_cam<T>(d, __ldg(d.img_cam + img), cam);
      T jp[6], ji[12];
      key_jacobian<T>(X, il, cam, jp, ji);
      T rw[4];
      load_vec<4>(rwb + 4LL * k, rw);
      const T sw = rw[2];
      if (d.key_wl) {
        const T l00 = T(__ldg(d.key_wl + 3LL * k)), l10 = T(__ldg(d.key_wl + 3LL * k + 1)),
                l11 = T(__ldg(d.key_wl + 3LL * k + 2));
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          T a = jp[m], b = jp[3 + m];
          jp[m] = (l00 * a + l10 * b) * sw;
          jp[3 + m] = l11 * b * sw;
        }
#pragma unroll
        for (int m = 0; m < 6; ++m) {
          T a = ji[m], b = ji[6 + m];
          ji[m] = (l00 * a + l10 * b) * sw;
          ji[6 + m] = l11 * b * sw;
        }
      } else {
#pragma unroll
        for (int m = 0; m < 6; ++m) jp[m] *= sw;
#pragma unroll
        for (int m = 0; m < 12; ++m) ji[m] *= sw;
      }
      T rec[kJRStride];
#pragma unroll
      for (int m = 0; m < 6; ++m) rec[m] = jp[m];
#pragma unroll
      for (int m = 0; m < 12; ++m) rec[6 + m] = ji[m];
      rec[18] = rw[0];
      rec[19] = rw[1];
      store_vec<kJRStride>(JR + (long long)kJRStride * k, rec);
      // V += Jp^T Jp (upper: 00 01 02 11 12 22), g += Jp^T r
      V[0] += jp[0] * jp[0] + jp[3] * jp[3];
      V[1] += jp[0] * jp[1] + jp[3] * jp[4];
      V[2] += jp[0] * jp[2] + jp[3] * jp[5];
      V[3] += jp[1] * jp[1] + jp[4] * jp[4];
      V[4] += jp[1] * jp[2] + jp[4] * jp[5];
      V[5] += jp[2] * jp[2] + jp[5] * jp[5];
      g[0] += jp[0] * rw[0] + jp[3] * rw[1];
      g[1] += jp[1] * rw[0] + jp[4] * rw[1];
      g[2] += jp[2] * rw[0] + jp[5] * rw[1];
    }
    T pv[12] = {V[0], V[1], V[2], V[3], V[4], V[5], g[0], g[1], g[2], T(0), T(0), T(0)};
    store_vec<12>(tptr_mut<T>(d.PV) + 12LL * pt, pv);
    vmax = fmax(fmax(double(V[0]), double(V[3])), double(V[5]));
    gmax = fmax(fmax(fabs(double(g[0])), fabs(double(g[1]))), fabs(double(g[2])));
  }
  double bv = block_max(vmax, red);
  double bg = block_max(gmax, red);
  if (threadIdx.x == 0) {
    LMState* sp = d.state + ch.prob;
    atomicMax(&sp->maxdiag_bits, dbits(bv));
    atomicMax(&sp->ginf_bits, dbits(bg));
  }
}

// ---------------------------------------------------------------------------
// image reduce: per image (warp), U_i and g_i with Kahan lane sums
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(32 * kImageChunk) k_image_reduce(DevPlan d) {
  const Chunk ch = d.img_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.relin || !st.active) return;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int img = ch.begin + w;
  if (img >= ch.end) return;
  const T* __restrict__ JR = tptr<T>(d.JR);
  T acc[27], cmp[27];
#pragma unroll
  for (int e = 0; e < 27; ++e) { acc[e] = T(0); cmp[e] = T(0); }
  const int qb = __ldg(d.img_key_off + img), qe = __ldg(d.img_key_off + img + 1);
  for (int q = qb + lane; q < qe; q += 32) {
    const int k = __ldg(d.img_keys + q);
    T rec[kJRStride];
    load_vec<kJRStride>(JR + (long long)kJRStride * k, rec);
    const T* ji = rec + 6;
    int e = 0;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
#pragma unroll
      for (int b = a; b < 6; ++b) {
        T term = ji[a] * ji[b] + ji[6 + a] * ji[6 + b];
        T y = term - cmp[e];
        T t = acc[e] + y;
        cmp[e] = (t - acc[e]) - y;
        acc[e] = t;
        ++e;
      }
    }
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      T term = ji[a] * rec[18] + ji[6 + a] * rec[19];
      T y = term - cmp[21 + a];
      T t = acc[21 + a] + y;
      cmp[21 + a] = (t - acc[21 + a]) - y;
      acc[21 + a] = t;
    }
  }
  double tot[27];
#pragma unroll
  for (int e = 0; e < 27; ++e) tot[e] = warp_sum(double(acc[e]) - double(cmp[e]));
  double* U = d.U + 36LL * img;
  int e = 0;
  double dmax = 0.0, gmax = 0.0;
#pragma unroll
  for (int a = 0; a < 6; ++a) {
#pragma unroll
    for (int b = a; b < 6; ++b) {
      if (lane == (e & 31)) { U[6 * a + b] = tot[e]; U[6 * b + a] = tot[e]; }
      if (a == b) dmax = fmax(dmax, tot[e]);
      ++e;
    }
  }
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    if (lane == a) d.gi[6LL * img + a] = tot[21 + a];
    gmax = fmax(gmax, fabs(tot[21 + a]));
  }
  if (lane == 0) {
    LMState* sp = d.state + ch.prob;
    atomicMax(&sp->maxdiag_bits, dbits(dmax));
    atomicMax(&sp->ginf_bits, dbits(gmax));
  }
}

// ---------------------------------------------------------------------------
// point Schur: C C^T = V + mu I, Z = C^-1 J_p^T J_i per key, h = C^-1 g
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPointChunk) k_point_schur(DevPlan d) {
  const Chunk ch = d.pt_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.active) return;
  const int pt = ch.begin + threadIdx.x;
  if (pt >= ch.end) return;
  const T mu = T(st.mu);
  T pv[12];
  load_vec<12>(tptr<T>(d.PV) + 12LL * pt, pv);
  // Cholesky of the damped 3x3 block (upper-stored V: 00 01 02 11 12 22)
  T a00 = pv[0] + mu, a01 = pv[1], a02 = pv[2], a11 = pv[3] + mu, a12 = pv[4], a22 = pv[5] + mu;
  bool ok = a00 > T(0);
  T c00 = sqrt(a00);
  T i00 = T(1) / c00;
  T c10 = a01 * i00, c20 = a02 * i00;
  T s11 = a11 - c10 * c10;
  ok = ok && s11 > T(0);
  T c11 = sqrt(s11);
  T i11 = T(1) / c11;
  T c21 = (a12 - c20 * c10) * i11;
  T s22 = a22 - c20 * c20 - c21 * c21;
  ok = ok && s22 > T(0);
  T c22 = sqrt(s22);
  T i22 = T(1) / c22;
  if (!ok) {
    atomicExch(d.factor_flag + ch.prob, 1);
    return;
  }
  // C^-1 (lower): rows [i00 0 0; m10 i11 0; m20 m21 i22]
  const T m10 = -c10 * i00 * i11;
  const T m21 = -c21 * i11 * i22;
  const T m20 = -(c20 * i00 + c21 * m10) * i22;
  const T g0 = pv[6], g1 = pv[7], g2 = pv[8];
  T ps[12] = {i00, m10, i11, m20, m21, i22,
              i00 * g0, m10 * g0 + i11 * g1, m20 * g0 + m21 * g1 + i22 * g2, T(0), T(0), T(0)};
  store_vec<12>(tptr_mut<T>(d.PS) + 12LL * pt, ps);
  const T* __restrict__ JR = tptr<T>(d.JR);
  T* __restrict__ Z = tptr_mut<T>(d.Z);
  const int kb = __ldg(d.pt_key_off + pt), ke = __ldg(d.pt_key_off + pt + 1);
  for (int k = kb; k < ke; ++k) {
    T rec[kJRStride];
    load_vec<kJRStride>(JR + (long long)kJRStride * k, rec);
    const T* jp = rec;
    const T* ji = rec + 6;
    T z[kZStride];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      // W[m][c] = jp[m] ji[c] + jp[3+m] ji[6+c]
      T w0 = jp[0] * ji[c] + jp[3] * ji[6 + c];
      T w1 = jp[1] * ji[c] + jp[4] * ji[6 + c];
      T w2 = jp[2] * ji[c] + jp[5] * ji[6 + c];
      z[c] = i00 * w0;
      z[6 + c] = m10 * w0 + i11 * w1;
      z[12 + c] = m20 * w0 + m21 * w1 + i22 * w2;
    }
    z[18] = T(0);
    z[19] = T(0);
    store_vec<kZStride>(Z + (long long)kZStride * k, z);
  }
}

// ---------------------------------------------------------------------------
// Schur assembly, one warp per work item (<= kPairItem pairs of one block)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_assemble_items(DevPlan d, int n_items) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= n_items) return;
  const int4 it = __ldg(d.items + wid);
  if (!d.state[it.w].active) return;
  const int2 ij = __ldg(d.blk_ij + it.x);
  const bool diag = ij.x == ij.y;
  const T* __restrict__ Z = tptr<T>(d.Z);
  const T* __restrict__ PS = tptr<T>(d.PS);
  T acc[36], racc[6];
#pragma unroll
  for (int e = 0; e < 36; ++e) acc[e] = T(0);
#pragma unroll
  for (int e = 0; e < 6; ++e) racc[e] = T(0);
  for (int q = it.y + lane; q < it.z; q += 32) {
    const int2 pr = __ldg(d.pairs + q);
    T za[kZStride], zb[kZStride];
    load_vec<kZStride>(Z + (long long)kZStride * pr.x, za);
    if (diag) {
#pragma unroll
      for (int e = 0; e < kZStride; ++e) zb[e] = za[e];
      T ps[12];
      load_vec<12>(PS + 12LL * __ldg(d.key_pt + pr.x), ps);
#pragma unroll
      for (int r = 0; r < 6; ++r) racc[r] += za[r] * ps[6] + za[6 + r] * ps[7] + za[12 + r] * ps[8];
    } else {
      load_vec<kZStride>(Z + (long long)kZStride * pr.y, zb);
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
#pragma unroll
      for (int c = 0; c < 6; ++c)
        acc[6 * r + c] += za[r] * zb[c] + za[6 + r] * zb[6 + c] + za[12 + r] * zb[12 + c];
    }
  }
  double* out = d.item_partial + (long long)kItemStride * wid;
#pragma unroll
  for (int e = 0; e < 36; ++e) {
    double v = warp_sum(double(acc[e]));
    if (lane == (e & 31)) out[e] = v;
  }
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    double v = warp_sum(double(racc[e]));
    if (lane == ((36 + e) & 31)) out[36 + e] = v;
  }
}

// Dense reduced system (lower triangle) and rhs, FP64.
__global__ void __launch_bounds__(256) k_assemble_S(DevPlan d) {
  const int p = blockIdx.y;
  const ProbInfo pi = d.prob[p];
  const LMState& st = d.state[p];
  if (!st.active) return;
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int n = pi.n;
  if (idx >= (long long)n * n) return;
  const int row = int(idx / n), col = int(idx % n);
  if (col > row) return;
  const int i = row / 6, a = row % 6, j = col / 6, bcol = col % 6;
  const int I = pi.num_images;
  const int blk = __ldg(d.blk_map + d.blk_map_off[p] + (long long)j * I + i);
  double v = 0.0, rv = 0.0;
  if (blk >= 0) {
    const int ib = __ldg(d.blk_item_off + blk), ie = __ldg(d.blk_item_off + blk + 1);
    for (int t = ib; t < ie; ++t) {
      v += d.item_partial[(long long)kItemStride * t + 6 * bcol + a];
    }
  }
  const int gi_img = pi.image_begin + i;
  double s;
  if (i == j) {
    s = d.U[36LL * gi_img + 6 * a + bcol] - v;
    if (a == bcol) s += st.mu;
  } else {
    s = -v;
  }
  d.S[pi.s_off + (long long)row * n + col] = s;
  if (col == 0) {
    // rhs b_i[a] = g_i[a] - sum over the diagonal block's items
    const int dblk = __ldg(d.blk_map + d.blk_map_off[p] + (long long)i * I + i);
    rv = 0.0;
    if (dblk >= 0) {
      const int ib = __ldg(d.blk_item_off + dblk), ie = __ldg(d.blk_item_off + dblk + 1);
      for (int t = ib; t < ie; ++t) rv += d.item_partial[(long long)kItemStride * t + 36 + a];
    }
    d.b[6LL * gi_img + a] = d.gi[6LL * gi_img + a] - rv;
  }
}

// ---------------------------------------------------------------------------
// Tiled FP64 Cholesky (lower), forward solve folded in, backward solve.
// ---------------------------------------------------------------------------
struct TileView {
  double* S;
  int n;
};

__device__ __forceinline__ int tile_rows(int n, int t) { return min(kTile, n - kTile * t); }

// Factor the diagonal tile k held in smem a[kTile][kTile+1] (m x m lower),
// write L back, its inverse to Linv, the forward solution y_k = L^-1 b_k,
// and for the last tile the first backward step delta = L^-T y.
__device__ void diag_factor(DevPlan& d, int p, const ProbInfo& pi, int k,
                            double (*a)[kTile + 1], double (*inv)[kTile + 1], int* fail) {
  const int n = pi.n, m = tile_rows(n, k);
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int j = 0; j < m; ++j) {
    if (tid == 0) {
      double dj = a[j][j];
      if (!(dj > 0.0) || !isfinite(dj)) *fail = 1;
      a[j][j] = sqrt(fmax(dj, 0.0));
    }
    __syncthreads();
    if (*fail) break;
    const double djj = a[j][j];
    for (int i = j + 1 + tid; i < m; i += nth) a[i][j] /= djj;
    __syncthreads();
    const int rem = m - j - 1;
    for (int e = tid; e < rem * rem; e += nth) {
      int i = j + 1 + e / rem, l = j + 1 + e % rem;
      if (l <= i) a[i][l] -= a[i][j] * a[l][j];
    }
    __syncthreads();
  }
  if (*fail) {
    if (tid == 0) d.factor_flag[p] = 1;
    return;
  }
  double* S = d.S + pi.s_off;
  const int r0 = kTile * k;
  for (int e = tid; e < m * m; e += nth) {
    int i = e / m, l = e % m;
    if (l <= i) S[(long long)(r0 + i) * n + r0 + l] = a[i][l];
  }
  // inverse of the lower-triangular tile, one column per thread
  for (int c = tid; c < kTile; c += nth) {
    for (int r = 0; r < kTile; ++r) inv[r][c] = 0.0;
    if (c < m) {
      for (int r = c; r < m; ++r) {
        double s = (r == c) ? 1.0 : 0.0;
        for (int q = c; q < r; ++q) s -= a[r][q] * inv[q][c];
        inv[r][c] = s / a[r][r];
      }
    }
  }
  __syncthreads();
  double* Li = d.Linv + ((long long)p * d.max_nt + k) * kTile * kTile;
  for (int e = tid; e < kTile * kTile; e += nth) Li[e] = inv[e / kTile][e % kTile];
  // forward solve y_k = L_kk^-1 b_k (b_k already has the panel updates)
  __shared__ double yk[kTile];
  double* bk = d.b + 6LL * pi.image_begin + r0;
  if (tid < m) {
    double s = 0.0;
    for (int q = 0; q <= tid; ++q) s += inv[tid][q] * bk[q];
    yk[tid] = s;
  }
  __syncthreads();
  if (k == pi.nt - 1) {
    // first backward step: delta_k = L_kk^-T y_k
    if (tid < m) {
      double s = 0.0;
      for (int q = tid; q < m; ++q) s += inv[q][tid] * yk[q];
      bk[tid] = s;
    }
  } else if (tid < m) {
    bk[tid] = yk[tid];
  }
  __syncthreads();
}

__device__ __forceinline__ void load_tile_sym(const double* S, int n, int r0, int m,
                                              double (*a)[kTile + 1]) {
  for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
    int i = e / kTile, l = e % kTile;
    double v = 0.0;
    if (i < m && l < m) {
      int gi = r0 + i, gl = r0 + l;
      v = (l <= i) ? S[(long long)gi * n + gl] : S[(long long)gl * n + gi];
    }
    a[i][l] = v;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_chol_diag0(DevPlan d) {
  __shared__ double a[kTile][kTile + 1];
  __shared__ double inv[kTile][kTile + 1];
  __shared__ int fail;
  const int p = blockIdx.x;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;
  const ProbInfo pi = d.prob[p];
  if (pi.nt <= 0) return;
  if (threadIdx.x == 0) fail = 0;
  load_tile_sym(d.S + pi.s_off, pi.n, 0, tile_rows(pi.n, 0), a);
  diag_factor(d, p, pi, 0, a, inv, &fail);
}

// L_ik = A_ik L_kk^-T for tiles i > k, and b_i -= L_ik y_k.
__global__ void __launch_bounds__(256) k_chol_panel(DevPlan d, int k) {
  __shared__ double A[kTile][kTile + 1];
  __shared__ double Li[kTile][kTile + 1];
  __shared__ double L[kTile][kTile + 1];
  __shared__ double yk[kTile];
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;
  const ProbInfo pi = d.prob[p];
  const int i = k + 1 + blockIdx.x;
  if (i >= pi.nt) return;
  const int n = pi.n, mi = tile_rows(n, i), m = tile_rows(n, k);
  const double* S = d.S + pi.s_off;
  const double* Lg = d.Linv + ((long long)p * d.max_nt + k) * kTile * kTile;
  for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
    int r = e / kTile, c = e % kTile;
    A[r][c] = (r < mi && c < m) ? S[(long long)(kTile * i + r) * n + kTile * k + c] : 0.0;
    Li[r][c] = Lg[e];
  }
  double* b = d.b + 6LL * pi.image_begin;
  if (threadIdx.x < kTile) yk[threadIdx.x] = threadIdx.x < m ? b[kTile * k + threadIdx.x] : 0.0;
  __syncthreads();
  for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
    int r = e / kTile, c = e % kTile;
    double s = 0.0;
    for (int q = 0; q <= c; ++q) s += A[r][q] * Li[c][q];
    L[r][c] = s;
  }
  __syncthreads();
  double* Sw = d.S + pi.s_off;
  for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
    int r = e / kTile, c = e % kTile;
    if (r < mi && c < m) Sw[(long long)(kTile * i + r) * n + kTile * k + c] = L[r][c];
  }
  if (threadIdx.x < mi) {
    double s = 0.0;
    for (int c = 0; c < m; ++c) s += L[threadIdx.x][c] * yk[c];
    b[kTile * i + threadIdx.x] -= s;
  }
}

// Trailing update A_ij -= L_ik L_jk^T for k < j <= i; the CTA owning tile
// (k+1, k+1) then factors it.
__global__ void __launch_bounds__(256) k_chol_update(DevPlan d, int k) {
  __shared__ double Lik[kTile][kTile + 1];
  __shared__ double Ljk[kTile][kTile + 1];
  __shared__ double inv[kTile][kTile + 1];
  __shared__ int fail;
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;
  const ProbInfo pi = d.prob[p];
  const int T = pi.nt - k - 1;   // trailing tiles of this problem (may be <= 0)
  const int lin = blockIdx.x;
  if (T <= 0 || lin >= T * (T + 1) / 2) return;
  // decode lin -> (ti, tj), tj <= ti
  int ti = int((sqrt(8.0 * lin + 1.0) - 1.0) * 0.5);
  while ((ti + 1) * (ti + 2) / 2 <= lin) ++ti;
  while (ti * (ti + 1) / 2 > lin) --ti;
  const int tj = lin - ti * (ti + 1) / 2;
  const int i = k + 1 + ti, j = k + 1 + tj;
  const int n = pi.n, mi = tile_rows(n, i), mj = tile_rows(n, j), m = tile_rows(n, k);
  double* S = d.S + pi.s_off;
  for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
    int r = e / kTile, c = e % kTile;
    Lik[r][c] = (r < mi && c < m) ? S[(long long)(kTile * i + r) * n + kTile * k + c] : 0.0;
    Ljk[r][c] = (r < mj && c < m) ? S[(long long)(kTile * j + r) * n + kTile * k + c] : 0.0;
  }
  __syncthreads();
  const bool diag = (i == j);
  for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
    int r = e / kTile, c = e % kTile;
    if (r < mi && c < mj && (!diag || c <= r)) {
      double s = 0.0;
#pragma unroll 8
      for (int q = 0; q < kTile; ++q) s += Lik[r][q] * Ljk[c][q];
      long long off = (long long)(kTile * i + r) * n + kTile * j + c;
      double v = S[off] - s;
      S[off] = v;
      if (diag && i == k + 1) inv[r][c] = v;  // stash for the fused factorization
    }
  }
  if (diag && i == k + 1) {
    __syncthreads();
    // mirror the lower part into a full symmetric tile
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
      int r = e / kTile, c = e % kTile;
      if (r < mi && c < mi) {
        if (c <= r) Lik[r][c] = inv[r][c];
      } else {
        Lik[r][c] = 0.0;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
      int r = e / kTile, c = e % kTile;
      if (r < mi && c < mi && c > r) Lik[r][c] = Lik[c][r];
    }
    if (threadIdx.x == 0) fail = 0;
    __syncthreads();
    diag_factor(d, p, pi, k + 1, Lik, inv, &fail);
  }
}

// Backward solve step k (k >= 1): y_j -= L_kj^T delta_k for j < k; the CTA
// for j = k-1 then computes delta_{k-1} = L_{k-1,k-1}^-T y_{k-1}.
__global__ void __launch_bounds__(128) k_chol_backward(DevPlan d, int k) {
  __shared__ double dk[kTile];
  __shared__ double yj[kTile];
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;
  const ProbInfo pi = d.prob[p];
  if (k >= pi.nt) return;
  const int j = blockIdx.x;
  if (j >= k) return;
  const int n = pi.n, m = tile_rows(n, k);
  const double* S = d.S + pi.s_off;
  double* b = d.b + 6LL * pi.image_begin;
  if (threadIdx.x < kTile) dk[threadIdx.x] = threadIdx.x < m ? b[kTile * k + threadIdx.x] : 0.0;
  __syncthreads();
  if (threadIdx.x < kTile) {
    const int c = threadIdx.x;
    double s = 0.0;
    for (int r = 0; r < m; ++r) s += S[(long long)(kTile * k + r) * n + kTile * j + c] * dk[r];
    double y = b[kTile * j + c] - s;
    yj[c] = y;
    if (j != k - 1) b[kTile * j + c] = y;
  }
  if (j == k - 1) {
    __syncthreads();
    const double* Li = d.Linv + ((long long)p * d.max_nt + j) * kTile * kTile;
    if (threadIdx.x < kTile) {
      const int c = threadIdx.x;
      double s = 0.0;
      for (int q = c; q < kTile; ++q) s += Li[q * kTile + c] * yj[q];
      b[kTile * j + c] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// back-substitution and update
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPointChunk) k_backsub(DevPlan d) {
  __shared__ double red[32];
  if (blockIdx.x < d.n_pt_chunks) {
    const Chunk ch = d.pt_chunks[blockIdx.x];
    const LMState& st = d.state[ch.prob];
    if (!st.active || d.factor_flag[ch.prob]) return;
    const int par = st.parity;
    const int pt = ch.begin + threadIdx.x;
    double dn2 = 0.0, xn2 = 0.0, gd = 0.0;
    if (pt < ch.end) {
      T ps[12];
      load_vec<12>(tptr<T>(d.PS) + 12LL * pt, ps);
      T t0 = ps[6], t1 = ps[7], t2 = ps[8];
      const T* __restrict__ Z = tptr<T>(d.Z);
      const int kb = __ldg(d.pt_key_off + pt), ke = __ldg(d.pt_key_off + pt + 1);
      for (int k = kb; k < ke; ++k) {
        T z[kZStride];
        load_vec<kZStride>(Z + (long long)kZStride * k, z);
        const double* di = d.b + 6LL * __ldg(d.key_img + k);
        T dl[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) dl[c] = T(di[c]);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          t0 -= z[c] * dl[c];
          t1 -= z[6 + c] * dl[c];
          t2 -= z[12 + c] * dl[c];
        }
      }
      // delta = C^-T t, C^-1 rows [i00 0 0; m10 i11 0; m20 m21 i22]
      const T i00 = ps[0], m10 = ps[1], i11 = ps[2], m20 = ps[3], m21 = ps[4], i22 = ps[5];
      const double dp[3] = {double(i00 * t0 + m10 * t1 + m20 * t2), double(i11 * t1 + m21 * t2),
                            double(i22 * t2)};
      T pv[12];
      load_vec<12>(tptr<T>(d.PV) + 12LL * pt, pv);
      const double* x = d.x_pt[par] + 3LL * pt;
      double* xn = d.x_pt[1 - par] + 3LL * pt;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        xn[a] = x[a] - dp[a];
        dn2 += dp[a] * dp[a];
        xn2 += x[a] * x[a];
        gd += double(pv[6 + a]) * dp[a];
      }
    }
    double s0 = block_sum(dn2, red), s1 = block_sum(xn2, red), s2 = block_sum(gd, red);
    if (threadIdx.x == 0) {
      d.pt_chunk_sum[3LL * blockIdx.x] = s0;
      d.pt_chunk_sum[3LL * blockIdx.x + 1] = s1;
      d.pt_chunk_sum[3LL * blockIdx.x + 2] = s2;
    }
  } else {
    const int c = blockIdx.x - d.n_pt_chunks;
    const Chunk ch = d.img_chunks[c];
    const LMState& st = d.state[ch.prob];
    if (!st.active || d.factor_flag[ch.prob]) return;
    const int par = st.parity;
    double dn2 = 0.0, xn2 = 0.0, gd = 0.0;
    const long long e0 = 6LL * ch.begin, e1 = 6LL * ch.end;
    for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      double dv = d.b[e], xv = d.x_img[par][e];
      d.x_img[1 - par][e] = xv - dv;
      dn2 += dv * dv;
      xn2 += xv * xv;
      gd += d.gi[e] * dv;
    }
    double s0 = block_sum(dn2, red), s1 = block_sum(xn2, red), s2 = block_sum(gd, red);
    if (threadIdx.x == 0) {
      d.img_chunk_sum[3LL * c] = s0;
      d.img_chunk_sum[3LL * c + 1] = s1;
      d.img_chunk_sum[3LL * c + 2] = s2;
    }
  }
}

// ---------------------------------------------------------------------------
// LM control (one warp per problem)
// ---------------------------------------------------------------------------
__device__ double prob_sum(const double* v, int stride, int off, const int* chunk_off, int p,
                           int lane) {
  double s = 0.0;
  for (int c = chunk_off[p] + lane; c < chunk_off[p + 1]; c += 32) s += v[(long long)stride * c + off];
  return warp_sum(s);
}

__global__ void k_ctrl_initial_cost(DevPlan d) {
  const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= d.B) return;
  LMState& st = d.state[p];
  if (!st.active) return;
  double F = prob_sum(d.key_chunk_sum, 1, 0, d.prob_key_chunk_off, p, lane);
  if (lane == 0) {
    st.F = F;
    st.initial_cost = F;
    if (!isfinite(F)) {
      st.status = GBA_ERR_NAN;
      st.stop = GBA_STOP_ERROR;
      st.active = 0;
    }
  }
}

__global__ void k_ctrl_after_linearize(DevPlan d) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= d.B) return;
  LMState& st = d.state[p];
  if (st.relin && st.active) {
    const double ginf = bitsd(st.ginf_bits);
    if (st.first) {
      st.mu = d.tau * bitsd(st.maxdiag_bits);
      st.first = 0;
    }
    if (ginf <= d.eps1) {
      st.active = 0;
      st.stop = GBA_STOP_SMALL_GRADIENT;
    }
  }
  st.relin = 0;
  if (st.active && st.iter >= d.max_iterations) {
    st.active = 0;
    st.stop = GBA_STOP_MAX_ITERATIONS;
  }
  d.factor_flag[p] = 0;
}

__global__ void k_ctrl_step(DevPlan d) {
  const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= d.B) return;
  LMState& st = d.state[p];
  if (!st.active) return;
  const bool failed = d.factor_flag[p] != 0;
  double dn2 = 0, xn2 = 0, gd = 0;
  if (!failed) {
    dn2 = prob_sum(d.pt_chunk_sum, 3, 0, d.prob_pt_chunk_off, p, lane) +
          prob_sum(d.img_chunk_sum, 3, 0, d.prob_img_chunk_off, p, lane);
    xn2 = prob_sum(d.pt_chunk_sum, 3, 1, d.prob_pt_chunk_off, p, lane) +
          prob_sum(d.img_chunk_sum, 3, 1, d.prob_img_chunk_off, p, lane);
    gd = prob_sum(d.pt_chunk_sum, 3, 2, d.prob_pt_chunk_off, p, lane) +
         prob_sum(d.img_chunk_sum, 3, 2, d.prob_img_chunk_off, p, lane);
  }
  if (lane != 0) return;
  st.iter += 1;
  st.evaluate = 0;
  if (failed) {
    st.factor_fail += 1;
    st.rejected += 1;
    st.mu *= st.nu;
    st.nu *= 2.0;
  } else {
    st.dn2 = dn2;
    st.xn2 = xn2;
    st.gd = gd;
    if (sqrt(dn2) <= d.eps2 * (sqrt(xn2) + d.eps2)) {
      st.active = 0;
      st.stop = GBA_STOP_SMALL_STEP;
    } else {
      st.evaluate = 1;
    }
  }
}

__global__ void k_ctrl_accept(DevPlan d) {
  const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= d.B) return;
  LMState& st = d.state[p];
  if (!st.evaluate) return;
  const double Fn = prob_sum(d.key_chunk_sum, 1, 0, d.prob_key_chunk_off, p, lane);
  if (lane != 0) return;
  st.evaluate = 0;
  st.F_new = Fn;
  const double denom = st.mu * st.dn2 + st.gd;
  const double rho = (st.F - Fn) / denom;
  if (isfinite(Fn) && rho > 0.0) {
    st.parity ^= 1;
    st.F = Fn;
    st.relin = 1;
    const double t = 2.0 * rho - 1.0;
    st.mu *= fmax(1.0 / 3.0, 1.0 - t * t * t);
    st.nu = 2.0;
    st.accepted += 1;
    st.ginf_bits = 0ull;
    st.maxdiag_bits = 0ull;
  } else {
    st.mu *= st.nu;
    st.nu *= 2.0;
    st.rejected += 1;
  }
}

// ---------------------------------------------------------------------------
// stage outputs for parity checks
// ---------------------------------------------------------------------------
__global__ void k_vector_function(DevPlan d, double* y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const int img = d.key_img[k], pt = d.key_pt[k];
  const int par = d.state[d.img_prob[img]].parity;
  double R[12];
  for (int j = 0; j < 12; ++j) R[j] = d.img_rot[par][12LL * img + j];
  const double* xp = d.x_pt[par] + 3LL * pt;
  double X[3] = {xp[0], xp[1], xp[2]};
  double cam[10];
  for (int j = 0; j < 10; ++j) cam[j] = d.cam64[10 * d.img_cam[img] + j];
  double u, v;
  project64(R, X, cam, u, v);
  y[2LL * k] = u;
  y[2LL * k + 1] = v;
}

template <typename T>
__global__ void k_jacobian_out(DevPlan d, double* jp_out, double* ji_out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const int img = d.key_img[k], pt = d.key_pt[k];
  const int par = d.state[d.img_prob[img]].parity;
  const double* xp = d.x_pt[par] + 3LL * pt;
  const T X[3] = {T(xp[0]), T(xp[1]), T(xp[2])};
  T il[12];
  for (int j = 0; j < 12; ++j) il[j] = tptr<T>(d.img_lin[par])[12LL * img + j];
  T cam[10];
  load_cam<T>(d, d.img_cam[img], cam);
  T jp[6], ji[12];
  key_jacobian<T>(X, il, cam, jp, ji);
  for (int j = 0; j < 6; ++j) jp_out[6LL * k + j] = double(jp[j]);
  for (int j = 0; j < 12; ++j) ji_out[12LL * k + j] = double(ji[j]);
}

template <typename T>
void run_image_prep(const DevPlan& d, int which, cudaStream_t s) {
  if (d.I > 0) k_image_prep<T><<<(d.I + 127) / 128, 128, 0, s>>>(d, which);
}

}  // namespace

// ===========================================================================
// launchers
// ===========================================================================
#define GBA_DISPATCH(d, KERNEL_CALL)                       \
  do {                                                     \
    if ((d).precision == GBA_PRECISION_MIXED) {            \
      using T = float;                                     \
      KERNEL_CALL;                                         \
    } else {                                               \
      using T = double;                                    \
      KERNEL_CALL;                                         \
    }                                                      \
  } while (0)

int launch_init(const DevPlan& d, cudaStream_t s) {
  k_init<<<(d.B + 127) / 128, 128, 0, s>>>(d);
  long long tot = 3LL * d.P + 6LL * d.I;
  if (tot > 0) {
    k_copy_x0<<<int((tot + 255) / 256), 256, 0, s>>>(d);
    return 2;
  }
  return 1;
}

int launch_image_prep(const DevPlan& d, int which, cudaStream_t s) {
  if (d.I <= 0) return 0;
  GBA_DISPATCH(d, run_image_prep<T>(d, which, s));
  return 1;
}

int launch_cost(const DevPlan& d, int which, cudaStream_t s) {
  if (d.n_key_chunks <= 0) return 0;
  GBA_DISPATCH(d, (k_cost<T><<<d.n_key_chunks, 256, 0, s>>>(d, which)));
  return 1;
}

int launch_ctrl_initial_cost(const DevPlan& d, cudaStream_t s) {
  k_ctrl_initial_cost<<<(d.B + 3) / 4, 128, 0, s>>>(d);
  return 1;
}

int launch_linearize(const DevPlan& d, cudaStream_t s) {
  if (d.n_pt_chunks <= 0) return 0;
  GBA_DISPATCH(d, (k_linearize<T><<<d.n_pt_chunks, kPointChunk, 0, s>>>(d)));
  return 1;
}

int launch_image_reduce(const DevPlan& d, cudaStream_t s) {
  if (d.n_img_chunks <= 0) return 0;
  GBA_DISPATCH(d, (k_image_reduce<T><<<d.n_img_chunks, 32 * kImageChunk, 0, s>>>(d)));
  return 1;
}

int launch_ctrl_after_linearize(const DevPlan& d, cudaStream_t s) {
  k_ctrl_after_linearize<<<(d.B + 127) / 128, 128, 0, s>>>(d);
  return 1;
}

int launch_point_schur(const DevPlan& d, cudaStream_t s) {
  if (d.n_pt_chunks <= 0) return 0;
  GBA_DISPATCH(d, (k_point_schur<T><<<d.n_pt_chunks, kPointChunk, 0, s>>>(d)));
  return 1;
}

int launch_assemble_items(const DevPlan& d, cudaStream_t s) {
  if (d.n_items <= 0) return 0;
  GBA_DISPATCH(d, (k_assemble_items<T><<<(d.n_items + 3) / 4, 128, 0, s>>>(d, d.n_items)));
  return 1;
}

int launch_assemble_S(const DevPlan& d, cudaStream_t s) {
  if (d.max_n <= 0) return 0;
  dim3 grid(unsigned((1LL * d.max_n * d.max_n + 255) / 256), unsigned(d.B));
  k_assemble_S<<<grid, 256, 0, s>>>(d);
  return 1;
}

int launch_assemble(const DevPlan& d, cudaStream_t s) {
  return launch_assemble_items(d, s) + launch_assemble_S(d, s);
}

int launch_cholesky(const DevPlan& d, cudaStream_t s) {
  if (d.max_nt <= 0) return 0;
  int n = 0;
  k_chol_diag0<<<d.B, 256, 0, s>>>(d);
  ++n;
  for (int k = 0; k + 1 < d.max_nt; ++k) {
    dim3 gp(unsigned(d.max_nt - 1 - k), unsigned(d.B));
    k_chol_panel<<<gp, 256, 0, s>>>(d, k);
    const int T = d.max_nt - k - 1;
    dim3 gu(unsigned(T * (T + 1) / 2), unsigned(d.B));
    k_chol_update<<<gu, 256, 0, s>>>(d, k);
    n += 2;
  }
  for (int k = d.max_nt - 1; k >= 1; --k) {
    dim3 gb(unsigned(k), unsigned(d.B));
    k_chol_backward<<<gb, 128, 0, s>>>(d, k);
    ++n;
  }
  return n;
}

int launch_backsub(const DevPlan& d, cudaStream_t s) {
  const int g = d.n_pt_chunks + d.n_img_chunks;
  if (g <= 0) return 0;
  GBA_DISPATCH(d, (k_backsub<T><<<g, kPointChunk, 0, s>>>(d)));
  return 1;
}

int launch_ctrl_step(const DevPlan& d, cudaStream_t s) {
  k_ctrl_step<<<(d.B + 3) / 4, 128, 0, s>>>(d);
  return 1;
}

int launch_ctrl_accept(const DevPlan& d, cudaStream_t s) {
  k_ctrl_accept<<<(d.B + 3) / 4, 128, 0, s>>>(d);
  return 1;
}

int launch_vector_function(const DevPlan& d, double* y, cudaStream_t s) {
  if (d.K <= 0) return 0;
  k_vector_function<<<(d.K + 255) / 256, 256, 0, s>>>(d, y);
  return 1;
}

int launch_jacobian_out(const DevPlan& d, double* jp, double* ji, cudaStream_t s) {
  if (d.K <= 0) return 0;
  GBA_DISPATCH(d, (k_jacobian_out<T><<<(d.K + 255) / 256, 256, 0, s>>>(d, jp, ji)));
  return 1;
}

}  // namespace gba
