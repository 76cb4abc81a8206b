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
  static_assert(N % 4 == 0 || N == 2, "float vectors of 4 (or one float2)");
  if constexpr (N == 2) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    out[0] = v.x;
    out[1] = v.y;
  } else {
#pragma unroll
    for (int i = 0; i < N / 4; ++i) {
      float4 v = __ldg(reinterpret_cast<const float4*>(p) + i);
      out[4 * i] = v.x; out[4 * i + 1] = v.y; out[4 * i + 2] = v.z; out[4 * i + 3] = v.w;
    }
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
template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
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

// ---------------------------------------------------------------------------
// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats (about 48 significant bits).  Error-free transformations: Knuth's
// two-sum, Dekker's fast two-sum, and the FMA-based exact product; the
// reciprocal is one Newton step from the float reciprocal.  Used by the
// mixed path to evaluate projections at FP64-class accuracy on the FP32
// pipes (the FP64 pipe of this part issues at 1/57 of the FP32 rate).
// ---------------------------------------------------------------------------
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ ff ff_add(ff x, ff y) {
  const ff s = ff_two_sum(x.hi, y.hi);
  return ff_fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
__device__ __forceinline__ ff ff_add_f(ff x, float y) {
  const ff s = ff_two_sum(x.hi, y);
  return ff_fast_two_sum(s.hi, s.lo + x.lo);
}
__device__ __forceinline__ ff ff_neg(ff x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ ff ff_mul(ff x, ff y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ ff ff_mul_f(ff x, float y) {
  const float p = x.hi * y;
  float e = fmaf(x.hi, y, -p);
  e = fmaf(x.lo, y, e);
  return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }
__device__ __forceinline__ ff ff_rcp(ff y) {
  const float r = 1.0f / y.hi;
  const ff e = ff_add_f(ff_neg(ff_mul_f(y, r)), 1.0f);   // 1 - y r
  return ff_add_f(ff_mul_f(e, r), r);                    // r + r (1 - y r)
}
__host__ __device__ __forceinline__ float2 ff_split(double d) {
  const float hi = float(d);
  return make_float2(hi, float(d - double(hi)));
}
__device__ __forceinline__ ff ff_ld(float2 v) { return {v.x, v.y}; }

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
  const double iz = 1.0 / y2;
  double n0 = y0 * iz, n1 = y1 * iz;
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
  if (i < np) {
    d.x_pt[0][i] = d.x0_pt[i];
    if (d.x_ff[0]) d.x_ff[0][i] = ff_split(d.x0_pt[i]);
  } else if (i < np + ni) {
    d.x_img[0][i - np] = d.x0_img[i - np];
  }
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
  if (d.img_rot_ff[par]) {
    float2* Rf = d.img_rot_ff[par] + 12LL * i;
#pragma unroll
    for (int j = 0; j < 12; ++j) Rf[j] = ff_split(R[j]);
  }
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
    const double sw = (w == 1.0) ? 1.0 : sqrt(w);
    T out[4] = {T(e0 * sw), T(e1 * sw), T(sw), T(0)};
    store_vec<4>(rw + 4LL * k, out);
  }
  double tot = block_sum(acc, red);
  if (threadIdx.x == 0) d.key_chunk_sum[blockIdx.x] = tot;
}

// Mixed-path cost: the projection in double-float from the double-float
// mirrors of x, R|t, the keys and the cameras; per-thread sums in
// double-float, block sums in FP64.
__global__ void __launch_bounds__(256) k_cost_ff(DevPlan d, int which) {
  __shared__ double red[32];
  const Chunk ch = d.key_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (which == 0 ? !st.active : !st.evaluate) return;
  const int par = which ? 1 - st.parity : st.parity;
  const float2* __restrict__ xp = d.x_ff[par];
  const float2* __restrict__ rot = d.img_rot_ff[par];
  float* __restrict__ rw = static_cast<float*>(d.RW[par]);
  ff acc = {0.0f, 0.0f};
  for (int k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    const int img = __ldg(d.key_img + k), pt = __ldg(d.key_pt + k);
    const float2* R = rot + 12LL * img;
    const ff X0 = ff_ld(xp[3LL * pt]), X1 = ff_ld(xp[3LL * pt + 1]), X2 = ff_ld(xp[3LL * pt + 2]);
    ff y[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      ff a = ff_ld(R[9 + m]);
      a = ff_fma(ff_ld(R[3 * m]), X0, a);
      a = ff_fma(ff_ld(R[3 * m + 1]), X1, a);
      y[m] = ff_fma(ff_ld(R[3 * m + 2]), X2, a);
    }
    const ff iz = ff_rcp(y[2]);
    ff n0 = ff_mul(y[0], iz), n1 = ff_mul(y[1], iz);
    const float2* cam = d.cam_ff + 10 * __ldg(d.img_cam + img);
    const ff k1 = ff_ld(cam[0]), k2 = ff_ld(cam[1]), k3 = ff_ld(cam[2]);
    const ff d1 = ff_ld(cam[3]), d2 = ff_ld(cam[4]);
    const ff r2 = ff_add(ff_mul(n0, n0), ff_mul(n1, n1));
    ff dx = {0.0f, 0.0f}, dy = {0.0f, 0.0f};
    if (k1.hi != 0.0f || k2.hi != 0.0f || k3.hi != 0.0f) {
      const ff coeff = ff_mul(r2, ff_fma(r2, ff_fma(r2, k3, k2), k1));
      dx = ff_mul(coeff, n0);
      dy = ff_mul(coeff, n1);
    }
    if (d1.hi != 0.0f || d2.hi != 0.0f) {
      const ff xy2 = ff_mul_f(ff_mul(n0, n1), 2.0f);
      dx = ff_add(dx, ff_add(ff_mul(d1, xy2), ff_mul(d2, ff_add(r2, ff_mul_f(ff_mul(n0, n0), 2.0f)))));
      dy = ff_add(dy, ff_add(ff_mul(d2, xy2), ff_mul(d1, ff_add(r2, ff_mul_f(ff_mul(n1, n1), 2.0f)))));
    }
    n0 = ff_add(n0, dx);
    n1 = ff_add(n1, dy);
    const ff f = ff_ld(cam[5]), sk = ff_ld(cam[6]), cx = ff_ld(cam[7]), cy = ff_ld(cam[8]);
    const ff fa = ff_ld(cam[9]);   // f * a, stored pre-multiplied
    const ff u = ff_add(ff_fma(f, n0, ff_mul(sk, n1)), cx);
    const ff v = ff_fma(fa, n1, cy);
    const float2 ob0 = d.key_obs_ff[2LL * k], ob1 = d.key_obs_ff[2LL * k + 1];
    ff e0f = ff_add(u, ff_neg(ff_ld(ob0))), e1f = ff_add(v, ff_neg(ff_ld(ob1)));   // r = f(x) - y
    if (d.key_wl) {   // whitened residual L^T r
      const ff l00 = ff_ld(ff_split(__ldg(d.key_wl + 3LL * k)));
      const ff l10 = ff_ld(ff_split(__ldg(d.key_wl + 3LL * k + 1)));
      const ff l11 = ff_ld(ff_split(__ldg(d.key_wl + 3LL * k + 2)));
      const ff w0 = ff_fma(l00, e0f, ff_mul(l10, e1f));
      e1f = ff_mul(l11, e1f);
      e0f = w0;
    }
    const ff sqf = ff_fma(e0f, e0f, ff_mul(e1f, e1f));
    const float e0 = e0f.hi + e0f.lo, e1 = e1f.hi + e1f.lo;
    float sw = 1.0f;
    const float hd = float(d.huber_delta);
    if (d.loss == GBA_LOSS_HUBER && sqf.hi > hd * hd) {
      const float r = sqrtf(sqf.hi);
      acc = ff_add_f(acc, 2.0f * hd * r - hd * hd);
      sw = sqrtf(hd / r);
    } else {
      acc = ff_add(acc, sqf);
    }
    float out[4] = {e0 * sw, e1 * sw, sw, 0.0f};
    store_vec<4>(rw + 4LL * k, out);
  }
  const double tot = block_sum(double(acc.hi) + double(acc.lo), red);
  if (threadIdx.x == 0) d.key_chunk_sum[blockIdx.x] = tot;
}

// ---------------------------------------------------------------------------
// linearize, one thread per key (coalesced JR records): the analytical
// Jacobian of the key, whitened by the key weight and the IRLS weight.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_linearize_keys(DevPlan d) {
  const Chunk ch = d.key_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.relin || !st.active) return;
  const int par = st.parity;
  const double* __restrict__ xp = d.x_pt[par];
  const T* __restrict__ IL = tptr<T>(d.img_lin[par]);
  const T* __restrict__ rwb = tptr<T>(d.RW[par]);
  T* __restrict__ JR = tptr_mut<T>(d.JR);
  for (int k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    const int img = __ldg(d.key_img + k), pt = __ldg(d.key_pt + k);
    T X[3];
    if (sizeof(T) == sizeof(float) && d.x_ff[par]) {   // mixed: high part of the mirror
      const float2* xf = d.x_ff[par] + 3LL * pt;
      X[0] = T(xf[0].x); X[1] = T(xf[1].x); X[2] = T(xf[2].x);
    } else {
      X[0] = T(xp[3LL * pt]); X[1] = T(xp[3LL * pt + 1]); X[2] = T(xp[3LL * pt + 2]);
    }
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
        const T a = jp[m], b = jp[3 + m];
        jp[m] = (l00 * a + l10 * b) * sw;
        jp[3 + m] = l11 * b * sw;
      }
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        const T a = ji[m], b = ji[6 + m];
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
  }
}

// Per point: V_p = sum J_p^T J_p, g_p = sum J_p^T r from its keys' records.
template <typename T>
__global__ void __launch_bounds__(kPointChunk) k_point_reduce(DevPlan d) {
  __shared__ double red[32];
  const Chunk ch = d.pt_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.relin || !st.active) return;
  const int pt = ch.begin + threadIdx.x;
  double vmax = 0.0, gmax = 0.0;
  if (pt < ch.end) {
    const T* __restrict__ JR = tptr<T>(d.JR);
    T V[6] = {0, 0, 0, 0, 0, 0}, g[3] = {0, 0, 0};
    const int kb = __ldg(d.pt_key_off + pt), ke = __ldg(d.pt_key_off + pt + 1);
    for (int k = kb; k < ke; ++k) {
      T jp[8], rr[2];
      load_vec<8>(JR + (long long)kJRStride * k, jp);
      load_vec<2>(JR + (long long)kJRStride * k + 18, rr);
      V[0] += jp[0] * jp[0] + jp[3] * jp[3];
      V[1] += jp[0] * jp[1] + jp[3] * jp[4];
      V[2] += jp[0] * jp[2] + jp[3] * jp[5];
      V[3] += jp[1] * jp[1] + jp[4] * jp[4];
      V[4] += jp[1] * jp[2] + jp[4] * jp[5];
      V[5] += jp[2] * jp[2] + jp[5] * jp[5];
      g[0] += jp[0] * rr[0] + jp[3] * rr[1];
      g[1] += jp[1] * rr[0] + jp[4] * rr[1];
      g[2] += jp[2] * rr[0] + jp[5] * rr[1];
    }
    T pv[12] = {V[0], V[1], V[2], V[3], V[4], V[5], g[0], g[1], g[2], T(0), T(0), T(0)};
    store_vec<12>(tptr_mut<T>(d.PV) + 12LL * pt, pv);
    vmax = fmax(fmax(double(V[0]), double(V[3])), double(V[5]));
    gmax = fmax(fmax(fabs(double(g[0])), fabs(double(g[1]))), fabs(double(g[2])));
  }
  const double bv = block_max(vmax, red);
  const double bg = block_max(gmax, red);
  if (threadIdx.x == 0) {
    LMState* sp = d.state + ch.prob;
    atomicMax(&sp->maxdiag_bits, dbits(bv));
    atomicMax(&sp->ginf_bits, dbits(bg));
  }
}

// ---------------------------------------------------------------------------
// image reduce: U_i = sum J_i^T J_i, g_i = sum J_i^T r.  Each image's keys
// are split into work items of <= kImageItem keys (one warp each, Kahan lane
// sums in T, warp sum in T); k_image_finalize adds an image's items in order
// in FP64.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_image_reduce(DevPlan d) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= d.n_img_items) return;
  const int4 it = __ldg(d.img_items + wid);   // (image, q begin, q end, prob)
  const LMState& st = d.state[it.w];
  if (!st.relin || !st.active) return;
  const T* __restrict__ JR = tptr<T>(d.JR);
  T acc[27], cmp[27];
#pragma unroll
  for (int e = 0; e < 27; ++e) { acc[e] = T(0); cmp[e] = T(0); }
  for (int q = it.y + lane; q < it.z; q += 32) {
    const int k = __ldg(d.img_keys + q);
    T rec[kJRStride];
    load_vec<kJRStride>(JR + (long long)kJRStride * k, rec);
    const T* ji = rec + 6;
    int e = 0;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
#pragma unroll
      for (int b = a; b < 6; ++b) {
        const T term = ji[a] * ji[b] + ji[6 + a] * ji[6 + b];
        const T y = term - cmp[e];
        const T t = acc[e] + y;
        cmp[e] = (t - acc[e]) - y;
        acc[e] = t;
        ++e;
      }
    }
#pragma unroll
    for (int a = 0; a < 6; ++a) {
      const T term = ji[a] * rec[18] + ji[6 + a] * rec[19];
      const T y = term - cmp[21 + a];
      const T t = acc[21 + a] + y;
      cmp[21 + a] = (t - acc[21 + a]) - y;
      acc[21 + a] = t;
    }
  }
  double* out = d.img_item_partial + 28LL * wid;
#pragma unroll
  for (int e = 0; e < 27; ++e) {
    const T v = warp_sum_t(T(acc[e] - cmp[e]));
    if (lane == e) out[e] = double(v);
  }
}

__global__ void __launch_bounds__(256) k_image_finalize(DevPlan d) {
  const int img = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (img >= d.I) return;
  const int prob = d.img_prob[img];
  const LMState& st = d.state[prob];
  if (!st.relin || !st.active) return;
  const int ib = d.img_item_off[img], ie = d.img_item_off[img + 1];
  double v = 0.0;
  if (lane < 27)
    for (int t = ib; t < ie; ++t) v += d.img_item_partial[28LL * t + lane];
  // lane e holds entry e of (upper U in row order, then g)
  double* U = d.U + 36LL * img;
  double dmax = 0.0, gmax = 0.0;
  if (lane < 21) {
    int a = 0, e = lane;
    while (e >= 6 - a) { e -= 6 - a; ++a; }
    const int b = a + e;
    U[6 * a + b] = v;
    U[6 * b + a] = v;
    if (a == b) dmax = v;
  } else if (lane < 27) {
    d.gi[6LL * img + (lane - 21)] = v;
    gmax = fabs(v);
  }
  dmax = warp_max(dmax);
  gmax = warp_max(gmax);
  if (lane == 0) {
    LMState* sp = d.state + prob;
    atomicMax(&sp->maxdiag_bits, dbits(dmax));
    atomicMax(&sp->ginf_bits, dbits(gmax));
  }
}

// ---------------------------------------------------------------------------
// point factor: C C^T = V_p + mu I, C^-1 and h_p = C^-1 g_p per point
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPointChunk) k_point_factor(DevPlan d) {
  const Chunk ch = d.pt_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.active) return;
  const int pt = ch.begin + threadIdx.x;
  if (pt >= ch.end) return;
  const T mu = T(st.mu);
  T pv[12];
  load_vec<12>(tptr<T>(d.PV) + 12LL * pt, pv);
  const T a00 = pv[0] + mu, a01 = pv[1], a02 = pv[2], a11 = pv[3] + mu, a12 = pv[4], a22 = pv[5] + mu;
  bool ok = a00 > T(0);
  const T c00 = sqrt(a00);
  const T i00 = T(1) / c00;
  const T c10 = a01 * i00, c20 = a02 * i00;
  const T s11 = a11 - c10 * c10;
  ok = ok && s11 > T(0);
  const T c11 = sqrt(s11);
  const T i11 = T(1) / c11;
  const T c21 = (a12 - c20 * c10) * i11;
  const T s22 = a22 - c20 * c20 - c21 * c21;
  ok = ok && s22 > T(0);
  const T c22 = sqrt(s22);
  const T i22 = T(1) / c22;
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
}

// Z_a = C_p^-1 J_p^T J_i per key (coalesced records).
template <typename T>
__global__ void __launch_bounds__(256) k_key_z(DevPlan d) {
  const Chunk ch = d.key_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.active) return;
  const T* __restrict__ JR = tptr<T>(d.JR);
  const T* __restrict__ PS = tptr<T>(d.PS);
  T* __restrict__ Z = tptr_mut<T>(d.Z);
  for (int k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    T rec[kJRStride], ps[8];
    load_vec<kJRStride>(JR + (long long)kJRStride * k, rec);
    load_vec<8>(PS + 12LL * __ldg(d.key_pt + k), ps);
    const T i00 = ps[0], m10 = ps[1], i11 = ps[2], m20 = ps[3], m21 = ps[4], i22 = ps[5];
    const T* jp = rec;
    const T* ji = rec + 6;
    T z[kZStride];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const T w0 = jp[0] * ji[c] + jp[3] * ji[6 + c];
      const T w1 = jp[1] * ji[c] + jp[4] * ji[6 + c];
      const T w2 = jp[2] * ji[c] + jp[5] * ji[6 + c];
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
  // the next pair's key indices are fetched one iteration ahead, so each
  // iteration waits on a single round trip (the Z records)
  int q = it.y + lane;
  int2 pr = q < it.z ? __ldg(d.pairs + q) : make_int2(0, 0);
  for (; q < it.z; q += 32) {
    const int qn = q + 32;
    const int2 prn = qn < it.z ? __ldg(d.pairs + qn) : pr;
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
    pr = prn;
  }
  // warp reduction in the working precision; each lane then converts only
  // the sums it stores (entries lane and lane + 32 of the 42)
  double* out = d.item_partial + (long long)kItemStride * wid;
  T mine0 = T(0), mine1 = T(0);
#pragma unroll
  for (int e = 0; e < 36; ++e) {
    const T v = warp_sum_t(acc[e]);
    if (lane == e) mine0 = v;
    if (lane + 32 == e) mine1 = v;
  }
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    const T v = warp_sum_t(racc[e]);
    if (lane == 36 + e) mine0 = v;
    if (lane + 32 == 36 + e) mine1 = v;
  }
  out[lane] = double(mine0);
  if (lane < 10) out[32 + lane] = double(mine1);
}

// Dense reduced system (lower triangle) and rhs in precision T; the block
// sums over work items are taken in FP64.
template <typename T>
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
  tptr_mut<T>(d.S)[pi.s_off + (long long)row * n + col] = T(s);
  if (col == 0) {
    // rhs b_i[a] = g_i[a] - sum over the diagonal block's items
    const int dblk = __ldg(d.blk_map + d.blk_map_off[p] + (long long)i * I + i);
    rv = 0.0;
    if (dblk >= 0) {
      const int ib = __ldg(d.blk_item_off + dblk), ie = __ldg(d.blk_item_off + dblk + 1);
      for (int t = ib; t < ie; ++t) rv += d.item_partial[(long long)kItemStride * t + 36 + a];
    }
    tptr_mut<T>(d.b)[6LL * gi_img + a] = T(d.gi[6LL * gi_img + a] - rv);
  }
}

// ---------------------------------------------------------------------------
// Tiled Cholesky of the reduced system S (lower, precision T), one launch per
// column step.  Launch k (k = -1 .. nt-2) subtracts column k's rank-32
// contribution from every trailing tile and factors column c = k+1: every
// CTA of column c recomputes the diagonal tile's factor and inverse itself
// (a 32x32 factorization held in one warp's registers), so no separate panel
// launch is needed; the CTA owning tile (c, c) publishes L_cc^-1 and the
// forward-solve value y_c = L_cc^-1 b_c.  S keeps its diagonal tiles (the
// factor lives in Linv), the off-diagonal tiles are overwritten by L.
// The backward solve L^T delta = y then takes one launch per tile row.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int tile_rows(int n, int t) { return min(kTile, n - kTile * t); }

template <typename T>
using Tile = T[kTile][kTile + 1];

// Tile loads for 256-thread CTAs: each thread fetches its 4 elements of a
// tile into registers first (all loads in flight together), then stores
// them to shared memory.  Rectangular tiles read 0 past the matrix; a
// diagonal tile keeps its stored lower triangle, reads 0 above it and has
// identity rows past the matrix.
constexpr int kCholThreads = 256;
constexpr int kPerThread = kTile * kTile / kCholThreads;

template <typename T>
struct TileFetch {
  T v[kPerThread];
  __device__ __forceinline__ void rect(const T* S, int n, int ti, int tj) {
    const int mi = tile_rows(n, ti), mj = tile_rows(n, tj);
#pragma unroll
    for (int u = 0; u < kPerThread; ++u) {
      const int e = threadIdx.x + u * kCholThreads, r = e / kTile, c = e % kTile;
      v[u] = (r < mi && c < mj) ? S[(long long)(kTile * ti + r) * n + kTile * tj + c] : T(0);
    }
  }
  __device__ __forceinline__ void diag(const T* S, int n, int ti) {
    const int m = tile_rows(n, ti);
#pragma unroll
    for (int u = 0; u < kPerThread; ++u) {
      const int e = threadIdx.x + u * kCholThreads, r = e / kTile, c = e % kTile;
      T x = T(0);
      if (r < m) {
        if (c <= r) x = S[(long long)(kTile * ti + r) * n + kTile * ti + c];
      } else if (r == c) {
        x = T(1);
      }
      v[u] = x;
    }
  }
  __device__ __forceinline__ void store(Tile<T>& t) const {
#pragma unroll
    for (int u = 0; u < kPerThread; ++u) {
      const int e = threadIdx.x + u * kCholThreads;
      t[e / kTile][e % kTile] = v[u];
    }
  }
};

// A -= X Y^T (32x32x32), 256 threads, 4 outputs each.
template <typename T>
__device__ __forceinline__ void tile_sub_xyt(Tile<T>& A, const Tile<T>& X, const Tile<T>& Y) {
  const int r = threadIdx.x >> 3, c0 = (threadIdx.x & 7) * 4;
  T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
#pragma unroll 8
  for (int q = 0; q < kTile; ++q) {
    const T x = X[r][q];
    s0 += x * Y[c0][q];
    s1 += x * Y[c0 + 1][q];
    s2 += x * Y[c0 + 2][q];
    s3 += x * Y[c0 + 3][q];
  }
  A[r][c0] -= s0;
  A[r][c0 + 1] -= s1;
  A[r][c0 + 2] -= s2;
  A[r][c0 + 3] -= s3;
}

// Factor the SPD tile D (lower triangle used; identity-padded) in one warp and
// write L^-1 to Dinv; D is overwritten by L.  Lane i keeps row i of the
// tile in registers; each factored column is broadcast through shared memory
// (col, double-buffered) and the reciprocal pivots are kept in rinv.  The
// inverse is formed one column per lane by forward substitution against L in
// shared memory, with the stored reciprocals (no divisions).  Returns false
// when a pivot was not positive.
template <typename T>
__device__ bool warp_potrf_inverse(Tile<T>& D, Tile<T>& Dinv, T* col, T* rinv, int lane) {
  constexpr unsigned FULL = 0xffffffffu;
  T a[kTile];
#pragma unroll
  for (int q = 0; q < kTile; ++q) a[q] = D[lane][q];
  bool ok = true;
#pragma unroll
  for (int j = 0; j < kTile; ++j) {
    const T djj = __shfl_sync(FULL, a[j], j);
    ok = ok && (djj > T(0));
    const T r = rsqrt(djj);
    const T ljj = djj * r;
    if (lane == j) rinv[j] = r;
    const T lij = (lane > j) ? a[j] * r : ((lane == j) ? ljj : T(0));
    a[j] = lij;
    T* cb = col + (j & 1) * kTile;
    cb[lane] = lij;
    __syncwarp();
#pragma unroll
    for (int l = j + 1; l < kTile; ++l) a[l] -= lij * cb[l];
  }
#pragma unroll
  for (int c = 0; c < kTile; ++c) D[lane][c] = (c <= lane) ? a[c] : T(0);
  __syncwarp();
  T x[kTile];
#pragma unroll
  for (int r = 0; r < kTile; ++r) x[r] = (r == lane) ? T(1) : T(0);
#pragma unroll
  for (int q = 0; q < kTile; ++q) {
    x[q] *= rinv[q];
#pragma unroll
    for (int r = q + 1; r < kTile; ++r) x[r] -= D[r][q] * x[q];
  }
#pragma unroll
  for (int r = 0; r < kTile; ++r) Dinv[r][lane] = x[r];
  return ok;
}

template <typename T>
__global__ void __launch_bounds__(256) k_chol_step(DevPlan d, int k) {
  __shared__ Tile<T> A, Li, Lj, D, Dinv;
  __shared__ T yk[kTile], tv[kTile];
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;
  const ProbInfo pi = d.prob[p];
  const int c = k + 1;
  const int Tn = pi.nt - c;           // tile rows c .. nt-1
  if (Tn <= 0) return;
  int i, j;
  if (k < 0) {                        // first launch: column 0 only
    if ((int)blockIdx.x >= Tn) return;
    i = blockIdx.x;
    j = 0;
  } else {
    const int lin = blockIdx.x;
    if (lin >= Tn * (Tn + 1) / 2) return;
    int ti = int((sqrtf(8.0f * float(lin) + 1.0f) - 1.0f) * 0.5f);
    while ((ti + 1) * (ti + 2) / 2 <= lin) ++ti;
    while (ti * (ti + 1) / 2 > lin) --ti;
    i = c + ti;
    j = c + (lin - ti * (ti + 1) / 2);
  }
  const int n = pi.n;
  T* S = tptr_mut<T>(d.S) + pi.s_off;
  T* b = tptr_mut<T>(d.b) + 6LL * pi.image_begin;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // own tile and, for k >= 0, the column-k factors: all loads issued first
  TileFetch<T> fa, fi, fj, fd;
  if (i == j) fa.diag(S, n, i); else fa.rect(S, n, i, j);
  if (k >= 0) {
    fi.rect(S, n, i, k);
    fj.rect(S, n, j, k);
  }
  const bool need_d = (j == c && i != c);
  if (need_d) fd.diag(S, n, c);
  T ykv = T(0), bv = T(0);
  if (k >= 0 && tid < kTile) ykv = b[kTile * k + tid];   // y_k (tile k is full)
  if (j == c && tid < kTile && tid < tile_rows(n, i)) bv = b[kTile * i + tid];
  fa.store(A);
  if (k >= 0) {
    fi.store(Li);
    fj.store(Lj);
    if (tid < kTile) yk[tid] = ykv;
  }
  if (need_d) fd.store(D);
  __syncthreads();
  if (k >= 0) {
    tile_sub_xyt<T>(A, Li, Lj);
    if (j == c && i != c) tile_sub_xyt<T>(D, Lj, Lj);
  }
  if (j == c && tid < kTile) {
    // b_i after column k: b_i - L_ik y_k
    T t = bv;
    if (k >= 0) {
#pragma unroll 8
      for (int q = 0; q < kTile; ++q) t -= Li[tid][q] * yk[q];
    }
    tv[tid] = t;
  }
  __syncthreads();
  if (j != c) {                       // trailing tile: write back
    const int mi = tile_rows(n, i), mj = tile_rows(n, j);
    for (int e = tid; e < kTile * kTile; e += blockDim.x) {
      const int r = e / kTile, q = e % kTile;
      if (r < mi && q < mj && (i != j || q <= r)) S[(long long)(kTile * i + r) * n + kTile * j + q] = A[r][q];
    }
    return;
  }
  // column c: factor the diagonal tile (own tile when i == c)
  __shared__ int ok_s;
  __shared__ T colbuf[2 * kTile], rinv[kTile];
  if (warp == 0) {
    const bool ok = warp_potrf_inverse<T>(i == c ? A : D, Dinv, colbuf, rinv, lane);
    if (lane == 0) ok_s = ok ? 1 : 0;
  }
  __syncthreads();
  if (!ok_s) {
    if (tid == 0) d.factor_flag[p] = 1;
    return;
  }
  const int mi = tile_rows(n, i);
  if (i == c) {
    T* Lg = tptr_mut<T>(d.Linv) + ((long long)p * d.max_nt + c) * kTile * kTile;
    for (int e = tid; e < kTile * kTile; e += blockDim.x) Lg[e] = Dinv[e / kTile][e % kTile];
    if (tid < kTile) {
      T y = T(0);
#pragma unroll 8
      for (int q = 0; q < kTile; ++q) y += Dinv[tid][q] * tv[q];
      yk[tid] = y;
    }
    __syncthreads();
    if (tid < mi) {
      if (c == pi.nt - 1) {           // last tile: first backward step
        T dl = T(0);
        for (int q = tid; q < kTile; ++q) dl += Dinv[q][tid] * yk[q];
        b[kTile * c + tid] = dl;
      } else {
        b[kTile * c + tid] = yk[tid];
      }
    }
    return;
  }
  // i > c: L_ic = A_ic L_cc^-T, and the column-k part of the forward solve
  if (tid < mi) b[kTile * i + tid] = tv[tid];
  {
    const int r = tid >> 3, c0 = (tid & 7) * 4;
    T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
#pragma unroll 8
    for (int q = 0; q < kTile; ++q) {
      const T x = A[r][q];
      s0 += x * Dinv[c0][q];
      s1 += x * Dinv[c0 + 1][q];
      s2 += x * Dinv[c0 + 2][q];
      s3 += x * Dinv[c0 + 3][q];
    }
    if (r < mi) {
      T* row = S + (long long)(kTile * i + r) * n + kTile * c;
      row[c0] = s0;
      row[c0 + 1] = s1;
      row[c0 + 2] = s2;
      row[c0 + 3] = s3;
    }
  }
}

// Backward solve step k (k >= 1): y_j -= L_kj^T delta_k for j < k; the CTA
// for j = k-1 then computes delta_{k-1} = L_{k-1,k-1}^-T y_{k-1}.
template <typename T>
__global__ void __launch_bounds__(256) k_chol_backward(DevPlan d, int k) {
  __shared__ Tile<T> L;
  __shared__ T dk[kTile], yj[kTile];
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;
  const ProbInfo pi = d.prob[p];
  if (k >= pi.nt) return;
  const int j = blockIdx.x;
  if (j >= k) return;
  const int n = pi.n, m = tile_rows(n, k);
  const T* S = tptr<T>(d.S) + pi.s_off;
  T* b = tptr_mut<T>(d.b) + 6LL * pi.image_begin;
  TileFetch<T> fl;
  fl.rect(S, n, k, j);
  T dv = T(0), yv = T(0);
  if (threadIdx.x < kTile) {
    dv = threadIdx.x < m ? b[kTile * k + threadIdx.x] : T(0);
    yv = b[kTile * j + threadIdx.x];
  }
  fl.store(L);
  if (threadIdx.x < kTile) dk[threadIdx.x] = dv;
  __syncthreads();
  if (threadIdx.x < kTile) {
    const int c = threadIdx.x;
    T s = T(0);
#pragma unroll 8
    for (int r = 0; r < kTile; ++r) s += L[r][c] * dk[r];
    const T y = yv - s;
    yj[c] = y;
    if (j != k - 1) b[kTile * j + c] = y;
  }
  if (j == k - 1) {
    __syncthreads();
    const T* Lv = tptr<T>(d.Linv) + ((long long)p * d.max_nt + j) * kTile * kTile;
    if (threadIdx.x < kTile) {
      const int c = threadIdx.x;
      T s = T(0);
      for (int q = c; q < kTile; ++q) s += Lv[q * kTile + c] * yj[q];
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
        const T* di = tptr<T>(d.b) + 6LL * __ldg(d.key_img + k);
        T dl[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) dl[c] = di[c];
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
      float2* xf = d.x_ff[1 - par] ? d.x_ff[1 - par] + 3LL * pt : nullptr;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        xn[a] = x[a] - dp[a];
        if (xf) xf[a] = ff_split(xn[a]);
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
      double dv = double(tptr<T>(d.b)[e]), xv = d.x_img[par][e];
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
int run_cholesky_factor(const DevPlan& d, cudaStream_t s) {
  int n = 0;
  k_chol_step<T><<<dim3(unsigned(d.max_nt), unsigned(d.B)), 256, 0, s>>>(d, -1);
  ++n;
  for (int k = 0; k + 1 < d.max_nt; ++k) {
    const int Tn = d.max_nt - k - 1;
    k_chol_step<T><<<dim3(unsigned(Tn * (Tn + 1) / 2), unsigned(d.B)), 256, 0, s>>>(d, k);
    ++n;
  }
  return n;
}

template <typename T>
int run_cholesky_solve(const DevPlan& d, cudaStream_t s) {
  int n = 0;
  for (int k = d.max_nt - 1; k >= 1; --k) {
    k_chol_backward<T><<<dim3(unsigned(k), unsigned(d.B)), 256, 0, s>>>(d, k);
    ++n;
  }
  return n;
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
  if (d.precision == GBA_PRECISION_MIXED)
    k_cost_ff<<<d.n_key_chunks, 256, 0, s>>>(d, which);
  else
    k_cost<double><<<d.n_key_chunks, 256, 0, s>>>(d, which);
  return 1;
}

int launch_ctrl_initial_cost(const DevPlan& d, cudaStream_t s) {
  k_ctrl_initial_cost<<<(d.B + 3) / 4, 128, 0, s>>>(d);
  return 1;
}

int launch_linearize(const DevPlan& d, cudaStream_t s) {
  int n = 0;
  if (d.n_key_chunks > 0) {
    GBA_DISPATCH(d, (k_linearize_keys<T><<<d.n_key_chunks, 256, 0, s>>>(d)));
    ++n;
  }
  if (d.n_pt_chunks > 0) {
    GBA_DISPATCH(d, (k_point_reduce<T><<<d.n_pt_chunks, kPointChunk, 0, s>>>(d)));
    ++n;
  }
  return n;
}

int launch_image_reduce(const DevPlan& d, cudaStream_t s) {
  if (d.n_img_items <= 0) return 0;
  GBA_DISPATCH(d, (k_image_reduce<T><<<(d.n_img_items + 7) / 8, 256, 0, s>>>(d)));
  k_image_finalize<<<(d.I + 7) / 8, 256, 0, s>>>(d);
  return 2;
}

int launch_ctrl_after_linearize(const DevPlan& d, cudaStream_t s) {
  k_ctrl_after_linearize<<<(d.B + 127) / 128, 128, 0, s>>>(d);
  return 1;
}

int launch_point_schur(const DevPlan& d, cudaStream_t s) {
  int n = 0;
  if (d.n_pt_chunks > 0) {
    GBA_DISPATCH(d, (k_point_factor<T><<<d.n_pt_chunks, kPointChunk, 0, s>>>(d)));
    ++n;
  }
  if (d.n_key_chunks > 0) {
    GBA_DISPATCH(d, (k_key_z<T><<<d.n_key_chunks, 256, 0, s>>>(d)));
    ++n;
  }
  return n;
}

int launch_assemble_items(const DevPlan& d, cudaStream_t s) {
  if (d.n_items <= 0) return 0;
  GBA_DISPATCH(d, (k_assemble_items<T><<<(d.n_items + 3) / 4, 128, 0, s>>>(d, d.n_items)));
  return 1;
}

int launch_assemble_S(const DevPlan& d, cudaStream_t s) {
  if (d.max_n <= 0) return 0;
  dim3 grid(unsigned((1LL * d.max_n * d.max_n + 255) / 256), unsigned(d.B));
  GBA_DISPATCH(d, (k_assemble_S<T><<<grid, 256, 0, s>>>(d)));
  return 1;
}

int launch_assemble(const DevPlan& d, cudaStream_t s) {
  return launch_assemble_items(d, s) + launch_assemble_S(d, s);
}

int launch_cholesky_factor(const DevPlan& d, cudaStream_t s) {
  if (d.max_nt <= 0) return 0;
  int n = 0;
  GBA_DISPATCH(d, n = run_cholesky_factor<T>(d, s));
  return n;
}

int launch_cholesky_solve(const DevPlan& d, cudaStream_t s) {
  if (d.max_nt <= 0) return 0;
  int n = 0;
  GBA_DISPATCH(d, n = run_cholesky_solve<T>(d, s));
  return n;
}

int launch_cholesky(const DevPlan& d, cudaStream_t s) {
  return launch_cholesky_factor(d, s) + launch_cholesky_solve(d, s);
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
