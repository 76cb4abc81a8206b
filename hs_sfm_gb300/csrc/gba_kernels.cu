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
//   k_assemble_S     dense reduced system S and rhs b (T), block sums in FP64
//   k_chol_*         tiled Cholesky (T) with the forward solve folded in,
//                    then the backward solve (normal_equation_solver.hpp:448-466)
//   k_backsub        delta_p = C^-T (h_p - sum Z_a delta_i), x_new = x - delta,
//                    and the candidate's image rotations
//                    (normal_equation_solver.hpp:468-538)
//   k_ctrl_*         the LM decisions per problem on the device (Madsen,
//                    Nielsen & Tingleff 2004, Alg. 3.16 as bound by
//                    camera_shared_nllso_meta_levenberg_marquardt.hpp:33-106)
//   free cameras:    k_cam_prep (camera arrays of x), J_c in k_linearize_keys,
//                    k_image_cam_reduce / k_image_cam_finalize / k_cam_finalize
//                    (E_i = J_i^T J_c, U_c, g_c), k_camrec_z (camera Z
//                    records), camera parts in k_assemble_S, k_cam_backsub
//                    (normal_equation_builder.hpp:157-205,309-349;
//                     normal_equation_solver.hpp:270-392,422-443)
//   PCG:             k_assemble_blocks, k_pcg_* (block-Jacobi PCG on the
//                    explicit 6x6 blocks of S)
#include "gba_internal.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstdio>

namespace gba {
namespace {

namespace cg = cooperative_groups;

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

// Z records (18 T each) at slot s: either records of kZStride T in slot
// order, or (DevPlan::z_planes) nine planes of T pairs, plane v holding the
// pair (z[2v], z[2v+1]) of every slot (plane stride z_n slots).
template <typename T> struct Pair2;
template <> struct Pair2<float> { using type = float2; };
template <> struct Pair2<double> { using type = double2; };

template <typename T>
__device__ __forceinline__ void load_z(const DevPlan& d, const T* __restrict__ Z, long long s, T* z) {
  if (d.z_planes) {
    const auto* zp = reinterpret_cast<const typename Pair2<T>::type*>(Z) + s;
#pragma unroll
    for (int v = 0; v < 9; ++v) {
      const auto t = __ldg(zp + v * d.z_n);
      z[2 * v] = t.x;
      z[2 * v + 1] = t.y;
    }
  } else {
    load_vec<kZStride>(Z + (long long)kZStride * s, z);
  }
}

template <typename T>
__device__ __forceinline__ void store_z(const DevPlan& d, T* Z, long long s, const T* z) {
  if (d.z_planes) {
    auto* zp = reinterpret_cast<typename Pair2<T>::type*>(Z) + s;
#pragma unroll
    for (int v = 0; v < 9; ++v) zp[v * d.z_n] = {z[2 * v], z[2 * v + 1]};
  } else {
    store_vec<kZStride>(Z + (long long)kZStride * s, z);
  }
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

// Arrival of this CTA at problem p's counter after thread 0 has written the
// CTA's partial sums; true in every thread of the CTA that arrives last of
// `total` (which then runs the problem's LM control step and resets the
// counter for the next launch).  The fence orders this CTA's partials
// before its arrival; the last CTA reads the others' through L2.
__device__ bool last_arrival(unsigned* counter, int total, int* flag_smem) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    const int last = prev == unsigned(total - 1);
    if (last) {
      atomicExch(counter, 0u);
      __threadfence();
    }
    *flag_smem = last;
  }
  __syncthreads();
  return *flag_smem != 0;
}

template <bool CG>
__device__ void ctrl_step_body(const DevPlan& d, int p, double* red);
template <bool CG>
__device__ void ctrl_accept_body(const DevPlan& d, int p, double* red);

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
__device__ __forceinline__ void key_jacobian(const T* X, const T* IL, const T* cam, T* jp, T* ji,
                                             T* nrm = nullptr) {
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
  if (nrm) {
    nrm[0] = n0;
    nrm[1] = n1;
  }
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
__device__ __forceinline__ void load_cam(const DevPlan& d, int par, int cam, T* out);
template <>
__device__ __forceinline__ void load_cam<float>(const DevPlan& d, int par, int cam, float* out) {
#pragma unroll
  for (int j = 0; j < 10; ++j) out[j] = d.cam32[par][10 * cam + j];
}
template <>
__device__ __forceinline__ void load_cam<double>(const DevPlan& d, int par, int cam, double* out) {
#pragma unroll
  for (int j = 0; j < 10; ++j) out[j] = d.cam64[par][10 * cam + j];
}

// Derivatives of the image key with respect to all ten camera parameters in
// the full model's order [k1 k2 k3][d1 d2][f s cx cy a]
// (camera_shared_analytical_jacobian_matrix_calculator.hpp:526-557), from the
// undistorted normalized key n: row 0 (u) in jc[0..9], row 1 (v) in
// jc[10..19].  Consumers pick the computed parameters' columns.
template <typename T>
__device__ __forceinline__ void camera_jacobian(T n0, T n1, const T* cam, T* jc) {
  const T r2 = n0 * n0 + n1 * n1, r4 = r2 * r2, r6 = r4 * r2;
  const T coeff = cam[0] * r2 + cam[1] * r4 + cam[2] * r6;
  const T d1 = cam[3], d2 = cam[4];
  const T e0 = n0 + coeff * n0 + (T(2) * d1 * n0 * n1 + d2 * (r2 + T(2) * n0 * n0));
  const T e1 = n1 + coeff * n1 + (T(2) * d2 * n0 * n1 + d1 * (r2 + T(2) * n1 * n1));
  const T f = cam[5], sk = cam[6], a = cam[9];
  // distortion columns through K: u = f e0 + s e1 + cx, v = f a e1 + cy
  const T de0[5] = {r2 * n0, r4 * n0, r6 * n0, T(2) * n0 * n1, r2 + T(2) * n0 * n0};
  const T de1[5] = {r2 * n1, r4 * n1, r6 * n1, r2 + T(2) * n1 * n1, T(2) * n0 * n1};
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    jc[m] = f * de0[m] + sk * de1[m];
    jc[10 + m] = f * a * de1[m];
  }
  jc[5] = e0;    jc[15] = a * e1;   // f
  jc[6] = e1;    jc[16] = T(0);     // s
  jc[7] = T(1);  jc[17] = T(0);     // cx
  jc[8] = T(0);  jc[18] = T(1);     // cy
  jc[9] = T(0);  jc[19] = f * e1;   // a
}

// Column of the full ten [k1 k2 k3 d1 d2 f s cx cy a] holding a camera's
// computed parameter m, or -1 past its count.
__host__ __device__ __forceinline__ int cam_full_col(unsigned mask, int m) {
  if (mask & GBA_COMPUTE_RADIAL_DISTORTION) {
    if (m < 3) return m;
    m -= 3;
  }
  if (mask & GBA_COMPUTE_DECENTERING_DISTORTION) {
    if (m < 2) return 3 + m;
    m -= 2;
  }
  if ((mask & GBA_COMPUTE_INTRINSIC_PARAMS) && m < 5) return 5 + m;
  return -1;
}

// The computed parameter held in full column j, or -1 when j is not computed.
__device__ __forceinline__ int cam_compact_col(unsigned mask, int j) {
  const int nr = (mask & GBA_COMPUTE_RADIAL_DISTORTION) ? 3 : 0;
  const int nd = (mask & GBA_COMPUTE_DECENTERING_DISTORTION) ? 2 : 0;
  if (j < 3) return nr ? j : -1;
  if (j < 5) return nd ? nr + j - 3 : -1;
  return (mask & GBA_COMPUTE_INTRINSIC_PARAMS) ? nr + nd + j - 5 : -1;
}

// Index of (a, b), a <= b, in the row-major upper triangle of a 10 x 10 block.
__device__ __forceinline__ int upper10(int a, int b) { return 10 * a - a * (a - 1) / 2 + (b - a); }


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
  long long np = 3LL * d.P, ni = 6LL * d.I, nc = d.free_cams ? 10LL * d.Ctot : 0;
  if (i < np) {
    d.x_pt[0][i] = d.x0_pt[i];
    if (d.x_ff[0]) d.x_ff[0][i] = ff_split(d.x0_pt[i]);
  } else if (i < np + ni) {
    d.x_img[0][i - np] = d.x0_img[i - np];
  } else if (i < np + ni + nc) {
    d.x_cam[0][i - np - ni] = d.x0_cam[i - np - ni];
  }
}

// Free cameras: the ten-parameter camera of x_cam (which = 0 current, 1
// candidate) in every form the key kernels read.  Fixed cameras keep the
// values uploaded at plan creation in both parities.
__global__ void k_cam_prep(DevPlan d, int which) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Ctot) return;
  const int4 ci = d.cam_info[c];
  if (ci.x == 0) return;
  const LMState& st = d.state[ci.z];
  if (which == 0 ? !st.active : !st.evaluate) return;
  const int par = which ? 1 - st.parity : st.parity;
  const double* x = d.x_cam[par] + 10LL * c;
  double full[10] = {0, 0, 0, 0, 0, 1, 0, 0, 0, 1};
#pragma unroll
  for (int j = 0; j < 10; ++j) {
    const int m = cam_compact_col(unsigned(ci.y), j);
    if (m >= 0) full[j] = x[m];
  }
#pragma unroll
  for (int j = 0; j < 10; ++j) {
    d.cam64[par][10LL * c + j] = full[j];
    d.cam32[par][10LL * c + j] = float(full[j]);
  }
  if (d.cam_ff[par]) {
#pragma unroll
    for (int j = 0; j < 9; ++j) d.cam_ff[par][10LL * c + j] = ff_split(full[j]);
    d.cam_ff[par][10LL * c + 9] = ff_split(full[5] * full[9]);   // f * a
  }
}

// ---------------------------------------------------------------------------
// image prep: which = 0 current x (at init), 1 candidate x (when evaluating)
// ---------------------------------------------------------------------------
// The rotation of image i's parameters in parity par in every form the key
// kernels read.
template <typename T>
__device__ void image_prep_one(const DevPlan& d, int i, int par) {
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

// which = 0: the current x of active problems (at init); 1: the candidate of
// problems whose step is evaluated.  The solve loop prepares the candidate in
// k_backsub instead; which = 1 is kept for callers that move x themselves.
template <typename T>
__global__ void k_image_prep(DevPlan d, int which) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.I) return;
  const LMState& st = d.state[d.img_prob[i]];
  if (which == 0 ? !st.active : !st.evaluate) return;
  image_prep_one<T>(d, i, which ? 1 - st.parity : st.parity);
}

// Soft-constraint and point-prior part of the cost, sum w (x - y)^2 and
// (x - y)^T L (x - y) (no loss), one CTA per problem over its rows
// (camera_shared_mahalanobis_distance_calculator.hpp:28-58).
__global__ void __launch_bounds__(256) k_cons_cost(DevPlan d, int which) {
  __shared__ double red[32];
  const int p = blockIdx.x;
  const LMState& st = d.state[p];
  if (which == 0 ? !st.active : !st.evaluate) return;
  const int par = which ? 1 - st.parity : st.parity;
  double acc = 0.0;
  if (d.n_cons > 0)
    for (int r = d.prob_cons_off[p] + threadIdx.x; r < d.prob_cons_off[p + 1]; r += blockDim.x) {
      const int4 c = d.cons[r];
      const double2 yw = d.cons_yw[r];
      const double x = c.x == 0   ? d.x_pt[par][3LL * c.y + c.z]
                       : c.x == 1 ? d.x_img[par][6LL * c.y + c.z]
                                  : d.x_cam[par][10LL * c.y + c.z];
      const double v = x - yw.x;
      acc += yw.y * v * v;
    }
  if (d.n_priors > 0)   // (x - y)^T L (x - y) per prior (ba_gcp_constrained_mahalanobis_distance_calculator.hpp:55-62)
    for (int i = d.prob_prior_off[p] + threadIdx.x; i < d.prob_prior_off[p + 1]; i += blockDim.x) {
      const double* xp = d.x_pt[par] + 3LL * d.prior_pt[i];
      const double* L = d.prior_info + 9LL * i;
      double v[3];
      for (int a = 0; a < 3; ++a) v[a] = xp[a] - d.prior_y[3LL * i + a];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) acc += v[a] * L[3 * a + b] * v[b];
    }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) d.cons_cost[p] = acc;
}

// ---------------------------------------------------------------------------
// cost: FP64 residual per key, whitened and weighted residual stored in T
// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// linearize, one thread per key (coalesced JR records): the analytical
// Jacobian of the key, whitened by the key weight and the IRLS weight, into
// the records of parity `par` (and the camera block with free cameras).
// X, il, cam are the point, the image's linearisation coefficients and the
// camera at that parity; rw0, rw1, sw the key's weighted residual and the
// square root of its IRLS weight.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void linearize_key(const DevPlan& d, int k, int par, int fix, const T* X, const T* il,
                                              const T* cam, T rw0, T rw1, T sw) {
  T jp[6], ji[12], nrm[2];
  key_jacobian<T>(X, il, cam, jp, ji, nrm);
  if (fix & 1) {   // fixed points: no point columns
#pragma unroll
    for (int m = 0; m < 6; ++m) jp[m] = T(0);
  }
  if (fix & 2) {   // fixed images: no image columns
#pragma unroll
    for (int m = 0; m < 12; ++m) ji[m] = T(0);
  }
  if (d.free_cams) {   // the camera block, whitened and weighted as the others
    T jc[20];
    camera_jacobian<T>(nrm[0], nrm[1], cam, jc);
    T l00 = T(1), l10 = T(0), l11 = T(1);
    if (d.key_wl) {
      l00 = T(__ldg(d.key_wl + 3LL * k));
      l10 = T(__ldg(d.key_wl + 3LL * k + 1));
      l11 = T(__ldg(d.key_wl + 3LL * k + 2));
    }
#pragma unroll
    for (int m = 0; m < 10; ++m) {
      const T a = jc[m], b = jc[10 + m];
      jc[m] = (l00 * a + l10 * b) * sw;
      jc[10 + m] = l11 * b * sw;
    }
    store_vec<20>(tptr_mut<T>(d.JC[par]) + 20LL * k, jc);
  }
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
  rec[18] = rw0;
  rec[19] = rw1;
  store_vec<kJRStride>(tptr_mut<T>(d.JR[par]) + (long long)kJRStride * k, rec);
}

// The records of a key chunk at parity par, one key per thread.
template <typename T>
__device__ __forceinline__ void linearize_chunk(const DevPlan& d, const Chunk& ch, int par) {
  const double* __restrict__ xp = d.x_pt[par];
  const T* __restrict__ IL = tptr<T>(d.img_lin[par]);
  const T* __restrict__ rwb = tptr<T>(d.RW[par]);
  const int fix = d.prob[ch.prob].fix;
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
    load_cam<T>(d, par, __ldg(d.img_cam + img), cam);
    T rw[4];
    load_vec<4>(rwb + 4LL * k, rw);
    linearize_key<T>(d, k, par, fix, X, il, cam, rw[0], rw[1], rw[2]);
  }
}

// The prologue's linearization (and, with DevPlan::fuse_lin off, every
// iteration's): the records at the problem's current parity.
template <typename T>
__global__ void __launch_bounds__(256) k_linearize_keys(DevPlan d) {
  const Chunk ch = d.key_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.relin || !st.active) return;
  linearize_chunk<T>(d, ch, st.parity);
}

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
  double acc = 0.0, acc_raw = 0.0;
  for (int k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    const int img = __ldg(d.key_img + k), pt = __ldg(d.key_pt + k);
    double R[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) R[j] = rot[12LL * img + j];
    double X[3] = {xp[3LL * pt], xp[3LL * pt + 1], xp[3LL * pt + 2]};
    double cam[10];
    const int ci = __ldg(d.img_cam + img);
#pragma unroll
    for (int j = 0; j < 10; ++j) cam[j] = d.cam64[par][10 * ci + j];
    double u, v;
    project64(R, X, cam, u, v);
    const double2 ob = __ldg(d.key_obs + k);
    double e0 = u - ob.x, e1 = v - ob.y;   // r = f(x) - y
    acc_raw += e0 * e0 + e1 * e1;
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
    if (which == 1 && d.fuse_lin) {   // the candidate's Jacobian records, used if it is accepted
      T Xl[3] = {T(X[0]), T(X[1]), T(X[2])}, il[12], cl[10];
      load_vec<12>(tptr<T>(d.img_lin[par]) + 12LL * img, il);
      load_cam<T>(d, par, ci, cl);
      linearize_key<T>(d, k, par, d.prob[ch.prob].fix, Xl, il, cl, out[0], out[1], out[2]);
    }
  }
  const double tot = block_sum(acc, red);
  const double tot_raw = block_sum(acc_raw, red);
  if (threadIdx.x == 0) {
    d.key_chunk_sum[2LL * blockIdx.x] = tot;
    d.key_chunk_sum[2LL * blockIdx.x + 1] = tot_raw;
  }
  if (which == 1 && d.fold_ctrl) {   // the accept decision in the last CTA of the problem
    __shared__ int last;
    const int p = ch.prob;
    if (last_arrival(d.fold_count + 2 * p + 1,
                     d.prob_key_chunk_off[p + 1] - d.prob_key_chunk_off[p], &last))
      ctrl_accept_body<true>(d, p, red);
  }
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
  double acc_raw = 0.0;
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
    const float2* cam = d.cam_ff[par] + 10 * __ldg(d.img_cam + img);
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
    {
      const float r0 = e0f.hi + e0f.lo, r1 = e1f.hi + e1f.lo;
      acc_raw += double(fmaf(r0, r0, r1 * r1));
    }
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
  // the candidate's Jacobian records, used if it is accepted: a second pass
  // over the chunk (each thread its own keys and the residuals it just
  // wrote), so the cost loop keeps its register count
  if (which == 1 && d.fuse_lin) linearize_chunk<float>(d, ch, par);
  const double tot = block_sum(double(acc.hi) + double(acc.lo), red);
  const double tot_raw = block_sum(acc_raw, red);
  if (threadIdx.x == 0) {
    d.key_chunk_sum[2LL * blockIdx.x] = tot;
    d.key_chunk_sum[2LL * blockIdx.x + 1] = tot_raw;
  }
  if (which == 1 && d.fold_ctrl) {   // the accept decision in the last CTA of the problem
    __shared__ int last;
    const int p = ch.prob;
    if (last_arrival(d.fold_count + 2 * p + 1,
                     d.prob_key_chunk_off[p + 1] - d.prob_key_chunk_off[p], &last))
      ctrl_accept_body<true>(d, p, red);
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
    const T* __restrict__ JR = tptr<T>(d.JR[st.parity]);
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
    if (d.pt_cons_off) {   // soft constraints: weight on the diagonal, w (x - y) in g
      const double* xp = d.x_pt[st.parity] + 3LL * pt;
      for (int c = d.pt_cons_off[pt]; c < d.pt_cons_off[pt + 1]; ++c) {
        const int row = d.cons_by_pt[c];
        const int b = d.cons[row].z;
        const double2 yw = d.cons_yw[row];
        V[b == 0 ? 0 : (b == 1 ? 3 : 5)] += T(yw.y);
        g[b] += T(yw.y * (xp[b] - yw.x));
      }
    }
    if (d.pt_prior_off) {   // point priors: V += L (its symmetric part), g += L (x - y)
      // (ba_gcp_constrained_normal_equation_builder.hpp:59-72)
      const double* xp = d.x_pt[st.parity] + 3LL * pt;
      for (int c = d.pt_prior_off[pt]; c < d.pt_prior_off[pt + 1]; ++c) {
        const int i = d.prior_by_pt[c];
        const double* L = d.prior_info + 9LL * i;
        const double v0 = xp[0] - d.prior_y[3LL * i], v1 = xp[1] - d.prior_y[3LL * i + 1],
                     v2 = xp[2] - d.prior_y[3LL * i + 2];
        V[0] += T(L[0]);
        V[1] += T(0.5 * (L[1] + L[3]));
        V[2] += T(0.5 * (L[2] + L[6]));
        V[3] += T(L[4]);
        V[4] += T(0.5 * (L[5] + L[7]));
        V[5] += T(L[8]);
        g[0] += T(L[0] * v0 + L[1] * v1 + L[2] * v2);
        g[1] += T(L[3] * v0 + L[4] * v1 + L[5] * v2);
        g[2] += T(L[6] * v0 + L[7] * v1 + L[8] * v2);
      }
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
  const T* __restrict__ JR = tptr<T>(d.JR[st.parity]);
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
  if (d.img_cons_off && lane < 27) {   // soft constraints on this image's parameters
    int a = -1, b = -1;
    if (lane < 21) {
      int e = lane;
      a = 0;
      while (e >= 6 - a) { e -= 6 - a; ++a; }
      b = a + e;
    }
    const double* xi = d.x_img[st.parity] + 6LL * img;
    for (int c = d.img_cons_off[img]; c < d.img_cons_off[img + 1]; ++c) {
      const int row = d.cons_by_img[c];
      const int prm = d.cons[row].z;
      const double2 yw = d.cons_yw[row];
      if (lane < 21 && a == b && a == prm) v += yw.y;
      if (lane >= 21 && lane - 21 == prm) v += yw.y * (xi[prm] - yw.x);
    }
  }
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
// Free cameras: per image work item (the items of k_image_reduce) the sums
// E = J_i^T J_c (6 x 10), the upper triangle of J_c^T J_c (55) and J_c^T r
// (10) over its keys (camera_shared_normal_equation_builder.hpp:111-462 for
// the camera blocks).  A CTA stages 32 keys' rows [J_i | J_c | r] in shared
// memory; thread e owns sum e (each batch in T, batches added in FP64, keys
// in order).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(128) k_image_cam_reduce(DevPlan d) {
  __shared__ T M[64][17];
  const int4 it = d.img_items[blockIdx.x];   // (image, q begin, q end, prob)
  const LMState& st = d.state[it.w];
  if (!st.relin || !st.active) return;
  if (d.cam_info[d.img_cam[it.x]].x == 0) return;
  const T* __restrict__ JR = tptr<T>(d.JR[st.parity]);
  const T* __restrict__ JC = tptr<T>(d.JC[st.parity]);
  const int e = threadIdx.x;
  int ca = 0, cb = 0;
  if (e < 60) {
    ca = e / 10;
    cb = 6 + e % 10;
  } else if (e < 115) {
    int t = e - 60, m = 0;
    while (t >= 10 - m) {
      t -= 10 - m;
      ++m;
    }
    ca = 6 + m;
    cb = 6 + m + t;
  } else if (e < 125) {
    ca = 6 + (e - 115);
    cb = 16;
  }
  double acc = 0.0;
  for (int q0 = it.y; q0 < it.z; q0 += 32) {
    const int nq = min(32, it.z - q0);
    if (threadIdx.x < 64) {   // thread r stages row r: key r/2, Jacobian row r%2
      const int row = threadIdx.x, kq = row >> 1, rr = row & 1;
      T v[17];
#pragma unroll
      for (int c = 0; c < 17; ++c) v[c] = T(0);
      if (kq < nq) {
        const long long k = __ldg(d.img_keys + q0 + kq);
        const T* jr = JR + kJRStride * k;
        const T* jc = JC + 20 * k + 10 * rr;
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = jr[6 + 6 * rr + c];
#pragma unroll
        for (int c = 0; c < 10; ++c) v[6 + c] = jc[c];
        v[16] = jr[18 + rr];
      }
#pragma unroll
      for (int c = 0; c < 17; ++c) M[row][c] = v[c];
    }
    __syncthreads();
    if (e < 125) {   // 32 keys in T, then into the FP64 total in key order
      T bs = T(0);
      for (int row = 0; row < 2 * nq; ++row) bs = fma(M[row][ca], M[row][cb], bs);
      acc += double(bs);
    }
    __syncthreads();
  }
  d.img_item_cam[(long long)kImgCamVals * blockIdx.x + e] = e < 125 ? acc : 0.0;
}

// Per image with a free camera: the FP64 sums of its work items' partials
// (items in order); E_i also goes to its own array for the assembly.
__global__ void __launch_bounds__(kImgCamVals) k_image_cam_finalize(DevPlan d) {
  const int img = blockIdx.x;
  const int4 ci = d.cam_info[d.img_cam[img]];
  if (ci.x == 0) return;
  const LMState& st = d.state[ci.z];
  if (!st.relin || !st.active) return;
  const int e = threadIdx.x;
  double v = 0.0;
  for (int t = d.img_item_off[img]; t < d.img_item_off[img + 1]; ++t)
    v += d.img_item_cam[(long long)kImgCamVals * t + e];
  d.img_cam_sum[(long long)kImgCamVals * img + e] = v;
  if (e < 60) d.Ei[60LL * img + e] = v;
}

// Per free camera: U_c and g_c summed over its images in FP64 (kCamGroups
// groups of kImgCamVals threads take every kCamGroups-th image in order, the
// group sums are added in group order), compacted to the computed
// parameters, with the camera's soft constraints
// (camera_shared_normal_equation_builder.hpp:309-349,418-459).
constexpr int kCamGroups = 8;
__global__ void __launch_bounds__(kImgCamVals * kCamGroups) k_cam_finalize(DevPlan d) {
  __shared__ double part[kCamGroups][kImgCamVals];
  __shared__ double sh[kImgCamVals];
  const int c = blockIdx.x;
  const int4 ci = d.cam_info[c];
  if (ci.x == 0) return;
  const LMState& st = d.state[ci.z];
  if (!st.relin || !st.active) return;
  const int e = threadIdx.x % kImgCamVals, grp = threadIdx.x / kImgCamVals;
  double tot = 0.0;
  for (int u = d.cam_img_off[c] + grp; u < d.cam_img_off[c + 1]; u += kCamGroups)
    tot += d.img_cam_sum[(long long)kImgCamVals * d.cam_imgs[u] + e];
  part[grp][e] = tot;
  __syncthreads();
  if (threadIdx.x < kImgCamVals) {
    double v = 0.0;
#pragma unroll
    for (int g = 0; g < kCamGroups; ++g) v += part[g][e];
    sh[e] = v;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int cps = ci.x;
  const unsigned mask = unsigned(ci.y);
  double* U = d.Uc + 100LL * c;
  double* g = d.gc + 10LL * c;
  for (int m = 0; m < cps; ++m) {
    const int fm = cam_full_col(mask, m);
    for (int n = 0; n < cps; ++n) {
      const int fn = cam_full_col(mask, n);
      U[10 * m + n] = sh[60 + upper10(min(fm, fn), max(fm, fn))];
    }
    g[m] = sh[115 + fm];
  }
  if (d.n_cons > 0) {
    const double* x = d.x_cam[st.parity] + 10LL * c;
    for (int r = d.prob_cons_off[ci.z]; r < d.prob_cons_off[ci.z + 1]; ++r) {
      const int4 cr = d.cons[r];
      if (cr.x != 2 || cr.y != c) continue;
      const double2 yw = d.cons_yw[r];
      U[11 * cr.z] += yw.y;
      g[cr.z] += yw.y * (x[cr.z] - yw.x);
    }
  }
  double dmax = 0.0, gmax = 0.0;
  for (int m = 0; m < cps; ++m) {
    dmax = fmax(dmax, U[11 * m]);
    gmax = fmax(gmax, fabs(g[m]));
  }
  LMState* sp = d.state + ci.z;
  atomicMax(&sp->maxdiag_bits, dbits(dmax));
  atomicMax(&sp->ginf_bits, dbits(gmax));
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

// Z_a = C_p^-1 J_p^T J_i per key, one slot per thread: slot s holds key s
// (records) or key img_keys[s], the keys image by image (planes), so the
// writes are coalesced either way.  DevPlan::key_z_split CTAs share each
// key chunk (a problem's slots are its keys' range), so the grid fills the
// GPU in even waves.
template <typename T>
__global__ void __launch_bounds__(256) k_key_z(DevPlan d) {
  const int split = d.key_z_split;
  const Chunk ch = d.key_chunks[blockIdx.x / split];
  const LMState& st = d.state[ch.prob];
  if (!st.active) return;
  const T* __restrict__ JR = tptr<T>(d.JR[st.parity]);
  const T* __restrict__ PS = tptr<T>(d.PS);
  T* __restrict__ Z = tptr_mut<T>(d.Z);
  const int sub = blockIdx.x % split;
  for (int sl = ch.begin + sub * 256 + threadIdx.x; sl < ch.end; sl += split * 256) {
    const int k = d.z_planes ? __ldg(d.img_keys + sl) : sl;
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
    store_z(d, Z, sl, z);
  }
}

// Free cameras: per camera record r of a point (camera c, part h) the Z
// record C_p^-1 W with W = sum over the point's keys seen through camera c
// of J_p^T J_c[:, 6h .. 6h+5] (computed parameters; zero past them).  The
// records of one camera are consecutive; one pass over the point's keys
// builds all of them (W for up to 12 computed columns).
template <typename T>
__global__ void __launch_bounds__(kPointChunk) k_camrec_z(DevPlan d) {
  const Chunk ch = d.pt_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.active) return;
  const int pt = ch.begin + threadIdx.x;
  if (pt >= ch.end) return;
  const int rb = d.pt_rec_off[pt], re = d.pt_rec_off[pt + 1];
  if (rb == re) return;
  const T* __restrict__ JR = tptr<T>(d.JR[st.parity]);
  const T* __restrict__ JC = tptr<T>(d.JC[st.parity]);
  T ps[8];
  load_vec<8>(tptr<T>(d.PS) + 12LL * pt, ps);
  const T i00 = ps[0], m10 = ps[1], i11 = ps[2], m20 = ps[3], m21 = ps[4], i22 = ps[5];
  const int kb = d.pt_key_off[pt], ke = d.pt_key_off[pt + 1];
  for (int r = rb; r < re;) {
    const int cam = d.rec_info[r - d.K].x;
    const int4 ci = d.cam_info[cam];
    const int nparts = (ci.x + 5) / 6;
    // W (3 x 12): the full-column index of each computed parameter
    T w[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) w[e] = T(0);
    for (int k = kb; k < ke; ++k) {
      if (__ldg(d.img_cam + __ldg(d.key_img + k)) != cam) continue;
      T jp[8], jc[20];
      load_vec<8>(JR + (long long)kJRStride * k, jp);
      load_vec<20>(JC + 20LL * k, jc);
#pragma unroll
      for (int m = 0; m < 12; ++m) {
        if (m >= ci.x) break;
        const int f = cam_full_col(unsigned(ci.y), m);
        T j0 = T(0), j1 = T(0);
#pragma unroll
        for (int q = 0; q < 10; ++q)
          if (q == f) {
            j0 = jc[q];
            j1 = jc[10 + q];
          }
#pragma unroll
        for (int i = 0; i < 3; ++i) w[12 * i + m] += jp[i] * j0 + jp[3 + i] * j1;
      }
    }
    for (int h = 0; h < nparts; ++h, ++r) {
      T z[kZStride];
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        T w0 = T(0), w1 = T(0), w2 = T(0);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh)
          if (hh == h) {
            w0 = w[6 * hh + a];
            w1 = w[12 + 6 * hh + a];
            w2 = w[24 + 6 * hh + a];
          }
        z[a] = i00 * w0;
        z[6 + a] = m10 * w0 + i11 * w1;
        z[12 + a] = m20 * w0 + m21 * w1 + i22 * w2;
      }
      z[18] = T(0);
      z[19] = T(0);
      store_z(d, tptr_mut<T>(d.Z), r, z);
    }
  }
}

// Plan build, Z planes: the slot of every key (the inverse of img_keys) ...
__global__ void __launch_bounds__(256) k_key_slots(const int* __restrict__ img_keys, int K, int* __restrict__ key_slot) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < K) key_slot[img_keys[s]] = s;
}

// ... and the key pairs of the assembly's work items as slots (a camera
// record's index, >= K, is its slot; a diagonal block's second entry is
// the point and stays).
__global__ void __launch_bounds__(128) k_pairs_to_slots(const int4* __restrict__ items, int n_items,
                                                        const int2* __restrict__ blk_ij,
                                                        const int* __restrict__ key_slot, int K,
                                                        int2* __restrict__ pairs) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= n_items) return;
  const int4 it = items[wid];
  const int2 ij = blk_ij[it.x];
  const bool diag = ij.x == ij.y;
  for (int q = it.y + lane; q < it.z; q += 32) {
    int2 pr = pairs[q];
    pr.x = pr.x < K ? key_slot[pr.x] : pr.x;
    if (!diag) pr.y = pr.y < K ? key_slot[pr.y] : pr.y;
    pairs[q] = pr;
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
  // the problem's state, the block and the first pair are independent
  // loads: all three are issued before the first of them is used
  const int active = d.state[it.w].active;
  const int2 ij = __ldg(d.blk_ij + it.x);
  int q = it.y + lane;
  int2 pr = q < it.z ? __ldg(d.pairs + q) : make_int2(0, 0);
  if (!active) return;
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
  for (; q < it.z; q += 32) {
    const int qn = q + 32;
    const int2 prn = qn < it.z ? __ldg(d.pairs + qn) : pr;
    T za[kZStride], zb[kZStride];
    load_z(d, Z, pr.x, za);
    if (diag) {
#pragma unroll
      for (int e = 0; e < kZStride; ++e) zb[e] = za[e];
      T ps[12];
      load_vec<12>(PS + 12LL * pr.y, ps);   // a diagonal block's pair carries the point
#pragma unroll
      for (int r = 0; r < 6; ++r) racc[r] += za[r] * ps[6] + za[6 + r] * ps[7] + za[12 + r] * ps[8];
    } else {
      load_z(d, Z, pr.y, zb);
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

// Sum of one entry over work items [ib, ie) (stride kItemStride): in order
// for short lists; else items t = ib + 4u + r go to partial r and the
// partials are added in order (four loads in flight).
__device__ __forceinline__ double sum_items4(const double* base, int ib, int ie) {
  if (ie - ib < 8) {   // the common short lists: in order
    double v = 0.0;
    for (int t = ib; t < ie; ++t) v += base[(long long)kItemStride * t];
    return v;
  }
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int t = ib;
  for (; t + 4 <= ie; t += 4) {
    s0 += base[(long long)kItemStride * t];
    s1 += base[(long long)kItemStride * (t + 1)];
    s2 += base[(long long)kItemStride * (t + 2)];
    s3 += base[(long long)kItemStride * (t + 3)];
  }
  if (t < ie) s0 += base[(long long)kItemStride * t];
  if (t + 1 < ie) s1 += base[(long long)kItemStride * (t + 1)];
  if (t + 2 < ie) s2 += base[(long long)kItemStride * (t + 2)];
  return (s0 + s1) + (s2 + s3);
}

// The entry (row 6i + a, column 6j + bcol), i >= j, of a problem's reduced
// system before the Schur terms and the damping (i, j local reduced-system
// images: the images, then each free camera's parts): U_i on an image's
// diagonal block, E_i between an image and the parts of its camera, U_c
// between parts of one camera; zero past a camera's parameters.
__device__ __forceinline__ double reduced_base(const DevPlan& d, const ProbInfo& pi, int i, int a, int j,
                                               int bcol) {
  const int ni = pi.num_images;
  if (i < ni) return i == j ? d.U[36LL * (pi.image_begin + i) + 6 * a + bcol] : 0.0;
  // camera part: global camera ci, parameter m of the row
  const int ci = pi.cam_begin + (i - ni) / pi.nc;
  const int4 cinf = d.cam_info[ci];
  const int m = 6 * ((i - ni) % pi.nc) + a;
  if (m >= cinf.x) return 0.0;
  if (j >= ni) {
    const int cj = pi.cam_begin + (j - ni) / pi.nc;
    const int mj = 6 * ((j - ni) % pi.nc) + bcol;
    return (cj == ci && mj < cinf.x) ? d.Uc[100LL * ci + 10 * m + mj] : 0.0;
  }
  const int gj = pi.image_begin + j;
  return d.img_cam[gj] == ci ? d.Ei[60LL * gj + 10 * bcol + cam_full_col(unsigned(cinf.y), m)] : 0.0;
}

// The gradient entry of row 6i + a of the reduced system (g_i or g_c).
__device__ __forceinline__ double reduced_grad(const DevPlan& d, const ProbInfo& pi, int i, int a) {
  const int ni = pi.num_images;
  if (i < ni) return d.gi[6LL * (pi.image_begin + i) + a];
  const int ci = pi.cam_begin + (i - ni) / pi.nc;
  const int m = 6 * ((i - ni) % pi.nc) + a;
  return m < d.cam_info[ci].x ? d.gc[10LL * ci + m] : 0.0;
}

// Dense reduced system (lower triangle) and rhs in precision T; the block
// sums over work items are taken in FP64.  Rows and columns run over the
// problem's reduced-system images: its images, then with free cameras nc
// 6-wide parts of each camera (camera_shared_normal_equation_solver.hpp:270-392,
// 422-443: U_c, the image-camera blocks E and g_c enter as the images' U and
// g do; columns past the camera's parameters hold mu alone).
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
  const int Ie = pi.num_ext, ni = pi.num_images;
  const int blk = __ldg(d.blk_map + d.blk_map_off[p] + (long long)j * Ie + i);
  double v = 0.0, rv = 0.0;
  if (blk >= 0) {   // four interleaved partial sums (loads in flight together), then in order
    const int ib = __ldg(d.blk_item_off + blk), ie = __ldg(d.blk_item_off + blk + 1);
    v = sum_items4(d.item_partial + 6 * bcol + a, ib, ie);
  }
  (void)ni;
  const double base = reduced_base(d, pi, i, a, j, bcol);
  const double g = col == 0 ? reduced_grad(d, pi, i, a) : 0.0;
  double s = base - v;
  if (row == col) s += st.mu;
  tptr_mut<T>(d.S)[pi.s_off + (long long)row * n + col] = T(s);
  if (col == 0) {
    // rhs b_i[a] = g_i[a] - sum over the diagonal block's items
    const int dblk = __ldg(d.blk_map + d.blk_map_off[p] + (long long)i * Ie + i);
    rv = 0.0;
    if (dblk >= 0) {
      const int ib = __ldg(d.blk_item_off + dblk), ie = __ldg(d.blk_item_off + dblk + 1);
      rv = sum_items4(d.item_partial + 36 + a, ib, ie);
    }
    tptr_mut<T>(d.b)[6LL * (pi.ext_begin + i) + a] = T(g - rv);
  }
}

// The same dense system, block by block (plans without free cameras): S is
// zeroed first (the entries of image pairs without a common point are 0),
// then one thread per entry of every block writes base - sum over the
// block's items (+ mu on the diagonal) exactly as k_assemble_S does, the 36
// threads of a block reading its items' partials together; the threads of
// row 0 of each diagonal block write the rhs.
template <typename T>
__global__ void __launch_bounds__(256) k_assemble_S_blocks(DevPlan d) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= 36LL * d.n_blocks) return;
  const int blk = int(e / 36), el = int(e % 36);
  const int p = __ldg(d.blk_prob + blk);
  const LMState& st = d.state[p];
  if (!st.active) return;
  const ProbInfo pi = d.prob[p];
  const int2 xy = __ldg(d.blk_ij + blk);   // column image x <= row image y
  const int a = el % 6, bcol = el / 6;     // partial entry 6 * bcol + a = el
  const int row = 6 * xy.y + a, col = 6 * xy.x + bcol;
  const int2 items = make_int2(__ldg(d.blk_item_off + blk), __ldg(d.blk_item_off + blk + 1));
  if (col <= row) {
    const double v = sum_items4(d.item_partial + el, items.x, items.y);
    const double base = reduced_base(d, pi, xy.y, a, xy.x, bcol);
    double s = base - v;
    if (row == col) s += st.mu;
    tptr_mut<T>(d.S)[pi.s_off + (long long)row * pi.n + col] = T(s);
  }
  if (xy.x == xy.y && bcol == 0) {   // rhs b_y[a] = g_y[a] - sum over the diagonal block's items
    const double rv = sum_items4(d.item_partial + 36 + a, items.x, items.y);
    const double g = reduced_grad(d, pi, xy.y, a);
    tptr_mut<T>(d.b)[6LL * (pi.ext_begin + xy.y) + a] = T(g - rv);
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

// Calls f(std::integral_constant<int, i>) for i = B, B + S, ... < E.
template <int B, int E, int S, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + S, E, S>(f);
  }
}

// Shared-memory tiles: rows padded to a 16-byte multiple (36 floats, 34
// doubles) so that 16-byte vector loads along a row are aligned and the
// rows touched together fall in different banks.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using V = float4;
  static constexpr int N = 4;
  __device__ __forceinline__ static void unpack(const V& v, float* o) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
  __device__ __forceinline__ static V pack(const float* o) { return make_float4(o[0], o[1], o[2], o[3]); }
};
template <>
struct Vec16<double> {
  using V = double2;
  static constexpr int N = 2;
  __device__ __forceinline__ static void unpack(const V& v, double* o) {
    o[0] = v.x;
    o[1] = v.y;
  }
  __device__ __forceinline__ static V pack(const double* o) { return make_double2(o[0], o[1]); }
};

template <typename T>
using Tile = T[kTile][kTile + Vec16<T>::N];

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

// s[u] = sum_q X[r][q] Y[c][q] (q ascending) for the 128 threads tid < 128:
// rows r = tid / 8 and r + 16, columns c = tid % 8 + 8u (u = 0..3); s[0..3]
// is row r, s[4..7] row r + 16.  Rows are read with 16-byte vector loads; the
// rows a warp reads at once lie in distinct banks.  Two rows per thread halve
// the shared-memory wavefronts per FMA against one row per thread.
template <typename T>
__device__ __forceinline__ void tile_xyt_t(const Tile<T>& X, const Tile<T>& Y, T s[8], int t) {
  using V = Vec16<T>;
  constexpr int N = V::N;
  const int r = t >> 3, c0 = t & 7;
#pragma unroll
  for (int u = 0; u < 8; ++u) s[u] = T(0);
#pragma unroll
  for (int q = 0; q < kTile; q += N) {
    T x0[N], x1[N];
    V::unpack(*reinterpret_cast<const typename V::V*>(&X[r][q]), x0);
    V::unpack(*reinterpret_cast<const typename V::V*>(&X[r + 16][q]), x1);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      T y[N];
      V::unpack(*reinterpret_cast<const typename V::V*>(&Y[c0 + 8 * u][q]), y);
#pragma unroll
      for (int e = 0; e < N; ++e) {
        s[u] = fma(x0[e], y[e], s[u]);
        s[4 + u] = fma(x1[e], y[e], s[4 + u]);
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void tile_xyt(const Tile<T>& X, const Tile<T>& Y, T s[8]) {
  tile_xyt_t<T>(X, Y, s, threadIdx.x);
}

// A -= X Y^T (32x32x32) by the 128 threads t = 0..127 of a thread group, 8
// outputs each (the same outputs and sums for every group).
template <typename T>
__device__ __forceinline__ void tile_sub_xyt_t(Tile<T>& A, const Tile<T>& X, const Tile<T>& Y, int t) {
  T s[8];
  tile_xyt_t<T>(X, Y, s, t);
  const int r = t >> 3, c0 = t & 7;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    A[r][c0 + 8 * u] -= s[u];
    A[r + 16][c0 + 8 * u] -= s[4 + u];
  }
}

// A -= X Y^T (32x32x32) by threads 0..127, 8 outputs each.
template <typename T>
__device__ __forceinline__ void tile_sub_xyt(Tile<T>& A, const Tile<T>& X, const Tile<T>& Y) {
  if (threadIdx.x >= 128) return;
  T s[8];
  tile_xyt<T>(X, Y, s);
  const int r = threadIdx.x >> 3, c0 = threadIdx.x & 7;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    A[r][c0 + 8 * u] -= s[u];
    A[r + 16][c0 + 8 * u] -= s[4 + u];
  }
}

// Factor the SPD tile D (lower triangle used; identity-padded) and write
// L^-1 to Dinv (D is left as it is), in two warps of the CTA: lane i of warp
// 0 keeps row i of the tile in registers, lane i of warp 1 column i of L^-1
// (forward substitution against L).  Columns are factored two at a time:
// every lane of warp 0 forms the 2x2 pivot block from three shuffles (both
// reciprocal square roots issued together: the second pivot is det / p0),
// then its own entries of both columns, which go to shared memory (col: two
// buffers of two columns, piv: two buffers of the pivot block's r0, l10,
// r1) for the trailing updates -- of the tile's rows in warp 0, of the
// inverse's columns in warp 1, after one 64-thread named barrier per column
// pair.  A buffer is rewritten two column pairs later, after warp 1 has
// passed the next barrier, so one barrier per pair suffices.  No divisions.
// Returns false (in warp 0) when a pivot was not positive.
constexpr int kPotrfBarrier = 1;   // named barrier id (0 is __syncthreads)

__device__ __forceinline__ void potrf_pair_sync() {
  asm volatile("bar.sync %0, 64;\n" ::"n"(kPotrfBarrier) : "memory");
}

template <typename T>
__device__ bool pair_potrf_inverse(const Tile<T>& D, Tile<T>& Dinv, T* col, T* piv, int warp, int lane) {
  using V = Vec16<T>;
  constexpr int N = V::N;
  constexpr unsigned FULL = 0xffffffffu;
  bool ok = true;
  if (warp == 0) {
    T a[kTile];
#pragma unroll
    for (int q = 0; q < kTile; q += N) V::unpack(*reinterpret_cast<const typename V::V*>(&D[lane][q]), a + q);
    // j is a compile-time constant in every step, so a[] stays in registers
    static_for<0, kTile, 2>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      const T p0 = __shfl_sync(FULL, a[j], j);
      const T p1 = __shfl_sync(FULL, a[j], j + 1);
      const T p2 = __shfl_sync(FULL, a[j + 1], j + 1);
      const T det = fma(p0, p2, -(p1 * p1));
      const T r0 = rsqrt(p0);
      const T rd = rsqrt(det);
      const T l00 = p0 * r0;             // sqrt(p0)
      const T l10 = p1 * r0;
      const T r1 = l00 * rd;             // 1 / sqrt(det / p0)
      const T l11 = det * rd * r0;       // sqrt(det / p0)
      ok = ok && (p0 > T(0)) && (det > T(0));
      const T li0 = (lane > j) ? a[j] * r0 : ((lane == j) ? l00 : T(0));
      const T li1 = (lane > j + 1) ? fma(-li0, l10, a[j + 1]) * r1 : ((lane == j + 1) ? l11 : T(0));
      a[j] = li0;
      a[j + 1] = li1;
      const int buf = (j >> 1) & 1;
      T* cb = col + buf * 2 * kTile;
      cb[lane] = li0;
      cb[kTile + lane] = li1;
      if (lane == 0) {
        piv[4 * buf] = r0;
        piv[4 * buf + 1] = l10;
        piv[4 * buf + 2] = r1;
      }
      potrf_pair_sync();
#pragma unroll
      for (int l = j + 2; l < kTile; ++l) {
        const T c0 = cb[l], c1 = cb[kTile + l];
        a[l] = fma(-li0, c0, a[l]);
        a[l] = fma(-li1, c1, a[l]);
      }
    });
  } else {
    T x[kTile];
#pragma unroll
    for (int r = 0; r < kTile; ++r) x[r] = (r == lane) ? T(1) : T(0);
    static_for<0, kTile, 2>([&](auto jc) {
      constexpr int j = decltype(jc)::value;
      potrf_pair_sync();
      const int buf = (j >> 1) & 1;
      const T* cb = col + buf * 2 * kTile;
      const T r0 = piv[4 * buf], l10 = piv[4 * buf + 1], r1 = piv[4 * buf + 2];
      x[j] *= r0;
      x[j + 1] = fma(-l10, x[j], x[j + 1]) * r1;
#pragma unroll
      for (int l = j + 2; l < kTile; ++l) {
        const T c0 = cb[l], c1 = cb[kTile + l];
        x[l] = fma(-c0, x[j], x[l]);
        x[l] = fma(-c1, x[j + 1], x[l]);
      }
    });
#pragma unroll
    for (int r = 0; r < kTile; ++r) Dinv[r][lane] = x[r];
  }
  return ok;
}

template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 1) k_chol_step(DevPlan d, int k) {
  __shared__ __align__(16) Tile<T> A, Li, Lj, D, Dinv;
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
  T* b = tptr_mut<T>(d.b) + 6LL * pi.ext_begin;
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
  __shared__ T colbuf[4 * kTile + 8];
  if (warp < 2) {
    const bool ok = pair_potrf_inverse<T>(i == c ? A : D, Dinv, colbuf, colbuf + 4 * kTile, warp, lane);
    if (warp == 0 && lane == 0) ok_s = ok ? 1 : 0;
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
    if (tid < mi) b[kTile * c + tid] = yk[tid];
    return;
  }
  // i > c: L_ic = A_ic L_cc^-T, and the column-k part of the forward solve
  if (tid < mi) b[kTile * i + tid] = tv[tid];
  if (tid < 128) {
    T sv[8];
    tile_xyt<T>(A, Dinv, sv);
    const int r = tid >> 3, c0 = tid & 7;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (r + 16 * h < mi) {
        T* row = S + (long long)(kTile * i + r + 16 * h) * n + kTile * c;
#pragma unroll
        for (int u = 0; u < 4; ++u) row[c0 + 8 * u] = sv[4 * h + u];
      }
    }
  }
}

// Dataflow factorization of one problem's reduced system in a single
// cooperative launch.  Every CTA owns a fixed set of tiles of the lower
// triangle and keeps them in shared memory for the whole factorization: the
// diagonal tile (i, i) and the tile left of it, (i, i-1), belong to the CTA
// of row i; the other tiles are spread by work (j + 1 tasks for tile (i, j))
// over all CTAs.  A tile's tasks are its updates A_ij -= L_ik L_jk^T for
// k = 0 .. j-1, in that order, then its factorization (i == j, with the
// forward solve y_j = L_jj^-1 b_j) or its panel L_ij = A_ij L_jj^-T.  A
// finished factor or panel is written to global memory (L into S, L_jj^-1
// into Linv, y_j into b) and announced by storing the launch's epoch into
// the tile's flag with release semantics; consumers poll flags with acquire
// loads and read the data through L2.  Each CTA runs, among its tiles whose
// next task has its inputs published, the one with the smallest (j, i), and
// applies up to kDfBatch consecutive ready updates of that tile with all of
// their loads in flight together.  Per element the arithmetic is exactly
// that of k_chol_step (same tile routines, same order of updates), so both
// schedules give the same bits.  Every wait is bounded: a CTA that sees
// nothing ready for DevPlan::df_spin_limit polls records a timeout and leaves; a
// failed pivot or a timeout raises the abort word, which every waiting CTA
// checks.
constexpr int kDfThreads = 256;

template <typename T>
__host__ __device__ constexpr int df_batch() { return 2; }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Tile loads through L2 (data another CTA published in this launch).
template <typename T>
__device__ __forceinline__ void fetch_rect_cg(TileFetch<T>& f, const T* S, int n, int ti, int tj) {
  const int mi = tile_rows(n, ti), mj = tile_rows(n, tj);
#pragma unroll
  for (int u = 0; u < kPerThread; ++u) {
    const int e = threadIdx.x + u * kCholThreads, r = e / kTile, c = e % kTile;
    f.v[u] = (r < mi && c < mj) ? __ldcg(S + (long long)(kTile * ti + r) * n + kTile * tj + c) : T(0);
  }
}

template <typename T>
size_t df_smem_bytes(int max_own) {
  return sizeof(Tile<T>) * size_t(max_own + 2 * df_batch<T>() + 1) +
         sizeof(T) * size_t(max_own) * kTile + sizeof(int) * size_t(5 * max_own + 8);
}

template <typename T>
__global__ void __launch_bounds__(kDfThreads, 1) k_chol_dataflow(DevPlan d) {
  constexpr int NB = df_batch<T>();
  enum { kIdle = 0, kUpdate = 1, kFinish = 2, kChain = 3, kExit = 4, kChain2 = 5 };
  extern __shared__ __align__(16) unsigned char df_raw[];
  __shared__ T yv[NB][kTile], colbuf[4 * kTile + 8];
  __shared__ int s_sel, s_cnt, s_mode, s_ok;
  const int p = 0;
  const ProbInfo pi = d.prob[p];
  const int n = pi.n, nt = pi.nt;
  const int ob = d.df_own_off[blockIdx.x], nown = d.df_own_off[blockIdx.x + 1] - ob;
  const int mo = d.df_max_own;
  Tile<T>* A = reinterpret_cast<Tile<T>*>(df_raw);   // [mo] owned tiles
  Tile<T>* W = A + mo;                                // [2 * NB] fetched L tiles
  Tile<T>& Dinv = W[2 * NB];
  T* bown = reinterpret_cast<T*>(W + 2 * NB + 1);     // [mo][kTile] rhs of owned diagonal tiles
  int* ti_s = reinterpret_cast<int*>(bown + size_t(mo) * kTile);
  int* tj_s = ti_s + mo;
  int* kt_s = tj_s + mo;       // next update step of each owned tile (j: factor/panel; j+1: done)
  int* rd_s = kt_s + mo;       // ready tasks found by the last poll
  int* pr_s = rd_s + mo;       // tile (i, i-1): local index of (i, i); otherwise -1
  T* S = tptr_mut<T>(d.S) + pi.s_off;
  T* b = tptr_mut<T>(d.b) + 6LL * pi.ext_begin;
  T* Lg = tptr_mut<T>(d.Linv) + (long long)p * d.max_nt * kTile * kTile;
  unsigned* flags = d.df_flags;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned epoch = *reinterpret_cast<volatile unsigned*>(d.df_sync) + 1u;

  // factor the diagonal tile A[t] of row i in warp 0 and publish L_ii^-1 and
  // y_i = L_ii^-1 b_i; false (after raising the abort word) on a bad pivot
  auto finish_diag = [&](int t, int i) -> bool {
    if (warp < 2) {
      const bool ok = pair_potrf_inverse<T>(A[t], Dinv, colbuf, colbuf + 4 * kTile, warp, lane);
      if (warp == 0 && lane == 0) s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) {
      if (tid == 0) {
        d.factor_flag[p] = 1;
        __threadfence();
        atomicExch(d.df_sync + 2, epoch);
      }
      return false;
    }
    T* Lo = Lg + (long long)i * kTile * kTile;
    for (int e = tid; e < kTile * kTile; e += blockDim.x) Lo[e] = Dinv[e / kTile][e % kTile];
    if (tid < kTile) {
      T y = T(0);
#pragma unroll 8
      for (int q = 0; q < kTile; ++q) y += Dinv[tid][q] * bown[t * kTile + q];
      if (tid < tile_rows(n, i)) b[kTile * i + tid] = y;
    }
    __syncthreads();
    if (tid == 0) {
      st_release_u32(flags + (long long)i * nt + i, epoch);
      kt_s[t] = i + 1;
    }
    return true;
  };

  const LMState& st = d.state[p];
  const bool run = st.active && !d.factor_flag[p];
  if (run) {
    for (int t = tid; t < nown; t += blockDim.x) {
      const int2 tl = d.df_own[ob + t];
      ti_s[t] = tl.x;
      tj_s[t] = tl.y;
      kt_s[t] = 0;
    }
    __syncthreads();
    for (int t = tid; t < nown; t += blockDim.x) {
      int pr = -1;
      if (tj_s[t] == ti_s[t] - 1)
        for (int u = 0; u < nown; ++u)
          if (ti_s[u] == ti_s[t] && tj_s[u] == ti_s[t]) pr = u;
      pr_s[t] = pr;
    }
    for (int t = 0; t < nown; ++t) {      // owned tiles and rhs
      TileFetch<T> f;
      const int i = ti_s[t], j = tj_s[t];
      if (i == j) f.diag(S, n, i); else f.rect(S, n, i, j);
      f.store(A[t]);
      if (i == j && tid < kTile) bown[t * kTile + tid] = tid < tile_rows(n, i) ? b[kTile * i + tid] : T(0);
    }
  }
  __syncthreads();
  int ndone = run ? 0 : nown;
  long long idle = 0;
  // optional timeline (thread 0): per task its wait start, selection, end
  unsigned long long* tr = d.df_trace ? d.df_trace + size_t(blockIdx.x) * kDfTraceCap * 4 : nullptr;
  unsigned long long tr_wait = 0, tr_sel = 0, tr_meta = 0;
  int tr_n = 0;
  bool tr_open = false;
  if (tr && tid == 0) tr_wait = global_ns();
  while (ndone < nown) {
    if (tr && tid == 0 && tr_open) {
      const unsigned long long now = global_ns();
      if (tr_n < kDfTraceCap) {
        unsigned long long* e = tr + 4 * tr_n;
        e[0] = tr_meta;
        e[1] = tr_wait;
        e[2] = tr_sel;
        e[3] = now;
      }
      ++tr_n;
      tr_open = false;
      tr_wait = now;
    }
    // poll: for each owned tile, how many of its next tasks have their inputs
    for (int t = tid; t < nown; t += blockDim.x) {
      const int i = ti_s[t], j = tj_s[t], k = kt_s[t];
      int c = 0;
      if (k < j) {
        unsigned fi[NB], fj[NB];
#pragma unroll
        for (int u = 0; u < NB; ++u) {
          fi[u] = (k + u < j) ? ld_acquire_u32(flags + (long long)i * nt + k + u) : 0u;
          fj[u] = (k + u < j && i != j) ? ld_acquire_u32(flags + (long long)j * nt + k + u) : epoch;
        }
#pragma unroll
        for (int u = 0; u < NB; ++u)
          if (c == u && k + u < j && fi[u] == epoch && fj[u] == epoch) c = u + 1;
      } else if (k == j) {
        c = (i == j || ld_acquire_u32(flags + (long long)j * nt + j) == epoch) ? 1 : 0;
      }
      // a subdiagonal tile one update short of its panel: is L_jj^-1 out too?
      int linv = 0;
      if (pr_s[t] >= 0 && k == j - 1) linv = ld_acquire_u32(flags + (long long)j * nt + j) == epoch;
      rd_s[t] = c | linv << 8;
    }
    __syncthreads();
    if (tid == 0) {
      int sel = -1, cnt = 0, mode = kIdle;
      for (int t = 0; t < nown; ++t) {
        if ((rd_s[t] & 0xff) > 0) {
          const bool diag_at = pr_s[t] >= 0 && kt_s[pr_s[t]] == ti_s[t] - 1;
          // the chain's subdiagonal tile keeps its last update for the fused
          // task (below) until L_jj^-1 is out and its diagonal tile has all
          // other updates: run alone it would split the chain into three
          // tasks on the critical path (the inputs it waits for never
          // depend on this tile)
          if (pr_s[t] >= 0 && kt_s[t] == tj_s[t] - 1 && (!(rd_s[t] >> 8) || !diag_at)) continue;
          sel = t;
          cnt = rd_s[t] & 0xff;
          mode = kt_s[t] < tj_s[t] ? kUpdate : kFinish;
          if (mode == kFinish && diag_at) mode = kChain;
          // the last update of a subdiagonal tile, its panel and the next
          // diagonal factor in one task when L_jj^-1 is already out
          if (mode == kUpdate && diag_at && kt_s[t] == tj_s[t] - 1 && (rd_s[t] >> 8)) mode = kChain2;
          break;
        }
      }
      if (sel < 0) {
        // the abort word is read every 16th idle round, the limit counted always
        if ((++idle & 15) == 0 && ld_acquire_u32(d.df_sync + 2) == epoch) {
          mode = kExit;
        } else if (idle > d.df_spin_limit) {
          d.factor_flag[p] = 2;                       // timed out
          __threadfence();
          atomicExch(d.df_sync + 2, epoch);
          mode = kExit;
        }
      }
      s_sel = sel;
      s_cnt = cnt;
      s_mode = mode;
      if (tr && sel >= 0) {
        tr_sel = global_ns();
        tr_meta = (unsigned long long)mode << 56 | (unsigned long long)ti_s[sel] << 40 |
                  (unsigned long long)tj_s[sel] << 24 | (unsigned long long)kt_s[sel] << 8 |
                  (unsigned long long)cnt;
        tr_open = true;
      }
    }
    __syncthreads();
    const int mode = s_mode, t = s_sel, cnt = s_cnt;
    if (mode == kExit) break;
    if (mode == kIdle) continue;
    const int i = ti_s[t], j = tj_s[t], k0 = kt_s[t];
    if (mode == kUpdate) {
      // cnt consecutive updates from columns k0 .. k0+cnt-1
      TileFetch<T> fi[NB], fj[NB];
      T yr[NB];
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        if (u < cnt) {
          fetch_rect_cg<T>(fi[u], S, n, i, k0 + u);
          if (i != j) fetch_rect_cg<T>(fj[u], S, n, j, k0 + u);
          if (i == j && tid < kTile) yr[u] = __ldcg(b + kTile * (k0 + u) + tid);
        }
      }
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        if (u < cnt) {
          fi[u].store(W[2 * u]);
          if (i != j) fj[u].store(W[2 * u + 1]);
          if (i == j && tid < kTile) yv[u][tid] = yr[u];
        }
      }
      __syncthreads();
      for (int u = 0; u < cnt; ++u) {
        tile_sub_xyt<T>(A[t], W[2 * u], i == j ? W[2 * u] : W[2 * u + 1]);
        if (i == j && tid < kTile) {
          T tv = bown[t * kTile + tid];
#pragma unroll 8
          for (int q = 0; q < kTile; ++q) tv -= W[2 * u][tid][q] * yv[u][q];
          bown[t * kTile + tid] = tv;
        }
      }
      __syncthreads();
      if (tid == 0) kt_s[t] = k0 + cnt;
      __syncthreads();
      continue;
    }
    if (i == j) {                          // factor a diagonal tile
      if (!finish_diag(t, i)) break;
      ++ndone;
      __syncthreads();
      continue;
    }
    // panel L_ij = A_ij L_jj^-T, kept in A[t] (kChain2: after the update
    // from column j-1)
    const bool chain = mode == kChain || mode == kChain2;
    {
      TileFetch<T> f, fi, fj;
      const T* Li = Lg + (long long)j * kTile * kTile;
#pragma unroll
      for (int u = 0; u < kPerThread; ++u) f.v[u] = __ldcg(Li + threadIdx.x + u * kCholThreads);
      if (mode == kChain2) {
        fetch_rect_cg<T>(fi, S, n, i, j - 1);
        fetch_rect_cg<T>(fj, S, n, j, j - 1);
      }
      T yj = T(0);
      if (chain && tid < kTile) yj = __ldcg(b + kTile * j + tid);
      f.store(Dinv);
      if (mode == kChain2) {
        fi.store(W[0]);
        fj.store(W[1]);
      }
      if (chain && tid < kTile) yv[0][tid] = yj;
    }
    __syncthreads();
    if (mode == kChain2) {
      tile_sub_xyt<T>(A[t], W[0], W[1]);
      __syncthreads();
    }
    {
      T sv[8];
      if (tid < 128) tile_xyt<T>(A[t], Dinv, sv);
      __syncthreads();
      if (tid < 128) {
        const int r = tid >> 3, c0 = tid & 7;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          A[t][r][c0 + 8 * u] = sv[u];
          A[t][r + 16][c0 + 8 * u] = sv[4 + u];
        }
      }
    }
    __syncthreads();
    {
      const int mi = tile_rows(n, i);
      const int r = tid >> 3, c0 = tid & 7;
      if (r < mi) {
        T* row = S + (long long)(kTile * i + r) * n + kTile * j;
#pragma unroll
        for (int u = 0; u < 4; ++u) row[c0 + 8 * u] = A[t][r][c0 + 8 * u];
      }
    }
    if (chain) {
      // the diagonal tile of row i: its last update (from this panel), then
      // its factorization; both are announced together
      const int td = pr_s[t];
      tile_sub_xyt<T>(A[td], A[t], A[t]);
      if (tid < kTile) {
        T tv = bown[td * kTile + tid];
#pragma unroll 8
        for (int q = 0; q < kTile; ++q) tv -= A[t][tid][q] * yv[0][q];
        bown[td * kTile + tid] = tv;
      }
      __syncthreads();
      if (!finish_diag(td, i)) break;
      ++ndone;
    } else {
      __syncthreads();
    }
    if (tid == 0) {
      st_release_u32(flags + (long long)i * nt + j, epoch);
      kt_s[t] = j + 1;
    }
    ++ndone;
    __syncthreads();
  }
  if (tr && tid == 0 && tr_open && tr_n < kDfTraceCap) {
    unsigned long long* e = tr + 4 * tr_n;
    e[0] = tr_meta;
    e[1] = tr_wait;
    e[2] = tr_sel;
    e[3] = global_ns();
  }
  // the last CTA to finish opens the next epoch
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(d.df_sync + 1, 1u);
    if (prev == gridDim.x - 1) {
      d.df_sync[1] = 0u;
      __threadfence();
      atomicAdd(d.df_sync, 1u);
    }
  }
}

// Backward solve L^T delta = y in one launch per batch.  Problems with more
// than kSolveSmallTiles tile rows get a cluster of kSolveRanks CTAs, the
// others one CTA (R = 1).  Rank q owns the tile rows t = q (mod R) of y in
// shared memory.  Step j (nt-1 down to 0): warp 7 of the owner of row j
// forms delta_j = L_jj^-T y_j (y_j is final: its last update came from this
// same CTA at step j+1) and stores it into every rank's shared memory; after
// a cluster barrier every rank subtracts L_ji^T delta_j from its rows i < j,
// warp w taking rows q + R*(w + 8u), reading row block j of L coalesced
// along the row with the next step's loads already in flight.  The barrier
// arrives relaxed (it must not wait for those loads); the delta stores are
// ordered by a cluster-scope fence in the storing warp.
constexpr int kSolveRanks = 8;
constexpr int kSolveSmallTiles = 8;
constexpr int kSolveOwnerWarp = 7;

__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
  asm volatile("barrier.cluster.wait.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void fence_cluster() {
  asm volatile("fence.acq_rel.cluster;\n" ::: "memory");
}

template <typename T, int R>
__device__ __forceinline__ void chol_solve_body(const DevPlan& d, int q) {
  constexpr int kRows = R == 1 ? kSolveSmallTiles : (6 * 2048 / kTile + R - 1) / R;
  __shared__ T ys[kRows][kTile];
  __shared__ T xb[2][kTile];
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;   // the same for every rank
  const ProbInfo pi = d.prob[p];
  const int nt = pi.nt, n = pi.n;
  const T* S = tptr<T>(d.S) + pi.s_off;
  T* b = tptr_mut<T>(d.b) + 6LL * pi.ext_begin;
  const T* Linv = tptr<T>(d.Linv) + (long long)p * d.max_nt * kTile * kTile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nown = nt > q ? (nt - q + R - 1) / R : 0;
  for (int e = tid; e < nown * kTile; e += blockDim.x) {
    const int lt = e / kTile, r = e % kTile, t = q + R * lt;
    ys[lt][r] = (kTile * t + r < n) ? b[kTile * t + r] : T(0);
  }
  // rows of step jj this warp handles first: i = q + R*warp
  T cur[kTile];
  auto fetch = [&](int jj) {
    const int i = q + R * warp;
    if (jj < 0 || i >= jj) return;
    const int mj = tile_rows(n, jj);
    const T* row = S + (long long)kTile * jj * n + kTile * i + lane;
#pragma unroll
    for (int r = 0; r < kTile; ++r) cur[r] = r < mj ? row[(long long)r * n] : T(0);
  };
  // column `lane` of L_jj^-1 for the next diagonal tile this rank owns
  T lv[kTile];
  int jown = nt - 1 - ((nt - 1 - q) % R + R) % R;
  auto fetch_linv = [&](int jj) {
    if (jj < 0 || warp != kSolveOwnerWarp) return;
    const T* Lv = Linv + (long long)jj * kTile * kTile + lane;
#pragma unroll
    for (int r = 0; r < kTile; ++r) lv[r] = r >= lane ? Lv[r * kTile] : T(0);
  };
  fetch(nt - 1);
  fetch_linv(jown);
  if constexpr (R == 1) {
    __syncthreads();
  } else {   // every rank has started before its shared memory is written
    __syncthreads();
    cluster_arrive_relaxed();
    cluster_wait();
  }
  for (int j = nt - 1; j >= 0; --j) {
    const int par = j & 1;
    T s = T(0);
    const bool owner = (j == jown && warp == kSolveOwnerWarp);
    if (owner) {
      const T* y = ys[j / R];
#pragma unroll
      for (int r = 0; r < kTile; ++r) s += lv[r] * y[r];
      if constexpr (R == 1) {
        xb[par][lane] = s;
      } else {
        cg::cluster_group cluster = cg::this_cluster();
        for (int rk = 0; rk < R; ++rk) *cluster.map_shared_rank(&xb[par][lane], rk) = s;
        fence_cluster();
      }
    }
    if constexpr (R == 1) {
      __syncthreads();
    } else {
      cluster_arrive_relaxed();
      cluster_wait();
    }
    if (owner) {
      if (kTile * j + lane < n) b[kTile * j + lane] = s;
      jown -= R;
      fetch_linv(jown);
    }
    const int nact = j > q ? (j - q + R - 1) / R : 0;
    if (warp < nact) {
      T acc = T(0);
#pragma unroll
      for (int r = 0; r < kTile; ++r) acc += cur[r] * xb[par][r];
      ys[warp][lane] -= acc;
    }
    for (int lt = warp + 8; lt < nact; lt += 8) {
      const int i = q + R * lt;
      const int mj = tile_rows(n, j);
      const T* row = S + (long long)kTile * j * n + kTile * i + lane;
      T acc = T(0);
      for (int r = 0; r < mj; ++r) acc += row[(long long)r * n] * xb[par][r];
      ys[lt][lane] -= acc;
    }
    fetch(j - 1);
    __syncthreads();
  }
}

// The cluster backward solve without a cluster-wide barrier per step.
// Rank q of the cluster owns the tile rows t = q (mod R) of y (local row
// lt = t / R) and warp w of the rank the local rows lt = w (mod 8).  Every
// rank keeps a slot per step j for delta_j and an mbarrier per step that
// completes once the 32 entries of delta_j have landed in the slot.  Step j
// (nt-1 down to 0): the warp owning row j forms delta_j = L_jj^-T y_j as
// soon as y_j is final (its last update, from step j+1, was this warp's
// own), and each of its lanes stores its entry into slot j of every rank
// with st.async, which counts the bytes against that rank's mbarrier j (no
// fence, no separate arrival).  Every warp waits on its own rank's
// mbarrier j (acquire), then subtracts L_ji^T delta_j from its rows i < j,
// the highest one (the next diagonal step's row when this warp owns it)
// from registers loaded one step ahead.  The per-row arithmetic is that of
// the single-CTA body.  Slots are not reused within a launch.  Waits are bounded
// (DevPlan::solve_spin_limit polls): a warp that gives up records a timeout
// in the problem's factor flag (the solve is void) and stops updating, but
// still sends its own deltas of the later steps; after a cluster barrier
// (every store issued) it waits, bounded again, for the stores into its rank
// that are still landing, so no CTA leaves while another writes into it.

template <typename T>
__host__ __device__ constexpr size_t solve_smem_bytes(int max_nt) {
  return size_t(max_nt) * 8 + size_t(max_nt) * kTile * sizeof(T) +
         size_t((max_nt + kSolveRanks - 1) / kSolveRanks) * kTile * sizeof(T);
}

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(b)), "r"(count) : "memory");
}
// An asynchronous store of v into rank `rank`'s copy of *dst that counts
// its bytes against that rank's copy of the mbarrier b (complete_tx): a
// waiter that sees the phase complete (acquire) sees the value.
template <typename T>
__device__ __forceinline__ void st_async_rank(T* dst, unsigned long long* b, int rank, T v) {
  unsigned ra, rb;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(ra) : "r"(smem_addr(dst)), "r"(rank));
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(rb) : "r"(smem_addr(b)), "r"(rank));
  if constexpr (sizeof(T) == 4)
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];\n" ::"r"(ra),
                 "r"(__float_as_uint(v)), "r"(rb)
                 : "memory");
  else
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];\n" ::"r"(ra),
                 "l"(__double_as_longlong(v)), "r"(rb)
                 : "memory");
}
// This thread's arrival on b, announcing `bytes` of asynchronous stores.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void cluster_sync_acq_rel() {
  asm volatile("barrier.cluster.arrive.aligned;\nbarrier.cluster.wait.aligned;\n" ::: "memory");
}

constexpr long long kSolveSpin = 1LL << 22;   // polls of a step's mbarrier (production)

// kProbe: the instantiation that reads the test controls of DevPlan
// (solve_spin_limit, solve_drop_step); production plans launch the other.
template <typename T, bool kProbe>
__global__ void __cluster_dims__(kSolveRanks, 1, 1) __launch_bounds__(256)
k_chol_solve(DevPlan d) {
  constexpr int R = kSolveRanks;
  const long long spin_limit = kProbe ? d.solve_spin_limit : kSolveSpin;
  const int drop_step = kProbe ? d.solve_drop_step : -1;
  extern __shared__ __align__(16) unsigned char solve_raw[];
  cg::cluster_group cluster = cg::this_cluster();
  const int q = int(cluster.block_rank());
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;   // the same for every rank
  const ProbInfo pi = d.prob[p];
  const int nt = pi.nt, n = pi.n, mt = d.max_nt;
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(solve_raw);   // [mt]
  T* xs = reinterpret_cast<T*>(bar + mt);                                         // [mt][kTile]
  T* ys = xs + size_t(mt) * kTile;                                                // [rows][kTile]
  const T* S = tptr<T>(d.S) + pi.s_off;
  T* b = tptr_mut<T>(d.b) + 6LL * pi.ext_begin;
  const T* Linv = tptr<T>(d.Linv) + (long long)p * d.max_nt * kTile * kTile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nown = nt > q ? (nt - q + R - 1) / R : 0;
  for (int e = tid; e < nown * kTile; e += blockDim.x) {
    const int lt = e / kTile, r = e % kTile, t = q + R * lt;
    ys[e] = (kTile * t + r < n) ? b[kTile * t + r] : T(0);
  }
  // barrier j completes when the owner's 32 stores of delta_j have landed
  for (int j = tid; j < nt; j += blockDim.x) {
    mbar_init(bar + j, 1);
    mbar_arrive_expect_tx(bar + j, unsigned(kTile * sizeof(T)));
  }
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  __syncthreads();
  cluster_sync_acq_rel();   // every rank's barriers exist before anyone arrives on them
  // the warp's rows, highest first: lt = lt_top, lt_top - 8, ...
  const int lt_top = warp < nown ? warp + 8 * ((nown - 1 - warp) / 8) : -1;
  // column `lane` of L_jj^-1 for the warp's next diagonal row
  T lv[kTile];
  auto fetch_linv = [&](int lt) {
    if (lt < 0) return;
    const T* Lv = Linv + (long long)(q + R * lt) * kTile * kTile + lane;
#pragma unroll
    for (int r = 0; r < kTile; ++r) lv[r] = r >= lane ? Lv[r * kTile] : T(0);
  };
  // L_ji (column `lane`) of the warp's highest row below j, loaded a step ahead
  T cur[kTile];
  int cur_lt = -1;
  auto fetch_cur = [&](int jj) {
    cur_lt = -1;
    if (jj < 0 || lt_top < 0) return;
    int lt = lt_top;
    while (lt >= 0 && q + R * lt >= jj) lt -= 8;
    if (lt < 0) return;
    cur_lt = lt;
    const int mj = tile_rows(n, jj);
    const T* row = S + (long long)kTile * jj * n + kTile * (q + R * lt) + lane;
#pragma unroll
    for (int r = 0; r < kTile; ++r) cur[r] = r < mj ? row[(long long)r * n] : T(0);
  };
  fetch_linv(lt_top);
  fetch_cur(nt - 1);
  int next_diag = lt_top;   // the warp's next diagonal row (local index)
  int j_fail = -1;
  for (int j = nt - 1; j >= 0; --j) {
    if (next_diag >= 0 && q + R * next_diag == j) {
      __syncwarp();   // y_j's entries are this warp's own, written in step j+1
      const T* y = ys + next_diag * kTile;
      T sj = T(0);
#pragma unroll
      for (int r = 0; r < kTile; ++r) sj += lv[r] * y[r];
      if (j != drop_step)
        for (int rk = 0; rk < R; ++rk) st_async_rank(xs + (size_t)j * kTile + lane, bar + j, rk, sj);
      if (kTile * j + lane < n) b[kTile * j + lane] = sj;
      next_diag -= 8;
      fetch_linv(next_diag);
    }
    long long spin = 0;
    while (!mbar_try_wait_cluster(bar + j, 0u))
      if (++spin > spin_limit) break;
    if (spin > spin_limit) {   // delta_j did not come: the solve is void
      if (lane == 0) d.factor_flag[p] = 2;
      j_fail = j;
      break;
    }
    const T* xj = xs + (size_t)j * kTile;
    if (cur_lt >= 0) {
      T acc = T(0);
#pragma unroll
      for (int r = 0; r < kTile; ++r) acc += cur[r] * xj[r];
      ys[cur_lt * kTile + lane] -= acc;
      for (int lt = cur_lt - 8; lt >= 0; lt -= 8) {   // the warp's other rows below j
        const int mj = tile_rows(n, j);
        const T* row = S + (long long)kTile * j * n + kTile * (q + R * lt) + lane;
        T a2 = T(0);
        for (int r = 0; r < mj; ++r) a2 += row[(long long)r * n] * xj[r];
        ys[lt * kTile + lane] -= a2;
      }
    }
    fetch_cur(j - 1);
  }
  if (j_fail >= 0) {
    // the warp gave up at step j_fail: it still sends its own deltas of the
    // steps below (void values), so every delta another warp waits for is sent
    for (int j = j_fail - 1; j >= 0; --j) {
      if (next_diag >= 0 && q + R * next_diag == j) {
        if (j != drop_step)
          for (int rk = 0; rk < R; ++rk) st_async_rank(xs + (size_t)j * kTile + lane, bar + j, rk, T(0));
        next_diag -= 8;
      }
    }
  }
  __syncthreads();
  cluster_sync_acq_rel();   // every rank has issued all of its stores
  if (j_fail >= 0) {
    // wait (bounded) for the stores into this rank that are still landing
    // before the CTA may leave
    for (int j = 0; j < nt; ++j) {
      long long spin = 0;
      while (!mbar_try_wait_cluster(bar + j, 0u) && ++spin <= spin_limit) {
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_chol_solve_small(DevPlan d) {
  chol_solve_body<T, 1>(d, 0);
}

// Batched factorization and solve of small reduced systems (at most
// kSolveSmallTiles tile rows, FP32): one CTA per problem keeps the tiles of
// the lower triangle in shared memory and runs the schedule of the
// per-column launches (k_chol_step) inside the CTA -- for each column c the
// diagonal tile's factor and inverse, the panels L_ic = A_ic L_cc^-T, the
// forward-solve updates b_i -= L_ic y_c, then the trailing updates A_ij -=
// L_ic L_jc^T, two tiles at a time -- with the same per-element arithmetic,
// so the result has the bits of k_chol_step and k_chol_dataflow; then the
// backward solve of k_chol_solve_small.  One launch per LM iteration
// instead of one per tile column plus the solve.
template <typename T>
__host__ __device__ constexpr size_t chol_small_smem(int max_nt) {
  return size_t(max_nt) * (max_nt + 1) / 2 * sizeof(Tile<T>);
}

template <typename T>
__global__ void __launch_bounds__(kCholThreads, 1) k_chol_small(DevPlan d) {
  extern __shared__ __align__(16) unsigned char cs_raw[];
  __shared__ __align__(16) Tile<T> Dinv;
  __shared__ T bs[kSolveSmallTiles][kTile];   // b after the columns done so far
  __shared__ T colbuf[4 * kTile + 8];
  __shared__ int ok_s;
  Tile<T>* A = reinterpret_cast<Tile<T>*>(cs_raw);   // tile (i, j), j <= i, at i (i + 1) / 2 + j
  const int p = blockIdx.y;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p]) return;
  const ProbInfo pi = d.prob[p];
  const int nt = pi.nt, n = pi.n;
  if (nt > kSolveSmallTiles || nt > d.max_nt) {   // (never: the planner's bound) fail loudly
    if (threadIdx.x == 0) d.factor_flag[p] = 1;
    return;
  }
  T* S = tptr_mut<T>(d.S) + pi.s_off;
  T* b = tptr_mut<T>(d.b) + 6LL * pi.ext_begin;
  T* Lg = tptr_mut<T>(d.Linv) + (long long)p * d.max_nt * kTile * kTile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto at = [&](int i, int j) -> Tile<T>& { return A[i * (i + 1) / 2 + j]; };
  for (int i = 0; i < nt; ++i)
    for (int j = 0; j <= i; ++j) {
      TileFetch<T> f;
      if (i == j) f.diag(S, n, i); else f.rect(S, n, i, j);
      f.store(at(i, j));
    }
  for (int e = tid; e < nt * kTile; e += blockDim.x) {
    const int t = e / kTile, r = e % kTile;
    bs[t][r] = r < tile_rows(n, t) ? b[kTile * t + r] : T(0);
  }
  __syncthreads();
  for (int c = 0; c < nt; ++c) {
    if (warp < 2) {
      const bool ok = pair_potrf_inverse<T>(at(c, c), Dinv, colbuf, colbuf + 4 * kTile, warp, lane);
      if (warp == 0 && lane == 0) ok_s = ok ? 1 : 0;
    }
    __syncthreads();
    if (!ok_s) {
      if (tid == 0) d.factor_flag[p] = 1;
      return;
    }
    // L_cc^-1 out, y_c = L_cc^-1 b_c (b_c after the columns before c)
    for (int e = tid; e < kTile * kTile; e += blockDim.x) Lg[(long long)c * kTile * kTile + e] = Dinv[e / kTile][e % kTile];
    if (tid < kTile) {
      T y = T(0);
#pragma unroll 8
      for (int q = 0; q < kTile; ++q) y += Dinv[tid][q] * bs[c][q];
      colbuf[tid] = y;   // (the factor's buffers are free again)
    }
    // panels L_ic = A_ic L_cc^-T, two tiles at a time
    for (int i = c + 1 + (tid >> 7); i < nt; i += 2) {
      T sv[8];
      tile_xyt_t<T>(at(i, c), Dinv, sv, tid & 127);
      const int r = (tid & 127) >> 3, c0 = tid & 7;
      // every read of this tile precedes its writes within the thread group
      asm volatile("bar.sync %0, 128;\n" ::"r"(2 + (tid >> 7)) : "memory");
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int u = 0; u < 4; ++u) at(i, c)[r + 16 * h][c0 + 8 * u] = sv[4 * h + u];
    }
    __syncthreads();
    if (tid < kTile) {
      bs[c][tid] = colbuf[tid];
      if (tid < tile_rows(n, c)) b[kTile * c + tid] = colbuf[tid];
    }
    for (int i = c + 1; i < nt; ++i) {   // the panels into S for the backward solve
      const int mi = tile_rows(n, i);
      for (int e = tid; e < kTile * kTile; e += blockDim.x) {
        const int r = e / kTile, q = e % kTile;
        if (r < mi) S[(long long)(kTile * i + r) * n + kTile * c + q] = at(i, c)[r][q];
      }
    }
    __syncthreads();
    // forward-solve updates of the rows below: b_i -= L_ic y_c
    for (int e = tid; e < (nt - c - 1) * kTile; e += blockDim.x) {
      const int i = c + 1 + e / kTile, r = e % kTile;
      T t = bs[i][r];
#pragma unroll 8
      for (int q = 0; q < kTile; ++q) t -= at(i, c)[r][q] * bs[c][q];
      bs[i][r] = t;
    }
    // trailing updates A_ij -= L_ic L_jc^T, c < j <= i, two tiles at a time
    const int m = nt - c - 1, ntr = m * (m + 1) / 2;
    for (int lin = tid >> 7; lin < ntr; lin += 2) {
      int ti = 0;
      while ((ti + 1) * (ti + 2) / 2 <= lin) ++ti;
      const int i = c + 1 + ti, j = c + 1 + (lin - ti * (ti + 1) / 2);
      tile_sub_xyt_t<T>(at(i, j), at(i, c), at(j, c), tid & 127);
    }
    __syncthreads();
  }
  chol_solve_body<T, 1>(d, 0);
}

// ---------------------------------------------------------------------------
// Block-Jacobi PCG on the block-sparse reduced system (large scenes).  The
// reduced system keeps one 6x6 block per co-visible image pair (first image
// <= second): Sblk[blk][6x + y] is the row of component x of the first image
// and the column of component y of the second.  The matrix-vector product
// runs one warp per image over the blocks touching it (each block read from
// both ends, no atomics); all sums have a fixed order, so a problem's
// iterates are the same alone and in a batch.  The solution overwrites b.
// Per problem and iteration: p.q, r.z, r.r and b.b are reduced from per-chunk
// partials (chunks of kImageChunk images) by every CTA that needs them.
// ---------------------------------------------------------------------------
__device__ double block_sum_all(double v, double* smem) {
  const double r = block_sum(v, smem);
  if (threadIdx.x == 0) smem[32] = r;
  __syncthreads();
  return smem[32];
}

__device__ __forceinline__ double pcg_prob_sum(const DevPlan& d, int p, int slot, double* red) {
  double v = 0.0;
  for (int c = d.prob_ext_chunk_off[p] + threadIdx.x; c < d.prob_ext_chunk_off[p + 1]; c += blockDim.x)
    v += d.pcg_part[(long long)kPcgSlots * c + slot];
  return block_sum_all(v, red);
}

template <typename T>
__global__ void __launch_bounds__(256) k_assemble_blocks(DevPlan d) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= 36LL * d.n_blocks) return;
  const int blk = int(e / 36), el = int(e % 36);
  const int2 g = __ldg(d.blk_gij + blk);   // global reduced-system images, g.x <= g.y
  const int p = __ldg(d.ext_prob + g.x);
  const LMState& st = d.state[p];
  if (!st.active) return;
  const ProbInfo& pi = d.prob[p];
  const int ib = __ldg(d.blk_item_off + blk), ie = __ldg(d.blk_item_off + blk + 1);
  double v = 0.0;
  for (int t = ib; t < ie; ++t) v += d.item_partial[(long long)kItemStride * t + el];
  double sv = -v;
  // entry (component el / 6 of g.x, component el % 6 of g.y); the base of
  // the symmetric system is read as row (g.y, el % 6), column (g.x, el / 6)
  const int lx = g.x - pi.ext_begin, ly = g.y - pi.ext_begin;
  if (ly < pi.num_images) {
    if (g.x == g.y) sv += d.U[36LL * (pi.image_begin + lx) + el];
  } else {
    sv += reduced_base(d, pi, ly, el % 6, lx, el / 6);
  }
  if (g.x == g.y && el % 7 == 0) sv += st.mu;
  tptr_mut<T>(d.Sblk)[36LL * blk + el] = T(sv);
  if (g.x == g.y && el < 6) {
    double rv = 0.0;
    for (int t = ib; t < ie; ++t) rv += d.item_partial[(long long)kItemStride * t + 36 + el];
    tptr_mut<T>(d.b)[6LL * g.x + el] = T(reduced_grad(d, pi, lx, el) - rv);
  }
}

// Inverse of each image's diagonal block (6x6 Cholesky, then L^-T L^-1).
template <typename T>
__global__ void __launch_bounds__(128) k_pcg_precond(DevPlan d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.I_ext) return;
  const int p = d.ext_prob[i];
  if (!d.state[p].active) return;
  const T* A = tptr<T>(d.Sblk) + 36LL * d.img_diag_blk[i];
  T L[6][6], X[6][6];
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    T sjj = A[7 * j];
#pragma unroll
    for (int k = 0; k < j; ++k) sjj -= L[j][k] * L[j][k];
    ok = ok && sjj > T(0);
    const T ljj = sqrt(sjj > T(0) ? sjj : T(1));
    const T rj = T(1) / ljj;
    L[j][j] = ljj;
#pragma unroll
    for (int r = j + 1; r < 6; ++r) {
      T sr = A[6 * r + j];
#pragma unroll
      for (int k = 0; k < j; ++k) sr -= L[r][k] * L[j][k];
      L[r][j] = sr * rj;
    }
  }
  // X = L^-1 (lower), column by column
#pragma unroll
  for (int c = 0; c < 6; ++c) {
#pragma unroll
    for (int r = 0; r < 6; ++r) {
      if (r < c) {
        X[r][c] = T(0);
        continue;
      }
      T v = (r == c) ? T(1) : T(0);
#pragma unroll
      for (int k = c; k < r; ++k) v -= L[r][k] * X[k][c];
      X[r][c] = v / L[r][r];
    }
  }
  T* M = tptr_mut<T>(d.Minv) + 36LL * i;
#pragma unroll
  for (int x = 0; x < 6; ++x)
#pragma unroll
    for (int y = 0; y < 6; ++y) {
      T v = T(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) v += X[k][x] * X[k][y];
      M[6 * x + y] = v;
    }
  if (!ok) atomicExch(d.factor_flag + p, 1);
}

// z = Minv r for this warp's image: lanes 0..5 hold r and return z.
template <typename T>
__device__ __forceinline__ T pcg_precond_apply(const DevPlan& d, int img, T rv, int lane) {
  const T* M = tptr<T>(d.Minv) + 36LL * img;
  T z = T(0);
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const T rk = __shfl_sync(0xffffffffu, rv, k);
    if (lane < 6) z += M[6 * lane + k] * rk;
  }
  return z;
}

// x = 0 (in b), r = b, z = Minv r, p_0 = 0; partials r.z, r.r, b.b.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_init(DevPlan d) {
  __shared__ double red[33];
  if (d.pcg_it && blockIdx.x == 0 && threadIdx.x == 0) *d.pcg_it = 0;   // the device-side loop's count
  const Chunk ch = d.ext_chunks[blockIdx.x];
  const LMState& st = d.state[ch.prob];
  if (!st.active || d.factor_flag[ch.prob]) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int img = ch.begin + warp;
  double rz = 0.0, rr = 0.0;
  if (img < ch.end) {
    T* b = tptr_mut<T>(d.b);
    const T rv = lane < 6 ? b[6LL * img + lane] : T(0);
    const T z = pcg_precond_apply<T>(d, img, rv, lane);
    if (lane < 6) {
      b[6LL * img + lane] = T(0);
      tptr_mut<T>(d.pcg_r)[6LL * img + lane] = rv;
      tptr_mut<T>(d.pcg_z)[6LL * img + lane] = z;
      tptr_mut<T>(d.pcg_p[0])[6LL * img + lane] = T(0);
      rz = double(rv) * double(z);
      rr = double(rv) * double(rv);
    }
  }
  rz = block_sum(rz, red);
  rr = block_sum(rr, red);
  if (threadIdx.x == 0) {
    double* part = d.pcg_part + (long long)kPcgSlots * blockIdx.x;
    part[1] = rz;
    part[3] = rr;
    part[5] = rr;
    part[6] = 0.0;
    if (blockIdx.x == d.prob_ext_chunk_off[ch.prob]) d.pcg_done[ch.prob] = 0;
  }
}

// Iteration it, part 1: beta from the last two r.z, p = z + beta p_old (own
// images stored, neighbours' formed on the fly), q = S p, partial p.q.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_spmv(DevPlan d, int it, int loop) {
  __shared__ double red[33];
  // in the device-side loop `it` is the half (0, 1) of the loop body's pass
  if (loop) it += 2 * *reinterpret_cast<volatile int*>(d.pcg_it);
  if (it >= d.pcg_max_iterations) return;
  const Chunk ch = d.ext_chunks[blockIdx.x];
  const int p = ch.prob;
  const LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p] || d.pcg_done[p]) return;
  const int par = it & 1;
  const double rz = pcg_prob_sum(d, p, 1 + par, red);
  const double rr = pcg_prob_sum(d, p, 3 + par, red);
  const double bb = pcg_prob_sum(d, p, 5, red);
  if (rr <= d.pcg_tol2 * bb) return;                  // converged (or b = 0)
  const double rzp = it > 0 ? pcg_prob_sum(d, p, 1 + (par ^ 1), red) : 1.0;
  const T beta = it > 0 ? T(rz / rzp) : T(0);
  const T* z = tptr<T>(d.pcg_z);
  const T* pold = tptr<T>(d.pcg_p[par]);
  T* pnew = tptr_mut<T>(d.pcg_p[par ^ 1]);
  const T* Sb = tptr<T>(d.Sblk);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int img = ch.begin + warp;
  double dot = 0.0;
  if (img < ch.end) {
    T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    const int a0 = __ldg(d.adj_off + img), a1 = __ldg(d.adj_off + img + 1);
    for (int e = a0 + lane; e < a1; e += 32) {
      const int2 en = __ldg(d.adj + e);
      const int j = en.y >> 1;
      T pj[6];
#pragma unroll
      for (int c = 0; c < 6; ++c) pj[c] = z[6LL * j + c] + beta * pold[6LL * j + c];
      const T* B = Sb + 36LL * en.x;
      if (!(en.y & 1)) {
#pragma unroll
        for (int x = 0; x < 6; ++x)
#pragma unroll
          for (int y = 0; y < 6; ++y) acc[x] += B[6 * x + y] * pj[y];
      } else {
#pragma unroll
        for (int x = 0; x < 6; ++x)
#pragma unroll
          for (int y = 0; y < 6; ++y) acc[y] += B[6 * x + y] * pj[x];
      }
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] = warp_sum_t<T>(acc[c]);
    if (lane < 6) {
      T qv = acc[0];
#pragma unroll
      for (int c = 1; c < 6; ++c)
        if (lane == c) qv = acc[c];
      const T pv = z[6LL * img + lane] + beta * pold[6LL * img + lane];
      pnew[6LL * img + lane] = pv;
      tptr_mut<T>(d.pcg_q)[6LL * img + lane] = qv;
      dot = double(pv) * double(qv);
    }
  }
  dot = block_sum(dot, red);
  if (threadIdx.x == 0) d.pcg_part[(long long)kPcgSlots * blockIdx.x] = dot;
}

// Iteration it, part 2: alpha = r.z / p.q, x += alpha p, r -= alpha q,
// z = Minv r, partials of the next r.z and r.r.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_update(DevPlan d, int it, int loop) {
  __shared__ double red[33];
  if (loop) it += 2 * *reinterpret_cast<volatile int*>(d.pcg_it);
  if (it >= d.pcg_max_iterations) return;
  const Chunk ch = d.ext_chunks[blockIdx.x];
  const int p = ch.prob;
  LMState& st = d.state[p];
  if (!st.active || d.factor_flag[p] || d.pcg_done[p]) return;
  const bool lead = blockIdx.x == d.prob_ext_chunk_off[p];
  const int par = it & 1;
  const double rz = pcg_prob_sum(d, p, 1 + par, red);
  const double rr = pcg_prob_sum(d, p, 3 + par, red);
  const double bb = pcg_prob_sum(d, p, 5, red);
  double* part = d.pcg_part + (long long)kPcgSlots * blockIdx.x;
  if (rr <= d.pcg_tol2 * bb) {
    // converged: carry this chunk's partials to the next parity so that
    // every later iteration sees the same sums and returns as well
    if (threadIdx.x == 0) {
      part[1 + (par ^ 1)] = part[1 + par];
      part[3 + (par ^ 1)] = part[3 + par];
      if (lead) d.pcg_done[p] = 1;   // later launches return at once
    }
    return;
  }
  const double pq = pcg_prob_sum(d, p, 0, red);
  if (!(pq > 0.0)) {
    // breakdown (the residual is at the rounding floor): keep x and stop, by
    // zeroing the next r.r, which the branch above then carries forward
    if (threadIdx.x == 0) {
      part[1 + (par ^ 1)] = part[1 + par];
      part[3 + (par ^ 1)] = 0.0;
    }
    return;
  }
  const T alpha = T(rz / pq);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int img = ch.begin + warp;
  double rzn = 0.0, rrn = 0.0, xr = 0.0;
  if (img < ch.end) {
    const long long o = 6LL * img + (lane < 6 ? lane : 0);
    T rv = T(0);
    if (lane < 6) {
      T* x = tptr_mut<T>(d.b);
      T* r = tptr_mut<T>(d.pcg_r);
      const T pv = tptr<T>(d.pcg_p[par ^ 1])[o];
      const T qv = tptr<T>(d.pcg_q)[o];
      const T xv = x[o] + alpha * pv;
      x[o] = xv;
      rv = r[o] - alpha * qv;
      r[o] = rv;
      xr = double(xv) * double(rv);
    }
    const T z = pcg_precond_apply<T>(d, img, rv, lane);
    if (lane < 6) {
      tptr_mut<T>(d.pcg_z)[o] = z;
      rzn = double(rv) * double(z);
      rrn = double(rv) * double(rv);
    }
  }
  rzn = block_sum(rzn, red);
  rrn = block_sum(rrn, red);
  xr = block_sum(xr, red);
  if (threadIdx.x == 0) {
    part[1 + (par ^ 1)] = rzn;
    part[3 + (par ^ 1)] = rrn;
    part[6] = xr;
    if (lead) st.pcg_iters += 1;
  }
}

// The device-side PCG loop (a CUDA-graph while node): after each pass of
// two iterations one warp counts the pass and ends the loop once every
// problem's inner solve has stopped (converged, broken down, not solving)
// or the iterations are used up.
__global__ void __launch_bounds__(32) k_pcg_loop_ctrl(DevPlan d, cudaGraphConditionalHandle h) {
  const int m = *reinterpret_cast<volatile int*>(d.pcg_it) + 1;
  bool more = 2 * m < d.pcg_max_iterations;
  if (more) {
    bool open = false;
    for (int p = threadIdx.x; p < d.B && !open; p += 32) {
      const LMState& st = d.state[p];
      open = st.active && !d.factor_flag[p] && !d.pcg_done[p];
    }
    more = __any_sync(0xffffffffu, open);
  }
  __syncwarp();
  if (threadIdx.x == 0) {
    *d.pcg_it = m;
    if (more) ++*d.pcg_extra;
    cudaGraphSetConditional(h, more ? 1u : 0u);
  }
}

// ---------------------------------------------------------------------------
// back-substitution and update
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kPointChunk) k_backsub(DevPlan d) {
  __shared__ double red[32];
  // With DevPlan::fold_ctrl the last CTA of a problem to finish runs the LM
  // step decision (k_ctrl_step's body), so every CTA of an active problem
  // arrives, also when the factorization failed and there is nothing to do.
  const int prob = blockIdx.x < d.n_pt_chunks ? d.pt_chunks[blockIdx.x].prob
                                              : d.img_chunks[blockIdx.x - d.n_pt_chunks].prob;
  if (!d.state[prob].active) return;
  const bool failed = d.factor_flag[prob] != 0;
  if (failed) {
    // nothing to compute
  } else if (blockIdx.x < d.n_pt_chunks) {
    const Chunk ch = d.pt_chunks[blockIdx.x];
    const LMState& st = d.state[ch.prob];
    const int par = st.parity;
    const int pt = ch.begin + threadIdx.x;
    double dn2 = 0.0, xn2 = 0.0, gd = 0.0;
    if (pt < ch.end) {
      T ps[12];
      load_vec<12>(tptr<T>(d.PS) + 12LL * pt, ps);
      const T i00 = ps[0], m10 = ps[1], i11 = ps[2], m20 = ps[3], m21 = ps[4], i22 = ps[5];
      const T* __restrict__ JR = tptr<T>(d.JR[st.parity]);
      const int kb = __ldg(d.pt_key_off + pt), ke = __ldg(d.pt_key_off + pt + 1);
      // w = sum over the point's keys of J_p^T (J_i delta_i) from the
      // Jacobian records (the point's keys are consecutive), then
      // t = C^-1 (g - w) with C^-1 g = h
      T w0 = T(0), w1 = T(0), w2 = T(0);
      for (int k = kb; k < ke; ++k) {
        T rec[kJRStride];
        load_vec<kJRStride>(JR + (long long)kJRStride * k, rec);
        const int ext = d.img_ext ? __ldg(d.img_ext + __ldg(d.key_img + k)) : __ldg(d.key_img + k);
        const T* di = tptr<T>(d.b) + 6LL * ext;
        T u0 = T(0), u1 = T(0);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const T dl = di[c];
          u0 += rec[6 + c] * dl;
          u1 += rec[12 + c] * dl;
        }
        w0 += rec[0] * u0 + rec[3] * u1;
        w1 += rec[1] * u0 + rec[4] * u1;
        w2 += rec[2] * u0 + rec[5] * u1;
      }
      T t0 = ps[6] - i00 * w0, t1 = ps[7] - (m10 * w0 + i11 * w1), t2 = ps[8] - (m20 * w0 + m21 * w1 + i22 * w2);
      // free cameras: the point's camera records (Z = C^-1 W) against their
      // reduced-system images' deltas
      if (d.pt_rec_off) {
        const T* __restrict__ Z = tptr<T>(d.Z);
        const int rb = __ldg(d.pt_rec_off + pt), re = __ldg(d.pt_rec_off + pt + 1);
        for (int r = rb; r < re; ++r) {
          T z[kZStride];
          load_z(d, Z, r, z);
          const T* di = tptr<T>(d.b) + 6LL * __ldg(&d.rec_info[r - d.K].y);
#pragma unroll
          for (int c = 0; c < 6; ++c) {
            const T dl = di[c];
            t0 -= z[c] * dl;
            t1 -= z[6 + c] * dl;
            t2 -= z[12 + c] * dl;
          }
        }
      }
      // delta = C^-T t, C^-1 rows [i00 0 0; m10 i11 0; m20 m21 i22]
      const double dp[3] = {double(i00 * t0 + m10 * t1 + m20 * t2), double(i11 * t1 + m21 * t2),
                            double(i22 * t2)};
      T pv[12];
      load_vec<12>(tptr<T>(d.PV) + 12LL * pt, pv);
      const double* x = d.x_pt[par] + 3LL * pt;
      double* xn = d.x_pt[1 - par] + 3LL * pt;
      float2* xf = d.x_ff[1 - par] ? d.x_ff[1 - par] + 3LL * pt : nullptr;
      const bool free_pt = !(d.prob[ch.prob].fix & 1);   // a fixed point is not in x
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        xn[a] = x[a] - dp[a];
        if (xf) xf[a] = ff_split(xn[a]);
        dn2 += dp[a] * dp[a];
        if (free_pt) xn2 += x[a] * x[a];
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
    const int par = st.parity;
    double dn2 = 0.0, xn2 = 0.0, gd = 0.0;
    const long long e0 = 6LL * ch.begin, e1 = 6LL * ch.end;
    const ProbInfo& pi = d.prob[ch.prob];
    const long long boff = 6LL * (pi.ext_begin - pi.image_begin);
    const bool free_img = !(pi.fix & 2);   // fixed images are not in x
    for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      double dv = double(tptr<T>(d.b)[e + boff]), xv = d.x_img[par][e];
      d.x_img[1 - par][e] = xv - dv;
      dn2 += dv * dv;
      if (free_img) xn2 += xv * xv;
      gd += d.gi[e] * dv;
    }
    double s0 = block_sum(dn2, red), s1 = block_sum(xn2, red), s2 = block_sum(gd, red);
    // the candidate's rotations (block_sum's barriers made x_img[1 - par] visible)
    if (threadIdx.x < ch.end - ch.begin) image_prep_one<T>(d, ch.begin + threadIdx.x, 1 - par);
    if (threadIdx.x == 0) {
      d.img_chunk_sum[3LL * c] = s0;
      d.img_chunk_sum[3LL * c + 1] = s1;
      d.img_chunk_sum[3LL * c + 2] = s2;
    }
  }
  if (d.fold_ctrl) {
    __shared__ int last;
    const int total = d.prob_pt_chunk_off[prob + 1] - d.prob_pt_chunk_off[prob] +
                      d.prob_img_chunk_off[prob + 1] - d.prob_img_chunk_off[prob];
    if (last_arrival(d.fold_count + 2 * prob, total, &last)) ctrl_step_body<true>(d, prob, red);
  }
}

// Free cameras: delta_c from the camera's parts of the reduced-system
// solution, the candidate x_c - delta_c, and the camera's terms of
// ||delta||^2, ||x||^2 and g^T delta.
template <typename T>
__global__ void k_cam_backsub(DevPlan d) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.Ctot) return;
  const int4 ci = d.cam_info[c];
  const LMState& st = d.state[ci.z];
  if (!st.active || d.factor_flag[ci.z]) return;
  double dn2 = 0.0, xn2 = 0.0, gd = 0.0;
  if (ci.x > 0) {
    const int par = st.parity;
    const T* b = tptr<T>(d.b) + 6LL * ci.w;
    for (int m = 0; m < ci.x; ++m) {
      const double dv = double(b[m]), xv = d.x_cam[par][10LL * c + m];
      d.x_cam[1 - par][10LL * c + m] = xv - dv;
      dn2 += dv * dv;
      xn2 += xv * xv;
      gd += d.gc[10LL * c + m] * dv;
    }
  }
  d.cam_sum[3LL * c] = dn2;
  d.cam_sum[3LL * c + 1] = xn2;
  d.cam_sum[3LL * c + 2] = gd;
}

// ---------------------------------------------------------------------------
// LM control (one warp per problem)
// ---------------------------------------------------------------------------
// Sum of one field of a problem's chunk partials by the whole CTA (thread t
// adds chunks t, t + blockDim, ... in order, then a fixed-shape tree):
// deterministic, and each thread waits on a few loads instead of one warp
// walking hundreds of chunks.  Result valid in thread 0.
// CG: the partials were written by other CTAs of the running kernel, so
// they are read through L2 (ld.global.cg), never from a stale L1 line.
template <bool CG = false>
__device__ double prob_sum(const double* v, int stride, int off, const int* chunk_off, int p,
                           double* red) {
  double s = 0.0;
  for (int c = chunk_off[p] + threadIdx.x; c < chunk_off[p + 1]; c += blockDim.x)
    s += CG ? __ldcg(v + (long long)stride * c + off) : v[(long long)stride * c + off];
  return block_sum(s, red);
}

// The first NF fields of a problem's chunk partials (stride fields per
// chunk) summed in one pass: each thread walks its chunks with NF loads per
// chunk, four chunks in flight, then fixed-shape trees.  Results in thread 0.
template <int NF, bool CG = false>
__device__ void prob_sums(const double* v, int stride, const int* chunk_off, int p, double* red,
                          double* out) {
  double s[NF];
#pragma unroll
  for (int f = 0; f < NF; ++f) s[f] = 0.0;
  const int c0 = chunk_off[p], c1 = chunk_off[p + 1];
#pragma unroll 4
  for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
#pragma unroll
    for (int f = 0; f < NF; ++f)
      s[f] += CG ? __ldcg(v + (long long)stride * c + f) : v[(long long)stride * c + f];
  }
#pragma unroll
  for (int f = 0; f < NF; ++f) out[f] = block_sum(s[f], red);
}

// LM control: one CTA per problem (kCtrlThreads), thread 0 decides.
constexpr int kCtrlThreads = 256;

__global__ void __launch_bounds__(kCtrlThreads) k_ctrl_initial_cost(DevPlan d) {
  __shared__ double red[32];
  const int p = blockIdx.x;
  LMState& st = d.state[p];
  if (!st.active) return;
  double fr[2];
  prob_sums<2>(d.key_chunk_sum, 2, d.prob_key_chunk_off, p, red, fr);
  if (threadIdx.x != 0) return;
  double F = fr[0];
  const double raw = fr[1];
  if (d.cons_cost) F += d.cons_cost[p];
  st.F = F;
  st.raw = raw;
  st.initial_cost = F;
  if (!isfinite(F)) {
    st.status = GBA_ERR_NAN;
    st.stop = GBA_STOP_ERROR;
    st.active = 0;
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
}

// The LM step decision of problem p from the back-substitution's partial
// sums (every thread of the CTA takes part; thread 0 decides).  Run by
// k_ctrl_step, or (CG = true) by the last CTA of k_backsub to finish for p.
template <bool CG>
__device__ void ctrl_step_body(const DevPlan& d, int p, double* red) {
  LMState& st = d.state[p];
  if (!st.active) return;
  const bool failed = d.factor_flag[p] != 0;
  double dn2 = 0, xn2 = 0, gd = 0, er = 0;
  if (!failed) {
    double sp[3], si[3];
    prob_sums<3, CG>(d.pt_chunk_sum, 3, d.prob_pt_chunk_off, p, red, sp);
    prob_sums<3, CG>(d.img_chunk_sum, 3, d.prob_img_chunk_off, p, red, si);
    dn2 = sp[0] + si[0];
    xn2 = sp[1] + si[1];
    gd = sp[2] + si[2];
    // PCG leaves the image rows with residual r: the model decrease gains r^T delta_i
    if (d.pcg) er = prob_sum<CG>(d.pcg_part, kPcgSlots, 6, d.prob_ext_chunk_off, p, red);
    if (d.free_cams) {
      double sc[3];
      prob_sums<3, CG>(d.cam_sum, 3, d.prob_cam_off, p, red, sc);
      dn2 += sc[0];
      xn2 += sc[1];
      gd += sc[2];
    }
  }
  if (threadIdx.x != 0) return;
  st.iter += 1;
  st.evaluate = 0;
  if (d.factor_flag[p] == 2) {        // a bounded wait of the factorization ran out
    st.active = 0;
    st.stop = GBA_STOP_ERROR;
    st.status = GBA_ERR_TIMEOUT;
    return;
  }
  // the flag is consumed: cleared here (the next iteration's point factor
  // may run beside the previous linearization's control, so not there)
  d.factor_flag[p] = 0;
  if (failed) {
    st.factor_fail += 1;
    st.rejected += 1;
    st.mu *= st.nu;
    st.nu *= 2.0;
  } else {
    st.dn2 = dn2;
    st.xn2 = xn2;
    st.gd = gd;
    st.er = er;
    if (sqrt(dn2) <= d.eps2 * (sqrt(xn2) + d.eps2)) {
      st.active = 0;
      st.stop = GBA_STOP_SMALL_STEP;
    } else {
      st.evaluate = 1;
    }
  }
}

__global__ void __launch_bounds__(kCtrlThreads) k_ctrl_step(DevPlan d) {
  __shared__ double red[32];
  ctrl_step_body<false>(d, blockIdx.x, red);
}

// The LM accept / reject decision of problem p from the candidate cost's
// partial sums.  Run by k_ctrl_accept, or (CG = true) by the last CTA of the
// candidate cost kernel to finish for p.
template <bool CG>
__device__ void ctrl_accept_body(const DevPlan& d, int p, double* red) {
  LMState& st = d.state[p];
  if (!st.evaluate) return;
  double fr[2];
  prob_sums<2, CG>(d.key_chunk_sum, 2, d.prob_key_chunk_off, p, red, fr);
  if (threadIdx.x != 0) return;
  double Fn = fr[0];
  const double raw_n = fr[1];
  if (d.cons_cost) Fn += d.cons_cost[p];
  st.evaluate = 0;
  st.F_new = Fn;
  // predicted decrease of the quadratic model, 2 g^T d - d^T N d, written
  // with (N + mu I) d = g - e (e = 0 for the exact factorization)
  const double denom = st.mu * st.dn2 + st.gd + st.er;
  const double rho = (st.F - Fn) / denom;
  if (isfinite(Fn) && denom > 0.0 && rho > 0.0) {
    if (d.ftol > 0.0 && st.F - Fn <= d.ftol * st.F) {   // Ceres' function tolerance
      st.active = 0;
      st.stop = GBA_STOP_SMALL_COST_CHANGE;
    }
    st.parity ^= 1;
    st.F = Fn;
    st.raw = raw_n;
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

__global__ void __launch_bounds__(kCtrlThreads) k_ctrl_accept(DevPlan d) {
  __shared__ double red[32];
  ctrl_accept_body<false>(d, blockIdx.x, red);
}

// The observed keys as double-float pairs (hi = float(v), lo = float(v - hi)).
__global__ void k_split_keys(DevPlan d, float2* out) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const double2 o = d.key_obs[k];
  out[2 * k] = ff_split(o.x);
  out[2 * k + 1] = ff_split(o.y);
}

// The current x of every problem (each in its own parity; x0 before a run)
// gathered into out = [points 3P][images 6I][cameras 10 Ctot].
__global__ void k_gather_x(DevPlan d, int ran, double* out) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long np = 3LL * d.P, ni = 6LL * d.I, nc = d.free_cams ? 10LL * d.Ctot : 0;
  if (e < np) {
    const int par = d.state[d.pt_prob[e / 3]].parity;
    out[e] = ran ? d.x_pt[par][e] : d.x0_pt[e];
  } else if (e < np + ni) {
    const long long f = e - np;
    const int par = d.state[d.img_prob[f / 6]].parity;
    out[e] = ran ? d.x_img[par][f] : d.x0_img[f];
  } else if (e < np + ni + nc) {
    const long long f = e - np - ni;
    const int par = d.state[d.cam_info[f / 10].z].parity;
    out[e] = ran ? d.x_cam[par][f] : d.x0_cam[f];
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
  for (int j = 0; j < 10; ++j) cam[j] = d.cam64[par][10 * d.img_cam[img] + j];
  double u, v;
  project64(R, X, cam, u, v);
  y[2LL * k] = u;
  y[2LL * k + 1] = v;
}

template <typename T>
__global__ void k_jacobian_out(DevPlan d, double* jp_out, double* ji_out, double* jc_out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= d.K) return;
  const int img = d.key_img[k], pt = d.key_pt[k];
  const int par = d.state[d.img_prob[img]].parity;
  const double* xp = d.x_pt[par] + 3LL * pt;
  const T X[3] = {T(xp[0]), T(xp[1]), T(xp[2])};
  T il[12];
  for (int j = 0; j < 12; ++j) il[j] = tptr<T>(d.img_lin[par])[12LL * img + j];
  T cam[10];
  load_cam<T>(d, par, d.img_cam[img], cam);
  T jp[6], ji[12], nrm[2];
  key_jacobian<T>(X, il, cam, jp, ji, nrm);
  for (int j = 0; j < 6; ++j) jp_out[6LL * k + j] = double(jp[j]);
  for (int j = 0; j < 12; ++j) ji_out[12LL * k + j] = double(ji[j]);
  if (jc_out) {   // all ten columns; the host keeps the computed ones
    T jc[20];
    camera_jacobian<T>(nrm[0], nrm[1], cam, jc);
    for (int j = 0; j < 20; ++j) jc_out[20LL * k + j] = double(jc[j]);
  }
}

template <typename T>
int run_cholesky_factor(const DevPlan& d, cudaStream_t s) {
  if (d.chol_small) {   // factor and solve in one launch (small systems, FP32)
    if constexpr (sizeof(T) == sizeof(float))
      k_chol_small<T><<<dim3(1u, unsigned(d.B)), kCholThreads, chol_small_smem<T>(d.max_nt), s>>>(d);
    return 1;
  }
  if (d.df_grid > 0) {
    if (d.df_trace)
      cudaMemsetAsync(d.df_trace, 0, sizeof(unsigned long long) * 4 * kDfTraceCap * size_t(d.df_grid), s);
    DevPlan dd = d;
    void* args[] = {&dd};
    const cudaError_t e = cudaLaunchCooperativeKernel(
        reinterpret_cast<const void*>(&k_chol_dataflow<T>), dim3(unsigned(d.df_grid)),
        dim3(kDfThreads), args, df_smem_bytes<T>(d.df_max_own), s);
    if (e != cudaSuccess) {
      std::fprintf(stderr, "gba: k_chol_dataflow launch failed: %s\n", cudaGetErrorString(e));
      throw CudaError{GBA_ERR_CUDA};
    }
    return 1;
  }
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
  if (d.chol_small) return 0;   // done by k_chol_small
  if (d.max_nt <= kSolveSmallTiles)
    k_chol_solve_small<T><<<dim3(1u, unsigned(d.B)), 256, 0, s>>>(d);
  else if (d.solve_drop_step >= 0 || d.solve_spin_limit != kSolveSpin)
    k_chol_solve<T, true><<<dim3(unsigned(kSolveRanks), unsigned(d.B)), 256, solve_smem_bytes<T>(d.max_nt), s>>>(d);
  else
    k_chol_solve<T, false><<<dim3(unsigned(kSolveRanks), unsigned(d.B)), 256, solve_smem_bytes<T>(d.max_nt), s>>>(d);
  return 1;
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
  long long tot = 3LL * d.P + 6LL * d.I + (d.free_cams ? 10LL * d.Ctot : 0);
  if (tot > 0) {
    k_copy_x0<<<int((tot + 255) / 256), 256, 0, s>>>(d);
    return 2;
  }
  return 1;
}

int launch_image_prep(const DevPlan& d, int which, cudaStream_t s) {
  int n = 0;
  if (d.free_cams && d.Ctot > 0) {
    k_cam_prep<<<(d.Ctot + 127) / 128, 128, 0, s>>>(d, which);
    ++n;
  }
  // the candidate's image rotations come from k_backsub
  if (d.I <= 0 || which == 1) return n;
  GBA_DISPATCH(d, run_image_prep<T>(d, which, s));
  return n + 1;
}

int launch_cost(const DevPlan& d, int which, cudaStream_t s) {
  int n = 0;
  // constraint and prior terms first: the accept decision folded into the
  // key cost kernel adds them
  if (d.n_cons > 0 || d.n_priors > 0) {
    k_cons_cost<<<d.B, 256, 0, s>>>(d, which);
    ++n;
  }
  if (d.n_key_chunks > 0) {
    if (d.precision == GBA_PRECISION_MIXED)
      k_cost_ff<<<d.n_key_chunks, 256, 0, s>>>(d, which);
    else
      k_cost<double><<<d.n_key_chunks, 256, 0, s>>>(d, which);
    ++n;
  }
  return n;
}

int launch_ctrl_initial_cost(const DevPlan& d, cudaStream_t s) {
  k_ctrl_initial_cost<<<d.B, kCtrlThreads, 0, s>>>(d);
  return 1;
}

int launch_linearize(const DevPlan& d, cudaStream_t s, bool keys) {
  int n = 0;
  if (keys && d.n_key_chunks > 0) {
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
  if (!d.free_cams) return 2;
  GBA_DISPATCH(d, (k_image_cam_reduce<T><<<d.n_img_items, 128, 0, s>>>(d)));
  k_image_cam_finalize<<<d.I, kImgCamVals, 0, s>>>(d);
  k_cam_finalize<<<d.Ctot, kImgCamVals * kCamGroups, 0, s>>>(d);
  return 5;
}

int launch_ctrl_after_linearize(const DevPlan& d, cudaStream_t s) {
  k_ctrl_after_linearize<<<(d.B + 127) / 128, 128, 0, s>>>(d);
  return 1;
}

int launch_z_slots(const DevPlan& d, int* key_slot, cudaStream_t s) {
  int n = 0;
  if (d.K > 0) {
    k_key_slots<<<(d.K + 255) / 256, 256, 0, s>>>(d.img_keys, d.K, key_slot);
    ++n;
  }
  if (d.n_items > 0) {
    k_pairs_to_slots<<<(d.n_items + 3) / 4, 128, 0, s>>>(d.items, d.n_items, d.blk_ij, key_slot, d.K,
                                                        const_cast<int2*>(d.pairs));
    ++n;
  }
  return n;
}

int launch_point_schur(const DevPlan& d, cudaStream_t s) {
  int n = 0;
  if (d.n_pt_chunks > 0) {
    GBA_DISPATCH(d, (k_point_factor<T><<<d.n_pt_chunks, kPointChunk, 0, s>>>(d)));
    ++n;
  }
  if (d.n_key_chunks > 0) {
    GBA_DISPATCH(d, (k_key_z<T><<<d.n_key_chunks * d.key_z_split, 256, 0, s>>>(d)));
    ++n;
  }
  if (d.free_cams && d.R > 0) {
    GBA_DISPATCH(d, (k_camrec_z<T><<<d.n_pt_chunks, kPointChunk, 0, s>>>(d)));
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
  if (d.blk_prob && d.n_blocks > 0) {
    const size_t tsz = d.precision == GBA_PRECISION_MIXED ? sizeof(float) : sizeof(double);
    if (cudaMemsetAsync(d.S, 0, size_t(d.s_elems) * tsz, s) != cudaSuccess) throw CudaError{GBA_ERR_CUDA};
    const unsigned g = unsigned((36LL * d.n_blocks + 255) / 256);
    GBA_DISPATCH(d, (k_assemble_S_blocks<T><<<g, 256, 0, s>>>(d)));
    return 1;
  }
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

int prepare_cholesky_solve(int max_nt, int precision) {
  if (max_nt <= kSolveSmallTiles) return GBA_OK;
  const bool mixed = precision == GBA_PRECISION_MIXED;
  const size_t bytes = mixed ? solve_smem_bytes<float>(max_nt) : solve_smem_bytes<double>(max_nt);
  if (bytes <= 48 * 1024) return GBA_OK;
  const void* f[2] = {mixed ? reinterpret_cast<const void*>(&k_chol_solve<float, false>)
                            : reinterpret_cast<const void*>(&k_chol_solve<double, false>),
                      mixed ? reinterpret_cast<const void*>(&k_chol_solve<float, true>)
                            : reinterpret_cast<const void*>(&k_chol_solve<double, true>)};
  for (const void* fn : f)
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)) != cudaSuccess) {
      cudaGetLastError();
      return GBA_ERR_UNSUPPORTED;
    }
  return GBA_OK;
}

bool prepare_chol_small(int max_nt, int precision) {
  if (precision != GBA_PRECISION_MIXED || max_nt < 1 || max_nt > kSolveSmallTiles) return false;
  const size_t bytes = chol_small_smem<float>(max_nt);
  if (bytes > 48 * 1024 &&
      cudaFuncSetAttribute(&k_chol_small<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)) !=
          cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

int launch_cholesky_solve(const DevPlan& d, cudaStream_t s) {
  if (d.max_nt <= 0) return 0;
  int n = 0;
  GBA_DISPATCH(d, n = run_cholesky_solve<T>(d, s));
  return n;
}

template <typename T>
bool dataflow_layout_t(int nt, int device, int* grid, int* max_own, std::vector<int>* own_off,
                       std::vector<int2>* own) {
  int sms = 0, coop = 0, optin = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (!coop || nt < 2) return false;
  const long long ntiles = (long long)nt * (nt + 1) / 2;
  const int G = int(std::min<long long>(sms, ntiles));
  // row i's diagonal tile and its left neighbour go to CTA i mod G; the
  // rest, heaviest first, to the CTA with the least work so far.  When
  // there are at least twice as many CTAs as tile rows, the chain's CTAs
  // take none of the rest: a CTA busy with an update when its row's chain
  // task becomes ready would delay the chain by that update
  std::vector<std::vector<int2>> lists(G);
  const int first_worker = (G >= 2 * nt) ? nt : 0;
  std::vector<long long> load(G, 0);
  for (int i = 0; i < nt; ++i) {
    const int g = i % G;
    lists[g].push_back(make_int2(i, i));
    load[g] += i + 1;
    if (i > 0) {
      lists[g].push_back(make_int2(i, i - 1));
      load[g] += i;
    }
  }
  std::vector<int2> rest;
  for (int j = 0; j < nt; ++j)
    for (int i = j + 2; i < nt; ++i) rest.push_back(make_int2(i, j));
  std::stable_sort(rest.begin(), rest.end(), [](const int2& a, const int2& b) { return a.y > b.y; });
  for (const int2& t : rest) {
    int g = first_worker;
    for (int h = first_worker + 1; h < G; ++h)
      if (load[h] < load[g]) g = h;
    lists[g].push_back(t);
    load[g] += t.y + 1;
  }
  int mo = 0;
  for (auto& l : lists) {
    std::sort(l.begin(), l.end(), [](const int2& a, const int2& b) {
      return a.y != b.y ? a.y < b.y : a.x < b.x;
    });
    mo = std::max(mo, int(l.size()));
  }
  const size_t smem = df_smem_bytes<T>(mo);
  if (smem > size_t(optin) || mo > kDfThreads) return false;
  if (cudaFuncSetAttribute(reinterpret_cast<const void*>(&k_chol_dataflow<T>),
                           cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chol_dataflow<T>, kDfThreads, smem) !=
          cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return false;
  }
  own_off->assign(1, 0);
  own->clear();
  for (auto& l : lists) {
    own->insert(own->end(), l.begin(), l.end());
    own_off->push_back(int(own->size()));
  }
  *grid = G;
  *max_own = mo;
  return true;
}

bool dataflow_layout(int nt, bool mixed, int device, int* grid, int* max_own,
                     std::vector<int>* own_off, std::vector<int2>* own) {
  return mixed ? dataflow_layout_t<float>(nt, device, grid, max_own, own_off, own)
               : dataflow_layout_t<double>(nt, device, grid, max_own, own_off, own);
}

int launch_assemble_blocks(const DevPlan& d, cudaStream_t s) {
  if (d.n_blocks <= 0) return 0;
  const long long n = 36LL * d.n_blocks;
  GBA_DISPATCH(d, (k_assemble_blocks<T><<<unsigned((n + 255) / 256), 256, 0, s>>>(d)));
  return 1;
}

int launch_pcg_setup(const DevPlan& d, cudaStream_t s) {
  if (d.I_ext <= 0) return 0;
  GBA_DISPATCH(d, (k_pcg_precond<T><<<(d.I_ext + 127) / 128, 128, 0, s>>>(d)));
  GBA_DISPATCH(d, (k_pcg_init<T><<<d.n_ext_chunks, 256, 0, s>>>(d)));
  return 2;
}

int launch_pcg_iterations(const DevPlan& d, cudaStream_t s) {
  if (d.I_ext <= 0) return 0;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (d.pcg_it && d.pcg_body_stream && cudaStreamIsCapturing(s, &cs) == cudaSuccess &&
      cs == cudaStreamCaptureStatusActive) {
    // in a CUDA graph: a while node whose body runs two iterations and the
    // loop control, so the iterations after convergence are not launched
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    cudaGraphConditionalHandle h = 0;
    cudaGraphNodeParams cp = {};
    cudaGraphNode_t node = nullptr;
    if (cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd) != cudaSuccess ||
        cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess)
      throw CudaError{GBA_ERR_CUDA};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if (cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp) != cudaSuccess) throw CudaError{GBA_ERR_CUDA};
    cudaStream_t bs = d.pcg_body_stream;
    if (cudaStreamBeginCaptureToGraph(bs, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      throw CudaError{GBA_ERR_CUDA};
    for (int u = 0; u < 2; ++u) {
      GBA_DISPATCH(d, (k_pcg_spmv<T><<<d.n_ext_chunks, 256, 0, bs>>>(d, u, 1)));
      GBA_DISPATCH(d, (k_pcg_update<T><<<d.n_ext_chunks, 256, 0, bs>>>(d, u, 1)));
    }
    k_pcg_loop_ctrl<<<1, 32, 0, bs>>>(d, h);
    cudaGraph_t body = nullptr;
    if (cudaStreamEndCapture(bs, &body) != cudaSuccess ||
        cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
      throw CudaError{GBA_ERR_CUDA};
    return 5;   // (one pass of the body; it runs as many passes as the solve needs)
  }
  for (int it = 0; it < d.pcg_max_iterations; ++it) {
    GBA_DISPATCH(d, (k_pcg_spmv<T><<<d.n_ext_chunks, 256, 0, s>>>(d, it, 0)));
    GBA_DISPATCH(d, (k_pcg_update<T><<<d.n_ext_chunks, 256, 0, s>>>(d, it, 0)));
  }
  return 2 * d.pcg_max_iterations;
}

int launch_cholesky(const DevPlan& d, cudaStream_t s) {
  return launch_cholesky_factor(d, s) + launch_cholesky_solve(d, s);
}

int launch_backsub(const DevPlan& d, cudaStream_t s) {
  const int g = d.n_pt_chunks + d.n_img_chunks;
  if (g <= 0) return 0;
  int n = 0;
  // the cameras' step first: with the control folded into k_backsub, its
  // last CTA reads the cameras' partial sums too
  if (d.free_cams && d.Ctot > 0) {
    GBA_DISPATCH(d, (k_cam_backsub<T><<<(d.Ctot + 127) / 128, 128, 0, s>>>(d)));
    ++n;
  }
  GBA_DISPATCH(d, (k_backsub<T><<<g, kPointChunk, 0, s>>>(d)));
  return n + 1;
}

int launch_ctrl_step(const DevPlan& d, cudaStream_t s) {
  if (d.fold_ctrl) return 0;   // done by the last CTA of each problem in k_backsub
  k_ctrl_step<<<d.B, kCtrlThreads, 0, s>>>(d);
  return 1;
}

int launch_ctrl_accept(const DevPlan& d, cudaStream_t s) {
  if (d.fold_ctrl) return 0;   // done by the last CTA of each problem in the candidate cost
  k_ctrl_accept<<<d.B, kCtrlThreads, 0, s>>>(d);
  return 1;
}

int launch_vector_function(const DevPlan& d, double* y, cudaStream_t s) {
  if (d.K <= 0) return 0;
  k_vector_function<<<(d.K + 255) / 256, 256, 0, s>>>(d, y);
  return 1;
}

int launch_split_keys(const DevPlan& d, float2* out, cudaStream_t s) {
  if (d.K <= 0) return 0;
  k_split_keys<<<unsigned((d.K + 255) / 256), 256, 0, s>>>(d, out);
  return 1;
}

int launch_gather_x(const DevPlan& d, int ran, double* out, cudaStream_t s) {
  const long long n = 3LL * d.P + 6LL * d.I + (d.free_cams ? 10LL * d.Ctot : 0);
  if (n <= 0) return 0;
  k_gather_x<<<unsigned((n + 255) / 256), 256, 0, s>>>(d, ran, out);
  return 1;
}

int launch_jacobian_out(const DevPlan& d, double* jp, double* ji, double* jc, cudaStream_t s) {
  if (d.K <= 0) return 0;
  GBA_DISPATCH(d, (k_jacobian_out<T><<<(d.K + 255) / 256, 256, 0, s>>>(d, jp, ji, jc)));
  return 1;
}

// ===========================================================================
// Key pairs of the Schur complement built on the device (plans without free
// cameras).  Problem q's image pairs (a, c), a <= c local images, have the
// codes first_code(q) + a * Ie + c; the problems' code ranges follow each
// other, so code order is the host's block order of the concatenated plan.
// The device counts the pairs of every code (atomics), marks the blocks
// (codes with pairs, and every diagonal), numbers them and their first pairs
// by exclusive scans, and returns the block list.  Every point then writes
// its pairs (a <= c over its keys, point-major) with their block id, and a
// stable LSD radix sort by block id leaves each block's pairs in point order
// -- the same list, in the same order, as the host build's placement.
// Problem records pinfo[q] = (first image, Ie, first code, 0).
// ===========================================================================
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortPerThread = 8;
constexpr int kSortTile = kSortThreads * kSortPerThread;   // elements per tile
constexpr int kScanChunk = 4096;                             // per scan CTA (1024 x 4)
constexpr int kScanTop = 8192;                               // chunk totals one CTA scans

// Pairs per code: one thread per point, one atomic per key pair (keys of a
// point are in image order).
__global__ void __launch_bounds__(128) k_count_pairs(int P, const int* __restrict__ pt_key_off,
                                                     const int* __restrict__ key_img,
                                                     const int* __restrict__ pt_prob,
                                                     const int4* __restrict__ pinfo, int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const int4 pq = pinfo[pt_prob[i]];
  const int k0 = pt_key_off[i], k1 = pt_key_off[i + 1];
  for (int a = k0; a < k1; ++a) {
    const long long row = pq.z + (long long)(key_img[a] - pq.x) * pq.y;
    for (int c = a; c < k1; ++c) atomicAdd(cnt + row + (key_img[c] - pq.x), 1);
  }
}

// Pairs of each point, k (k + 1) / 2; entry P is 0 (the scan makes it the total).
__global__ void __launch_bounds__(256) k_point_pairs(int P, const int* __restrict__ pt_key_off,
                                                     int* __restrict__ pp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > P) return;
  int v = 0;
  if (i < P) {
    const int k = pt_key_off[i + 1] - pt_key_off[i];
    v = k * (k + 1) / 2;
  }
  pp[i] = v;
}

// A block for every image pair a < c with pairs and for every diagonal
// (a == c, even without keys).
__device__ __forceinline__ bool block_present(int local, int Ie, int count) {
  const int a = local / Ie, c = local - a * Ie;
  return a == c || (c > a && count > 0);
}

// grid (codes of the largest problem / 256, problems)
__global__ void __launch_bounds__(256) k_block_marks(const int4* __restrict__ pinfo, const int* __restrict__ cnt,
                                                     int* __restrict__ mark, int* __restrict__ off) {
  const int4 pq = pinfo[blockIdx.y];
  const int local = blockIdx.x * blockDim.x + threadIdx.x;
  if (local >= pq.y * pq.y) return;
  const int e = pq.z + local;
  const int v = cnt[e];
  mark[e] = block_present(local, pq.y, v) ? 1 : 0;
  off[e] = v;
}

// After the scans: bid[e] = the block id (or -1); the block list (local
// code, first pair) in block order; each problem's first block (its block
// (0, 0) is always present); info = (blocks, pairs) from the last code of
// problem qlast (the last with images: its block (Ie-1, Ie-1)).
__global__ void __launch_bounds__(256) k_block_lists(const int4* __restrict__ pinfo, int qlast,
                                                     const int* __restrict__ cnt, int* __restrict__ bid,
                                                     const int* __restrict__ off, int* __restrict__ blk_code,
                                                     int* __restrict__ blk_first, int* __restrict__ prob_block,
                                                     int* __restrict__ info) {
  const int q = blockIdx.y;
  const int4 pq = pinfo[q];
  const int local = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = pq.y * pq.y;
  if (local >= L) return;
  const int e = pq.z + local;
  const int v = cnt[e];
  const bool m = block_present(local, pq.y, v);
  const int b = bid[e];
  if (m) {
    blk_code[b] = local;
    blk_first[b] = off[e];
  }
  bid[e] = m ? b : -1;
  if (local == 0) prob_block[q] = b;
  if (q == qlast && local == L - 1) {
    info[0] = b + 1;
    info[1] = off[e] + v;
  }
}

__global__ void __launch_bounds__(128) k_enumerate_pairs(int P, const int* __restrict__ pt_key_off,
                                                         const int* __restrict__ key_img,
                                                         const int* __restrict__ pt_prob,
                                                         const int4* __restrict__ pinfo,
                                                         const int* __restrict__ pp_off,
                                                         const int* __restrict__ bid, int* __restrict__ keys,
                                                         int2* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P) return;
  const int4 pq = pinfo[pt_prob[i]];
  const int k0 = pt_key_off[i], k1 = pt_key_off[i + 1];
  int pos = pp_off[i];
  for (int a = k0; a < k1; ++a) {
    const long long row = pq.z + (long long)(key_img[a] - pq.x) * pq.y;
    for (int c = a; c < k1; ++c, ++pos) {
      keys[pos] = bid[row + (key_img[c] - pq.x)];
      // a pair of a diagonal block is a key with itself: carry its point instead
      vals[pos] = make_int2(a, a == c ? i : c);
    }
  }
}

// Per tile, the count of each 8-bit digit of the keys (digit-major output).
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const int* __restrict__ keys, long long n, int shift,
                                                               int ntiles, int* __restrict__ hist) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long t0 = (long long)blockIdx.x * kSortTile;
#pragma unroll
  for (int j = 0; j < kSortPerThread; ++j) {
    const long long e = t0 + (long long)j * kSortThreads + threadIdx.x;
    if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255], 1);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of v [n] in chunks of kScanChunk: each CTA scans its chunk
// and writes the chunk total to sums.
__global__ void __launch_bounds__(1024) k_scan_chunks(int* __restrict__ v, long long n, int* __restrict__ sums) {
  __shared__ int wsum[32];
  const long long base = (long long)blockIdx.x * kScanChunk + 4LL * threadIdx.x;
  int x[4], t = 0;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    x[u] = base + u < n ? v[base + u] : 0;
    t += x[u];
  }
  // inclusive scan of the thread totals across the CTA
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    int ws = wsum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += y;
    }
    wsum[lane] = ws;   // inclusive over warps
  }
  __syncthreads();
  int run = inc - t + (w > 0 ? wsum[w - 1] : 0);   // exclusive prefix of this thread
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    if (base + u < n) v[base + u] = run;
    run += x[u];
  }
  if (threadIdx.x == 1023) sums[blockIdx.x] = run;
}

// Exclusive scan of the chunk totals (at most 8192) in one CTA.
__global__ void __launch_bounds__(1024) k_scan_totals(int* __restrict__ sums, int m) {
  __shared__ int part[1024];
  const int per = (m + 1023) / 1024;
  const int b = threadIdx.x * per;
  int t = 0;
  for (int u = 0; u < per; ++u)
    if (b + u < m) t += sums[b + u];
  part[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {   // 1024 values: serial in one thread, fixed order
    int run = 0;
    for (int u = 0; u < 1024; ++u) {
      const int y = part[u];
      part[u] = run;
      run += y;
    }
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int u = 0; u < per; ++u)
    if (b + u < m) {
      const int y = sums[b + u];
      sums[b + u] = run;
      run += y;
    }
}

__global__ void __launch_bounds__(1024) k_scan_add(int* __restrict__ v, long long n, const int* __restrict__ sums) {
  const long long base = (long long)blockIdx.x * kScanChunk + 4LL * threadIdx.x;
  const int add = sums[blockIdx.x];
#pragma unroll
  for (int u = 0; u < 4; ++u)
    if (base + u < n) v[base + u] += add;
}

// Stable scatter of one tile by the digit at `shift`: elements are ranked in
// tile order (256 at a time, warp by warp, lane by lane).  A position outside
// [0, n) is not written and raises *bad.
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const int* __restrict__ keys,
                                                                  const int2* __restrict__ vals, long long n,
                                                                  int shift, int ntiles,
                                                                  const int* __restrict__ offs,
                                                                  int* __restrict__ okeys,
                                                                  int2* __restrict__ ovals, int* bad) {
  __shared__ int base[256], run[256], wc[kSortThreads / 32][256];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  base[t] = offs[(long long)t * ntiles + blockIdx.x];
  run[t] = 0;
  const long long t0 = (long long)blockIdx.x * kSortTile;
  for (int j = 0; j < kSortPerThread; ++j) {
#pragma unroll
    for (int ww = 0; ww < kSortThreads / 32; ++ww) wc[ww][t] = 0;
    __syncthreads();
    const long long e = t0 + (long long)j * kSortThreads + t;
    const bool valid = e < n;
    const int key = valid ? keys[e] : 0;
    const int dgt = valid ? (key >> shift) & 255 : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, dgt);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && rank == 0) wc[w][dgt] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pos = base[dgt] + run[dgt] + rank;
      for (int ww = 0; ww < w; ++ww) pos += wc[ww][dgt];
      if (pos >= 0 && (long long)pos < n) {
        okeys[pos] = key;
        ovals[pos] = vals[e];
      } else {
        atomicExch(bad, 1);
      }
    }
    __syncthreads();
    int add = 0;
#pragma unroll
    for (int ww = 0; ww < kSortThreads / 32; ++ww) add += wc[ww][t];
    run[t] += add;
    __syncthreads();
  }
}

// Exclusive scan of v [L] in place: chunks of kScanChunk, their totals
// scanned the same way (one CTA once there are at most kScanTop of them).
// scratch holds scan_scratch_ints(L) ints.
int scan_exclusive(int* v, long long L, int* scratch, cudaStream_t s) {
  if (L <= 0) return 0;
  const long long nchunks = (L + kScanChunk - 1) / kScanChunk;
  k_scan_chunks<<<unsigned(nchunks), 1024, 0, s>>>(v, L, scratch);
  int n = 1;
  if (nchunks <= kScanTop) {
    k_scan_totals<<<1, 1024, 0, s>>>(scratch, int(nchunks));
    ++n;
  } else {
    n += scan_exclusive(scratch, nchunks, scratch + nchunks, s);
  }
  k_scan_add<<<unsigned(nchunks), 1024, 0, s>>>(v, L, scratch);
  return n + 1;
}

}  // namespace

long long scan_scratch_ints(long long L) {
  long long t = 0;
  while (L > 0) {
    const long long c = (L + kScanChunk - 1) / kScanChunk;
    t += c;
    if (c <= kScanTop) break;
    L = c;
  }
  return std::max<long long>(t, 1);
}

int count_blocks_on_device(int nprob, int qlast, int max_ie, int P, const int4* d_pinfo, const int* d_pt_key_off,
                           const int* d_key_img, const int* d_pt_prob, long long L, int* d_cnt, int* d_bid,
                           int* d_off, int* d_scratch, int* d_blk_code, int* d_blk_first, int* d_prob_block,
                           int* d_info, cudaStream_t s) {
  int launches = 0;
  if (L <= 0 || nprob <= 0 || nprob > 65535) return -1;
  if (cudaMemsetAsync(d_cnt, 0, sizeof(int) * size_t(L), s) != cudaSuccess) return -1;
  if (P > 0) {
    k_count_pairs<<<unsigned((P + 127) / 128), 128, 0, s>>>(P, d_pt_key_off, d_key_img, d_pt_prob, d_pinfo, d_cnt);
    ++launches;
  }
  const dim3 g(unsigned(((long long)max_ie * max_ie + 255) / 256), unsigned(nprob));
  k_block_marks<<<g, 256, 0, s>>>(d_pinfo, d_cnt, d_bid, d_off);
  launches += 1 + scan_exclusive(d_bid, L, d_scratch, s) + scan_exclusive(d_off, L, d_scratch, s);
  k_block_lists<<<g, 256, 0, s>>>(d_pinfo, qlast, d_cnt, d_bid, d_off, d_blk_code, d_blk_first, d_prob_block,
                                  d_info);
  return launches + 1;
}

int build_pairs_on_device(int P, int nblocks, const int4* d_pinfo, const int* d_pt_key_off, const int* d_key_img,
                          const int* d_pt_prob, int* d_pp, const int* d_bid, long long n, int* d_keys0,
                          int2* d_vals0, int* d_keys1, int2* d_vals1, int* d_hist, int* d_scratch, int* d_bad,
                          int2** out, cudaStream_t s) {
  int launches = 0;
  if (P > 0) {
    k_point_pairs<<<unsigned((P + 256) / 256), 256, 0, s>>>(P, d_pt_key_off, d_pp);
    launches += 1 + scan_exclusive(d_pp, (long long)P + 1, d_scratch, s);
    k_enumerate_pairs<<<unsigned((P + 127) / 128), 128, 0, s>>>(P, d_pt_key_off, d_key_img, d_pt_prob, d_pinfo,
                                                                  d_pp, d_bid, d_keys0, d_vals0);
    ++launches;
  }
  int bits = 1;
  while (bits < 31 && (1LL << bits) < nblocks) ++bits;
  const int passes = (bits + 7) / 8;
  const int ntiles = int((n + kSortTile - 1) / kSortTile);
  const long long L = 256LL * ntiles;
  int* kin = d_keys0;
  int2* vin = d_vals0;
  int* kout = d_keys1;
  int2* vout = d_vals1;
  for (int pass = 0; pass < passes && n > 0; ++pass) {
    const int shift = 8 * pass;
    k_radix_hist<<<unsigned(ntiles), kSortThreads, 0, s>>>(kin, n, shift, ntiles, d_hist);
    launches += 2 + scan_exclusive(d_hist, L, d_scratch, s);
    k_radix_scatter<<<unsigned(ntiles), kSortThreads, 0, s>>>(kin, vin, n, shift, ntiles, d_hist, kout, vout,
                                                              d_bad);
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  *out = vin;
  return launches;
}

void pairs_sort_scratch(long long n, int P, long long* hist_ints, long long* scratch_ints) {
  const long long ntiles = (n + kSortTile - 1) / kSortTile;
  *hist_ints = 256LL * std::max<long long>(ntiles, 1);
  *scratch_ints = std::max(scan_scratch_ints(*hist_ints), scan_scratch_ints((long long)P + 1));
}

}  // namespace gba
