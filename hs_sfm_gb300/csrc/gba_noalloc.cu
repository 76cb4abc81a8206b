// gba_noalloc.cu -- gba_cost_noalloc(): the reprojection cost of a problem
// whose arrays already live in device memory, computed without allocating.
//
// Who needs it: callers that must not call cudaMalloc -- a plugin running
// inside a host application that owns every device allocation (a memory pool
// or an arena it accounts for), code paths between a framework's allocator
// teardown and process exit, or hosts that forbid device allocations after
// start-up.  The caller passes device pointers for every input and for the
// output; the temporaries of the computation (one rotation matrix per image,
// one partial sum per block and a count of rejected keys) live in the fixed
// array g_noalloc_scratch below, which every GPU that loads libgba.so holds
// until the process exits.
//
// Limits and sharing rules:
//   - at most GBA_NOALLOC_MAX_IMAGES images per call; larger problems are
//     rejected with GBA_ERR_INVALID before anything is launched;
//   - every call on a device uses the same scratch array, and it keeps the
//     last call's contents.  Calls whose kernels overlap on the GPU (two
//     streams, or two host threads) race on it: serialize them;
//   - every call looks up the scratch array's device address with
//     cudaGetSymbolAddress on the current device (so a device reset or a new
//     primary context never leaves a stale address behind); the first call
//     on a device also loads the library's kernels there, so make it before
//     any stream capture;
//   - a key whose image, point or camera id is out of range is skipped and
//     counted on the device, and the cost written is then NaN.
#include "gba_internal.h"

#include <cmath>

namespace gba {
namespace {

constexpr int kNoAllocBlocks = 1024;     // grid of the cost kernel (partials)
constexpr int kNoAllocThreads = 256;
constexpr long long kRotDoubles = 12LL * GBA_NOALLOC_MAX_IMAGES;
// rotations, block partials, then one word counting the rejected keys
constexpr long long kScratchDoubles = kRotDoubles + kNoAllocBlocks + 1;

// The scratch: image rotations [12 * max images], block partials, bad-key count.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void k_na_rotations(gba_device_problem p, double* rot, unsigned long long* bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *bad = 0ull;  // cleared before the cost kernel runs (same stream)
  if (i >= p.number_of_images) return;
  const double* x = p.images + 6LL * i;
  const double r0 = x[0], r1 = x[1], r2 = x[2];
  const double theta = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
  double* R = rot + 12LL * i;
  if (theta == 0.0) {  // camera_shared_vector_function.hpp:695-698
    R[0] = 1; R[1] = 0; R[2] = 0; R[3] = 0; R[4] = 1; R[5] = 0; R[6] = 0; R[7] = 0; R[8] = 1;
  } else {
    double st, ct;
    sincos(theta, &st, &ct);
    const double k0 = r0 / theta, k1 = r1 / theta, k2 = r2 / theta, omc = 1.0 - ct;
    R[0] = ct + omc * k0 * k0; R[1] = -st * k2 + omc * k0 * k1; R[2] = st * k1 + omc * k0 * k2;
    R[3] = st * k2 + omc * k1 * k0; R[4] = ct + omc * k1 * k1; R[5] = -st * k0 + omc * k1 * k2;
    R[6] = -st * k1 + omc * k2 * k0; R[7] = st * k0 + omc * k2 * k1; R[8] = ct + omc * k2 * k2;
  }
  R[9] = x[3]; R[10] = x[4]; R[11] = x[5];
}

// Grid-stride variant of the cost kernel: one FP64 partial per block.  Every
// index read from the caller's arrays is checked before it is used; a key
// that fails is skipped and counted in *bad.
__global__ void __launch_bounds__(kNoAllocThreads) k_na_cost(gba_device_problem p, int loss,
                                                             double delta, const double* rot,
                                                             double* partial,
                                                             unsigned long long* bad) {
  __shared__ double red[kNoAllocThreads / 32];
  double acc = 0.0;
  unsigned long long rejected = 0;
  const long long K = p.number_of_keys;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K;
       k += (long long)gridDim.x * blockDim.x) {
    const int img = p.key_image[k], pt = p.key_point[k];
    if (img < 0 || img >= p.number_of_images || pt < 0 || pt >= p.number_of_points) {
      ++rejected;
      continue;
    }
    const int c = p.image_camera[img];
    if (c < 0 || c >= p.number_of_cameras) {
      ++rejected;
      continue;
    }
    const double* R = rot + 12LL * img;
    const double* X = p.points + 3LL * pt;
    const double* cam = p.cameras + 10LL * c;
    const double y0 = R[0] * X[0] + R[1] * X[1] + R[2] * X[2] + R[9];
    const double y1 = R[3] * X[0] + R[4] * X[1] + R[5] * X[2] + R[10];
    const double y2 = R[6] * X[0] + R[7] * X[1] + R[8] * X[2] + R[11];
    double n0 = y0 / y2, n1 = y1 / y2;
    const double r2 = n0 * n0 + n1 * n1;
    const double coeff = cam[0] * r2 + cam[1] * (r2 * r2) + cam[2] * (r2 * r2 * r2);
    const double dx = coeff * n0 + (2.0 * cam[3] * n0 * n1 + cam[4] * (r2 + 2.0 * n0 * n0));
    const double dy = coeff * n1 + (2.0 * cam[4] * n0 * n1 + cam[3] * (r2 + 2.0 * n1 * n1));
    n0 += dx;
    n1 += dy;
    const double u = cam[5] * n0 + cam[6] * n1 + cam[7];
    const double v = cam[5] * cam[9] * n1 + cam[8];
    const double e0 = u - p.keys[2 * k], e1 = v - p.keys[2 * k + 1];
    const double s = e0 * e0 + e1 * e1;
    if (loss == GBA_LOSS_HUBER && s > delta * delta)
      acc += 2.0 * delta * sqrt(s) - delta * delta;
    else
      acc += s;
  }
  if (rejected) atomicAdd(bad, rejected);
  acc = na_warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < kNoAllocThreads / 32 ? red[threadIdx.x] : 0.0;
    v = na_warp_sum(v);
    if (threadIdx.x == 0) partial[blockIdx.x] = v;
  }
}

__global__ void k_na_final(const double* partial, int n, const unsigned long long* bad,
                           double* out) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += 32) v += partial[i];
  v = na_warp_sum(v);
  if (threadIdx.x == 0) *out = *bad ? nan("") : v;
}

// Device address of the scratch array on the current device.
double* scratch_on_current_device(int* status) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *status = GBA_ERR_NO_DEVICE;
    return nullptr;
  }
  void* ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
    *status = GBA_ERR_CUDA;
    return nullptr;
  }
  *status = GBA_OK;
  return static_cast<double*>(ptr);
}

}  // namespace
}  // namespace gba

extern "C" int gba_cost_noalloc(const gba_device_problem* problem, int32_t loss,
                                double huber_delta, double* d_cost, void* stream) {
  if (!problem || !d_cost) return GBA_ERR_INVALID;
  const gba_device_problem& p = *problem;
  if (p.number_of_images < 0 || p.number_of_keys < 0 || p.number_of_points < 0 ||
      p.number_of_cameras < 0)
    return GBA_ERR_INVALID;
  if (p.number_of_images > GBA_NOALLOC_MAX_IMAGES) return GBA_ERR_INVALID;
  // Every array a launch may read must be there: the rotations read images,
  // the cost kernel reads the key arrays and, through them, the rest.
  if (p.number_of_images > 0 && !p.images) return GBA_ERR_INVALID;
  if (p.number_of_keys > 0 &&
      (!p.key_image || !p.key_point || !p.keys || !p.points || !p.images || !p.image_camera ||
       !p.cameras || p.number_of_images == 0 || p.number_of_points == 0 ||
       p.number_of_cameras == 0))
    return GBA_ERR_INVALID;
  if (loss != GBA_LOSS_TRIVIAL && loss != GBA_LOSS_HUBER) return GBA_ERR_INVALID;
  int status = GBA_OK;
  double* scratch = gba::scratch_on_current_device(&status);
  if (!scratch) return status;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* rot = scratch;
  double* partial = scratch + gba::kRotDoubles;
  unsigned long long* bad =
      reinterpret_cast<unsigned long long*>(scratch + gba::kRotDoubles + gba::kNoAllocBlocks);
  long long need = (p.number_of_keys + gba::kNoAllocThreads - 1) / gba::kNoAllocThreads;
  int blocks = int(need < gba::kNoAllocBlocks ? need : gba::kNoAllocBlocks);
  if (blocks < 1) blocks = 1;
  // Each launch's own status (cudaLaunchKernel returns it) decides the
  // result, so an earlier error of the caller's is neither reported as this
  // call's nor cleared.
  gba_device_problem pv = p;
  int rot_blocks = p.number_of_images > 0 ? (p.number_of_images + 127) / 128 : 1;
  void* a_rot[] = {&pv, &rot, &bad};
  if (cudaLaunchKernel((const void*)gba::k_na_rotations, dim3(rot_blocks), dim3(128), a_rot, 0,
                       s) != cudaSuccess)
    return GBA_ERR_CUDA;
  int lossv = loss;
  double delta = huber_delta;
  void* a_cost[] = {&pv, &lossv, &delta, &rot, &partial, &bad};
  if (cudaLaunchKernel((const void*)gba::k_na_cost, dim3(blocks), dim3(gba::kNoAllocThreads),
                       a_cost, 0, s) != cudaSuccess)
    return GBA_ERR_CUDA;
  const double* cpartial = partial;
  const unsigned long long* cbad = bad;
  void* a_fin[] = {&cpartial, &blocks, &cbad, &d_cost};
  if (cudaLaunchKernel((const void*)gba::k_na_final, dim3(1), dim3(32), a_fin, 0, s) !=
      cudaSuccess)
    return GBA_ERR_CUDA;
  gba::count_launches(3);
  return GBA_OK;
}
