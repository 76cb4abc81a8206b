// gba_calibrate.cu -- gba_fma_peak(): the FP32 / FP64 FMA throughput of the
// current device at its current clocks, the compute roof of the kernels that
// run on the CUDA cores (the dense factorization and the triangulation).
//
// Every thread keeps 16 independent accumulator chains and runs kSteps FMA
// steps on each (no memory traffic inside the timed loop); the grid is 8
// CTAs of 256 threads per SM.  Throughput = 2 * FMAs / kernel time (CUDA
// events, best of several launches after a warm-up).
#include "gba_internal.h"

#include <cstdio>

namespace gba {
namespace {

constexpr int kChains = 16;
constexpr int kSteps = 4096;

template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(T a, T b, T* out) {
  T acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = T(threadIdx.x + c) * T(1e-7);
  for (int s = 0; s < kSteps; ++s) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = fma(acc[c], a, b);
  }
  T r = T(0);
#pragma unroll
  for (int c = 0; c < kChains; ++c) r += acc[c];
  if (r == T(-1.2345)) out[0] = r;   // keeps the chains live; never true for these inputs
}

template <typename T>
double measure(int device) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return -1;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const dim3 grid(unsigned(sms * 8)), block(256);
  const T a = T(0.999999), b = T(1e-6);
  k_fma_peak<T><<<grid, block>>>(a, b, out);
  double best = 0.0;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    k_fma_peak<T><<<grid, block>>>(a, b, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * double(grid.x) * block.x * kChains * double(kSteps);
    if (ms > 0.0f) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return err == cudaSuccess ? best : -1.0;
}

}  // namespace
}  // namespace gba

extern "C" int gba_fma_peak(int32_t precision, int32_t device, double* tflops) {
  if (!tflops) return GBA_ERR_INVALID;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return GBA_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return GBA_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return GBA_ERR_CUDA;
  const double v = precision == GBA_PRECISION_FP64 ? gba::measure<double>(device)
                                                   : gba::measure<float>(device);
  gba::count_launches(6);
  if (v < 0) return GBA_ERR_CUDA;
  *tflops = v;
  return GBA_OK;
}
