// msv_probe.cu -- measures the integer-pipe peak the roofline is quoted against.
//
// The MSV cost model counts one packed 32-bit integer operation per DP cell
// (four uint8 lane operations of the reference's SSE loop, msvfilter.c:150-153).
// The peak is the sustained rate of independent 32-bit integer max
// instructions over all SMs, measured here at whatever clock the GPU runs.
#include <cuda_runtime.h>
#include <string>

#include "../../include/msvgb.h"
#include "msv_internal.h"

namespace {
constexpr int kIters = 2048, kChains = 8;

__global__ void __launch_bounds__(256) int_max_kernel(uint32_t *out, uint32_t seed) {
  int v[kChains];
  int b = (int) (seed * 2654435761u + threadIdx.x);
#pragma unroll
  for (int j = 0; j < kChains; ++j) v[j] = (int) (seed + 97 * j + threadIdx.x);
  for (int i = 0; i < kIters; ++i) {
#pragma unroll
    for (int j = 0; j < kChains; ++j) {
      int r;
      asm volatile("max.s32 %0, %1, %2;" : "=r"(r) : "r"(v[j]), "r"(b));
      v[j] = r ^ j;          // keeps the chain live; the xor pairs with the max
    }
    b += 0x9E3779B9;
  }
  int r = 0;
#pragma unroll
  for (int j = 0; j < kChains; ++j) r ^= v[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (uint32_t) r;
}
}  // namespace

extern "C" int msvgb_measure_int_peak(int device, double *ops_per_second) {
  using msvgb_detail::fail;
  if (!ops_per_second) return fail(MSVGB_eslEINVAL, "NULL argument");
  int old = -1;
  cudaGetDevice(&old);
  cudaError_t e = cudaSetDevice(device);
  int sms = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256;
  uint32_t *d = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(uint32_t) * blocks * threads);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) {
    int_max_kernel<<<blocks, threads>>>(d, 1u);                  // warm-up
    cudaEventRecord(a);
    for (int r = 0; r < 5; ++r) int_max_kernel<<<blocks, threads>>>(d, 2u + r);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
  }
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(d);
  if (old >= 0) cudaSetDevice(old);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("int peak probe: ") + cudaGetErrorString(e));
  // each chain step is one max.s32 and one xor: both are 32-bit integer ops
  const double ops = 5.0 * blocks * threads * (double) kIters * kChains * 2.0;
  *ops_per_second = ops / (ms * 1e-3);
  return MSVGB_eslOK;
}
