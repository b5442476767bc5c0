// msv_probe.cu -- the benchmark's peak probes (libmsvgb_probe.so, declared in
// include/msvgb_probe.h). Not linked into the filter library.
//
// Integer pipe: the MSV cost model counts one packed 32-bit integer operation
// per DP cell (four uint8 lane operations of the reference's SSE loop,
// msvfilter.c:150-153); the peak is the sustained rate of independent 32-bit
// integer max instructions over all SMs.
// Shared memory: every DP cell of the table-driven kernels reads its cost
// from shared memory; the peak is the sustained rate of conflict-free 16-byte
// loads over all SMs.
// Both are measured at whatever clock the GPU runs.
#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "../../include/msvgb_probe.h"

namespace {
thread_local std::string g_err;
int fail(const std::string &m) { g_err = m; return 12; }

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

// 16 KiB of shared memory per CTA (4 CTAs of 256 threads per SM): thread t
// reads word (row * 256 + t) of a 1024-row-of-16-B table, so a warp's 32 loads
// are 512 contiguous bytes (4 wavefronts, no bank conflict). The row index
// comes from the data, so loads cannot be hoisted.
constexpr int kSmemRows = 4, kSmemIters = 4096;

__global__ void __launch_bounds__(256) smem_read_kernel(uint32_t *out, uint32_t seed) {
  __shared__ uint4 tab[kSmemRows * 256];
  for (int i = threadIdx.x; i < kSmemRows * 256; i += blockDim.x)
    tab[i] = make_uint4(seed + i, seed ^ i, (uint32_t) i * 3u, 0u);
  __syncthreads();
  uint32_t acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
  uint32_t r = seed & 3u;
  for (int i = 0; i < kSmemIters; ++i) {
#pragma unroll
    for (int j = 0; j < kSmemRows; ++j) {
      const uint4 v = tab[((r + j) & (kSmemRows - 1)) * 256 + threadIdx.x];
      acc0 ^= v.x; acc1 += v.y; acc2 ^= v.z; acc3 |= v.w;
    }
    r = (r + (acc3 & 1u) + 1u) & 3u;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc0 ^ acc1 ^ acc2 ^ acc3;
}

// Times `launch` five times after one warm-up; returns milliseconds.
template <class F>
cudaError_t time_launches(F launch, float *ms) {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) {
    launch(1u);
    cudaEventRecord(a);
    for (uint32_t r = 0; r < 5; ++r) launch(2u + r);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  return e;
}

struct DeviceGuard {
  int old = -1;
  DeviceGuard() { cudaGetDevice(&old); }
  ~DeviceGuard() { if (old >= 0) cudaSetDevice(old); }
};
}  // namespace

extern "C" const char *msvgb_probe_last_error(void) { return g_err.c_str(); }

extern "C" int msvgb_measure_int_peak(int device, double *ops_per_second) {
  if (!ops_per_second) return fail("NULL argument");
  DeviceGuard guard;
  cudaError_t e = cudaSetDevice(device);
  int sms = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256;
  uint32_t *d = nullptr;
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(uint32_t) * blocks * threads);
  if (e == cudaSuccess)
    e = time_launches([&](uint32_t s) { int_max_kernel<<<blocks, threads>>>(d, s); }, &ms);
  cudaFree(d);
  if (e != cudaSuccess) return fail(std::string("int peak probe: ") + cudaGetErrorString(e));
  // each chain step is one max.s32 and one xor: both are 32-bit integer ops
  const double ops = 5.0 * blocks * threads * (double) kIters * kChains * 2.0;
  *ops_per_second = ops / (ms * 1e-3);
  return 0;
}

extern "C" int msvgb_measure_smem_peak(int device, double *bytes_per_second) {
  if (!bytes_per_second) return fail("NULL argument");
  DeviceGuard guard;
  cudaError_t e = cudaSetDevice(device);
  int sms = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 4, threads = 256;
  uint32_t *d = nullptr;
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(uint32_t) * blocks * threads);
  if (e == cudaSuccess)
    e = time_launches([&](uint32_t s) { smem_read_kernel<<<blocks, threads>>>(d, s); }, &ms);
  cudaFree(d);
  if (e != cudaSuccess) return fail(std::string("shared-memory probe: ") + cudaGetErrorString(e));
  const double bytes = 5.0 * blocks * threads * (double) kSmemIters * kSmemRows * 16.0;
  *bytes_per_second = bytes / (ms * 1e-3);
  return 0;
}
