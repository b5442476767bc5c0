// msv_pack.cu -- device-side database packing.
//
// The GB300 replacement of the fork's host packing loops (loadDBQuad,
// code/src/GPUFunction.cu:219-255): the raw residues arrive in one DMA and a
// kernel scatters them into the length-sorted, 16-byte-padded layout the
// search kernels read, checking every code on the way.
#include <cuda_runtime.h>

#include "msv_internal.h"

namespace {

__global__ void __launch_bounds__(256)
pack_kernel(const uint8_t *__restrict__ raw, const int64_t *__restrict__ src, const int64_t *__restrict__ start,
            const int32_t *__restrict__ len, int64_t n, uint8_t *__restrict__ packed, int *__restrict__ bad) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t) gridDim.x * blockDim.x) >> 5;
  int badl = 0;
  for (int64_t s = warp; s < n; s += nwarps) {
    const int L = len[s];
    const int padded = (L + 15) & ~15;
    const uint8_t *in = raw + src[s];
    uint8_t *out = packed + start[s];
    for (int j = lane; j < padded; j += 32) {
      uint8_t c = (uint8_t) msvgb::PAD_CODE;
      if (j < L) {
        c = in[j];
        badl |= (c >= 29);
      }
      out[j] = c;
    }
  }
  if (__any_sync(0xffffffffu, badl) && lane == 0) atomicOr(bad, 1);
}

}  // namespace

cudaError_t msvgb_detail::launch_pack(const uint8_t *raw, const int64_t *src, const int64_t *start,
                                      const int32_t *len, int64_t n, uint8_t *packed, int *bad,
                                      int num_sms, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  long long blocks = (n + 7) / 8;
  const long long cap = (long long) num_sms * 8;
  if (blocks > cap) blocks = cap;
  (void) cudaGetLastError();   // clear a stale error left by an unrelated call
  pack_kernel<<<(unsigned) blocks, 256, 0, stream>>>(raw, src, start, len, n, packed, bad);
  return cudaGetLastError();
}
