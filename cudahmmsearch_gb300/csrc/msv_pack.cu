// msv_pack.cu -- device-side database packing.
//
// The GB300 replacement of the fork's host packing loops (loadDBQuad,
// code/src/GPUFunction.cu:219-255) and of its offline length sort (dbsort):
// the raw residues arrive in one DMA; kernels compute the lengths, count them
// per length, place every sequence in descending-length order (its slot and
// 16-byte-aligned start follow from the per-length counts, which the host
// scans) and scatter the residues into the padded layout the search kernels
// read, checking every code on the way. Sequences of equal length may land in
// any order among themselves: each result is written to its original index.
// The input may be cut into chunks of consecutive sequences (ChunkCuts): the
// sort key is then (chunk, length), so every chunk keeps its own range of
// sorted slots and of packed bytes, longest first within it.
#include <algorithm>

#include <cuda_runtime.h>

#include "msv_internal.h"

namespace {

// One packed word: bytes at or past the sequence's end (valid = the bytes of
// w still inside it, any value) become padding; codes >= 29 inside it are
// flagged and become padding too (a search enqueued before the flag is read
// must never index past the cost tables' rows). Per byte b, bit 7 of
// ((b & 0x7f) + 99) | b is set exactly when b >= 29, with no carry between
// bytes ((b & 0x7f) + 99 <= 226).
__device__ __forceinline__ uint32_t pack_word(uint32_t w, int valid, int &badl) {
  const uint32_t keep = valid >= 4 ? 0xFFFFFFFFu : valid <= 0 ? 0u : (1u << (8 * valid)) - 1u;
  const uint32_t ge = ((((w & 0x7F7F7F7Fu) + 0x63636363u) | w) & 0x80808080u) & keep;
  badl |= ge != 0u;
  const uint32_t pad = ~keep | ((ge >> 7) * 0xFFu);
  return (w & ~pad) | (0x1D1D1D1Du & pad);
}

// One warp per sequence; each lane writes 16 packed bytes at a time (the
// packed starts are 16-byte aligned and the padded length a multiple of 16),
// from the five aligned words that cover them in the raw buffer, shifted
// into place. The raw buffer has 64 bytes of slack after its last residue.
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
    const uintptr_t in = (uintptr_t) (raw + src[s]);
    const uint32_t *w = reinterpret_cast<const uint32_t *>(in & ~(uintptr_t) 3);
    const unsigned sh = (unsigned) (in & 3) * 8u;
    uint4 *out = reinterpret_cast<uint4 *>(packed + start[s]);
    for (int j = lane * 16; j < padded; j += 32 * 16) {
      const uint32_t *q = w + j / 4;
      const uint32_t x0 = __ldg(q), x1 = __ldg(q + 1), x2 = __ldg(q + 2), x3 = __ldg(q + 3);
      const uint32_t x4 = sh ? __ldg(q + 4) : 0u;
      uint4 o;
      o.x = pack_word(__funnelshift_r(x0, x1, sh), L - j, badl);
      o.y = pack_word(__funnelshift_r(x1, x2, sh), L - j - 4, badl);
      o.z = pack_word(__funnelshift_r(x2, x3, sh), L - j - 8, badl);
      o.w = pack_word(__funnelshift_r(x3, x4, sh), L - j - 12, badl);
      out[j / 16] = o;
    }
  }
  if (__any_sync(0xffffffffu, badl) && lane == 0) atomicOr(bad, 1);
}

constexpr int64_t kMaxLen = 100000000;

// len[i] = off[i+1] - off[i]; the maximum into *lmax; *bad = 1 for a negative
// or absurd length (then len[i] = 0).
__global__ void __launch_bounds__(256)
len_kernel(const int64_t *__restrict__ off, int64_t n, int32_t *__restrict__ len, unsigned *lmax, int *bad) {
  unsigned m = 0;
  int b = 0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x) {
    int64_t L = off[i + 1] - off[i];
    if (L < 0 || L > kMaxLen) { b = 1; L = 0; }
    len[i] = (int32_t) L;
    m = max(m, (unsigned) L);
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(lmax, m);
  if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

// Chunk of input sequence i.
__device__ __forceinline__ int chunk_of(const msvgb_detail::ChunkCuts &c, int64_t i) {
  int k = 0;
  while (k + 1 < c.K && i >= c.cut[k + 1]) ++k;
  return k;
}

// hist[k * nb + L] = number of sequences of length L in chunk k
// (warp-aggregated atomics).
__global__ void __launch_bounds__(256)
hist_kernel(const int32_t *__restrict__ len, int64_t n, unsigned long long *__restrict__ hist,
            msvgb_detail::ChunkCuts cuts, int nb) {
  const int64_t stride = (int64_t) gridDim.x * blockDim.x;
  for (int64_t i0 = (int64_t) blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
    const int64_t i = i0 + threadIdx.x;
    const bool in = i < n;
    const unsigned act = __ballot_sync(0xffffffffu, in);
    if (!in) continue;
    const int key = chunk_of(cuts, i) * nb + len[i];
    const unsigned peers = __match_any_sync(act, key);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&hist[key], (unsigned long long) __popc(peers));
  }
}

// Sorted slot of every sequence: the next free slot of its key (chunk,
// length) (cursor[key] starts at the key's first slot); its padded start
// follows from the slot's rank within the key.
__global__ void __launch_bounds__(256)
place_kernel(const int64_t *__restrict__ off, const int32_t *__restrict__ len_in, int64_t n,
             unsigned long long *__restrict__ cursor, const int64_t *__restrict__ bin_slot,
             const int64_t *__restrict__ bin_byte, int64_t *__restrict__ start, int64_t *__restrict__ orig,
             int32_t *__restrict__ len, int64_t *__restrict__ src, msvgb_detail::ChunkCuts cuts, int nb) {
  const int64_t stride = (int64_t) gridDim.x * blockDim.x;
  for (int64_t i0 = (int64_t) blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
    const int64_t i = i0 + threadIdx.x;
    const bool in = i < n;
    const unsigned act = __ballot_sync(0xffffffffu, in);
    if (!in) continue;
    const int L = len_in[i];
    const int key = chunk_of(cuts, i) * nb + L;
    const unsigned peers = __match_any_sync(act, key);
    const int leader = __ffs(peers) - 1, lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&cursor[key], (unsigned long long) __popc(peers));
    base = __shfl_sync(peers, base, leader);
    const int64_t s = (int64_t) base + __popc(peers & ((1u << lane) - 1u));
    const int64_t padded = ((int64_t) L + 15) / 16 * 16;
    start[s] = bin_byte[key] + (s - bin_slot[key]) * padded;
    orig[s] = i;
    len[s] = L;
    src[s] = off[i] - off[0];
  }
}

// Exclusive scans of the per-key counts, chunk by chunk and within a chunk
// by descending length: the first sorted slot and first packed byte of every
// key (chunk, length), the packed size *pos, and the padding tail after it
// in the packed buffer. One block of 1024.
__global__ void __launch_bounds__(1024)
bins_kernel(const unsigned long long *__restrict__ hist, int Lmax, int K, int64_t *__restrict__ bin_slot,
            int64_t *__restrict__ bin_byte, int64_t *__restrict__ pos_out, uint8_t *__restrict__ codes) {
  __shared__ int64_t s_cnt[1024], s_byt[1024];
  const int T = blockDim.x, t = threadIdx.x;
  const int nb = Lmax + 1, nr = K * nb, per = (nr + T - 1) / T;
  const int r0 = min(nr, t * per), r1 = min(nr, (t + 1) * per);   // rank r: chunk r / nb, L = Lmax - r % nb
  int64_t c = 0, b = 0;
  for (int r = r0; r < r1; ++r) {
    const int L = Lmax - r % nb, key = (r / nb) * nb + L;
    c += (int64_t) hist[key];
    b += (int64_t) hist[key] * (((int64_t) L + 15) / 16 * 16);
  }
  s_cnt[t] = c; s_byt[t] = b;
  __syncthreads();
  for (int d = 1; d < T; d <<= 1) {                 // inclusive scan
    const int64_t vc = t >= d ? s_cnt[t - d] : 0, vb = t >= d ? s_byt[t - d] : 0;
    __syncthreads();
    s_cnt[t] += vc; s_byt[t] += vb;
    __syncthreads();
  }
  int64_t slot = t ? s_cnt[t - 1] : 0, byte = t ? s_byt[t - 1] : 0;
  for (int r = r0; r < r1; ++r) {
    const int L = Lmax - r % nb, key = (r / nb) * nb + L;
    bin_slot[key] = slot; bin_byte[key] = byte;
    slot += (int64_t) hist[key];
    byte += (int64_t) hist[key] * (((int64_t) L + 15) / 16 * 16);
  }
  const int64_t pos = s_byt[T - 1];
  if (t == 0) *pos_out = pos;
  if (t < 64) codes[pos + t] = (uint8_t) msvgb::PAD_CODE;
}

// inv[orig[s]] = s: original index -> sorted slot
__global__ void __launch_bounds__(256)
invert_kernel(const int64_t *__restrict__ orig, int64_t n, int64_t *__restrict__ inv) {
  for (int64_t s = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t) gridDim.x * blockDim.x)
    inv[orig[s]] = s;
}

// ids[j] = inv[ids[j]]
__global__ void __launch_bounds__(256)
gather_ids_kernel(int64_t *__restrict__ ids, int64_t n, const int64_t *__restrict__ inv) {
  for (int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t) gridDim.x * blockDim.x)
    ids[j] = inv[ids[j]];
}

// Listed sequences in database order (longest first): a counting sort of the
// list positions j into kOrderBuckets buckets of consecutive slots (the
// database is sorted by length, so a bucket holds similar lengths; within one
// the order is arbitrary). cnt[bucket] counts, is scanned to the first
// position of each bucket, then hands out positions.
constexpr int kOrderBuckets = 1024;

__device__ __forceinline__ int slot_bucket(int64_t slot, int64_t nslots) {
  return (int) ((slot * kOrderBuckets) / nslots);
}

__global__ void __launch_bounds__(256)
slot_count_kernel(const int64_t *__restrict__ slots, int64_t n, int64_t nslots, int32_t *__restrict__ cnt) {
  for (int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t) gridDim.x * blockDim.x)
    atomicAdd(&cnt[slot_bucket(slots[j], nslots)], 1);
}

// exclusive scan of the kOrderBuckets counts in place; one block, one count per thread
__global__ void __launch_bounds__(kOrderBuckets)
slot_scan_kernel(int32_t *__restrict__ cnt) {
  __shared__ int32_t s_sum[kOrderBuckets];
  const int t = threadIdx.x;
  const int32_t c = cnt[t];
  s_sum[t] = c;
  __syncthreads();
  for (int d = 1; d < kOrderBuckets; d <<= 1) {
    const int32_t v = t >= d ? s_sum[t - d] : 0;
    __syncthreads();
    s_sum[t] += v;
    __syncthreads();
  }
  cnt[t] = s_sum[t] - c;
}

__global__ void __launch_bounds__(256)
slot_place_kernel(const int64_t *__restrict__ slots, int64_t n, int64_t nslots, int32_t *__restrict__ cnt,
                  int64_t *__restrict__ order) {
  for (int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t) gridDim.x * blockDim.x)
    order[atomicAdd(&cnt[slot_bucket(slots[j], nslots)], 1)] = j;
}

int grid_for(int64_t n, int num_sms) {
  const long long blocks = std::min<long long>((n + 255) / 256, (long long) num_sms * 8);
  return (int) std::max<long long>(1, blocks);
}

}  // namespace

cudaError_t msvgb_detail::launch_lengths(const int64_t *off, int64_t n, int32_t *len, unsigned *lmax, int *bad,
                                         int num_sms, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  (void) cudaGetLastError();
  len_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(off, n, len, lmax, bad);
  return cudaGetLastError();
}

cudaError_t msvgb_detail::launch_histogram(const int32_t *len, int64_t n, unsigned long long *hist,
                                           const ChunkCuts &cuts, int nb, int num_sms, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  (void) cudaGetLastError();
  hist_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(len, n, hist, cuts, nb);
  return cudaGetLastError();
}

cudaError_t msvgb_detail::launch_invert(const int64_t *orig, int64_t n, int64_t *inv, int num_sms,
                                        cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  (void) cudaGetLastError();
  invert_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(orig, n, inv);
  return cudaGetLastError();
}

cudaError_t msvgb_detail::launch_gather_ids(int64_t *ids, int64_t n, const int64_t *inv, int num_sms,
                                            cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  (void) cudaGetLastError();
  gather_ids_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(ids, n, inv);
  return cudaGetLastError();
}

cudaError_t msvgb_detail::launch_order_by_slot(const int64_t *slots, int64_t n, int64_t nslots, int32_t *cnt,
                                               int64_t *order, int num_sms, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(cnt, 0, kOrderBuckets * sizeof(int32_t), stream);
  if (e != cudaSuccess) return e;
  (void) cudaGetLastError();
  slot_count_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(slots, n, nslots, cnt);
  slot_scan_kernel<<<1, kOrderBuckets, 0, stream>>>(cnt);
  slot_place_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(slots, n, nslots, cnt, order);
  return cudaGetLastError();
}

cudaError_t msvgb_detail::launch_bins(const unsigned long long *hist, int Lmax, int K, int64_t *bin_slot,
                                      int64_t *bin_byte, int64_t *pos, uint8_t *codes, cudaStream_t stream) {
  (void) cudaGetLastError();
  bins_kernel<<<1, 1024, 0, stream>>>(hist, Lmax, K, bin_slot, bin_byte, pos, codes);
  return cudaGetLastError();
}

cudaError_t msvgb_detail::launch_place(const int64_t *off, const int32_t *len_in, int64_t n,
                                       unsigned long long *cursor, const int64_t *bin_slot, const int64_t *bin_byte,
                                       int64_t *start, int64_t *orig, int32_t *len, int64_t *src,
                                       const ChunkCuts &cuts, int nb, int num_sms, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  (void) cudaGetLastError();
  place_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(off, len_in, n, cursor, bin_slot, bin_byte, start, orig,
                                                         len, src, cuts, nb);
  return cudaGetLastError();
}

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
