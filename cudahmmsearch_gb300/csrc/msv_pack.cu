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

// Keys in sorted order: chunk k, then descending length L, at k * nb + (Lmax - L)
// (nb = Lmax + 1).
__device__ __forceinline__ int sort_key(int k, int L, int Lmax) { return k * (Lmax + 1) + (Lmax - L); }

// Counts and placement run one block per part of the input (a contiguous
// range of sequences). Keys of short sequences (L < lb, with K * lb <=
// kSmemKeys) are counted in shared memory: block b's count of small key j goes
// to blk[b * K * lb + j] and, summed, to hist; a column scan over the blocks
// turns blk into each block's first rank within the key, and placement ranks
// the block's own sequences in shared memory. Longer sequences (rare) take one
// global atomic each, in hist and at placement. (One global atomic per
// sequence took 0.11 + 0.14 ms for 2,000,000 sequences, bound by the atomics
// on the most frequent lengths.)
constexpr int kSmemKeys = 8192, kPartThreads = 512;

__device__ __forceinline__ void part_range(int64_t n, int64_t *a, int64_t *e) {
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  *a = min(n, (int64_t) blockIdx.x * per);
  *e = min(n, *a + per);
}

__global__ void __launch_bounds__(kPartThreads)
hist_kernel(const int32_t *__restrict__ len, int64_t n, unsigned long long *__restrict__ hist,
            uint32_t *__restrict__ blk, msvgb_detail::ChunkCuts cuts, int Lmax, int lb) {
  __shared__ uint32_t cnt[kSmemKeys];
  const int K = cuts.K, sk = K * lb;
  for (int j = threadIdx.x; j < sk; j += blockDim.x) cnt[j] = 0u;
  __syncthreads();
  int64_t a, e;
  part_range(n, &a, &e);
  for (int64_t i = a + threadIdx.x; i < e; i += blockDim.x) {
    const int L = len[i], k = chunk_of(cuts, i);
    if (L < lb) atomicAdd(&cnt[k * lb + L], 1u);
    else atomicAdd(&hist[sort_key(k, L, Lmax)], 1ull);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < sk; j += blockDim.x) {
    const uint32_t c = cnt[j];
    blk[(int64_t) blockIdx.x * sk + j] = c;
    if (c) atomicAdd(&hist[sort_key(j / lb, j % lb, Lmax)], (unsigned long long) c);
  }
}

// blk[b * sk + j] <- the count of small key j in blocks before b. Rows are
// loaded 16 at a time, independently (a chain of dependent loads took 60 us).
__global__ void __launch_bounds__(256)
part_scan_kernel(uint32_t *__restrict__ blk, int nparts, int sk) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= sk) return;
  uint32_t run = 0u;
  int b = 0;
  for (; b + 16 <= nparts; b += 16) {
    uint32_t c[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) c[u] = blk[(int64_t) (b + u) * sk + j];
#pragma unroll
    for (int u = 0; u < 16; ++u) { blk[(int64_t) (b + u) * sk + j] = run; run += c[u]; }
  }
  for (; b < nparts; ++b) {
    const uint32_t c = blk[(int64_t) b * sk + j];
    blk[(int64_t) b * sk + j] = run;
    run += c;
  }
}

// Sorted slot of every sequence: a short one at its key's first slot + its
// block's first rank within the key + its rank in the block (shared-memory
// counter); a long one from the key's global cursor (which starts at the
// key's first slot). Its padded start follows from the slot's rank within
// the key. Equal keys land in any order.
__global__ void __launch_bounds__(kPartThreads)
place_kernel(const int64_t *__restrict__ off, const int32_t *__restrict__ len_in, int64_t n,
             unsigned long long *__restrict__ cursor, const uint32_t *__restrict__ blk,
             const int64_t *__restrict__ bin_slot, const int64_t *__restrict__ bin_byte,
             int64_t *__restrict__ start, int64_t *__restrict__ orig, int32_t *__restrict__ len,
             int64_t *__restrict__ src, msvgb_detail::ChunkCuts cuts, int Lmax, int lb) {
  __shared__ uint32_t rank[kSmemKeys];
  const int K = cuts.K, sk = K * lb;
  for (int j = threadIdx.x; j < sk; j += blockDim.x) rank[j] = 0u;
  __syncthreads();
  int64_t a, e;
  part_range(n, &a, &e);
  for (int64_t i = a + threadIdx.x; i < e; i += blockDim.x) {
    const int L = len_in[i], k = chunk_of(cuts, i);
    const int key = sort_key(k, L, Lmax);
    int64_t s;
    if (L < lb) {
      const int j = k * lb + L;
      s = bin_slot[key] + (int64_t) blk[(int64_t) blockIdx.x * sk + j] + (int64_t) atomicAdd(&rank[j], 1u);
    } else {
      s = (int64_t) atomicAdd(&cursor[key], 1ull);
    }
    const int64_t padded = ((int64_t) L + 15) / 16 * 16;
    start[s] = bin_byte[key] + (s - bin_slot[key]) * padded;
    orig[s] = i;
    len[s] = L;
    src[s] = off[i] - off[0];
  }
}

// Exclusive scans of the per-key counts in key order (chunk by chunk, and
// within a chunk by descending length): the first sorted slot and first
// packed byte of every key, the packed size *pos, and the padding tail after
// it in the packed buffer. Three phases over tiles of kScanTile keys: per-tile
// totals, a scan of the totals in one block, then every tile's own scan from
// its offset. A thread takes kScanPer consecutive keys.
constexpr int kScanPer = 16, kScanThreads = 256, kScanTile = kScanPer * kScanThreads;

__device__ __forceinline__ int64_t key_bytes(int r, int Lmax) {   // packed bytes of one sequence of key r
  const int L = Lmax - r % (Lmax + 1);
  return ((int64_t) L + 15) / 16 * 16;
}

// Inclusive scan of (a, b) over the block (Hillis-Steele in shared memory); T threads.
template <int T>
__device__ __forceinline__ void block_scan2(int64_t &a, int64_t &b, int64_t *sa, int64_t *sb) {
  const int t = threadIdx.x;
  sa[t] = a; sb[t] = b;
  __syncthreads();
  for (int d = 1; d < T; d <<= 1) {
    const int64_t va = t >= d ? sa[t - d] : 0, vb = t >= d ? sb[t - d] : 0;
    __syncthreads();
    sa[t] += va; sb[t] += vb;
    __syncthreads();
  }
  a = sa[t]; b = sb[t];
}

__global__ void __launch_bounds__(kScanThreads)
bins_tile_kernel(const unsigned long long *__restrict__ hist, int nr, int Lmax, int64_t *__restrict__ tile_cnt,
                 int64_t *__restrict__ tile_byt) {
  __shared__ int64_t sa[kScanThreads], sb[kScanThreads];
  const int r0 = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  int64_t c = 0, b = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; ++j)
    if (r0 + j < nr) {
      const int64_t h = (int64_t) hist[r0 + j];
      c += h;
      b += h * key_bytes(r0 + j, Lmax);
    }
  block_scan2<kScanThreads>(c, b, sa, sb);
  if (threadIdx.x == kScanThreads - 1) { tile_cnt[blockIdx.x] = c; tile_byt[blockIdx.x] = b; }
}

// Exclusive scan of the ntiles totals in place (one block of 1024; ntiles <=
// 4 * 1024); the grand total of bytes is the packed size.
__global__ void __launch_bounds__(1024)
bins_top_kernel(int64_t *__restrict__ tile_cnt, int64_t *__restrict__ tile_byt, int ntiles,
                int64_t *__restrict__ pos_out, uint8_t *__restrict__ codes) {
  __shared__ int64_t sa[1024], sb[1024];
  const int t = threadIdx.x, per = (ntiles + 1023) / 1024;
  const int i0 = min(ntiles, t * per), i1 = min(ntiles, (t + 1) * per);
  int64_t c = 0, b = 0;
  for (int i = i0; i < i1; ++i) { c += tile_cnt[i]; b += tile_byt[i]; }
  int64_t ic = c, ib = b;
  block_scan2<1024>(ic, ib, sa, sb);
  int64_t oc = ic - c, ob = ib - b;                  // exclusive offsets of this thread's first tile
  for (int i = i0; i < i1; ++i) {
    const int64_t tc = tile_cnt[i], tb = tile_byt[i];
    tile_cnt[i] = oc; tile_byt[i] = ob;
    oc += tc; ob += tb;
  }
  const int64_t pos = sb[1023];
  if (t == 0) *pos_out = pos;
  if (t < 64) codes[pos + t] = (uint8_t) msvgb::PAD_CODE;
}

__global__ void __launch_bounds__(kScanThreads)
bins_fill_kernel(const unsigned long long *__restrict__ hist, int nr, int Lmax, const int64_t *__restrict__ tile_cnt,
                 const int64_t *__restrict__ tile_byt, int64_t *__restrict__ bin_slot,
                 int64_t *__restrict__ bin_byte) {
  __shared__ int64_t sa[kScanThreads], sb[kScanThreads];
  const int r0 = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  int64_t h[kScanPer];
  int64_t c = 0, b = 0;
#pragma unroll
  for (int j = 0; j < kScanPer; ++j) {
    h[j] = r0 + j < nr ? (int64_t) hist[r0 + j] : 0;
    c += h[j];
    b += h[j] * key_bytes(r0 + j, Lmax);
  }
  int64_t ic = c, ib = b;
  block_scan2<kScanThreads>(ic, ib, sa, sb);
  int64_t slot = tile_cnt[blockIdx.x] + ic - c, byte = tile_byt[blockIdx.x] + ib - b;
#pragma unroll
  for (int j = 0; j < kScanPer; ++j)
    if (r0 + j < nr) {
      bin_slot[r0 + j] = slot; bin_byte[r0 + j] = byte;
      slot += h[j];
      byte += h[j] * key_bytes(r0 + j, Lmax);
    }
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

// Listed sequences longest first: a counting sort of the list positions j
// into kOrderBuckets buckets of descending length (bucket 1023 - 1023 *
// sqrt(L / Lmax): finer where lengths are common; within a bucket the order
// is arbitrary). It does not assume the database's own order (a database
// built chunk by chunk is sorted within each chunk only). cnt[bucket] counts,
// is scanned to the first position of each bucket, then hands out positions.
constexpr int kOrderBuckets = 1024;

__device__ __forceinline__ int len_bucket(int L, int Lmax) {
  const float r = Lmax > 0 ? sqrtf((float) min(L, Lmax) / (float) Lmax) : 0.f;
  return (kOrderBuckets - 1) - min(kOrderBuckets - 1, (int) (r * (float) (kOrderBuckets - 1)));
}

__global__ void __launch_bounds__(256)
slot_count_kernel(const int64_t *__restrict__ slots, int64_t n, const int32_t *__restrict__ len, int Lmax,
                  int32_t *__restrict__ cnt) {
  for (int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t) gridDim.x * blockDim.x)
    atomicAdd(&cnt[len_bucket(len[slots[j]], Lmax)], 1);
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
slot_place_kernel(const int64_t *__restrict__ slots, int64_t n, const int32_t *__restrict__ len, int Lmax,
                  int32_t *__restrict__ cnt, int64_t *__restrict__ order) {
  for (int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t) gridDim.x * blockDim.x)
    order[atomicAdd(&cnt[len_bucket(len[slots[j]], Lmax)], 1)] = j;
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

int msvgb_detail::sort_parts(int num_sms) { return std::max(1, 2 * num_sms); }   // two 512-thread blocks per SM

int msvgb_detail::sort_small_bound(int Lmax, int K) { return std::max(1, std::min(Lmax + 1, kSmemKeys / std::max(1, K))); }

cudaError_t msvgb_detail::launch_histogram(const int32_t *len, int64_t n, unsigned long long *hist, uint32_t *blk,
                                           const ChunkCuts &cuts, int Lmax, int num_sms, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  (void) cudaGetLastError();
  const int parts = sort_parts(num_sms), lb = sort_small_bound(Lmax, cuts.K), sk = cuts.K * lb;
  hist_kernel<<<parts, kPartThreads, 0, stream>>>(len, n, hist, blk, cuts, Lmax, lb);
  part_scan_kernel<<<(sk + 255) / 256, 256, 0, stream>>>(blk, parts, sk);
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

cudaError_t msvgb_detail::launch_order_by_length(const int64_t *slots, int64_t n, const int32_t *len, int Lmax, int32_t *cnt,
                                               int64_t *order, int num_sms, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(cnt, 0, kOrderBuckets * sizeof(int32_t), stream);
  if (e != cudaSuccess) return e;
  (void) cudaGetLastError();
  slot_count_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(slots, n, len, Lmax, cnt);
  slot_scan_kernel<<<1, kOrderBuckets, 0, stream>>>(cnt);
  slot_place_kernel<<<grid_for(n, num_sms), 256, 0, stream>>>(slots, n, len, Lmax, cnt, order);
  return cudaGetLastError();
}

int msvgb_detail::bins_scratch_words(int Lmax, int K) {
  const int nr = K * (Lmax + 1);
  return 2 * ((nr + kScanTile - 1) / kScanTile);
}

cudaError_t msvgb_detail::launch_bins(const unsigned long long *hist, int Lmax, int K, int64_t *bin_slot,
                                      int64_t *bin_byte, int64_t *scratch, int64_t *pos, uint8_t *codes,
                                      cudaStream_t stream) {
  const int nr = K * (Lmax + 1), ntiles = (nr + kScanTile - 1) / kScanTile;
  if (ntiles > 4 * 1024) return cudaErrorInvalidValue;                 // bins_top_kernel's limit
  int64_t *tile_cnt = scratch, *tile_byt = scratch + ntiles;
  (void) cudaGetLastError();
  bins_tile_kernel<<<ntiles, kScanThreads, 0, stream>>>(hist, nr, Lmax, tile_cnt, tile_byt);
  bins_top_kernel<<<1, 1024, 0, stream>>>(tile_cnt, tile_byt, ntiles, pos, codes);
  bins_fill_kernel<<<ntiles, kScanThreads, 0, stream>>>(hist, nr, Lmax, tile_cnt, tile_byt, bin_slot, bin_byte);
  return cudaGetLastError();
}

cudaError_t msvgb_detail::launch_place(const int64_t *off, const int32_t *len_in, int64_t n,
                                       unsigned long long *cursor, const uint32_t *blk, const int64_t *bin_slot,
                                       const int64_t *bin_byte, int64_t *start, int64_t *orig, int32_t *len,
                                       int64_t *src, const ChunkCuts &cuts, int Lmax, int num_sms,
                                       cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  (void) cudaGetLastError();
  place_kernel<<<sort_parts(num_sms), kPartThreads, 0, stream>>>(off, len_in, n, cursor, blk, bin_slot, bin_byte,
                                                                start, orig, len, src, cuts, Lmax,
                                                                sort_small_bound(Lmax, cuts.K));
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
