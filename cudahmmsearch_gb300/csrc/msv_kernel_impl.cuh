// msv_kernel_impl.cuh -- the search kernel and its launcher (instantiated per C
// in inst_*.cu so the translation units compile in parallel).
#pragma once
#include <cuda_fp16.h>
#include "msv_device.cuh"

namespace msvgb {

struct LaunchArgs {
  ProfDev             P;
  DbDev               db;
  uint8_t            *out_xj;     // [n] in original sequence order
  uint8_t            *out_flags;  // [n]
  unsigned long long *ticket;     // zeroed before the launch
  cudaStream_t        stream;
  int                 grid;       // 0: fill the GPU
  int                 skip_empty; // 1: L == 0 is skipped as p7_Pipeline does; 0: scored like p7_MSVFilter
  // List mode: score only the sorted sequences list[0 .. *list_count) with the
  // full MSV recurrence (they are the ones the G-lane SSV pass left undecided).
  const int64_t            *list = nullptr;
  const unsigned long long *list_count = nullptr;
  // Range mode (range_end > 0): only the sorted sequences [0, range_end).
  int64_t                   range_end = 0;
};

constexpr int WARPS_PER_CTA = 8;
constexpr int MAX_WARPS_PER_CTA = 16;   // used when the tables leave room for one CTA per SM

// f16 tables wider than 40 words per lane (M >= 2560: 154 KB of SSV costs
// and up) do not fit in shared memory beside the MSV table: such profiles keep
// both tables in global memory, where they stream through L1 and L2 (a few
// hundred KB, resident in the 129 MB L2 for the whole launch).
template <int C, bool F16>
__host__ __device__ constexpr bool tables_in_global() { return F16 && C > 40; }

template <int C, bool F16>
constexpr size_t smem_bytes() {   // SSV table + MSV table
  if (tables_in_global<C, F16>()) return 0;
  return ((size_t) (F16 ? NRES * C * 32 : NRES * (C / 2) * 32) + (size_t) NRES * ((C + 1) / 2) * 32) * 4;
}

// Threads per CTA: 8 warps, or 16 when the tables leave room for only one CTA per SM.
template <int C, bool F16>
constexpr int cta_threads() { return 2 * smem_bytes<C, F16>() > 227 * 1024 ? MAX_WARPS_PER_CTA * 32 : WARPS_PER_CTA * 32; }

// Persistent kernel: every CTA stages the profile's cost tables into shared
// memory once, then its warps pull sequences (longest first) from a global
// ticket until the database is exhausted.
template <int C, bool F16>
__global__ void __launch_bounds__(cta_threads<C, F16>())
msv_search_kernel(ProfDev P, DbDev db, uint8_t *__restrict__ out_xj, uint8_t *__restrict__ out_flags,
                  unsigned long long *__restrict__ ticket, int skip_empty,
                  const int64_t *__restrict__ list, const unsigned long long *__restrict__ list_count,
                  int64_t range_end) {
  extern __shared__ __align__(16) uint32_t smem[];
  constexpr int SW = F16 ? NRES * C * 32 : NRES * (C / 2) * 32;   // words of the SSV table
  constexpr int MW = NRES * ((C + 1) / 2) * 32;                    // words of the MSV table
  const uint32_t *stab = P.stab, *mtab = P.mtab;
  if constexpr (!tables_in_global<C, F16>()) {
    const uint4 *gs = reinterpret_cast<const uint4 *>(P.stab);
    const uint4 *gm = reinterpret_cast<const uint4 *>(P.mtab);
    uint4 *ss = reinterpret_cast<uint4 *>(smem);
    uint4 *sm = reinterpret_cast<uint4 *>(smem + SW);
    for (int i = threadIdx.x; i < SW / 4; i += blockDim.x) ss[i] = __ldg(gs + i);
    for (int i = threadIdx.x; i < MW / 4; i += blockDim.x) sm[i] = __ldg(gm + i);
    stab = smem;
    mtab = smem + SW;
    __syncthreads();
  }

  const int lane = threadIdx.x & 31;
  const unsigned long long nitems = list ? *list_count : (unsigned long long) (range_end > 0 ? range_end : db.n);
  for (;;) {
    unsigned long long s = 0;
    if (lane == 0) s = atomicAdd(ticket, 1ull);
    s = __shfl_sync(FULL, s, 0);
    if (s >= nitems) break;
    if (list) s = (unsigned long long) list[s];
    const int L = db.len[s];
    const int64_t oi = db.orig[s];
    if (L == 0 && skip_empty) {
      if (lane == 0) { out_xj[oi] = 0; out_flags[oi] = 0x08; }   // MSVGB_FLAG_EMPTY
      continue;
    }
    const uint32_t *sq = reinterpret_cast<const uint32_t *>(db.codes + db.start[s]);
    int xj, full;
    const int st = msv_one<C, F16>(P, stab, mtab, sq, L, lane, xj, full, list != nullptr);
    if (lane == 0) {
      int flags = full ? 0x04 : 0;
      if (st == ST_ERANGE) flags |= 0x01 | 0x02;                 // +inf always passes F1
      else if (xj >= P.xjmin[L]) flags |= 0x02;
      out_xj[oi] = (uint8_t) xj;
      out_flags[oi] = (uint8_t) flags;
    }
  }
}

template <int C, bool F16>
cudaError_t launch_search(const LaunchArgs &a, int num_sms) {
  auto kern = msv_search_kernel<C, F16>;
  constexpr size_t smem = smem_bytes<C, F16>();
  static std::atomic<unsigned long long> configured{0};
  {
    cudaError_t e = ensure_smem_attr((const void *) kern, smem, configured);
    if (e != cudaSuccess) return e;
  }
  constexpr int threads = cta_threads<C, F16>();
  int grid = a.grid;
  if (grid <= 0) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    grid = per_sm * num_sms;
    const int warps = threads / 32;
    const long long need = ((a.range_end > 0 ? a.range_end : a.db.n) + warps - 1) / warps;
    if (!a.list && need < grid) grid = (int) (need > 0 ? need : 1);
  }
  (void) cudaGetLastError();   // clear a stale error left by an unrelated call
  kern<<<grid, threads, smem, a.stream>>>(a.P, a.db, a.out_xj, a.out_flags, a.ticket, a.skip_empty,
                                               a.list, a.list_count, a.range_end);
  return cudaGetLastError();
}

}  // namespace msvgb

#define MSVGB_INSTANTIATE_I8(C) \
  template cudaError_t msvgb::launch_search<C, false>(const msvgb::LaunchArgs &, int);
#define MSVGB_INSTANTIATE_F16(C) \
  template cudaError_t msvgb::launch_search<C, true>(const msvgb::LaunchArgs &, int);
