// msv_multi.cuh -- device code shared by the kernels that serve many
// profiles from one launch (batched search, serving loop): one warp scores one
// sorted sequence against a profile whose DP width C is a runtime value,
// dispatched to a compile-time instantiation.
#pragma once
#include "msv_device.cuh"

namespace msvgb {

// DP widths available to the multi-profile kernels; a profile whose tight
// width is not listed runs at the next larger one (extra nodes are padding).
constexpr int kMultiC[] = {1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 14, 16, 20, 24, 28, 32};
constexpr int kMultiMaxC = 32;

inline int multi_C(int M) {
  const int need = M / 64 + 1;
  for (int c : kMultiC) if (c >= need) return c;
  return -1;
}

template <int C>
__device__ __forceinline__ void run_seq(const ProfDev &P, const uint32_t *stab, const uint32_t *mtab,
                                        const DbDev &db, int64_t s, int lane, uint8_t *out_xj,
                                        uint8_t *out_flags) {
  const int L = db.len[s];
  const int64_t oi = db.orig[s];
  if (L == 0) {
    if (lane == 0) { out_xj[oi] = 0; out_flags[oi] = 0x08; }
    return;
  }
  const uint32_t *sq = reinterpret_cast<const uint32_t *>(db.codes + db.start[s]);
  int xj, full;
  const int st = msv_one<C, true>(P, stab, mtab, sq, L, lane, xj, full);
  if (lane == 0) {
    int flags = full ? 0x04 : 0;
    if (st == ST_ERANGE) flags |= 0x01 | 0x02;
    else if (xj >= P.xjmin[L]) flags |= 0x02;
    out_xj[oi] = (uint8_t) xj;
    out_flags[oi] = (uint8_t) flags;
  }
}

__device__ __forceinline__ void run_seq_any(int C, const ProfDev &P, const uint32_t *stab, const uint32_t *mtab,
                                            const DbDev &db, int64_t s, int lane, uint8_t *oxj, uint8_t *ofl) {
  switch (C) {
#define MSVGB_MULTI_CASE(c) case c: run_seq<c>(P, stab, mtab, db, s, lane, oxj, ofl); break;
    MSVGB_MULTI_CASE(1) MSVGB_MULTI_CASE(2) MSVGB_MULTI_CASE(3) MSVGB_MULTI_CASE(4)
    MSVGB_MULTI_CASE(5) MSVGB_MULTI_CASE(6) MSVGB_MULTI_CASE(7) MSVGB_MULTI_CASE(8)
    MSVGB_MULTI_CASE(10) MSVGB_MULTI_CASE(12) MSVGB_MULTI_CASE(14) MSVGB_MULTI_CASE(16)
    MSVGB_MULTI_CASE(20) MSVGB_MULTI_CASE(24) MSVGB_MULTI_CASE(28) MSVGB_MULTI_CASE(32)
#undef MSVGB_MULTI_CASE
    default: break;
  }
}

// Stages a profile's f16 SSV table and MSV table into shared memory.
__device__ __forceinline__ void stage_tables(const ProfDev &P, uint32_t *smem) {
  const int C = P.C;
  const int sw = NRES * C * 32, mw = NRES * ((C + 1) / 2) * 32;
  const uint4 *gs = reinterpret_cast<const uint4 *>(P.stab);
  const uint4 *gm = reinterpret_cast<const uint4 *>(P.mtab);
  uint4 *ss = reinterpret_cast<uint4 *>(smem);
  uint4 *sm = reinterpret_cast<uint4 *>(smem + sw);
  for (int i = threadIdx.x; i < sw / 4; i += blockDim.x) ss[i] = __ldg(gs + i);
  for (int i = threadIdx.x; i < mw / 4; i += blockDim.x) sm[i] = __ldg(gm + i);
}

inline size_t multi_smem_bytes(int cmax) {
  return ((size_t) NRES * cmax * 32 + (size_t) NRES * ((cmax + 1) / 2) * 32) * 4;
}

}  // namespace msvgb
