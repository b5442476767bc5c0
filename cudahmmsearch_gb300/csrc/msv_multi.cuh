// msv_multi.cuh -- device code shared by the kernels that serve many
// profiles from one launch (batched search, serving loop). A CTA takes a work
// item (one profile, a chunk of the sorted database) and scores it either with
// one warp per sequence (SSV and full MSV fused) or, for the profiles the
// lane choice puts on 16 or 8 lanes, with the lane-group SSV pass followed by
// the full MSV on the sequences it left undecided. The DP widths are runtime
// values dispatched to compile-time instantiations.
#pragma once
#include "msv_device.cuh"
#include "msv_group.cuh"

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

// Lane-group SSV widths: the tight width M / (2G) + 1 rounded up in kMultiC
// (at least 2); -1 when it exceeds 32.
inline int group_C(int M, int G) {
  const int need = M / (2 * G) + 1;
  for (int c : kMultiC) if (c >= need && c >= 2) return c;
  return -1;
}

// Sequences per work item when the SSV pass runs on lane groups (the
// undecided list of a chunk lives in shared memory).
constexpr int kChunkMaxSeqs = 2048;

template <int C>
__device__ __forceinline__ void run_seq(const ProfDev &P, const uint32_t *stab, const uint32_t *mtab,
                                        const DbDev &db, int64_t s, int lane, uint8_t *out_xj,
                                        uint8_t *out_flags, bool skip_ssv) {
  const int L = db.len[s];
  const int64_t oi = db.orig[s];
  if (L == 0) {
    if (lane == 0) { out_xj[oi] = 0; out_flags[oi] = 0x08; }
    return;
  }
  const uint32_t *sq = reinterpret_cast<const uint32_t *>(db.codes + db.start[s]);
  int xj, full;
  const int st = msv_one<C, true>(P, stab, mtab, sq, L, lane, xj, full, skip_ssv);
  if (lane == 0) {
    int flags = full ? 0x04 : 0;
    if (st == ST_ERANGE) flags |= 0x01 | 0x02;
    else if (xj >= P.xjmin[L]) flags |= 0x02;
    out_xj[oi] = (uint8_t) xj;
    out_flags[oi] = (uint8_t) flags;
  }
}

__device__ __forceinline__ void run_seq_any(int C, const ProfDev &P, const uint32_t *stab, const uint32_t *mtab,
                                            const DbDev &db, int64_t s, int lane, uint8_t *oxj, uint8_t *ofl,
                                            bool skip_ssv = false) {
  switch (C) {
#define MSVGB_MULTI_CASE(c) case c: run_seq<c>(P, stab, mtab, db, s, lane, oxj, ofl, skip_ssv); break;
    MSVGB_MULTI_CASE(1) MSVGB_MULTI_CASE(2) MSVGB_MULTI_CASE(3) MSVGB_MULTI_CASE(4)
    MSVGB_MULTI_CASE(5) MSVGB_MULTI_CASE(6) MSVGB_MULTI_CASE(7) MSVGB_MULTI_CASE(8)
    MSVGB_MULTI_CASE(10) MSVGB_MULTI_CASE(12) MSVGB_MULTI_CASE(14) MSVGB_MULTI_CASE(16)
    MSVGB_MULTI_CASE(20) MSVGB_MULTI_CASE(24) MSVGB_MULTI_CASE(28) MSVGB_MULTI_CASE(32)
#undef MSVGB_MULTI_CASE
    default: break;
  }
}

// 8-bit words per lane of the mixed-width table the multi-profile kernels
// use at lane-group width Cg (0: f16 table): the single-query default
// (hyb_default_words) at the group widths these kernels compile (kMultiC).
__host__ __device__ constexpr int multi_hyb_words(int Cg, int G) {
  return G == 8 ? (Cg < 10 ? 0 : Cg < 18 ? 4 : 8) : G == 16 ? (Cg < 13 ? 0 : Cg < 24 ? 4 : 8) : 0;
}

// The lane-group SSV pass of one chunk at (G, Cg), with the f16 or the
// mixed-width table as P.CI says (0, or multi_hyb_words(Cg, G)).
__device__ __forceinline__ void ssv_group_chunk_any(int G, int Cg, const ProfDev &P, const uint32_t *tab,
                                                    const DbDev &db, int64_t s0, int nseq, uint8_t *oxj,
                                                    uint8_t *ofl, unsigned *next_seq, uint16_t *und,
                                                    unsigned *n_und) {
#define MSVGB_GROUP_VARIANT(c, g)                                                                          \
  if (G == g) {                                                                                            \
    constexpr int ci = multi_hyb_words(c, g);                                                              \
    bool done = false;                                                                                     \
    if constexpr (ci > 0) {                                                                                \
      if (P.CI == ci) { ssv_group_chunk<c, g, ci>(P, tab, db, s0, nseq, oxj, ofl, next_seq, und, n_und); done = true; } \
    }                                                                                                      \
    if (!done) ssv_group_chunk<c, g, 0>(P, tab, db, s0, nseq, oxj, ofl, next_seq, und, n_und);             \
  }
#define MSVGB_GROUP_CASE(c) case c: MSVGB_GROUP_VARIANT(c, 8) else MSVGB_GROUP_VARIANT(c, 16) break;
  switch (Cg) {
    MSVGB_GROUP_CASE(2) MSVGB_GROUP_CASE(3) MSVGB_GROUP_CASE(4) MSVGB_GROUP_CASE(5)
    MSVGB_GROUP_CASE(6) MSVGB_GROUP_CASE(7) MSVGB_GROUP_CASE(8) MSVGB_GROUP_CASE(10)
    MSVGB_GROUP_CASE(12) MSVGB_GROUP_CASE(14) MSVGB_GROUP_CASE(16) MSVGB_GROUP_CASE(20)
    MSVGB_GROUP_CASE(24) MSVGB_GROUP_CASE(28) MSVGB_GROUP_CASE(32)
    default: break;
  }
#undef MSVGB_GROUP_CASE
#undef MSVGB_GROUP_VARIANT
}

// Shared state of one CTA's work item.
struct ChunkShared {
  unsigned next_seq, n_und, next_und;
  uint16_t und[kChunkMaxSeqs];
};

// Words of a profile's SSV table in shared memory (the MSV table follows it):
// the lane-group layout with its region copies (group_words), or the 32-lane one.
__host__ __device__ inline int ssv_words(const ProfDev &P) {
  return P.G < 32 ? group_words(P.Cg, P.G, P.CI) : NRES * P.C * 32;
}

// One CTA scores the sorted sequences [s0, s0 + nseq) against P, whose tables
// are in shared memory. The caller zeroed cs's counters (and synchronized);
// with lane groups, nseq <= kChunkMaxSeqs.
__device__ __forceinline__ void run_chunk(const ProfDev &P, const uint32_t *stab, const uint32_t *mtab,
                                          const DbDev &db, int64_t s0, int64_t nseq, uint8_t *oxj, uint8_t *ofl,
                                          ChunkShared &cs) {
  const int lane = threadIdx.x & 31;
  if (P.G == 32) {
    for (;;) {
      unsigned k = 0;
      if (lane == 0) k = atomicAdd(&cs.next_seq, 1u);
      k = __shfl_sync(FULL, k, 0);
      if ((int64_t) k >= nseq) break;
      run_seq_any(P.C, P, stab, mtab, db, s0 + (int64_t) k, lane, oxj, ofl);
    }
    return;
  }
  ssv_group_chunk_any(P.G, P.Cg, P, stab, db, s0, (int) nseq, oxj, ofl, &cs.next_seq, cs.und, &cs.n_und);
  __syncthreads();                                   // the undecided list is complete
  const unsigned nu = cs.n_und;
  for (;;) {
    unsigned k = 0;
    if (lane == 0) k = atomicAdd(&cs.next_und, 1u);
    k = __shfl_sync(FULL, k, 0);
    if (k >= nu) break;
    run_seq_any(P.C, P, nullptr, mtab, db, s0 + (int64_t) cs.und[k], lane, oxj, ofl, true);
  }
}

// Stages a profile's SSV table (f16, 32-lane or lane-group layout) and MSV
// table into shared memory.
__device__ __forceinline__ void stage_tables(const ProfDev &P, uint32_t *smem) {
  const int C = P.C;
  const int sw = ssv_words(P), mw = NRES * ((C + 1) / 2) * 32;
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
