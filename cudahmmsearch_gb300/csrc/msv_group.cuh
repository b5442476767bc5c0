// msv_group.cuh -- SSV pass with G < 32 lanes per sequence.
//
// For small models a whole warp per sequence leaves each lane only a few DP
// words per row, so the per-row overhead (the shuffle, the residue decode,
// the table address) dominates. Here G lanes (8 or 16) score one sequence and
// a warp carries 32/G sequences in lockstep: each group owns its sequence
// state (index, row, residue word) and fetches the next sequence when its own
// ends, while all lanes execute the same row code every step (finished groups
// run pad rows, whose costs keep every cell at the floor). Lane g of a group
// owns nodes g*2C+1 .. (g+1)*2C with the same two-way striping as the 32-lane
// kernel. Only phase A (SSV) runs here; sequences SSV leaves undecided, or
// whose length disables SSV, are appended to a list that the 32-lane kernel
// then scores with the full MSV recurrence (list mode).
#pragma once
#include "msv_device.cuh"

namespace msvgb {

// Copies of the 8-byte and 4-byte table regions. A shared-memory access is
// served in phases of 128 bytes (8 lanes for 16-byte loads, 16 for 8-byte,
// 32 for 4-byte loads); with 8-byte loads at 8 lanes per group, or 4-byte
// loads at 8 or 16, one phase holds several groups, each reading its own
// residue's row, and two rows whose offsets meet on the same banks conflict.
// Those regions are therefore stored once per group of a phase, each copy on
// its own banks: group j of the phase reads copy j.
template <int G> struct GroupCopies {
  static constexpr int PAIR = G < 16 ? 16 / G : 1;       // 8-byte loads: groups per 16 lanes
  static constexpr int SINGLE = 32 / G;                   // 4-byte loads: groups per warp
};

template <int C, int G>
struct GroupLayout {
  static constexpr int Q4 = C / 4, R = C % 4;
  static constexpr int A_WORDS = NRES * Q4 * G * 4;                                    // quads [x][q][g][4]
  static constexpr int B_WORDS = (R >= 2) ? NRES * GroupCopies<G>::PAIR * G * 2 : 0;   // pair  [x][copy][g][2]
  static constexpr int C_WORDS = (R & 1) ? NRES * GroupCopies<G>::SINGLE * G : 0;      // single [x][copy][g]
  static constexpr int WORDS = A_WORDS + B_WORDS + C_WORDS;
};

template <int C, int G>
__device__ __forceinline__ void ssv_row_group(uint32_t (&dp)[C], uint32_t &acc0, uint32_t &acc1,
                                              const uint32_t *__restrict__ tab, int x, int glane, int gidx,
                                              int src_lane) {
  using Lay = GroupLayout<C, G>;
  using Cp = GroupCopies<G>;
  constexpr uint32_t one2 = 0x3C003C00u;
  uint32_t s[C];
#pragma unroll
  for (int q = 0; q < Lay::Q4; ++q) {
    const uint4 v = *reinterpret_cast<const uint4 *>(tab + ((x * Lay::Q4 + q) * G + glane) * 4);
    s[4 * q] = v.x; s[4 * q + 1] = v.y; s[4 * q + 2] = v.z; s[4 * q + 3] = v.w;
  }
  if constexpr (Lay::R >= 2) {
    const int cp = gidx % Cp::PAIR;
    const uint2 v = *reinterpret_cast<const uint2 *>(tab + Lay::A_WORDS + ((x * Cp::PAIR + cp) * G + glane) * 2);
    s[4 * Lay::Q4] = v.x; s[4 * Lay::Q4 + 1] = v.y;
  }
  if constexpr (Lay::R & 1) s[C - 1] = tab[Lay::A_WORDS + Lay::B_WORDS + (x * Cp::SINGLE + gidx) * G + glane];
  const uint32_t pred0 = pred_word0(dp[C - 1], src_lane);   // all 32 lanes, every row
#pragma unroll
  for (int w = C - 1; w >= 0; --w) dp[w] = fma_relu_f16x2(w ? dp[w - 1] : pred0, one2, s[w]);
  // the running maximum on the bits (non-negative f16 order like signed
  // integers), one three-input maximum per two words as in ssv_row_hyb
  if constexpr (C & 1) acc1 = max_s16x2(acc1, dp[C - 1]);
#pragma unroll
  for (int w = 0; w + 1 < C; w += 2) acc0 = __vimax3_s16x2(acc0, dp[w], dp[w + 1]);
}

// ---- mixed-width SSV table (f16 and 8-bit costs) ------------------------------
// The f16 row reads 2 bytes of cost per cell from shared memory and is bound
// by shared-memory bandwidth (one 128-byte wavefront per clock and SM) while
// the FMA and ALU pipes idle half the time. Here the last CI words of every
// lane keep their costs as bytes (1 byte per cell) and widen them in
// registers, trading shared-memory bytes for instructions on the idle pipes.
//
// Units: cells and costs are integers times 2^-24, i.e. f16 subnormals (and
// the smallest normals): an integer n with |n| < 2048 is exact, its bits are
// sign-magnitude (n < 0: 0x8000 | -n). A byte t is widened to a cost with one
// PRMT (t as the low byte of a zero high byte: t * 2^-24) and one f16 add of
// -128 units, so the table stores t = s + 128. Cell updates stay one
// fma.relu per word as in the f16 row, and they are exact for the same
// reason (integers below 2048 units; the relu clamps at 0). Non-negative f16
// bits order like signed 16-bit integers, so the running maximum is taken on
// the bits with integer instructions (ALU pipe) instead of f16 maxima (FMA
// pipe).
//
// Layout for residue x (CF = C - CI f16 words, CI a multiple of 4): the f16
// regions of GroupLayout<CF, G> (quads, pair, single), then 16-byte octets
// [x][o][g][4 words], then, when CI % 8 == 4, one 8-byte half octet
// [x][copy][g][2 words] (copies as GroupCopies): word k of octet o of lane g holds the bytes
// [t(w, h0), t(w+1, h0), t(w, h1), t(w+1, h1)] of DP words w = CF + 8o + 2k
// and w + 1 (the half octet: w = CF + 8 * NO + 2k).
template <int C, int CI, int G>
struct HybLayout {
  static_assert(CI % 4 == 0 && CI >= 4 && CI <= C, "8-bit words come in fours");
  static constexpr int CF = C - CI;
  static constexpr int Q4 = CF / 4, R = CF % 4, NO = CI / 8, HALF = (CI % 8) / 4;
  static constexpr int A_WORDS = NRES * Q4 * G * 4;
  static constexpr int B_WORDS = (R >= 2) ? NRES * GroupCopies<G>::PAIR * G * 2 : 0;
  static constexpr int C_WORDS = (R & 1) ? NRES * GroupCopies<G>::SINGLE * G : 0;
  static constexpr int D_WORDS = NRES * NO * G * 4;
  static constexpr int E_WORDS = NRES * HALF * GroupCopies<G>::PAIR * G * 2;   // [x][copy][g][2]
  static constexpr int WORDS = A_WORDS + B_WORDS + C_WORDS + D_WORDS + E_WORDS;
};

__device__ __forceinline__ uint32_t add_f16x2(uint32_t a, uint32_t b) {
  uint32_t d; asm("add.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d;
}

template <int C, int CI, int G>
__device__ __forceinline__ void ssv_row_hyb(uint32_t (&dp)[C], uint32_t &acc0, uint32_t &acc1,
                                            const uint32_t *__restrict__ tab, int x, int glane, int gidx,
                                            int src_lane) {
  using Lay = HybLayout<C, CI, G>;
  using Cp = GroupCopies<G>;
  constexpr int CF = Lay::CF;
  constexpr uint32_t one2 = 0x3C003C00u;        // f16x2 (1.0, 1.0)
  constexpr uint32_t m128 = 0x80808080u;        // f16x2 (-128, -128) units of 2^-24
  uint32_t s[C];
#pragma unroll
  for (int q = 0; q < Lay::Q4; ++q) {
    const uint4 v = *reinterpret_cast<const uint4 *>(tab + ((x * Lay::Q4 + q) * G + glane) * 4);
    s[4 * q] = v.x; s[4 * q + 1] = v.y; s[4 * q + 2] = v.z; s[4 * q + 3] = v.w;
  }
  if constexpr (Lay::R >= 2) {
    const int cp = gidx % Cp::PAIR;
    const uint2 v = *reinterpret_cast<const uint2 *>(tab + Lay::A_WORDS + ((x * Cp::PAIR + cp) * G + glane) * 2);
    s[4 * Lay::Q4] = v.x; s[4 * Lay::Q4 + 1] = v.y;
  }
  if constexpr (Lay::R & 1) s[CF - 1] = tab[Lay::A_WORDS + Lay::B_WORDS + (x * Cp::SINGLE + gidx) * G + glane];
  const uint32_t *td = tab + Lay::A_WORDS + Lay::B_WORDS + Lay::C_WORDS;
#pragma unroll
  for (int o = 0; o < Lay::NO; ++o) {
    const uint4 v = *reinterpret_cast<const uint4 *>(td + ((x * Lay::NO + o) * G + glane) * 4);
    const uint32_t tw[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      s[CF + 8 * o + 2 * k]     = add_f16x2(prmt(tw[k], 0u, 0x4240u), m128);   // bytes 0, 2
      s[CF + 8 * o + 2 * k + 1] = add_f16x2(prmt(tw[k], 0u, 0x4341u), m128);   // bytes 1, 3
    }
  }
  if constexpr (Lay::HALF) {
    const int cp = gidx % Cp::PAIR;
    const uint2 v = *reinterpret_cast<const uint2 *>(td + Lay::D_WORDS + ((x * Cp::PAIR + cp) * G + glane) * 2);
    const uint32_t tw[2] = {v.x, v.y};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      s[CF + 8 * Lay::NO + 2 * k]     = add_f16x2(prmt(tw[k], 0u, 0x4240u), m128);
      s[CF + 8 * Lay::NO + 2 * k + 1] = add_f16x2(prmt(tw[k], 0u, 0x4341u), m128);
    }
  }
  const uint32_t pred0 = pred_word0(dp[C - 1], src_lane);
#pragma unroll
  for (int w = C - 1; w >= 0; --w) dp[w] = fma_relu_f16x2(w ? dp[w - 1] : pred0, one2, s[w]);
  // running maximum on the bits (signed: a -0 from the relu is the smallest):
  // one three-input maximum per two words takes fewer issue slots than two
  // maxima, and issue, not the integer pipe, is what this row runs short of
  // (measured: 16.3 vs 17.0 ms at M = 400 on 2,000,000 sequences)
  if constexpr (C & 1) acc1 = max_s16x2(acc1, dp[C - 1]);
#pragma unroll
  for (int w = 0; w + 1 < C; w += 2) acc0 = __vimax3_s16x2(acc0, dp[w], dp[w + 1]);
}

// The group maximum of a hybrid accumulator as a float number of units
// (capped at 4096: above 2047 units values are not exact, and past the trust
// bound only "large" matters).
__device__ __forceinline__ float hyb_units(uint32_t acc) {
  const int lo = (int) (int16_t) (acc & 0xFFFFu), hi = (int) (int16_t) (acc >> 16);
  const int b = max(max(lo, hi), 0);
  if (b >= 0x7C00) return 4096.0f;                         // inf: far past any bound
  const float f = __half2float(__ushort_as_half((unsigned short) b)) * 16777216.0f;
  return fminf(f, 4096.0f);
}

struct GroupArgs {
  ProfDev P;                       // P.stab: the G-lane f16 SSV table
  DbDev db;
  uint8_t *out_xj, *out_flags;
  unsigned long long *ticket;
  int64_t *undecided;              // sorted indices left for the full MSV pass
  unsigned long long *n_undecided;
  int64_t s_begin = 0;             // first sorted sequence of the pass (the rest of the database follows)
  cudaStream_t stream;
};

constexpr uint32_t kPadWord = 0x1D1D1D1Du;   // four PAD_CODE residues

// The lockstep SSV loop of one warp. fetch() (called by lane 0 of a group)
// returns the next sorted sequence index, or a negative value when there is
// none; undecided(s) (lane 0 of a group) records a sequence that needs the full
// MSV. Decided sequences (and empty ones) are written to out_xj / out_flags.
// CI > 0: the mixed-width table (HybLayout<C, CI, G>, units of 2^-24).
template <int C, int G, int CI = 0, class Fetch, class Undecided>
__device__ __forceinline__ void ssv_group_loop(const ProfDev &P, const uint32_t *__restrict__ tab, const DbDev &db,
                                               uint8_t *__restrict__ out_xj, uint8_t *__restrict__ out_flags,
                                               Fetch fetch, Undecided undecided) {
  const int lane = threadIdx.x & 31, glane = lane % G, gbase = lane - glane, gidx = lane / G;
  const int src_lane = gbase + (glane + G - 1) % G;
  const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << gbase);
  const int tbm = P.tbm, tec = P.tec, base = P.base, bias = P.bias;

  int64_t s = 0;
  int L = 0, i = 0, tjb = 0;
  const uint32_t *sq = nullptr;
  uint32_t nextw = kPadWord;
  bool need = true, done = false;
  uint32_t dp[C];
  uint32_t acc0 = 0u, acc1 = 0u;
#pragma unroll
  for (int w = 0; w < C; ++w) dp[w] = 0u;

  for (;;) {
    if (need && !done) {                              // group-uniform: take the next sequence
      long long t = 0;
      if (glane == 0) t = fetch();
      t = __shfl_sync(gmask, t, gbase);
      if (t < 0) {
        done = true;
      } else {
        s = (int64_t) t;
        L = db.len[s];
        tjb = P.tjb[L];
        if (L == 0) {                                 // skipped, as p7_Pipeline does
          if (glane == 0) { const int64_t oi = db.orig[s]; out_xj[oi] = 0; out_flags[oi] = 0x08; }
        } else if (tjb + tbm + tec + bias >= 127) {   // SSV disabled for this length: full MSV
          if (glane == 0) undecided(s);
        } else {
          sq = reinterpret_cast<const uint32_t *>(db.codes + db.start[s]);
          nextw = __ldg(sq);
          i = 0;
          need = false;
#pragma unroll
          for (int w = 0; w < C; ++w) dp[w] = 0u;
          acc0 = acc1 = 0u;
        }
      }
    }
    if (__all_sync(FULL, done)) break;
    const bool active = !need && !done;
    const uint32_t w4 = active ? nextw : kPadWord;
    if (active && i + 4 < L) nextw = __ldg(sq + (i >> 2) + 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if constexpr (CI > 0) ssv_row_hyb<C, CI, G>(dp, acc0, acc1, tab, (w4 >> (8 * j)) & 0xFF, glane, gidx, src_lane);
      else                  ssv_row_group<C, G>(dp, acc0, acc1, tab, (w4 >> (8 * j)) & 0xFF, glane, gidx, src_lane);
    }
    i += 4;
    const bool fin = active && i >= L;
    if (__any_sync(FULL, fin)) {                      // group maxima (all lanes take part)
      float f;
      if constexpr (CI > 0) {
        f = hyb_units(max_s16x2(acc0, acc1));
      } else {
        const __half2 a = __hmax2(*reinterpret_cast<const __half2 *>(&acc0),
                                  *reinterpret_cast<const __half2 *>(&acc1));
        f = fminf(fmaxf(__low2float(a), __high2float(a)), 4096.0f);
      }
#pragma unroll
      for (int off = G / 2; off >= 1; off >>= 1) f = fmaxf(f, __shfl_xor_sync(FULL, f, off));
      if (fin) {
        int xj = 0;
        const int st = ssv_decide((int) f, tjb, tbm, tec, base, bias, xj);
        if (glane == 0) {
          if (st < 0) {
            undecided(s);
          } else {
            const int64_t oi = db.orig[s];
            int flags = 0;
            if (st == ST_ERANGE) flags |= 0x01 | 0x02;
            else if (xj >= P.xjmin[L]) flags |= 0x02;
            out_xj[oi] = (uint8_t) xj;
            out_flags[oi] = (uint8_t) flags;
          }
        }
        need = true;
      }
    }
  }
}

// Stand-alone SSV pass over the sorted sequences [s_begin, n) (global
// ticket); undecided sequences go to a global list for the full-MSV launch.
// Table words of a lane-group SSV table at run-time (Cg, G, CI): the layouts
// above (GroupLayout, or HybLayout when CI > 0) with their region copies.
__host__ __device__ constexpr int group_words(int Cg, int G, int CI) {
  return NRES * G * ((Cg - CI) / 4 * 4 + ((Cg - CI) % 4 >= 2 ? 2 * (G < 16 ? 16 / G : 1) : 0) +
                     (((Cg - CI) % 4) & 1 ? 32 / G : 0) + CI / 8 * 4 + ((CI % 8) / 4) * 2 * (G < 16 ? 16 / G : 1));
}

// Table words of the lane-group SSV pass: f16 (CI = 0) or mixed width.
template <int C, int G, int CI>
__host__ __device__ constexpr int group_table_words() {
  if constexpr (CI > 0) return HybLayout<C, CI, G>::WORDS;
  else return GroupLayout<C, G>::WORDS;
}

template <int C, int G, int CI = 0>
__global__ void __launch_bounds__(256)
msv_ssv_group_kernel(ProfDev P, DbDev db, uint8_t *__restrict__ out_xj, uint8_t *__restrict__ out_flags,
                     unsigned long long *__restrict__ ticket, int64_t *__restrict__ undecided,
                     unsigned long long *__restrict__ n_undecided, int64_t s_begin) {
  extern __shared__ __align__(16) uint32_t smem[];
  {
    const uint4 *gs = reinterpret_cast<const uint4 *>(P.stab);
    uint4 *ss = reinterpret_cast<uint4 *>(smem);
    for (int i = threadIdx.x; i < group_table_words<C, G, CI>() / 4; i += blockDim.x) ss[i] = __ldg(gs + i);
  }
  __syncthreads();
  const unsigned long long n = (unsigned long long) db.n;
  ssv_group_loop<C, G, CI>(
      P, smem, db, out_xj, out_flags,
      [&]() -> long long {
        const unsigned long long t = atomicAdd(ticket, 1ull) + (unsigned long long) s_begin;
        return t < n ? (long long) t : -1ll;
      },
      [&](int64_t s) { undecided[atomicAdd(n_undecided, 1ull)] = s; });
}

// SSV pass of one CTA over the sorted sequences [s0, s0 + nseq) (a work item
// of the multi-profile kernels): next_seq and n_und are shared counters the
// caller zeroed; und (room for nseq entries) receives the chunk-relative
// indices of the undecided sequences. CI > 0: the mixed-width table.
template <int C, int G, int CI = 0>
__device__ __forceinline__ void ssv_group_chunk(const ProfDev &P, const uint32_t *tab, const DbDev &db, int64_t s0,
                                                int nseq, uint8_t *oxj, uint8_t *ofl, unsigned *next_seq,
                                                uint16_t *und, unsigned *n_und) {
  ssv_group_loop<C, G, CI>(
      P, tab, db, oxj, ofl,
      [&]() -> long long {
        const unsigned k = atomicAdd(next_seq, 1u);
        return k < (unsigned) nseq ? (long long) (s0 + k) : -1ll;
      },
      [&](int64_t s) { und[atomicAdd(n_und, 1u)] = (uint16_t) (s - s0); });
}

template <int C, int G, int CI = 0>
cudaError_t launch_ssv_group(const GroupArgs &a, int num_sms) {
  auto kern = msv_ssv_group_kernel<C, G, CI>;
  static_assert(group_words(C, G, CI) == group_table_words<C, G, CI>(), "host and device table sizes agree");
  constexpr size_t smem = (size_t) group_table_words<C, G, CI>() * 4;
  static std::atomic<unsigned long long> configured{0};
  {
    cudaError_t e = ensure_smem_attr((const void *) kern, smem, configured);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
  if (e != cudaSuccess) return e;
  int grid = std::max(1, per_sm) * num_sms;
  const long long need = ((a.db.n - a.s_begin) * G + 255) / 256;   // 256 threads hold 256/G sequences
  if (need < grid) grid = (int) std::max(1LL, need);
  (void) cudaGetLastError();
  kern<<<grid, 256, smem, a.stream>>>(a.P, a.db, a.out_xj, a.out_flags, a.ticket, a.undecided, a.n_undecided,
                                      a.s_begin);
  return cudaGetLastError();
}

}  // namespace msvgb

#define MSVGB_INSTANTIATE_GROUP(C, G) \
  template cudaError_t msvgb::launch_ssv_group<C, G, 0>(const msvgb::GroupArgs &, int);
#define MSVGB_INSTANTIATE_HYB(C, G, CI) \
  template cudaError_t msvgb::launch_ssv_group<C, G, CI>(const msvgb::GroupArgs &, int);

namespace msvgb {

// ---- Full MSV (phase B) on lane groups -----------------------------------------
// The sequences SSV leaves undecided are scored with the full MSV recurrence
// (msvfilter.c:112-212) by the same lane groups, 32/G sequences per warp in
// lockstep, instead of one warp per sequence: a lane holds C words (2C cells)
// of its sequence's row, so the per-row work (shuffle, residue decode, the
// row maximum and the J/B updates) is spread over more cells.
//
// Cells are f16 in unit 1, exact: every value is an integer in [0, 255] and
// every sum below 255 + bias. The table (GroupLayout<C, G>, "MSV group
// table") holds c = bias - rbv unclamped, and bias - 255 for padding nodes and
// the pad residue, which keeps those cells at 0 (the previous row's overflow
// test bounds every cell below 255 - bias). Per cell, as msv_row does in
// 16-bit lanes: sv = max(max(mpv, xBc) + c, 0) with xBc = min(xB, 255 - bias).
template <int C, int G>
__device__ __forceinline__ uint32_t msv_row_group(uint32_t (&dp)[C], uint32_t xB2, const uint32_t *__restrict__ tab,
                                                  int x, int glane, int gidx, int src_lane) {
  using Lay = GroupLayout<C, G>;
  using Cp = GroupCopies<G>;
  constexpr uint32_t one2 = 0x3C003C00u;
  uint32_t s[C];
#pragma unroll
  for (int q = 0; q < Lay::Q4; ++q) {
    const uint4 v = *reinterpret_cast<const uint4 *>(tab + ((x * Lay::Q4 + q) * G + glane) * 4);
    s[4 * q] = v.x; s[4 * q + 1] = v.y; s[4 * q + 2] = v.z; s[4 * q + 3] = v.w;
  }
  if constexpr (Lay::R >= 2) {
    const int cp = gidx % Cp::PAIR;
    const uint2 v = *reinterpret_cast<const uint2 *>(tab + Lay::A_WORDS + ((x * Cp::PAIR + cp) * G + glane) * 2);
    s[4 * Lay::Q4] = v.x; s[4 * Lay::Q4 + 1] = v.y;
  }
  if constexpr (Lay::R & 1) s[C - 1] = tab[Lay::A_WORDS + Lay::B_WORDS + (x * Cp::SINGLE + gidx) * G + glane];
  const uint32_t pred0 = pred_word0(dp[C - 1], src_lane);
#pragma unroll
  for (int w = C - 1; w >= 0; --w) dp[w] = fma_relu_f16x2(max_f16x2(w ? dp[w - 1] : pred0, xB2), one2, s[w]);
  // the row maximum on the bits (non-negative f16 bits order like integers):
  // one three-input maximum per two words, in four short chains (the
  // maximum is on the critical path of the next row)
  uint32_t acc[4] = {0u, 0u, 0u, 0u};
#pragma unroll
  for (int w = 0; w + 1 < C; w += 2) acc[(w / 2) & 3] = __vimax3_s16x2(acc[(w / 2) & 3], dp[w], dp[w + 1]);
  if constexpr (C & 1) acc[3] = max_s16x2(acc[3], dp[C - 1]);
  return max_s16x2(max_s16x2(acc[0], acc[1]), max_s16x2(acc[2], acc[3]));
}

// Full MSV of the listed sequences list[*ticket .. *list_count) (taken one
// per group from the ticket), written as msv_search_kernel's list mode does.
template <int C, int G>
__global__ void __launch_bounds__(256)
msv_list_group_kernel(ProfDev P, DbDev db, uint8_t *__restrict__ out_xj, uint8_t *__restrict__ out_flags,
                      unsigned long long *__restrict__ ticket, const int64_t *__restrict__ list,
                      const unsigned long long *__restrict__ list_count) {
  extern __shared__ __align__(16) uint32_t smem[];
  {
    const uint4 *gs = reinterpret_cast<const uint4 *>(P.mtab);
    uint4 *ss = reinterpret_cast<uint4 *>(smem);
    for (int i = threadIdx.x; i < GroupLayout<C, G>::WORDS / 4; i += blockDim.x) ss[i] = __ldg(gs + i);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, glane = lane % G, gbase = lane - glane, gidx = lane / G;
  const int src_lane = gbase + (glane + G - 1) % G;
  const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << gbase);
  const int tbm = P.tbm, tec = P.tec, base = P.base, bias = P.bias;
  const unsigned long long cnt = *list_count;

  int64_t s = 0;
  int L = 0, i = 0, tjbm = 0, xJ = 0, xB = 0;
  const uint32_t *sq = nullptr;
  uint32_t nextw = kPadWord;
  bool need = true, done = false, er = false;
  uint32_t dp[C];
#pragma unroll
  for (int w = 0; w < C; ++w) dp[w] = 0u;

  for (;;) {
    if (need && !done) {                              // group-uniform: take the next listed sequence
      long long t = -1;
      if (glane == 0) {
        const unsigned long long k = atomicAdd(ticket, 1ull);
        if (k < cnt) t = list[k];
      }
      t = __shfl_sync(gmask, t, gbase);
      if (t < 0) {
        done = true;
      } else {
        s = (int64_t) t;
        L = db.len[s];
        tjbm = (P.tjb[L] + tbm) & 0xFF;               // (int8_t) tjb + (int8_t) tbm, splatted as bytes
        xJ = 0;
        xB = max(base - tjbm, 0);
        er = false;
        sq = reinterpret_cast<const uint32_t *>(db.codes + db.start[s]);
        nextw = __ldg(sq);
        i = 0;
        need = false;
#pragma unroll
        for (int w = 0; w < C; ++w) dp[w] = 0u;
      }
    }
    if (__all_sync(FULL, done)) break;
    const bool active = !need && !done;
    const uint32_t w4 = active ? nextw : kPadWord;
    if (active && i + 4 < L) nextw = __ldg(sq + (i >> 2) + 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t xb = (uint32_t) __half_as_ushort(__int2half_rn(min(xB, 255 - bias)));
      uint32_t a = msv_row_group<C, G>(dp, xb | (xb << 16), smem, (w4 >> (8 * j)) & 0xFF, glane, gidx, src_lane);
      int m = max((int) (a & 0xFFFFu), (int) (a >> 16));   // f16 bits of values in [0, 255]
#pragma unroll
      for (int off = G / 2; off >= 1; off >>= 1) m = max(m, __shfl_xor_sync(FULL, m, off));
      const int xE = (int) __half2float(__ushort_as_half((unsigned short) m));
      if (active && !er && i + j < L) {               // rows past the end change nothing
        if (xE + bias >= 255) er = true;              // adds(xE, bias) == 255: +inf
        else {
          xJ = max(xJ, max(xE - tec, 0));
          xB = max(max(base, xJ) - tjbm, 0);
        }
      }
    }
    i += 4;
    if (active && (er || i >= L)) {
      if (glane == 0) {
        const int64_t oi = db.orig[s];
        int flags = 0x04;
        if (er) flags |= 0x01 | 0x02;
        else if (xJ >= P.xjmin[L]) flags |= 0x02;
        out_xj[oi] = (uint8_t) (er ? 255 : xJ);
        out_flags[oi] = (uint8_t) flags;
      }
      need = true;
    }
  }
}

template <int C, int G>
cudaError_t launch_list_group(const ProfDev &P, const DbDev &db, uint8_t *out_xj, uint8_t *out_flags,
                              unsigned long long *ticket, const int64_t *list, const unsigned long long *list_count,
                              int num_sms, cudaStream_t stream) {
  auto kern = msv_list_group_kernel<C, G>;
  constexpr size_t smem = (size_t) GroupLayout<C, G>::WORDS * 4;
  static std::atomic<unsigned long long> configured{0};
  {
    cudaError_t e = ensure_smem_attr((const void *) kern, smem, configured);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
  if (e != cudaSuccess) return e;
  (void) cudaGetLastError();
  kern<<<std::max(1, per_sm) * num_sms, 256, smem, stream>>>(P, db, out_xj, out_flags, ticket, list, list_count);
  return cudaGetLastError();
}

}  // namespace msvgb

#define MSVGB_INSTANTIATE_LIST(C, G)                                                                       \
  template cudaError_t msvgb::launch_list_group<C, G>(const msvgb::ProfDev &, const msvgb::DbDev &, uint8_t *, \
                                                      uint8_t *, unsigned long long *, const int64_t *,      \
                                                      const unsigned long long *, int, cudaStream_t);
