// msv_device.cuh -- MSV filter kernels for sm_103a (GB300).
//
// One warp scores one (profile, sequence) pair. The 32 lanes split the model:
// lane l owns nodes l*2C+1 .. (l+1)*2C, held as C 32-bit words of two 16-bit
// cells. Inside a lane the nodes are striped two ways: DP word w, half h holds
// node  l*2C + h*C + w + 1,  so the diagonal predecessor of (w,h) is (w-1,h);
// only word 0 needs a neighbour: (C-1, 0) of its own lane for h=1 and, through
// one warp shuffle, (C-1, 1) of lane l-1 for h=0. Per row and lane that is one
// SHFL and one PRMT, then C words of pure packed arithmetic.
//
// Phase A is the SSV filter of the reference (src/impl_sse/ssvfilter.c:1364-1413):
// the J-free recurrence u(i,k) = max(u(i-1,k-1) + bias - rbv[x_i][k], 0), with
// u = v - (base - tjb - tbm) the cell value above the constant begin score,
// and its decision logic. Phase B, only where SSV is undecided, is the full
// MSV recurrence with the J state (src/impl_sse/msvfilter.c:112-212) in exact
// uint8-saturating semantics carried in 16-bit lanes.
//
// Exactness notes (proved in the comments at each step):
//  * SSV: trusted cells are u < 127-bias; the reference only trusts those too and
//    detects larger ones through xE >= 255-bias. s = bias-rbv is clamped to
//    [-128,127], which changes no cell below 128.
//  * MSV: sat_add(max(mpv,xB),bias) never clips before the row whose overflow
//    test fires, except through xB; clamping xB to 255-bias per row reproduces it.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace msvgb {

constexpr int NRES = 30;       // residue slots in device tables: codes 0..28, pad 29
constexpr int PAD_CODE = 29;   // padding residue after a sequence's end: floor costs everywhere
constexpr unsigned FULL = 0xffffffffu;

// Status codes carried from device to host.
enum : int { ST_OK = 0, ST_ERANGE = 1 };

struct ProfDev {
  int      M;
  int      C;            // DP words per lane of the 32-lane kernels: the warp covers 64*C nodes > M
  int      tbm, tec, base, bias;
  const uint32_t *stab;  // SSV costs, see layout_ssv_*() in the host code
  const uint32_t *mtab;  // MSV costs, 255 - rbv, uint8x4 [NRES][C/2][32]
  const uint8_t  *tjb;   // [Lmax+1] tjb_b per target length
  const uint8_t  *xjmin; // [Lmax+1] smallest passing xJ per length (255: xJ never passes)
  int      ssv_f16;      // 1: stab is f16x2 [NRES][C][32]; 0: int8x4 [NRES][C/2][32]
  int      G = 32;       // lanes per sequence of the SSV pass; < 32: stab is the lane-group table
  int      Cg = 0;       // DP words per lane of the lane-group SSV pass (G < 32)
  int      CI = 0;       // of those, words with 8-bit costs (mixed-width table, HybLayout); 0: f16 table
};

struct DbDev {
  const uint8_t  *codes;   // packed residues, every sequence starts 16-byte aligned
  const int64_t  *start;   // byte offset of sorted sequence s
  const int32_t  *len;     // length of sorted sequence s
  const int64_t  *orig;    // original index of sorted sequence s
  int64_t         n;
};

// ---- packed 16-bit integer helpers (native on sm_90+) ------------------------
__device__ __forceinline__ uint32_t add_s16x2(uint32_t a, uint32_t b) {
  uint32_t d; asm("add.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d;
}
__device__ __forceinline__ uint32_t max_s16x2(uint32_t a, uint32_t b) {
  uint32_t d; asm("max.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d;
}
__device__ __forceinline__ uint32_t max_relu_s16x2(uint32_t a, uint32_t b) {
  uint32_t d; asm("max.relu.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d;
}
__device__ __forceinline__ uint32_t min_s16x2(uint32_t a, uint32_t b) {
  uint32_t d; asm("min.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d;
}
// prmt with the sign-replicate bit honoured (bit 3 of each selector nibble).
__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
  uint32_t d; asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel)); return d;
}
// ---- packed f16 helpers (exact on integers of magnitude <= 2048) ---------------
__device__ __forceinline__ uint32_t fma_relu_f16x2(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d; asm("fma.rn.relu.f16x2 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c)); return d;
}
__device__ __forceinline__ uint32_t max_f16x2(uint32_t a, uint32_t b) {
  uint32_t d; asm("max.f16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b)); return d;
}

// Diagonal predecessor of DP word 0: low half <- high half of lane-1's word C-1,
// high half <- low half of this lane's word C-1. Lane 0 reads lane 31, whose
// last node 64*C is always a padding node (the host picks C with 64*C > M):
// its cell is 0 -- the begin/floor value node 0 must supply -- in phase B
// always, and in phase A whenever no cell has reached the overflow bound
// (after that the outcome no longer depends on any cell value).
__device__ __forceinline__ uint32_t pred_word0(uint32_t last, int src_lane) {
  const uint32_t up = __shfl_sync(FULL, last, src_lane);
  return prmt(last, up, 0x1076u);  // bytes [up.b2, up.b3, last.b0, last.b1]
}

// ---- Phase A: SSV row, int8 table unpacked by sign-extending prmt ---------------
// Table word (x, p, lane) bytes: [s(2p,h0), s(2p+1,h0), s(2p,h1), s(2p+1,h1)].
template <int C>
__device__ __forceinline__ void ssv_row_i8(uint32_t (&dp)[C], uint32_t &acc0, uint32_t &acc1,
                                           const uint32_t *__restrict__ t, int src_lane) {
  static_assert(C % 2 == 0, "the int8 table packs two DP words per table word");
  const uint32_t pred0 = pred_word0(dp[C - 1], src_lane);
#pragma unroll
  for (int p = C / 2 - 1; p >= 0; --p) {
    const uint32_t tw = t[p * 32];
    const uint32_t sA = prmt(tw, 0u, 0xA280u);   // [b0, sign(b0), b2, sign(b2)]
    const uint32_t sB = prmt(tw, 0u, 0xB391u);   // [b1, sign(b1), b3, sign(b3)]
    dp[2 * p + 1] = max_relu_s16x2(add_s16x2(dp[2 * p], sB), 0u);
    dp[2 * p]     = max_relu_s16x2(add_s16x2(p ? dp[2 * p - 1] : pred0, sA), 0u);
    acc1 = max_s16x2(acc1, dp[2 * p + 1]);
    acc0 = max_s16x2(acc0, dp[2 * p]);
  }
}

// ---- Phase A: SSV row, f16 table ----------------------------------------------
// One f16x2 cost word per DP word. For residue x the lane's C words sit in
// up to three lane-contiguous regions so that every load is a conflict-free
// vector load: quads [x][q][lane][4] (LDS.128), then a pair [x][lane][2]
// (LDS.64) if C%4 >= 2, then a single [x][lane] (LDS.32) if C is odd.
template <int C>
struct F16Layout {
  static constexpr int Q4 = C / 4, R = C % 4;
  static constexpr int A_WORDS = NRES * Q4 * 32 * 4;                 // quads
  static constexpr int B_WORDS = (R >= 2) ? NRES * 32 * 2 : 0;       // pair
  static constexpr int C_WORDS = (R & 1) ? NRES * 32 : 0;            // single
  static constexpr int WORDS = A_WORDS + B_WORDS + C_WORDS;          // == NRES * 32 * C
};

template <int C>
__device__ __forceinline__ void ssv_row_f16(uint32_t (&dp)[C], uint32_t &acc0, uint32_t &acc1,
                                            const uint32_t *__restrict__ tab, int x, int lane, int src_lane) {
  using Lay = F16Layout<C>;
  constexpr uint32_t one2 = 0x3C003C00u;        // f16x2 (1.0, 1.0)
  auto cell = [&](int w, uint32_t sw, uint32_t pred0) {
    dp[w] = fma_relu_f16x2(w ? dp[w - 1] : pred0, one2, sw);
    if (w & 1) acc1 = max_f16x2(acc1, dp[w]); else acc0 = max_f16x2(acc0, dp[w]);
  };
  if constexpr (C <= 64) {
    // all of the row's costs are loaded first (latency hidden behind the row)
    uint32_t s[C];
#pragma unroll
    for (int q = 0; q < Lay::Q4; ++q) {
      const uint4 v = *reinterpret_cast<const uint4 *>(tab + ((x * Lay::Q4 + q) * 32 + lane) * 4);
      s[4 * q] = v.x; s[4 * q + 1] = v.y; s[4 * q + 2] = v.z; s[4 * q + 3] = v.w;
    }
    if constexpr (Lay::R >= 2) {
      const uint2 v = *reinterpret_cast<const uint2 *>(tab + Lay::A_WORDS + (x * 32 + lane) * 2);
      s[4 * Lay::Q4] = v.x; s[4 * Lay::Q4 + 1] = v.y;
    }
    if constexpr (Lay::R & 1) s[C - 1] = tab[Lay::A_WORDS + Lay::B_WORDS + x * 32 + lane];
    const uint32_t pred0 = pred_word0(dp[C - 1], src_lane);
#pragma unroll
    for (int w = C - 1; w >= 0; --w) cell(w, s[w], pred0);
    return;
  }
  // rows wider than 64 words: words are updated from the highest down (dp[w]
  // reads the old dp[w-1]) and each table region is loaded just before its
  // words, so only the DP row and one quad of costs are live (no spills)
  const uint32_t pred0 = pred_word0(dp[C - 1], src_lane);
  if constexpr (Lay::R & 1) cell(C - 1, tab[Lay::A_WORDS + Lay::B_WORDS + x * 32 + lane], pred0);
  if constexpr (Lay::R >= 2) {
    const uint2 v = *reinterpret_cast<const uint2 *>(tab + Lay::A_WORDS + (x * 32 + lane) * 2);
    cell(4 * Lay::Q4 + 1, v.y, pred0);
    cell(4 * Lay::Q4, v.x, pred0);
  }
#pragma unroll
  for (int q = Lay::Q4 - 1; q >= 0; --q) {
    const uint4 v = *reinterpret_cast<const uint4 *>(tab + ((x * Lay::Q4 + q) * 32 + lane) * 4);
    cell(4 * q + 3, v.w, pred0);
    cell(4 * q + 2, v.z, pred0);
    cell(4 * q + 1, v.y, pred0);
    cell(4 * q, v.x, pred0);
  }
}

// ---- Phase B: full MSV row (exact uint8 semantics in 16-bit lanes) ----------------
// Table word bytes n = 255 - rbv in the same byte order as the SSV int8 table.
//   sv = sat_sub(sat_add(max(mpv, xB), bias), rbv) = max(max(mpv, xBc) + n + (bias-255), 0)
// with xBc = min(xB, 255-bias): mpv + bias < 255 always holds here because the
// previous row's overflow test (xE + bias >= 255 -> ERANGE) did not fire.
template <int C>
__device__ __forceinline__ uint32_t msv_row(uint32_t (&dp)[C], uint32_t xBp, uint32_t kneg,
                                            const uint32_t *__restrict__ t, int src_lane) {
  constexpr int NP = (C + 1) / 2;                 // table words per lane: 4 nodes each
  const uint32_t pred0 = pred_word0(dp[C - 1], src_lane);
  uint32_t acc0 = 0u, acc1 = 0u;
#pragma unroll
  for (int p = NP - 1; p >= 0; --p) {
    const uint32_t tw = t[p * 32];
    const uint32_t nA = tw & 0x00FF00FFu;          // bytes 0,2 zero-extended
    const uint32_t nB = (tw >> 8) & 0x00FF00FFu;   // bytes 1,3 zero-extended
    // halves of max(..) and n are <= 255: a 32-bit add cannot carry across halves
    if (2 * p + 1 < C) {
      dp[2 * p + 1] = max_relu_s16x2(add_s16x2(max_s16x2(dp[2 * p], xBp) + nB, kneg), 0u);
      acc1 = max_s16x2(acc1, dp[2 * p + 1]);
    }
    dp[2 * p] = max_relu_s16x2(add_s16x2(max_s16x2(p ? dp[2 * p - 1] : pred0, xBp) + nA, kneg), 0u);
    acc0 = max_s16x2(acc0, dp[2 * p]);
  }
  const uint32_t a = max_s16x2(acc0, acc1);
  return max(a & 0xFFFFu, a >> 16);               // halves are in [0,255]
}

// Scores one (profile, sequence). Returns status; *xj_out the final xJ;
// *full_out whether phase B ran.
// Decision logic of p7_SSVFilter (ssvfilter.c:1364-1413) from the maximum
// cell u_max of the J-free recurrence, in the reference's own uint16
// arithmetic. The reference's xE is the max over cells of the unsigned byte
// (u+128); any cell with u >= 127-bias makes it >= 255-bias (first-crossing
// argument: a diagonal rises by at most bias per step), otherwise xE = u_max+128.
// Returns ST_OK / ST_ERANGE, or -1 when SSV is undecided.
__device__ __forceinline__ int ssv_decide(int umax, int tjb, int tbm, int tec, int base, int bias, int &xj_out) {
  const int d = base - tjb - tbm;
  if (umax >= 127 - bias) {
    if (d >= 128) { xj_out = 255; return ST_ERANGE; }
    return -1;                                   // the plain MSV may not overflow
  }
  uint16_t xE = (uint16_t) (umax + 128);
  xE = (uint16_t) (xE + base - tjb - tbm);
  xE = (uint16_t) (xE - 128);
  if (xE >= 255 - bias) { xj_out = 255; return ST_ERANGE; }
  const uint16_t xJ = (uint16_t) (xE - tec);
  if (xJ <= base) { xj_out = xJ; return ST_OK; }
  return -1;                                     // the J state could have been used
}

template <int C, bool F16>
__device__ __forceinline__ int msv_one(const ProfDev &P, const uint32_t *__restrict__ stab,
                                       const uint32_t *__restrict__ mtab,
                                       const uint32_t *__restrict__ sq, int L, int lane,
                                       int &xj_out, int &full_out, bool skip_ssv = false) {
  const int tjb  = P.tjb[L];
  const int tbm  = P.tbm, tec = P.tec, base = P.base, bias = P.bias;
  full_out = 0;

  // ---------- Phase A: SSV (ssvfilter.c:1364-1413) ----------
  if (!skip_ssv && tjb + tbm + tec + bias < 127) {
    uint32_t dp[C];
#pragma unroll
    for (int w = 0; w < C; ++w) dp[w] = 0u;
    uint32_t acc0 = 0u, acc1 = 0u;
    const int src_lane = (lane + 31) & 31;
    uint32_t nextw = (L > 0) ? __ldg(sq) : 0u;
    for (int i0 = 0; i0 < L; i0 += 4) {
      const uint32_t w4 = nextw;
      if (i0 + 4 < L) nextw = __ldg(sq + (i0 >> 2) + 1);
      // Rows past L hold PAD_CODE, whose costs keep every cell at the floor:
      // processing them cannot raise the running maximum.
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int x = (w4 >> (8 * j)) & 0xFF;
        if constexpr (F16) ssv_row_f16<C>(dp, acc0, acc1, stab, x, lane, src_lane);
        else               ssv_row_i8<C>(dp, acc0, acc1, stab + lane + x * ((C / 2) * 32), src_lane);
      }
    }
    int umax;
    if constexpr (F16) {
      const __half2 a = __hmax2(*reinterpret_cast<const __half2 *>(&acc0),
                                *reinterpret_cast<const __half2 *>(&acc1));
      float f = fmaxf(__low2float(a), __high2float(a));
      f = fminf(f, 4096.0f);                      // garbage above the trust bound stays large
      umax = (int) f;
    } else {
      const uint32_t a = max_s16x2(acc0, acc1);
      const int lo = (int) (int16_t) (a & 0xFFFFu), hi = (int) (int16_t) (a >> 16);
      umax = max(max(lo, hi), 0);
    }
    umax = (int) __reduce_max_sync(FULL, (unsigned) umax);

    const int st = ssv_decide(umax, tjb, tbm, tec, base, bias, xj_out);
    if (st >= 0) return st;
  }

  // ---------- Phase B: full MSV (msvfilter.c:112-212) ----------
  full_out = 1;
  uint32_t dp[C];
#pragma unroll
  for (int w = 0; w < C; ++w) dp[w] = 0u;
  const int tjbm = (tjb + tbm) & 0xFF;                 // (int8_t) tjb + (int8_t) tbm, splatted as bytes
  int xJ = 0, xB = max(base - tjbm, 0);
  const uint32_t kneg = ((uint32_t) (bias - 255) & 0xFFFFu) * 0x00010001u;
  const uint32_t *tl = mtab + lane;
  const int src_lane = (lane + 31) & 31;
  uint32_t nextw = (L > 0) ? __ldg(sq) : 0u;
  for (int i0 = 0; i0 < L; i0 += 4) {
    const uint32_t w4 = nextw;
    if (i0 + 4 < L) nextw = __ldg(sq + (i0 >> 2) + 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (i0 + j < L) {
        const int x = (w4 >> (8 * j)) & 0xFF;
        const uint32_t xBp = (uint32_t) min(xB, 255 - bias) * 0x00010001u;
        uint32_t r = msv_row<C>(dp, xBp, kneg, tl + x * (((C + 1) / 2) * 32), src_lane);
        const int xE = (int) __reduce_max_sync(FULL, r);
        if (xE + bias >= 255) { xj_out = 255; return ST_ERANGE; }   // adds(xE,bias)==255
        xJ = max(xJ, max(xE - tec, 0));
        xB = max(max(base, xJ) - tjbm, 0);
      }
    }
  }
  xj_out = xJ;
  return ST_OK;
}

// The dynamic shared memory opt-in of a kernel, once per device (the
// attribute belongs to the current device's context).
inline cudaError_t ensure_smem_attr(const void *kern, size_t smem, std::atomic<unsigned long long> &done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
  return e;
}

}  // namespace msvgb
