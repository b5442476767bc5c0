// msv_vit.cu -- the stage after MSV: p7_ViterbiFilter on the GPU.
//
// The reference runs the striped int16 Viterbi filter (src/impl_sse/
// vitfilter.c:84-250) on the CPU for every sequence that passes the MSV and
// bias gates (src/p7_pipeline.c:694-702). Here one warp scores one listed
// sequence of a resident database in model-node order: lane l owns nodes
// l*CV+1 .. (l+1)*CV (the reference's striping, 8 lanes of Q8 = max(2,
// ceil(M/8)) vectors, is a permutation of the same 8*Q8 nodes, padding
// included, so every cell, xE and the lazy-F bound see the same values). Per
// row and node, with signed 16-bit saturation (_mm_adds_epi16 semantics):
//   M(i,k) = sat(max(sat(xB+tBM), sat(M'(k-1)+tMM), sat(I'(k-1)+tIM),
//                    sat(D'(k-1)+tDM)) + e(k,x_i))
//   I(i,k) = max(sat(M'(k)+tMI), sat(I'(k)+tII))
//   D(i,k) = sat(M(i,k-1)+tMD), closed under D->D only when
//            max_k D + ddbound > xB (the reference's lazy F).
// The D->D closure is a (max,+) recurrence whose costs are <= 0, so it has
// no upper saturation and composes: each lane's block is max(c, v + b), and
// a 5-step warp scan hands every lane its incoming value. Special states are
// C int arithmetic stored to int16_t, as the reference's are. The kernel
// returns the final xC (or overflow); the score and the per-length N/J/C
// move costs (p7_oprofile_ReconfigRestLength, p7_oprofile.c:944-962) are
// computed on the host with the reference's float expressions.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using namespace msvgb;
using msvgb_detail::fail;

namespace {

constexpr int kNT = 8;     // per-node transitions: BM MM IM DM (into k), MD MI II (out of k), DD into k

// Cost tables are lane-interleaved 16-byte vectors, the 32 lanes' vectors v
// adjacent so that one warp load reads 512 contiguous bytes. Emissions are
// int16 (vector v of a lane: its nodes 8v .. 8v+7), one unpack per cell,
// which keeps the 29 residue tables of the widest model within L1.
// Transitions are int32 (nodes 4v .. 4v+3), ready for the adds, in the
// one-node-per-register kernel (up to 32 nodes per lane); the shared-memory
// kernel (above 48) reads them as int16 (8 nodes per vector); the packed
// kernel (40, 48) has its own tables.
struct VitDev {
  int CV;                  // nodes per lane
  int16_t base_w, ddbound_w;
  int16_t xwE_move, xwE_loop, xwN_loop, xwJ_loop, xwC_loop;
  const void *trans;       // [kNT][NT][32] vectors of int32 (4 nodes) or int16 (8 nodes)
  const uint4 *emit;       // [NRES][NV][32]
  const int16_t *move;     // [Lmax+1]: N/J/C move cost at target length L
};

__host__ __device__ constexpr int vit_nv(int CV) { return (CV + 7) / 8; }
__host__ __device__ constexpr bool vit_t32(int CV) { return CV <= 32; }
// nodes per transition vector and vectors per lane
__host__ __device__ constexpr int vit_tnodes(int CV) { return vit_t32(CV) ? 4 : 8; }
__host__ __device__ constexpr int vit_nt(int CV) { return (CV + vit_tnodes(CV) - 1) / vit_tnodes(CV); }

__device__ __forceinline__ int i32(const int4 &w, int e) { return e == 0 ? w.x : e == 1 ? w.y : e == 2 ? w.z : w.w; }

__device__ __forceinline__ int sat16(int v) { return min(32767, max(-32768, v)); }

// a + b as an integer multiply-add by a register holding 1 (which the
// compiler cannot fold): it issues on the FMA pipe, leaving the ALU pipe --
// the one the max/clamp operations saturate -- to the rest
__device__ __forceinline__ int add_f(int a, int b, int one) {
  int r;
  asm("mad.lo.s32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(one), "r"(b));
  return r;
}

// signed 16-bit element e (0..7) of a vector
__device__ __forceinline__ int h16(const uint4 &w, int e) {
  const uint32_t u = e < 2 ? w.x : e < 4 ? w.y : e < 6 ? w.z : w.w;
  return (e & 1) ? ((int) u >> 16) : (int) (int16_t) (u & 0xffffu);
}

// Saturation is monotone, so max(sat(a), sat(b)) = sat(max(a, b)); every
// transition cost is <= 0, so a sum of a stored int16 score and a transition
// can only leave the range downwards: one clamp per cell value instead of
// one per sum. Only the emission can raise a score.
template <int CV>
__device__ int vit_one(const VitDev &V, const uint8_t *sq, int L, int lane, int &xc_out) {
  static_assert(vit_t32(CV), "the one-node-per-register row reads int32 transitions");
  constexpr int NV = vit_nv(CV), NT = vit_nt(CV), TN = vit_tnodes(CV);
  int Mv[CV], Iv[CV], Dv[CV];
#pragma unroll
  for (int j = 0; j < CV; ++j) Mv[j] = Iv[j] = Dv[j] = -32768;
  const int move = V.move[L];
  int xN = V.base_w;
  int xB = (int16_t) (xN + move), xJ = -32768, xC = -32768;
  for (int i = 0; i < L; ++i) {
    const int x = sq[i];
    const uint4 *em = V.emit + (size_t) x * NV * 32 + lane;
    // the transition costs are read anew each row (from L1): kept in
    // registers across rows they would crowd out the DP state
    int opaque, one;
    asm volatile("mov.u32 %0, 0;" : "=r"(opaque));
    asm volatile("mov.u32 %0, 1;" : "=r"(one));
    const int4 *tr = static_cast<const int4 *>(V.trans) + lane + opaque;
    // predecessors of this lane's first node: the previous lane's last node (old row)
    int pM = __shfl_up_sync(FULL, Mv[CV - 1], 1), pI = __shfl_up_sync(FULL, Iv[CV - 1], 1),
        pD = __shfl_up_sync(FULL, Dv[CV - 1], 1);
    if (lane == 0) pM = pI = pD = -32768;
    int xe = -32768, dmax = -32768, dc = -32768;
    uint4 e4;                                       // emission vector of nodes 8*(j/8) ..
#pragma unroll
    for (int q = 0; q < NT; ++q) {                  // transition vector q: nodes TN*q ..
      int4 t4[7];
#pragma unroll
      for (int t = 0; t < 7; ++t) t4[t] = tr[(t * NT + q) * 32];
#pragma unroll
      for (int e = 0; e < TN; ++e) {
        const int j = q * TN + e;
        if (j >= CV) break;
        if (j % 8 == 0) e4 = em[(j / 8) * 32];
        auto tv = [&](int t) { return i32(t4[t], e); };
        const int cM = Mv[j], cI = Iv[j], cD = Dv[j];
        int sv = max(max(add_f(xB, tv(0), one), pM + tv(1)), max(add_f(pI, tv(2), one), pD + tv(3)));
        sv = sat16(max(sv, -32768) + h16(e4, j % 8));
        xe = max(xe, sv);
        Mv[j] = sv;
        Iv[j] = max(max(cM + tv(5), add_f(cI, tv(6), one)), -32768);
        Dv[j] = dc;                                 // M->D from node k-1 (the delayed store)
        dc = max(add_f(sv, tv(4), one), -32768);
        dmax = max(dmax, dc);
        pM = cM; pI = cI; pD = cD;
      }
    }
    // the first node's M->D comes from the previous lane's last node
    const int dprev = __shfl_up_sync(FULL, dc, 1);
    Dv[0] = lane == 0 ? -32768 : dprev;
    xe = __reduce_max_sync(FULL, xe);
    dmax = __reduce_max_sync(FULL, dmax);
    if (xe >= 32767) { xc_out = 32767; return 1; }  // eslERANGE
    xN = (int16_t) (xN + V.xwN_loop);
    xC = (int16_t) max(xC + V.xwC_loop, xe + V.xwE_move);
    xJ = (int16_t) max(xJ + V.xwJ_loop, xe + V.xwE_loop);
    xB = (int16_t) max(xJ + move, xN + move);
    if (dmax + V.ddbound_w > xB) {                  // D->D closure over all nodes
      // this lane's block as max(c, v + b) of the incoming value v
      int tdd[CV];
#pragma unroll
      for (int q = 0; q < NT; ++q) {
        const int4 t7 = tr[(7 * NT + q) * 32];      // D(k-1) -> D(k)
#pragma unroll
        for (int e = 0; e < TN; ++e)
          if (q * TN + e < CV) tdd[q * TN + e] = i32(t7, e);
      }
      int c = -2000000000, b = 0;
#pragma unroll
      for (int j = 0; j < CV; ++j) {
        c = max(Dv[j], c + tdd[j]);
        b += tdd[j];
        if (b < -2000000) b = -2000000;             // far below any value: keeps the sums in range
      }
      // exclusive warp scan of the blocks: (c1,b1) then (c2,b2) = (max(c2, c1+b2), b1+b2)
      int sc_c = c, sc_b = b;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int oc = __shfl_up_sync(FULL, sc_c, d), ob = __shfl_up_sync(FULL, sc_b, d);
        if (lane >= d) { sc_c = max(sc_c, oc + sc_b); sc_b = max(ob + sc_b, -2000000); }
      }
      int vin = __shfl_up_sync(FULL, sc_c, 1);
      if (lane == 0) vin = -2000000000;
#pragma unroll
      for (int j = 0; j < CV; ++j) {
        Dv[j] = max(Dv[j], vin + tdd[j]);
        vin = Dv[j];
      }
    }
  }
  xc_out = xC;
  return 0;
}

// ---- packed form: two nodes per 32-bit word ------------------------------------
// Lane l owns nodes l*CV+1 .. (l+1)*CV as W = CV/2 words; word w holds node
// l*CV + w + 1 in its low half and node l*CV + W + w + 1 in its high half, so
// the predecessors of word w are word w-1 (both halves) and, for word 0, the
// previous lane's last node (low half) and this lane's word W-1 low half
// (high half). Every operation is a 16x2 SIMD instruction on both nodes. A
// saturating add of a cost t <= 0 is add(max(v, -32768 - t), t) with the bound
// from a table; the emission add clamps between -32768 - min(e, 0) =
// ~(min(e, 0) + 32767) and 32767 - max(e, 0) = max(e, 0) ^ 0x7fff.
// Tables: uint4 vectors of 4 words, [table][NV4][32]: the 7 costs BM MM IM DM
// MD MI II, their 7 bounds, DD into the node; emissions [NRES][NV4][32].
constexpr int kPT = 15;
__host__ __device__ constexpr int vitp_nv4(int CV) { return (CV / 2 + 3) / 4; }

__device__ __forceinline__ uint32_t v2add(uint32_t a, uint32_t b) { return add_s16x2(a, b); }
__device__ __forceinline__ uint32_t v2max(uint32_t a, uint32_t b) { return max_s16x2(a, b); }
__device__ __forceinline__ uint32_t v2min(uint32_t a, uint32_t b) { return min_s16x2(a, b); }
__device__ __forceinline__ uint32_t u4w(const uint4 &v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }
__device__ __forceinline__ int lo16(uint32_t x) { return (int) (int16_t) (x & 0xffffu); }
__device__ __forceinline__ int hi16(uint32_t x) { return (int) x >> 16; }
__device__ __forceinline__ uint32_t set_lo(uint32_t x, int v) { return __byte_perm(x, (uint32_t) v, 0x3254); }
__device__ __forceinline__ uint32_t set_hi(uint32_t x, int v) { return __byte_perm(x, (uint32_t) v, 0x5410); }

template <int CV>
__device__ int vitp_one(const VitDev &V, const uint8_t *sq, int L, int lane, int &xc_out) {
  constexpr int W = CV / 2, NV4 = vitp_nv4(CV);
  constexpr uint32_t FLOOR = 0x80008000u;
  uint32_t Mv[W], Iv[W], Dv[W];
#pragma unroll
  for (int w = 0; w < W; ++w) Mv[w] = Iv[w] = Dv[w] = FLOOR;
  const int move = V.move[L];
  int xN = V.base_w;
  int xB = (int16_t) (xN + move), xJ = -32768, xC = -32768;
  for (int i = 0; i < L; ++i) {
    const int x = sq[i];
    const uint4 *em = V.emit + (size_t) x * NV4 * 32 + lane;
    int opaque;
    asm volatile("mov.u32 %0, 0;" : "=r"(opaque));
    const uint4 *tr = static_cast<const uint4 *>(V.trans) + lane + opaque;
    const uint32_t xBp = (uint32_t) (xB & 0xffff) * 0x10001u;
    // predecessors of word 0 (old row): previous lane's last node, this lane's word W-1 low half
    uint32_t sM = __shfl_up_sync(FULL, Mv[W - 1], 1), sI = __shfl_up_sync(FULL, Iv[W - 1], 1),
             sD = __shfl_up_sync(FULL, Dv[W - 1], 1);
    if (lane == 0) sM = sI = sD = FLOOR;
    uint32_t pM = __byte_perm(sM, Mv[W - 1], 0x5432), pI = __byte_perm(sI, Iv[W - 1], 0x5432),
             pD = __byte_perm(sD, Dv[W - 1], 0x5432);
    uint32_t xe = FLOOR, dmax = FLOOR, dc = FLOOR;
#pragma unroll
    for (int q = 0; q < NV4; ++q) {
      // a zero computed from the previous group's result: this group's table
      // loads cannot be hoisted above it, so one group's 56 words are live at a time
      int zq;
      asm volatile("and.b32 %0, %1, 0;" : "=r"(zq) : "r"(dc));
      uint4 t4[14];
#pragma unroll
      for (int t = 0; t < 14; ++t) t4[t] = tr[(t * NV4 + q) * 32 + zq];
      const uint4 e4 = em[q * 32 + zq];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int w = q * 4 + e;
        if (w >= W) break;
        const uint32_t cM = Mv[w], cI = Iv[w], cD = Dv[w];
        const uint32_t c1 = v2add(v2max(xBp, u4w(t4[7], e)), u4w(t4[0], e));
        const uint32_t c2 = v2add(v2max(pM, u4w(t4[8], e)), u4w(t4[1], e));
        const uint32_t c3 = v2add(v2max(pI, u4w(t4[9], e)), u4w(t4[2], e));
        const uint32_t c4 = v2add(v2max(pD, u4w(t4[10], e)), u4w(t4[3], e));
        uint32_t sv = v2max(v2max(c1, c2), v2max(c3, c4));
        const uint32_t ev = u4w(e4, e);
        const uint32_t en = v2min(ev, 0u), ep = v2max(ev, 0u);
        sv = v2add(v2min(v2max(sv, ~v2add(en, 0x7fff7fffu)), ep ^ 0x7fff7fffu), ev);
        xe = v2max(xe, sv);
        Mv[w] = sv;
        Iv[w] = v2max(v2add(v2max(cM, u4w(t4[12], e)), u4w(t4[5], e)), v2add(v2max(cI, u4w(t4[13], e)), u4w(t4[6], e)));
        Dv[w] = dc;                                 // M->D from word w-1 (the delayed store)
        dc = v2add(v2max(sv, u4w(t4[11], e)), u4w(t4[4], e));
        dmax = v2max(dmax, dc);
        pM = cM; pI = cI; pD = cD;
      }
    }
    // word 0's M->D: the previous lane's last node (low half), this lane's word W-1 low half (high half)
    uint32_t sdc = __shfl_up_sync(FULL, dc, 1);
    if (lane == 0) sdc = FLOOR;
    Dv[0] = __byte_perm(sdc, dc, 0x5432);
    int xes = max(lo16(xe), hi16(xe)), dms = max(lo16(dmax), hi16(dmax));
    xes = __reduce_max_sync(FULL, xes);
    dms = __reduce_max_sync(FULL, dms);
    if (xes >= 32767) { xc_out = 32767; return 1; } // eslERANGE
    xN = (int16_t) (xN + V.xwN_loop);
    xC = (int16_t) max(xC + V.xwC_loop, xes + V.xwE_move);
    xJ = (int16_t) max(xJ + V.xwJ_loop, xes + V.xwE_loop);
    xB = (int16_t) max(xJ + move, xN + move);
    if (dms + V.ddbound_w > xB) {                   // D->D closure over all nodes (as vit_one), in node order:
      // the low halves of words 0 .. W-1, then the high halves; DD costs reread from L1
      int c = -2000000000, b = 0;
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < NV4; ++q) {
          int zq;                                   // loads wait for the running value (no hoisting)
          asm volatile("and.b32 %0, %1, 0;" : "=r"(zq) : "r"(c));
          const uint4 t7 = tr[(14 * NV4 + q) * 32 + zq];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int w = q * 4 + e;
            if (w >= W) break;
            const int t = h ? hi16(u4w(t7, e)) : lo16(u4w(t7, e));
            c = max(h ? hi16(Dv[w]) : lo16(Dv[w]), c + t);
            b += t;
            if (b < -2000000) b = -2000000;
          }
        }
      int sc_c = c, sc_b = b;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int oc = __shfl_up_sync(FULL, sc_c, d), ob = __shfl_up_sync(FULL, sc_b, d);
        if (lane >= d) { sc_c = max(sc_c, oc + sc_b); sc_b = max(ob + sc_b, -2000000); }
      }
      int vin = __shfl_up_sync(FULL, sc_c, 1);
      if (lane == 0) vin = -2000000000;
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < NV4; ++q) {
          int zq;
          asm volatile("and.b32 %0, %1, 0;" : "=r"(zq) : "r"(vin));
          const uint4 t7 = tr[(14 * NV4 + q) * 32 + zq];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int w = q * 4 + e;
            if (w >= W) break;
            const int t = h ? hi16(u4w(t7, e)) : lo16(u4w(t7, e));
            const int dv = max(h ? hi16(Dv[w]) : lo16(Dv[w]), vin + t);
            Dv[w] = h ? set_hi(Dv[w], dv) : set_lo(Dv[w], dv);
            vin = dv;
          }
        }
    }
  }
  xc_out = xC;
  return 0;
}

// Wide models (more than 48 nodes per lane, M > 1536, up to 256 per lane: M
// <= 8192): the same recurrence with the M, I, D row in shared memory as
// int16 (node-major, lane-minor: a warp's access to one node is 64
// contiguous bytes, conflict-free) and a runtime width; transitions int16.
// Two warps per block; 6 * 32 * CV bytes of shared memory per warp.
__device__ int vit_one_wide(const VitDev &V, const uint8_t *sq, int L, int lane, int16_t *Ms, int16_t *Is,
                            int16_t *Ds, int &xc_out) {
  const int CV = V.CV, NV = vit_nv(CV), NT = NV;    // transition vectors hold 8 nodes, like the emissions
  for (int j = 0; j < CV; ++j) Ms[j * 32 + lane] = Is[j * 32 + lane] = Ds[j * 32 + lane] = -32768;
  __syncwarp();
  const int move = V.move[L];
  int xN = V.base_w;
  int xB = (int16_t) (xN + move), xJ = -32768, xC = -32768;
  const int4 *tr = static_cast<const int4 *>(V.trans) + lane;
  for (int i = 0; i < L; ++i) {
    const int x = sq[i];
    const uint4 *em = V.emit + (size_t) x * NV * 32 + lane;
    int pM = __shfl_up_sync(FULL, (int) Ms[(CV - 1) * 32 + lane], 1);
    int pI = __shfl_up_sync(FULL, (int) Is[(CV - 1) * 32 + lane], 1);
    int pD = __shfl_up_sync(FULL, (int) Ds[(CV - 1) * 32 + lane], 1);
    if (lane == 0) pM = pI = pD = -32768;
    int xe = -32768, dmax = -32768, dc = -32768;
#pragma unroll 1
    for (int q = 0; q < NT; ++q) {
      uint4 t4[7];
#pragma unroll
      for (int t = 0; t < 7; ++t) t4[t] = *reinterpret_cast<const uint4 *>(&tr[(t * NT + q) * 32]);
      const uint4 e4 = em[q * 32];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int j = q * 8 + e;
        const int a = j * 32 + lane;
        const int cM = Ms[a], cI = Is[a], cD = Ds[a];
        int sv = max(max(xB + h16(t4[0], e), pM + h16(t4[1], e)), max(pI + h16(t4[2], e), pD + h16(t4[3], e)));
        sv = sat16(max(sv, -32768) + h16(e4, e));
        xe = max(xe, sv);
        Ms[a] = (int16_t) sv;
        Is[a] = (int16_t) max(max(cM + h16(t4[5], e), cI + h16(t4[6], e)), -32768);
        Ds[a] = (int16_t) dc;                       // M->D from node k-1 (the delayed store)
        dc = max(sv + h16(t4[4], e), -32768);
        dmax = max(dmax, dc);
        pM = cM; pI = cI; pD = cD;
      }
    }
    const int dprev = __shfl_up_sync(FULL, dc, 1);
    Ds[lane] = (int16_t) (lane == 0 ? -32768 : dprev);
    xe = __reduce_max_sync(FULL, xe);
    dmax = __reduce_max_sync(FULL, dmax);
    if (xe >= 32767) { xc_out = 32767; return 1; }  // eslERANGE
    xN = (int16_t) (xN + V.xwN_loop);
    xC = (int16_t) max(xC + V.xwC_loop, xe + V.xwE_move);
    xJ = (int16_t) max(xJ + V.xwJ_loop, xe + V.xwE_loop);
    xB = (int16_t) max(xJ + move, xN + move);
    if (dmax + V.ddbound_w > xB) {                  // D->D closure over all nodes (as vit_one)
      int c = -2000000000, b = 0;
#pragma unroll 1
      for (int q = 0; q < NT; ++q) {
        const uint4 t7 = *reinterpret_cast<const uint4 *>(&tr[(7 * NT + q) * 32]);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int t = h16(t7, e);
          c = max((int) Ds[(q * 8 + e) * 32 + lane], c + t);
          b += t;
          if (b < -2000000) b = -2000000;
        }
      }
      int sc_c = c, sc_b = b;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int oc = __shfl_up_sync(FULL, sc_c, d), ob = __shfl_up_sync(FULL, sc_b, d);
        if (lane >= d) { sc_c = max(sc_c, oc + sc_b); sc_b = max(ob + sc_b, -2000000); }
      }
      int vin = __shfl_up_sync(FULL, sc_c, 1);
      if (lane == 0) vin = -2000000000;
#pragma unroll 1
      for (int q = 0; q < NT; ++q) {
        const uint4 t7 = *reinterpret_cast<const uint4 *>(&tr[(7 * NT + q) * 32]);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const int a = (q * 8 + e) * 32 + lane;
          const int dv = max((int) Ds[a], vin + h16(t7, e));
          Ds[a] = (int16_t) dv;
          vin = dv;
        }
      }
    }
  }
  xc_out = xC;
  return 0;
}

constexpr int kVitThreads = 64;   // two warps: occupancy in steps of two warps at any register count

template <int CV>
__global__ void __launch_bounds__(kVitThreads)
vit_kernel(VitDev V, DbDev db, const int64_t *__restrict__ slots, const int64_t *__restrict__ order, int64_t nids,
           int *__restrict__ out_xc, uint8_t *__restrict__ out_st, unsigned long long *__restrict__ ticket) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1ull);
    t = __shfl_sync(FULL, t, 0);
    if (t >= (unsigned long long) nids) break;
    const int64_t j = order[t];                     // database order: the longest sequences first
    const int64_t s = slots[j];
    const int L = db.len[s];
    int xc = -32768;
    const int st = L > 0 ? vit_one<CV>(V, db.codes + db.start[s], L, lane, xc) : 0;
    if (lane == 0) { out_xc[j] = xc; out_st[j] = (uint8_t) (L > 0 ? st : 2); }
  }
}

template <int CV>
__global__ void __launch_bounds__(kVitThreads)
vitp_kernel(VitDev V, DbDev db, const int64_t *__restrict__ slots, const int64_t *__restrict__ order, int64_t nids,
            int *__restrict__ out_xc, uint8_t *__restrict__ out_st, unsigned long long *__restrict__ ticket) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1ull);
    t = __shfl_sync(FULL, t, 0);
    if (t >= (unsigned long long) nids) break;
    const int64_t j = order[t];                     // database order: the longest sequences first
    const int64_t s = slots[j];
    const int L = db.len[s];
    int xc = -32768;
    const int st = L > 0 ? vitp_one<CV>(V, db.codes + db.start[s], L, lane, xc) : 0;
    if (lane == 0) { out_xc[j] = xc; out_st[j] = (uint8_t) (L > 0 ? st : 2); }
  }
}

template <int CV>
cudaError_t launch_vitp(const VitDev &V, const DbDev &db, const int64_t *ids, const int64_t *order, int64_t n, int *xc,
                        uint8_t *st, unsigned long long *ticket, int sms, cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vitp_kernel<CV>, kVitThreads, 0);
  if (e != cudaSuccess) return e;
  constexpr int warps = kVitThreads / 32;
  long long grid = (long long) std::max(1, per_sm) * sms;
  grid = std::min<long long>(grid, (n + warps - 1) / warps);
  (void) cudaGetLastError();
  vitp_kernel<CV><<<(unsigned) std::max<long long>(1, grid), kVitThreads, 0, stream>>>(V, db, ids, order, n, xc, st,
                                                                                       ticket);
  return cudaGetLastError();
}

template <int CV>
cudaError_t launch_vit(const VitDev &V, const DbDev &db, const int64_t *ids, const int64_t *order, int64_t n, int *xc,
                       uint8_t *st, unsigned long long *ticket, int sms, cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vit_kernel<CV>, kVitThreads, 0);
  if (e != cudaSuccess) return e;
  constexpr int warps = kVitThreads / 32;
  long long grid = (long long) std::max(1, per_sm) * sms;
  grid = std::min<long long>(grid, (n + warps - 1) / warps);
  (void) cudaGetLastError();
  vit_kernel<CV><<<(unsigned) std::max<long long>(1, grid), kVitThreads, 0, stream>>>(V, db, ids, order, n, xc, st,
                                                                                      ticket);
  return cudaGetLastError();
}

// nodes per lane compiled (none spills; a model runs at the smallest width
// that holds its 8*Q8 nodes): one node per int32 register up to 32 (measured
// faster there than the packed form: 733 vs 604 GCUPS at M=200, 734 vs 652 at
// M=400), two per register (the packed form) at 40 and 48, where the int32
// form would need 16-bit transitions (851 vs 802 GCUPS at M=1500), the
// shared-memory row above 48
constexpr int kVitCV[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 20, 24, 28, 32, 40, 48};
constexpr bool vit_packed(int CV) { return CV == 40 || CV == 48; }

__global__ void __launch_bounds__(kVitThreads)
vit_wide_kernel(VitDev V, DbDev db, const int64_t *__restrict__ slots, const int64_t *__restrict__ order, int64_t nids,
                int *__restrict__ out_xc, uint8_t *__restrict__ out_st, unsigned long long *__restrict__ ticket) {
  extern __shared__ int16_t s_row[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int16_t *Ms = s_row + (size_t) w * 3 * 32 * V.CV, *Is = Ms + 32 * V.CV, *Ds = Is + 32 * V.CV;
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1ull);
    t = __shfl_sync(FULL, t, 0);
    if (t >= (unsigned long long) nids) break;
    const int64_t j = order[t];
    const int64_t s = slots[j];
    const int L = db.len[s];
    int xc = -32768;
    const int st = L > 0 ? vit_one_wide(V, db.codes + db.start[s], L, lane, Ms, Is, Ds, xc) : 0;
    if (lane == 0) { out_xc[j] = xc; out_st[j] = (uint8_t) (L > 0 ? st : 2); }
    __syncwarp();
  }
}

constexpr int kVitWideMax = 256;   // nodes per lane of the widest model (M <= 8192)

size_t vit_wide_smem(int CV) { return (size_t) (kVitThreads / 32) * 3 * 32 * CV * sizeof(int16_t); }

cudaError_t launch_vit_wide(const VitDev &V, const DbDev &db, const int64_t *ids, const int64_t *order, int64_t n,
                            int *xc, uint8_t *st, unsigned long long *ticket, int sms, cudaStream_t stream) {
  const size_t smem = vit_wide_smem(V.CV);
  cudaError_t e = cudaFuncSetAttribute(vit_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vit_wide_kernel, kVitThreads, smem);
  if (e != cudaSuccess) return e;
  constexpr int warps = kVitThreads / 32;
  long long grid = (long long) std::max(1, per_sm) * sms;
  grid = std::min<long long>(grid, (n + warps - 1) / warps);
  (void) cudaGetLastError();
  vit_wide_kernel<<<(unsigned) std::max<long long>(1, grid), kVitThreads, smem, stream>>>(V, db, ids, order, n, xc,
                                                                                          st, ticket);
  return cudaGetLastError();
}

cudaError_t dispatch_vit(int CV, const VitDev &V, const DbDev &db, const int64_t *ids, const int64_t *order, int64_t n,
                         int *xc, uint8_t *st, unsigned long long *ticket, int sms, cudaStream_t stream) {
  if (CV > 48) return launch_vit_wide(V, db, ids, order, n, xc, st, ticket, sms, stream);
  switch (CV) {
#define VCASE(c) case c: return launch_vit<c>(V, db, ids, order, n, xc, st, ticket, sms, stream);
    VCASE(1) VCASE(2) VCASE(3) VCASE(4) VCASE(5) VCASE(6) VCASE(7) VCASE(8) VCASE(9) VCASE(10) VCASE(11)
    VCASE(12) VCASE(13) VCASE(14) VCASE(15) VCASE(16) VCASE(20) VCASE(24) VCASE(28) VCASE(32)
#undef VCASE
#define PCASE(c) case c: return launch_vitp<c>(V, db, ids, order, n, xc, st, ticket, sms, stream);
    PCASE(40) PCASE(48)
#undef PCASE
  }
  return cudaErrorInvalidValue;
}

// wordify(): src/impl_sse/p7_oprofile.c:527-534
int16_t wordify(float scale_w, float sc) {
  sc = roundf(scale_w * sc);
  if (sc >= 32767.0) return 32767;
  else if (sc <= -32768.0) return -32768;
  else return (int16_t) sc;
}

}  // namespace

cudaError_t msvgb_detail::ensure_inverse(msvgb_ctx *c, const msvgb_db *db) {
  static std::mutex mu;                      // a database may be listed from several contexts at once
  std::lock_guard<std::mutex> lk(mu);
  if (db->d_inv) return cudaSuccess;
  // pool memory (freed in stream order with the database's other arrays);
  // complete before it is published, so that a search on another context's
  // stream never reads it half built
  cudaMemPool_t pool = scratch_pool(c->device);
  if (!pool) return cudaErrorMemoryAllocation;
  int64_t *inv = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync((void **) &inv, std::max<int64_t>(db->n, 1) * 8, pool, c->stream);
  if (e == cudaSuccess) e = launch_invert(db->d_orig, db->n, inv, c->num_sms, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    if (inv) { cudaFreeAsync(inv, c->stream); cudaStreamSynchronize(c->stream); }
    return e;
  }
  const_cast<msvgb_db *>(db)->d_inv = inv;   // a cache of the database's own order: logically const
  return cudaSuccess;
}

struct msvgb_vprofile {
  msvgb_ctx *ctx = nullptr;
  int device = 0;
  int M = 0, Q8 = 0, CV = 0;
  float scale_w = 0.f, nj = 0.f;
  int16_t base_w = 0, ddbound_w = 0;
  int16_t xw[4][2] = {};
  void *d_trans = nullptr;
  uint4 *d_emit = nullptr;
  int16_t *d_move = nullptr;
  int move_cap = 0;
  std::vector<int16_t> h_move;
  std::mutex move_mu;                        // the move table grows under concurrent calls
  std::vector<int16_t *> retired;            // smaller move tables other calls may still read
};

extern "C" int16_t msvgb_vit_move_cost(float scale_w, float nj, int L) {
  const float pmove = (2.0f + nj) / ((float) L + 2.0f + nj);   // p7_oprofile_ReconfigRestLength
  return wordify(scale_w, logf(pmove));
}

extern "C" float msvgb_vit_score(int xc, int status, int L, const msvgb_vom *vom) {
  if (status == 1) return INFINITY;
  if (xc <= -32768) return -INFINITY;
  float sc = (float) xc + (float) msvgb_vit_move_cost(vom->scale_w, vom->nj, L) - (float) vom->base_w;
  sc /= vom->scale_w;
  sc -= 3.0;                                                    // vitfilter.c:241-245
  return sc;
}

extern "C" int msvgb_vprofile_create(msvgb_ctx *ctx, const msvgb_vom *v, msvgb_vprofile **ret) {
  if (!ctx || !v || !ret || !v->twv || !v->rwv) return fail(MSVGB_eslEINVAL, "NULL argument");
  *ret = nullptr;
  if (v->M < 1 || v->Kp != 29) return fail(MSVGB_eslEINVAL, "ViterbiFilter profile: M >= 1 and amino (Kp = 29) only");
  const int Q8 = std::max(2, (v->M - 1) / 8 + 1), Np = 8 * Q8;
  for (int i = 0; i < 8 * Q8 * 8; ++i)
    if (v->twv[i] > 0) return fail(MSVGB_eslEINVAL, "ViterbiFilter profile: transition costs must be <= 0 (log probabilities)");
  int CV = -1;
  for (int c : kVitCV) if (32 * c >= Np) { CV = c; break; }
  if (CV < 0) CV = ((Np + 31) / 32 + 7) / 8 * 8;   // the shared-memory row, in whole transition vectors
  if (CV > kVitWideMax) return fail(MSVGB_eslEINVAL, "ViterbiFilter profile: M exceeds the supported maximum (8192 nodes)");
  // node-order tables, lane-interleaved vectors of 8 nodes; nodes past 8*Q8
  // (and padding inside it) cost -32768 as the reference's do
  const int NV = vit_nv(CV), NT = vit_nt(CV), TN = vit_tnodes(CV);
  auto node_of = [&](int lane, int j) { return lane * CV + j + 1; };
  auto striped = [&](const int16_t *base, int vec_q, int k) {   // element of node k in vector block vec_q
    const int q = (k - 1) % Q8, z = (k - 1) / Q8;
    return base[(vec_q + q) * 8 + z];
  };
  auto at_t = [&](int table, int lane, int j) { return (((size_t) table * NT + j / TN) * 32 + lane) * TN + j % TN; };
  auto at_e = [&](int x, int lane, int j) { return (((size_t) x * NV + j / 8) * 32 + lane) * 8 + j % 8; };
  std::vector<int32_t> trans((size_t) kNT * NT * 32 * TN, -32768);
  std::vector<int16_t> emit((size_t) NRES * NV * 32 * 8, -32768);
  for (int lane = 0; lane < 32; ++lane)
    for (int j = 0; j < CV; ++j) {
      const int k = node_of(lane, j);
      if (k > Np) continue;
      const int q = (k - 1) % Q8, z = (k - 1) / Q8;
      for (int t = 0; t < 7; ++t) trans[at_t(t, lane, j)] = v->twv[(q * 7 + t) * 8 + z];
      // DD into node k is node k-1's DD cost (the Q8 vectors after the 7*Q8 others)
      trans[at_t(7, lane, j)] = k > 1 ? striped(v->twv, 7 * Q8, k - 1) : (int16_t) -32768;
      for (int x = 0; x < v->Kp; ++x) emit[at_e(x, lane, j)] = v->rwv[(x * Q8 + q) * 8 + z];
    }
  std::vector<int16_t> trans16;                     // the int16 form the shared-memory kernel reads
  if (!vit_t32(CV) && !vit_packed(CV)) trans16.assign(trans.begin(), trans.end());
  const void *tsrc = vit_t32(CV) ? (const void *) trans.data() : (const void *) trans16.data();
  size_t tbytes = trans.size() * (vit_t32(CV) ? 4 : 2);
  const void *esrc = emit.data();
  size_t ebytes = emit.size() * 2;
  // the packed form (8 .. 96 nodes per lane): two nodes per word
  const bool packed = vit_packed(CV);
  std::vector<uint32_t> ptr, pem;
  if (packed) {
    const int W = CV / 2, NV4 = vitp_nv4(CV);
    auto at_p = [&](int table, int lane, int w) { return (((size_t) table * NV4 + w / 4) * 32 + lane) * 4 + w % 4; };
    auto put = [](uint32_t &word, int h, int v) {
      word = h ? (word & 0xffffu) | ((uint32_t) (uint16_t) v << 16) : (word & 0xffff0000u) | (uint16_t) v;
    };
    ptr.assign((size_t) kPT * NV4 * 32 * 4, 0);
    pem.assign((size_t) NRES * NV4 * 32 * 4, 0);
    for (int lane = 0; lane < 32; ++lane)
      for (int w = 0; w < W; ++w)
        for (int h = 0; h < 2; ++h) {
          const int k = lane * CV + h * W + w + 1;
          const bool real = k <= Np;
          const int q = (k - 1) % Q8, z = (k - 1) / Q8;
          for (int t = 0; t < 7; ++t) {
            const int c = real ? v->twv[(q * 7 + t) * 8 + z] : -32768;
            put(ptr[at_p(t, lane, w)], h, c);
            put(ptr[at_p(7 + t, lane, w)], h, -32768 - c);          // the saturating add's bound
          }
          put(ptr[at_p(14, lane, w)], h, real && k > 1 ? striped(v->twv, 7 * Q8, k - 1) : -32768);
          for (int x = 0; x < NRES; ++x)
            put(pem[at_p(x, lane, w)], h, real && x < v->Kp ? v->rwv[(x * Q8 + q) * 8 + z] : -32768);
        }
    tsrc = ptr.data(); tbytes = ptr.size() * 4;
    esrc = pem.data(); ebytes = pem.size() * 4;
  }
  msvgb_vprofile *p = new msvgb_vprofile();
  p->ctx = ctx; p->device = ctx->device; p->M = v->M; p->Q8 = Q8; p->CV = CV;
  p->scale_w = v->scale_w; p->nj = v->nj; p->base_w = v->base_w; p->ddbound_w = v->ddbound_w;
  memcpy(p->xw, v->xw, sizeof p->xw);
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_trans, tbytes);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_emit, ebytes);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_trans, tsrc, tbytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_emit, esrc, ebytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    msvgb_vprofile_destroy(p);
    return fail(MSVGB_eslESYS, std::string("vprofile upload: ") + cudaGetErrorString(e));
  }
  *ret = p;
  return MSVGB_eslOK;
}

extern "C" int msvgb_vprofile_destroy(msvgb_vprofile *p) {
  if (!p) return MSVGB_eslOK;
  cudaSetDevice(p->device);
  cudaFree(p->d_trans); cudaFree(p->d_emit); cudaFree(p->d_move);
  for (int16_t *t : p->retired) cudaFree(t);
  delete p;
  return MSVGB_eslOK;
}

// ids: original indices of the sequences to score; out_xc[j], out_status[j]
// (0 ok, 1 overflow, 2 empty) for ids[j].
extern "C" int msvgb_vitfilter(msvgb_ctx *c, msvgb_vprofile *p, const msvgb_db *db, const int64_t *ids, int64_t nids,
                               int *out_xc, uint8_t *out_status) {
  if (!c || !p || !db || nids < 0 || (nids && (!ids || !out_xc || !out_status)))
    return fail(MSVGB_eslEINVAL, "NULL argument");
  if (nids == 0) return MSVGB_eslOK;
  CUDA_TRY(cudaSetDevice(c->device));
  for (int64_t j = 0; j < nids; ++j)
    if (ids[j] < 0 || ids[j] >= db->n) return fail(MSVGB_eslEINVAL, "sequence index out of range");
  // per-length move costs up to the database's longest sequence; a smaller
  // table is retired, not freed, while the profile lives (a call on another
  // thread may have taken its pointer and not launched yet)
  const int16_t *d_move = nullptr;
  {
    std::lock_guard<std::mutex> lk(p->move_mu);
    if (p->move_cap < db->Lmax + 1) {
      const int cap = std::max(db->Lmax + 1, 2 * p->move_cap);
      for (int L = (int) p->h_move.size(); L < cap; ++L) p->h_move.push_back(msvgb_vit_move_cost(p->scale_w, p->nj, L));
      int16_t *d = nullptr;
      CUDA_TRY(cudaMalloc(&d, cap * 2));
      const cudaError_t e = cudaMemcpy(d, p->h_move.data(), cap * 2, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) { cudaFree(d); return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
      if (p->d_move) p->retired.push_back(p->d_move);
      p->d_move = d; p->move_cap = cap;
    }
    d_move = p->d_move;
  }
  CUDA_TRY(msvgb_detail::ensure_inverse(c, db));
  // one scratch block: list slots and order (int64), bucket counts, xC and statuses
  const size_t a8 = ((size_t) nids * 8 + 255) & ~(size_t) 255, a4 = ((size_t) nids * 4 + 255) & ~(size_t) 255;
  char *d_scr = nullptr;
  CUDA_TRY(cudaMallocAsync((void **) &d_scr, 2 * a8 + 4096 + a4 + (size_t) nids, c->stream));
  int64_t *d_ids = (int64_t *) d_scr, *d_order = (int64_t *) (d_scr + a8);
  int32_t *d_cnt = (int32_t *) (d_scr + 2 * a8);
  int *d_xc = (int *) (d_scr + 2 * a8 + 4096);
  uint8_t *d_st = (uint8_t *) (d_scr + 2 * a8 + 4096 + a4);
  cudaError_t e = cudaMemcpyAsync(d_ids, ids, nids * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = msvgb_detail::launch_gather_ids(d_ids, nids, db->d_inv, c->num_sms, c->stream);
  if (e == cudaSuccess)
    e = msvgb_detail::launch_order_by_length(d_ids, nids, db->d_len, db->Lmax, d_cnt, d_order, c->num_sms, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_ticket, 0, sizeof(unsigned long long), c->stream);
  VitDev V;
  V.CV = p->CV; V.base_w = p->base_w; V.ddbound_w = p->ddbound_w;
  V.xwE_move = p->xw[0][0]; V.xwE_loop = p->xw[0][1];
  V.xwN_loop = p->xw[1][1]; V.xwJ_loop = p->xw[2][1]; V.xwC_loop = p->xw[3][1];
  V.trans = p->d_trans; V.emit = p->d_emit; V.move = d_move;
  DbDev dbv{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  if (e == cudaSuccess)
    e = dispatch_vit(p->CV, V, dbv, d_ids, d_order, nids, d_xc, d_st, c->d_ticket, c->num_sms, c->stream);
  if (e == cudaSuccess) msvgb_detail::count_launch();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_xc, d_xc, nids * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_status, d_st, nids, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d_scr, c->stream);
  const cudaError_t e2 = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("vitfilter: ") + cudaGetErrorString(e));
  return MSVGB_eslOK;
}
