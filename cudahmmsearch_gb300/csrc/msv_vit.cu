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

struct VitDev {
  int CV;                  // nodes per lane
  int16_t base_w, ddbound_w;
  int16_t xwE_move, xwE_loop, xwN_loop, xwJ_loop, xwC_loop;
  const int16_t *trans;    // [kNT][32][CV]
  const int16_t *emit;     // [NRES][32][CV]
  const int16_t *move;     // [Lmax+1]: N/J/C move cost at target length L
};

__device__ __forceinline__ int sat16(int v) { return min(32767, max(-32768, v)); }

template <int CV>
__device__ int vit_one(const VitDev &V, const uint8_t *sq, int L, int lane, int &xc_out) {
  const int stride_t = 32 * CV;
  int Mv[CV], Iv[CV], Dv[CV];
#pragma unroll
  for (int j = 0; j < CV; ++j) Mv[j] = Iv[j] = Dv[j] = -32768;
  const int move = V.move[L];
  int xN = V.base_w;
  int xB = (int16_t) (xN + move), xJ = -32768, xC = -32768;
  for (int i = 0; i < L; ++i) {
    const int x = sq[i];
    const int16_t *em = V.emit + (x * 32 + lane) * CV;
    // the transition costs are read anew each row (from L1): kept in
    // registers across rows they would crowd out the DP state
    int opaque;
    asm volatile("mov.u32 %0, 0;" : "=r"(opaque));
    const int16_t *tr = V.trans + lane * CV + opaque;
    // predecessors of this lane's first node: the previous lane's last node (old row)
    int pM = __shfl_up_sync(FULL, Mv[CV - 1], 1), pI = __shfl_up_sync(FULL, Iv[CV - 1], 1),
        pD = __shfl_up_sync(FULL, Dv[CV - 1], 1);
    if (lane == 0) pM = pI = pD = -32768;
    int xe = -32768, dmax = -32768, dc = -32768;
#pragma unroll
    for (int j = 0; j < CV; ++j) {
      const int cM = Mv[j], cI = Iv[j], cD = Dv[j];
      int sv = sat16(xB + tr[0 * stride_t + j]);
      sv = max(sv, sat16(pM + tr[1 * stride_t + j]));
      sv = max(sv, sat16(pI + tr[2 * stride_t + j]));
      sv = max(sv, sat16(pD + tr[3 * stride_t + j]));
      sv = sat16(sv + em[j]);
      xe = max(xe, sv);
      Mv[j] = sv;
      Iv[j] = max(sat16(cM + tr[5 * stride_t + j]), sat16(cI + tr[6 * stride_t + j]));
      Dv[j] = dc;                                   // M->D from node k-1 (the delayed store)
      dc = sat16(sv + tr[4 * stride_t + j]);
      dmax = max(dmax, dc);
      pM = cM; pI = cI; pD = cD;
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
      int c = -2000000000, b = 0;
#pragma unroll
      for (int j = 0; j < CV; ++j) {
        const int t = tr[7 * stride_t + j];         // D(k-1) -> D(k)
        c = max(Dv[j], c + t);
        b += t;
        if (b < -2000000) b = -2000000;             // far below any value: keeps the sums in range
      }
      // exclusive warp scan of the blocks: (c1,b1) then (c2,b2) = (max(c2, c1+b2), b1+b2)
      int sc_c = c, sc_b = b;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int oc = __shfl_up_sync(FULL, sc_c, d), ob = __shfl_up_sync(FULL, sc_b, d);
        if (lane >= d) { sc_c = max(sc_c, oc + sc_b); sc_b = max(ob + sc_b, -2000000); }
      }
      int v = __shfl_up_sync(FULL, sc_c, 1);
      if (lane == 0) v = -2000000000;
#pragma unroll
      for (int j = 0; j < CV; ++j) {
        Dv[j] = max(Dv[j], v + tr[7 * stride_t + j]);
        v = Dv[j];
      }
    }
  }
  xc_out = xC;
  return 0;
}

template <int CV>
__global__ void __launch_bounds__(256)
vit_kernel(VitDev V, DbDev db, const int64_t *__restrict__ sorted_ids, int64_t nids, int *__restrict__ out_xc,
           uint8_t *__restrict__ out_st, unsigned long long *__restrict__ ticket) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1ull);
    t = __shfl_sync(FULL, t, 0);
    if (t >= (unsigned long long) nids) break;
    const int64_t s = sorted_ids[t];
    const int L = db.len[s];
    int xc = -32768;
    const int st = L > 0 ? vit_one<CV>(V, db.codes + db.start[s], L, lane, xc) : 0;
    if (lane == 0) { out_xc[t] = xc; out_st[t] = (uint8_t) (L > 0 ? st : 2); }
  }
}

template <int CV>
cudaError_t launch_vit(const VitDev &V, const DbDev &db, const int64_t *ids, int64_t n, int *xc, uint8_t *st,
                       unsigned long long *ticket, int sms, cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vit_kernel<CV>, 256, 0);
  if (e != cudaSuccess) return e;
  long long grid = (long long) std::max(1, per_sm) * sms;
  grid = std::min<long long>(grid, (n + 7) / 8);
  (void) cudaGetLastError();
  vit_kernel<CV><<<(unsigned) std::max<long long>(1, grid), 256, 0, stream>>>(V, db, ids, n, xc, st, ticket);
  return cudaGetLastError();
}

// nodes per lane compiled (the widths between spill registers: the next
// larger one runs instead)
constexpr int kVitCV[] = {1, 2, 3, 4, 6, 8, 12, 32, 48};

cudaError_t dispatch_vit(int CV, const VitDev &V, const DbDev &db, const int64_t *ids, int64_t n, int *xc,
                         uint8_t *st, unsigned long long *ticket, int sms, cudaStream_t stream) {
  switch (CV) {
#define VCASE(c) case c: return launch_vit<c>(V, db, ids, n, xc, st, ticket, sms, stream);
    VCASE(1) VCASE(2) VCASE(3) VCASE(4) VCASE(6) VCASE(8) VCASE(12) VCASE(32) VCASE(48)
#undef VCASE
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

struct msvgb_vprofile {
  msvgb_ctx *ctx = nullptr;
  int device = 0;
  int M = 0, Q8 = 0, CV = 0;
  float scale_w = 0.f, nj = 0.f;
  int16_t base_w = 0, ddbound_w = 0;
  int16_t xw[4][2] = {};
  int16_t *d_trans = nullptr, *d_emit = nullptr, *d_move = nullptr;
  int move_cap = 0;
  std::vector<int16_t> h_move;
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
  int CV = -1;
  for (int c : kVitCV) if (32 * c >= Np) { CV = c; break; }
  if (CV < 0) return fail(MSVGB_eslEINVAL, "ViterbiFilter profile: M exceeds the supported maximum (1536 nodes)");
  // node-order, lane-major tables; nodes past 8*Q8 (and padding inside it) cost -32768 as the reference's do
  const int N = 32 * CV;
  auto node_of = [&](int lane, int j) { return lane * CV + j + 1; };
  auto striped = [&](const int16_t *base, int vec_q, int k) {   // element of node k in vector block vec_q
    const int q = (k - 1) % Q8, z = (k - 1) / Q8;
    return base[(vec_q + q) * 8 + z];
  };
  std::vector<int16_t> trans((size_t) kNT * N, -32768), emit((size_t) NRES * N, -32768);
  for (int lane = 0; lane < 32; ++lane)
    for (int j = 0; j < CV; ++j) {
      const int k = node_of(lane, j);
      if (k > Np) continue;
      const int q = (k - 1) % Q8, z = (k - 1) / Q8;
      for (int t = 0; t < 7; ++t) trans[((size_t) t * 32 + lane) * CV + j] = v->twv[(q * 7 + t) * 8 + z];
      // DD into node k is node k-1's DD cost (the Q8 vectors after the 7*Q8 others)
      trans[((size_t) 7 * 32 + lane) * CV + j] = k > 1 ? striped(v->twv, 7 * Q8, k - 1) : (int16_t) -32768;
      for (int x = 0; x < v->Kp; ++x) emit[((size_t) x * 32 + lane) * CV + j] = v->rwv[(x * Q8 + q) * 8 + z];
    }
  msvgb_vprofile *p = new msvgb_vprofile();
  p->ctx = ctx; p->device = ctx->device; p->M = v->M; p->Q8 = Q8; p->CV = CV;
  p->scale_w = v->scale_w; p->nj = v->nj; p->base_w = v->base_w; p->ddbound_w = v->ddbound_w;
  memcpy(p->xw, v->xw, sizeof p->xw);
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_trans, trans.size() * 2);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_emit, emit.size() * 2);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_trans, trans.data(), trans.size() * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_emit, emit.data(), emit.size() * 2, cudaMemcpyHostToDevice);
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
  // per-length move costs up to the database's longest sequence
  if (p->move_cap < db->Lmax + 1) {
    const int cap = std::max(db->Lmax + 1, 2 * p->move_cap);
    for (int L = (int) p->h_move.size(); L < cap; ++L) p->h_move.push_back(msvgb_vit_move_cost(p->scale_w, p->nj, L));
    int16_t *d = nullptr;
    CUDA_TRY(cudaMalloc(&d, cap * 2));
    const cudaError_t e = cudaMemcpy(d, p->h_move.data(), cap * 2, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(d); return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
    CUDA_TRY(cudaStreamSynchronize(c->stream));                // an older table may still be read
    cudaFree(p->d_move);
    p->d_move = d; p->move_cap = cap;
  }
  // original -> sorted indices of the database
  if (!db->d_inv) {
    msvgb_db *mdb = const_cast<msvgb_db *>(db);
    CUDA_TRY(cudaMalloc(&mdb->d_inv, std::max<int64_t>(db->n, 1) * 8));
    CUDA_TRY(msvgb_detail::launch_invert(db->d_orig, db->n, mdb->d_inv, c->num_sms, c->stream));
  }
  int64_t *d_ids = nullptr;
  int *d_xc = nullptr;
  uint8_t *d_st = nullptr;
  CUDA_TRY(cudaMallocAsync((void **) &d_ids, nids * 8, c->stream));
  CUDA_TRY(cudaMallocAsync((void **) &d_xc, nids * 4, c->stream));
  CUDA_TRY(cudaMallocAsync((void **) &d_st, nids, c->stream));
  cudaError_t e = cudaMemcpyAsync(d_ids, ids, nids * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = msvgb_detail::launch_gather_ids(d_ids, nids, db->d_inv, c->num_sms, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_ticket, 0, sizeof(unsigned long long), c->stream);
  VitDev V;
  V.CV = p->CV; V.base_w = p->base_w; V.ddbound_w = p->ddbound_w;
  V.xwE_move = p->xw[0][0]; V.xwE_loop = p->xw[0][1];
  V.xwN_loop = p->xw[1][1]; V.xwJ_loop = p->xw[2][1]; V.xwC_loop = p->xw[3][1];
  V.trans = p->d_trans; V.emit = p->d_emit; V.move = p->d_move;
  DbDev dbv{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  if (e == cudaSuccess) e = dispatch_vit(p->CV, V, dbv, d_ids, nids, d_xc, d_st, c->d_ticket, c->num_sms, c->stream);
  if (e == cudaSuccess) msvgb_detail::count_launch();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_xc, d_xc, nids * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_status, d_st, nids, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d_ids, c->stream); cudaFreeAsync(d_xc, c->stream); cudaFreeAsync(d_st, c->stream);
  const cudaError_t e2 = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("vitfilter: ") + cudaGetErrorString(e));
  return MSVGB_eslOK;
}
