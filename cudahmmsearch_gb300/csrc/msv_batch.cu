// msv_batch.cu -- many profiles against one database in a single persistent
// launch, captured as a CUDA graph.
//
// The work queue holds (profile, sequence-chunk) items over the length-sorted
// database: profile-major (largest models first), and within a profile from
// the longest sequences to the shortest, so the tail of the launch is made of
// short items. Each CTA pops an item, stages that profile's cost tables into
// shared memory if it is not the one already there, and its warps take the
// chunk's sequences one by one (one warp per sequence, as in the single-query
// kernel). The profile's DP width C is a per-item runtime value dispatched to
// a compile-time instantiation, so profiles of any length share one launch.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"
#include "msv_multi.cuh"

using namespace msvgb;
using msvgb_detail::fail;

namespace {


struct BatchItem {
  int32_t prof;
  int32_t pad;
  int64_t s_begin, s_end;      // sorted-sequence range
};

struct BatchArgs {
  const ProfDev *profs;        // [nprof], f16 tables
  DbDev db;
  const BatchItem *items;
  int64_t nitems;
  uint8_t *out_xj;             // [nprof][n]
  uint8_t *out_flags;
  unsigned long long *ticket;
};

__global__ void __launch_bounds__(512) msv_batch_kernel(BatchArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ long long item_sh;
  __shared__ int loaded_sh;
  __shared__ unsigned long long next_seq;
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) loaded_sh = -1;
  for (;;) {
    __syncthreads();                                   // previous item fully done
    if (threadIdx.x == 0) {
      item_sh = (long long) atomicAdd(a.ticket, 1ull);
      next_seq = 0ull;
    }
    __syncthreads();
    const long long it = item_sh;
    if (it >= a.nitems) break;
    const BatchItem item = a.items[it];
    const ProfDev &P = a.profs[item.prof];
    const int C = P.C;
    uint32_t *stab = smem;
    uint32_t *mtab = smem + NRES * C * 32;
    if (loaded_sh != item.prof) {                       // stage this profile's tables
      stage_tables(P, smem);
      __syncthreads();
      if (threadIdx.x == 0) loaded_sh = item.prof;
    }
    uint8_t *oxj = a.out_xj + (int64_t) item.prof * a.db.n;
    uint8_t *ofl = a.out_flags + (int64_t) item.prof * a.db.n;
    const int64_t nseq = item.s_end - item.s_begin;
    for (;;) {
      unsigned long long k = 0;
      if (lane == 0) k = atomicAdd(&next_seq, 1ull);
      k = __shfl_sync(FULL, k, 0);
      if ((long long) k >= nseq) break;
      const int64_t s = item.s_begin + (int64_t) k;
      run_seq_any(C, P, stab, mtab, a.db, s, lane, oxj, ofl);
    }
  }
}


}  // namespace

struct msvgb_batch {
  msvgb_ctx *ctx = nullptr;
  int device = 0;
  int nprof = 0;
  int64_t n = 0;
  std::vector<msvgb_profile *> own;     // re-laid profiles at the batch DP widths
  ProfDev *d_profs = nullptr;
  BatchItem *d_items = nullptr;
  int64_t nitems = 0;
  unsigned long long *d_ticket = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t smem = 0;
  int threads = 256, grid = 0;
};

extern "C" int msvgb_batch_destroy(msvgb_batch *b) {
  if (!b) return MSVGB_eslOK;
  cudaSetDevice(b->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->d_profs); cudaFree(b->d_items); cudaFree(b->d_ticket);
  for (auto *p : b->own) msvgb_profile_destroy(p);
  delete b;
  return MSVGB_eslOK;
}

extern "C" int msvgb_batch_create(msvgb_ctx *ctx, const msvgb_om *const *oms, int nprof, const msvgb_db *db,
                                  double F1, void *d_xj, void *d_flags, msvgb_batch **ret) {
  if (!ctx || !oms || nprof < 1 || !db || !ret || (db->n && (!d_xj || !d_flags)))
    return fail(MSVGB_eslEINVAL, "msvgb_batch_create: bad arguments");
  *ret = nullptr;
  msvgb_batch *b = new msvgb_batch();
  b->ctx = ctx; b->device = ctx->device; b->nprof = nprof; b->n = db->n;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) { delete b; return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
  // profiles re-laid at the batch DP widths (f16 SSV tables) with their length tables
  std::vector<ProfDev> hp(nprof);
  std::vector<int> order(nprof);
  int cmax = 1;
  for (int i = 0; i < nprof; ++i) {
    if (!oms[i]) { msvgb_batch_destroy(b); return fail(MSVGB_eslEINVAL, "NULL profile"); }
    const int C = multi_C(oms[i]->M);
    if (C < 0) { msvgb_batch_destroy(b); return fail(MSVGB_eslEINVAL, "batched profiles are limited to M <= 2047"); }
    msvgb_profile *p = nullptr;
    int st = msvgb_detail::profile_build_width(ctx, oms[i], 1, C, &p);
    if (st != MSVGB_eslOK) { msvgb_batch_destroy(b); return st; }
    b->own.push_back(p);
    LenTables *t = nullptr;
    st = msvgb_detail::ensure_tables(p, db, F1, &t);
    if (st != MSVGB_eslOK) { msvgb_batch_destroy(b); return st; }
    ProfDev &P = hp[i];
    P.M = p->M; P.C = p->C; P.tbm = p->tbm; P.tec = p->tec; P.base = p->base; P.bias = p->bias;
    P.stab = p->d_stab; P.mtab = p->d_mtab; P.tjb = t->d_tjb; P.xjmin = t->d_xjmin; P.ssv_f16 = 1;
    cmax = std::max(cmax, C);
    order[i] = i;
  }
  // work items: profile-major, largest models first; chunks of the sorted
  // database sized so there are several items per CTA
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return oms[x]->M > oms[y]->M; });
  b->smem = multi_smem_bytes(cmax);
  b->threads = b->smem > 100 * 1024 ? 512 : 256;
  e = cudaFuncSetAttribute(msv_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) b->smem);
  int per_sm = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msv_batch_kernel, b->threads, b->smem);
  if (e != cudaSuccess) { msvgb_batch_destroy(b); return fail(MSVGB_eslESYS, std::string("batch kernel setup: ") + cudaGetErrorString(e)); }
  b->grid = std::max(1, per_sm) * ctx->num_sms;
  std::vector<int32_t> len(db->n);
  if (db->n) {
    e = cudaMemcpy(len.data(), db->d_len, db->n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { msvgb_batch_destroy(b); return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
  }
  const double want_items = 8.0 * b->grid;
  const double per_item = std::max(4096.0, (double) db->residues * nprof / want_items);
  std::vector<BatchItem> items;
  for (int oi = 0; oi < nprof; ++oi) {
    const int pi = order[oi];
    int64_t s = 0;
    while (s < db->n) {
      int64_t e2 = s;
      double acc = 0;
      const int64_t min_seqs = b->threads / 32;
      while (e2 < db->n && (acc < per_item || e2 - s < min_seqs)) acc += std::max(1, len[e2++]);
      items.push_back(BatchItem{pi, 0, s, e2});
      s = e2;
    }
  }
  b->nitems = (int64_t) items.size();
  e = cudaMalloc(&b->d_profs, sizeof(ProfDev) * nprof);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_items, sizeof(BatchItem) * std::max<int64_t>(1, b->nitems));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ticket, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemcpy(b->d_profs, hp.data(), sizeof(ProfDev) * nprof, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && b->nitems)
    e = cudaMemcpy(b->d_items, items.data(), sizeof(BatchItem) * b->nitems, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { msvgb_batch_destroy(b); return fail(MSVGB_eslESYS, std::string("batch upload: ") + cudaGetErrorString(e)); }

  // capture: reset the ticket, run the persistent kernel
  BatchArgs a;
  a.profs = b->d_profs; a.db = DbDev{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  a.items = b->d_items; a.nitems = b->nitems;
  a.out_xj = (uint8_t *) d_xj; a.out_flags = (uint8_t *) d_flags; a.ticket = b->d_ticket;
  cudaStream_t cs = nullptr;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaMemsetAsync(b->d_ticket, 0, sizeof(unsigned long long), cs);
    msv_batch_kernel<<<b->grid, b->threads, b->smem, cs>>>(a);
    cudaError_t e1 = cudaGetLastError();
    e = cudaStreamEndCapture(cs, &b->graph);
    if (e == cudaSuccess) e = e1;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) { msvgb_batch_destroy(b); return fail(MSVGB_eslESYS, std::string("batch graph: ") + cudaGetErrorString(e)); }
  *ret = b;
  return MSVGB_eslOK;
}

extern "C" int msvgb_batch_run(msvgb_batch *b) {
  if (!b) return fail(MSVGB_eslEINVAL, "NULL batch");
  cudaError_t e = cudaSetDevice(b->device);
  if (e == cudaSuccess) e = cudaGraphLaunch(b->exec, b->ctx->stream);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("batch launch: ") + cudaGetErrorString(e));
  msvgb_detail::count_launch();
  return MSVGB_eslOK;
}

extern "C" int64_t msvgb_batch_items(const msvgb_batch *b) { return b ? b->nitems : -1; }

extern "C" int msvgb_search_batch(msvgb_ctx *ctx, const msvgb_om *const *oms, int nprof, const msvgb_db *db,
                                  double F1, uint8_t *out_xj, uint8_t *out_flags) {
  if (!ctx || !db || nprof < 1 || (db->n && (!out_xj || !out_flags)))
    return fail(MSVGB_eslEINVAL, "msvgb_search_batch: bad arguments");
  if (db->n == 0) return MSVGB_eslOK;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, cudaGetErrorString(e));
  const size_t bytes = (size_t) nprof * db->n;
  uint8_t *d = nullptr;
  e = cudaMalloc(&d, 2 * bytes);
  if (e != cudaSuccess) return fail(MSVGB_eslEMEM, std::string("batch outputs: ") + cudaGetErrorString(e));
  msvgb_batch *b = nullptr;
  int st = msvgb_batch_create(ctx, oms, nprof, db, F1, d, d + bytes, &b);
  if (st == MSVGB_eslOK) st = msvgb_batch_run(b);
  if (st == MSVGB_eslOK) {
    e = cudaMemcpyAsync(out_xj, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_flags, d + bytes, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) st = fail(MSVGB_eslESYS, std::string("batch copy: ") + cudaGetErrorString(e));
  }
  msvgb_batch_destroy(b);
  cudaFree(d);
  return st;
}
