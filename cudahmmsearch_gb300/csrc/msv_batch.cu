// msv_batch.cu -- many profiles against one database in a single persistent
// launch, captured as a CUDA graph.
//
// The work queue holds (profile, sequence-chunk) items over the length-sorted
// database: profile-major (largest models first), and within a profile from
// the longest sequences to the shortest, so the tail of the launch is made of
// short items. Each CTA pops an item, stages that item's cost tables into
// shared memory if they are not the ones already there, and scores the chunk:
// one warp per sequence (SSV and MSV fused, as in the single-query kernel), or
// for items whose (model length, target-length bin) the lane choice puts on 16
// or 8 lanes, the lane-group SSV pass and then the full MSV on the sequences
// it left undecided. DP widths and lane counts are per-item runtime values
// dispatched to compile-time instantiations, so profiles of any length share
// one launch.
#include <algorithm>
#include <array>
#include <climits>
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
  int32_t var;                 // profile variant (tables at one lane count)
  int32_t prof;                // output block
  int64_t s_begin, s_end;      // sorted-sequence range
};

struct BatchArgs {
  const ProfDev *vars;         // [nvar]: each profile at the lane counts its items use
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
  __shared__ ChunkShared cs;
  if (threadIdx.x == 0) loaded_sh = -1;
  for (;;) {
    __syncthreads();                                   // previous item fully done
    if (threadIdx.x == 0) {
      item_sh = (long long) atomicAdd(a.ticket, 1ull);
      cs.next_seq = 0u; cs.n_und = 0u; cs.next_und = 0u;
    }
    __syncthreads();
    const long long it = item_sh;
    if (it >= a.nitems) break;
    const BatchItem item = a.items[it];
    const ProfDev &P = a.vars[item.var];
    if (loaded_sh != item.var) {                        // stage this variant's tables
      stage_tables(P, smem);
      __syncthreads();
      if (threadIdx.x == 0) loaded_sh = item.var;
    }
    uint8_t *oxj = a.out_xj + (int64_t) item.prof * a.db.n;
    uint8_t *ofl = a.out_flags + (int64_t) item.prof * a.db.n;
    run_chunk(P, smem, smem + ssv_words(P), a.db, item.s_begin, item.s_end - item.s_begin, oxj, ofl, cs);
  }
}


}  // namespace

// Graph branches the profiles' own searches rotate over: one search's tail
// and its full-MSV list run under the next ones' starts (256 profiles vs
// 1,000,000 sequences: 1.021x the back-to-back launches with 2 branches,
// 1.028x with 3, 1.029x with 4).
constexpr int kSoloBranches = 4;

struct msvgb_batch {
  msvgb_ctx *ctx = nullptr;
  int device = 0;
  int nprof = 0;
  int64_t n = 0;
  std::vector<msvgb_profile *> own;     // re-laid profiles at the batch DP widths
  std::vector<uint32_t *> gtabs;        // lane-group SSV tables
  ProfDev *d_vars = nullptr;
  BatchItem *d_items = nullptr;
  int64_t nitems = 0;
  int nvars = 0;
  unsigned long long *d_ticket = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t smem = 0;
  int threads = 256, grid = 0;
  int nsolo = 0;                        // profiles scored by their own search (single-query kernels)
  // per branch of those searches: its scratch (ticket, 3 counters, list) and capture stream
  unsigned long long *d_solo_counters[kSoloBranches] = {};
  int64_t *d_solo_list[kSoloBranches] = {};
  cudaStream_t branch[kSoloBranches] = {};
  cudaEvent_t ev[kSoloBranches + 1] = {};                // per branch: joined; last: forked
};

extern "C" int msvgb_batch_destroy(msvgb_batch *b) {
  if (!b) return MSVGB_eslOK;
  cudaSetDevice(b->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->d_vars); cudaFree(b->d_items); cudaFree(b->d_ticket);
  for (auto *t : b->gtabs) cudaFree(t);
  for (auto *p : b->own) msvgb_profile_destroy(p);
  for (int k = 0; k < kSoloBranches; ++k) {
    cudaFree(b->d_solo_counters[k]); cudaFree(b->d_solo_list[k]);
    if (b->branch[k]) cudaStreamDestroy(b->branch[k]);
  }
  for (auto ev : b->ev) if (ev) cudaEventDestroy(ev);
  delete b;
  return MSVGB_eslOK;
}

// Profiles whose search alone fills the GPU (M x residues >= 40e9 cells, the
// size at which a single query switches to lane groups) are scored by their
// own single-query searches -- lane-group pass, then the full MSV of its
// undecided sequences -- on four graph branches taken in turn, so that one
// search's tail overlaps the next one's start; so are profiles above 2047
// nodes (up to the single-query maximum). The other profiles share the
// persistent kernel, on the origin stream.
// Work items: for each profile (largest models first), for each target-length
// bin of the sorted database (longest first), chunks of about per_item
// residues -- at most kChunkMaxSeqs sequences when the bin's lane count is
// below 32 -- all scored with the variant the lane choice gives that
// (profile, bin).
int msvgb_detail::batch_create(msvgb_ctx *ctx, const msvgb_om *const *oms, int nprof, const msvgb_db *db,
                               double F1, void *d_xj, void *d_flags, int force_lanes, msvgb_batch **ret) {
  if (!ctx || !oms || nprof < 1 || !db || !ret || (db->n && (!d_xj || !d_flags)))
    return fail(MSVGB_eslEINVAL, "msvgb_batch_create: bad arguments");
  *ret = nullptr;
  msvgb_batch *b = new msvgb_batch();
  b->ctx = ctx; b->device = ctx->device; b->nprof = nprof; b->n = db->n;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) { delete b; return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
  auto bail = [&](int code, const std::string &msg) { msvgb_batch_destroy(b); return fail(code, msg); };

  // length bins of the sorted (descending) database: bin_end[k] = first sorted index of a shorter bin
  std::vector<int32_t> len(db->n);
  if (db->n) {
    e = cudaMemcpy(len.data(), db->d_len, db->n * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return bail(MSVGB_eslESYS, cudaGetErrorString(e));
  }
  struct Range { int bin; int64_t a, b; };
  std::vector<Range> ranges;                                  // longest bin first
  for (int64_t s = 0; s < db->n;) {
    const int bin = msvgb_detail::lbin_of(len[s]);
    int64_t t = s;
    while (t < db->n && msvgb_detail::lbin_of(len[t]) == bin) ++t;
    ranges.push_back(Range{bin, s, t});
    s = t;
  }

  // variants: every profile at 32 lanes (its MSV table serves all), plus the
  // lane-group tables its bins ask for
  std::vector<ProfDev> vars;
  std::vector<std::array<int, msvgb_detail::kNLBins>> var_of(nprof);
  std::vector<std::pair<int, msvgb_profile *>> large;          // own searches in the graph
  size_t smem = 0;
  for (int i = 0; i < nprof; ++i) {
    if (!oms[i]) return bail(MSVGB_eslEINVAL, "NULL profile");
    const int M = oms[i]->M;
    const int C = multi_C(M);
    const bool solo = C < 0 || (!force_lanes && (double) M * (double) db->residues >= 4e10);
    if (solo) {
      msvgb_profile *p = nullptr;
      int st = msvgb_detail::profile_build_width(ctx, oms[i], 1, 0, &p);
      const int G = st == MSVGB_eslOK ? msvgb_detail::lanes_for(ctx, M, -1, nullptr) : 32;
      if (st == MSVGB_eslOK && p->f16) st = msvgb_profile_set_lanes(p, oms[i], G);   // 32: split passes for M 1024-2047
      if (p) b->own.push_back(p);
      if (st != MSVGB_eslOK) { msvgb_batch_destroy(b); return st; }
      p->lanes_auto = true;
      large.emplace_back(i, p);
      continue;
    }
    msvgb_profile *p = nullptr;
    int st = msvgb_detail::profile_build_width(ctx, oms[i], 1, C, &p);
    if (st != MSVGB_eslOK) { msvgb_batch_destroy(b); return st; }
    b->own.push_back(p);
    LenTables *t = nullptr;
    st = msvgb_detail::ensure_tables(p, db, F1, &t);
    if (st != MSVGB_eslOK) { msvgb_batch_destroy(b); return st; }
    ProfDev P;
    P.M = p->M; P.C = p->C; P.tbm = p->tbm; P.tec = p->tec; P.base = p->base; P.bias = p->bias;
    P.stab = p->d_stab; P.mtab = p->d_mtab; P.tjb = t->d_tjb; P.xjmin = t->d_xjmin; P.ssv_f16 = 1;
    P.G = 32; P.Cg = 0;
    int vidx[3] = {-1, -1, -1};                               // 32, 16, 8 lanes
    for (int bin = 0; bin < msvgb_detail::kNLBins; ++bin) {
      int G = force_lanes ? force_lanes : msvgb_detail::lanes_for(ctx, M, bin, nullptr);
      if (G < 32 && group_C(M, G) < 0) G = 32;
      const int k = G == 32 ? 0 : G == 16 ? 1 : 2;
      if (vidx[k] < 0) {
        ProfDev V = P;
        if (G < 32) {
          V.G = G; V.Cg = group_C(M, G); V.CI = multi_hyb_words(V.Cg, G);
          const std::vector<uint32_t> gt = V.CI ? msvgb_detail::build_hyb_table(oms[i], V.Cg, G, V.CI)
                                                : msvgb_detail::build_group_table(oms[i], V.Cg, G);
          uint32_t *d = nullptr;
          e = cudaMalloc(&d, gt.size() * 4);
          if (e == cudaSuccess) b->gtabs.push_back(d);
          if (e == cudaSuccess) e = cudaMemcpy(d, gt.data(), gt.size() * 4, cudaMemcpyHostToDevice);
          if (e != cudaSuccess) return bail(MSVGB_eslEMEM, std::string("batch tables: ") + cudaGetErrorString(e));
          V.stab = d;
        }
        vidx[k] = (int) vars.size();
        vars.push_back(V);
        smem = std::max(smem, ((size_t) ssv_words(V) + (size_t) NRES * ((C + 1) / 2) * 32) * 4);
      }
      var_of[i][bin] = vidx[k];
    }
  }
  b->nvars = (int) vars.size();
  std::vector<LenTables *> large_tables;
  for (auto &lp : large) {
    LenTables *t = nullptr;
    const int st = msvgb_detail::ensure_tables(lp.second, db, F1, &t);
    if (st != MSVGB_eslOK) { msvgb_batch_destroy(b); return st; }
    large_tables.push_back(t);
  }
  std::vector<char> is_solo(nprof, 0);
  for (auto &lp : large) is_solo[lp.first] = 1;
  std::vector<int> order;
  for (int i = 0; i < nprof; ++i) if (!is_solo[i]) order.push_back(i);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return oms[x]->M > oms[y]->M; });
  std::vector<size_t> solo_order(large.size());
  for (size_t j = 0; j < large.size(); ++j) solo_order[j] = j;
  std::stable_sort(solo_order.begin(), solo_order.end(),
                   [&](size_t x, size_t y) { return large[x].second->M > large[y].second->M; });
  b->nsolo = (int) large.size();

  b->smem = smem;
  b->threads = b->smem > 100 * 1024 ? 512 : 256;
  e = cudaFuncSetAttribute(msv_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) b->smem);
  int per_sm = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msv_batch_kernel, b->threads, b->smem);
  if (e != cudaSuccess) return bail(MSVGB_eslESYS, std::string("batch kernel setup: ") + cudaGetErrorString(e));
  b->grid = std::max(1, per_sm) * ctx->num_sms;

  const double want_items = 8.0 * b->grid;
  const double per_item = std::max(4096.0, (double) db->residues * nprof / want_items);
  const int64_t min_seqs = b->threads / 32;
  std::vector<BatchItem> items;
  for (size_t oi = 0; oi < order.size(); ++oi) {
    const int pi = order[oi];
    for (const Range &r : ranges) {
      const int v = var_of[pi][r.bin];
      const int64_t max_seqs = vars[v].G < 32 ? kChunkMaxSeqs : INT64_MAX;
      for (int64_t s = r.a; s < r.b;) {
        int64_t e2 = s;
        double acc = 0;
        while (e2 < r.b && e2 - s < max_seqs && (acc < per_item || e2 - s < min_seqs)) acc += std::max(1, len[e2++]);
        items.push_back(BatchItem{v, pi, s, e2});
        s = e2;
      }
    }
  }
  b->nitems = (int64_t) items.size();
  e = cudaMalloc(&b->d_vars, sizeof(ProfDev) * std::max(1, b->nvars));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_items, sizeof(BatchItem) * std::max<int64_t>(1, b->nitems));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_ticket, sizeof(unsigned long long));
  for (int k = 0; k < kSoloBranches && e == cudaSuccess && !large.empty(); ++k) {
    e = cudaMalloc(&b->d_solo_counters[k], 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_solo_list[k], sizeof(int64_t) * std::max<int64_t>(1, db->n));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking);
  }
  for (int k = 0; k <= kSoloBranches && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&b->ev[k], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_vars, vars.data(), sizeof(ProfDev) * b->nvars, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && b->nitems)
    e = cudaMemcpy(b->d_items, items.data(), sizeof(BatchItem) * b->nitems, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bail(MSVGB_eslESYS, std::string("batch upload: ") + cudaGetErrorString(e));

  // capture: reset the ticket, run the persistent kernel
  BatchArgs a;
  a.vars = b->d_vars; a.db = DbDev{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  a.items = b->d_items; a.nitems = b->nitems;
  a.out_xj = (uint8_t *) d_xj; a.out_flags = (uint8_t *) d_flags; a.ticket = b->d_ticket;
  cudaStream_t cs = nullptr;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    // the persistent kernel on the origin stream; the profiles' own searches
    // rotate over kSoloBranches branches forked from it and joined back
    cudaError_t e1 = cudaMemsetAsync(b->d_ticket, 0, sizeof(unsigned long long), cs);
    const bool fork = !large.empty();
    if (e1 == cudaSuccess && fork) {
      e1 = cudaEventRecord(b->ev[kSoloBranches], cs);
      for (int k = 0; k < kSoloBranches && e1 == cudaSuccess; ++k) e1 = cudaStreamWaitEvent(b->branch[k], b->ev[kSoloBranches], 0);
    }
    for (size_t jj = 0; jj < solo_order.size() && e1 == cudaSuccess; ++jj) {
      const size_t j = solo_order[jj];
      const int k = (int) (jj % kSoloBranches);
      msvgb_detail::SearchScratch sc;
      sc.stream = b->branch[k]; sc.side = nullptr;
      sc.ticket = b->d_solo_counters[k]; sc.aux = b->d_solo_counters[k] + 1; sc.list = b->d_solo_list[k];
      const int st = msvgb_detail::enqueue_search(sc, large[j].second, db, large_tables[j],
                                                  (uint8_t *) d_xj + (int64_t) large[j].first * db->n,
                                                  (uint8_t *) d_flags + (int64_t) large[j].first * db->n,
                                                  ctx->num_sms);
      if (st != MSVGB_eslOK) e1 = cudaErrorInvalidValue;
    }
    if (e1 == cudaSuccess && b->nitems) {
      msv_batch_kernel<<<b->grid, b->threads, b->smem, cs>>>(a);
      e1 = cudaGetLastError();
    }
    for (int k = 0; k < kSoloBranches && e1 == cudaSuccess && fork; ++k) {
      e1 = cudaEventRecord(b->ev[k], b->branch[k]);
      if (e1 == cudaSuccess) e1 = cudaStreamWaitEvent(cs, b->ev[k], 0);
    }
    e = cudaStreamEndCapture(cs, &b->graph);
    if (e == cudaSuccess) e = e1;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) return bail(MSVGB_eslESYS, std::string("batch graph: ") + cudaGetErrorString(e));
  *ret = b;
  return MSVGB_eslOK;
}

extern "C" int msvgb_batch_create(msvgb_ctx *ctx, const msvgb_om *const *oms, int nprof, const msvgb_db *db,
                                  double F1, void *d_xj, void *d_flags, msvgb_batch **ret) {
  return msvgb_detail::batch_create(ctx, oms, nprof, db, F1, d_xj, d_flags, 0, ret);
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
