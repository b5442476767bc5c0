// msv_serve.cu -- serving loop: continuous batching of query profiles
// against a database resident in HBM.
//
// A persistent kernel consumes (request slot, sequence chunk) work items from
// a ring in host-mapped memory that the host keeps appending to while the
// kernel runs. A request is admitted when a device-memory slot is free (its
// cost tables, per-length tables and result buffers live in the slot), its
// items are published by advancing the ring's tail, and CTAs already running
// pick them up between items: requests that arrive while others are on the
// GPU overlap with them on the device. Each finished item bumps the slot's
// completion counter (host-mapped, system-scope atomics), which the host polls.
//
// Every device-side wait is bounded: a CTA that finds no work for about half a
// second leaves (re-checking the ring once more after leaving, so a request
// published at that moment is not lost); the host relaunches the kernel when
// it publishes work and no CTA is alive.
//
// A request whose search fills the GPU alone (M x residues >= 40e9 cells, as
// in the batched path) does not go through the ring: it runs as its own
// single-query search -- the tables and lane choice msvgb_profile_create
// would make, the lane-group pass and its full-MSV list -- on one of two
// streams taken in turn, so one search's tail overlaps the next one's start.
// While such searches are queued the ring kernel's CTAs leave as soon as the
// ring is empty instead of waiting, so that they hold no SM the searches need.
//
// The reference's counterpart is the per-block host loop of the fork's
// pipeline_thread (code/src/cudaHmmsearch.cu:725-810) and, conceptually, the
// hmmpgmd daemon's resident sequence cache (src/hmmdwrkr.c:600-646).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"
#include "msv_multi.cuh"

using namespace msvgb;
using msvgb_detail::fail;

namespace {

constexpr int kMaxSlots = 256;
constexpr unsigned long long kIdleNs = 500000000ull;   // a CTA leaves after 0.5 s without work
constexpr int kIdleIters = 2000000;         // and after this many polls (each sleeps >= 1 us) in any case
constexpr double kSoloCells = 4e10;         // M x residues from which a request runs as its own search

struct ServeCtl {                            // host-mapped
  unsigned long long tail;                   // items published (host writes)
  int stop;                                  // host: bit 0 leave; bit 1 leave when idle (searches
                                             // of their own are queued)
  int live;                                  // CTAs currently running
  unsigned long long done[kMaxSlots];        // finished items per slot (device increments)
};

struct ServeItem {
  int32_t slot, gen;
  int64_t s_begin, s_end;
};

struct SlotOut { uint8_t *xj, *flags; };

struct ServeArgs {
  ServeCtl *ctl;
  unsigned long long *head;                  // device memory: items claimed
  const ServeItem *ring;                     // host-mapped
  long long cap;
  const ProfDev *slots;                      // device memory, one per slot
  const SlotOut *outs;
  DbDev db;
};

__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_volatile_i32(const int *p) { return *(const volatile int *) p; }
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__global__ void __launch_bounds__(512) msv_serve_kernel(ServeArgs a) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ long long item_sh;
  __shared__ ServeItem it_sh;
  __shared__ int loaded_slot, loaded_gen;
  __shared__ ChunkShared cs;
  if (threadIdx.x == 0) { loaded_slot = -1; loaded_gen = -1; atomicAdd_system(&a.ctl->live, 1); }
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) {
      long long got = -1;
      const unsigned long long t_idle = globaltimer_ns();
      for (int iter = 0; iter < kIdleIters && globaltimer_ns() - t_idle < kIdleNs; ++iter) {
        const unsigned long long t = ld_acquire_sys(&a.ctl->tail);
        const unsigned long long h = *(volatile unsigned long long *) a.head;
        if (h < t) {
          if (atomicCAS(a.head, h, h + 1) == h) { got = (long long) h; break; }
          continue;
        }
        if (ld_volatile_i32(&a.ctl->stop)) break;
        __nanosleep(1000);
      }
      if (got < 0) {
        // leave, then look once more: a request published while we were
        // deciding to leave is picked up here or by the host's relaunch
        atomicSub_system(&a.ctl->live, 1);
        __threadfence_system();
        const unsigned long long t = ld_acquire_sys(&a.ctl->tail);
        const unsigned long long h = *(volatile unsigned long long *) a.head;
        if (h < t && !(ld_volatile_i32(&a.ctl->stop) & 1)) { atomicAdd_system(&a.ctl->live, 1); got = -2; }
      }
      if (got >= 0) {
        const volatile ServeItem *src = a.ring + (got & (a.cap - 1));   // cap is a power of two
        it_sh.slot = src->slot; it_sh.gen = src->gen; it_sh.s_begin = src->s_begin; it_sh.s_end = src->s_end;
      }
      item_sh = got;
      cs.next_seq = 0u; cs.n_und = 0u; cs.next_und = 0u;
    }
    __syncthreads();
    const long long got = item_sh;
    if (got == -2) continue;
    if (got < 0) break;
    const ServeItem item = it_sh;
    const ProfDev &P = a.slots[item.slot];
    if (loaded_slot != item.slot || loaded_gen != item.gen) {
      stage_tables(P, smem);
      __syncthreads();
      if (threadIdx.x == 0) { loaded_slot = item.slot; loaded_gen = item.gen; }
    }
    const SlotOut o = a.outs[item.slot];
    run_chunk(P, smem, smem + ssv_words(P), a.db, item.s_begin, item.s_end - item.s_begin, o.xj, o.flags, cs);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence_system();                           // results visible before the count
      atomicAdd_system(&a.ctl->done[item.slot], 1ull);
    }
  }
}

}  // namespace

struct msvgb_server {
  msvgb_ctx *ctx = nullptr;
  const msvgb_db *db = nullptr;
  int device = 0;
  double F1 = 0.02;
  int nslots = 0;
  size_t smem = 0;
  int threads = 512, grid = 0;
  int64_t items_per_req = 0;
  std::vector<int64_t> chunk_begin;          // item boundaries over the sorted database
  // device
  uint8_t *d_slot_mem = nullptr;
  size_t slot_bytes = 0, tab_off_m = 0, tab_off_tjb = 0, tab_off_xjm = 0, off_xj = 0, off_fl = 0;
  ProfDev *d_slots = nullptr;
  SlotOut *d_outs = nullptr;
  unsigned long long *d_head = nullptr;
  // host-mapped
  ServeCtl *h_ctl = nullptr, *d_ctl = nullptr;
  ServeItem *h_ring = nullptr, *d_ring = nullptr;
  long long cap = 0;
  // host state
  std::mutex mu;
  std::condition_variable slot_freed;
  std::vector<int> free_slots;
  std::vector<int> gen;
  std::vector<uint64_t> ticket_of;
  uint64_t next_ticket = 1;
  unsigned long long tail = 0;
  cudaStream_t upload = nullptr;
  std::vector<cudaStream_t> kstreams;
  size_t next_kstream = 0;
  std::vector<uint8_t> tjb;                  // shared per-length tjb_b table (scale of the first profile)
  float tjb_scale = -1.f;
  uint64_t launches = 0;
  cudaEvent_t last_done = nullptr;           // completes when the latest launch has fully exited
  bool launched = false;
  // requests scored by their own single-query searches
  std::vector<char> solo;                    // per slot: its request runs as its own search
  std::vector<cudaEvent_t> solo_done;        // per slot: completes when that search has finished
  cudaStream_t solo_stream[2] = {nullptr, nullptr};
  unsigned long long *d_solo_counters[2] = {nullptr, nullptr};   // per stream: ticket + 3 counters
  int64_t *d_solo_list[2] = {nullptr, nullptr};                  // per stream: undecided list
  int next_solo = 0;
  int solo_pending = 0;                      // submitted, not yet collected by msvgb_server_wait
  uint64_t solo_searches = 0;
};

// True while the most recent launch has CTAs running or still to start.
static bool kernel_running(msvgb_server *s) {
  return s->launched && cudaEventQuery(s->last_done) == cudaErrorNotReady;
}

static int launch_serve(msvgb_server *s) {
  ServeArgs a;
  a.ctl = s->d_ctl; a.head = s->d_head; a.ring = s->d_ring; a.cap = s->cap;
  a.slots = s->d_slots; a.outs = s->d_outs;
  a.db = DbDev{s->db->d_codes, s->db->d_start, s->db->d_len, s->db->d_orig, s->db->n};
  cudaStream_t st = s->kstreams[s->next_kstream++ % s->kstreams.size()];
  (void) cudaGetLastError();
  msv_serve_kernel<<<s->grid, s->threads, s->smem, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(s->last_done, st);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("serve launch: ") + cudaGetErrorString(e));
  s->launched = true;
  s->launches++;
  msvgb_detail::count_launch();
  return MSVGB_eslOK;
}

extern "C" int msvgb_server_destroy(msvgb_server *s) {
  if (!s) return MSVGB_eslOK;
  cudaSetDevice(s->device);
  if (s->h_ctl) {
    __atomic_fetch_or(&s->h_ctl->stop, 1, __ATOMIC_SEQ_CST);
    for (auto st : s->kstreams) cudaStreamSynchronize(st);
  }
  for (auto st : s->kstreams) cudaStreamDestroy(st);
  if (s->last_done) cudaEventDestroy(s->last_done);
  for (int k = 0; k < 2; ++k) {
    if (s->solo_stream[k]) { cudaStreamSynchronize(s->solo_stream[k]); cudaStreamDestroy(s->solo_stream[k]); }
    cudaFree(s->d_solo_counters[k]);
    cudaFree(s->d_solo_list[k]);
  }
  for (auto ev : s->solo_done) if (ev) cudaEventDestroy(ev);
  if (s->upload) { cudaStreamSynchronize(s->upload); cudaStreamDestroy(s->upload); }
  cudaFree(s->d_slot_mem); cudaFree(s->d_slots); cudaFree(s->d_outs); cudaFree(s->d_head);
  if (s->h_ctl) cudaFreeHost(s->h_ctl);
  if (s->h_ring) cudaFreeHost(s->h_ring);
  delete s;
  return MSVGB_eslOK;
}

extern "C" int msvgb_server_create(msvgb_ctx *ctx, const msvgb_db *db, double F1, int max_slots,
                                   size_t mem_budget, msvgb_server **ret) {
  if (!ctx || !db || !ret || max_slots < 1) return fail(MSVGB_eslEINVAL, "msvgb_server_create: bad arguments");
  *ret = nullptr;
  msvgb_server *s = new msvgb_server();
  s->ctx = ctx; s->db = db; s->device = ctx->device; s->F1 = F1;
  cudaError_t e = cudaSetDevice(ctx->device);
  // slot layout: f16 SSV table and MSV table at the widest batched width, per-length tables, results
  const size_t tab = multi_smem_bytes(kMultiMaxC);
  auto align = [](size_t x) { return (x + 255) / 256 * 256; };
  s->tab_off_m = (size_t) NRES * kMultiMaxC * 32 * 4;
  s->tab_off_tjb = align(tab);
  s->tab_off_xjm = s->tab_off_tjb + align((size_t) db->Lmax + 1);
  s->off_xj = s->tab_off_xjm + align((size_t) db->Lmax + 1);
  s->off_fl = s->off_xj + align((size_t) db->n);
  s->slot_bytes = s->off_fl + align((size_t) db->n);
  // admission bound: as many slots as the budget holds (at least one)
  s->nslots = std::max(1, std::min({max_slots, kMaxSlots, (int) std::max<size_t>(1, mem_budget / s->slot_bytes)}));
  s->smem = tab;
  e = cudaFuncSetAttribute(msv_serve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) s->smem);
  int per_sm = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, msv_serve_kernel, s->threads, s->smem);
  s->grid = std::max(1, per_sm) * ctx->num_sms;
  // items per request: several per CTA, by residue count
  std::vector<int32_t> len(db->n);
  if (e == cudaSuccess && db->n) e = cudaMemcpy(len.data(), db->d_len, db->n * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { msvgb_server_destroy(s); return fail(MSVGB_eslESYS, std::string("server setup: ") + cudaGetErrorString(e)); }
  const double per_item = std::max(4096.0, (double) db->residues / (2.0 * s->grid));
  for (int64_t i = 0; i < db->n;) {
    s->chunk_begin.push_back(i);
    double acc = 0;
    const int64_t i0 = i;
    while (i < db->n && i - i0 < kChunkMaxSeqs && (acc < per_item || i - i0 < s->threads / 32))
      acc += std::max(1, len[i++]);
  }
  s->chunk_begin.push_back(db->n);
  s->items_per_req = (int64_t) s->chunk_begin.size() - 1;
  s->cap = 1;                                           // a power of two: the kernel masks, no 64-bit modulo
  while (s->cap < (long long) s->nslots * std::max<int64_t>(1, s->items_per_req) + 1) s->cap <<= 1;
  if (e == cudaSuccess) e = cudaMalloc(&s->d_slot_mem, s->slot_bytes * s->nslots);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_slots, sizeof(ProfDev) * s->nslots);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_outs, sizeof(SlotOut) * s->nslots);
  if (e == cudaSuccess) e = cudaMalloc(&s->d_head, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(s->d_head, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaHostAlloc(&s->h_ctl, sizeof(ServeCtl), cudaHostAllocMapped);
  if (e == cudaSuccess) e = cudaHostAlloc(&s->h_ring, sizeof(ServeItem) * s->cap, cudaHostAllocMapped);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **) &s->d_ctl, s->h_ctl, 0);
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **) &s->d_ring, s->h_ring, 0);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->upload, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->last_done, cudaEventDisableTiming);
  for (int i = 0; e == cudaSuccess && i < 4; ++i) {
    cudaStream_t st;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) s->kstreams.push_back(st);
  }
  // searches of their own: only where some profile's search can fill the GPU
  // (M <= 2047 are served)
  if (e == cudaSuccess && 2047.0 * (double) db->residues >= kSoloCells)
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      e = cudaStreamCreateWithFlags(&s->solo_stream[k], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaMalloc(&s->d_solo_counters[k], 4 * sizeof(unsigned long long));
      if (e == cudaSuccess) e = cudaMalloc(&s->d_solo_list[k], sizeof(int64_t) * std::max<int64_t>(1, db->n));
    }
  s->solo.assign(s->nslots, 0);
  s->solo_done.assign(s->nslots, nullptr);
  for (int i = 0; e == cudaSuccess && i < s->nslots && s->solo_stream[0]; ++i)
    e = cudaEventCreateWithFlags(&s->solo_done[i], cudaEventDisableTiming);
  if (e != cudaSuccess) { msvgb_server_destroy(s); return fail(MSVGB_eslEMEM, std::string("server memory: ") + cudaGetErrorString(e)); }
  memset(s->h_ctl, 0, sizeof(ServeCtl));
  std::vector<SlotOut> outs(s->nslots);
  for (int i = 0; i < s->nslots; ++i) {
    uint8_t *base = s->d_slot_mem + s->slot_bytes * i;
    outs[i] = SlotOut{base + s->off_xj, base + s->off_fl};
    s->free_slots.push_back(s->nslots - 1 - i);
  }
  s->gen.assign(s->nslots, 0);
  s->ticket_of.assign(s->nslots, 0);
  e = cudaMemcpy(s->d_outs, outs.data(), sizeof(SlotOut) * s->nslots, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { msvgb_server_destroy(s); return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
  *ret = s;
  return MSVGB_eslOK;
}

extern "C" int msvgb_server_slots(const msvgb_server *s) { return s ? s->nslots : -1; }

// The request's own single-query search (slot already taken, its per-length
// tables uploaded): the profile's tables go to pool memory on the upload
// stream, the search is enqueued on the next search stream, and the slot's
// event records its end.
static int submit_solo(msvgb_server *s, const msvgb_om *om, const msvgb_detail::ProfileTables &pt, int slot) {
  uint8_t *base = s->d_slot_mem + s->slot_bytes * slot;
  const std::vector<uint32_t> *parts[4] = {&pt.st, &pt.mt, &pt.stg, &pt.mtg};
  size_t off[5] = {0, 0, 0, 0, 0};
  for (int k = 0; k < 4; ++k) off[k + 1] = off[k] + (parts[k]->size() * 4 + 255) / 256 * 256;
  cudaMemPool_t pool = msvgb_detail::scratch_pool(s->device);
  if (!pool) return fail(MSVGB_eslESYS, "serve: no memory pool");
  uint8_t *tabs = nullptr;
  cudaError_t e = cudaMallocFromPoolAsync((void **) &tabs, off[4], pool, s->upload);
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    if (!parts[k]->empty())
      e = cudaMemcpyAsync(tabs + off[k], parts[k]->data(), parts[k]->size() * 4, cudaMemcpyHostToDevice, s->upload);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->upload);
  if (e != cudaSuccess) {
    if (tabs) cudaFreeAsync(tabs, s->upload);
    return fail(MSVGB_eslEMEM, std::string("serve tables: ") + cudaGetErrorString(e));
  }
  // a device view of those tables (kernel arguments only: nothing outlives the enqueue)
  msvgb_profile p;
  p.ctx = s->ctx; p.device = s->device; p.M = om->M; p.C = pt.C; p.f16 = pt.f16;
  p.tbm = om->tbm_b; p.tec = om->tec_b; p.base = om->base_b; p.bias = om->bias_b;
  p.scale = om->scale_b; p.mmu = om->mmu; p.mlambda = om->mlambda;
  p.d_stab = (uint32_t *) (tabs + off[0]); p.d_mtab = (uint32_t *) (tabs + off[1]);
  if (!pt.stg.empty()) {
    p.G = pt.G; p.Cg = pt.Cg; p.CI = pt.CI;
    p.d_stab_g = (uint32_t *) (tabs + off[2]); p.d_mtab_g = (uint32_t *) (tabs + off[3]);
  }
  p.lanes_auto = true;
  LenTables lt;
  lt.d_tjb = base + s->tab_off_tjb;
  lt.d_xjmin = base + s->tab_off_xjm;
  std::lock_guard<std::mutex> lk(s->mu);
  const int k = s->next_solo;
  s->next_solo ^= 1;
  msvgb_detail::SearchScratch sc;
  sc.stream = s->solo_stream[k];
  sc.ticket = s->d_solo_counters[k]; sc.aux = s->d_solo_counters[k] + 1; sc.list = s->d_solo_list[k];
  int st = msvgb_detail::enqueue_search(sc, &p, s->db, &lt, base + s->off_xj, base + s->off_fl, s->ctx->num_sms);
  cudaFreeAsync(tabs, sc.stream);                      // after the search, in stream order
  if (st != MSVGB_eslOK) return st;
  e = cudaEventRecord(s->solo_done[slot], sc.stream);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("serve search: ") + cudaGetErrorString(e));
  s->solo[slot] = 1;
  if (s->solo_pending++ == 0) __atomic_fetch_or(&s->h_ctl->stop, 2, __ATOMIC_SEQ_CST);
  s->solo_searches++;
  return MSVGB_eslOK;
}

static void release_slot(msvgb_server *s, int slot) {
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->ticket_of[slot] = 0;
    if (s->solo[slot]) {
      s->solo[slot] = 0;
      if (--s->solo_pending == 0) __atomic_fetch_and(&s->h_ctl->stop, ~2, __ATOMIC_SEQ_CST);
    }
    s->free_slots.push_back(slot);
  }
  s->slot_freed.notify_one();
}

extern "C" int msvgb_server_submit(msvgb_server *s, const msvgb_om *om, uint64_t *ret_ticket) {
  if (!s || !om || !ret_ticket) return fail(MSVGB_eslEINVAL, "msvgb_server_submit: bad arguments");
  const int C = multi_C(om->M);
  if (C < 0) return fail(MSVGB_eslEINVAL, "served profiles are limited to M <= 2047");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, cudaGetErrorString(e));
  const bool alone = s->solo_stream[0] && (double) om->M * (double) s->db->residues >= kSoloCells;
  // host-side tables first (no lock held): costs and the per-length pass thresholds
  std::vector<uint32_t> st, mt;
  msvgb_detail::ProfileTables pt;
  int G = 32, Cg = 0, CI = 0;
  if (alone) {
    int rc = msvgb_detail::build_profile_tables(s->ctx, om, pt);
    if (rc != MSVGB_eslOK) return rc;
  } else {
    int rc = msvgb_detail::build_cost_tables(om, 1, C, st, mt);
    if (rc != MSVGB_eslOK) return rc;
    G = msvgb_detail::lanes_for(s->ctx, om->M, -1, nullptr);     // lanes per sequence of the SSV pass
    if (G < 32 && group_C(om->M, G) < 0) G = 32;
    Cg = G < 32 ? group_C(om->M, G) : 0;
    CI = G < 32 ? multi_hyb_words(Cg, G) : 0;                    // mixed-width table where the width has one
    if (G < 32) st = CI ? msvgb_detail::build_hyb_table(om, Cg, G, CI) : msvgb_detail::build_group_table(om, Cg, G);
  }
  msvgb_profile tmp;                                   // scalar view for the threshold search
  tmp.M = om->M; tmp.C = C; tmp.tbm = om->tbm_b; tmp.tec = om->tec_b; tmp.base = om->base_b;
  tmp.bias = om->bias_b; tmp.scale = om->scale_b; tmp.mmu = om->mmu; tmp.mlambda = om->mlambda;
  const int Lmax = s->db->Lmax;
  std::vector<uint8_t> xjm(Lmax + 1, 255), tjb(Lmax + 1);
  for (int L = 0; L <= Lmax; ++L) tjb[L] = msvgb_tjb_b(om->scale_b, L);
  int hint = -1;                                       // the last length's answer (lengths ascend)
  for (int L : s->db->distinct_len) {
    if (L == 0) continue;
    const int v = msvgb_detail::xjmin_for(&tmp, L, s->F1, hint);
    if (v < 0) return fail(MSVGB_eslESYS, "F1 pass set is not monotone in xJ");
    xjm[L] = (uint8_t) v;
    hint = v;
  }
  // admission: wait for a free slot
  int slot;
  uint64_t ticket;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->slot_freed.wait(lk, [&] { return !s->free_slots.empty(); });
    slot = s->free_slots.back();
    s->free_slots.pop_back();
    ticket = s->next_ticket++;
    s->ticket_of[slot] = ticket;
    s->gen[slot]++;
  }
  uint8_t *base = s->d_slot_mem + s->slot_bytes * slot;
  e = cudaMemcpyAsync(base + s->tab_off_tjb, tjb.data(), Lmax + 1, cudaMemcpyHostToDevice, s->upload);
  if (e == cudaSuccess) e = cudaMemcpyAsync(base + s->tab_off_xjm, xjm.data(), Lmax + 1, cudaMemcpyHostToDevice, s->upload);
  if (e != cudaSuccess) {
    release_slot(s, slot);
    return fail(MSVGB_eslESYS, std::string("serve upload: ") + cudaGetErrorString(e));
  }
  if (alone) {
    const int rc = submit_solo(s, om, pt, slot);
    if (rc != MSVGB_eslOK) {
      cudaStreamSynchronize(s->upload);
      release_slot(s, slot);
      return rc;
    }
    *ret_ticket = ((uint64_t) slot << 48) | ticket;
    return MSVGB_eslOK;
  }
  ProfDev P;
  P.M = om->M; P.C = C; P.tbm = om->tbm_b; P.tec = om->tec_b; P.base = om->base_b; P.bias = om->bias_b;
  P.G = G; P.Cg = Cg; P.CI = CI;
  P.stab = (const uint32_t *) base; P.mtab = (const uint32_t *) (base + st.size() * 4);
  P.tjb = base + s->tab_off_tjb; P.xjmin = base + s->tab_off_xjm; P.ssv_f16 = 1;
  __atomic_store_n(&s->h_ctl->done[slot], 0ull, __ATOMIC_SEQ_CST);
  e = cudaMemcpyAsync(base, st.data(), st.size() * 4, cudaMemcpyHostToDevice, s->upload);
  if (e == cudaSuccess) e = cudaMemcpyAsync((uint8_t *) P.mtab, mt.data(), mt.size() * 4, cudaMemcpyHostToDevice, s->upload);
  if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_slots + slot, &P, sizeof(ProfDev), cudaMemcpyHostToDevice, s->upload);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->upload);       // visible before the items are
  if (e != cudaSuccess) {
    release_slot(s, slot);
    return fail(MSVGB_eslESYS, std::string("serve upload: ") + cudaGetErrorString(e));
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (int64_t k = 0; k < s->items_per_req; ++k) {
      ServeItem &it = s->h_ring[(s->tail + k) & (s->cap - 1)];
      it.slot = slot; it.gen = s->gen[slot];
      it.s_begin = s->chunk_begin[k]; it.s_end = s->chunk_begin[k + 1];
    }
    s->tail += s->items_per_req;
    __atomic_store_n(&s->h_ctl->tail, s->tail, __ATOMIC_SEQ_CST);     // publish
    if (!kernel_running(s)) {                                         // the loop left: start it
      int r = launch_serve(s);
      if (r != MSVGB_eslOK) return r;
    }
  }
  *ret_ticket = ((uint64_t) slot << 48) | ticket;
  return MSVGB_eslOK;
}

extern "C" int msvgb_server_wait(msvgb_server *s, uint64_t ticket, uint8_t *out_xj, uint8_t *out_flags,
                                 double timeout_s) {
  if (!s) return fail(MSVGB_eslEINVAL, "NULL server");
  const int slot = (int) (ticket >> 48);
  if (slot < 0 || slot >= s->nslots || s->ticket_of[slot] != (ticket & 0xFFFFFFFFFFFFull))
    return fail(MSVGB_eslEINVAL, "unknown ticket");
  cudaSetDevice(s->device);
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    if (s->solo[slot]) {                                              // its own search
      const cudaError_t q = cudaEventQuery(s->solo_done[slot]);
      if (q == cudaSuccess) break;
      if (q != cudaErrorNotReady) return fail(MSVGB_eslESYS, std::string("serve search: ") + cudaGetErrorString(q));
    } else {
      const unsigned long long d = __atomic_load_n(&s->h_ctl->done[slot], __ATOMIC_ACQUIRE);
      if ((int64_t) d >= s->items_per_req) break;
      if (__atomic_load_n(&s->h_ctl->live, __ATOMIC_ACQUIRE) == 0) {
        std::lock_guard<std::mutex> lk(s->mu);                        // the loop left with work
        if (!kernel_running(s)) {                                     // still queued: restart it
          int r = launch_serve(s);
          if (r != MSVGB_eslOK) return r;
        }
      }
    }
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > timeout_s) return fail(MSVGB_eslESYS, "msvgb_server_wait: timed out");
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  uint8_t *base = s->d_slot_mem + s->slot_bytes * slot;
  cudaError_t e = cudaSuccess;
  if (out_xj) e = cudaMemcpy(out_xj, base + s->off_xj, s->db->n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && out_flags) e = cudaMemcpy(out_flags, base + s->off_fl, s->db->n, cudaMemcpyDeviceToHost);
  release_slot(s, slot);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("serve results: ") + cudaGetErrorString(e));
  return MSVGB_eslOK;
}

extern "C" uint64_t msvgb_server_launches(const msvgb_server *s) { return s ? s->launches : 0; }

extern "C" uint64_t msvgb_server_solo_searches(const msvgb_server *s) { return s ? s->solo_searches : 0; }
