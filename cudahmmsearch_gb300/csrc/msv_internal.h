// msv_internal.h -- definitions shared by the translation units of the C ABI
// (not part of the public interface).
#pragma once
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_kernel_impl.cuh"
#include "msv_group.cuh"

struct TuneTable;                                       // msv_tune.cu

// A profile of the drop-in msvgb_MSVFilter's per-context cache: the device
// tables and a copy of the bytes they were built from (the om's scalar MSV
// fields and its rbv vectors), so a hit is confirmed byte for byte.
struct DropinEntry {
  const uint8_t *rbv_ptr = nullptr;   // fast-path key: the caller's vectors and M
  int M = 0;
  uint64_t hash = 0;                  // content hash (masked: see msvgb_ctx::hash_mask)
  std::vector<uint8_t> image;         // M, Kp, tbm, tec, base, bias, scale, then rbv
  msvgb_profile *p = nullptr;
  uint64_t last_use = 0;
};

struct msvgb_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  unsigned long long *d_ticket = nullptr;
  std::mutex mu;                                        // serialises the single-call path
  std::vector<DropinEntry> dropin;                      // single-call profile cache (least recently used out)
  uint64_t dropin_clock = 0;
  uint64_t hash_mask = ~0ull;                           // content-hash bits kept (tests force collisions)
  // single-call scratch: one block [ticket | meta | tjb/xjmin table | residues]
  // staged in pinned host memory and uploaded in one copy
  uint8_t *d_one = nullptr; size_t d_one_cap = 0;
  uint8_t *h_one = nullptr; size_t h_one_cap = 0;
  uint8_t *d_out = nullptr;
  int *d_bad = nullptr;                                 // database packing: invalid-code flag
  int64_t *d_list = nullptr; size_t list_cap = 0;       // G-lane search: sequences left for the full MSV
  unsigned long long *d_aux = nullptr;                  // [0] second ticket, [1] list count, [2] third ticket
  cudaStream_t side = nullptr;                          // long targets of the lane-group search
  cudaStream_t upload = nullptr;                        // chunk uploads of msvgb_search_host
  cudaStream_t dma = nullptr;                           // raw residue copies of database creation
  void *h_pin = nullptr; size_t h_pin_cap = 0;          // small pinned scratch (length counts, flags)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  TuneTable *tune = nullptr;                            // lane counts measured by msvgb_autotune
  std::mutex tune_mu;
};

// Per-length tables of a profile at one F1 threshold: tjb_b(L) and the
// smallest passing xJ at length L. They depend on L only, not on the
// database, so they grow with the longest sequence seen and entries are
// computed for the lengths that occur.
struct LenTables {
  double F1 = -1.0;
  int cap = 0;                        // entries 0..cap-1
  std::vector<uint8_t> tjb;
  std::vector<int16_t> xjm;           // -1: not computed yet
  uint8_t *d_tjb = nullptr;
  uint8_t *d_xjmin = nullptr;         // 255 where not computed (never read)
  std::vector<void *> retired;        // smaller device tables of earlier sizes (kernels may still read them)
};

struct msvgb_profile {
  msvgb_ctx *ctx = nullptr;
  int device = 0;            // own copy: destroy must not touch ctx (it may be gone)
  int M = 0, C = 0, f16 = 0;
  uint8_t tbm = 0, tec = 0, base = 0, bias = 0;
  float scale = 0.f, mmu = 0.f, mlambda = 0.f;
  uint32_t *d_stab = nullptr, *d_mtab = nullptr;
  int G = 32;                         // lanes per sequence in the SSV pass (32: fused kernel)
  bool lanes_auto = false;            // G chosen by msvgb_profile_create (small searches then use 32)
  int Cg = 0;                         // DP words per lane of the G-lane table
  int CI = 0;                         // of those, words whose costs are bytes (mixed-width table); 0: all f16
  uint32_t *d_stab_g = nullptr;       // SSV table in the G-lane layout (GroupLayout, or HybLayout when CI > 0)
  uint32_t *d_mtab_g = nullptr;       // MSV table in the G-lane layout (GroupLayout, unclamped costs)
  std::vector<LenTables *> tables;    // one per F1 value used
  std::mutex tables_mu;
};

struct msvgb_db {
  msvgb_ctx *ctx = nullptr;
  int device = 0;            // own copy: destroy must not touch ctx (it may be gone)
  int64_t n = 0, residues = 0;
  int Lmax = 0;
  uint8_t *d_codes = nullptr;
  int64_t *d_start = nullptr, *d_orig = nullptr;
  int32_t *d_len = nullptr;
  std::vector<int32_t> distinct_len;  // sorted ascending
  std::vector<int64_t> len_count;     // sequences of each distinct length
  uint64_t serial = 0;
  int64_t n_long = 0;                 // sequences of length >= kLongTarget (they sort first)
  // Sequences of length >= T (they sort first).
  int64_t count_at_least(int T) const {
    int64_t c = 0;
    for (size_t i = distinct_len.size(); i-- > 0 && distinct_len[i] >= T;) c += len_count[i];
    return c;
  }
  int64_t packed_bytes = 0;           // size of d_codes
  cudaEvent_t ready = nullptr;        // set when packed asynchronously: completes when the data is in place
  int64_t *d_inv = nullptr;           // original index -> sorted slot, built on first use
  // Created in chunks (msvgb_search_host): sorted slots [chunk_slot[k],
  // chunk_slot[k+1]) hold the input's chunk k, longest first within it; the
  // chunk's residues are in d_raw once chunk_up[k] completes and are packed
  // by pack_chunk_on (then d_raw and d_src are released by release_chunks_on).
  std::vector<int64_t> chunk_slot;
  std::vector<std::vector<int32_t>> chunk_len;    // per chunk: its distinct lengths, descending
  std::vector<std::vector<int64_t>> chunk_cnt;    // and their counts
  std::vector<cudaEvent_t> chunk_up;
  uint8_t *d_raw = nullptr;
  int64_t *d_src = nullptr;
  int *d_bad_chunks = nullptr;
  // Sequences of length >= T in chunk k (they open its range).
  int64_t chunk_count_at_least(size_t k, int T) const {
    int64_t c = 0;
    for (size_t i = 0; i < chunk_len[k].size() && chunk_len[k][i] >= T; ++i) c += chunk_cnt[k][i];
    return c;
  }
};

// Targets this long are scored with 32 lanes per sequence even when the
// profile's SSV pass runs on lane groups: at 8 or 16 lanes one sequence takes
// 2-4x longer, and a single long target would set the length of the launch.
constexpr int kLongTarget = 2400;

// From this model length up to 2047 nodes, 32-lane profiles also get the
// split passes (32-lane groups with the mixed-width SSV table, then the full
// MSV of the undecided), which large searches use instead of the fused
// kernel (measured on 1,000,000 sequences: +2% at M = 1100, +8% at 1500,
// +2% at 1984).
constexpr int kWideSplitMinM = 1024;

namespace msvgb_detail {
// Device-side timeline of one call (MSVGB_GPU_TRACE; unlike MSVGB_TRACE it
// adds no synchronization): timed events recorded on the streams the work
// runs on (and host times of the marks), printed relative to the first
// timed mark once the call's work is done. Marks may come from several
// threads.
inline bool gpu_trace_on() { static const bool on = getenv("MSVGB_GPU_TRACE") != nullptr; return on; }
struct GpuTrace {
  struct Mark { std::string what; cudaEvent_t ev; std::chrono::steady_clock::time_point host; };
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  std::vector<Mark> marks;
  std::mutex mu;
  // s: the stream to time on; null: host time only
  void mark(const std::string &what, cudaStream_t s) {
    if (!gpu_trace_on()) return;
    cudaEvent_t e = nullptr;
    if (s && cudaEventCreate(&e) == cudaSuccess && cudaEventRecord(e, s) != cudaSuccess) { cudaEventDestroy(e); e = nullptr; }
    std::lock_guard<std::mutex> lk(mu);
    marks.push_back(Mark{what, e, std::chrono::steady_clock::now()});
  }
  void print() {
    std::lock_guard<std::mutex> lk(mu);
    cudaEvent_t first = nullptr;
    for (auto &m : marks) if (m.ev) { first = m.ev; break; }
    for (auto &m : marks) {
      float ms = -1.f;
      if (m.ev && cudaEventSynchronize(m.ev) == cudaSuccess) cudaEventElapsedTime(&ms, first, m.ev);
      fprintf(stderr, "msvgb trace: %-30s gpu %8.3f ms   host %8.3f ms\n", m.what.c_str(), ms,
              std::chrono::duration<double, std::milli>(m.host - t0).count());
    }
    for (auto &m : marks) if (m.ev) cudaEventDestroy(m.ev);      // after the loop: first is the reference
    marks.clear();
  }
};
// The database's original-index -> sorted-slot table (db->d_inv), built on
// the context's stream at first use.
cudaError_t ensure_inverse(msvgb_ctx *c, const msvgb_db *db);
// HMMER's amino background frequencies, Easel code order A..Y (msv_sample.cu).
extern const float kAminoBg[20];
// Records msg as the calling thread's last error and returns code.
int fail(int code, const std::string &msg);
// Launches the search kernel instantiated for C words per lane.
cudaError_t dispatch(int C, bool f16, const msvgb::LaunchArgs &a, int sms);
// Smallest xJ passing the F1 gate at length L (255: none); -1 if the pass set
// is not monotone in xJ.
// hint: the answer at a nearby length (walked from instead of a binary search), or -1.
int xjmin_for(const msvgb_profile *p, int L, double F1, int hint = -1);
// Device tables of a profile; force_C > 0 imposes the DP width.
int profile_build_width(msvgb_ctx *ctx, const msvgb_om *om, int want_f16, int force_C, msvgb_profile **ret);
// Host images of the device cost tables of a profile at DP width C.
int build_cost_tables(const msvgb_om *om, int f16, int C, std::vector<uint32_t> &st, std::vector<uint32_t> &mt);
// Host images of every device table msvgb_profile_create makes for om, at the
// same widths, lane choice and table types.
struct ProfileTables {
  int C = 0, f16 = 1;                   // 32-lane tables: DP width, f16 or int8 SSV costs
  int G = 32, Cg = 0, CI = 0;           // lane-group tables: lanes, DP width, 8-bit words (none when empty)
  std::vector<uint32_t> st, mt;         // 32-lane SSV and MSV tables
  std::vector<uint32_t> stg, mtg;       // G-lane SSV (mixed width when CI > 0) and MSV tables
};
int build_profile_tables(msvgb_ctx *ctx, const msvgb_om *om, ProfileTables &t);
// Launches the G-lane SSV pass (msv_group.cuh); CI > 0: the mixed-width table.
cudaError_t dispatch_group(int C, int G, int CI, const msvgb::GroupArgs &a, int sms);
// Default 8-bit words per lane of the G-lane SSV pass at DP width C (0: f16 only).
int hyb_default_words(int C, int G);
// Whether a mixed-width lane-group kernel is compiled for (C, G, CI).
bool hyb_compiled(int C, int G, int CI);
// Mixed-width lane-group SSV table (HybLayout<C, CI, G>, msv_group.cuh).
std::vector<uint32_t> build_hyb_table(const msvgb_om *om, int C, int G, int CI);
// Per-length tjb_b and pass-threshold tables of (profile, database, F1), cached in the profile.
int ensure_tables(msvgb_profile *p, const msvgb_db *db, double F1, LenTables **out);
// Lane-group SSV table of a profile (layout GroupLayout<C, G>, msv_group.cuh).
std::vector<uint32_t> build_group_table(const msvgb_om *om, int C, int G);
// Lane-group MSV table of the full recurrence (GroupLayout<C, G>, msv_row_group).
std::vector<uint32_t> build_group_msv_table(const msvgb_om *om, int C, int G);
// Launches the full-MSV pass of a list on lane groups (msv_list_group_kernel).
cudaError_t dispatch_list_group(int C, int G, const msvgb::ProfDev &P, const msvgb::DbDev &db, uint8_t *out_xj,
                                uint8_t *out_flags, unsigned long long *ticket, const int64_t *list,
                                const unsigned long long *list_count, int sms, cudaStream_t stream);
// Target-length bins of the lane choice: [0,150) [150,600) [600,2400) [2400,inf).
constexpr int kNLBins = 4;
int lbin_of(int L);
// Whether the lane-group SSV pass supports G lanes for a model of length M.
bool lanes_valid(int M, int G);
// Lanes per sequence for model length M on target-length bin lbin (-1: the
// whole mix), from the context's tuning table or the fixed rule; *variant
// (may be NULL) gets the SSV table type for 32 lanes.
int lanes_for(msvgb_ctx *c, int M, int lbin, int *variant);
void tune_free(msvgb_ctx *c);
// msvgb_batch_create with every (profile, length bin) at force_lanes lanes
// where the model length allows it (0: the context's choice).
int batch_create(msvgb_ctx *ctx, const msvgb_om *const *oms, int nprof, const msvgb_db *db, double F1,
                 void *d_xj, void *d_flags, int force_lanes, msvgb_batch **ret);
// Device scratch and streams of one single-profile search.
struct SearchScratch {
  cudaStream_t stream = nullptr;     // the search's stream
  cudaStream_t side = nullptr;       // long targets run here, concurrently (null: on stream, first)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;   // needed with side
  unsigned long long *ticket = nullptr;               // 1 counter
  unsigned long long *aux = nullptr;                  // 3 counters
  int64_t *list = nullptr;                            // room for every sequence of the database
};
// Enqueues the single-profile search of db (per-length tables t) with the
// lane-group pass when the profile has one (and the search is not small),
// else the 32-lane kernel. The database must be in place on sc.stream.
int enqueue_search(const SearchScratch &sc, const msvgb_profile *p, const msvgb_db *db, const LenTables *t,
                   uint8_t *d_xj, uint8_t *d_flags, int num_sms);
// Chunks of consecutive input sequences [cut[k], cut[k+1]), k < K, sorted
// each on its own (msv_pack.cu).
constexpr int kMaxChunks = 16;
struct ChunkCuts {
  int K = 1;
  int64_t cut[kMaxChunks + 1] = {0};
};
// Asynchronous creation (db_create_on).
struct AsyncPack {
  int *d_bad;      // device flag: set if a residue code is >= 29
  // Chunked: the input cut at these sequence indices (0 first, n last, at
  // most kMaxChunks chunks) is sorted chunk by chunk into one database; every
  // chunk's residues go up on the context's dma stream right after the
  // offsets, and nothing is packed: pack_chunk_on packs a chunk.
  const std::vector<int64_t> *cuts = nullptr;
};
// msvgb_search_host; with keep_db, the packed database is returned (resident,
// complete) instead of freed, for later stages on the same sequences.
int host_search(msvgb_ctx *c, const msvgb_profile *p, const uint8_t *codes, const int64_t *off, int64_t n,
                double F1, int64_t chunk_residues, uint8_t *out_xj, uint8_t *out_flags, msvgb_db **keep_db);
// Packs chunk k of a chunked database on stream st, once its residues are up.
int pack_chunk_on(msvgb_ctx *ctx, msvgb_db *db, int k, cudaStream_t st);
// Frees a chunked database's raw residues and scatter offsets on stream st,
// which must be ordered after every pack_chunk_on.
void release_chunks_on(msvgb_db *db, cudaStream_t st);
// msvgb_db_create on stream st; with a, asynchronous (see msv_api.cu).
int db_create_on(msvgb_ctx *ctx, const uint8_t *codes, const int64_t *off, int64_t n, cudaStream_t st,
                 msvgb_db **ret, const AsyncPack *a = nullptr);
// msvgb_db_destroy of a database made by db_create_on (every array pool
// memory) without cudaFree's device-wide wait: the arrays are freed in
// stream order on st, which must follow the database's last use.
void db_release_on(msvgb_db *db, cudaStream_t st);
// A fresh database serial (keys the per-length table caches).
uint64_t next_db_serial();
// Adds one to the count msvgb_kernel_launches() reports.
void count_launch();
// Scatters raw residues into the packed database layout (msv_pack.cu); sets
// *bad to nonzero if any code is >= 29.
cudaError_t launch_pack(const uint8_t *raw, const int64_t *src, const int64_t *start, const int32_t *len,
                        int64_t n, uint8_t *packed, int *bad, int num_sms, cudaStream_t stream);
// Device-side length sort (msv_pack.cu): lengths, their maximum and a
// validity flag; per-length counts; sorted placement.
cudaError_t launch_lengths(const int64_t *off, int64_t n, int32_t *len, unsigned *lmax, int *bad, int num_sms,
                           cudaStream_t stream);
// Counts per (chunk, length), in sorted key order: hist[k * (Lmax + 1) + Lmax - L]
// (zeroed by the caller); blk: sort_parts x K x sort_small_bound uint32 of
// scratch, left holding each part's first rank per short key for launch_place.
int sort_parts(int num_sms);
int sort_small_bound(int Lmax, int K);
cudaError_t launch_histogram(const int32_t *len, int64_t n, unsigned long long *hist, uint32_t *blk,
                             const ChunkCuts &cuts, int Lmax, int num_sms, cudaStream_t stream);
// inv[orig[s]] = s (original index -> sorted slot); ids[j] = inv[ids[j]].
cudaError_t launch_invert(const int64_t *orig, int64_t n, int64_t *inv, int num_sms, cudaStream_t stream);
cudaError_t launch_gather_ids(int64_t *ids, int64_t n, const int64_t *inv, int num_sms, cudaStream_t stream);
// order[k] = the list positions j sorted longest first by len[slots[j]] in
// 1024 length buckets (up to the order within a bucket); Lmax: the
// database's longest; cnt: 1024 int32 of scratch.
cudaError_t launch_order_by_length(const int64_t *slots, int64_t n, const int32_t *len, int Lmax, int32_t *cnt,
                                   int64_t *order, int num_sms, cudaStream_t stream);
// First slot and first packed byte of every key (scratch: bins_scratch_words
// int64); *pos the packed size, and 64 padding codes after it in codes.
int bins_scratch_words(int Lmax, int K);
cudaError_t launch_bins(const unsigned long long *hist, int Lmax, int K, int64_t *bin_slot, int64_t *bin_byte,
                        int64_t *scratch, int64_t *pos, uint8_t *codes, cudaStream_t stream);
// Stream-ordered scratch allocations of database creation come from this
// pool, which keeps up to 4 GiB mapped between calls (the default pool would
// unmap and map again every time).
cudaMemPool_t scratch_pool(int device);
// cursor: each key's first slot (used by the long sequences); blk as
// launch_histogram left it.
cudaError_t launch_place(const int64_t *off, const int32_t *len_in, int64_t n, unsigned long long *cursor,
                         const uint32_t *blk, const int64_t *bin_slot, const int64_t *bin_byte, int64_t *start,
                         int64_t *orig, int32_t *len, int64_t *src, const ChunkCuts &cuts, int Lmax, int num_sms,
                         cudaStream_t stream);
}  // namespace msvgb_detail

// Returns eslESYS (with the failing call in the message) from the enclosing
// function when a CUDA call fails.
#define CUDA_TRY(expr)                                                                       \
  do {                                                                                       \
    cudaError_t _e = (expr);                                                                 \
    if (_e != cudaSuccess)                                                                   \
      return fail(MSVGB_eslESYS, std::string(#expr) + ": " + cudaGetErrorString(_e));         \
  } while (0)

