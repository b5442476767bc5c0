// msv_tune.cu -- lanes per sequence (and SSV table type) per (model length,
// target-length bin), measured on the GPU at hand.
//
// The SSV pass runs with 32 lanes per sequence (one warp; f16 or int8 cost
// table) or with 16 or 8 lanes (2 or 4 sequences per warp in lockstep, f16
// table). Which is fastest depends on the model length M (words per lane per
// row against the per-row overhead) and on the target lengths (per-sequence
// setup against the row loop). For a ladder of model lengths the tuner times
//   - each choice per target-length bin inside the batched kernel (the one
//     that applies per-bin choices), on a batch of 8 copies of one sampled
//     profile against that bin's synthetic sequences, so that work items of
//     the copies interleave and the timing is throughput, not one long tail;
//   - each choice (int8 table included) on the single-query path against a
//     database with the usual protein length law (lognormal, median 300,
//     sigma 0.7): the choice for a whole length mix.
// It keeps the fastest per (M, bin) and for the mix, and can save / load the
// table. Without a table the choice is a fixed rule (default_lanes) that
// measurements on GB300 support.
// The reference has no counterpart: its SSE filter has one layout.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using msvgb_detail::fail;

namespace {

constexpr int kTuneM[] = {24, 40, 64, 96, 128, 192, 256, 320, 400, 480, 560, 680, 800, 920, 1000};
constexpr int kNM = sizeof(kTuneM) / sizeof(kTuneM[0]);
constexpr int kLEdge[] = {150, 600, 2400};                  // bins [0,150) [150,600) [600,2400) [2400,inf)
constexpr int kBinLo[] = {10, 150, 600, 2400};
constexpr int kBinHi[] = {150, 600, 2400, 9600};
constexpr int64_t kBinResidues[] = {16 << 20, 24 << 20, 32 << 20, 48 << 20};
constexpr int kNB = msvgb_detail::kNLBins;
constexpr int kCopies = 8;                                  // profiles per timed batch
struct Cand { int lanes, variant; };
constexpr Cand kCand[] = {{32, 1}, {32, 0}, {16, 1}, {8, 1}};
constexpr int kNC = sizeof(kCand) / sizeof(kCand[0]);
constexpr int kNV = kNB + 1;                                // values per candidate: bins, then the mix

// The rule used without a measured table (from the tuner's measurements on
// GB300): 8 lanes up to M = 511 (the widest 8-lane row, 32 words); up to
// M = 1023, 16 lanes for the length mix and for targets shorter than 600 in
// the batched kernel, 32 for longer ones; 32 above. (With the mixed-width
// table 8 lanes beat 16 at M = 504: 18.0 vs 16.4 TCUPS on 1,000,000
// sequences; with f16 tables alone, 16.6 vs 16.4.)
int default_lanes(int M, int lbin) {
  if (M >= 16 && M < 512) return 8;
  if (M >= 32 && M < 1024 && lbin <= 1) return 16;
  return 32;
}

bool cand_valid(int M, const Cand &c) {
  if (c.lanes == 32) return c.variant == 1 || M <= 3199;
  return msvgb_detail::lanes_valid(M, c.lanes);
}

std::string device_tag(int device, int *sms) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { *sms = 0; return "unknown"; }
  *sms = prop.multiProcessorCount;
  std::string s = prop.name;
  for (char &ch : s) if (ch == ' ' || ch == '\t') ch = '_';
  return s;
}

// Deterministic synthetic sequences: residues i.i.d. from HMMER's amino
// background (the composition decides how often SSV leaves a sequence to the
// full MSV: uniform residues would send a third of them there), lengths from
// 64 values spread over [lo, hi) (few distinct lengths keep the per-length
// pass tables cheap to build).
void synth_bin(int b, std::vector<uint8_t> &codes, std::vector<int64_t> &off) {
  uint64_t x = 0x9E3779B97F4A7C15ull ^ (uint64_t) (b + 1) * 0xBF58476D1CE4E5B9ull;
  auto next = [&]() { x ^= x << 13; x ^= x >> 7; x ^= x << 17; return x; };
  uint8_t lut[4096];                                        // inverse CDF of the background
  {
    double sum = 0, tot = 0;
    for (int a = 0; a < 20; ++a) tot += msvgb_detail::kAminoBg[a];
    int a = 0;
    for (int i = 0; i < 4096; ++i) {
      const double u = (i + 0.5) / 4096.0 * tot;
      while (a < 19 && sum + msvgb_detail::kAminoBg[a] <= u) sum += msvgb_detail::kAminoBg[a++];
      lut[i] = (uint8_t) a;
    }
  }
  codes.clear(); off.assign(1, 0);
  while ((int64_t) codes.size() < kBinResidues[b]) {
    const int L = kBinLo[b] + (int) ((next() % 64) * (uint64_t) (kBinHi[b] - kBinLo[b]) / 64);
    for (int i = 0; i < L; ++i) codes.push_back(lut[next() >> 52]);
    off.push_back((int64_t) codes.size());
  }
}

// The length mix: lognormal(ln 300, 0.7) lengths clipped to [10, 35000],
// residues from the background, about 192M residues (larger than L2, and
// long enough that launch overheads do not decide the choice).
void synth_mix(std::vector<uint8_t> &codes, std::vector<int64_t> &off) {
  uint64_t x = 0xD1B54A32D192ED03ull;
  auto next = [&]() { x ^= x << 13; x ^= x >> 7; x ^= x << 17; return x; };
  auto unif = [&]() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
  uint8_t lut[4096];
  {
    double sum = 0, tot = 0;
    for (int a = 0; a < 20; ++a) tot += msvgb_detail::kAminoBg[a];
    int a = 0;
    for (int i = 0; i < 4096; ++i) {
      const double u = (i + 0.5) / 4096.0 * tot;
      while (a < 19 && sum + msvgb_detail::kAminoBg[a] <= u) sum += msvgb_detail::kAminoBg[a++];
      lut[i] = (uint8_t) a;
    }
  }
  codes.clear(); off.assign(1, 0);
  while ((int64_t) codes.size() < (192 << 20)) {
    const double z = std::sqrt(-2.0 * std::log(unif())) * std::cos(6.283185307179586 * unif());
    const int L = (int) std::min(35000.0, std::max(10.0, std::exp(std::log(300.0) + 0.7 * z)));
    for (int i = 0; i < L; ++i) codes.push_back(lut[next() >> 52]);
    off.push_back((int64_t) codes.size());
  }
}

// Best-of-3 milliseconds of run() on the context's stream, after one warm-up.
template <class Run>
int time_best(msvgb_ctx *ctx, cudaEvent_t ev0, cudaEvent_t ev1, Run run, float *best_ms) {
  int st = run();
  *best_ms = 1e30f;
  for (int r = 0; r < 3 && st == MSVGB_eslOK; ++r) {
    cudaError_t e = cudaEventRecord(ev0, ctx->stream);
    if (e == cudaSuccess) st = run();
    if (e == cudaSuccess && st == MSVGB_eslOK) e = cudaEventRecord(ev1, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
    if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("autotune timing: ") + cudaGetErrorString(e));
    *best_ms = std::min(*best_ms, ms);
  }
  return st;
}

}  // namespace

struct TuneTable {
  std::string device;
  int sms = 0;
  // per measured model length: GCUPS of each candidate in each bin (0: not valid)
  std::vector<int> M;
  std::vector<std::vector<double>> gcups;   // [m][c * kNV + v], v = bin or kNB (mix)
  std::vector<std::vector<int>> best;       // [m][b], b == kNB: whole mix; candidate index
};

int msvgb_detail::lbin_of(int L) {
  int b = 0;
  while (b < kNB - 1 && L >= kLEdge[b]) ++b;
  return b;
}

bool msvgb_detail::lanes_valid(int M, int G) {
  if (G == 32) return true;
  if (G != 16 && G != 8) return false;
  const int C = M / (2 * G) + 1;
  return C >= 2 && C <= 32;
}

int msvgb_detail::lanes_for(msvgb_ctx *c, int M, int lbin, int *variant) {
  if (variant) *variant = 1;
  std::lock_guard<std::mutex> lk(c->tune_mu);
  const TuneTable *t = c->tune;
  if (t && !t->M.empty()) {
    size_t m = 0;                                           // nearest measured length (log scale)
    for (size_t i = 1; i < t->M.size(); ++i)
      if (std::fabs(std::log((double) M / t->M[i])) < std::fabs(std::log((double) M / t->M[m]))) m = i;
    const int ci = t->best[m][lbin < 0 || lbin >= kNB ? kNB : lbin];
    if (ci >= 0 && cand_valid(M, kCand[ci])) {
      if (variant) *variant = kCand[ci].variant;
      return kCand[ci].lanes;
    }
  }
  return default_lanes(M, lbin);
}

void msvgb_detail::tune_free(msvgb_ctx *c) {
  delete c->tune;
  c->tune = nullptr;
}

extern "C" int msvgb_autotune(msvgb_ctx *ctx, double budget_s) {
  if (!ctx) return fail(MSVGB_eslEINVAL, "ctx is NULL");
  if (budget_s <= 0) budget_s = 60.0;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, cudaGetErrorString(e));
  const auto t0 = std::chrono::steady_clock::now();
  TuneTable *t = new TuneTable();
  t->device = device_tag(ctx->device, &t->sms);

  msvgb_db *db[kNB] = {};
  msvgb_db *mix = nullptr;
  int64_t residues[kNB] = {}, mix_res = 0;
  uint8_t *d_out = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int st = MSVGB_eslOK;
  int64_t nmax = 0;
  {
    std::vector<uint8_t> codes;
    std::vector<int64_t> off;
    for (int b = 0; b < kNB && st == MSVGB_eslOK; ++b) {
      synth_bin(b, codes, off);
      const int64_t n = (int64_t) off.size() - 1;
      st = msvgb_db_create(ctx, codes.data(), off.data(), n, &db[b]);
      residues[b] = (int64_t) codes.size();
      nmax = std::max(nmax, kCopies * n);
    }
    synth_mix(codes, off);
    if (st == MSVGB_eslOK) st = msvgb_db_create(ctx, codes.data(), off.data(), (int64_t) off.size() - 1, &mix);
    mix_res = (int64_t) codes.size();
    nmax = std::max(nmax, (int64_t) off.size() - 1);
  }
  if (st == MSVGB_eslOK) {
    e = cudaMalloc(&d_out, 2 * (size_t) nmax);
    if (e == cudaSuccess) e = cudaEventCreate(&ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ev1);
    if (e != cudaSuccess) st = fail(MSVGB_eslEMEM, std::string("autotune: ") + cudaGetErrorString(e));
  }
  for (int mi = 0; mi < kNM && st == MSVGB_eslOK; ++mi) {
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el > budget_s) break;                                   // the rest keep the default rule
    const int M = kTuneM[mi];
    const int Q = std::max(2, (M + 15) / 16);
    std::vector<uint8_t> rbv((size_t) 29 * Q * 16);
    msvgb_om om;
    double lambda = 0;
    st = msvgb_sample_om(1000u + (uint32_t) M, M, rbv.data(), &om, &lambda);
    if (st != MSVGB_eslOK) break;
    std::vector<double> g(kNC * kNV, 0.0);
    float ms = 0;
    // the whole mix on the single-query path
    for (int ci = 0; ci < kNC && st == MSVGB_eslOK; ++ci) {
      if (!cand_valid(M, kCand[ci])) continue;
      msvgb_profile *p = nullptr;
      st = msvgb_profile_create_ex(ctx, &om, kCand[ci].variant, &p);
      if (st == MSVGB_eslOK && kCand[ci].lanes < 32) st = msvgb_profile_set_lanes(p, &om, kCand[ci].lanes);
      const bool as_asked = st == MSVGB_eslOK && p->f16 == kCand[ci].variant;
      if (as_asked) {
        const int64_t n = msvgb_db_nseq(mix);
        st = time_best(ctx, ev0, ev1, [&] { return msvgb_search_device(ctx, p, mix, 0.02, d_out, d_out + n); }, &ms);
        if (st == MSVGB_eslOK) g[ci * kNV + kNB] = (double) M * mix_res / (ms * 1e-3) / 1e9;
      }
      msvgb_profile_destroy(p);
    }
    // each length bin in the batched kernel (f16 tables)
    const msvgb_om *copies[kCopies];
    for (auto &c : copies) c = &om;
    for (int ci = 0; ci < kNC && st == MSVGB_eslOK; ++ci) {
      if (kCand[ci].variant != 1 || !cand_valid(M, kCand[ci])) continue;
      for (int b = 0; b < kNB && st == MSVGB_eslOK; ++b) {
        const int64_t n = msvgb_db_nseq(db[b]);
        msvgb_batch *bt = nullptr;
        st = msvgb_detail::batch_create(ctx, copies, kCopies, db[b], 0.02, d_out, d_out + kCopies * n,
                                        kCand[ci].lanes, &bt);
        if (st == MSVGB_eslOK) st = time_best(ctx, ev0, ev1, [&] { return msvgb_batch_run(bt); }, &ms);
        if (st == MSVGB_eslOK) g[ci * kNV + b] = (double) kCopies * M * residues[b] / (ms * 1e-3) / 1e9;
        msvgb_batch_destroy(bt);
      }
    }
    if (st != MSVGB_eslOK) break;
    std::vector<int> best(kNV, -1);
    for (int v = 0; v < kNV; ++v)
      for (int ci = 0; ci < kNC; ++ci)
        if (g[ci * kNV + v] > 0 && (best[v] < 0 || g[ci * kNV + v] > g[best[v] * kNV + v])) best[v] = ci;
    t->M.push_back(M);
    t->gcups.push_back(g);
    t->best.push_back(best);
  }
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  cudaFree(d_out);
  for (auto *d : db) msvgb_db_destroy(d);
  msvgb_db_destroy(mix);
  if (st != MSVGB_eslOK) { delete t; return st; }
  std::lock_guard<std::mutex> lk(ctx->tune_mu);
  delete ctx->tune;
  ctx->tune = t;
  return MSVGB_eslOK;
}

extern "C" int msvgb_tune_save(msvgb_ctx *ctx, const char *path) {
  if (!ctx || !path) return fail(MSVGB_eslEINVAL, "NULL argument");
  std::lock_guard<std::mutex> lk(ctx->tune_mu);
  const TuneTable *t = ctx->tune;
  if (!t) return fail(MSVGB_eslEINVAL, "no tuning table in this context");
  FILE *f = fopen(path, "w");
  if (!f) return fail(MSVGB_eslENOTFOUND, std::string("cannot write ") + path);
  fprintf(f, "msvgb-tune 2\ndevice %s %d\nlbins", t->device.c_str(), t->sms);
  for (int b = 0; b < kNB - 1; ++b) fprintf(f, " %d", kLEdge[b]);
  fprintf(f, "\ncandidates");
  for (const Cand &c : kCand) fprintf(f, " %d/%d", c.lanes, c.variant);
  fprintf(f, "\n");
  for (size_t m = 0; m < t->M.size(); ++m) {
    fprintf(f, "m %d best", t->M[m]);
    for (int b = 0; b <= kNB; ++b) fprintf(f, " %d", t->best[m][b]);
    fprintf(f, " gcups");
    for (double v : t->gcups[m]) fprintf(f, " %.1f", v);
    fprintf(f, "\n");
  }
  const bool ok = ferror(f) == 0;
  if (fclose(f) != 0 || !ok) return fail(MSVGB_eslEWRITE, std::string("write failed: ") + path);
  return MSVGB_eslOK;
}

extern "C" int msvgb_tune_load(msvgb_ctx *ctx, const char *path) {
  if (!ctx || !path) return fail(MSVGB_eslEINVAL, "NULL argument");
  FILE *f = fopen(path, "r");
  if (!f) return fail(MSVGB_eslENOTFOUND, std::string("cannot open ") + path);
  TuneTable *t = new TuneTable();
  char name[256] = {0};
  int ver = 0, sms = 0;
  int ok = fscanf(f, " msvgb-tune %d device %255s %d", &ver, name, &sms) == 3 && ver == 2;
  for (int b = 0; ok && b < kNB - 1; ++b) {
    int v = 0;
    ok = fscanf(f, b == 0 ? " lbins %d" : " %d", &v) == 1 && v == kLEdge[b];
  }
  for (int c = 0; ok && c < kNC; ++c) {
    int l = 0, v = 0;
    ok = fscanf(f, c == 0 ? " candidates %d/%d" : " %d/%d", &l, &v) == 2 && l == kCand[c].lanes &&
         v == kCand[c].variant;
  }
  while (ok) {
    int M = 0;
    const int r = fscanf(f, " m %d best", &M);
    if (r == EOF) break;
    if (r != 1 || M < 1) { ok = 0; break; }
    std::vector<int> best(kNB + 1);
    for (int b = 0; ok && b <= kNB; ++b) ok = fscanf(f, " %d", &best[b]) == 1 && best[b] >= -1 && best[b] < kNC;
    ok = ok && fscanf(f, " gcups") == 0;
    std::vector<double> g(kNC * kNV);
    for (size_t i = 0; ok && i < g.size(); ++i) ok = fscanf(f, " %lf", &g[i]) == 1;
    if (ok) { t->M.push_back(M); t->best.push_back(best); t->gcups.push_back(g); }
  }
  fclose(f);
  if (!ok) { delete t; return fail(MSVGB_eslEFORMAT, std::string("not a tuning table: ") + path); }
  t->device = name;
  t->sms = sms;
  int here_sms = 0;
  const std::string here = device_tag(ctx->device, &here_sms);
  if (here != t->device || here_sms != t->sms) {
    delete t;
    return fail(MSVGB_eslEINCOMPAT, "tuning table was measured on " + std::string(name) + ", this GPU is " + here);
  }
  std::lock_guard<std::mutex> lk(ctx->tune_mu);
  delete ctx->tune;
  ctx->tune = t;
  return MSVGB_eslOK;
}

extern "C" int msvgb_tune_lanes(msvgb_ctx *ctx, int M, int L, int *ret_variant) {
  if (!ctx || M < 1) return -1;
  return msvgb_detail::lanes_for(ctx, M, L < 0 ? -1 : msvgb_detail::lbin_of(L), ret_variant);
}
