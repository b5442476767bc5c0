// msv_bias.cu -- the bias filter of p7_Pipeline on the GPU, and the gate of
// every filter stage.
//
// p7_bg_FilterScore (src/p7_bg.c:473-483) scores a sequence with a two-state
// HMM: state 0 emits the background composition, state 1 the model's
// (p7_bg_SetFilter, src/p7_bg.c:431-453, with p7_bg_SetLength's t[0][0]);
// esl_hmm_Forward (easel/esl_hmm.c:351-409) runs it scaled, dividing every
// row by its maximum and summing the logs of those maxima. The recurrence is
// sequential in the residues and has two states, so one thread scores one
// listed sequence, with the reference's float operations in its order:
// round-to-nearest multiplies, adds and divides written as intrinsics (no
// contraction into FMA), and each row's log taken in double and rounded to
// float as the reference's double log() of a float is. The double log is a
// table-driven one (Tang's method, ACM TOMS 15(2), 1989: reduce by a table
// entry, then a short polynomial; here 512 entries and the Taylor series of
// log1p to degree 6), about 8 double operations instead of the library
// log's many more on this part's narrow FP64 pipe; a row whose result lies
// within 64 units in the last place of a float rounding boundary takes the
// library log instead. The length term (logf of p1 and 1 - p1) is added on the host with
// the C library's logf.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using namespace msvgb;
using msvgb_detail::fail;

namespace {

constexpr int kLogTab = 512;

struct BiasDev {
  float eo[NRES][2];       // emission odds: [x][0] background state, [x][1] model-composition state
  float t10, t11;          // biased-state transitions 1->0, 1->1 (t[1][2] = 1)
  float pi0, pi1;
  double2 logtab[kLogTab]; // per top-9-mantissa-bit interval: (1/c, log c) of its reduction point c
};

// float(log((double) m)) for a float m > 0: m = 2^e f, f in [1, 2); the top 9
// bits of f pick the interval [1 + j/512, 1 + (j+1)/512), whose point c is its
// midpoint (halved, with e + 1, from j = 212 (f > 1.414) up, so that f/c stays
// near 1 and no sum cancels); the intervals next to 1 use c = 1 (m near 1:
// log m = log1p(f - 1), no table term). f, halved or not, is assembled as a
// double from the float's bits. log m = e ln2 + log c + log1p(r), r = f (1/c)
// - 1 by one fused multiply-add, |r| < 2^-9; log1p to degree 6 (truncation <
// 2^-56 relative). The result's distance to the nearest float rounding
// boundary is read from the low 29 bits of the double: within 64 units of the
// last place the library log decides instead.
__device__ __forceinline__ float log_row(float m, const double2 *tab) {
  const uint32_t b = __float_as_uint(m);
  if (b - 0x00800000u >= 0x7f000000u) return (float) log((double) m);   // 0, subnormal, inf, nan, negative
  const int j = (b >> 14) & 0x1ff;
  const int half = j >= 212;
  const int e = (int) (b >> 23) - 127 + half;
  const double f = __longlong_as_double((long long) (((uint64_t) (b & 0x7fffffu) << 29) |
                                                     ((uint64_t) (1023 - half) << 52)));
  const double2 t = tab[j];
  const double r = fma(f, t.x, -1.0);
  double p = fma(-1.0 / 6, r, 1.0 / 5);
  p = fma(p, r, -1.0 / 4);
  p = fma(p, r, 1.0 / 3);
  p = fma(p, r, -1.0 / 2);
  p = fma(p, r, 1.0);
  double y;
  if (e == 0) {
    y = fma(p, r, t.y);
  } else {
    const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10;
    const double de = (double) e;
    y = fma(de, ln2_hi, t.y + fma(de, ln2_lo, p * r));
  }
  const long long dist = (long long) ((uint64_t) __double_as_longlong(y) & 0x1fffffffull) - 0x10000000ll;
  if (dist > -64 && dist < 64) return (float) log((double) m);      // near a float rounding boundary
  return __double2float_rn(y);
}

// float(log(m)) in float-float arithmetic on the FP32 pipe, for m in
// [2^-8.5, 2^8.5) (exponents -8 .. 8 after the reduction; the row maxima of
// the filter's scaled Forward lie there): the top 11 mantissa bits pick a
// reduction point c (2048 intervals; c = 1 next to 1) with 1/c and log c
// stored as float pairs; d = f - c is exact, r = d/c a float pair by fused
// multiply-adds, log1p(r) = r - r^2/2 (pairs) + r^3/3 - r^4/4 + r^5/5 (float;
// |r| < 2^-11.5, truncation < 2^-57), summed with error-free two-sums. The
// result is returned only when it is at least 2^-42 (relative) away from a
// float rounding boundary -- every float in [2^-8, 2^8) checked on the host
// against the C library's double log: 0 differences, 737 of 134 M left to
// the double path; otherwise (and for other exponents) the double path
// decides.
__device__ float4 g_logff[2048];

__device__ __forceinline__ float fsub(float a, float b) { return __fadd_rn(a, -b); }

// Branch-free: ok says whether the returned value is the result (the
// arithmetic runs on any input; the table index is always in range).
__device__ __forceinline__ float log_ff(float m, bool &ok) {
  const uint32_t b = __float_as_uint(m);
  const int j = (b >> 12) & 0x7ff;
  const int half = j >= 849;
  const int e = (int) (b >> 23) - 127 + half;
  const bool in_range = b - 0x00800000u < 0x7f000000u && e >= -8 && e <= 8;
  const float f = __uint_as_float((b & 0x7fffffu) | ((uint32_t) (127 - half) << 23));
  const float4 t = g_logff[j];                               // 1/c (hi, lo), log c (hi, lo)
  const float c = (j == 0 || j == 2047) ? 1.0f : __fmul_rn(half ? 0.5f : 1.0f, 1.0f + ((float) j + 0.5f) / 2048.0f);
  const float d = fsub(f, c);                                // exact
  const float rh = __fmul_rn(d, t.x);
  const float rl = __fadd_rn(__fmaf_rn(d, t.x, -rh), __fmul_rn(d, t.y));
  const float sh = __fmul_rn(rh, rh);
  const float sl = __fadd_rn(__fmaf_rn(rh, rh, -sh), __fmul_rn(__fmul_rn(2.0f, rh), rl));
  const float q3 = __fmul_rn(__fmul_rn(rh, sh),
                             __fadd_rn(1.0f / 3.0f, __fmul_rn(rh, __fadd_rn(-0.25f, __fmul_rn(rh, 0.2f)))));
  // e ln2 in three parts: a 16-bit head (e * head exact for |e| <= 8), the
  // middle as an exact product, the tail
  const float l2h = 0.693145751953125f, l2m = 0x1.7f7d1cp-20f, l2l = 5.49560397e-14f;
  const float fe = (float) e;
  const float A = __fmul_rn(fe, l2h);
  const float bh = __fmul_rn(fe, l2m), bl = __fmaf_rn(fe, l2m, -bh);
  float H = A, L = 0.0f, sm, bb;
  auto two_sum = [&](float x) {                              // H + x = sm + error, the error into L
    sm = __fadd_rn(H, x); bb = fsub(sm, H);
    L = __fadd_rn(L, __fadd_rn(fsub(H, fsub(sm, bb)), fsub(x, bb)));
    H = sm;
  };
  two_sum(t.z);
  two_sum(bh);
  two_sum(rh);
  two_sum(__fmul_rn(-0.5f, sh));
  L = __fadd_rn(L, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(t.w, bl), __fmul_rn(fe, l2l)), rl),
                                       __fmul_rn(-0.5f, sl)), q3));
  const float res = __fadd_rn(H, L);
  const float bv = fsub(res, H);
  const float tr = __fadd_rn(fsub(H, fsub(res, bv)), fsub(L, bv));   // H + L - res, exactly
  const uint32_t rb = __float_as_uint(res);
  const float ulp = __uint_as_float((rb & 0x7f800000u) - (23u << 23));
  ok = in_range && (rb & 0x7fffffffu) >= 0x01000000u &&
       !(fsub(__fmul_rn(0.5f, ulp), fabsf(tr)) < __fmul_rn(fabsf(res), 0x1p-42f));
  return res;
}

__device__ __forceinline__ float log_rowf(float m, const double2 *tab) {
  bool ok;
  const float r = log_ff(m, ok);
  return ok ? r : log_row(m, tab);
}

// One thread per listed sequence; threads take the list in database order
// (order[t]: longest first), so a warp's sequences have similar lengths. Rows
// go 16 at a time. The row logs of one batch are taken while the next batch's
// recurrence runs -- row b's log next to row b's step, in straight-line code,
// so its instructions fill the latency of the serial chain through the
// divisions -- and then summed in row order.
__global__ void __launch_bounds__(128)
bias_kernel(BiasDev B, DbDev db, const int64_t *__restrict__ slots, const int64_t *__restrict__ order, int64_t nids,
            float *__restrict__ out, int32_t *__restrict__ out_len) {
  __shared__ float s_eo[NRES][2];
  __shared__ double2 s_log[kLogTab];
  for (int i = threadIdx.x; i < NRES * 2; i += blockDim.x) (&s_eo[0][0])[i] = (&B.eo[0][0])[i];
  for (int i = threadIdx.x; i < kLogTab; i += blockDim.x) s_log[i] = B.logtab[i];
  __syncthreads();
  const int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nids) return;
  const int64_t j = order[t];
  const int64_t s = slots[j];
  const int L = db.len[s];
  out_len[j] = L;
  if (L <= 0) { out[j] = 0.0f; return; }
  const uint4 *sq = reinterpret_cast<const uint4 *>(db.codes + db.start[s]);   // 16-byte aligned, padded to 16
  const float p1 = __fdiv_rn((float) L, (float) (L + 1));
  const float t00 = p1, t01 = __fadd_rn(1.0f, -p1);
  float d0 = 0.0f, d1 = 0.0f, logsc = 0.0f;
  float mx[16];                                  // row maxima of the last batch, logs not yet taken
  {                                              // rows 0 .. 15: the first starts from pi
    const uint4 w = sq[0];
    const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      mx[b] = 1.0f;
      if (b >= L) continue;
      const int x = (words[b >> 2] >> (8 * (b & 3))) & 0xff;
      float n0, n1;
      if (b == 0) {
        n0 = __fmul_rn(s_eo[x][0], B.pi0);
        n1 = __fmul_rn(s_eo[x][1], B.pi1);
      } else {
        n0 = __fmul_rn(__fadd_rn(__fmul_rn(d0, t00), __fmul_rn(d1, B.t10)), s_eo[x][0]);
        n1 = __fmul_rn(__fadd_rn(__fmul_rn(d0, t01), __fmul_rn(d1, B.t11)), s_eo[x][1]);
      }
      float m = 0.0f;                            // ESL_MAX(dp, max) over k = 0, 1
      m = n0 > m ? n0 : m;
      m = n1 > m ? n1 : m;
      d0 = __fdiv_rn(n0, m);
      d1 = __fdiv_rn(n1, m);
      mx[b] = m;
    }
  }
  for (int i0 = 16; i0 < L; i0 += 16) {          // the previous batch (rows i0-16 .. i0-1) is full
    const uint4 w = sq[i0 >> 4];
    const uint32_t words[4] = {w.x, w.y, w.z, w.w};
    float lg[16], pm[16];
    uint32_t fail = 0;
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      bool ok;
      pm[b] = mx[b];
      lg[b] = log_ff(pm[b], ok);
      fail |= ok ? 0u : 1u << b;
      // rows past L are computed from residue 0 and dropped
      const bool live = i0 + b < L;
      const int x = live ? (int) ((words[b >> 2] >> (8 * (b & 3))) & 0xff) : 0;
      const float n0 = __fmul_rn(__fadd_rn(__fmul_rn(d0, t00), __fmul_rn(d1, B.t10)), s_eo[x][0]);
      const float n1 = __fmul_rn(__fadd_rn(__fmul_rn(d0, t01), __fmul_rn(d1, B.t11)), s_eo[x][1]);
      float m = 0.0f;
      m = n0 > m ? n0 : m;
      m = n1 > m ? n1 : m;
      const float q0 = __fdiv_rn(n0, m), q1 = __fdiv_rn(n1, m);
      d0 = live ? q0 : d0;
      d1 = live ? q1 : d1;
      mx[b] = live ? m : 1.0f;
    }
    if (fail) {
#pragma unroll
      for (int b = 0; b < 16; ++b)
        if (fail >> b & 1u) lg[b] = log_row(pm[b], s_log);
    }
#pragma unroll
    for (int b = 0; b < 16; ++b) logsc = __fadd_rn(logsc, lg[b]);
  }
  const int last = ((L - 1) >> 4) << 4;          // first row of the last batch
#pragma unroll
  for (int b = 0; b < 16; ++b)
    if (last + b < L) logsc = __fadd_rn(logsc, log_rowf(mx[b], s_log));
  const float end = __fadd_rn(d0, d1);           // dp[L][0] * 1 + dp[L][1] * 1
  out[j] = __fadd_rn(logsc, log_rowf(end, s_log));
}

// degenerate amino codes 21..26 (B J Z O U X) as sets of canonical codes
// (easel/esl_alphabet.c:282-292; X is every residue)
bool degen(int x, int y) {
  switch (x) {
    case 21: return y == 2 || y == 11;     // B: D N
    case 22: return y == 7 || y == 9;      // J: I L
    case 23: return y == 3 || y == 13;     // Z: E Q
    case 24: return y == 8;                // O: K
    case 25: return y == 1;                // U: C
    case 26: return true;                  // X
  }
  return false;
}

// esl_hmm_Configure (easel/esl_hmm.c:116-153) of the filter HMM with fq = bg->f
void filter_hmm(const float *compo, int M, BiasDev &B) {
  const float *bg = msvgb_detail::kAminoBg;
  const float *e[2] = {bg, compo};
  for (int x = 0; x < 20; ++x)
    for (int k = 0; k < 2; ++k) B.eo[x][k] = e[k][x] / bg[x];
  for (int k = 0; k < 2; ++k) B.eo[20][k] = B.eo[27][k] = B.eo[28][k] = 1.0f;
  for (int x = 21; x <= 26; ++x)
    for (int k = 0; k < 2; ++k) {
      float num = 0.0f, denom = 0.0f;
      for (int y = 0; y < 20; ++y)
        if (degen(x, y)) { num += e[k][y]; denom += bg[y]; }
      B.eo[x][k] = (denom > 0.0f) ? num / denom : 0.0f;
    }
  const float L1 = (float) ((double) M / 8.0);    // p7_bg_SetFilter: L1 = (float) M / 8.0
  B.t10 = 1.0f / (L1 + 1.0f);
  B.t11 = L1 / (L1 + 1.0f);
  B.pi0 = 0.999f;
  B.pi1 = 0.001f;
  for (int j = 0; j < kLogTab; ++j) {
    double c = 1.0 + (j + 0.5) / kLogTab;
    if (j >= 212) c *= 0.5;                         // f >= 1 + 212/512 is halved
    if (j == 0 || j == kLogTab - 1) c = 1.0;        // the intervals next to 1
    const double inv = 1.0 / c;
    B.logtab[j] = make_double2(inv, -std::log(inv));
  }
}

}  // namespace

// The float-pair table of log_ff, uploaded once per device.
static cudaError_t ensure_logff(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lk(mu);
  for (int d : done) if (d == device) return cudaSuccess;
  std::vector<float4> t(2048);
  for (int j = 0; j < 2048; ++j) {
    double c = 1.0 + (j + 0.5) / 2048.0;
    if (j >= 849) c *= 0.5;
    if (j == 0 || j == 2047) c = 1.0;
    const double inv = 1.0 / c, lg = std::log(c);
    const float ih = (float) inv, th = (float) lg;
    t[j] = make_float4(ih, (float) (inv - (double) ih), th, (float) (lg - (double) th));
  }
  const cudaError_t e = cudaMemcpyToSymbol(g_logff, t.data(), sizeof(float4) * 2048);
  if (e == cudaSuccess) done.push_back(device);
  return e;
}

extern "C" float msvgb_bias_length_term(float fwd, int L) {
  // p7_bg_FilterScore: nullsc + (float) L * logf(bg->p1) + logf(1. - bg->p1)
  const float p1 = (float) L / (float) (L + 1);
  return fwd + (float) L * logf(p1) + logf((float) (1. - (double) p1));
}

extern "C" int msvgb_stage_pass(float sc, float base, double mu, double lambda, double F, double *ret_P) {
  const float seq_score = (float) ((double) (sc - base) / 0.69314718055994529);
  const double y = lambda * ((double) seq_score - mu);
  const double ey = -exp(-y);
  const double P = (fabs(ey) < 5e-9) ? -ey : 1 - exp(ey);      // esl_gumbel_surv, easel/esl_gumbel.c:129-137
  if (ret_P) *ret_P = P;
  return (P > F) ? 0 : 1;
}

extern "C" float msvgb_null_score(int L) {
  const float p1 = (float) L / (float) (L + 1);                  // p7_bg_NullOne, src/p7_bg.c:359-363
  return (float) ((double) (float) L * ::log((double) p1) + ::log(1. - (double) p1));
}

extern "C" int msvgb_biasfilter(msvgb_ctx *c, const float *compo, int M, const msvgb_db *db, const int64_t *ids,
                                int64_t nids, float *out_sc) {
  if (!c || !compo || !db || M < 1 || nids < 0 || (nids && (!ids || !out_sc)))
    return fail(MSVGB_eslEINVAL, "msvgb_biasfilter: bad arguments");
  if (nids == 0) return MSVGB_eslOK;
  for (int64_t j = 0; j < nids; ++j)
    if (ids[j] < 0 || ids[j] >= db->n) return fail(MSVGB_eslEINVAL, "sequence index out of range");
  CUDA_TRY(cudaSetDevice(c->device));
  BiasDev B;
  filter_hmm(compo, M, B);
  CUDA_TRY(ensure_logff(c->device));
  CUDA_TRY(msvgb_detail::ensure_inverse(c, db));
  std::vector<int32_t> lens((size_t) nids);
  // one scratch block: list slots and order (int64), bucket counts, scores and lengths
  const size_t a8 = ((size_t) nids * 8 + 255) & ~(size_t) 255, a4 = ((size_t) nids * 4 + 255) & ~(size_t) 255;
  char *d_scr = nullptr;
  CUDA_TRY(cudaMallocAsync((void **) &d_scr, 2 * a8 + 4096 + 2 * a4, c->stream));
  int64_t *d_ids = (int64_t *) d_scr, *d_order = (int64_t *) (d_scr + a8);
  int32_t *d_cnt = (int32_t *) (d_scr + 2 * a8);
  float *d_out = (float *) (d_scr + 2 * a8 + 4096);
  int32_t *d_len = (int32_t *) (d_scr + 2 * a8 + 4096 + a4);
  cudaError_t e = cudaMemcpyAsync(d_ids, ids, nids * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = msvgb_detail::launch_gather_ids(d_ids, nids, db->d_inv, c->num_sms, c->stream);
  if (e == cudaSuccess)
    e = msvgb_detail::launch_order_by_length(d_ids, nids, db->d_len, db->Lmax, d_cnt, d_order, c->num_sms, c->stream);
  DbDev dbv{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  if (e == cudaSuccess) {
    (void) cudaGetLastError();
    bias_kernel<<<(unsigned) ((nids + 127) / 128), 128, 0, c->stream>>>(B, dbv, d_ids, d_order, nids, d_out, d_len);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) msvgb_detail::count_launch();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_sc, d_out, nids * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lens.data(), d_len, nids * 4, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d_scr, c->stream);
  const cudaError_t e2 = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("biasfilter: ") + cudaGetErrorString(e));
  for (int64_t j = 0; j < nids; ++j)
    out_sc[j] = lens[j] > 0 ? msvgb_bias_length_term(out_sc[j], lens[j]) : 0.0f;
  return MSVGB_eslOK;
}
