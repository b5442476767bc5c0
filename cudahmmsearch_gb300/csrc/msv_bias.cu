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
// contraction into FMA), and each row's log taken in double and stored to
// float as the reference's double log() of a float is. The length term
// (logf of p1 and 1 - p1) is added on the host with the C library's logf.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using namespace msvgb;
using msvgb_detail::fail;

namespace {

struct BiasDev {
  float eo[NRES][2];       // emission odds: [x][0] background state, [x][1] model-composition state
  float t10, t11;          // biased-state transitions 1->0, 1->1 (t[1][2] = 1)
  float pi0, pi1;
};

__global__ void __launch_bounds__(128)
bias_kernel(BiasDev B, DbDev db, const int64_t *__restrict__ slots, int64_t nids, float *__restrict__ out,
            int32_t *__restrict__ out_len) {
  __shared__ float s_eo[NRES][2];
  for (int i = threadIdx.x; i < NRES * 2; i += blockDim.x) (&s_eo[0][0])[i] = (&B.eo[0][0])[i];
  __syncthreads();
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nids) return;
  const int64_t s = slots[j];
  const int L = db.len[s];
  out_len[j] = L;
  if (L <= 0) { out[j] = 0.0f; return; }
  const uint4 *sq = reinterpret_cast<const uint4 *>(db.codes + db.start[s]);   // 16-byte aligned, padded to 16
  const float p1 = __fdiv_rn((float) L, (float) (L + 1));
  const float t00 = p1, t01 = __fadd_rn(1.0f, -p1);
  float d0 = 0.0f, d1 = 0.0f, logsc = 0.0f;
  for (int i0 = 0; i0 < L; i0 += 16) {
    const uint4 w = sq[i0 >> 4];
    const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int b = 0; b < 16; ++b) {
      const int i = i0 + b;
      if (i >= L) break;
      const int x = (words[b >> 2] >> (8 * (b & 3))) & 0xff;
      float n0, n1;
      if (i == 0) {
        n0 = __fmul_rn(s_eo[x][0], B.pi0);
        n1 = __fmul_rn(s_eo[x][1], B.pi1);
      } else {
        n0 = __fmul_rn(__fadd_rn(__fmul_rn(d0, t00), __fmul_rn(d1, B.t10)), s_eo[x][0]);
        n1 = __fmul_rn(__fadd_rn(__fmul_rn(d0, t01), __fmul_rn(d1, B.t11)), s_eo[x][1]);
      }
      float mx = 0.0f;                           // ESL_MAX(dp, max) over k = 0, 1
      mx = n0 > mx ? n0 : mx;
      mx = n1 > mx ? n1 : mx;
      d0 = __fdiv_rn(n0, mx);
      d1 = __fdiv_rn(n1, mx);
      logsc = __fadd_rn(logsc, (float) log((double) mx));
    }
  }
  const float end = __fadd_rn(d0, d1);           // dp[L][0] * 1 + dp[L][1] * 1
  out[j] = __fadd_rn(logsc, (float) log((double) end));
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
}

}  // namespace

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
  CUDA_TRY(msvgb_detail::ensure_inverse(c, db));
  int64_t *d_ids = nullptr;
  float *d_out = nullptr;
  int32_t *d_len = nullptr;
  std::vector<int32_t> lens((size_t) nids);
  CUDA_TRY(cudaMallocAsync((void **) &d_ids, nids * 8, c->stream));
  CUDA_TRY(cudaMallocAsync((void **) &d_out, nids * 4, c->stream));
  CUDA_TRY(cudaMallocAsync((void **) &d_len, nids * 4, c->stream));
  cudaError_t e = cudaMemcpyAsync(d_ids, ids, nids * 8, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = msvgb_detail::launch_gather_ids(d_ids, nids, db->d_inv, c->num_sms, c->stream);
  DbDev dbv{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  if (e == cudaSuccess) {
    (void) cudaGetLastError();
    bias_kernel<<<(unsigned) ((nids + 127) / 128), 128, 0, c->stream>>>(B, dbv, d_ids, nids, d_out, d_len);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) msvgb_detail::count_launch();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out_sc, d_out, nids * 4, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lens.data(), d_len, nids * 4, cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(d_ids, c->stream);
  cudaFreeAsync(d_out, c->stream);
  cudaFreeAsync(d_len, c->stream);
  const cudaError_t e2 = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("biasfilter: ") + cudaGetErrorString(e));
  for (int64_t j = 0; j < nids; ++j)
    out_sc[j] = lens[j] > 0 ? msvgb_bias_length_term(out_sc[j], lens[j]) : 0.0f;
  return MSVGB_eslOK;
}
