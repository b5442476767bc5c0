// msv_sample.cu -- profile preparation: HMMER's random-profile sampling,
// configuration, MSV byte conversion and MSV calibration.
//
// Host code that restates, from the reference's algorithm, the chain that
// produces a P7_OPROFILE's MSV fields for a sampled model:
//   p7_hmm_Sample            src/p7_hmm.c:877-918 (Dirichlet-uniform draws)
//   esl_randomness_Create    easel/esl_random.c:84, 197-205, 298-359 (MT19937, Knuth-LCG seeded table)
//   esl_rnd_Gamma(1.0)       easel/esl_random.c:620-630, 657-668 (gamma_integer: -log of a uniform)
//   esl_dirichlet_FSampleUniform  easel/esl_dirichlet.c:964-971 (+ esl_vec_FNorm, esl_vectorops.c:842)
//   p7_ProfileConfig match scores src/modelconfig.c:165-176 (+ esl_abc_FExpectScVec, esl_alphabet.c:1399-1513)
//   mf_conversion            src/impl_sse/p7_oprofile.c:601-640 (byteify :495-519)
//   p7_Lambda                src/evalues.c:186-192 (+ p7_MeanMatchRelativeEntropy, src/modelstats.c:81-98)
//   p7_MSVMu                 src/evalues.c:240-283 with the calibration RNG
//                            esl_randomness_CreateFast(42) (evalues.c:80-81; Knuth LCG,
//                            jenkins_mix3 seeding, esl_random.c:130-146, 279-284, 384-396),
//                            esl_rsq_xfIID (easel/esl_randomseq.c:764) / esl_rnd_FChoose
//                            (easel/esl_random.c:718-738), esl_gumbel_FitCompleteLoc
//                            (easel/esl_gumbel.c:492-502); the MSV scores come from this
//                            library's own GPU search.
// Float/double evaluation order follows the C sources (this file is compiled
// with -ffp-contract=off), so on the same libm the bytes equal the reference's.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using msvgb_detail::fail;

// HMMER's amino background (src/hmmer.c:163-186), Easel code order A..Y.
const float msvgb_detail::kAminoBg[20] = {
    0.0787945f, 0.0151600f, 0.0535222f, 0.0668298f, 0.0397062f, 0.0695071f, 0.0229198f,
    0.0590092f, 0.0594422f, 0.0963728f, 0.0237718f, 0.0414386f, 0.0482904f, 0.0395639f,
    0.0540978f, 0.0683364f, 0.0540687f, 0.0673417f, 0.0114135f, 0.0304133f};

namespace {

constexpr int K = 20, KP = 29;
constexpr double kLog2 = 0.69314718055994529;   // eslCONST_LOG2
constexpr double kE = 2.71828182845904523536028747135;

const float *const kBg = msvgb_detail::kAminoBg;

// Mersenne twister MT19937 as Easel seeds it (a Knuth LCG fills the table).
struct Mersenne {
  uint32_t mt[624];
  int mti = 0;
  explicit Mersenne(uint32_t seed) {
    mt[0] = seed;
    for (int z = 1; z < 624; ++z) mt[z] = 69069u * mt[z - 1];
    fill();
  }
  void fill() {
    static const uint32_t mag01[2] = {0x0u, 0x9908b0dfu};
    uint32_t y;
    int z;
    for (z = 0; z < 227; ++z) {
      y = (mt[z] & 0x80000000u) | (mt[z + 1] & 0x7fffffffu);
      mt[z] = mt[z + 397] ^ (y >> 1) ^ mag01[y & 1u];
    }
    for (; z < 623; ++z) {
      y = (mt[z] & 0x80000000u) | (mt[z + 1] & 0x7fffffffu);
      mt[z] = mt[z - 227] ^ (y >> 1) ^ mag01[y & 1u];
    }
    y = (mt[623] & 0x80000000u) | (mt[0] & 0x7fffffffu);
    mt[623] = mt[396] ^ (y >> 1) ^ mag01[y & 1u];
    mti = 0;
  }
  uint32_t next() {
    if (mti >= 624) fill();
    uint32_t x = mt[mti++];
    x ^= (x >> 11);
    x ^= (x << 7) & 0x9d2c5680u;
    x ^= (x << 15) & 0xefc60000u;
    x ^= (x >> 18);
    return x;
  }
  double uniform() { return (double) next() / 4294967296.0; }
};

// Bob Jenkins' 96-bit mix, used by Easel to disperse a seed.
uint32_t jenkins_mix3(uint32_t a, uint32_t b, uint32_t c) {
  a -= b; a -= c; a ^= (c >> 13);
  b -= c; b -= a; b ^= (a << 8);
  c -= a; c -= b; c ^= (b >> 13);
  a -= b; a -= c; a ^= (c >> 12);
  b -= c; b -= a; b ^= (a << 16);
  c -= a; c -= b; c ^= (b >> 5);
  a -= b; a -= c; a ^= (c >> 3);
  b -= c; b -= a; b ^= (a << 10);
  c -= a; c -= b; c ^= (b >> 15);
  return c;
}

// Easel's "fast" generator: a 32-bit Knuth linear congruential generator.
struct KnuthLCG {
  uint32_t x;
  explicit KnuthLCG(uint32_t seed) { x = jenkins_mix3(seed, 87654321u, 12345678u); if (x == 0) x = 42; }
  double uniform() { x *= 69069u; x += 1u; return (double) x / 4294967296.0; }
};

double uniform_positive(Mersenne &r) { double x; do { x = r.uniform(); } while (x == 0.0); return x; }

// Dirichlet(1,...,1) draw of n floats: Gamma(1) = -log(U), normalised in float.
void dirichlet_uniform(Mersenne &r, int n, float *p) {
  for (int x = 0; x < n; ++x) p[x] = (float) (-::log(uniform_positive(r)));
  float sum = 0.f;
  for (int x = 0; x < n; ++x) sum += p[x];
  if (sum != 0.0) for (int x = 0; x < n; ++x) p[x] /= sum;
  else for (int x = 0; x < n; ++x) p[x] = 1. / (float) n;
}

// degenerate codes 21..26 (B J Z O U X) and their base residues (esl_alphabet.c:268-295, 150-166)
bool degen(int code, int i) {
  switch (code) {
    case 21: return i == 11 || i == 2;            // B: N, D
    case 22: return i == 7 || i == 9;             // J: I, L
    case 23: return i == 13 || i == 3;            // Z: Q, E
    case 24: return i == 8;                       // O: K
    case 25: return i == 1;                       // U: C
    case 26: return true;                         // X: any
    default: return false;
  }
}

uint8_t unbiased_byteify(float scale, float sc) {
  sc = -1.0f * roundf(scale * sc);
  return (sc > 255.) ? 255 : (uint8_t) sc;
}

// biased_byteify for a cost in [-bias, 255-bias] or +inf; the reference's
// "(uint8_t) sc + bias" is the same value taken modulo 256.
uint8_t biased_byteify(float scale, uint8_t bias, float sc) {
  sc = -1.0f * roundf(scale * sc);
  return (sc > 255 - bias) ? 255 : (uint8_t) ((int) sc + (int) bias);
}

}  // namespace

extern "C" int msvgb_sample_om(uint32_t seed, int M, uint8_t *rbv, msvgb_om *om, double *ret_lambda) {
  if (!rbv || !om || M < 1 || seed == 0) return fail(MSVGB_eslEINVAL, "msvgb_sample_om: bad arguments");
  Mersenne r(seed);
  // p7_hmm_Sample: node 0..M draws in the reference's order
  std::vector<float> mat((size_t) (M + 1) * K, 0.f);
  float scratch[K];
  for (int k = 0; k <= M; ++k) {
    if (k > 0) dirichlet_uniform(r, K, &mat[(size_t) k * K]);
    dirichlet_uniform(r, K, scratch);      // insert emissions
    dirichlet_uniform(r, 3, scratch);      // M->M, M->I, M->D
    dirichlet_uniform(r, 2, scratch);      // I->M, I->I
    if (k > 0) dirichlet_uniform(r, 2, scratch);   // D->M, D->D
  }
  dirichlet_uniform(r, 2, scratch);        // node M: M->M, M->I only

  // p7_ProfileConfig match scores, then mf_conversion
  const int Qn = std::max(2, (M - 1) / 16 + 1);   // p7O_NQB(M)
  std::vector<float> msc((size_t) (M + 1) * KP);
  float max = 0.0f;
  for (int k = 1; k <= M; ++k) {
    float sc[KP];
    sc[K] = -INFINITY; sc[KP - 2] = -INFINITY; sc[KP - 1] = -INFINITY;
    // C's log() of a float argument computes in double (not C++'s float overload)
    for (int x = 0; x < K; ++x) sc[x] = (float) ::log((double) (mat[(size_t) k * K + x] / kBg[x]));
    for (int x = K + 1; x <= KP - 3; ++x) {           // esl_abc_FExpectScVec
      float result = 0.f, denom = 0.f;
      for (int i = 0; i < K; ++i)
        if (degen(x, i)) { result += sc[i] * kBg[i]; denom += kBg[i]; }
      result /= denom;
      sc[x] = result;
    }
    for (int x = 0; x < KP; ++x) msc[(size_t) k * KP + x] = sc[x];
    for (int x = 0; x < K; ++x) max = std::max(max, sc[x]);
  }
  const float scale = 3.0 / kLog2;
  const uint8_t bias = unbiased_byteify(scale, -1.0 * max);
  for (int x = 0; x < KP; ++x)
    for (int q = 0; q < Qn; ++q)
      for (int z = 0; z < 16; ++z) {
        const int k = q + 1 + z * Qn;
        rbv[((size_t) x * Qn + q) * 16 + z] = (k <= M) ? biased_byteify(scale, bias, msc[(size_t) k * KP + x]) : 255;
      }
  om->M = M; om->Kp = KP; om->rbv = rbv;
  om->scale_b = scale; om->base_b = 190; om->bias_b = bias;
  om->tbm_b = unbiased_byteify(scale, logf(2.0f / ((float) M * (float) (M + 1))));
  om->tec_b = unbiased_byteify(scale, logf(0.5f));
  om->tjb_b = unbiased_byteify(scale, logf(3.0f / (float) (350 + 3)));

  // p7_Lambda: lambda = log 2 + 1.44 / (M * mean match relative entropy)
  double KL = 0.;
  for (int k = 1; k <= M; ++k) {
    float kl = 0.;
    const float *p = &mat[(size_t) k * K];
    for (int i = 0; i < K; ++i)
      if (p[i] > 0.) kl += p[i] * ::log((double) (p[i] / kBg[i]));
    KL += (float) (1.44269504 * kl);
  }
  KL /= (double) M;
  const double lambda = kLog2 + 1.44 / ((double) M * KL);
  om->mlambda = (float) lambda;
  om->mmu = 0.0f;
  if (ret_lambda) *ret_lambda = lambda;
  return MSVGB_eslOK;
}

extern "C" int msvgb_calibrate(msvgb_ctx *ctx, msvgb_om *om, double lambda) {
  if (!ctx || !om) return fail(MSVGB_eslEINVAL, "msvgb_calibrate: NULL argument");
  const int L = 200, N = 200;                       // EmL, EmN defaults (evalues.c:70-71)
  KnuthLCG r(42);
  std::vector<uint8_t> codes((size_t) L * N);
  std::vector<int64_t> off(N + 1);
  for (int i = 0; i < N; ++i) {
    off[i] = (int64_t) i * L;
    for (int j = 0; j < L; ++j) {                   // esl_rsq_xfIID / esl_rnd_FChoose
      double norm = 0.0, sum = 0.0, roll = r.uniform();
      for (int x = 0; x < K; ++x) norm += kBg[x];
      int pick = K - 1;
      for (int x = 0; x < K; ++x) { sum += kBg[x]; if (roll < (sum / norm)) { pick = x; break; } }
      codes[(size_t) i * L + j] = (uint8_t) pick;
    }
  }
  off[N] = (int64_t) N * L;
  msvgb_profile *prof = nullptr;
  msvgb_db *db = nullptr;
  int st = msvgb_profile_create(ctx, om, &prof);
  if (st == MSVGB_eslOK) st = msvgb_db_create(ctx, codes.data(), off.data(), N, &db);
  std::vector<uint8_t> xj(N), fl(N);
  if (st == MSVGB_eslOK) st = msvgb_search(ctx, prof, db, 0.02, xj.data(), fl.data());
  msvgb_db_destroy(db);
  msvgb_profile_destroy(prof);
  if (st != MSVGB_eslOK) return st;
  // p7_MSVMu: scores in bits over the null model, ERANGE scored as maxsc
  const float maxsc = (255 - om->base_b) / om->scale_b;
  const float p1 = (float) L / (float) (L + 1);
  const float nullsc = (float) ((double) (float) L * ::log((double) p1) + ::log(1. - (double) p1));
  double esum = 0.;
  for (int i = 0; i < N; ++i) {
    float sc = msvgb_score(xj[i], fl[i], L, om->base_b, om->scale_b);
    if (fl[i] & MSVGB_FLAG_ERANGE) sc = maxsc;
    const double xv = (sc - nullsc) / kLog2;
    esum += ::exp(-lambda * xv);                    // esl_gumbel_FitCompleteLoc
  }
  const double mu = -::log(esum / N) / lambda;
  om->mmu = (float) mu;
  om->mlambda = (float) lambda;
  return MSVGB_eslOK;
}
