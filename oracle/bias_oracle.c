/* bias_oracle.c -- CPU oracle for the bias filter and the filter-stage gates
 * of p7_Pipeline (TEST INFRASTRUCTURE ONLY).
 *
 * A scalar C restatement of HMMER 3.1b1's composition-bias filter: the
 * two-state filter HMM of p7_bg_SetFilter (src/p7_bg.c:431-453) with the
 * length of p7_bg_SetLength (:191-199), its emission odds from
 * esl_hmm_Configure (easel/esl_hmm.c:116-153), the scaled Forward of
 * esl_hmm_Forward (easel/esl_hmm.c:351-409) and the length term of
 * p7_bg_FilterScore (src/p7_bg.c:473-483); and of the gates that p7_Pipeline
 * puts around the bias filter and p7_ViterbiFilter (src/p7_pipeline.c:666-705).
 * It is the checker for the CUDA bias filter and for the pipeline's GPU
 * filter stages; the product library never links it.
 *
 * Parity pin: tests/golden/pipe_*.pres hold p7_bg_FilterScore's score for
 * every sequence and the stage each sequence reached in the reference's own
 * p7_Pipeline code (oracle/ref/refgen.c "pipe"/"pipefile"); the oracle
 * reproduces every one (tests/test_bias_oracle.py).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "bias_oracle.h"

/* p7_AminoFrequencies (src/hmmer.c:163-186), A..Y in Easel code order */
static const float kBg[20] = {
  0.0787945f, 0.0151600f, 0.0535222f, 0.0668298f, 0.0397062f, 0.0695071f, 0.0229198f,
  0.0590092f, 0.0594422f, 0.0963728f, 0.0237718f, 0.0414386f, 0.0482904f, 0.0395639f,
  0.0540978f, 0.0683364f, 0.0540687f, 0.0673417f, 0.0114135f, 0.0304133f };

/* degenerate amino codes 21..26 (B J Z O U X) as sets of canonical codes
 * (easel/esl_alphabet.c:282-292; X is every residue) */
static int degen(int x, int y) {
  switch (x) {
    case 21: return y == 2 || y == 11;     /* B: D N */
    case 22: return y == 7 || y == 9;      /* J: I L */
    case 23: return y == 3 || y == 13;     /* Z: E Q */
    case 24: return y == 8;                /* O: K */
    case 25: return y == 1;                /* U: C */
    case 26: return 1;                     /* X */
  }
  return 0;
}

/* eo[x][k], k = 0 background, 1 model composition (esl_hmm_Configure with fq = bg->f) */
static void emission_odds(const float compo[20], float eo[29][2]) {
  const float *e[2] = { kBg, compo };
  for (int x = 0; x < 20; x++)
    for (int k = 0; k < 2; k++) eo[x][k] = e[k][x] / kBg[x];
  for (int k = 0; k < 2; k++) eo[20][k] = eo[27][k] = eo[28][k] = 1.0f;   /* gap, nonresidue, missing */
  for (int x = 21; x <= 26; x++)
    for (int k = 0; k < 2; k++) {
      float num = 0.0f, denom = 0.0f;
      for (int y = 0; y < 20; y++)
        if (degen(x, y)) { num += e[k][y]; denom += kBg[y]; }
      eo[x][k] = (denom > 0.0f) ? num / denom : 0.0f;
    }
}

float orc_bias_filter(const float compo[20], int M, const uint8_t *dsq, int L) {
  float eo[29][2];
  emission_odds(compo, eo);
  const float L1 = (float) M / 8.0;
  const float p1 = (float) L / (float) (L + 1);
  float t[2][3];
  t[0][0] = p1;                   t[0][1] = 1.0f - p1;          t[0][2] = 1.0f;
  t[1][0] = 1.0f / (L1 + 1.0f);   t[1][1] = L1 / (L1 + 1.0f);   t[1][2] = 1.0f;
  const float pi[2] = { 0.999f, 0.001f };
  /* esl_hmm_Forward, two rows */
  float dp[2], nx[2], mx, logsc = 0.0f, sc;
  mx = 0.0f;
  for (int k = 0; k < 2; k++) { dp[k] = eo[dsq[1]][k] * pi[k]; mx = dp[k] > mx ? dp[k] : mx; }
  for (int k = 0; k < 2; k++) dp[k] /= mx;
  sc = log(mx);
  logsc += sc;
  for (int i = 2; i <= L; i++) {
    mx = 0.0f;
    for (int k = 0; k < 2; k++) {
      nx[k] = 0.0f;
      for (int m = 0; m < 2; m++) nx[k] += dp[m] * t[m][k];
      nx[k] *= eo[dsq[i]][k];
      mx = nx[k] > mx ? nx[k] : mx;
    }
    for (int k = 0; k < 2; k++) dp[k] = nx[k] / mx;
    sc = log(mx);
    logsc += sc;
  }
  sc = 0.0f;
  for (int m = 0; m < 2; m++) sc += dp[m] * t[m][2];
  sc = log(sc);
  logsc += sc;
  return logsc + (float) L * logf(p1) + logf(1. - p1);
}

double orc_gumbel_P(float sc, float base, double mu, double lambda) {
  const float seq_score = (sc - base) / 0.69314718055994529;
  const double y = lambda * ((double) seq_score - mu);
  const double ey = -exp(-y);
  return (fabs(ey) < 5e-9) ? -ey : 1 - exp(ey);
}

void orc_pipe_stages(const uint8_t *dsq, int L, float usc, const float compo[20], int do_bias,
                     const orc_vprofile *vp, double mmu, double mlambda, double vmu, double vlambda,
                     double F1, double F2, orc_pipe_result *r) {
  r->usc = usc;
  r->vfsc = NAN;
  r->nullsc = r->filtersc = 0.0f;
  if (L == 0) { r->stage = ORC_STAGE_EMPTY; return; }
  const float p1 = (float) L / (float) (L + 1);
  r->nullsc = (float) L * log(p1) + log(1. - p1);            /* p7_bg_NullOne, src/p7_bg.c:359-363 */
  double P = orc_gumbel_P(usc, r->nullsc, mmu, mlambda);
  if (P > F1) { r->stage = ORC_STAGE_MSV; return; }
  if (do_bias) {
    r->filtersc = orc_bias_filter(compo, vp->M, dsq, L);
    P = orc_gumbel_P(usc, r->filtersc, mmu, mlambda);
    if (P > F1) { r->stage = ORC_STAGE_BIAS; return; }
  } else {
    r->filtersc = r->nullsc;
  }
  if (P > F2) {
    float vfsc;
    orc_vit_filter(dsq, L, vp, &vfsc, NULL);
    r->vfsc = vfsc;
    P = orc_gumbel_P(vfsc, r->filtersc, vmu, vlambda);
    if (P > F2) { r->stage = ORC_STAGE_VIT; return; }
  }
  r->stage = ORC_STAGE_PASSED;
}
