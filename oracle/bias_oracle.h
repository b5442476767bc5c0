/* bias_oracle.h -- CPU oracle for the bias filter and the filter-stage gates
 * of p7_Pipeline (TEST INFRASTRUCTURE ONLY). See bias_oracle.c. */
#ifndef BIAS_ORACLE_H
#define BIAS_ORACLE_H
#include <stdint.h>

#include "vit_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* p7_bg_FilterScore (src/p7_bg.c:473-483) of dsq[1..L] with the filter HMM of
 * p7_bg_SetFilter(bg, M, compo) (src/p7_bg.c:431-453) and p7_bg_SetLength(bg, L). */
float orc_bias_filter(const float compo[20], int M, const uint8_t *dsq, int L);

/* esl_gumbel_surv((sc - base) / log(2), mu, lambda) with the pipeline's float
 * seq_score (src/p7_pipeline.c:673-674); returns P. */
double orc_gumbel_P(float sc, float base, double mu, double lambda);

/* Stage results of p7_Pipeline's filters (src/p7_pipeline.c:662-705). */
enum { ORC_STAGE_MSV = 0, ORC_STAGE_BIAS = 1, ORC_STAGE_VIT = 2, ORC_STAGE_PASSED = 3, ORC_STAGE_EMPTY = 255 };

typedef struct {
  float  usc, nullsc, filtersc, vfsc;   /* vfsc NaN where Viterbi did not run */
  int    stage;
} orc_pipe_result;

/* Given the MSV score usc of dsq[1..L] (p7_MSVFilter), runs the bias filter
 * (unless do_bias is 0: --nobias) and the ViterbiFilter with the reference's
 * gates: F1 on the MSV and bias scores (mmu, mlambda), Viterbi only when the
 * bias-stage P > F2, and F2 on the Viterbi score (vmu, vlambda). */
void orc_pipe_stages(const uint8_t *dsq, int L, float usc, const float compo[20], int do_bias,
                     const orc_vprofile *vp, double mmu, double mlambda, double vmu, double vlambda,
                     double F1, double F2, orc_pipe_result *r);

#ifdef __cplusplus
}
#endif
#endif
