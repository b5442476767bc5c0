/* msv_oracle.h -- CPU oracle for the MSV filter (TEST INFRASTRUCTURE ONLY).
 *
 * A portable scalar C restatement of HMMER 3.1b1's p7_MSVFilter
 * (src/impl_sse/msvfilter.c:77-213), including the SSV fast path it calls
 * first (src/impl_sse/ssvfilter.c:1364-1413), and of the MSV stage of
 * p7_Pipeline (src/p7_pipeline.c:662-677). It is the checker for the CUDA
 * implementation: only tests, the smoke check and the CPU-baseline leg of the
 * benchmark may call it. The product library never links it.
 *
 * Parity pin: tests/golden/ holds outputs of the reference's own compiled
 * p7_MSVFilter (generated on x86-64 by oracle/ref/refgen.c); the oracle must
 * reproduce every status, score bit pattern and F1 pass flag there.
 */
#ifndef MSV_ORACLE_H
#define MSV_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Easel status codes (easel/easel.h:95-114) */
#define ORC_eslOK        0
#define ORC_eslEINVAL   11
#define ORC_eslERANGE   16
#define ORC_eslENORESULT 19

/* MSV part of a P7_OPROFILE (src/impl_sse/impl_sse.h:77-87). rbv is the
 * striped [Kp][Q][16] uint8 table: byte z of vector q holds node k=q+1+z*Q. */
typedef struct {
  int            M;
  int            Q;        /* p7O_NQB(M) = max(2, ceil(M/16)) */
  int            Kp;       /* 29 for amino */
  const uint8_t *rbv;
  uint8_t        tbm_b, tec_b, base_b, bias_b;
  float          scale_b;
  double         mmu, mlambda;  /* evparam[p7_MMU], evparam[p7_MLAMBDA] */
} orc_profile;

/* tjb_b for target length L (src/impl_sse/p7_oprofile.c:920-925, 511-519). */
uint8_t orc_tjb_b(float scale_b, int L);

/* One call of p7_MSVFilter on dsq[1..L] (dsq[0], dsq[L+1] ignored) with
 * om->tjb_b = tjb_b. Returns eslOK or eslERANGE; *ret_sc as the reference
 * writes it; *ret_xj the final uint8 xJ (255 on eslERANGE); *ret_path
 * 0 = decided by SSV, 1 = full MSV recurrence ran. */
int orc_msv_filter(const uint8_t *dsq, int L, const orc_profile *om, uint8_t tjb_b,
                   uint8_t *ret_xj, float *ret_sc, int *ret_path);

/* The plain MSV recurrence alone (msvfilter.c:112-212), without SSV. */
int orc_msv_full(const uint8_t *dsq, int L, const orc_profile *om, uint8_t tjb_b,
                 uint8_t *ret_xj, float *ret_sc);

/* Float score from xJ (msvfilter.c:205-210). */
float orc_score_from_xj(uint8_t xj, uint8_t tjb_b, uint8_t base_b, float scale_b);

/* MSV stage of p7_Pipeline for one sequence of length L with filter score usc:
 * nullsc (p7_bg.c:191-199, 359-363), seq_score, esl_gumbel_surv P-value
 * (easel/esl_gumbel.c:129-137) and the F1 gate (P <= F1 passes). */
int orc_f1_pass(float usc, int L, double mmu, double mlambda, double F1,
                float *ret_nullsc, double *ret_P);

/* Batch over a concatenated sequence set: residues[off[i]..off[i+1]) are the
 * codes of sequence i (no sentinels). Runs with nthreads host threads
 * (<=0: all online cores). Any output pointer may be NULL.
 * status[i] = -1 for an empty sequence (the pipeline skips them). */
int orc_msv_batch(const orc_profile *om, const uint8_t *residues, const int64_t *off,
                  int64_t n, double F1, int nthreads,
                  int32_t *status, uint8_t *xj, float *sc, uint8_t *pass, uint8_t *path);

/* Vectorized port of the reference's SSE2 algorithm (msv_port.c): the timed
 * CPU baseline. Same outputs as orc_msv_batch (path not reported). */
int port_msv_batch(const orc_profile *om, const uint8_t *residues, const int64_t *off, int64_t n,
                   double F1, int nthreads, int32_t *status, uint8_t *xj, float *sc, uint8_t *pass);

#ifdef __cplusplus
}
#endif
#endif
