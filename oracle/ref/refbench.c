/* refbench: times the reference CPU p7_MSVFilter (impl_sse/msvfilter.c:78,
 * SSV first, full MSV on ENORESULT) over a sequence file with all host
 * threads, the way hmmsearch's worker threads call it (src/hmmsearch.c:1372-1406):
 * one p7_oprofile_Clone (impl_sse/p7_oprofile.c:398) and one private P7_OMX
 * per thread, p7_oprofile_ReconfigLength before every call.
 *
 * With stage "vit" it times p7_ViterbiFilter (impl_sse/vitfilter.c:84) the
 * same way; with stage "bias", p7_bg_FilterScore (src/p7_bg.c:473) with a
 * private P7_BG per thread (p7_bg_SetFilter with the model's composition, as
 * p7_pli_NewModel does, src/p7_pipeline.c:480; p7_bg_SetLength per sequence).
 * The sampled HMM gets the composition hmmbuild would give it.
 *
 * Test infrastructure (x86-64 only; the reference's filters are SSE2 code).
 *   refbench M seed Lcfg mode seqs nthreads reps [msv|vit|bias]
 * prints one line: "cells=<M*sum L*reps> seconds=<wall> gcups=<...> threads=<n>"
 */
#include "p7_config.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <time.h>
#include <pthread.h>

#include "easel.h"
#include "esl_alphabet.h"
#include "esl_random.h"
#include "hmmer.h"

static void die(const char *m) { fprintf(stderr, "refbench: %s\n", m); exit(1); }

typedef struct {
  const P7_OPROFILE *om0; const int64_t *off; const uint8_t *res;
  int64_t lo, hi; int reps; double sink; int stage;   /* 0 msv, 1 vit, 2 bias */
} job_t;

static void *worker(void *arg)
{
  job_t *j = (job_t *) arg;
  P7_OPROFILE *om = p7_oprofile_Clone(j->om0);
  P7_OMX *ox = p7_omx_Create(om->M, 0, 0);
  P7_BG *bg = p7_bg_Create(om->abc);
  p7_bg_SetFilter(bg, om->M, om->compo);
  int64_t maxL = 1;
  for (int64_t i = j->lo; i < j->hi; i++) if (j->off[i+1] - j->off[i] > maxL) maxL = j->off[i+1] - j->off[i];
  ESL_DSQ *dsq = malloc(maxL + 2);
  double acc = 0.0;
  for (int r = 0; r < j->reps; r++)
    for (int64_t i = j->lo; i < j->hi; i++) {
      int L = (int) (j->off[i+1] - j->off[i]); float sc;
      if (L == 0) continue;
      dsq[0] = eslDSQ_SENTINEL; memcpy(dsq + 1, j->res + j->off[i], L); dsq[L+1] = eslDSQ_SENTINEL;
      if (j->stage == 2) {
        p7_bg_SetLength(bg, L);
        p7_bg_FilterScore(bg, dsq, L, &sc);
      } else {
        p7_oprofile_ReconfigLength(om, L);
        if (j->stage == 1) p7_ViterbiFilter(dsq, L, om, ox, &sc);
        else p7_MSVFilter(dsq, L, om, ox, &sc);
      }
      acc += sc;
    }
  j->sink = acc;
  free(dsq); p7_omx_Destroy(ox); p7_oprofile_Destroy(om); p7_bg_Destroy(bg);
  return NULL;
}

int main(int argc, char **argv)
{
  if (argc != 8 && argc != 9) die("usage: refbench M seed Lcfg mode seqs nthreads reps [msv|vit|bias]");
  const int stage = argc == 9 ? (!strcmp(argv[8], "vit") ? 1 : !strcmp(argv[8], "bias") ? 2 : 0) : 0;
  int M = atoi(argv[1]), Lcfg = atoi(argv[3]), mode = atoi(argv[4]);
  int nth = atoi(argv[6]), reps = atoi(argv[7]);
  ESL_RANDOMNESS *r = esl_randomness_Create((uint32_t) atol(argv[2]));
  ESL_ALPHABET *abc = esl_alphabet_Create(eslAMINO);
  P7_BG *bg = p7_bg_Create(abc); P7_HMM *hmm = NULL;
  if (p7_hmm_Sample(r, M, abc, &hmm) != eslOK) die("sample");
  if (p7_Calibrate(hmm, NULL, NULL, &bg, NULL, NULL) != eslOK) die("calibrate");
  if (p7_hmm_SetComposition(hmm) != eslOK) die("composition");
  P7_PROFILE *gm = p7_profile_Create(M, abc);
  p7_ProfileConfig(hmm, bg, gm, Lcfg, mode);
  P7_OPROFILE *om = p7_oprofile_Create(M, abc);
  p7_oprofile_Convert(gm, om);

  FILE *fp = fopen(argv[5], "rb"); char mag[8]; int64_t n, total;
  if (!fp || fread(mag, 1, 8, fp) != 8 || memcmp(mag, "MSVSEQS1", 8)) die("seqs");
  if (fread(&n, 8, 1, fp) != 1 || fread(&total, 8, 1, fp) != 1) die("seqs hdr");
  int64_t *off = malloc(8 * (n + 1)); uint8_t *res = malloc(total + 1);
  if (fread(off, 8, n + 1, fp) != (size_t)(n + 1) || fread(res, 1, total, fp) != (size_t) total) die("seqs body");
  fclose(fp);

  /* static, residue-balanced partition of the sequence range */
  job_t *jobs = calloc(nth, sizeof(job_t)); pthread_t *th = calloc(nth, sizeof(pthread_t));
  int64_t s = 0;
  for (int t = 0; t < nth; t++) {
    int64_t target = (total * (t + 1)) / nth, e = s;
    while (e < n && off[e] < target) e++;
    if (t == nth - 1) e = n;
    jobs[t] = (job_t){ om, off, res, s, e, reps, 0.0, stage };
    s = e;
  }
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < nth; t++) pthread_create(&th[t], NULL, worker, &jobs[t]);
  for (int t = 0; t < nth; t++) pthread_join(th[t], NULL);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  double sec = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
  double cells = (double) M * (double) total * reps;
  printf("cells=%.0f seconds=%.6f gcups=%.4f threads=%d\n", cells, sec, cells / sec * 1e-9, nth);
  return 0;
}
