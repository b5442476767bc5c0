/* refgen: golden-vector generator built on the reference HMMER 3.1b1 sources.
 *
 * Test infrastructure only. Links the reference's own libraries (compiled by
 * oracle/ref/Makefile into oracle/_ref/) and runs its real code:
 *   profile  : p7_hmm_Sample -> p7_Calibrate -> p7_ProfileConfig -> p7_oprofile_Convert
 *              (hmmer src/p7_hmm.c:877, src/evalues.c:60, src/modelconfig.c:49,
 *               src/impl_sse/p7_oprofile.c:839) and dumps the MSV part of the
 *              P7_OPROFILE (impl_sse.h:77-87) plus evparam[MMU, MLAMBDA].
 *   emit     : p7_ProfileEmit (src/emit.c:186) homologs of that profile, and
 *              "saturation" sequences (an emitted core repeated R times).
 *   randseq  : esl_rsq_xfIID (easel/esl_randomseq.c:764) i.i.d. background residues.
 *   score    : per sequence, exactly the MSV stage of p7_Pipeline
 *              (src/p7_pipeline.c:662-677, with the per-sequence length
 *              reconfiguration of src/hmmsearch.c:1402-1404):
 *              p7_bg_SetLength, p7_oprofile_ReconfigLength, p7_bg_NullOne,
 *              p7_MSVFilter (impl_sse/msvfilter.c:78), esl_gumbel_surv, F1 gate.
 *
 *   hmmfile  : the hmmsearch path for a model read from an HMM file
 *              (p7_hmmfile_OpenE / p7_hmmfile_Read, src/p7_hmmfile.c:127, 1181;
 *              p7_ProfileConfig(hmm, bg, gm, 100, p7_LOCAL) + p7_oprofile_Convert
 *              as src/hmmsearch.c:502-503 does), or the pressed MSV part read back
 *              with p7_oprofile_ReadMSV (src/impl_sse/io.c:233).
 *   seqfile  : any sequence file Easel reads (esl_sqfile_OpenDigital, format
 *              autodetected, easel/esl_sqio.c:300), digitized with the amino alphabet.
 *
 *   pipe     : the filter stages of p7_Pipeline (src/p7_pipeline.c:646-705) per sequence,
 *              after p7_pli_NewModel's p7_bg_SetFilter (src/p7_pipeline.c:480) and
 *              p7_pli_NewSeq's p7_bg_SetLength: NullOne, MSVFilter and the F1 gate,
 *              p7_bg_FilterScore (src/p7_bg.c:473) and the F1 gate on it, then
 *              p7_ViterbiFilter when P > F2 and the F2 gate. Also the bias-filter
 *              score of every sequence, gated or not. Optionally the MSV
 *              profile (MSVPROF1) of the model as configured there.
 *   vit      : the ViterbiFilter stage (src/impl_sse/vitfilter.c:84-250) on the same
 *              configured model: its int16 profile part (vf_conversion,
 *              src/impl_sse/p7_oprofile.c:653-760) dumped, and per sequence
 *              p7_oprofile_ReconfigLength + p7_ViterbiFilter status and score.
 *
 * File formats (little-endian, written and read by this project only):
 *   profile "MSVPROF1": int32 M, Q, Kp, Lcfg; uint8 tbm,tec,tjb,base,bias,pad[3];
 *                       float scale; double mmu, mlambda; uint8 rbv[Kp*Q*16]
 *   seqs    "MSVSEQS1": int64 n, total; int64 off[n+1]; uint8 dsq[total]   (codes, no sentinels)
 *   result  "MSVRES01": int64 n; int32 status[n]; float sc[n]; double nullsc[n];
 *                       double P[n]; uint8 pass[n]
 *   vprof   "VITPROF1": int32 M, Q8, Kp; float scale_w, nj; int16 base_w, ddbound_w;
 *                       int16 xw[4][2] (E,N,J,C x MOVE,LOOP, as configured);
 *                       float vmu, vlambda; int16 twv[8*Q8][8]; int16 rwv[Kp][Q8][8]
 *   vres    "VITRES01": int64 n; int32 status[n]; float sc[n]
 *   pres    "PIPERES1": int32 M; float compo[20]; float mmu, mlambda, vmu, vlambda;
 *                       double F1, F2; int64 n; float nullsc[n], usc[n], fsc[n] (bias
 *                       filter score, every sequence), vfsc[n] (NaN where not run);
 *                       uint8 stage[n] (0 rejected by MSV, 1 by the bias filter,
 *                       2 by Viterbi, 3 passed Viterbi, 255 empty)
 */
#include "p7_config.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdint.h>

#include "easel.h"
#include "esl_alphabet.h"
#include "esl_random.h"
#include "esl_randomseq.h"
#include "esl_sq.h"
#include "esl_sqio.h"
#include "esl_gumbel.h"
#include "hmmer.h"

static void die(const char *m) { fprintf(stderr, "refgen: %s\n", m); exit(1); }

typedef struct {
  ESL_ALPHABET *abc; P7_BG *bg; P7_HMM *hmm; P7_PROFILE *gm; P7_OPROFILE *om;
} model_t;

/* Sample, calibrate, configure and convert a model exactly as hmmbuild-style
 * code paths do; calibration uses its default internal RNG (seed 42). */
static void make_model(model_t *m, int M, uint32_t seed, int Lcfg, int mode)
{
  ESL_RANDOMNESS *r = esl_randomness_Create(seed);
  m->abc = esl_alphabet_Create(eslAMINO);
  m->bg  = p7_bg_Create(m->abc);
  if (p7_hmm_Sample(r, M, m->abc, &m->hmm) != eslOK) die("p7_hmm_Sample");
  if (p7_Calibrate(m->hmm, NULL, NULL, &m->bg, NULL, NULL) != eslOK) die("p7_Calibrate");
  m->gm = p7_profile_Create(M, m->abc);
  if (p7_ProfileConfig(m->hmm, m->bg, m->gm, Lcfg, mode) != eslOK) die("p7_ProfileConfig");
  m->om = p7_oprofile_Create(M, m->abc);
  if (p7_oprofile_Convert(m->gm, m->om) != eslOK) die("p7_oprofile_Convert");
  esl_randomness_Destroy(r);
}

static void write_profile(const model_t *m, int Lcfg, const char *path)
{
  FILE *fp = fopen(path, "wb"); if (!fp) die("open profile out");
  int32_t hdr[4]; int Q = p7O_NQB(m->om->M);
  hdr[0] = m->om->M; hdr[1] = Q; hdr[2] = m->abc->Kp; hdr[3] = Lcfg;
  uint8_t b[8] = { m->om->tbm_b, m->om->tec_b, m->om->tjb_b, m->om->base_b, m->om->bias_b, 0, 0, 0 };
  float scale = m->om->scale_b;
  double ev[2] = { m->om->evparam[p7_MMU], m->om->evparam[p7_MLAMBDA] };
  fwrite("MSVPROF1", 1, 8, fp);
  fwrite(hdr, 4, 4, fp); fwrite(b, 1, 8, fp); fwrite(&scale, 4, 1, fp); fwrite(ev, 8, 2, fp);
  for (int x = 0; x < m->abc->Kp; x++) fwrite(m->om->rbv[x], 16, Q, fp);
  fclose(fp);
}

/* The idx-th model of an HMM file, configured and converted as hmmsearch
 * does; with pressed=1 the MSV part is instead read from the .h3f file. */
static void file_model(model_t *m, const char *hmmfile, int idx, int pressed)
{
  char errbuf[eslERRBUFSIZE];
  P7_HMMFILE *hfp = NULL;
  m->abc = NULL; m->hmm = NULL; m->gm = NULL; m->om = NULL;
  if (p7_hmmfile_OpenE((char *) hmmfile, NULL, &hfp, errbuf) != eslOK) die(errbuf);
  if (pressed) {
    for (int i = 0; i <= idx; i++) {
      if (m->om) p7_oprofile_Destroy(m->om);
      m->om = NULL;
      if (p7_oprofile_ReadMSV(hfp, &m->abc, &m->om) != eslOK) die("p7_oprofile_ReadMSV");
    }
  } else {
    for (int i = 0; i <= idx; i++) {
      if (m->hmm) p7_hmm_Destroy(m->hmm);
      m->hmm = NULL;
      if (p7_hmmfile_Read(hfp, &m->abc, &m->hmm) != eslOK) die("p7_hmmfile_Read");
    }
    m->bg = p7_bg_Create(m->abc);
    m->gm = p7_profile_Create(m->hmm->M, m->abc);
    m->om = p7_oprofile_Create(m->hmm->M, m->abc);
    if (p7_ProfileConfig(m->hmm, m->bg, m->gm, 100, p7_LOCAL) != eslOK) die("p7_ProfileConfig");
    if (p7_oprofile_Convert(m->gm, m->om) != eslOK) die("p7_oprofile_Convert");
  }
  m->bg = p7_bg_Create(m->abc);
  p7_hmmfile_Close(hfp);
}

static void write_vprofile(const model_t *m, const char *path)
{
  FILE *fp = fopen(path, "wb"); if (!fp) die("open vprofile out");
  const P7_OPROFILE *om = m->om;
  int32_t hdr[3]; int Q8 = p7O_NQW(om->M);
  hdr[0] = om->M; hdr[1] = Q8; hdr[2] = m->abc->Kp;
  fwrite("VITPROF1", 1, 8, fp);
  fwrite(hdr, 4, 3, fp);
  fwrite(&om->scale_w, 4, 1, fp); fwrite(&om->nj, 4, 1, fp);
  fwrite(&om->base_w, 2, 1, fp); fwrite(&om->ddbound_w, 2, 1, fp);
  fwrite(om->xw, 2, 8, fp);
  float ev[2] = { om->evparam[p7_VMU], om->evparam[p7_VLAMBDA] };
  fwrite(ev, 4, 2, fp);
  fwrite(om->twv, 16, 8 * Q8, fp);
  for (int x = 0; x < m->abc->Kp; x++) fwrite(om->rwv[x], 16, Q8, fp);
  fclose(fp);
}

typedef struct { int64_t n, total; int64_t *off; uint8_t *dsq; } seqs_t;

static void write_seqs(const seqs_t *s, const char *path)
{
  FILE *fp = fopen(path, "wb"); if (!fp) die("open seqs out");
  fwrite("MSVSEQS1", 1, 8, fp);
  fwrite(&s->n, 8, 1, fp); fwrite(&s->total, 8, 1, fp);
  fwrite(s->off, 8, s->n + 1, fp); fwrite(s->dsq, 1, s->total, fp);
  fclose(fp);
}

static void read_seqs(seqs_t *s, const char *path)
{
  char mag[8]; FILE *fp = fopen(path, "rb"); if (!fp) die("open seqs in");
  if (fread(mag, 1, 8, fp) != 8 || memcmp(mag, "MSVSEQS1", 8)) die("bad seqs magic");
  if (fread(&s->n, 8, 1, fp) != 1 || fread(&s->total, 8, 1, fp) != 1) die("short seqs");
  s->off = malloc(8 * (s->n + 1)); s->dsq = malloc(s->total > 0 ? s->total : 1);
  if (fread(s->off, 8, s->n + 1, fp) != (size_t)(s->n + 1)) die("short offsets");
  if (fread(s->dsq, 1, s->total, fp) != (size_t) s->total) die("short residues");
  fclose(fp);
}

static void push_seq(seqs_t *s, int64_t *cap, const ESL_DSQ *dsq, int L)
{
  while (s->total + L > *cap) { *cap = *cap * 2 + L; s->dsq = realloc(s->dsq, *cap); }
  memcpy(s->dsq + s->total, dsq + 1, L);
  s->total += L; s->n++;
  s->off = realloc(s->off, 8 * (s->n + 1)); s->off[s->n] = s->total;
}

int main(int argc, char **argv)
{
  if (argc < 2) die("usage: refgen profile|emit|randseq|score ...");
  const char *cmd = argv[1];

  if (!strcmp(cmd, "profile")) {            /* profile M seed Lcfg mode out */
    if (argc != 7) die("profile M seed Lcfg mode(1=local,3=unilocal) out");
    model_t m; int M = atoi(argv[2]), Lcfg = atoi(argv[4]);
    make_model(&m, M, (uint32_t) atol(argv[3]), Lcfg, atoi(argv[5]));
    write_profile(&m, Lcfg, argv[6]);
    return 0;
  }
  if (!strcmp(cmd, "emit")) {               /* emit M seed Lcfg mode n emitseed repeat out */
    if (argc != 10) die("emit M seed Lcfg mode n emitseed repeat out");
    model_t m; int M = atoi(argv[2]), Lcfg = atoi(argv[4]);
    make_model(&m, M, (uint32_t) atol(argv[3]), Lcfg, atoi(argv[5]));
    int n = atoi(argv[6]), rep = atoi(argv[8]);
    ESL_RANDOMNESS *r = esl_randomness_Create((uint32_t) atol(argv[7]));
    ESL_SQ *sq = esl_sq_CreateDigital(m.abc);
    seqs_t s = {0, 0, NULL, NULL}; int64_t cap = 0;
    s.off = malloc(8); s.off[0] = 0;
    ESL_DSQ *buf = NULL;
    for (int i = 0; i < n; i++) {
      esl_sq_Reuse(sq);
      if (p7_ProfileEmit(r, m.hmm, m.gm, m.bg, sq, NULL) != eslOK) die("p7_ProfileEmit");
      int L = (int) sq->n;
      if (rep <= 1) { push_seq(&s, &cap, sq->dsq, L); continue; }
      buf = realloc(buf, (size_t) L * rep + 2);
      buf[0] = eslDSQ_SENTINEL;
      for (int k = 0; k < rep; k++) memcpy(buf + 1 + (size_t) k * L, sq->dsq + 1, L);
      buf[(size_t) L * rep + 1] = eslDSQ_SENTINEL;
      push_seq(&s, &cap, buf, L * rep);
    }
    write_seqs(&s, argv[9]);
    return 0;
  }
  if (!strcmp(cmd, "randseq")) {            /* randseq n L seed out */
    if (argc != 6) die("randseq n L seed out");
    ESL_ALPHABET *abc = esl_alphabet_Create(eslAMINO);
    P7_BG *bg = p7_bg_Create(abc);
    int n = atoi(argv[2]), L = atoi(argv[3]);
    ESL_RANDOMNESS *r = esl_randomness_Create((uint32_t) atol(argv[4]));
    ESL_DSQ *dsq = malloc(L + 2);
    seqs_t s = {0, 0, NULL, NULL}; int64_t cap = 0;
    s.off = malloc(8); s.off[0] = 0;
    for (int i = 0; i < n; i++) {
      if (esl_rsq_xfIID(r, bg->f, abc->K, L, dsq) != eslOK) die("esl_rsq_xfIID");
      push_seq(&s, &cap, dsq, L);
    }
    write_seqs(&s, argv[5]);
    return 0;
  }
  if (!strcmp(cmd, "hmmfile")) {            /* hmmfile path idx pressed(0/1) out */
    if (argc != 6) die("hmmfile path idx pressed out");
    model_t m;
    file_model(&m, argv[2], atoi(argv[3]), atoi(argv[4]));
    write_profile(&m, 100, argv[5]);
    return 0;
  }
  if (!strcmp(cmd, "seqfile")) {            /* seqfile path out */
    if (argc != 4) die("seqfile path out");
    ESL_ALPHABET *abc = esl_alphabet_Create(eslAMINO);
    ESL_SQFILE *sqfp = NULL;
    if (esl_sqfile_OpenDigital(abc, argv[2], eslSQFILE_UNKNOWN, NULL, &sqfp) != eslOK) die("esl_sqfile_OpenDigital");
    ESL_SQ *sq = esl_sq_CreateDigital(abc);
    seqs_t s = {0, 0, NULL, NULL}; int64_t cap = 0;
    s.off = malloc(8); s.off[0] = 0;
    int st;
    while ((st = esl_sqio_Read(sqfp, sq)) == eslOK) { push_seq(&s, &cap, sq->dsq, (int) sq->n); esl_sq_Reuse(sq); }
    if (st != eslEOF) die("esl_sqio_Read");
    write_seqs(&s, argv[3]);
    return 0;
  }
  if (!strcmp(cmd, "emitfile")) {           /* emitfile hmmfile idx n emitseed out */
    if (argc != 7) die("emitfile hmmfile idx n emitseed out");
    model_t m;
    file_model(&m, argv[2], atoi(argv[3]), 0);
    int n = atoi(argv[4]);
    ESL_RANDOMNESS *r = esl_randomness_Create((uint32_t) atol(argv[5]));
    ESL_SQ *sq = esl_sq_CreateDigital(m.abc);
    seqs_t s = {0, 0, NULL, NULL}; int64_t cap = 0;
    s.off = malloc(8); s.off[0] = 0;
    for (int i = 0; i < n; i++) {
      esl_sq_Reuse(sq);
      if (p7_ProfileEmit(r, m.hmm, m.gm, m.bg, sq, NULL) != eslOK) die("p7_ProfileEmit");
      push_seq(&s, &cap, sq->dsq, (int) sq->n);
    }
    write_seqs(&s, argv[6]);
    return 0;
  }
  if (!strcmp(cmd, "vit") || !strcmp(cmd, "vitfile")) {  /* vit M seed prof res seqs | vitfile hmmfile idx prof res seqs */
    model_t m;
    seqs_t s;
    if (!strcmp(cmd, "vit")) {
      if (argc != 7) die("vit M seed vprof vres seqs");
      make_model(&m, atoi(argv[2]), (uint32_t) atol(argv[3]), 100, p7_LOCAL);
    } else {
      if (argc != 7) die("vitfile hmmfile idx vprof vres seqs");
      file_model(&m, argv[2], atoi(argv[3]), 0);
    }
    write_vprofile(&m, argv[4]);
    read_seqs(&s, argv[6]);
    int64_t maxL = 1;
    for (int64_t i = 0; i < s.n; i++) if (s.off[i+1] - s.off[i] > maxL) maxL = s.off[i+1] - s.off[i];
    P7_OMX *ox = p7_omx_Create(m.om->M, 0, 0);
    ESL_DSQ *dsq = malloc(maxL + 2);
    int32_t *st = calloc(s.n, 4); float *sc = calloc(s.n, 4);
    for (int64_t i = 0; i < s.n; i++) {
      int L = (int) (s.off[i+1] - s.off[i]);
      if (L == 0) { st[i] = -1; continue; }
      dsq[0] = eslDSQ_SENTINEL; memcpy(dsq + 1, s.dsq + s.off[i], L); dsq[L+1] = eslDSQ_SENTINEL;
      p7_oprofile_ReconfigLength(m.om, L);
      st[i] = p7_ViterbiFilter(dsq, L, m.om, ox, &sc[i]);
    }
    FILE *fp = fopen(argv[5], "wb"); if (!fp) die("open vres out");
    fwrite("VITRES01", 1, 8, fp); fwrite(&s.n, 8, 1, fp);
    fwrite(st, 4, s.n, fp); fwrite(sc, 4, s.n, fp);
    fclose(fp);
    return 0;
  }
  if (!strcmp(cmd, "pipe") || !strcmp(cmd, "pipefile")) {  /* pipe M seed pres seqs [prof] | pipefile hmmfile idx pres seqs [prof] */
    model_t m;
    seqs_t s;
    if (argc != 6 && argc != 7) die("pipe M seed pres seqs [prof] | pipefile hmmfile idx pres seqs [prof]");
    if (!strcmp(cmd, "pipe")) {
      make_model(&m, atoi(argv[2]), (uint32_t) atol(argv[3]), 100, p7_LOCAL);
      /* a sampled HMM has no composition; give it the one hmmbuild would
       * (p7_hmm_SetComposition, src/p7_hmm.c:625), copied as p7_ProfileConfig
       * and p7_oprofile_Convert copy it (modelconfig.c:84, p7_oprofile.c:870) */
      if (p7_hmm_SetComposition(m.hmm) != eslOK) die("p7_hmm_SetComposition");
      for (int z = 0; z < p7_MAXABET; z++) m.gm->compo[z] = m.om->compo[z] = m.hmm->compo[z];
    } else file_model(&m, argv[2], atoi(argv[3]), 0);
    if (argc == 7) write_profile(&m, 100, argv[6]);       /* the MSV part of the same configured model */
    read_seqs(&s, argv[5]);
    const double F1 = 0.02, F2 = 1e-3;      /* p7_pipeline.c:210-211 defaults */
    p7_bg_SetFilter(m.bg, m.om->M, m.om->compo);
    int64_t maxL = 1;
    for (int64_t i = 0; i < s.n; i++) if (s.off[i+1] - s.off[i] > maxL) maxL = s.off[i+1] - s.off[i];
    P7_OMX *ox = p7_omx_Create(m.om->M, 0, 0);
    ESL_DSQ *dsq = malloc(maxL + 2);
    float *ns = calloc(s.n, 4), *us = calloc(s.n, 4), *fs = calloc(s.n, 4), *vs = calloc(s.n, 4);
    uint8_t *stage = calloc(s.n, 1);
    for (int64_t i = 0; i < s.n; i++) {
      int L = (int) (s.off[i+1] - s.off[i]);
      float usc, nullsc, filtersc, vfsc, seq_score;
      double P;
      vs[i] = NAN;
      if (L == 0) { stage[i] = 255; continue; }
      dsq[0] = eslDSQ_SENTINEL; memcpy(dsq + 1, s.dsq + s.off[i], L); dsq[L+1] = eslDSQ_SENTINEL;
      p7_bg_SetLength(m.bg, L);
      p7_oprofile_ReconfigLength(m.om, L);
      p7_bg_NullOne(m.bg, dsq, L, &nullsc);
      p7_MSVFilter(dsq, L, m.om, ox, &usc);
      p7_bg_FilterScore(m.bg, dsq, L, &filtersc);
      ns[i] = nullsc; us[i] = usc; fs[i] = filtersc;
      seq_score = (usc - nullsc) / eslCONST_LOG2;
      P = esl_gumbel_surv(seq_score, m.om->evparam[p7_MMU], m.om->evparam[p7_MLAMBDA]);
      if (P > F1) { stage[i] = 0; continue; }
      seq_score = (usc - filtersc) / eslCONST_LOG2;
      P = esl_gumbel_surv(seq_score, m.om->evparam[p7_MMU], m.om->evparam[p7_MLAMBDA]);
      if (P > F1) { stage[i] = 1; continue; }
      if (P > F2) {
        p7_ViterbiFilter(dsq, L, m.om, ox, &vfsc);
        vs[i] = vfsc;
        seq_score = (vfsc - filtersc) / eslCONST_LOG2;
        P = esl_gumbel_surv(seq_score, m.om->evparam[p7_VMU], m.om->evparam[p7_VLAMBDA]);
        if (P > F2) { stage[i] = 2; continue; }
      }
      stage[i] = 3;
    }
    FILE *fp = fopen(argv[4], "wb"); if (!fp) die("open pres out");
    int32_t M = m.om->M;
    float ev[4] = { m.om->evparam[p7_MMU], m.om->evparam[p7_MLAMBDA], m.om->evparam[p7_VMU], m.om->evparam[p7_VLAMBDA] };
    double F[2] = { F1, F2 };
    fwrite("PIPERES1", 1, 8, fp); fwrite(&M, 4, 1, fp); fwrite(m.om->compo, 4, 20, fp);
    fwrite(ev, 4, 4, fp); fwrite(F, 8, 2, fp); fwrite(&s.n, 8, 1, fp);
    fwrite(ns, 4, s.n, fp); fwrite(us, 4, s.n, fp); fwrite(fs, 4, s.n, fp); fwrite(vs, 4, s.n, fp);
    fwrite(stage, 1, s.n, fp);
    fclose(fp);
    return 0;
  }
  if (!strcmp(cmd, "score") || !strcmp(cmd, "scorefile")) {  /* score M seed Lcfg mode seqs out | scorefile hmmfile idx seqs out */
    model_t m; int M;
    seqs_t s;
    const char *outpath;
    if (!strcmp(cmd, "score")) {
      if (argc != 8) die("score M seed Lcfg mode seqs out");
      M = atoi(argv[2]);
      make_model(&m, M, (uint32_t) atol(argv[3]), atoi(argv[4]), atoi(argv[5]));
      read_seqs(&s, argv[6]);
      outpath = argv[7];
    } else {
      if (argc != 6) die("scorefile hmmfile idx seqs out");
      file_model(&m, argv[2], atoi(argv[3]), 0);
      M = m.om->M;
      read_seqs(&s, argv[4]);
      outpath = argv[5];
    }
    int64_t maxL = 1;
    for (int64_t i = 0; i < s.n; i++) if (s.off[i+1] - s.off[i] > maxL) maxL = s.off[i+1] - s.off[i];
    P7_OMX *ox = p7_omx_Create(M, 0, 0);
    ESL_DSQ *dsq = malloc(maxL + 2);
    int32_t *st = calloc(s.n, 4); float *sc = calloc(s.n, 4);
    double *ns = calloc(s.n, 8), *P = calloc(s.n, 8); uint8_t *pass = calloc(s.n, 1);
    const double F1 = 0.02;                 /* p7_pipeline.c:210 default */
    for (int64_t i = 0; i < s.n; i++) {
      int L = (int) (s.off[i+1] - s.off[i]);
      float usc, nullsc;
      if (L == 0) { st[i] = -1; continue; } /* the pipeline skips empty sequences (p7_pipeline.c:662) */
      dsq[0] = eslDSQ_SENTINEL; memcpy(dsq + 1, s.dsq + s.off[i], L); dsq[L+1] = eslDSQ_SENTINEL;
      p7_bg_SetLength(m.bg, L);
      p7_oprofile_ReconfigLength(m.om, L);
      p7_bg_NullOne(m.bg, dsq, L, &nullsc);
      st[i] = p7_MSVFilter(dsq, L, m.om, ox, &usc);
      sc[i] = usc; ns[i] = nullsc;
      float seq_score = (usc - nullsc) / eslCONST_LOG2;
      P[i] = esl_gumbel_surv(seq_score, m.om->evparam[p7_MMU], m.om->evparam[p7_MLAMBDA]);
      pass[i] = (P[i] > F1) ? 0 : 1;
    }
    FILE *fp = fopen(outpath, "wb"); if (!fp) die("open result out");
    fwrite("MSVRES01", 1, 8, fp); fwrite(&s.n, 8, 1, fp);
    fwrite(st, 4, s.n, fp); fwrite(sc, 4, s.n, fp); fwrite(ns, 8, s.n, fp);
    fwrite(P, 8, s.n, fp); fwrite(pass, 1, s.n, fp);
    fclose(fp);
    return 0;
  }
  die("unknown command");
  return 1;
}
