/* msv_oracle.c -- CPU oracle for the MSV filter (TEST INFRASTRUCTURE ONLY).
 *
 * Scalar C restatement of HMMER 3.1b1's p7_MSVFilter with its SSV fast path,
 * written from the reference's documented algorithm; see msv_oracle.h.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Build: cc -O2 -ffp-contract=off -fPIC -shared -pthread msv_oracle.c -lm
 * (-ffp-contract=off matters: the reference's x86 build has no FMA, and the
 * float/double expressions of the score and P-value must round identically.)
 */
#include "msv_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static inline uint8_t sat_add_u8(int a, int b) { int s = a + b; return (uint8_t) (s > 255 ? 255 : s); }
static inline uint8_t sat_sub_u8(int a, int b) { int s = a - b; return (uint8_t) (s < 0 ? 0 : s); }
static inline int8_t  sat_sub_s8(int a, int b) { int s = a - b; return (int8_t) (s > 127 ? 127 : (s < -128 ? -128 : s)); }
static inline uint8_t max_u8(uint8_t a, uint8_t b) { return a > b ? a : b; }

/* rbv byte for residue x at node k (1..16Q): striped slot q=(k-1)%Q, z=(k-1)/Q
 * (src/impl_sse/p7_oprofile.c:619-635). */
static inline uint8_t rbv_at(const orc_profile *om, int x, int k)
{
  int q = (k - 1) % om->Q, z = (k - 1) / om->Q;
  return om->rbv[((size_t) x * om->Q + q) * 16 + z];
}

/* unbiased_byteify(logf(3/(L+3))): src/impl_sse/p7_oprofile.c:511-519, 920-925 */
uint8_t orc_tjb_b(float scale_b, int L)
{
  float sc = logf(3.0f / (float) (L + 3));
  sc = -1.0f * roundf(scale_b * sc);
  return (sc > 255.) ? 255 : (uint8_t) sc;
}

/* src/impl_sse/msvfilter.c:205-210 (same in ssvfilter.c:1408-1410) */
float orc_score_from_xj(uint8_t xj, uint8_t tjb_b, uint8_t base_b, float scale_b)
{
  float sc = ((float) ((int) xj - (int) tjb_b) - (float) base_b);
  sc /= scale_b;
  sc -= 3.0;
  return sc;
}

/* SSV filter: src/impl_sse/ssvfilter.c:1364-1413, with get_xE (:1320-1361)
 * restated as the plain diagonal recurrence it sweeps in bands:
 *   v(i,k) = sat_s8( v(i-1,k-1) - sb(x_i,k) ),  v(.,0) = v(0,.) = -128,
 *   sb = ((127 + bias) -sat rbv) ^ 127      (sf_conversion, p7_oprofile.c:549-590)
 *   xE = unsigned max over all cells of (uint8) v, starting at 128.
 * The reference ORs the sign bit into every lane at stripe boundaries
 * (CONVERT_STEP, ssvfilter.c:590-596); that only alters cells that are
 * already >= 0, which can only be reached through a cell in [-bias,-1],
 * i.e. after xE >= 255-bias has been recorded, so the decision is unchanged.
 * Returns eslOK / eslERANGE / eslENORESULT. */
static int ssv_filter(const uint8_t *dsq, int L, const orc_profile *om, uint8_t tjb_b,
                      int8_t *v, uint8_t *ret_xj, float *ret_sc)
{
  const int M = om->M;
  int tbm = om->tbm_b, tec = om->tec_b, base = om->base_b, bias = om->bias_b, tjb = tjb_b;

  if (tjb + tbm + tec + bias >= 127) return ORC_eslENORESULT;

  uint8_t xEu = 128;
  for (int k = 0; k <= M; k++) v[k] = -128;
  for (int i = 1; i <= L; i++) {
    int x = dsq[i];
    for (int k = M; k >= 1; k--) {
      int r  = rbv_at(om, x, k);
      int sb = (int8_t) (uint8_t) (sat_sub_u8(127 + bias, r) ^ 127);
      int8_t nv = sat_sub_s8(v[k - 1], sb);
      v[k] = nv;
      xEu  = max_u8(xEu, (uint8_t) nv);
    }
  }

  uint16_t xE = xEu, xJ;
  if (xE >= 255 - bias) {
    *ret_sc = INFINITY;
    if (base - tjb - tbm < 128) return ORC_eslENORESULT;
    *ret_xj = 255;
    return ORC_eslERANGE;
  }
  xE = (uint16_t) (xE + base - tjb - tbm);
  xE = (uint16_t) (xE - 128);
  if (xE >= 255 - bias) { *ret_sc = INFINITY; *ret_xj = 255; return ORC_eslERANGE; }
  xJ = (uint16_t) (xE - tec);
  if (xJ > base) return ORC_eslENORESULT;
  *ret_xj = (uint8_t) xJ;
  *ret_sc = orc_score_from_xj((uint8_t) xJ, tjb_b, om->base_b, om->scale_b);
  return ORC_eslOK;
}

/* Full MSV: src/impl_sse/msvfilter.c:112-212 in node order k=1..M
 * (the striped predecessor of node k is node k-1; node 0 is -inf = 0). */
static int msv_full(const uint8_t *dsq, int L, const orc_profile *om, uint8_t tjb_b,
                    uint8_t *dp, uint8_t *ret_xj, float *ret_sc)
{
  const int M = om->M;
  const int bias = om->bias_b, base = om->base_b, tec = om->tec_b;
  /* (int8_t) tjb_b + (int8_t) tbm_b splatted into bytes: sum modulo 256 (msvfilter.c:120) */
  const uint8_t tjbm = (uint8_t) ((int8_t) tjb_b + (int8_t) om->tbm_b);
  uint8_t xJ = 0, xB = sat_sub_u8(base, tjbm);

  memset(dp, 0, (size_t) M + 1);
  for (int i = 1; i <= L; i++) {
    int x = dsq[i];
    uint8_t xE = 0;
    for (int k = M; k >= 1; k--) {
      uint8_t sv = max_u8(dp[k - 1], xB);
      sv = sat_add_u8(sv, bias);
      sv = sat_sub_u8(sv, rbv_at(om, x, k));
      dp[k] = sv;
      xE = max_u8(xE, sv);
    }
    if (sat_add_u8(xE, bias) == 255) { *ret_sc = INFINITY; *ret_xj = 255; return ORC_eslERANGE; }
    xE = sat_sub_u8(xE, tec);
    xJ = max_u8(xJ, xE);
    xB = sat_sub_u8(max_u8(base, xJ), tjbm);
  }
  *ret_xj = xJ;
  *ret_sc = orc_score_from_xj(xJ, tjb_b, om->base_b, om->scale_b);
  return ORC_eslOK;
}

int orc_msv_full(const uint8_t *dsq, int L, const orc_profile *om, uint8_t tjb_b,
                 uint8_t *ret_xj, float *ret_sc)
{
  uint8_t *dp = malloc((size_t) om->M + 1);
  if (!dp) return ORC_eslEINVAL;
  int st = msv_full(dsq, L, om, tjb_b, dp, ret_xj, ret_sc);
  free(dp);
  return st;
}

static int msv_filter_ws(const uint8_t *dsq, int L, const orc_profile *om, uint8_t tjb_b,
                         void *ws, uint8_t *ret_xj, float *ret_sc, int *ret_path)
{
  int st = ssv_filter(dsq, L, om, tjb_b, (int8_t *) ws, ret_xj, ret_sc);  /* msvfilter.c:106-108 */
  if (st != ORC_eslENORESULT) { if (ret_path) *ret_path = 0; return st; }
  if (ret_path) *ret_path = 1;
  return msv_full(dsq, L, om, tjb_b, (uint8_t *) ws, ret_xj, ret_sc);
}

int orc_msv_filter(const uint8_t *dsq, int L, const orc_profile *om, uint8_t tjb_b,
                   uint8_t *ret_xj, float *ret_sc, int *ret_path)
{
  void *ws = malloc((size_t) om->M + 1);
  if (!ws) return ORC_eslEINVAL;
  int st = msv_filter_ws(dsq, L, om, tjb_b, ws, ret_xj, ret_sc, ret_path);
  free(ws);
  return st;
}

/* p7_bg_SetLength + p7_bg_NullOne (src/p7_bg.c:191-199, 359-363), the score
 * transform and F1 test of p7_Pipeline (src/p7_pipeline.c:673-676) and
 * esl_gumbel_surv (easel/esl_gumbel.c:129-137). */
int orc_f1_pass(float usc, int L, double mmu, double mlambda, double F1,
                float *ret_nullsc, double *ret_P)
{
  float  p1 = (float) L / (float) (L + 1);
  float  nullsc = (float) L * log(p1) + log(1. - p1);
  float  seq_score = (usc - nullsc) / 0.69314718055994529;
  double y  = mlambda * ((double) seq_score - mmu);
  double ey = -exp(-y);
  double P  = (fabs(ey) < 5e-9) ? -ey : 1 - exp(ey);
  if (ret_nullsc) *ret_nullsc = nullsc;
  if (ret_P) *ret_P = P;
  return (P > F1) ? 0 : 1;
}

typedef struct {
  const orc_profile *om; const uint8_t *res; const int64_t *off; int64_t n; double F1;
  int32_t *status; uint8_t *xj; float *sc; uint8_t *pass; uint8_t *path;
  int64_t next; pthread_mutex_t mu;
} batch_t;

static void *batch_worker(void *arg)
{
  batch_t *b = (batch_t *) arg;
  int64_t maxL = 0;
  for (int64_t i = 0; i < b->n; i++) if (b->off[i + 1] - b->off[i] > maxL) maxL = b->off[i + 1] - b->off[i];
  uint8_t *dsq = malloc((size_t) maxL + 2);
  void    *ws  = malloc((size_t) b->om->M + 1);
  for (;;) {
    int64_t lo, hi;
    pthread_mutex_lock(&b->mu);
    lo = b->next; hi = lo + 64 < b->n ? lo + 64 : b->n; b->next = hi;
    pthread_mutex_unlock(&b->mu);
    if (lo >= b->n) break;
    for (int64_t i = lo; i < hi; i++) {
      int L = (int) (b->off[i + 1] - b->off[i]);
      uint8_t xj = 0; float sc = 0.0f; int path = 0, st;
      if (L == 0) {
        if (b->status) b->status[i] = -1;
        if (b->xj) b->xj[i] = 0;
        if (b->sc) b->sc[i] = 0.0f;
        if (b->pass) b->pass[i] = 0;
        if (b->path) b->path[i] = 0;
        continue;
      }
      dsq[0] = 255; memcpy(dsq + 1, b->res + b->off[i], (size_t) L); dsq[L + 1] = 255;
      uint8_t tjb = orc_tjb_b(b->om->scale_b, L);
      st = msv_filter_ws(dsq, L, b->om, tjb, ws, &xj, &sc, &path);
      if (b->status) b->status[i] = st;
      if (b->xj) b->xj[i] = xj;
      if (b->sc) b->sc[i] = sc;
      if (b->path) b->path[i] = (uint8_t) path;
      if (b->pass) b->pass[i] = (uint8_t) orc_f1_pass(sc, L, b->om->mmu, b->om->mlambda, b->F1, NULL, NULL);
    }
  }
  free(dsq); free(ws);
  return NULL;
}

int orc_msv_batch(const orc_profile *om, const uint8_t *residues, const int64_t *off,
                  int64_t n, double F1, int nthreads,
                  int32_t *status, uint8_t *xj, float *sc, uint8_t *pass, uint8_t *path)
{
  batch_t b = { om, residues, off, n, F1, status, xj, sc, pass, path, 0 };
  pthread_mutex_init(&b.mu, NULL);
  if (nthreads <= 0) { long c = sysconf(_SC_NPROCESSORS_ONLN); nthreads = c > 0 ? (int) c : 1; }
  pthread_t *th = malloc(sizeof(pthread_t) * (size_t) nthreads);
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, batch_worker, &b);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&b.mu);
  return nthreads;
}
