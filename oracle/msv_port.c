/* msv_port.c -- vectorized CPU port of the reference MSV filter
 * (TEST INFRASTRUCTURE AND CPU BASELINE ONLY).
 *
 * A 16-lane uint8 restatement of HMMER 3.1b1's SSE2 p7_MSVFilter
 * (src/impl_sse/msvfilter.c:77-213) and of the SSV filter it calls first
 * (src/impl_sse/ssvfilter.c:1364-1413, signed-saturation trick with the sbv
 * costs of sf_conversion, src/impl_sse/p7_oprofile.c:549-590), over the same
 * striped [Kp][Q][16] profile layout. It is the timed CPU baseline on hosts
 * where the reference's own SSE2 code cannot run (the aarch64 GPU hosts):
 * bench.py's cpu_baseline leg and `bench.py --impl reference`. Its results
 * are pinned to the reference's golden vectors (tests/test_port_golden.py).
 * The product never links it.
 *
 * The few vector operations it needs are wrapped below: NEON intrinsics on
 * aarch64 (the hosts it is timed on), and elsewhere GCC vector extensions
 * with the saturating byte arithmetic written out (slower; used by the tests
 * on other hosts): unsigned/signed saturating byte arithmetic, byte max, a
 * one-byte lane shift and a horizontal max.
 *
 * The SSV pass follows the reference's register scheme
 * (ssvfilter.c:215-330): with no J state the diagonals never meet, so a
 * register follows 16 diagonals down the whole sequence -- one saturating
 * subtract, one max and one profile load per row, a byte shift where its
 * vector index wraps -- and the Q vectors are covered by sweeps of up to 8
 * registers; no DP row is kept in memory.
 *
 * Build: cc -O3 -ffp-contract=off -fPIC -shared -pthread msv_port.c msv_oracle.c -lm
 */
#include "msv_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#if defined(__aarch64__)
#include <arm_neon.h>
typedef uint8x16_t v16;
static inline v16 v_set1(uint8_t x) { return vdupq_n_u8(x); }
static inline v16 v_subs_u8(v16 a, v16 b) { return vqsubq_u8(a, b); }
static inline v16 v_adds_u8(v16 a, v16 b) { return vqaddq_u8(a, b); }
static inline v16 v_max_u8(v16 a, v16 b) { return vmaxq_u8(a, b); }
static inline v16 v_subs_s8(v16 a, v16 b) { return vreinterpretq_u8_s8(vqsubq_s8(vreinterpretq_s8_u8(a), vreinterpretq_s8_u8(b))); }
static inline v16 v_shl1(v16 a) { return vextq_u8(vdupq_n_u8(0), a, 15); }  /* lane z <- lane z-1, lane 0 <- 0 */
static inline v16 v_or(v16 a, v16 b) { return vorrq_u8(a, b); }
static inline uint8_t v_hmax(v16 a) { return vmaxvq_u8(a); }
static inline v16 v_load(const uint8_t *p) { return vld1q_u8(p); }
#else
typedef uint8_t v16 __attribute__((vector_size(16)));
typedef int8_t v16s __attribute__((vector_size(16)));
static inline v16 v_set1(uint8_t x) { v16 r; for (int z = 0; z < 16; z++) r[z] = x; return r; }
static inline v16 v_subs_u8(v16 a, v16 b) { return (v16) ((a - b) & (v16) (a >= b)); }
static inline v16 v_adds_u8(v16 a, v16 b) { v16 s = a + b; return (v16) (s | (v16) (s < a)); }
static inline v16 v_max_u8(v16 a, v16 b) { const v16 m = (v16) (a > b); return (a & m) | (b & ~m); }
static inline v16 v_subs_s8(v16 a, v16 b) {
  const v16s x = (v16s) a, y = (v16s) b, r = x - y;
  const v16s ov = ((x ^ y) & (x ^ r)) < 0;                 /* signed overflow lanes */
  const v16s sat = (x >> 7) ^ (v16s) {127, 127, 127, 127, 127, 127, 127, 127, 127, 127, 127, 127, 127, 127, 127, 127};
  return (v16) ((ov & sat) | (~ov & r));
}
static inline v16 v_shl1(v16 a) {
  const v16 z = {0};
  return __builtin_shuffle(z, a, (v16) {0, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30});
}
static inline v16 v_or(v16 a, v16 b) { return a | b; }
static inline uint8_t v_hmax(v16 a) { uint8_t m = 0; for (int z = 0; z < 16; z++) if (a[z] > m) m = a[z]; return m; }
static inline v16 v_load(const uint8_t *p) { v16 r; memcpy(&r, p, 16); return r; }
#endif

typedef struct {
  int Q;
  v16 *sbv;      /* [Kp][Q]: SSV costs, ((127 + bias) -sat rbv) ^ 127 */
  v16 *rbv;      /* [Kp][Q] */
} port_prof;

static int port_prepare(const orc_profile *om, port_prof *pp)
{
  const int Q = om->Q, Kp = om->Kp;
  pp->Q = Q;
  if (posix_memalign((void **) &pp->sbv, 16, sizeof(v16) * Kp * Q)) return -1;
  if (posix_memalign((void **) &pp->rbv, 16, sizeof(v16) * Kp * Q)) return -1;
  for (int x = 0; x < Kp; x++)
    for (int q = 0; q < Q; q++) {
      uint8_t t[16];
      const uint8_t *r = om->rbv + ((size_t) x * Q + q) * 16;
      for (int z = 0; z < 16; z++) {
        int s = 127 + om->bias_b - r[z];
        t[z] = (uint8_t) ((s < 0 ? 0 : s) ^ 127);
      }
      pp->sbv[x * Q + q] = v_load(t);
      pp->rbv[x * Q + q] = v_load(r);
    }
  return 0;
}

/* One sweep of the SSV pass: W registers, register j holding the 16
 * diagonals that sit in striped vector q0 + j at row 1. Each row a register
 * moves one vector on (cell (i, q) -> (i+1, q+1)); from the last vector it
 * wraps to vector 0 with its lanes shifted by one (node k -> k+1 across the
 * stripe boundary) and the begin value entering lane 0. */
#define SSV_SWEEP(W)                                                                                   \
  static v16 ssv_sweep_##W(const uint8_t *dsq, int L, const v16 *sbv, int Q, int q0, v16 xEv,          \
                           v16 beginv, v16 begin0)                                                      \
  {                                                                                                    \
    v16 sv[W], xe[W];                  /* one max accumulator per register: no chain across them */  \
    int p[W];                                                                                          \
    for (int j = 0; j < W; j++) { sv[j] = beginv; xe[j] = xEv; p[j] = q0 + j; }                        \
    for (int i = 1; i <= L;) {                                                                         \
      /* rows until a register reaches the last vector; none wraps before that */                      \
      int seg = L - i + 1;                                                                             \
      for (int j = 0; j < W; j++) if (Q - p[j] < seg) seg = Q - p[j];                                  \
      for (int t = 0; t < seg; t++, i++) {                                                             \
        const v16 *sc = sbv + (size_t) dsq[i] * Q + t;                                                 \
        for (int j = 0; j < W; j++) { sv[j] = v_subs_s8(sv[j], sc[p[j]]); xe[j] = v_max_u8(xe[j], sv[j]); } \
      }                                                                                                \
      for (int j = 0; j < W; j++) {                                                                    \
        p[j] += seg;                                                                                   \
        if (p[j] == Q) { p[j] = 0; sv[j] = v_or(v_shl1(sv[j]), begin0); }                              \
      }                                                                                                \
    }                                                                                                  \
    for (int j = 0; j < W; j++) xEv = v_max_u8(xEv, xe[j]);                                            \
    return xEv;                                                                                        \
  }
SSV_SWEEP(1) SSV_SWEEP(2) SSV_SWEEP(3) SSV_SWEEP(4) SSV_SWEEP(5) SSV_SWEEP(6) SSV_SWEEP(7) SSV_SWEEP(8)
#define SSV_WMAX 8

/* SSV filter: the J-free diagonal recurrence in the reference's signed
 * domain (begin = -128 = 0x80); xE is the unsigned max over all cells,
 * computed by sweeps of up to SSV_WMAX registers of diagonals. */
static int port_ssv(const uint8_t *dsq, int L, const orc_profile *om, const port_prof *pp, uint8_t tjb,
                    uint8_t *ret_xj, float *ret_sc)
{
  const int Q = pp->Q;
  int tbm = om->tbm_b, tec = om->tec_b, base = om->base_b, bias = om->bias_b;
  if (tjb + tbm + tec + bias >= 127) return ORC_eslENORESULT;
  const v16 beginv = v_set1(128);
  uint8_t lane0[16] = {128, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  const v16 begin0 = v_load(lane0);
  v16 xEv = beginv;
  const int ns = (Q + SSV_WMAX - 1) / SSV_WMAX;         /* sweeps of balanced widths */
  for (int k = 0, q0 = 0; k < ns; k++) {
    const int w = Q / ns + (k < Q % ns ? 1 : 0);
    switch (w) {
      case 1: xEv = ssv_sweep_1(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
      case 2: xEv = ssv_sweep_2(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
      case 3: xEv = ssv_sweep_3(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
      case 4: xEv = ssv_sweep_4(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
      case 5: xEv = ssv_sweep_5(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
      case 6: xEv = ssv_sweep_6(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
      case 7: xEv = ssv_sweep_7(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
      default: xEv = ssv_sweep_8(dsq, L, pp->sbv, Q, q0, xEv, beginv, begin0); break;
    }
    q0 += w;
  }
  uint16_t xE = v_hmax(xEv), xJ;
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
  *ret_sc = orc_score_from_xj((uint8_t) xJ, tjb, om->base_b, om->scale_b);
  return ORC_eslOK;
}

/* Full MSV: the striped loop of msvfilter.c:112-212. */
static int port_msv(const uint8_t *dsq, int L, const orc_profile *om, const port_prof *pp, uint8_t tjb,
                    v16 *dp, uint8_t *ret_xj, float *ret_sc)
{
  const int Q = pp->Q;
  const v16 biasv = v_set1(om->bias_b), basev = v_set1(om->base_b), tecv = v_set1(om->tec_b);
  const v16 tjbmv = v_set1((uint8_t) ((int8_t) tjb + (int8_t) om->tbm_b));
  v16 xJv = v_set1(0), xBv = v_subs_u8(basev, tjbmv);
  for (int q = 0; q < Q; q++) dp[q] = v_set1(0);
  for (int i = 1; i <= L; i++) {
    const v16 *rsc = pp->rbv + (size_t) dsq[i] * Q;
    v16 xEv = v_set1(0);
    v16 mpv = v_shl1(dp[Q - 1]);
    for (int q = 0; q < Q; q++) {
      v16 sv = v_max_u8(mpv, xBv);
      sv = v_adds_u8(sv, biasv);
      sv = v_subs_u8(sv, rsc[q]);
      xEv = v_max_u8(xEv, sv);
      mpv = dp[q];
      dp[q] = sv;
    }
    const uint8_t xE = v_hmax(xEv);
    if ((int) xE + om->bias_b >= 255) { *ret_sc = INFINITY; *ret_xj = 255; return ORC_eslERANGE; }
    const v16 e = v_subs_u8(v_set1(xE), tecv);
    xJv = v_max_u8(xJv, e);
    xBv = v_subs_u8(v_max_u8(basev, xJv), tjbmv);
  }
  uint8_t xj = v_hmax(xJv);
  *ret_xj = xj;
  *ret_sc = orc_score_from_xj(xj, tjb, om->base_b, om->scale_b);
  return ORC_eslOK;
}

typedef struct {
  const orc_profile *om; const port_prof *pp; const uint8_t *res; const int64_t *off; int64_t n; double F1;
  int32_t *status; uint8_t *xj; float *sc; uint8_t *pass;
  int64_t next; pthread_mutex_t mu;
} port_batch_t;

static void *port_worker(void *arg)
{
  port_batch_t *b = (port_batch_t *) arg;
  int64_t maxL = 0;
  for (int64_t i = 0; i < b->n; i++) if (b->off[i + 1] - b->off[i] > maxL) maxL = b->off[i + 1] - b->off[i];
  uint8_t *dsq = malloc((size_t) maxL + 2);
  v16 *dp = NULL;
  if (posix_memalign((void **) &dp, 16, sizeof(v16) * b->pp->Q)) { free(dsq); return NULL; }
  for (;;) {
    int64_t lo, hi;
    pthread_mutex_lock(&b->mu);
    lo = b->next; hi = lo + 256 < b->n ? lo + 256 : b->n; b->next = hi;
    pthread_mutex_unlock(&b->mu);
    if (lo >= b->n) break;
    for (int64_t i = lo; i < hi; i++) {
      int L = (int) (b->off[i + 1] - b->off[i]);
      uint8_t xj = 0; float sc = 0.f; int st;
      if (L == 0) { if (b->status) b->status[i] = -1; if (b->pass) b->pass[i] = 0; continue; }
      dsq[0] = 255; memcpy(dsq + 1, b->res + b->off[i], (size_t) L); dsq[L + 1] = 255;
      uint8_t tjb = orc_tjb_b(b->om->scale_b, L);
      st = port_ssv(dsq, L, b->om, b->pp, tjb, &xj, &sc);
      if (st == ORC_eslENORESULT) st = port_msv(dsq, L, b->om, b->pp, tjb, dp, &xj, &sc);
      if (b->status) b->status[i] = st;
      if (b->xj) b->xj[i] = xj;
      if (b->sc) b->sc[i] = sc;
      if (b->pass) b->pass[i] = (uint8_t) orc_f1_pass(sc, L, b->om->mmu, b->om->mlambda, b->F1, NULL, NULL);
    }
  }
  free(dsq); free(dp);
  return NULL;
}

/* Batch over a concatenated sequence set with nthreads host threads
 * (<= 0: all online cores); outputs as orc_msv_batch. Returns threads used. */
int port_msv_batch(const orc_profile *om, const uint8_t *residues, const int64_t *off, int64_t n,
                   double F1, int nthreads, int32_t *status, uint8_t *xj, float *sc, uint8_t *pass)
{
  port_prof pp;
  if (port_prepare(om, &pp) != 0) return -1;
  port_batch_t b = { om, &pp, residues, off, n, F1, status, xj, sc, pass, 0 };
  pthread_mutex_init(&b.mu, NULL);
  if (nthreads <= 0) { long c = sysconf(_SC_NPROCESSORS_ONLN); nthreads = c > 0 ? (int) c : 1; }
  pthread_t *th = malloc(sizeof(pthread_t) * (size_t) nthreads);
  for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, port_worker, &b);
  for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(th);
  pthread_mutex_destroy(&b.mu);
  free(pp.sbv); free(pp.rbv);
  return nthreads;
}
