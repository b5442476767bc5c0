/* vit_oracle.c -- CPU oracle for the ViterbiFilter stage (TEST INFRASTRUCTURE ONLY).
 *
 * A scalar C restatement of HMMER 3.1b1's p7_ViterbiFilter
 * (src/impl_sse/vitfilter.c:84-250) in model-node order instead of the
 * reference's 8-lane striping, reading the reference's own striped int16
 * profile (vf_conversion, src/impl_sse/p7_oprofile.c:653-760) with the
 * per-length specials of p7_oprofile_ReconfigRestLength (:944-962). It is the
 * checker for the CUDA ViterbiFilter; the product library never links it.
 *
 * Parity pin: tests/golden/vit_*.vres hold p7_ViterbiFilter's own statuses
 * and scores (oracle/ref/refgen.c "vit"/"vitfile"); the oracle reproduces
 * every one (tests/test_vit_oracle.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include "vit_oracle.h"

/* wordify(): src/impl_sse/p7_oprofile.c:527-534 */
static int16_t wordify(float scale_w, float sc) {
  sc = roundf(scale_w * sc);
  if (sc >= 32767.0) return 32767;
  else if (sc <= -32768.0) return -32768;
  else return (int16_t) sc;
}

static int sat16(int v) { return v > 32767 ? 32767 : (v < -32768 ? -32768 : v); }
static int imax(int a, int b) { return a > b ? a : b; }

/* node k (1..8*Q8) sits in striped vector q = (k-1) % Q8, element z = (k-1) / Q8 */
static int twv_at(const orc_vprofile *vp, int t, int k) {
  const int q = (k - 1) % vp->Q8, z = (k - 1) / vp->Q8;
  if (t == 7) return vp->twv[(7 * vp->Q8 + q) * 8 + z];      /* DD vectors follow the 7-per-q block */
  return vp->twv[(q * 7 + t) * 8 + z];                        /* BM MM IM DM MD MI II */
}
static int rwv_at(const orc_vprofile *vp, int x, int k) {
  const int q = (k - 1) % vp->Q8, z = (k - 1) / vp->Q8;
  return vp->rwv[(x * vp->Q8 + q) * 8 + z];
}

void orc_vit_specials(const orc_vprofile *vp, int L, int16_t xw[4][2]) {
  for (int s = 0; s < 4; s++) for (int t = 0; t < 2; t++) xw[s][t] = vp->xw[s][t];
  const float pmove = (2.0f + vp->nj) / ((float) L + 2.0f + vp->nj);
  const int16_t mv = wordify(vp->scale_w, logf(pmove));
  xw[ORC_XN][ORC_MOVE] = xw[ORC_XC][ORC_MOVE] = xw[ORC_XJ][ORC_MOVE] = mv;
}

float orc_vit_score(const orc_vprofile *vp, int L, int xC) {
  int16_t xw[4][2];
  if (xC <= -32768) return -INFINITY;
  orc_vit_specials(vp, L, xw);
  float sc = (float) xC + (float) xw[ORC_XC][ORC_MOVE] - (float) vp->base_w;
  sc /= vp->scale_w;
  sc -= 3.0;
  return sc;
}

int orc_vit_filter(const uint8_t *dsq, int L, const orc_vprofile *vp, float *ret_sc, int *ret_xc) {
  const int Np = 8 * vp->Q8;
  int16_t xw[4][2];
  orc_vit_specials(vp, L, xw);
  int *Mp = malloc(sizeof(int) * (Np + 2)), *Ip = malloc(sizeof(int) * (Np + 2)), *Dp = malloc(sizeof(int) * (Np + 2));
  int *Mn = malloc(sizeof(int) * (Np + 2)), *In = malloc(sizeof(int) * (Np + 2)), *Dn = malloc(sizeof(int) * (Np + 2));
  for (int k = 0; k <= Np + 1; k++) Mp[k] = Ip[k] = Dp[k] = Mn[k] = In[k] = Dn[k] = -32768;   /* [0]: no node 0 */
  int16_t xN = vp->base_w, xB = (int16_t) (xN + xw[ORC_XN][ORC_MOVE]), xJ = -32768, xC = -32768, xE = -32768;
  int status = ORC_VIT_OK;
  for (int i = 1; i <= L; i++) {
    const int x = dsq[i];
    int xe = -32768, dmax = -32768;
    Dn[1] = -32768;
    for (int k = 1; k <= Np; k++) {
      /* M(i,k): B->M, M->M, I->M, D->M from node k-1 of the previous row, then the emission */
      int sv = sat16(xB + twv_at(vp, 0, k));
      sv = imax(sv, sat16(Mp[k - 1] + twv_at(vp, 1, k)));
      sv = imax(sv, sat16(Ip[k - 1] + twv_at(vp, 2, k)));
      sv = imax(sv, sat16(Dp[k - 1] + twv_at(vp, 3, k)));
      sv = sat16(sv + rwv_at(vp, x, k));
      xe = imax(xe, sv);
      Mn[k] = sv;
      /* M->D into node k+1 (its Dmax counts even past the last node) */
      const int dc = sat16(sv + twv_at(vp, 4, k));
      dmax = imax(dmax, dc);
      if (k < Np) Dn[k + 1] = dc;
      /* I(i,k): M->I, I->I from node k of the previous row */
      In[k] = imax(sat16(Mp[k] + twv_at(vp, 5, k)), sat16(Ip[k] + twv_at(vp, 6, k)));
    }
    xE = (int16_t) xe;
    if (xE >= 32767) { status = ORC_VIT_ERANGE; break; }
    xN = (int16_t) (xN + xw[ORC_XN][ORC_LOOP]);
    xC = (int16_t) imax(xC + xw[ORC_XC][ORC_LOOP], xE + xw[ORC_XE][ORC_MOVE]);
    xJ = (int16_t) imax(xJ + xw[ORC_XJ][ORC_LOOP], xE + xw[ORC_XE][ORC_LOOP]);
    xB = (int16_t) imax(xJ + xw[ORC_XJ][ORC_MOVE], xN + xw[ORC_XN][ORC_MOVE]);
    /* lazy F (vitfilter.c:197-235): D->D paths only when they could beat B->M on the next row */
    if (dmax + vp->ddbound_w > xB)
      for (int k = 1; k < Np; k++) Dn[k + 1] = imax(Dn[k + 1], sat16(Dn[k] + twv_at(vp, 7, k)));
    int *t;
    t = Mp; Mp = Mn; Mn = t;
    t = Ip; Ip = In; In = t;
    t = Dp; Dp = Dn; Dn = t;
  }
  free(Mp); free(Ip); free(Dp); free(Mn); free(In); free(Dn);
  if (ret_xc) *ret_xc = status == ORC_VIT_OK ? xC : 32767;
  if (ret_sc) *ret_sc = status == ORC_VIT_OK ? orc_vit_score(vp, L, xC) : INFINITY;
  return status;
}
