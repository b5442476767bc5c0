/* vit_oracle.h -- CPU oracle for the ViterbiFilter stage (TEST INFRASTRUCTURE ONLY).
 * See vit_oracle.c. */
#ifndef VIT_ORACLE_H
#define VIT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_VIT_OK     0
#define ORC_VIT_ERANGE 16

/* special states and transitions of P7_OPROFILE's xw (src/impl_sse/impl_sse.h:73-74) */
enum { ORC_XE = 0, ORC_XN = 1, ORC_XJ = 2, ORC_XC = 3 };
enum { ORC_MOVE = 0, ORC_LOOP = 1 };

/* The ViterbiFilter part of a P7_OPROFILE (impl_sse.h:88-96), striped as the
 * reference stores it: Q8 = max(2, ceil(M/8)); twv holds, per vector q, the
 * 7 vectors BM MM IM DM MD MI II, then the Q8 DD vectors; rwv[x][q]; element
 * z of vector q is node q+1+z*Q8. */
typedef struct {
  int            M, Q8, Kp;
  float          scale_w, nj;
  int16_t        base_w, ddbound_w;
  int16_t        xw[4][2];
  const int16_t *twv;
  const int16_t *rwv;
} orc_vprofile;

/* xw after p7_oprofile_ReconfigRestLength(om, L) */
void  orc_vit_specials(const orc_vprofile *vp, int L, int16_t xw[4][2]);
/* p7_ViterbiFilter's score from the final xC at length L */
float orc_vit_score(const orc_vprofile *vp, int L, int xC);
/* p7_ViterbiFilter(dsq, L, om, ox, &sc) after p7_oprofile_ReconfigLength(om, L):
 * eslOK or eslERANGE (*ret_sc = +inf); *ret_xc the final xC (32767 on overflow). */
int   orc_vit_filter(const uint8_t *dsq, int L, const orc_vprofile *vp, float *ret_sc, int *ret_xc);

#ifdef __cplusplus
}
#endif
#endif
