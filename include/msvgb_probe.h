/* msvgb_probe.h -- measurement helpers of the benchmark (libmsvgb_probe.so).
 *
 * Not part of the MSV filter and with no counterpart in the reference: short
 * kernels that measure, on the GPU they run on and at its current clock, the
 * peaks the benchmark's rooflines are quoted against. Each returns eslOK (0)
 * or eslESYS (12) with a message from msvgb_probe_last_error(). */
#ifndef MSVGB_PROBE_H
#define MSVGB_PROBE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Sustained rate of independent 32-bit integer max/xor instructions over all
 * SMs (ops/s): the integer-pipe roofline, one DP cell = one packed 32-bit op. */
int msvgb_measure_int_peak(int device, double *ops_per_second);
/* Sustained shared-memory read bandwidth over all SMs (bytes/s): conflict-free
 * 16-byte loads by every thread, the bound of table-driven DP rows. */
int msvgb_measure_smem_peak(int device, double *bytes_per_second);
const char *msvgb_probe_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
