/*
 * hrweno_diag.h - diagnostics of the GB300 library (no counterpart in the reference).
 *
 * The stage kernels of the FP64 path are bound by the FP64 pipe, not by HBM; this call
 * measures that pipe on the current device so that a benchmark can report the kernel's
 * fraction of it next to its HBM roofline fraction.
 */
#ifndef HRWENO_DIAG_H
#define HRWENO_DIAG_H
#ifdef __cplusplus
extern "C" {
#endif

/* DFMA instructions retired per second by the whole device (independent FMA chains on every
 * SM), and FFMA likewise; either pointer may be NULL. */
int hrw_diag_fma_rates(double* dfma_per_second, double* ffma_per_second);

#ifdef __cplusplus
}
#endif
#endif /* HRWENO_DIAG_H */
