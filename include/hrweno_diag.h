/*
 * hrweno_diag.h - diagnostics of the GB300 library (no counterpart in the reference).
 *
 * The stage kernels of the FP64 path are bound by the FP64 pipe, not by HBM; one call
 * measures that pipe on the current device so that a benchmark can report the kernel's
 * fraction of it next to its HBM roofline fraction.  The others expose internals to the tests:
 * the 2D kernels' bounded wait, the FAST path's reciprocal, the MIXED kernel's choice
 * between its FP32 and FP64 paths, and the 2D kernels' upwind specialisation.
 */
#ifndef HRWENO_DIAG_H
#define HRWENO_DIAG_H
#ifdef __cplusplus
extern "C" {
#endif

/* DFMA instructions retired per second by the whole device (independent FMA chains on every
 * SM), and FFMA likewise; either pointer may be NULL. */
int hrw_diag_fma_rates(double* dfma_per_second, double* ffma_per_second);

/* Poll limit of the 2D stage kernels' first wait for their TMA tile copies, on the current
 * device (FP64 and compensated FP32 kernels).  A block whose wait runs out flags its handle,
 * waits for its copies with the default bound and leaves; hrw_integrate / hrw_rhs then return
 * HRW_ETIMEOUT.  A small limit (0: no poll at all) lets a test drive that path to expiry
 * without any copy going missing.  polls < 0 restores the default (2^20 polls). */
int hrw_diag_set_tile_wait_limit(int polls);

/* Reciprocals by the FAST path's rcp_fast (an rcp.approx.f64 seed and one cubic
 * Newton-Raphson step) and by IEEE division (__ddiv_rn(1, x)), for n device doubles x:
 * fast[i], exact[i].  Device pointers; synchronous. */
int hrw_diag_rcp(const double* x, double* fast, double* exact, int n);

/* MIXED numerics: enable = 0 sends every warp of the MIXED stage kernel through its FP64 path
 * (the FAST arithmetic), 1 restores the default; the setting holds for the current device.
 * Tests use it to check the FP64 path on its own. */
int hrw_diag_mixed_soft(int enable);
/* Warps of the MIXED stage kernel, away from the line ends, that took the FP64 path since the
 * last reset (*count; reset != 0 clears the counter), on the current device. */
int hrw_diag_mixed_hard_warps(unsigned long long* count, int reset);
/* enable = 0: handles created afterwards do not take the upwind specialisation of the 2D
 * kernels (Godunov's flux of g(x) u with g > 0 everywhere reconstructs only the left state of
 * each interface); 1 restores it.  Process-wide.  Tests use it to check that both give the
 * same bits. */
int hrw_diag_upwind(int enable);

#ifdef __cplusplus
}
#endif
#endif /* HRWENO_DIAG_H */
