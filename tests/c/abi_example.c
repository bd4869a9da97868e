/* A C caller of the drop-in boundary: the calls a Fortran or C driver of HR-WENO makes, with
 * host arrays, no Python.  Prints the reconstruction of a pulse and the state after an
 * rktvd(3) integration of the 500-cell Burgers line (example/example1_burgers_1d_fv.f90 with
 * the Lax-Friedrichs flux) as "%.17g" values, one per line, after a tag line. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "hrweno_gpu.h"

#define CHECK(call)                                                         \
  do {                                                                      \
    int rc_ = (call);                                                       \
    if (rc_ != HRW_OK) {                                                    \
      fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, hrw_last_error()); \
      return 1;                                                             \
    }                                                                       \
  } while (0)

int main(int argc, char** argv) {
  const int numerics = argc > 1 ? atoi(argv[1]) : HRW_NUMERICS_STRICT;
  enum { NC = 500 };
  static double v[NC], vl[NC], vr[NC], u[NC];
  const double xmin = -5.0, xmax = 5.0, dx = (xmax - xmin) / NC;
  for (int i = 0; i < NC; ++i) {
    const double x = xmin + dx * (i + 0.5);
    v[i] = fabs(x) < 1.0 ? 1.0 : 0.0; /* a pulse (test/test_hrweno.f90's kind of input) */
    u[i] = exp(-x * x);                 /* example1's initial condition */
  }

  /* weno(ncells, k, eps) and reconstruct(v, vl, vr) */
  hrw_weno* w = NULL;
  CHECK(hrw_weno_create(NC, 3, 1e-6, NULL, &w));
  CHECK(hrw_weno_set_numerics(w, numerics));
  CHECK(hrw_weno_reconstruct(w, HRW_F64, HRW_MEM_HOST, v, vl, vr));
  CHECK(hrw_weno_destroy(w));

  /* rktvd(fu, neq, 3) with fu the example1 right-hand side, integrate(u, t, tout, dt) */
  hrw_problem p;
  hrw_problem_init(&p);
  p.kind = HRW_PROBLEM_FV1D;
  p.ncells[0] = NC;
  p.ncells[1] = 1;
  p.k = 3;
  p.eps = 1e-6;
  p.flux = HRW_FLUX_LAX_FRIEDRICHS;
  p.fn[0] = HRW_FN_BURGERS;
  p.alpha[0] = 1.0;
  p.bc[0] = HRW_BC_COPY;
  p.xmin[0] = xmin;
  p.xmax[0] = xmax;
  p.numerics = numerics;
  hrw_ode* ode = NULL;
  CHECK(hrw_rktvd_create(&p, NC, 3, HRW_F64, &ode));
  double t = 0.0;
  CHECK(hrw_integrate(ode, HRW_MEM_HOST, u, &t, 1.0, 1e-2, 1));
  int fevals = 0, istate = 0;
  long long nsteps = 0;
  int64_t ns = 0;
  CHECK(hrw_ode_info(ode, &fevals, &istate, &ns));
  nsteps = (long long)ns;
  CHECK(hrw_ode_destroy(ode));

  /* an invalid input returns a status and the reference's message, it does not abort */
  hrw_weno* bad = NULL;
  const int rc = hrw_weno_create(NC, 4, 1e-6, NULL, &bad);

  printf("t %.17g nsteps %lld fevals %d istate %d\n", t, nsteps, fevals, istate);
  printf("invalid_k %d %s\n", rc, hrw_last_error());
  printf("vl\n");
  for (int i = 0; i < NC; ++i) printf("%.17g\n", vl[i]);
  printf("vr\n");
  for (int i = 0; i < NC; ++i) printf("%.17g\n", vr[i]);
  printf("u\n");
  for (int i = 0; i < NC; ++i) printf("%.17g\n", u[i]);
  return 0;
}
