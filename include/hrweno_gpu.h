/*
 * hrweno_gpu.h - C ABI of the GB300 (sm_103a) implementation of HR-WENO's hot path:
 * WENO reconstruction, the monotone numerical fluxes and the TVD Runge-Kutta /
 * multistep stage updates, fused into one CUDA kernel per stage.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and returns a
 * status code (HRW_OK == 0).  Where the Fortran reference aborts with `error stop`,
 * this library returns HRW_EINVAL and keeps the reference's message, readable through
 * hrw_last_error().  Handles are not thread-safe; each handle owns one CUDA stream, created
 * blocking, so that its work is ordered after earlier work of the legacy default stream
 * (device arrays that the caller filled there are complete before a stage kernel reads them).
 *
 * Reference interfaces replaced (paths inside HugoMVale/HR-WENO):
 *   weno(ncells,k,eps,xedges)          src/hrweno_weno.f90:48-50,54-127
 *   weno%reconstruct(v,vl,vr)          src/hrweno_weno.f90:44,129-219
 *   lax_friedrichs / godunov           src/hrweno_fluxes.f90:22-45,47-76
 *   rktvd(fu,neq,order)                src/hrweno_tvdode.f90:59-61,69-95
 *   mstvd(fu,neq)                      src/hrweno_tvdode.f90:63-65,180-201
 *   ode%integrate(u,t,tout,dt,itask)   src/hrweno_tvdode.f90:97-178,203-271
 *   the user right-hand side `fu`      example/example1_burgers_1d_fv.f90:72-109,
 *                                      example/example2_pbe_2d_fv.f90:73-129
 * The reference stores the right-hand side as a procedure pointer
 * (src/hrweno_tvdode.f90:16,50-57).  A GPU stage kernel cannot call back into host code,
 * so the right-hand side is described by an hrw_problem instead.
 */
#ifndef HRWENO_GPU_H
#define HRWENO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
enum {
  HRW_OK = 0,
  HRW_EINVAL = 1,   /* invalid input; message as in the reference's `msg` field */
  HRW_ECUDA = 2,    /* a CUDA runtime call failed */
  HRW_ESTATE = 3,   /* handle is in an error state (reference: istate < 1) */
  HRW_ETIMEOUT = 4, /* a bounded device-side wait ran out; the context stays usable */
  HRW_ENOMEM = 5    /* device allocation failed */
};

/* ---- element type and memory space of user arrays -------------------------------- */
/* HRW_F64:  the FP64 method itself; user arrays are doubles.
 * HRW_F32:  what a REAL32 build of the reference computes (rk = real32, src/hrweno_kinds.F90:9-10):
 *           user arrays are floats; eps, the grid, cnu, the state, every stage and the time
 *           t, tout, dt are held in FP32 and computed in the reference's operation order (the
 *           numerics field is ignored), so results are bit-identical to an FP32 CPU build of
 *           the reference's formulas.  Integrators, reconstruct and hrw_rhs; all problem kinds.
 *           The *t of hrw_integrate is rounded to FP32 on entry and returned exactly.
 * HRW_F32C: compensated FP32 bulk precision (FV1D and FV2D): user arrays stay doubles; inside,
 *           the state is a float pair hi + lo and the right-hand side is evaluated in FP32 in
 *           difference form (compensated neighbour differences, flux differences relative
 *           to each cell's own flux, two-sum accumulation of u); t stays FP64. */
enum { HRW_F64 = 0, HRW_F32 = 1, HRW_F32C = 2 };
/* Memory space of the arrays a call receives: host arrays are copied in and out (page-locked
 * ones asynchronously); device arrays are used in place.  Other values return HRW_EINVAL. */
enum { HRW_MEM_HOST = 0, HRW_MEM_DEVICE = 1 };

/* ---- problem descriptor: the right-hand side L(u) -------------------------------- */
enum {
  HRW_PROBLEM_FV1D = 1,       /* example1: WENO + flux + conservative difference on a line */
  HRW_PROBLEM_FV2D = 2,       /* example2: dimension-by-dimension sweeps, x1 fastest */
  HRW_PROBLEM_LINEAR_ODE = 3  /* u_i' = a_i u_i (test/test_tvdode.f90:107-111) */
};
enum { HRW_FLUX_LAX_FRIEDRICHS = 0, HRW_FLUX_GODUNOV = 1 };
/* physical flux f(u, x): BURGERS = u^2/2; LINEAR = (a + b*x) * u, x = interface coordinate;
 * BURGERS_LINEAR = u^2/2 + (a + b*x) * u (convex: Burgers carried by a velocity field; the FP64
 * paths, not HRW_F32C) */
enum { HRW_FN_BURGERS = 0, HRW_FN_LINEAR = 1, HRW_FN_BURGERS_LINEAR = 2 };
/* domain-boundary fluxes (per dimension):
 *   COPY        F_{1/2} = F_{3/2}, F_{nc+1/2} = F_{nc-1/2}  (example1...f90:103-104)
 *   ZERO        F_{1/2} = F_{nc+1/2} = 0                   (example2...f90:117-120)
 *   ZERO_INFLOW F_{1/2} = 0, F_{nc+1/2} = f(vr(nc)): no inflow, free outflow */
enum { HRW_BC_COPY = 0, HRW_BC_ZERO = 1, HRW_BC_ZERO_INFLOW = 2 };
/* FAST: the FP64 method with the fewest FP64 instructions (product-form WENO weights, one
 * reciprocal per cell, fused multiply-adds); agrees with the reference to rounding level.
 * STRICT: the reference's operation order with no fused multiply-add and true divisions;
 * bit-identical to a non-fused CPU build of the reference's formulas.
 * MIXED: the FP64 state and stage combines with the right-hand side evaluated in difference
 * form on the FP32 pipe: FP64 neighbour differences split into float pairs, the linear-weight
 * part of the reconstruction in float-pair precision, the WENO weights' deviations from the
 * linear weights in FP32, stage increments stored as float pairs.  A warp whose data would let
 * the FP32 parts move dt L by more than 2^-53 max|u| per stage (steep or under-resolved
 * data, the line ends, max|u| outside [2^-40, 2^60]) runs the FAST arithmetic instead; so does
 * everything the MIXED kernel does not cover.  Covered: rktvd integrators of FV1D lines of at
 * least 65536 uniform cells, k = 2 or 3, Lax-Friedrichs flux, Burgers or linear advection at
 * constant speed (b = 0); eps >= 1e-8.  Agrees with the reference to the same 1e-12 (normwise
 * relative) bar as FAST. */
enum { HRW_NUMERICS_FAST = 0, HRW_NUMERICS_STRICT = 1, HRW_NUMERICS_MIXED = 2 };

typedef struct hrw_problem {
  int32_t kind;       /* HRW_PROBLEM_* */
  int32_t ncells[2];  /* FV1D: ncells[0]; FV2D: [nc1, nc2], u((j-1)*nc1+i) as example2:124 */
  int32_t k;          /* WENO order 2k-1, 1 <= k <= 3 */
  double eps;         /* WENO smoothing factor, eps > epsilon */
  int32_t flux;       /* HRW_FLUX_* (same numerical flux in every dimension) */
  int32_t fn[2];      /* HRW_FN_* per dimension */
  double coef_a[2];   /* LINEAR: a per dimension */
  double coef_b[2];   /* LINEAR: b per dimension */
  double alpha[2];    /* Lax-Friedrichs alpha = max|f'(u)| per dimension */
  int32_t bc[2];      /* HRW_BC_* per dimension */
  double xmin[2];     /* uniform grid as grid1%linear: edges(i) = xmin + (xmax-xmin)/nc*i */
  double xmax[2];
  const double* width[2]; /* optional host array(nc) of cell widths; NULL: (xmax-xmin)/nc */
  const double* rates;    /* LINEAR_ODE: host array(neq) of rates a_i */
  int32_t numerics;       /* HRW_NUMERICS_* */
  /* optional host array(nc+1) of cell edges of a non-uniform line, per dimension (FV1D and
   * FV2D; HRW_F64, HRW_F32 and HRW_F32C handles, batches and the adjoint, not the
   * allocation-free steps): the WENO coefficients become cnu(xedges) as weno(ncells, k, eps,
   * xedges) builds them (src/hrweno_weno.f90:100-104,221-297), the widths edges(i) - edges(i-1)
   * and the flux's x the edges themselves; xmin/xmax are then unused and width[] must be NULL.
   * NULL: uniform grid. */
  const double* xedges[2];
} hrw_problem;

/* Fill *p with the defaults: FV1D, k=3, eps=1e-6, Lax-Friedrichs, Burgers, alpha=1,
 * COPY boundaries, grid [0,1], FAST numerics.  ncells must still be set. */
void hrw_problem_init(hrw_problem* p);

/* ---- errors ----------------------------------------------------------------------- */
/* Message of the last failing call on this host thread ("" if none). */
const char* hrw_last_error(void);

/* ---- WENO reconstruction (weno type) ---------------------------------------------- */
typedef struct hrw_weno hrw_weno;

/* weno(ncells, k, eps, xedges): xedges is NULL (uniform grid) or a host array(ncells+1).
 * k <= 0 selects the default k = 3; eps <= 0 selects the default 1e-6
 * (the reference's optional arguments, src/hrweno_weno.f90:60-69). */
int hrw_weno_create(int ncells, int k, double eps, const double* xedges, hrw_weno** out);
/* Select HRW_NUMERICS_FAST (default) or HRW_NUMERICS_STRICT for later reconstructions. */
int hrw_weno_set_numerics(hrw_weno* w, int numerics);
/* w%reconstruct(v, vl, vr): arrays of ncells elements of `dtype` (HRW_F64, or HRW_F32 for the
 * REAL32 reconstruction, which needs eps > epsilon(1.0_real32)) in memory space `mem`. */
int hrw_weno_reconstruct(hrw_weno* w, int dtype, int mem, const void* v, void* vl, void* vr);
/* Copy the non-uniform coefficients cnu(0:k-1,-1:k-1,1:nc), Fortran order, to the host. */
int hrw_weno_cnu(const hrw_weno* w, double* cnu_host);
int hrw_weno_destroy(hrw_weno* w);

/* ---- TVD ODE integrators (rktvd / mstvd types) ------------------------------------ */
typedef struct hrw_ode hrw_ode;

/* rktvd(fu, neq, order): order 1..3; dtype HRW_F64 (the method itself), HRW_F32 (a REAL32
 * build) or HRW_F32C (compensated FP32 bulk precision, FV1D and FV2D problems; the user array
 * stays FP64). */
int hrw_rktvd_create(const hrw_problem* p, int neq, int order, int dtype, hrw_ode** out);
/* mstvd(fu, neq): 5-step, 3rd-order TVD multistep with an RK3 start. */
int hrw_mstvd_create(const hrw_problem* p, int neq, int dtype, hrw_ode** out);
/* ode%integrate(u, t, tout, dt[, itask]): u (neq elements of the ode's dtype) is updated
 * in place, *t advances like the reference (it stops at the first step with t > tout).  A dt
 * too small to change t (t + dt == t in the handle's precision) returns HRW_EINVAL, where the
 * reference would never return.
 * itask: 1 normal integration until tout, 2 single step.  A CUDA failure part-way leaves u
 * undefined and puts the handle in the error state (istate = -1; later calls return
 * HRW_ESTATE), as the reference's integrate refuses to continue after an error. */
int hrw_integrate(hrw_ode* ode, int mem, void* u, double* t, double tout, double dt, int itask);
/* fevals, istate (1 first call, 2 later calls, -1 error) and steps taken so far. */
int hrw_ode_info(const hrw_ode* ode, int* fevals, int* istate, int64_t* nsteps);
/* integrate calls of 4 or more steps replay a CUDA graph of captured steps (the stage
 * launches of up to 64 consecutive rktvd steps, or 20/60 mstvd steps), recorded once per
 * device array, dt, stream and step count, so a driver loop over output times captures once
 * and replays on every later call; enable = 0 launches every stage directly.  Both give the
 * same results bit for bit.  Default: enabled. */
int hrw_ode_set_graphs(hrw_ode* ode, int enable);
/* rktvd integrate calls on a uniform FV1D line of 6 to 4096 cells (FP64, FAST or STRICT) run all
 * their steps in one launch of one thread-block cluster of up to 16 CTAs that keeps the line in
 * distributed shared memory, one cluster barrier per stage, instead of a launch per stage: such
 * lines are bound by launch latency.  The same results bit for bit.  enable = 0 launches stage by
 * stage (with graphs as set above).  Default: enabled. */
int hrw_ode_set_cluster(hrw_ode* ode, int enable);
/* Run this handle's kernels on `stream` (a cudaStream_t); NULL restores its own stream. */
int hrw_ode_set_stream(hrw_ode* ode, void* stream);
int hrw_ode_destroy(hrw_ode* ode);

/* ---- right-hand side alone (fu of the reference's driver) -------------------------- */
/* vdot = L(v) at time t for problem p, both arrays device pointers of doubles
 * (LINEAR_ODE: neq = ncells[0]); dtype HRW_F64, HRW_F32C to evaluate L in the compensated
 * FP32 form (FV1D and FV2D problems), or HRW_F32 with float arrays (a REAL32 build). */
int hrw_rhs(const hrw_problem* p, int dtype, double t, const void* v, void* vdot, void* stream);

/* ---- batches of independent 1D problems ------------------------------------------- */
/* A batch holds nprob independent FV1D problems on uniform or non-uniform grids
 * given as xedges (each its own rktvd(fu,
 * neq, order) of the reference, src/hrweno_tvdode.f90:69-178, with its own ncells, k, flux,
 * flux function, alpha and boundaries; all share `order`, the dtype (HRW_F64, or HRW_F32C:
 * the compensated FP32 form, states still packed as FP64) and one numerics mode).  Their states are packed in one array: problem i occupies cells
 * [offsets[i], offsets[i] + ncells_i) of the layout returned by hrw_batch_layout
 * (offsets[nprob] is the packed length).  One call advances every problem with one
 * persistent launch per size class, the classes running concurrently. */
typedef struct hrw_batch hrw_batch;
int hrw_batch_create(const hrw_problem* problems, int nprob, int order, int dtype, hrw_batch** out);
/* A batch of mstvd(fu_i, neq_i) solves (src/hrweno_tvdode.f90:180-271), HRW_F64 or HRW_F32C (the
 * compensated form of a single mstvd handle, its history in float pairs): each problem keeps
 * its 5-step history between calls and runs the RK3 start (4 steps; the 4 extra rhs calls of the
 * reference) on its first call that takes a step.  hrw_batch_integrate follows mstvd_integrate
 * (itask is ignored, as the reference's mstvd has none); hrw_batch_advance runs the start on a
 * problem's first call and then nsteps multistep steps; hrw_batch_tune probes RK3 steps of the
 * same stage code and leaves the histories as they are. */
int hrw_batch_create_mstvd(const hrw_problem* problems, int nprob, int dtype, hrw_batch** out);
/* offsets[0 .. nprob] of the packed layout */
int hrw_batch_layout(const hrw_batch* b, int64_t* offsets);
/* Per problem i: integrate(u_i, t[i], tout, dt[i], itask) with the reference's stopping rule
 * (itask 1: to the first t > tout; 2: one step); t[] is updated.  u: packed state in `mem`. */
int hrw_batch_integrate(hrw_batch* b, int mem, double* u, double* t, double tout, const double* dt,
                        int itask);
/* Exactly nsteps steps of every problem (nsteps integrate calls with itask = 2 each) in one
 * persistent launch per size class; t[] is advanced by the reference's t = t + dt. */
int hrw_batch_advance(hrw_batch* b, int mem, double* u, double* t, const double* dt, int64_t nsteps);
/* Autotuner: time probe_steps steps of each size class with every candidate (group size,
 * cells per thread) shape on a scratch copy of u and keep the fastest; cache_path (nullable)
 * is a text cache keyed by device and class. */
int hrw_batch_tune(hrw_batch* b, int mem, const double* u, const double* dt, int probe_steps,
                   const char* cache_path);
/* shapes[2c], shapes[2c+1]: group threads and cells per thread of size class c (3 classes:
 * < 512, < 4096, >= 4096 cells); steps_done[i]: steps taken by problem i so far (nullable). */
int hrw_batch_info(const hrw_batch* b, int* shapes, int64_t* steps_done);
/* Run on `stream` (a cudaStream_t; NULL restores the handle's own stream). */
int hrw_batch_set_stream(hrw_batch* b, void* stream);
int hrw_batch_destroy(hrw_batch* b);

/* ---- discrete adjoint --------------------------------------------------------------- */
/* No counterpart in the reference.  Gradient of J = 0.5 ||u(T) - target||^2 with respect to
 * the initial state u0, where u(T) is nsteps rktvd(order 3) steps of dt of an FV1D problem
 * with the global Lax-Friedrichs flux at fixed alpha (eps > 0 keeps the WENO weights smooth).
 * The state holds nseg independent problems of p->ncells[0] cells each (packed; with
 * nseg > 1, ncells must be a multiple of 8); J has one entry per problem.  The reverse sweep
 * recomputes the forward from checkpoints taken every `checkpoint_every` steps (about
 * sqrt(nsteps) is the usual choice).  The pass that records a segment also records each
 * cell's WENO-map derivatives (a WENO tape of 20 doubles per cell and stage for k = 3, 12 for
 * k = 2) when they fit in 80% of the free device memory, so the reverse pass does not
 * recompute them.  checkpoint_every = 0 picks the first that fits that budget: the whole
 * trajectory with the WENO tape, sqrt(nsteps) segments with it, the whole trajectory's
 * states without it, sqrt(nsteps) segments without it.  A non-uniform line (p->xedges[0],
 * the same edges for every problem of the state) keeps no WENO tape: the reverse pass
 * recomputes each cell's map with its own coefficients; width[] is refused. */
typedef struct hrw_adjoint hrw_adjoint;
int hrw_adjoint_create(const hrw_problem* p, int nseg, int checkpoint_every, hrw_adjoint** out);
/* grad = dJ/du0 (nseg * ncells doubles), J[nseg]; arrays in memory space `mem` (J on the host) */
int hrw_adjoint_gradient(hrw_adjoint* a, int mem, const double* u0, const double* target, double dt,
                         int64_t nsteps, double* J, double* grad);
/* grad = d <lambda_T, u(T)> / du0 for any lambda_T: the vector-Jacobian product of the whole
 * forward map (what an automatic-differentiation framework calls backward) */
int hrw_adjoint_vjp(hrw_adjoint* a, int mem, const double* u0, const double* lambda_T, double dt,
                    int64_t nsteps, double* grad);
/* The forward solve alone: u(T) (nullable) and, when target is not NULL, J[nseg] */
int hrw_adjoint_forward(hrw_adjoint* a, int mem, const double* u0, const double* target, double dt,
                        int64_t nsteps, double* J, double* uT);
/* forward steps (initial pass plus recompute) and the checkpoint interval of the last
 * gradient call; either pointer may be NULL */
int hrw_adjoint_info(const hrw_adjoint* a, int64_t* forward_steps, int64_t* checkpoint_every);
/* Device memory the last gradient call kept for its segment: the states (3E + 1 of them) and
 * the WENO tape (0 when it did not fit: the reverse pass then recomputes each cell's WENO map
 * from the states); either pointer may be NULL */
int hrw_adjoint_tape_info(const hrw_adjoint* a, int64_t* state_bytes, int64_t* weno_tape_bytes);
int hrw_adjoint_set_stream(hrw_adjoint* a, void* stream);
int hrw_adjoint_destroy(hrw_adjoint* a);

/* ---- RK3 steps that allocate no device memory -------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device memory: a
 * framework whose caching allocator already owns the whole device, or a step loop that must
 * not pay the implicit device synchronisation of cudaMalloc/cudaFree.  Runs nsteps rktvd
 * order-3 steps of a uniform-grid FV1D problem (width[0] must be NULL) on the device array
 * u (ncells[0] doubles), in place, on `stream` (a cudaStream_t; NULL is the legacy default
 * stream), and returns without waiting for the GPU.  The two RK stage arrays live in one
 * fixed buffer inside the library (2 * HRW_NOALLOC_MAX_CELLS doubles, 16 MiB, held by every
 * GPU that loads the library until the process exits); larger lines are rejected with
 * HRW_EINVAL.  A call looks up that buffer's device address when its stream is not being
 * captured; a captured call reuses the address found by the last uncaptured call on the
 * device, so make the first call on a device (and the first after a device reset) outside any
 * stream capture.  All calls share the buffer: calls whose work overlaps on the GPU (other
 * streams, other threads) race and give wrong results; calls on one stream are ordered and
 * safe.  On HRW_ECUDA some steps may have been queued: the contents of u are then undefined.
 * Same kernels and operation order as hrw_integrate, so the results are bit-identical to an
 * rktvd(order 3) handle's. */
#define HRW_NOALLOC_MAX_CELLS (1 << 20)
int hrw_rktvd3_steps_noalloc(const hrw_problem* p, double* u, double dt, int nsteps, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HRWENO_GPU_H */
