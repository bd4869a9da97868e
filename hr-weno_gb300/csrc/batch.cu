// batch.cu - many independent 1D problems of uneven size in one persistent launch.
//
// Each problem is one reference solve: its own rktvd(fu, neq, order) object integrated with its
// own dt (src/hrweno_tvdode.f90:69-178), or its own mstvd(fu, neq) (:180-271), whose fu is the example1 right-hand side
// (example/example1_burgers_1d_fv.f90:72-109) with its own flux, k and alpha.  Here all of them
// advance together:
//
//  * a persistent grid of thread groups (a group is 32..256 threads) claims problems from an
//    atomic queue ordered by decreasing cost (cells x steps), so the longest solves start first;
//  * a group runs all of its problem's steps inside the launch: for every stage it sweeps the
//    line in passes of G*C cells (each warp reconstructs 32*C consecutive cells from register
//    windows, neighbouring lanes exchange the edge states by shuffles), then the group meets at a
//    barrier before the next stage reads the stage output.  A problem's three arrays (u, u1, u2)
//    are touched by one SM for thousands of consecutive stages, so they stay in L1/L2;
//  * problems are split by size into classes, each class with the group size and cells per
//    thread that the autotuner measured fastest for it (capi_batch.cu).
//
// Stage arithmetic is the shared FP64 code of the single-problem kernels (hrw_device.cuh,
// hrw_stage.cuh), FAST or STRICT, so a batched solve matches the single-problem path.
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_batch.h"
#include "hrw_device.cuh"
#include "hrw_batch_dev.cuh"
#include "hrw_internal.h"
#include "hrw_stage.cuh"

namespace hrw {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int NT = kBatchThreads;


// One warp-pass of stage ST over cells j0 .. j0 + C - 1 of this lane (all 32 lanes call it).
// NU: a non-uniform line (a.cnu, L.width, L.rws, L.xe): each cell reconstructs with its own
// coefficients and divides by its own width, as stage1d_nu.cu.
template <int K, int ST, bool STRICT, int C, bool NU>
__device__ __forceinline__ void stage_pass(const StageArgs& a, const LineArgs& L, int64_t j0,
                                           int lane) {
  constexpr int NCF = K * (K + 1);  // coefficients per cell
  const int64_t nc = L.nc;
  double w[C + 2 * K];  // w[q] = v(j0 - K + q), ghosts replicate v(1), v(nc)
#pragma unroll
  for (int q = 0; q < C + 2 * K; ++q) {
    int64_t g = j0 - K + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    w[q] = a.v[g];
  }
  double vl[C], vr[C];
  if constexpr (NU) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t jc = j0 + c < nc ? j0 + c : nc - 1;
      recon_nu<K, STRICT>(&w[K + c], a.cnu + NCF * jc, a.eps, vl[c], vr[c]);
    }
  } else if constexpr (STRICT) {
#pragma unroll
    for (int c = 0; c < C; ++c) recon_strict<K>(&w[K + c], a.eps, vl[c], vr[c]);
  } else {
    recon_fast<K, C>(w, a.eps, vl, vr);
  }
  // states of the cells just outside this lane's range: from the neighbouring lanes, and for
  // lanes 0 / 31 (the warp's ends) reconstructed here; every lane runs the same edge code so
  // that the warp stays converged (cell j0-1 uses w[0 .. 2K-2], cell j0+C uses w[C+1 ..])
  double e[2 * K - 1];
#pragma unroll
  for (int q = 0; q < 2 * K - 1; ++q) e[q] = lane == 31 ? w[C + 1 + q] : w[q];
  double el, er;
  if constexpr (NU) {
    int64_t je = lane == 31 ? j0 + C : j0 - 1;
    je = je < 0 ? 0 : (je >= nc ? nc - 1 : je);
    recon_nu<K, STRICT>(&e[K - 1], a.cnu + NCF * je, a.eps, el, er);
  } else if constexpr (STRICT) {
    recon_strict<K>(&e[K - 1], a.eps, el, er);
  } else {
    recon_fast_one<K>(&e[K - 1], a.eps, el, er);
  }
  const double vr_up = __shfl_up_sync(FULL, vr[C - 1], 1);
  const double vl_dn = __shfl_down_sync(FULL, vl[0], 1);
  const double vr_m = lane == 0 ? er : vr_up;
  const double vl_p = lane == 31 ? el : vl_dn;
  double F[C + 1];
  F[0] = numflux<STRICT>(L, vr_m, vl[0], j0);
#pragma unroll
  for (int c = 1; c < C; ++c) F[c] = numflux<STRICT>(L, vr[c - 1], vl[c], j0 + c);
  F[C] = numflux<STRICT>(L, vr[C - 1], vl_p, j0 + C);
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int64_t j = j0 + c;
    if (j >= nc) break;
    const double dF = flux_diff<STRICT>(L, j, F[c], F[c + 1], vr[c]);
    if constexpr (STRICT) combine_strict<ST>(a, j, w[K + c], __ddiv_rn(-dF, NU ? L.width[j] : L.rx));
    else combine_fast<ST>(a, j, w[K + c], dF, NU ? L.rws[j] : L.rws0);
  }
}

template <int K, int ST, bool STRICT, int G, int C, bool NU>
__device__ __forceinline__ void stage_sweep(const StageArgs& a, const LineArgs& L, int lt, int gid) {
  const int lane = lt & 31;
  const int warp_in_group = lt >> 5;
  for (int64_t base = 0; base < L.nc; base += (int64_t)G * C) {
    const int64_t wbase = base + (int64_t)warp_in_group * 32 * C;
    if (wbase < L.nc) stage_pass<K, ST, STRICT, C, NU>(a, L, wbase + (int64_t)lane * C, lane);
  }
  group_sync<G>(gid);
}

// the line of problem P as the stage code sees it (with its non-uniform arrays when NU)
template <bool NU>
__device__ __forceinline__ LineArgs problem_line(const BatchProblem& P) {
  LineArgs L{};
  L.nc = P.nc;
  L.fn = P.fn;
  L.bc = P.bc;
  L.flux = P.flux;
  L.a = P.a;
  L.b = P.b;
  L.alpha = P.alpha;
  L.xmin = P.xmin;
  L.rx = P.rx;
  L.rws0 = P.rws0;
  if constexpr (NU) {
    L.width = P.width;
    L.rws = P.rws;
    L.xe = P.xe;
  }
  return L;
}

// all steps of one problem
template <int K, bool STRICT, int G, int C, bool NU>
__device__ void run_problem(const BatchArgs& B, const BatchProblem& P, int lt, int gid) {
  const LineArgs L = problem_line<NU>(P);
  double* u = B.u + P.off;
  double* u1 = B.u1 + P.off;
  double* u2 = B.u2 + P.off;
  StageArgs a{};
  a.eps = P.eps;
  a.dt = P.dt;
  if constexpr (NU) a.cnu = P.cnu;
  for (int64_t n = 0; n < P.nsteps; ++n) {
    if (B.order == 1) {  // u' = u + dt L(u): out of place, then copied back by the next pass
      a.v = u, a.u = u, a.out = u1;
      stage_sweep<K, ST_EULER, STRICT, G, C, NU>(a, L, lt, gid);
      for (int64_t j = lt; j < L.nc; j += G) u[j] = u1[j];
      group_sync<G>(gid);
      continue;
    }
    a.v = u, a.u = u, a.out = u1;  // (src/hrweno_tvdode.f90:148-150 / 161-163)
    stage_sweep<K, ST_EULER, STRICT, G, C, NU>(a, L, lt, gid);
    if (B.order == 2) {  // (:151-152)
      a.v = u1, a.u = u, a.out = u;
      stage_sweep<K, ST_RK2B, STRICT, G, C, NU>(a, L, lt, gid);
      continue;
    }
    a.v = u1, a.u = u, a.out = u2;  // (:164-165)
    stage_sweep<K, ST_RK3B, STRICT, G, C, NU>(a, L, lt, gid);
    a.v = u2, a.u = u, a.out = u;  // (:166-167)
    stage_sweep<K, ST_RK3C, STRICT, G, C, NU>(a, L, lt, gid);
  }
}

// mstvd (src/hrweno_tvdode.f90:203-271) of one problem: the packed state u is copied into its
// ring slot, the RK3 start (:236-249) runs on the problem's first call, then P.nsteps
// multistep steps (:252-268), each reading u^m, u^{m-4}, L(u^{m-4}) and writing u^{m+1} and
// L(u^m) over the two oldest entries; the newest state is copied back to u.
template <int K, bool STRICT, int G, int C, bool NU>
__device__ void run_problem_ms(const BatchArgs& B, const BatchProblem& P, int lt, int gid) {
  const LineArgs L = problem_line<NU>(P);
  double* u = B.u + P.off;
  double* u1 = B.u1 + P.off;
  double* u2 = B.u2 + P.off;
  double* R[5];
  double* Lr[4];
#pragma unroll
  for (int q = 0; q < 5; ++q) R[q] = B.ring_u[q] + P.off;
#pragma unroll
  for (int q = 0; q < 4; ++q) Lr[q] = B.ring_l[q] + P.off;
  StageArgs a{};
  a.eps = P.eps;
  a.dt = P.dt;
  if constexpr (NU) a.cnu = P.cnu;
  int64_t level = P.level;
  double* cur = R[P.start ? 0 : level % 5];
  for (int64_t j = lt; j < L.nc; j += G) cur[j] = u[j];
  group_sync<G>(gid);
  if (P.start) {  // u^m and L(u^m), m = 0..3, by RK3 steps (the start's rhs calls)
    for (int m = 0; m < 4; ++m) {
      double* um = R[m % 5];
      a.v = um, a.u = um, a.out = Lr[m % 4];
      stage_sweep<K, ST_RHS, STRICT, G, C, NU>(a, L, lt, gid);
      a.v = um, a.u = um, a.out = u1;
      stage_sweep<K, ST_EULER, STRICT, G, C, NU>(a, L, lt, gid);
      a.v = u1, a.u = um, a.out = u2;
      stage_sweep<K, ST_RK3B, STRICT, G, C, NU>(a, L, lt, gid);
      a.v = u2, a.u = um, a.out = R[(m + 1) % 5];
      stage_sweep<K, ST_RK3C, STRICT, G, C, NU>(a, L, lt, gid);
    }
    level = 4;
  }
  for (int64_t n = 0; n < P.nsteps; ++n, ++level) {
    double* um = R[level % 5];
    double* un = R[(level + 1) % 5];  // holds u^{m-4}, overwritten with u^{m+1}
    double* lm = Lr[level % 4];       // holds L(u^{m-4}), overwritten with L(u^m)
    a.v = um, a.u = um, a.out = un, a.lout = lm, a.uo4 = un, a.lo4 = lm;
    stage_sweep<K, ST_MS, STRICT, G, C, NU>(a, L, lt, gid);
  }
  cur = R[level % 5];
  for (int64_t j = lt; j < L.nc; j += G) u[j] = cur[j];
  group_sync<G>(gid);
}

// NU: a launch of the batch's non-uniform lines (the uniform ones run in the tuned launches of
// their size classes), one shape for all of them
template <bool STRICT, int G, int C, bool NU>
__global__ void __launch_bounds__(NT, 1) batch_kernel(BatchArgs B) {
  static_assert(NT % G == 0 && G % 32 == 0 && NT / G <= 15, "groups of whole warps");
  constexpr int GPB = NT / G;
  __shared__ int s_pid[GPB];
  const int gid = threadIdx.x / G, lt = threadIdx.x % G;
  for (;;) {
    if (lt == 0) s_pid[gid] = atomicAdd(B.counter, 1);
    group_sync<G>(gid);
    const int pid = s_pid[gid];
    group_sync<G>(gid);  // every lane has read s_pid before lane 0 claims again
    if (pid >= B.nprob) break;
    const BatchProblem P = B.probs[B.order_idx[pid]];
    if (P.nsteps <= 0 && !P.start) continue;
    if (B.method == 1) {
      if (P.k == 3) run_problem_ms<3, STRICT, G, C, NU>(B, P, lt, gid);
      else if (P.k == 2) run_problem_ms<2, STRICT, G, C, NU>(B, P, lt, gid);
      else run_problem_ms<1, STRICT, G, C, NU>(B, P, lt, gid);
    } else {
      if (P.k == 3) run_problem<3, STRICT, G, C, NU>(B, P, lt, gid);
      else if (P.k == 2) run_problem<2, STRICT, G, C, NU>(B, P, lt, gid);
      else run_problem<1, STRICT, G, C, NU>(B, P, lt, gid);
    }
  }
}

template <bool STRICT, int G, int C, bool NU = false>
cudaError_t launch_shape(const BatchArgs& B, int blocks, cudaStream_t s) {
  batch_kernel<STRICT, G, C, NU><<<blocks, NT, 0, s>>>(B);
  return cudaGetLastError();
}

template <bool STRICT, int G, int C, bool NU = false>
int occupancy() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<STRICT, G, C, NU>, NT, 0);
  return n;
}

}  // namespace

// The kernels of one numerics mode over every shape, and the non-uniform kernels.  The three
// compile as separate objects, HRW_PART = 0 (FAST), 1 (STRICT), 2 (non-uniform lines), in
// parallel; part 0 also holds the dispatch.  Built without HRW_PART, the file holds all.
template <bool STRICT>
int batch_occupancy(int shape) {
  switch (shape) {
    case 0: return occupancy<STRICT, 32, 2>();
    case 1: return occupancy<STRICT, 32, 4>();
    case 2: return occupancy<STRICT, 32, 8>();
    case 3: return occupancy<STRICT, 128, 4>();
    case 4: return occupancy<STRICT, 128, 8>();
    default: return occupancy<STRICT, 256, 8>();
  }
}

template <bool STRICT>
cudaError_t batch_launch(const BatchArgs& B, int shape, int blocks, cudaStream_t s) {
  switch (shape) {
    case 0: return launch_shape<STRICT, 32, 2>(B, blocks, s);
    case 1: return launch_shape<STRICT, 32, 4>(B, blocks, s);
    case 2: return launch_shape<STRICT, 32, 8>(B, blocks, s);
    case 3: return launch_shape<STRICT, 128, 4>(B, blocks, s);
    case 4: return launch_shape<STRICT, 128, 8>(B, blocks, s);
    case 5: return launch_shape<STRICT, 256, 8>(B, blocks, s);
  }
  return cudaErrorInvalidValue;
}

// the non-uniform lines: 128-thread groups, 4 cells per thread and pass
template <bool STRICT>
int batch_nu_occupancy() { return occupancy<STRICT, 128, 4, true>(); }
template <bool STRICT>
cudaError_t batch_nu_launch(const BatchArgs& B, int blocks, cudaStream_t s) {
  return launch_shape<STRICT, 128, 4, true>(B, blocks, s);
}

extern template int batch_occupancy<false>(int);
extern template int batch_occupancy<true>(int);
extern template cudaError_t batch_launch<false>(const BatchArgs&, int, int, cudaStream_t);
extern template cudaError_t batch_launch<true>(const BatchArgs&, int, int, cudaStream_t);
extern template int batch_nu_occupancy<false>();
extern template int batch_nu_occupancy<true>();
extern template cudaError_t batch_nu_launch<false>(const BatchArgs&, int, cudaStream_t);
extern template cudaError_t batch_nu_launch<true>(const BatchArgs&, int, cudaStream_t);
#if !defined(HRW_PART) || HRW_PART == 0
template int batch_occupancy<false>(int);
template cudaError_t batch_launch<false>(const BatchArgs&, int, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 1
template int batch_occupancy<true>(int);
template cudaError_t batch_launch<true>(const BatchArgs&, int, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 2
template int batch_nu_occupancy<false>();
template int batch_nu_occupancy<true>();
template cudaError_t batch_nu_launch<false>(const BatchArgs&, int, cudaStream_t);
template cudaError_t batch_nu_launch<true>(const BatchArgs&, int, cudaStream_t);
#endif

#if !defined(HRW_PART) || HRW_PART == 0
const BatchShape kBatchShapes[kNumBatchShapes] = {{32, 2}, {32, 4}, {32, 8}, {128, 4}, {128, 8}, {256, 8}};

int batch_blocks_per_sm(int shape, bool strict) {
  return strict ? batch_occupancy<true>(shape) : batch_occupancy<false>(shape);
}

cudaError_t launch_batch(const BatchArgs& B, int shape, bool strict, int blocks, cudaStream_t s) {
  if (B.nprob <= 0) return cudaSuccess;
  return strict ? batch_launch<true>(B, shape, blocks, s) : batch_launch<false>(B, shape, blocks, s);
}

int batch_nu_blocks_per_sm(bool strict) {
  return strict ? batch_nu_occupancy<true>() : batch_nu_occupancy<false>();
}

cudaError_t launch_batch_nu(const BatchArgs& B, bool strict, int blocks, cudaStream_t s) {
  if (B.nprob <= 0) return cudaSuccess;
  return strict ? batch_nu_launch<true>(B, blocks, s) : batch_nu_launch<false>(B, blocks, s);
}
#endif

}  // namespace hrw
