// batch_f32c.cu - the batched solver (batch.cu) in the compensated FP32 form (hrw_f32c.cuh):
// the same persistent grid of groups and the same queue of problems, each group advancing its
// problem through every step with the warp pass of the single-line compensated kernel.
//
// A step's stages run one copy of the pass with the stage kind as a run-time value, and the
// numerical flux is resolved once per problem (a template argument; Burgers or linear is a
// warp-uniform branch): per-stage and per-flux-kind copies of the pass inside one persistent
// kernel overflow the instruction cache, and its groups run different problems at once.  The
// arithmetic of every stage is that of the single-line kernel, so batched and single-line
// solves give the same bits.
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_batch.h"
#include "hrw_batch_dev.cuh"
#include "hrw_f32c.cuh"
#include "hrw_internal.h"

namespace hrw {

namespace {

constexpr int NT = kBatchThreads;

// ---- compensated FP32 batches ----------------------------------------------------------------
__device__ __forceinline__ void split_scalar(double x, float& hi, float& lo) {
  hi = __double2float_rn(x);
  lo = __double2float_rn(x - (double)hi);
}

// MS: an mstvd batch's sweep (the pass also takes the right-hand side and multistep stages)
template <int K, int G, int C, int FK, bool NU, bool MS = false>
__device__ __forceinline__ void f32c_sweep(const F32CArgs& a, int lt, int gid, int stage) {
  const int lane = lt & 31;
  const int warp_in_group = lt >> 5;
  for (int64_t base = 0; base < a.L.nc; base += (int64_t)G * C) {
    const int64_t wbase = base + (int64_t)warp_in_group * 32 * C;
    if (wbase < a.L.nc) f32c_pass<K, -1, C, FK, NU, MS>(a, wbase + (int64_t)lane * C, lane, stage);
  }
  group_sync<G>(gid);
}

// all steps of one problem in the increment form of the compensated kernels (stage1d_f32c.cu):
// the state ping-pongs between slots 0 and 1 and ends in slot 0
// FK: the problem's flux kind as flux_g_t takes it (4 or 5 here: the numerical flux fixed, the
// flux function chosen at run time), or -1 (resolved per call).  NU: a non-uniform line (its
// per-cell coefficients, widths and edges in P.fcnu, P.frw, P.fgst, P.fxe; FK = -1)
// the problem's line and time-step constants, as a single-line handle sets them up
template <bool NU>
__device__ __forceinline__ void problem_args(const BatchProblem& P, F32CArgs& a) {
  {
    a = F32CArgs{};
    a.eps = (float)P.eps;
    a.L.nc = P.nc;
    a.L.fn = P.fn;
    a.L.bc = P.bc;
    a.L.flux = P.flux;
    a.L.a = (float)P.a;
    a.L.b = (float)P.b;
    a.L.alpha = (float)P.alpha;
    a.L.xmin = (float)P.xmin;
    a.L.rx = (float)P.rx;
    a.L.gstep = (float)(P.b * P.rx);
    a.L.rw = nullptr;
    split_scalar(P.dt / P.rx, a.c_hi, a.c_lo);
    split_scalar(P.dt, a.dt_hi, a.dt_lo);
    a.lscale = (float)(1.0 / P.rx);
    if constexpr (NU) {  // as a single non-uniform line: dt L = dt (-dF / width)
      a.L.cnu = P.fcnu;
      a.L.rw = P.frw;
      a.L.gst = P.fgst;
      a.L.xe = P.fxe;
      split_scalar(P.dt, a.c_hi, a.c_lo);
      a.lscale = 1.0f;
    }
  }
}

template <int K, int G, int C, int FK, bool NU = false>
__device__ void run_problem_f32c(const BatchArgs& B, const BatchProblem& P, int lt, int gid,
                                 F32CArgs& a) {
  // a: this group's arguments in shared memory (registers stay free for the warp pass);
  // thread 0 of the group writes them between sweeps, each sweep ends with a group barrier
  float* const h0 = B.fhi[0] + P.off;
  float* const h1 = B.fhi[1] + P.off;
  float* const l0 = B.flo[0] + P.off;
  float* const l1 = B.flo[1] + P.off;
  float* const d1 = B.fd1 + P.off;
  float* const d2 = B.fd2 + P.off;
  if (lt == 0) problem_args<NU>(P, a);
  // the step's stages in order, each one sweep through the single call site below (one copy of
  // the pass serves them all): order 1: RK1; 2: E1, RK2B; 3: E1, RK3B, RK3C
  const int nst = B.order < 1 ? 1 : (B.order > 3 ? 3 : B.order);
  int slot = 0;
  for (int64_t n = 0; n < P.nsteps; ++n) {
    for (int k = 0; k < nst; ++k) {
      const int st = nst == 1 ? FC_RK1 : (k == 0 ? FC_E1 : (nst == 2 ? FC_RK2B : (k == 1 ? FC_RK3B : FC_RK3C)));
      if (lt == 0) {
        a.hi = slot ? h1 : h0, a.lo = slot ? l1 : l0;
        a.hi_out = slot ? h0 : h1, a.lo_out = slot ? l0 : l1;
        a.dv = k == 0 ? nullptr : (k == 1 ? d1 : d2);
        a.out = k == 0 ? d1 : d2;  // (the last stage writes the state pair instead)
      }
      group_sync<G>(gid);
      f32c_sweep<K, G, C, FK, NU>(a, lt, gid, st);
    }
    slot = 1 - slot;
  }
  if (slot == 1) {
    for (int64_t j = lt; j < P.nc; j += G) h0[j] = h1[j], l0[j] = l1[j];
    group_sync<G>(gid);
  }
}

// mstvd (src/hrweno_tvdode.f90:203-271) of one problem, as a single-line compensated mstvd
// handle runs it: the packed FP64 state split into the ring slot of the current level (slot 0
// on the first call, which then takes the four RK3 start steps, each after a right-hand side
// into the L ring), the multistep steps from slot to slot, and the final slot merged back into
// the packed state.  Ring slots u^m (hi, lo) in fring_h/fring_lo[m % 5], L(u^m) in
// fring_L[m % 4]; the start's stage increments in fd1, fd2.
template <int K, int G, int C, int FK, bool NU = false>
__device__ void run_problem_f32c_ms(const BatchArgs& B, const BatchProblem& P, int lt, int gid,
                                    F32CArgs& a) {
  float* H[5];
  float* Lo[5];
  float* Lr[4];
#pragma unroll
  for (int q = 0; q < 5; ++q) H[q] = B.fring_h[q] + P.off, Lo[q] = B.fring_lo[q] + P.off;
#pragma unroll
  for (int q = 0; q < 4; ++q) Lr[q] = B.fring_L[q] + P.off;
  float* const d1 = B.fd1 + P.off;
  float* const d2 = B.fd2 + P.off;
  double* const u = B.u + P.off;
  if (lt == 0) problem_args<NU>(P, a);
  int64_t level = P.start ? 0 : P.level;
  int cur = (int)(level % 5);
  for (int64_t j = lt; j < P.nc; j += G) {
    const double x = u[j];
    const float h = __double2float_rn(x);
    H[cur][j] = h;
    Lo[cur][j] = __double2float_rn(x - (double)h);
  }
  group_sync<G>(gid);
  if (P.start) {  // the RK3 start (:236-249): L(u^m) into the ring, then an RK3 step to u^{m+1}
    for (int m = 0; m < 4; ++m) {
      for (int k = 0; k < 4; ++k) {
        const int st = k == 0 ? FC_RHS : k == 1 ? FC_E1 : k == 2 ? FC_RK3B : FC_RK3C;
        if (lt == 0) {
          a.hi = H[m], a.lo = Lo[m];
          a.dv = k < 2 ? nullptr : (k == 2 ? d1 : d2);
          a.out = k == 0 ? Lr[m] : (k == 1 ? d1 : d2);
          a.hi_out = H[m + 1], a.lo_out = Lo[m + 1];
        }
        group_sync<G>(gid);
        f32c_sweep<K, G, C, FK, NU, true>(a, lt, gid, st);
      }
    }
    level = 4;
  }
  for (int64_t n = 0; n < P.nsteps; ++n, ++level) {  // (:252-268)
    const int c0 = (int)(level % 5), c1 = (int)((level + 1) % 5);  // c1 holds u^{m-4}
    float* const lm = Lr[level % 4];                                  // holds L(u^{m-4})
    if (lt == 0) {
      a.hi = H[c0], a.lo = Lo[c0], a.dv = nullptr;
      a.hi_out = H[c1], a.lo_out = Lo[c1];
      a.hi4 = H[c1], a.lo4 = Lo[c1], a.l4 = lm, a.lout = lm;
    }
    group_sync<G>(gid);
    f32c_sweep<K, G, C, FK, NU, true>(a, lt, gid, FC_MS);
  }
  cur = (int)(level % 5);
  for (int64_t j = lt; j < P.nc; j += G) u[j] = (double)H[cur][j] + (double)Lo[cur][j];
  group_sync<G>(gid);
}

// MS: the kernel of mstvd batches (a kernel of its own, so that the rktvd batches' pass
// carries no multistep code)
template <int G, int C, bool NU = false, bool MS = false>
__global__ void __launch_bounds__(NT, C == 4 ? 3 : 2) batch_f32c_kernel(BatchArgs B) {
  static_assert(NT % G == 0 && G % 32 == 0 && NT / G <= 15, "groups of whole warps");
  constexpr int GPB = NT / G;
  __shared__ int s_pid[GPB];
  __shared__ F32CArgs s_args[GPB];
  const int gid = threadIdx.x / G, lt = threadIdx.x % G;
  for (;;) {
    if (lt == 0) s_pid[gid] = atomicAdd(B.counter, 1);
    group_sync<G>(gid);
    const int pid = s_pid[gid];
    group_sync<G>(gid);
    if (pid >= B.nprob) break;
    const BatchProblem P = B.probs[B.order_idx[pid]];
    if (P.nsteps <= 0 && !(MS && P.start)) continue;
    // one copy of the pass per (k, numerical flux); Burgers or linear is a uniform branch
    const bool god = P.flux != HRW_FLUX_LAX_FRIEDRICHS;
    F32CArgs& a = s_args[gid];
#define HRW_RUN(K_, FK_, NU_)                                                        \
  do {                                                                               \
    if constexpr (MS) run_problem_f32c_ms<K_, G, C, FK_, NU_>(B, P, lt, gid, a);     \
    else run_problem_f32c<K_, G, C, FK_, NU_>(B, P, lt, gid, a);                     \
  } while (0)
    if constexpr (NU) {  // one copy of the general pass per k
      if (P.k == 3) HRW_RUN(3, -1, true);
      else if (P.k == 2) HRW_RUN(2, -1, true);
      else HRW_RUN(1, -1, true);
    } else if (P.k == 3) {
      if (!god) HRW_RUN(3, 4, false);
      else HRW_RUN(3, 5, false);
    } else if (P.k == 2) {
      if (!god) HRW_RUN(2, 4, false);
      else HRW_RUN(2, 5, false);
    } else {
      HRW_RUN(1, -1, false);
    }
#undef HRW_RUN
  }
}

template <int G, int C, bool NU = false>
int occupancy_f32(bool ms) {
  int n = 0;
  if (ms) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_f32c_kernel<G, C, NU, true>, NT, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_f32c_kernel<G, C, NU, false>, NT, 0);
  return n;
}

template <int G, int C, bool NU = false>
cudaError_t launch_f32(const BatchArgs& B, int blocks, cudaStream_t s) {
  if (B.method == 1) batch_f32c_kernel<G, C, NU, true><<<blocks, NT, 0, s>>>(B);
  else batch_f32c_kernel<G, C, NU, false><<<blocks, NT, 0, s>>>(B);
  return cudaGetLastError();
}

}  // namespace

const BatchShape kBatchShapesF32[kNumBatchShapesF32] = {{64, 4}, {128, 4}, {256, 4}};

int batch_f32_blocks_per_sm(int shape, bool ms) {
  switch (shape) {
    case 0: return occupancy_f32<64, 4>(ms);
    case 1: return occupancy_f32<128, 4>(ms);
    default: return occupancy_f32<256, 4>(ms);
  }
}

int batch_f32c_nu_blocks_per_sm(bool ms) { return occupancy_f32<kBatchNuGroup, 4, true>(ms); }

cudaError_t launch_batch_f32c_nu(const BatchArgs& B, int blocks, cudaStream_t s) {
  if (B.nprob <= 0) return cudaSuccess;
  return launch_f32<kBatchNuGroup, 4, true>(B, blocks, s);
}

cudaError_t launch_batch_f32c(const BatchArgs& B, int shape, int blocks, cudaStream_t s) {
  if (B.nprob <= 0) return cudaSuccess;
  switch (shape) {
    case 0: return launch_f32<64, 4>(B, blocks, s);
    case 1: return launch_f32<128, 4>(B, blocks, s);
    case 2: return launch_f32<256, 4>(B, blocks, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace hrw
