// stage1d.cu - fused 1D stage kernel: WENO reconstruction + numerical flux + conservative
// difference + TVD stage combine, one read of the line and one write per cell.
//
// Follows, for one stage of the reference's time loop:
//   weno_reconstruct            src/hrweno_weno.f90:129-219
//   lax_friedrichs / godunov    src/hrweno_fluxes.f90:22-76
//   1D right-hand side + BCs    example/example1_burgers_1d_fv.f90:93-107
//   rktvd / mstvd stage update  src/hrweno_tvdode.f90:136-171,257
//
// Layout: one block owns a tile of NT*C consecutive cells.  The tile plus a k-cell halo on
// each side is staged in shared memory (ghost cells replicate v(1) and v(nc),
// src/hrweno_weno.f90:172-173).  Each thread reconstructs C consecutive cells from a register
// window; the two block-edge cells whose reconstruction the neighbouring tiles own are
// recomputed by two lanes.  Fluxes at the thread's C+1 interfaces use the neighbours'
// edge values through shared memory, then each cell's update is written once.
#include <cmath>
#include <type_traits>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"
#include "hrw_stage.cuh"

namespace hrw {

double fast_flux_scale(int flux, int fn) {
  if (flux == HRW_FLUX_LAX_FRIEDRICHS) return fn == HRW_FN_LINEAR ? 0.5 : 0.25;
  return fn == HRW_FN_LINEAR ? 1.0 : 0.5;
}

std::atomic<int> g_upwind_enabled{1};

bool positive_velocity(const LineArgs& L, double rel_margin) {
  if (!g_upwind_enabled.load(std::memory_order_relaxed)) return false;
  if (L.fn != HRW_FN_LINEAR) return false;
  // g(x_e) = a + b*(xmin + rx*e) is monotone in e under any rounding of its three operations,
  // so its minimum over the interfaces e = 0..nc sits at an end; the margin stays far above
  // the rounding differences between the host and the device evaluation orders
  for (int64_t e : {(int64_t)0, (int64_t)L.nc}) {
    const double x = L.xmin + L.rx * (double)e;
    const double g = L.a + L.b * x;
    if (!(g > rel_margin * (std::fabs(L.a) + std::fabs(L.b * x)))) return false;
  }
  return true;
}

// Stage combine for cell j.  dF = F_{j+1/2} - F_{j-1/2} in the flux form of the mode.
template <int ST, bool STRICT, class T>
__device__ __forceinline__ void combine(const StageArgsT<T>& a, const LineArgsT<T>& L, int64_t j,
                                        T v, T dF) {
  if constexpr (STRICT) {
    const T w = L.width ? L.width[j] : L.rx;
    combine_strict<ST>(a, j, v, rn_div(-dF, w));  // vdot = -(F_i - F_{i-1})/width (ex1:107)
  } else {
    combine_fast<ST>(a, j, v, dF, L.rws ? L.rws[j] : L.rws0);
  }
}

// --------------------------------------------------------------------------------------------
// The kernel.  R = double (HRW_F64, FAST or STRICT) or float (HRW_F32, reference order only).
// --------------------------------------------------------------------------------------------
template <class R, int K, int ST, bool STRICT, int NT, int C>
__global__ void __launch_bounds__(NT) stage1d_kernel(StageArgsT<R> a) {
  static_assert(STRICT || std::is_same<R, double>::value, "float lines take the reference order");
  constexpr int T = NT * C;
  constexpr int H = K;  // halo: cell j needs v(j-K .. j+K) through its two interfaces
  // the tile with one padding element after every 8: thread t's window starts at cell 8t, and
  // unpadded those windows (64 bytes apart) would fall on two bank groups (16-way conflicts)
  constexpr int TP = T + 2 * H;
  __shared__ R sv[TP + TP / 8 + 1];
  __shared__ R sL[NT + 1];  // sL[t] = vl of thread t's first cell; sL[NT] = vl(s+T)
  __shared__ R sR[NT + 1];  // sR[t+1] = vr of thread t's last cell; sR[0] = vr(s-1)
  const LineArgsT<R>& L = a.L;
  const int64_t nc = L.nc;
  const int64_t s = a.cell0 + (int64_t)blockIdx.x * T;
  const int tid = threadIdx.x;
  // launched as a programmatic dependent of the previous kernel on the stream: wait here, before
  // any memory access, until that kernel has completed and its writes are visible (its launch
  // and this grid's scheduling overlap its tail)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // a grid of at most one wave (every block resident from the start) lets the next stage's
  // grid launch at once, its blocks queueing behind this one's; larger grids trigger it as
  // their blocks exit, so that waiting blocks take no slots from their later waves
  if ((int)gridDim.x <= a.wave_blocks) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

  for (int q = tid; q < T + 2 * H; q += NT) {
    int64_t g = s - H + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    sv[q + (q >> 3)] = a.v[g];
  }
  __syncthreads();

  // ---- reconstruction of the thread's C cells --------------------------------------------
  const int l0 = tid * C;  // first local cell; its centre is tile cell H + l0
  R vl[C], vr[C];
  R w[C + 2 * K];
#pragma unroll
  for (int q = 0; q < C + 2 * K; ++q) w[q] = sv[l0 + q + ((l0 + q) >> 3)];  // v(j0 - K + q)
  if constexpr (STRICT) {
#pragma unroll
    for (int c = 0; c < C; ++c) recon_strict<K>(&w[K + c], a.eps, vl[c], vr[c]);
  } else {
    recon_fast<K, C>(w, a.eps, vl, vr);
  }
  sL[tid] = vl[0];
  sR[tid + 1] = vr[C - 1];
  // block-edge cells s-1 (vr) and s+T (vl), one lane each of the last warp
  if (tid >= NT - 2) {
    const int which = tid - (NT - 2);  // 0: cell s-1, 1: cell s+T
    const int lc = which == 0 ? H - 1 : H + T;
    R p[2 * K - 1];  // the cell's stencil, lc - (K-1) .. lc + K-1
#pragma unroll
    for (int q = 0; q < 2 * K - 1; ++q) {
      const int i = lc - (K - 1) + q;
      p[q] = sv[i + (i >> 3)];
    }
    R el, er;
    if constexpr (STRICT) recon_strict<K>(&p[K - 1], a.eps, el, er);
    else recon_fast_one<K>(&p[K - 1], a.eps, el, er);
    if (which == 0) sR[0] = er;
    else sL[NT] = el;
  }
  __syncthreads();

  // ---- fluxes at the C+1 interfaces and the stage update ---------------------------------
  const int64_t j0 = s + l0;
  if (j0 >= nc) return;
  R F[C + 1];
  F[0] = numflux<STRICT>(L, sR[tid], vl[0], j0);
#pragma unroll
  for (int c = 1; c < C; ++c) F[c] = numflux<STRICT>(L, vr[c - 1], vl[c], j0 + c);
  F[C] = numflux<STRICT>(L, vr[C - 1], sL[tid + 1], j0 + C);

  if constexpr (ST == ST_RECON) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t j = j0 + c;
      if (j < nc) { a.out[j] = vl[c]; a.lout[j] = vr[c]; }
    }
    return;
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t j = j0 + c;
      if (j >= nc) break;
      const R dF = flux_diff<STRICT>(L, j, F[c], F[c + 1], vr[c]);
      combine<ST, STRICT>(a, L, j, w[K + c], dF);
    }
  }
}

template <class R, int K, int ST, bool STRICT, int NT, int C>
static cudaError_t launch_shape(const StageArgsT<R>& a, cudaStream_t s) {
  const int64_t span = a.ncell > 0 ? a.ncell : (int64_t)a.L.nc - a.cell0;
  const int64_t nblk = (span + NT * C - 1) / (NT * C);
  if (nblk <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)nblk);
  cfg.blockDim = dim3(NT);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  StageArgsT<R> b = a;
  b.wave_blocks = device_sms() * 4;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, stage1d_kernel<R, K, ST, STRICT, NT, C>, b);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Tile shape by line length: 1024-cell tiles (128 threads x 8 cells) once there are at least
// two tiles per SM; shorter lines use 256- or 64-cell tiles so that their few cells still
// spread over many SMs (each SM retires only about 2 FP64 instructions per clock).
template <class R, int K, int ST, bool STRICT>
static cudaError_t launch_k(const StageArgsT<R>& a, cudaStream_t s) {
  const int64_t nc = a.L.nc, sms = device_sms();
  if (nc >= 2 * sms * 1024) return launch_shape<R, K, ST, STRICT, 128, 8>(a, s);
  if (nc >= 2 * sms * 256) return launch_shape<R, K, ST, STRICT, 64, 4>(a, s);
  return launch_shape<R, K, ST, STRICT, 32, 2>(a, s);
}

template <class R, int K, bool STRICT>
static cudaError_t launch_st(const StageArgsT<R>& a, int stage, cudaStream_t s) {
  switch (stage) {
    case ST_RHS: return launch_k<R, K, ST_RHS, STRICT>(a, s);
    case ST_EULER: return launch_k<R, K, ST_EULER, STRICT>(a, s);
    case ST_RK2B: return launch_k<R, K, ST_RK2B, STRICT>(a, s);
    case ST_RK3B: return launch_k<R, K, ST_RK3B, STRICT>(a, s);
    case ST_RK3C: return launch_k<R, K, ST_RK3C, STRICT>(a, s);
    case ST_MS: return launch_k<R, K, ST_MS, STRICT>(a, s);
    case ST_RECON: return launch_k<R, K, ST_RECON, STRICT>(a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_stage1d(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s) {
  if (a.L.nc <= 0) return cudaSuccess;
  using D = double;
  if (k == 1) return strict ? launch_st<D, 1, true>(a, stage, s) : launch_st<D, 1, false>(a, stage, s);
  if (k == 2) return strict ? launch_st<D, 2, true>(a, stage, s) : launch_st<D, 2, false>(a, stage, s);
  return strict ? launch_st<D, 3, true>(a, stage, s) : launch_st<D, 3, false>(a, stage, s);
}

cudaError_t launch_stage1d(const StageArgs32& a, int k, int stage, cudaStream_t s) {
  if (a.L.nc <= 0) return cudaSuccess;
  if (k == 1) return launch_st<float, 1, true>(a, stage, s);
  if (k == 2) return launch_st<float, 2, true>(a, stage, s);
  return launch_st<float, 3, true>(a, stage, s);
}

}  // namespace hrw
