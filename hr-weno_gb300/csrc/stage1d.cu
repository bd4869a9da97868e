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
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"

namespace hrw {

double fast_flux_scale(int flux, int fn) {
  if (flux == HRW_FLUX_LAX_FRIEDRICHS) return fn == HRW_FN_BURGERS ? 0.25 : 0.5;
  return fn == HRW_FN_BURGERS ? 0.5 : 1.0;
}

// --------------------------------------------------------------------------------------------
// Numerical fluxes.  e = edge index of the interface (x = xmin + rx*e, grid1%right).
// --------------------------------------------------------------------------------------------
// FAST: returns F / fast_flux_scale(flux, fn).
__device__ __forceinline__ double flux_fast(const LineArgs& L, double vm, double vp, int64_t e) {
  if (L.fn == HRW_FN_BURGERS) {
    if (L.flux == HRW_FLUX_LAX_FRIEDRICHS)  // 4F = vm^2 + vp^2 - 2 alpha (vp - vm)
      return fma(-2.0 * L.alpha, vp - vm, fma(vp, vp, vm * vm));
    const double fm = vm * vm, fp = vp * vp;  // 2F
    return vm <= vp ? fmin(fm, fp) : fmax(fm, fp);
  }
  double g = L.a;
  if (L.b != 0.0) g = fma(L.b, fma(L.rx, (double)e, L.xmin), L.a);
  if (L.flux == HRW_FLUX_LAX_FRIEDRICHS)  // 2F = (g + alpha) vm + (g - alpha) vp
    return fma(g + L.alpha, vm, (g - L.alpha) * vp);
  const double fm = g * vm, fp = g * vp;  // F
  return vm <= vp ? fmin(fm, fp) : fmax(fm, fp);
}
// FAST physical flux f(v) at edge e, same scaling as flux_fast.
__device__ __forceinline__ double phys_fast(const LineArgs& L, double v, int64_t e) {
  const double s = L.flux == HRW_FLUX_LAX_FRIEDRICHS ? 2.0 : 1.0;
  if (L.fn == HRW_FN_BURGERS) return s * (v * v);
  double g = L.a;
  if (L.b != 0.0) g = fma(L.b, fma(L.rx, (double)e, L.xmin), L.a);
  return s * (g * v);
}

// STRICT: reference order (src/hrweno_fluxes.f90:43,67-74; example1...f90:111-122).
__device__ __forceinline__ double phys_strict(const LineArgs& L, double v, int64_t e) {
  if (L.fn == HRW_FN_BURGERS) return __ddiv_rn(__dmul_rn(v, v), 2.0);
  const double x = __dadd_rn(L.xmin, __dmul_rn(L.rx, (double)e));
  return __dmul_rn(__dadd_rn(L.a, __dmul_rn(L.b, x)), v);
}
__device__ __forceinline__ double flux_strict(const LineArgs& L, double vm, double vp, int64_t e) {
  const double fm = phys_strict(L, vm, e), fp = phys_strict(L, vp, e);
  if (L.flux == HRW_FLUX_LAX_FRIEDRICHS)
    return __ddiv_rn(__dsub_rn(__dadd_rn(fm, fp), __dmul_rn(L.alpha, __dsub_rn(vp, vm))), 2.0);
  if (vm <= vp) return fm < fp ? fm : fp;
  return fm > fp ? fm : fp;
}

template <bool STRICT>
__device__ __forceinline__ double numflux(const LineArgs& L, double vm, double vp, int64_t e) {
  if constexpr (STRICT) return flux_strict(L, vm, vp, e);
  else return flux_fast(L, vm, vp, e);
}
template <bool STRICT>
__device__ __forceinline__ double physflux(const LineArgs& L, double v, int64_t e) {
  if constexpr (STRICT) return phys_strict(L, v, e);
  else return phys_fast(L, v, e);
}

// --------------------------------------------------------------------------------------------
// Stage combine for cell j.  dF = F_{j+1/2} - F_{j-1/2} in the flux form of the mode.
// --------------------------------------------------------------------------------------------
template <int ST, bool STRICT>
__device__ __forceinline__ void combine(const StageArgs& a, const LineArgs& L, int64_t j,
                                        double v, double dF) {
  if constexpr (STRICT) {
    const double w = L.width ? L.width[j] : L.rx;
    const double udot = __ddiv_rn(-dF, w);  // vdot = -(F_i - F_{i-1})/width  (example1:107)
    const double dt = a.dt;
    if constexpr (ST == ST_RHS) {
      a.out[j] = udot;
    } else if constexpr (ST == ST_EULER) {
      a.out[j] = __dadd_rn(v, __dmul_rn(dt, udot));
    } else if constexpr (ST == ST_RK2B) {
      a.out[j] = __ddiv_rn(__dadd_rn(__dadd_rn(a.u[j], v), __dmul_rn(dt, udot)), 2.0);
    } else if constexpr (ST == ST_RK3B) {
      a.out[j] = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(3.0, a.u[j]), v), __dmul_rn(dt, udot)), 4.0);
    } else if constexpr (ST == ST_RK3C) {
      a.out[j] = __ddiv_rn(
          __dadd_rn(__dadd_rn(a.u[j], __dmul_rn(2.0, v)), __dmul_rn(__dmul_rn(2.0, dt), udot)), 3.0);
    } else if constexpr (ST == ST_MS) {
      const double t1 = __dadd_rn(__dmul_rn(25.0, v), __dmul_rn(__dmul_rn(50.0, dt), udot));
      const double t2 = __dadd_rn(t1, __dmul_rn(7.0, a.uo4[j]));
      a.out[j] = __ddiv_rn(__dadd_rn(t2, __dmul_rn(__dmul_rn(10.0, dt), a.lo4[j])), 32.0);
      a.lout[j] = udot;
    }
  } else {
    const double rws = L.rws ? L.rws[j] : L.rws0;
    if constexpr (ST == ST_RHS) {
      a.out[j] = -(rws * dF);
    } else if constexpr (ST == ST_EULER) {
      a.out[j] = fma(-a.dt * rws, dF, v);
    } else if constexpr (ST == ST_RK2B) {
      a.out[j] = fma(0.5, a.u[j], fma(0.5, v, (-0.5 * a.dt * rws) * dF));
    } else if constexpr (ST == ST_RK3B) {
      a.out[j] = fma(0.75, a.u[j], fma(0.25, v, (-0.25 * a.dt * rws) * dF));
    } else if constexpr (ST == ST_RK3C) {
      a.out[j] = fma(1.0 / 3.0, a.u[j], fma(2.0 / 3.0, v, (-(2.0 / 3.0) * a.dt * rws) * dF));
    } else if constexpr (ST == ST_MS) {
      const double udot = -(rws * dF);
      a.out[j] = fma(25.0 / 32.0, v,
                     fma((50.0 / 32.0) * a.dt, udot,
                         fma(7.0 / 32.0, a.uo4[j], ((10.0 / 32.0) * a.dt) * a.lo4[j])));
      a.lout[j] = udot;
    }
  }
}

// --------------------------------------------------------------------------------------------
// The kernel.
// --------------------------------------------------------------------------------------------
template <int K, int ST, bool STRICT, int NT, int C>
__global__ void __launch_bounds__(NT) stage1d_kernel(StageArgs a) {
  constexpr int T = NT * C;
  constexpr int H = K;  // halo: cell j needs v(j-K .. j+K) through its two interfaces
  __shared__ double sv[T + 2 * H];
  __shared__ double sL[NT + 1];  // sL[t] = vl of thread t's first cell; sL[NT] = vl(s+T)
  __shared__ double sR[NT + 1];  // sR[t+1] = vr of thread t's last cell; sR[0] = vr(s-1)
  const LineArgs& L = a.L;
  const int64_t nc = L.nc;
  const int64_t s = (int64_t)blockIdx.x * T;
  const int tid = threadIdx.x;

  for (int q = tid; q < T + 2 * H; q += NT) {
    int64_t g = s - H + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    sv[q] = a.v[g];
  }
  __syncthreads();

  // ---- reconstruction of the thread's C cells --------------------------------------------
  const int l0 = tid * C;  // first local cell; its centre is sv[H + l0]
  double vl[C], vr[C];
  if constexpr (STRICT) {
#pragma unroll
    for (int c = 0; c < C; ++c) recon_strict<K>(&sv[H + l0 + c], a.eps, vl[c], vr[c]);
  } else {
    double w[C + 2 * K];
#pragma unroll
    for (int q = 0; q < C + 2 * K; ++q) w[q] = sv[l0 + q];  // v(j0 - K + q)
    recon_fast<K, C>(w, a.eps, vl, vr);
  }
  sL[tid] = vl[0];
  sR[tid + 1] = vr[C - 1];
  // block-edge cells s-1 (vr) and s+T (vl), one lane each of the last warp
  if (tid >= NT - 2) {
    const int which = tid - (NT - 2);  // 0: cell s-1, 1: cell s+T
    const int lc = which == 0 ? H - 1 : H + T;
    double el, er;
    if constexpr (STRICT) recon_strict<K>(&sv[lc], a.eps, el, er);
    else recon_fast_one<K>(&sv[lc], a.eps, el, er);
    if (which == 0) sR[0] = er;
    else sL[NT] = el;
  }
  __syncthreads();

  // ---- fluxes at the C+1 interfaces and the stage update ---------------------------------
  const int64_t j0 = s + l0;
  if (j0 >= nc) return;
  double F[C + 1];
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
      double FL = F[c], FR = F[c + 1];
      if (j == 0 || j == nc - 1) {
        if (L.bc == HRW_BC_COPY) {  // F_0 = F_1, F_nc = F_{nc-1}  (example1:103-104)
          FL = FR = 0.0;
        } else {
          if (j == 0) FL = 0.0;  // ZERO and ZERO_INFLOW (example2:117-120)
          if (j == nc - 1) FR = L.bc == HRW_BC_ZERO ? 0.0 : physflux<STRICT>(L, vr[c], j + 1);
        }
      }
      const double dF = STRICT ? __dsub_rn(FR, FL) : FR - FL;
      combine<ST, STRICT>(a, L, j, sv[H + l0 + c], dF);
    }
  }
}

template <int K, int ST, bool STRICT>
static cudaError_t launch_k(const StageArgs& a, cudaStream_t s) {
  constexpr int NT = 128, C = 8;
  const int64_t nblk = ((int64_t)a.L.nc + NT * C - 1) / (NT * C);
  stage1d_kernel<K, ST, STRICT, NT, C><<<(unsigned)nblk, NT, 0, s>>>(a);
  return cudaGetLastError();
}

template <int K, bool STRICT>
static cudaError_t launch_st(const StageArgs& a, int stage, cudaStream_t s) {
  switch (stage) {
    case ST_RHS: return launch_k<K, ST_RHS, STRICT>(a, s);
    case ST_EULER: return launch_k<K, ST_EULER, STRICT>(a, s);
    case ST_RK2B: return launch_k<K, ST_RK2B, STRICT>(a, s);
    case ST_RK3B: return launch_k<K, ST_RK3B, STRICT>(a, s);
    case ST_RK3C: return launch_k<K, ST_RK3C, STRICT>(a, s);
    case ST_MS: return launch_k<K, ST_MS, STRICT>(a, s);
    case ST_RECON: return launch_k<K, ST_RECON, STRICT>(a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_stage1d(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s) {
  if (a.L.nc <= 0) return cudaSuccess;
  if (k == 1) return strict ? launch_st<1, true>(a, stage, s) : launch_st<1, false>(a, stage, s);
  if (k == 2) return strict ? launch_st<2, true>(a, stage, s) : launch_st<2, false>(a, stage, s);
  return strict ? launch_st<3, true>(a, stage, s) : launch_st<3, false>(a, stage, s);
}

}  // namespace hrw
