// hrw_stage.cuh - numerical fluxes and TVD stage combines shared by the 1D and 2D fused
// stage kernels.
//
//   lax_friedrichs / godunov    src/hrweno_fluxes.f90:22-76 (formulas :43, :67-74)
//   physical fluxes             example/example1_burgers_1d_fv.f90:111-122 (u^2/2),
//                               example/example2_pbe_2d_fv.f90:131-155 (g(x) u)
//   rktvd / mstvd stage update  src/hrweno_tvdode.f90:139-167,257
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"

namespace hrw {

// --------------------------------------------------------------------------------------------
// Numerical fluxes.  e = edge index of the interface (x = xmin + rx*e, grid1%right).
// --------------------------------------------------------------------------------------------
__device__ __forceinline__ double g_fast(const LineArgs& L, int64_t e) {
  if (L.b == 0.0) return L.a;
  return fma(L.b, L.xe ? L.xe[e] : fma(L.rx, (double)e, L.xmin), L.a);
}

// FAST: returns F / fast_flux_scale(flux, fn).
__device__ __forceinline__ double flux_fast(const LineArgs& L, double vm, double vp, int64_t e) {
  if (L.fn == HRW_FN_BURGERS) {
    if (L.flux == HRW_FLUX_LAX_FRIEDRICHS)  // 4F = vm^2 + vp^2 - 2 alpha (vp - vm)
      return fma(-2.0 * L.alpha, vp - vm, fma(vp, vp, vm * vm));
    const double fm = vm * vm, fp = vp * vp;  // 2F
    return vm <= vp ? fmin(fm, fp) : fmax(fm, fp);
  }
  if (L.fn == HRW_FN_BURGERS_LINEAR) {  // 2f(v) = v (v + 2g)
    const double g2 = 2.0 * g_fast(L, e);
    const double fm = vm * (vm + g2), fp = vp * (vp + g2);
    if (L.flux == HRW_FLUX_LAX_FRIEDRICHS)  // 4F = 2f(vm) + 2f(vp) - 2 alpha (vp - vm)
      return fma(-2.0 * L.alpha, vp - vm, fm + fp);
    return vm <= vp ? fmin(fm, fp) : fmax(fm, fp);  // 2F
  }
  const double g = g_fast(L, e);
  if (L.flux == HRW_FLUX_LAX_FRIEDRICHS)  // 2F = (g + alpha) vm + (g - alpha) vp
    return fma(g + L.alpha, vm, (g - L.alpha) * vp);
  const double fm = g * vm, fp = g * vp;  // F
  return vm <= vp ? fmin(fm, fp) : fmax(fm, fp);
}
// FAST physical flux f(v) at edge e, same scaling as flux_fast.
__device__ __forceinline__ double phys_fast(const LineArgs& L, double v, int64_t e) {
  const double s = L.flux == HRW_FLUX_LAX_FRIEDRICHS ? 2.0 : 1.0;
  if (L.fn == HRW_FN_BURGERS) return s * (v * v);
  if (L.fn == HRW_FN_BURGERS_LINEAR) return s * (v * (v + 2.0 * g_fast(L, e)));
  return s * (g_fast(L, e) * v);
}

// Reference order (src/hrweno_fluxes.f90:43,67-74; example1...f90:111-122), in double (STRICT)
// or float (REAL32).
template <class T>
__device__ __forceinline__ T g_strict(const LineArgsT<T>& L, int64_t e) {
  const T x = L.xe ? L.xe[e] : rn_add(L.xmin, rn_mul(L.rx, (T)e));
  return rn_add(L.a, rn_mul(L.b, x));
}
template <class T>
__device__ __forceinline__ T phys_strict(const LineArgsT<T>& L, T v, int64_t e) {
  if (L.fn == HRW_FN_BURGERS) return rn_div(rn_mul(v, v), T(2));
  if (L.fn == HRW_FN_BURGERS_LINEAR)  // (u*u)/2 + (a + b*x)*u
    return rn_add(rn_div(rn_mul(v, v), T(2)), rn_mul(g_strict(L, e), v));
  return rn_mul(g_strict(L, e), v);
}
template <class T>
__device__ __forceinline__ T flux_strict(const LineArgsT<T>& L, T vm, T vp, int64_t e) {
  const T fm = phys_strict(L, vm, e), fp = phys_strict(L, vp, e);
  if (L.flux == HRW_FLUX_LAX_FRIEDRICHS)
    return rn_div(rn_sub(rn_add(fm, fp), rn_mul(L.alpha, rn_sub(vp, vm))), T(2));
  if (vm <= vp) return fm < fp ? fm : fp;
  return fm > fp ? fm : fp;
}

// FAST exists for double only; a float line always takes the reference order
template <bool STRICT, class T>
__device__ __forceinline__ T numflux(const LineArgsT<T>& L, T vm, T vp, int64_t e) {
  if constexpr (STRICT) return flux_strict(L, vm, vp, e);
  else return flux_fast(L, vm, vp, e);
}
template <bool STRICT, class T>
__device__ __forceinline__ T physflux(const LineArgsT<T>& L, T v, int64_t e) {
  if constexpr (STRICT) return phys_strict(L, v, e);
  else return phys_fast(L, v, e);
}

// Godunov flux of f = g(x) u with g > 0 on the whole line is g vm (upwind).  For g > 0 and
// vm <= vp, rounding is monotone so fl(g vm) <= fl(g vp) and min() picks fl(g vm); for
// vm > vp max() picks it too: the result is bit-identical to numflux<STRICT>() and needs
// only the left state.
template <bool STRICT, class T>
__device__ __forceinline__ T upwind_flux(const LineArgsT<T>& L, T vm, int64_t e) {
  if constexpr (STRICT) return rn_mul(g_strict(L, e), vm);
  else return g_fast(L, e) * vm;
}

// Flux difference dF = F_{j+1/2} - F_{j-1/2} of cell j with the domain-boundary fluxes:
//   COPY        F_{1/2} = F_{3/2}, F_{nc+1/2} = F_{nc-1/2}  (example1...f90:103-104)
//   ZERO        F_{1/2} = F_{nc+1/2} = 0                    (example2...f90:117-120)
//   ZERO_INFLOW F_{1/2} = 0, F_{nc+1/2} = f(vr(nc))
template <bool STRICT, class T>
__device__ __forceinline__ T flux_diff(const LineArgsT<T>& L, int64_t j, T FL, T FR, T vr_j) {
  if (j == 0 || j == L.nc - 1) {
    if (L.bc == HRW_BC_COPY) {
      FL = FR = T(0);
    } else {
      if (j == 0) FL = T(0);
      if (j == L.nc - 1) FR = L.bc == HRW_BC_ZERO ? T(0) : physflux<STRICT>(L, vr_j, j + 1);
    }
  }
  if constexpr (STRICT) return rn_sub(FR, FL);
  else return FR - FL;
}

// --------------------------------------------------------------------------------------------
// Stage combines of cell j.
// STRICT: udot is the exact right-hand side value, reference order.
// FAST:   q = sum over dimensions of rws * dF (= -udot), or for 1D dF and rws separately.
// --------------------------------------------------------------------------------------------
template <int ST, class T>
__device__ __forceinline__ void combine_strict(const StageArgsT<T>& a, int64_t j, T v, T udot) {
  const T dt = a.dt;
  if constexpr (ST == ST_RHS) {
    a.out[j] = udot;
  } else if constexpr (ST == ST_EULER) {  // ui = u + dt*udot  (:139,150,163)
    a.out[j] = rn_add(v, rn_mul(dt, udot));
  } else if constexpr (ST == ST_RK2B) {  // u = (u + ui + dt*udot)/2  (:152)
    a.out[j] = rn_div(rn_add(rn_add(a.u[j], v), rn_mul(dt, udot)), T(2));
  } else if constexpr (ST == ST_RK3B) {  // ui = (3*u + ui + dt*udot)/4  (:165)
    a.out[j] = rn_div(rn_add(rn_add(rn_mul(T(3), a.u[j]), v), rn_mul(dt, udot)), T(4));
  } else if constexpr (ST == ST_RK3C) {  // u = (u + 2*ui + 2*dt*udot)/3  (:167)
    a.out[j] = rn_div(rn_add(rn_add(a.u[j], rn_mul(T(2), v)), rn_mul(rn_mul(T(2), dt), udot)), T(3));
  } else if constexpr (ST == ST_MS) {  // (25u + 50dt udot + 7 uold4 + 10dt udotold4)/32  (:257)
    const T t1 = rn_add(rn_mul(T(25), v), rn_mul(rn_mul(T(50), dt), udot));
    const T t2 = rn_add(t1, rn_mul(T(7), a.uo4[j]));
    a.out[j] = rn_div(rn_add(t2, rn_mul(rn_mul(T(10), dt), a.lo4[j])), T(32));
    a.lout[j] = udot;
  }
}

// out from v and q = rws * dF (rws passed separately so that 1D folds it into dt)
template <int ST>
__device__ __forceinline__ void combine_fast(const StageArgs& a, int64_t j, double v, double dF,
                                             double rws) {
  if constexpr (ST == ST_RHS) {
    a.out[j] = -(rws * dF);
  } else if constexpr (ST == ST_EULER) {
    a.out[j] = fma(-a.dt * rws, dF, v);
  } else if constexpr (ST == ST_RK2B) {
    a.out[j] = fma(0.5, a.u[j], fma(0.5, v, (-0.5 * a.dt * rws) * dF));
  } else if constexpr (ST == ST_RK3B) {
    a.out[j] = fma(0.75, a.u[j], fma(0.25, v, (-0.25 * a.dt * rws) * dF));
  } else if constexpr (ST == ST_RK3C) {
    // (u + 2v + 2 dt L)/3 = u + 2/3 ((v - u) + dt L): the rounded 2/3 touches only the small
    // increment.  fl(1/3) u + fl(2/3) v would scale u by fl(1/3) + fl(2/3) = 1 - 2^-54 each
    // step, a coherent loss of mass that moves shocks.
    const double u = a.u[j];
    a.out[j] = fma(2.0 / 3.0, fma(-a.dt * rws, dF, v - u), u);
  } else if constexpr (ST == ST_MS) {
    const double udot = -(rws * dF);
    a.out[j] = fma(25.0 / 32.0, v,
                   fma((50.0 / 32.0) * a.dt, udot,
                       fma(7.0 / 32.0, a.uo4[j], ((10.0 / 32.0) * a.dt) * a.lo4[j])));
    a.lout[j] = udot;
  }
}

}  // namespace hrw
