// stage1d_mixed.cu - the 1D stage kernel of the MIXED numerics mode (hrw_mixed.cuh): WENO
// reconstruction + Lax-Friedrichs flux + conservative difference + TVD stage combine with the
// FP64 state in HBM and the right-hand side evaluated in difference form on the FP32 pipe.
//
// Follows, for one rktvd stage (src/hrweno_tvdode.f90:136-171) of the 1D Burgers or linear
// advection right-hand side (example/example1_burgers_1d_fv.f90:93-107):
//   weno_reconstruct    src/hrweno_weno.f90:129-219
//   lax_friedrichs      src/hrweno_fluxes.f90:43
//
// Stage kinds, in increment form (u = u^n, FP64; dv, dout = float-pair increments):
//   MX_E1    dout = d1 = dt L(u)                                  (rktvd :139,:150,:163)
//   MX_RK1   uout = u + dt L(u)                                   (rktvd :139)
//   MX_RK2B  uout = u + (d1 + dt L(u + d1)) / 2                   (rktvd :152)
//   MX_RK3B  dout = d2 = (d1 + dt L(u + d1)) / 4                  (rktvd :165)
//   MX_RK3C  uout = u + 2/3 (d2 + dt L(u + d2))                   (rktvd :167)
// uout is never the array u itself: other warps read u as their stencil while a stage runs.
//
// Layout: a warp owns 128 consecutive cells, 4 per lane, and keeps each lane's stencil window
// in registers (no shared memory).  The neighbour differences of the lane's own cells come from
// its own loads; the window's edges come from the neighbouring lanes by shuffles, and five
// lanes compute the warp's edge differences.  A warp whose cells touch a line end, or whose
// rounding-error bound (mx_bound) exceeds 2^-53 of the line's largest |u|, runs the FAST FP64
// arithmetic of stage1d.cu on its cells instead, with the same stage formulas.
#include <cmath>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"
#include "hrw_mixed.cuh"
#include "hrw_stage.cuh"

namespace hrw {

namespace {

// 4 cells per lane, 256-thread blocks, 4 blocks (32 warps) per SM at <= 64 registers: on the
// 2^24-cell line 0.349 ms per RK3 step (k = 3), against 0.376 ms at 3 blocks per SM and
// 0.425 / 0.451 ms for 8 cells per lane at 3 / 2 blocks (the kernel is bound by instruction
// issue and latency, so resident warps count)
constexpr int C = 4;            // cells per lane
constexpr int WC = 32 * C;      // cells per warp
constexpr int NT = 256;         // threads per block
constexpr int MINB = 4;         // resident blocks per SM
constexpr int ND_MAX = C + 4;   // differences of a lane's window for k <= 3
constexpr unsigned FULL = 0xffffffffu;
static_assert(C % 2 == 0 && C >= 3, "pairs of cells per vector access; the window's edges (up to 3 "
              "differences) come from one neighbouring lane");

__device__ int g_mixed_soft = 1;                 // 0: every warp takes the FP64 path (tests)
__device__ unsigned long long g_mixed_hard = 0;  // warps that took the FP64 path

template <int ST>
constexpr bool writes_state() { return ST == MX_RK1 || ST == MX_RK2B || ST == MX_RK3C; }
template <int ST>
constexpr bool reads_inc() { return ST == MX_RK2B || ST == MX_RK3B || ST == MX_RK3C; }

__device__ __forceinline__ mx::F2 ld2(const float2* p, int64_t i) {
  const float2 v = p[i];
  return {v.x, v.y};
}
__device__ __forceinline__ mx::F2 shfl_up2(mx::F2 v) {
  return {__shfl_up_sync(FULL, v.h, 1), __shfl_up_sync(FULL, v.l, 1)};
}
__device__ __forceinline__ mx::F2 shfl_down2(mx::F2 v) {
  return {__shfl_down_sync(FULL, v.h, 1), __shfl_down_sync(FULL, v.l, 1)};
}
__device__ __forceinline__ mx::F2 shfl_idx2(mx::F2 v, int src) {
  return {__shfl_sync(FULL, v.h, src), __shfl_sync(FULL, v.l, src)};
}

// the stage's FP64 value from the increment dv (float pair) and u: u + dv_h + dv_l
__device__ __forceinline__ double with_inc(double u, mx::F2 dv) {
  return (u + mx::widen(dv.h)) + mx::widen(dv.l);
}

// ------------------------------------------------------------------------------------------------
// FP64 path of a warp: the FAST arithmetic (recon_fast, flux_fast, flux_diff of stage1d.cu) on
// the FP64 stage values, with the increment-form stage formulas above.  Handles the line ends
// (ghost cells replicate v(1) and v(nc), src/hrweno_weno.f90:172-173; boundary fluxes of
// example1...f90:103-104) and any data.
// ------------------------------------------------------------------------------------------------
template <int K, int ST>
__device__ __noinline__ void fp64_pass(const MixedArgs& a, int64_t j0) {
  const LineArgs& L = a.L;
  const int64_t nc = L.nc;
  double w[C + 2 * K];  // stage values v(j0 - K + q)
#pragma unroll
  for (int q = 0; q < C + 2 * K; ++q) {
    int64_t g = j0 - K + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    double v = a.u[g];
    if constexpr (reads_inc<ST>()) v = with_inc(v, ld2(a.dv, g));
    w[q] = v;
  }
  double vl[C], vr[C];
  recon_fast<K, C>(w, a.eps, vl, vr);
  double el, er, fl, fr;
  recon_fast_one<K>(&w[K - 1], a.eps, el, er);   // cell j0 - 1 (its vr)
  recon_fast_one<K>(&w[K + C], a.eps, fl, fr);   // cell j0 + C (its vl)
  double F[C + 1];
  F[0] = flux_fast(L, er, vl[0], j0);
#pragma unroll
  for (int c = 1; c < C; ++c) F[c] = flux_fast(L, vr[c - 1], vl[c], j0 + c);
  F[C] = flux_fast(L, vr[C - 1], fl, j0 + C);
  const double k = -a.dt * L.rws0;  // dt L = k dF
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int64_t j = j0 + c;
    if (j >= nc) break;
    const double dtL = k * flux_diff<false>(L, j, F[c], F[c + 1], vr[c]);
    if constexpr (ST == MX_E1) {
      const mx::F2 o = mx::split(dtL);
      a.dout[j] = make_float2(o.h, o.l);
    } else if constexpr (ST == MX_RK3B) {
      const mx::F2 dv = ld2(a.dv, j);
      const mx::F2 o = mx::split(0.25 * ((mx::widen(dv.h) + mx::widen(dv.l)) + dtL));
      a.dout[j] = make_float2(o.h, o.l);
    } else if constexpr (ST == MX_RK1) {
      a.uout[j] = a.u[j] + dtL;
    } else {
      const mx::F2 dv = ld2(a.dv, j);
      a.uout[j] = fma(ST == MX_RK2B ? 0.5 : 2.0 / 3.0, (mx::widen(dv.h) + mx::widen(dv.l)) + dtL, a.u[j]);
    }
  }
}

// ------------------------------------------------------------------------------------------------
// The FP32 path of a lane's C cells: reconstructions in difference form, the interface sums, the
// flux differences and dt L as float pairs (out).  NL = false: linear weights only (the caller has
// shown that the weight deviations cannot move dt L by more than the budget); NL = true: the full
// WENO weights.  Returns the NL pass's bound on the rounding error of dt L (mx_bound), 0 for the
// linear pass.
// ------------------------------------------------------------------------------------------------
template <int K, int ST, bool LIN, bool NL>
__device__ __forceinline__ float soft_cells(const MixedArgs& a, const double* u, const mx::F2* dv,
                                            const mx::F2* dd, const float* d, const float* D,
                                            float Md, float Mdd, mx::F2* out) {
  // reconstructions of cells j0-1 .. j0+C (window position m = K-1 .. K+C; cell m uses
  // d[m-K+1 .. m+K-2] and D[m-K+1 .. m-1])
  float rr[C + 2], rl[C + 2], rrn[C + 2], rln[C + 2];
  float dev = 0.f;
  if constexpr (NL) {
    float tA[ND_MAX];
    if constexpr (K == 3) {
#pragma unroll
      for (int q = 0; q < C + 2 * K - 2; ++q) tA[q] = fmaf((13.f / 12.f) * D[q], D[q], a.epsf);
    }
#pragma unroll
    for (int i = 0; i < C + 2; ++i) {
      const int m = K - 1 + i;
      mx::Rec R;
      if constexpr (K == 3) R = mx::rec3(&d[m - 2], &D[m - 2], &tA[m - 2]);
      else R = mx::rec2(&d[m - 1], &D[m - 1], a.epsf);
      rr[i] = R.rr, rl[i] = R.rl, rrn[i] = R.rrn, rln[i] = R.rln;
      dev = fmaxf(dev, R.dev);
    }
  } else {
#pragma unroll
    for (int i = 0; i < C + 2; ++i) {
      const int m = K - 1 + i;
      mx::lin<K>(&d[m - K + 1], rr[i], rl[i]);
      rrn[i] = rln[i] = 0.f;
    }
  }
  // interface sums of the linear-weight states at interface i + 1/2 (window position m):
  //   k = 3: X = -Dd_{i-2} + 6 Dd_{i-1} + 6 Dd_i - Dd_{i+1},  Y = Dd_{i+1} - 3 Dd_i + 3 Dd_{i-1} - Dd_{i-2}
  //          vr_lin(i) + vl_lin(i+1) - 2 v_i = d_i - X/30,  vr_lin(i) - vl_lin(i+1) = -Y/30
  //   k = 2: X = Dd_{i-1} + Dd_i, Y = Dd_i - Dd_{i-1}: d_i - X/6 and Y/6
  // (X[] and Y[] below hold X/30 and the second expression, resp. X/6 and Y/6)
  float X[C + 1], Y[C + 1];
#pragma unroll
  for (int i = 0; i < C + 1; ++i) {
    const int m = K - 1 + i;
    if constexpr (K == 3) {
      X[i] = fmaf(6.f, D[m - 1] + D[m], -(D[m - 2] + D[m + 1])) * (1.f / 30.f);
      Y[i] = -fmaf(-3.f, D[m] - D[m - 1], D[m + 1] - D[m - 2]) * (1.f / 30.f);
    } else {
      X[i] = (D[m - 1] + D[m]) * (1.f / 6.f);
      Y[i] = (D[m] - D[m - 1]) * (1.f / 6.f);
    }
  }
  float Vh = 0.f, Vl = 0.f, Vmax = 0.f;
  if constexpr (LIN) Vh = a.g_h, Vl = a.g_l;
  float errmax = 0.f;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int m = K + c;  // d[m] = d_j, d[m-1] = d_{j-1}
    // offsets of the interface states from v_j (FP32)
    const float aR = rr[c + 1], bR = d[m] + rl[c + 2];
    const float aL = rr[c] - d[m - 1], bL = rl[c + 1];
    // S = (aR + bR) - (aL + bL), T = (aR - bR) - (aL - bL): linear parts in pairs, the
    // nonlinear parts (FP32) added to the low word
    float sh, se;
    mx::two_sum(dd[m].h, dd[m - 1].h, sh, se);
    float sl = (se + (dd[m].l + dd[m - 1].l)) - (X[c + 1] - X[c]);
    float T = Y[c + 1] - Y[c];
    if constexpr (NL) {
      sl += (rrn[c + 1] + rln[c + 2]) - (rrn[c] + rln[c + 1]);
      T += (rrn[c + 1] - rln[c + 2]) - (rrn[c] - rln[c + 1]);
    }
    // 4 dF = 2 V S + Q + 2 alpha T: Burgers V = v_j (Q = aR^2 + bR^2 - aL^2 - bL^2), linear V = g
    if constexpr (!LIN) {
      const mx::F2 v = mx::split_t(u[c]);
      Vh = v.h;
      Vl = v.l;
      if constexpr (reads_inc<ST>()) Vl += dv[c].h + dv[c].l;
      Vmax = fmaxf(Vmax, fabsf(Vh));
    }
    const float p = 2.f * Vh * sh;
    float pl = fmaf(2.f * Vh, sh, -p);
    pl = fmaf(2.f * Vh, sl, pl);
    pl = fmaf(2.f * Vl, sh, pl);
    float q = 2.f * a.alpha_f * T;
    if constexpr (!LIN) q += fmaf(aR, aR, bR * bR) - fmaf(aL, aL, bL * bL);
    // dt L = -c (4 dF), c = dt / (4 dx) as a pair
    const mx::F2 F = mx::renorm(p, pl + q);
    const float th = a.c_h * F.h;
    float tl = fmaf(a.c_h, F.h, -th);
    tl = fmaf(a.c_h, F.l, fmaf(a.c_l, F.h, tl));
    out[c] = mx::renorm(-th, -tl);
    if constexpr (NL && !LIN)
      errmax = fmaxf(errmax, fmaxf(fabsf(aR), fabsf(bR)) + fmaxf(fabsf(aL), fabsf(bL)));
  }
  if constexpr (!NL) return 0.f;
  // mx_bound: |error of 4 dF| <= 2|V| eS + 2 alpha eT + eQ with
  //   eS, eT <= 2^-21 Mdd (the interface sums) + 2^-46 Md (the difference pairs) + eNL
  //   eNL = 2^-18 Mdd dev + 2^-12 Mdd^2 (Md + Mdd) / eps: the four reconstructions' weight
  //         deviations, rounded (a few ulps of dev) and moved by the rounding of the indicator
  //         differences (at most 2^-18 Mdd (Md + Mdd) each; |dw / dbeta| <= 2 / eps)
  //   eQ <= 2^-21 Md (|aR| + |bR| + |aL| + |bL|): each offset is within 2^-22.2 Md of its
  //         value (d rounded to FP32, the rounding of the linear stencils), its square and the sum
  //         add a few roundings of Md^2
  // (the 2^-92 (V + alpha) floor covers differences below 2^-74, whose low words are dropped)
  const float eNL = fmaf(0x1p-18f * Mdd, dev, 0x1p-12f * Mdd * Mdd * (Md + Mdd) * a.inv_eps);
  const float eST = fmaf(0x1p-21f, Mdd, fmaf(0x1p-46f, Md, eNL));
  const float Vb = LIN ? fabsf(a.g_h) : Vmax * 1.001f;
  float e4 = fmaf(2.f * Vb, eST, fmaf(2.f * a.alpha_f, eST, 0x1p-92f * (Vb + a.alpha_f)));
  if constexpr (!LIN) e4 = fmaf(0x1p-21f * Md, 2.f * errmax, e4);
  return a.c_h * e4;  // NaN for NaN and infinite inputs: the caller's test fails
}

// ------------------------------------------------------------------------------------------------
// The kernel.
// ------------------------------------------------------------------------------------------------
template <int K, int ST, bool LIN>
__global__ void __launch_bounds__(NT, MINB) stage1d_mixed_kernel(MixedArgs a) {
  constexpr int ND = C + 2 * K - 1;  // window of differences d_{j0-K} .. d_{j0+C+K-2}
  constexpr int NH = 2 * K - 1;      // the warp's edge differences: K on the left, K-1 on the right
  const int lane = threadIdx.x & 31;
  const int64_t w0 = a.cell0 + ((int64_t)blockIdx.x * NT + (threadIdx.x & ~31)) / 32 * WC;
  const int64_t nc = a.L.nc;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (w0 >= nc) return;  // the whole warp is past the line
  const int64_t j0 = w0 + (int64_t)lane * C;

  // own cells: u (FP64) and the stage increment
  double u[C];
  mx::F2 dv[C];
  const bool inside = w0 >= 4 && w0 + WC + 4 <= nc;  // no ghost cell and no boundary flux
  if (inside) {
#pragma unroll
    for (int c = 0; c < C; c += 2) {
      const double2 x = *reinterpret_cast<const double2*>(a.u + j0 + c);
      u[c] = x.x, u[c + 1] = x.y;
    }
    if constexpr (reads_inc<ST>()) {
#pragma unroll
      for (int c = 0; c < C; c += 2) {
        const float4 x = *reinterpret_cast<const float4*>(a.dv + j0 + c);
        dv[c] = {x.x, x.y}, dv[c + 1] = {x.z, x.w};
      }
    }
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t g = j0 + c < nc ? j0 + c : nc - 1;
      u[c] = a.u[g];
      if constexpr (reads_inc<ST>()) dv[c] = ld2(a.dv, g);
    }
  }
  bool soft = inside && g_mixed_soft != 0;

  // ---- the scale: the line's largest |u| at the start of the integrate call (its high word,
  // *a.scale), as a power of two below it; 2^-53 of it (half an FP64 ulp of the largest values)
  // is the per-stage error budget of dt L.
  // Soft range: 2^-40 <= max|u| < 2^60.
  float bound_lim = 0.f;
  if (soft) {
    const int E = (int)(*a.scale >> 20) - 1023;  // 2^E <= max|u|
    soft = E >= -40 && E < 60;
    bound_lim = __int_as_float((E - 53 + 127) << 23);
  }

  // ---- float-pair differences of the stage values, v = u (+ dv) ----------------------------------
  mx::F2 dd[ND];
  if (soft) {
    double un = __shfl_down_sync(FULL, u[0], 1);
    mx::F2 dvn = {0.f, 0.f};
    if constexpr (reads_inc<ST>()) dvn = shfl_down2(dv[0]);
    if (lane == 31) {
      un = a.u[j0 + C];
      if constexpr (reads_inc<ST>()) dvn = ld2(a.dv, j0 + C);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const double hi = c + 1 < C ? u[c + 1] : un;
      mx::F2 p = mx::split_t(hi - u[c]);
      if constexpr (reads_inc<ST>()) {
        const mx::F2 n = c + 1 < C ? dv[c + 1] : dvn;
        p = mx::add(p, {n.h - dv[c].h, n.l - dv[c].l});
      }
      dd[K + c] = p;
    }
    // the warp's edge differences: lane i < K computes d_{w0-K+i}, lane K+i computes
    // d_{w0+WC+i} (i < K-1)
    mx::F2 h = {0.f, 0.f};
    if (lane < NH) {
      const int64_t q = lane < K ? w0 - K + lane : w0 + WC + (lane - K);
      h = mx::split_t(a.u[q + 1] - a.u[q]);
      if constexpr (reads_inc<ST>()) {
        const mx::F2 x = ld2(a.dv, q), y = ld2(a.dv, q + 1);
        h = mx::add(h, {y.h - x.h, y.l - x.l});
      }
    }
#pragma unroll
    for (int s = 0; s < K; ++s) {  // left: the previous lane's last K
      const mx::F2 x = shfl_up2(dd[C + s]);
      const mx::F2 y = shfl_idx2(h, s);
      dd[s] = lane == 0 ? y : x;
    }
#pragma unroll
    for (int s = 0; s < K - 1; ++s) {  // right: the next lane's first K-1
      const mx::F2 x = shfl_down2(dd[K + s]);
      const mx::F2 y = shfl_idx2(h, K + s);
      dd[K + C + s] = lane == 31 ? y : x;
    }
  }

  // ---- the soft path: reconstruction, fluxes, dt L in difference form ------------------------------
  mx::F2 out[C];
  if (soft) {
    float d[ND], D[ND - 1];
    float Md = 0.f, Mdd = 0.f;
#pragma unroll
    for (int q = 0; q < ND; ++q) {
      d[q] = dd[q].h + dd[q].l;  // d to FP32 precision (the pair rounded to nearest)
      Md = fmaxf(Md, fabsf(d[q]));
    }
#pragma unroll
    for (int q = 0; q < ND - 1; ++q) {
      D[q] = (dd[q + 1].h - dd[q].h) + (dd[q + 1].l - dd[q].l);
      Mdd = fmaxf(Mdd, fabsf(D[q]));
    }
    // The weight deviations w_r - d_r are at most 2.01 |Dbeta| / eps while the indicator
    // differences |Dbeta| <= Db = 4 Mdd (Md + 2.5 Mdd) stay below eps / 100, and their share of
    // rr or rl at most 1.34 |Dbeta| Mdd / eps.  Where dropping them moves dt L by less than the
    // budget in every lane of the warp (mx_bound with the dropped parts as an error term), the
    // warp takes the linear-weight pass, which skips the weights altogether.
    // |V| <= 2^(E+1) + |dv| with E the exponent of the lane's largest |u| (from high words:
    // an FP64-to-FP32 conversion would take the narrow FP64 unit)
    float Vb = LIN ? fabsf(a.g_h) : 0.f;
    if constexpr (!LIN) {
      unsigned m = 0;
      float x = 0.f;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        m = max(m, (unsigned)__double2hiint(u[c]) & 0x7FFFFFFFu);
        if constexpr (reads_inc<ST>()) x = fmaxf(x, fabsf(dv[c].h));
      }
      Vb = __int_as_float(max((int)(m >> 20) - 1023 + 1, -126) + 127 << 23) + 1.001f * x;
    }
    const float Db = 4.f * Mdd * fmaf(2.5f, Mdd, Md);
    const float eSkip = 6.f * Db * Mdd * a.inv_eps;  // the four reconstructions' dropped parts
    const float eL = fmaf(0x1p-21f, Mdd, fmaf(0x1p-46f, Md, eSkip));
    float e4 = fmaf(2.f * Vb, eL, fmaf(2.f * a.alpha_f, eL, 0x1p-92f * (Vb + a.alpha_f)));
    // quadratic terms: eQ with |aR| + |bR| + |aL| + |bL| <= 4 Md, and the dropped parts' effect
    if constexpr (!LIN) e4 = fmaf(Md, fmaf(0x1p-18f, Md, 8.f * eSkip), e4);
    const bool lin_ok = Db * a.inv_eps <= 0.01f && a.c_h * e4 <= bound_lim;
    bool ok;
    if (__all_sync(FULL, lin_ok)) {
      soft_cells<K, ST, LIN, false>(a, u, dv, dd, d, D, Md, Mdd, out);
      ok = true;
    } else {
      ok = soft_cells<K, ST, LIN, true>(a, u, dv, dd, d, D, Md, Mdd, out) <= bound_lim;
    }
    soft = !__any_sync(FULL, !ok);
  }

  if (!soft) {
    if (lane == 0 && inside) atomicAdd(&g_mixed_hard, 1ull);
    fp64_pass<K, ST>(a, j0);
    return;
  }

  // ---- stage update --------------------------------------------------------------------------------
  if constexpr (ST == MX_E1 || ST == MX_RK3B) {
#pragma unroll
    for (int c = 0; c < C; c += 2) {
      mx::F2 o0 = out[c], o1 = out[c + 1];
      if constexpr (ST == MX_RK3B) {  // d2 = (d1 + dt L) / 4
        o0 = mx::add(dv[c], o0);
        o1 = mx::add(dv[c + 1], o1);
        o0 = {0.25f * o0.h, 0.25f * o0.l};
        o1 = {0.25f * o1.h, 0.25f * o1.l};
      }
      *reinterpret_cast<float4*>(a.dout + j0 + c) = make_float4(o0.h, o0.l, o1.h, o1.l);
    }
  } else {
#pragma unroll
    for (int c = 0; c < C; c += 2) {
      double r[2];
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        mx::F2 inc = out[c + s];
        if constexpr (ST == MX_RK2B) {
          inc = mx::add(dv[c + s], inc);
          inc = {0.5f * inc.h, 0.5f * inc.l};
        } else if constexpr (ST == MX_RK3C) {
          inc = mx::mul(mx::add(dv[c + s], inc), {a.two3_h, a.two3_l});
        }
        r[s] = u[c + s] + mx::pack(inc);  // one FP64 addition
      }
      *reinterpret_cast<double2*>(a.uout + j0 + c) = make_double2(r[0], r[1]);
    }
  }
}

template <int K, int ST>
cudaError_t launch_st(const MixedArgs& a, cudaStream_t s) {
  static_assert(NT / 32 * WC == kMixedTile, "the block tile of cell ranges");
  const int64_t span = a.ncell > 0 ? a.ncell : (int64_t)a.L.nc - a.cell0;
  const int64_t warps = (span + WC - 1) / WC;
  const int64_t nblk = (warps + NT / 32 - 1) / (NT / 32);
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
  const bool lin = a.L.fn == HRW_FN_LINEAR;
  const cudaError_t e = lin ? cudaLaunchKernelEx(&cfg, stage1d_mixed_kernel<K, ST, true>, a)
                            : cudaLaunchKernelEx(&cfg, stage1d_mixed_kernel<K, ST, false>, a);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <int K>
cudaError_t launch_k(const MixedArgs& a, int stage, cudaStream_t s) {
  switch (stage) {
    case MX_E1: return launch_st<K, MX_E1>(a, s);
    case MX_RK1: return launch_st<K, MX_RK1>(a, s);
    case MX_RK2B: return launch_st<K, MX_RK2B>(a, s);
    case MX_RK3B: return launch_st<K, MX_RK3B>(a, s);
    case MX_RK3C: return launch_st<K, MX_RK3C>(a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

bool mixed_supported(const LineArgs& L, int k) {
  return (k == 2 || k == 3) && L.flux == HRW_FLUX_LAX_FRIEDRICHS && !L.width && !L.xe &&
         (L.fn == HRW_FN_BURGERS || (L.fn == HRW_FN_LINEAR && L.b == 0.0));
}

void mixed_fill(MixedArgs& a, double eps, double dt) {
  a.eps = eps;
  a.dt = dt;
  a.epsf = (float)eps;
  a.inv_eps = (float)(1.0 / eps);
  a.alpha_f = (float)a.L.alpha;
  const double c = dt / (4.0 * a.L.rx);  // dt L = -c (4 dF) on a uniform grid
  a.c_h = (float)c;
  a.c_l = (float)(c - (double)a.c_h);
  const double g = a.L.a;
  a.g_h = (float)g;
  a.g_l = (float)(g - (double)a.g_h);
  a.two3_h = (float)(2.0 / 3.0);
  a.two3_l = (float)(2.0 / 3.0 - (double)a.two3_h);
}

cudaError_t launch_stage1d_mixed(const MixedArgs& a, int k, int stage, cudaStream_t s) {
  if (a.L.nc <= 0) return cudaSuccess;
  if (!mixed_supported(a.L, k) || a.uout == a.u) return cudaErrorInvalidValue;
  if (k == 2) return launch_k<2>(a, stage, s);
  return launch_k<3>(a, stage, s);
}

// The line's largest |u| as the high word of its FP64 value (positive doubles order like
// their high words): *word = max over i of hiword(|u_i|).  *word must be zero on entry.
__global__ void mixed_scale_kernel(const double* __restrict__ u, int64_t n, unsigned* word) {
  unsigned m = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    m = max(m, (unsigned)__double2hiint(u[i]) & 0x7FFFFFFFu);
  m = __reduce_max_sync(FULL, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(word, m);
}

cudaError_t launch_mixed_scale(const double* u, int64_t n, unsigned* word, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(word, 0, sizeof(unsigned), s);
  if (e != cudaSuccess || n <= 0) return e;
  const int64_t nb = (n + 255) / 256;
  const int64_t cap = (int64_t)device_sms() * 8;
  mixed_scale_kernel<<<(unsigned)(nb < cap ? nb : cap), 256, 0, s>>>(u, n, word);
  return cudaGetLastError();
}

cudaError_t mixed_set_soft(int enable) {
  const int v = enable != 0;
  return cudaMemcpyToSymbol(g_mixed_soft, &v, sizeof(v));
}

cudaError_t mixed_hard_warps(unsigned long long* count, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(count, g_mixed_hard, sizeof(*count));
  if (e == cudaSuccess && reset) {
    const unsigned long long z = 0;
    e = cudaMemcpyToSymbol(g_mixed_hard, &z, sizeof(z));
  }
  return e;
}

}  // namespace hrw
