// hrw_f32c.cuh - device building blocks of the compensated FP32 form.
//
// The FP32 form keeps the state as a pair of floats u = hi + lo (about 48 significant bits)
// and evaluates the right-hand side in *difference form*.  Plain FP32 loses the flux
// difference: F_{j+1/2} - F_{j-1/2} is a difference of O(1) numbers that agree to O(dx), so
// a rounding of eps|u| in each reconstructed state becomes an error of eps|u|/dx in L(u) --
// at 2^24 cells that is of the order of L itself.  Here every quantity that enters a
// cancellation is formed from compensated neighbour differences d_m = u_{m+1} - u_m:
//
//  * the WENO candidates and smoothness indicators of src/hrweno_weno.f90:178-204 are linear
//    and quadratic forms in the differences (rewritten below, same method);
//  * the reconstructed states are carried as offsets a, b from the cell's own value v;
//  * the flux difference of cell j is G(right) - G(left) with G = F - f(v_j) computed from the
//    offsets, so the O(1) part f(v_j) cancels exactly instead of in rounding;
//  * stage values are stored as small increments relative to u, and the increment of the
//    final stage is added to (hi, lo) by an error-free two-sum.
//
// The rounding errors that remain are relative to the small quantities (differences,
// increments), which is what keeps the FP32 form within 1e-6 relative L1 of FP64.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_internal.h"

namespace hrw {

// error-free transformation: s + e == x + y exactly
__device__ __forceinline__ void two_sum(float x, float y, float& s, float& e) {
  s = __fadd_rn(x, y);
  const float bb = __fsub_rn(s, x);
  e = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(y, bb));
}

// (hi, lo) += x, renormalised so that |lo| <= ulp(hi)/2
__device__ __forceinline__ void acc_add(float& hi, float& lo, float x) {
  float s, e;
  two_sum(hi, x, s, e);
  const float t = __fadd_rn(lo, e);
  hi = __fadd_rn(s, t);
  lo = __fsub_rn(t, __fsub_rn(hi, s));
}

// 1/x by the MUFU approximation (about 1 ulp); x normal and positive
__device__ __forceinline__ float rcpf(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// ---------------------------------------------------------------------------------------------
// WENO offsets of one cell from its differences (k = 1..3).
//   d[q] = d_{j-K+1+q}, q = 0 .. 2K-3  (k=3: d_{j-2}, d_{j-1}, d_j, d_{j+1}; k=2: d_{j-1}, d_j)
// Returns rr = vr(j) - v(j) and rl = vl(j) - v(j).
//
// In terms of the differences (d_{-2} = v_{j-1} - v_{j-2}, ..., d_1 = v_{j+2} - v_{j+1}), the
// reference's k = 3 candidates (c3 table, src/hrweno_weno.f90:19-21) minus v_j are
//   vrr0 (4 d0 - d1)/6      vrr1 (d_{-1} + 2 d0)/6     vrr2 (5 d_{-1} - 2 d_{-2})/6
//   vlr0 (2 d1 - 5 d0)/6    vlr1 -(2 d_{-1} + d0)/6    vlr2 (d_{-2} - 4 d_{-1})/6
// and its smoothness indicators (:194-202) are
//   beta0 = 13/12 (d1 - d0)^2      + 1/4 (d1 - 3 d0)^2
//   beta1 = 13/12 (d0 - d_{-1})^2  + 1/4 (d_{-1} + d0)^2
//   beta2 = 13/12 (d_{-1} - d_{-2})^2 + 1/4 (3 d_{-1} - d_{-2})^2.
// For k = 2 (c2 table, :16-18; :189-191): vrr0 = d0/2, vrr1 = d_{-1}/2, vlr0 = -d0/2,
// vlr1 = -d_{-1}/2, beta0 = d0^2, beta1 = d_{-1}^2.
// Weights (:207-210) in product form with two reciprocals; cells whose squared indicators
// leave the float range of the products take the quotient form.
// ---------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void recon_diff(const float* d, float eps, float& rl, float& rr) {
  if constexpr (K == 1) {
    rl = 0.f;
    rr = 0.f;
  } else if constexpr (K == 2) {
    const float dm = d[0], d0 = d[1];
    const float e0 = fmaf(d0, d0, eps), e1 = fmaf(dm, dm, eps);
    const float s0 = e0 * e0, s1 = e1 * e1;
    // w0 = (2/3)/s0 / (...) = 2 s1 / (2 s1 + s0);  mirrored d: w~0 = s1 / (s1 + 2 s0)
    if (fmaxf(s0, s1) < 1e30f) {
      const float den = fmaf(2.f, s1, s0), dent = fmaf(2.f, s0, s1);
      // rr = (w0 d0 + w1 d_{-1}) / 2, rl = -(w~0 d0 + w~1 d_{-1}) / 2
      rr = 0.5f * fmaf(2.f * s1, d0, s0 * dm) * rcpf(den);
      rl = -0.5f * fmaf(s1, d0, 2.f * s0 * dm) * rcpf(dent);
    } else {
      const float a0 = (2.f / 3.f) / s0, a1 = (1.f / 3.f) / s1;
      const float t0 = (1.f / 3.f) / s0, t1 = (2.f / 3.f) / s1;
      rr = 0.5f * (a0 * d0 + a1 * dm) / (a0 + a1);
      rl = -0.5f * (t0 * d0 + t1 * dm) / (t0 + t1);
    }
  } else {
    const float dmm = d[0], dm = d[1], d0 = d[2], d1 = d[3];
    const float c13 = 13.f / 12.f;
    const float A0 = d1 - d0, A1 = d0 - dm, A2 = dm - dmm;
    const float B0 = fmaf(-3.f, d0, d1), B1 = dm + d0, B2 = fmaf(3.f, dm, -dmm);
    const float b0 = fmaf(c13 * A0, A0, 0.25f * B0 * B0);
    const float b1 = fmaf(c13 * A1, A1, 0.25f * B1 * B1);
    const float b2 = fmaf(c13 * A2, A2, 0.25f * B2 * B2);
    const float e0 = eps + b0, e1 = eps + b1, e2 = eps + b2;
    const float s0 = e0 * e0, s1 = e1 * e1, s2 = e2 * e2;
    // candidates x6
    const float R0 = fmaf(4.f, d0, -d1), R1 = fmaf(2.f, d0, dm), R2 = fmaf(5.f, dm, -2.f * dmm);
    const float L0 = fmaf(2.f, d1, -5.f * d0), L1 = -fmaf(2.f, dm, d0), L2 = fmaf(-4.f, dm, dmm);
    // The product form's numerator is at most 30.4 max(s)^2.25 (|R_r| <= 3.04 sqrt(e_r), the
    // indicators being positive definite forms in the same differences), finite in FP32 up to
    // max(s) = 2.9e16; above 1e16 the division form.
    if (fmaxf(s0, fmaxf(s1, s2)) < 1e16f) {
      // d = (3, 6, 1)/10: w_r ~ d_r P_r with P_0 = s1 s2, P_1 = s0 s2, P_2 = s0 s1
      const float P0 = s1 * s2, P1 = s0 * s2, P2 = s0 * s1;
      const float den = fmaf(3.f, P0, fmaf(6.f, P1, P2));
      const float dent = fmaf(3.f, P2, fmaf(6.f, P1, P0));  // mirrored d = (1, 6, 3)/10
      const float num = fmaf(3.f * P0, R0, fmaf(6.f * P1, R1, P2 * R2));
      const float numt = fmaf(P0, L0, fmaf(6.f * P1, L1, 3.f * P2 * L2));
      rr = (num * rcpf(den)) * (1.f / 6.f);
      rl = (numt * rcpf(dent)) * (1.f / 6.f);
    } else {
      const float a0 = 0.3f / s0, a1 = 0.6f / s1, a2 = 0.1f / s2;
      const float t0 = 0.1f / s0, t1 = 0.6f / s1, t2 = 0.3f / s2;
      rr = (a0 * R0 + a1 * R1 + a2 * R2) / (6.f * (a0 + a1 + a2));
      rl = (t0 * L0 + t1 * L1 + t2 * L2) / (6.f * (t0 + t1 + t2));
    }
  }
}

// eps + 13/12 D^2 for the second difference D = d_m - d_{m-1} at one window position
__device__ __forceinline__ float shared_t(float dm1, float dm, float eps) {
  const float D = dm - dm1;
  return fmaf((13.f / 12.f) * D, D, eps);
}

// K = 3 reconstruction of one cell with eps + 13/12 (second difference)^2 of its three
// indicators precomputed (neighbouring cells share them; shared_t below): t0, t1, t2 for
// beta0, beta1, beta2.  Same weights and candidates as recon_diff<3>, eps added once per
// window position instead of once per indicator.  WL = false computes rr only (rl untouched),
// with the same operations for rr: an upwind flux needs the left state of each interface alone.
template <bool WL = true>
__device__ __forceinline__ void recon_diff3_shared(const float* d, float t0, float t1, float t2,
                                                   float& rl, float& rr) {
  const float dmm = d[0], dm = d[1], d0 = d[2], d1 = d[3];
  const float B0 = fmaf(-3.f, d0, d1), B1 = dm + d0, B2 = fmaf(3.f, dm, -dmm);
  const float e0 = fmaf(0.25f * B0, B0, t0);  // eps + beta0
  const float e1 = fmaf(0.25f * B1, B1, t1);
  const float e2 = fmaf(0.25f * B2, B2, t2);
  const float s0 = e0 * e0, s1 = e1 * e1, s2 = e2 * e2;
  const float R0 = fmaf(4.f, d0, -d1), R1 = fmaf(2.f, d0, dm), R2 = fmaf(5.f, dm, -2.f * dmm);
  const float L0 = fmaf(2.f, d1, -5.f * d0), L1 = -fmaf(2.f, dm, d0), L2 = fmaf(-4.f, dm, dmm);
  if (fmaxf(s0, fmaxf(s1, s2)) < 1e16f) {  // the bound of recon_diff<3>
    const float P0 = s1 * s2, P1 = s0 * s2, P2 = s0 * s1;
    const float den = fmaf(3.f, P0, fmaf(6.f, P1, P2));
    const float num = fmaf(3.f * P0, R0, fmaf(6.f * P1, R1, P2 * R2));
    rr = (num * rcpf(den)) * (1.f / 6.f);
    if constexpr (WL) {
      const float dent = fmaf(3.f, P2, fmaf(6.f, P1, P0));
      const float numt = fmaf(P0, L0, fmaf(6.f * P1, L1, 3.f * P2 * L2));
      rl = (numt * rcpf(dent)) * (1.f / 6.f);
    }
  } else {
    const float a0 = 0.3f / s0, a1 = 0.6f / s1, a2 = 0.1f / s2;
    rr = (a0 * R0 + a1 * R1 + a2 * R2) / (6.f * (a0 + a1 + a2));
    if constexpr (WL) {
      const float u0 = 0.1f / s0, u1 = 0.6f / s1, u2 = 0.3f / s2;
      rl = (u0 * L0 + u1 * L1 + u2 * L2) / (6.f * (u0 + u1 + u2));
    }
  }
}

// ---------------------------------------------------------------------------------------------
// WENO offsets of one cell of a non-uniform line from its differences, with the cell's own
// coefficients ci(q, r) at [q + K (r + 1)] (cnu of src/hrweno_weno.f90:170,177-181).  Each
// candidate minus v_j is sum_q c(q, r) (v_{j-r+q} - v_j), the neighbour values relative to v_j
// being sums of differences (S(m) below), so the rounding of the coefficients touches only the
// small offsets.  The indicators and the weights are the uniform ones (:183-210, as the
// reference computes them on any grid); d as recon_diff.
// ---------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void recon_diff_nu(const float* d, const float* ci, float eps, float& rl,
                                              float& rr) {
  if constexpr (K == 1) {
    rl = 0.f;
    rr = 0.f;
  } else {
    // S[m + K - 1] = v_{j+m} - v_j, m = -(K-1) .. K-1
    float S[2 * K - 1];
    S[K - 1] = 0.f;
#pragma unroll
    for (int m = 1; m < K; ++m) {
      S[K - 1 + m] = S[K - 2 + m] + d[K - 2 + m];
      S[K - 1 - m] = S[K - m] - d[K - 1 - m];
    }
    float R[K], Lc[K];
#pragma unroll
    for (int r = 0; r < K; ++r) {
      float sr = 0.f, sl = 0.f;
#pragma unroll
      for (int q = 0; q < K; ++q) {
        if (q == r) continue;  // the cell itself: v_j - v_j
        const float x = S[K - 1 - r + q];
        sr = fmaf(ci[q + K * (r + 1)], x, sr);
        sl = fmaf(ci[q + K * r], x, sl);
      }
      R[r] = sr;
      Lc[r] = sl;
    }
    if constexpr (K == 2) {
      const float dm = d[0], d0 = d[1];
      const float e0 = fmaf(d0, d0, eps), e1 = fmaf(dm, dm, eps);
      const float s0 = e0 * e0, s1 = e1 * e1;
      // w0 = 2 s1 / (2 s1 + s0), mirrored w~0 = s1 / (s1 + 2 s0); the candidates carry the
      // coefficients' sums (a few units on graded lines), hence a lower bound than uniform k = 2
      if (fmaxf(s0, s1) < 1e28f) {
        rr = fmaf(2.f * s1, R[0], s0 * R[1]) * rcpf(fmaf(2.f, s1, s0));
        rl = fmaf(s1, Lc[0], 2.f * s0 * Lc[1]) * rcpf(fmaf(2.f, s0, s1));
      } else {
        const float a0 = (2.f / 3.f) / s0, a1 = (1.f / 3.f) / s1;
        const float t0 = (1.f / 3.f) / s0, t1 = (2.f / 3.f) / s1;
        rr = (a0 * R[0] + a1 * R[1]) / (a0 + a1);
        rl = (t0 * Lc[0] + t1 * Lc[1]) / (t0 + t1);
      }
    } else {
      const float dmm = d[0], dm = d[1], d0 = d[2], d1 = d[3];
      const float c13 = 13.f / 12.f;
      const float A0 = d1 - d0, A1 = d0 - dm, A2 = dm - dmm;
      const float B0 = fmaf(-3.f, d0, d1), B1 = dm + d0, B2 = fmaf(3.f, dm, -dmm);
      const float e0 = eps + fmaf(c13 * A0, A0, 0.25f * B0 * B0);
      const float e1 = eps + fmaf(c13 * A1, A1, 0.25f * B1 * B1);
      const float e2 = eps + fmaf(c13 * A2, A2, 0.25f * B2 * B2);
      const float s0 = e0 * e0, s1 = e1 * e1, s2 = e2 * e2;
      if (fmaxf(s0, fmaxf(s1, s2)) < 1e14f) {  // as recon_diff<3>, with room for the coefficients
        const float P0 = s1 * s2, P1 = s0 * s2, P2 = s0 * s1;
        const float den = fmaf(3.f, P0, fmaf(6.f, P1, P2));
        const float dent = fmaf(3.f, P2, fmaf(6.f, P1, P0));
        rr = fmaf(3.f * P0, R[0], fmaf(6.f * P1, R[1], P2 * R[2])) * rcpf(den);
        rl = fmaf(P0, Lc[0], fmaf(6.f * P1, Lc[1], 3.f * P2 * Lc[2])) * rcpf(dent);
      } else {
        const float a0 = 0.3f / s0, a1 = 0.6f / s1, a2 = 0.1f / s2;
        const float t0 = 0.1f / s0, t1 = 0.6f / s1, t2 = 0.3f / s2;
        rr = (a0 * R[0] + a1 * R[1] + a2 * R[2]) / (a0 + a1 + a2);
        rl = (t0 * Lc[0] + t1 * Lc[1] + t2 * Lc[2]) / (t0 + t1 + t2);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// G = F(v + a, v + b) - f_base at interface e, for a cell of value v whose left-hand side
// state at the interface is v + a and right-hand side state v + b.  f_base is f(v) for
// Burgers and g(x_L) v for the linear flux, where x_L is the cell's left edge: the part of
// the two interface fluxes that cancels in the cell's flux difference.
//   Lax-Friedrichs (src/hrweno_fluxes.f90:43), Godunov (:67-74).
// ---------------------------------------------------------------------------------------------
// Flux kind as a compile-time constant: FK = 2 * (fn == LINEAR) + (flux == GODUNOV), or
// FK = 4 + (flux == GODUNOV) with the flux function (Burgers or linear) chosen at run time.
template <int FK>
__device__ __forceinline__ float flux_g_t(const LineF& L, float v, float a, float b, float g) {
  if constexpr (FK >= 4) {
    return L.fn == HRW_FN_BURGERS ? flux_g_t<FK - 4>(L, v, a, b, g) : flux_g_t<FK - 2>(L, v, a, b, g);
  } else if constexpr (FK == 0) {  // Burgers, LF: 4F - 2v^2 = a(2v + a + 2 alpha) + b(2v + b - 2 alpha)
    return 0.25f * fmaf(a, 2.f * v + a + 2.f * L.alpha, b * (2.f * v + b - 2.f * L.alpha));
  } else if constexpr (FK == 1) {  // Burgers, Godunov: 2F - v^2 = a(2v + a) or b(2v + b)
    const float fa = a * (2.f * v + a), fb = b * (2.f * v + b);
    return 0.5f * (a <= b ? fminf(fa, fb) : fmaxf(fa, fb));  // min if vm <= vp (a <= b)
  } else if constexpr (FK == 2) {  // linear f = g u, LF: F - g v = ((g + alpha) a + (g - alpha) b)/2
    return 0.5f * fmaf(g + L.alpha, a, (g - L.alpha) * b);
  } else {  // linear, Godunov: g a or g b
    const float fa = g * a, fb = g * b;
    return a <= b ? fminf(fa, fb) : fmaxf(fa, fb);
  }
}
__device__ __forceinline__ int flux_kind(const LineF& L) {
  return 2 * (L.fn != HRW_FN_BURGERS) + (L.flux != HRW_FLUX_LAX_FRIEDRICHS);
}
__device__ __forceinline__ float flux_g(const LineF& L, float v, float a, float b, float g) {
  switch (flux_kind(L)) {
    case 0: return flux_g_t<0>(L, v, a, b, g);
    case 1: return flux_g_t<1>(L, v, a, b, g);
    case 2: return flux_g_t<2>(L, v, a, b, g);
    default: return flux_g_t<3>(L, v, a, b, g);
  }
}
// physical flux minus the same base, for the free-outflow boundary: f(v + a) - f_base
__device__ __forceinline__ float phys_g(const LineF& L, float v, float a, float g) {
  if (L.fn == HRW_FN_BURGERS) return __fmul_rn(__fmul_rn(0.5f, a), __fadd_rn(__fmul_rn(2.f, v), a));
  return __fmul_rn(g, a);
}
// g at interface e (e <= nc < 2^31): the 32-bit conversion stays on the FP32 side; an int64
// to float conversion would run on the narrow FP64 unit
__device__ __forceinline__ float g_at(const LineF& L, int64_t e) {
  return L.b != 0.f ? fmaf(L.b, fmaf(L.rx, __int2float_rn((int)e), L.xmin), L.a) : L.a;
}

// Flux difference F_{j+1/2} - F_{j-1/2} of cell j (value v) from the offsets:
//   left interface:  left state  v + (rr_{j-1} - d_{j-1}),  right state v + rl_j
//   right interface: left state  v + rr_j,                  right state v + (d_j + rl_{j+1})
// with the boundary fluxes of example1...f90:103-104 / example2...f90:117-120.
// NU: a non-uniform line, g at the true edges and g_R - g_L = b width_j per cell
template <bool NU = false>
__device__ __forceinline__ float flux_diff_f32c(const LineF& L, int64_t j, float v, float rr_m,
                                                float d_m, float rl_j, float rr_j, float d_j,
                                                float rl_p) {
  const bool lin = L.fn != HRW_FN_BURGERS;
  const float gL = lin ? (NU ? fmaf(L.b, L.xe[j], L.a) : g_at(L, j)) : 0.f;
  const float gR = lin ? (NU ? fmaf(L.b, L.xe[j + 1], L.a) : g_at(L, j + 1)) : 0.f;
  // G_R - G_L, with the base f(v) (Burgers) or g v (linear) of both interfaces removed; the
  // linear flux adds back (g_R - g_L) v = b rx v (b width_j v on a non-uniform line)
  // every operation between the offsets and G_R - G_L rounded as written (intrinsics): a
  // compiler that contracted one into a neighbouring product would round differently where
  // that product underflows, and the single-line, batched and 2D copies of this arithmetic
  // (inlined into different code) would then disagree
  float GL = flux_g(L, v, __fsub_rn(rr_m, d_m), rl_j, gL);
  float GR = flux_g(L, v, rr_j, __fadd_rn(d_j, rl_p), gR);
  float extra = lin ? (NU ? L.gst[j] : L.gstep) * v : 0.f;
  if (j == 0 || j == L.nc - 1) {
    // boundary fluxes in full (no cancellation there): F = fbase + G, each operation rounded
    // as written (no contraction), so that inlined and out-of-line copies give the same bits
    const float hv = __fmul_rn(__fmul_rn(0.5f, v), v);
    const float fbL = lin ? __fmul_rn(gL, v) : hv, fbR = lin ? __fmul_rn(gR, v) : hv;
    float FL = __fadd_rn(fbL, GL), FR = __fadd_rn(fbR, GR);
    if (L.bc == HRW_BC_COPY) {
      return 0.f;  // F_0 = F_1 or F_nc = F_{nc-1}: the boundary cell's difference vanishes
    }
    if (j == 0) FL = 0.f;
    if (j == L.nc - 1) FR = L.bc == HRW_BC_ZERO ? 0.f : __fadd_rn(fbR, phys_g(L, v, rr_j, gR));
    return __fsub_rn(FR, FL);
  }
  return __fadd_rn(__fsub_rn(GR, GL), extra);  // never contracted with gstep * v
}

// flux_diff_f32c out of line: the warp pass's path for the few threads whose cells touch a
// line end (inlining it into every cell of every specialised pass costs instruction cache
// and compile time for nothing)
static __device__ __noinline__ float flux_diff_f32c_call(const LineF& L, int j, float v, float rr_m,
                                                  float d_m, float rl_j, float rr_j, float d_j,
                                                  float rl_p) {
  return flux_diff_f32c(L, j, v, rr_m, d_m, rl_j, rr_j, d_j, rl_p);
}

// flux_diff_f32c of a cell that touches no boundary, flux kind known at compile time (the same
// operations as flux_diff_f32c's interior branch, so both give the same bits)
template <int FK>
__device__ __forceinline__ float flux_diff_interior(const LineF& L, int j, float v, float rr_m,
                                                    float d_m, float rl_j, float rr_j, float d_j,
                                                    float rl_p) {
  const bool lin = FK >= 4 ? L.fn != HRW_FN_BURGERS : FK >= 2;
  const float gL = lin ? g_at(L, j) : 0.f;
  const float gR = lin ? g_at(L, j + 1) : 0.f;
  const float GL = flux_g_t<FK>(L, v, __fsub_rn(rr_m, d_m), rl_j, gL);
  const float GR = flux_g_t<FK>(L, v, rr_j, __fadd_rn(d_j, rl_p), gR);
  const float extra = lin ? L.gstep * v : 0.f;
  return __fadd_rn(__fsub_rn(GR, GL), extra);
}

// flux_diff_f32c of an interior cell when the flux is Godunov's of f = g(x) u with g > 0 at
// every interface: F = g vm exactly (flux_g_t<3> picks g a for any finite right state, g > 0
// and rounding being monotone), so G_L = g_L (rr_{j-1} - d_{j-1}) and G_R = g_R rr_j, the same
// bits as flux_diff_interior with the right states.  The products are rounded on their own
// (no contraction of G_R - G_L into a multiply-add), as there the min/max stands between them.
__device__ __forceinline__ float flux_diff_upwind(const LineF& L, int j, float v, float rr_m,
                                                  float d_m, float rr_j) {
  const float GL = __fmul_rn(g_at(L, j), __fsub_rn(rr_m, d_m));
  const float GR = __fmul_rn(g_at(L, j + 1), rr_j);
  return __fadd_rn(__fsub_rn(GR, GL), L.gstep * v);
}

// Stage update of one cell in increment form.  h, l: the state u = h + l; dv: the stored
// stage increment (d1 or d2, zero for the first stage); dtL = dt L(v); Lv = L(v).
// Writes the stage output, or the new state pair, as stage kind ST requires.
// h4, l4v, L4v: the multistep history u^{n-4} = h4 + l4v and L(u^{n-4}) (FC_MS only).
template <int ST>
__device__ __forceinline__ void f32c_update_h(const F32CArgs& a, int64_t j, float h, float l,
                                              float dv, float dtL, float Lv, float h4, float l4v,
                                              float L4v) {
  if constexpr (ST == FC_RHS) {
    a.out[j] = Lv;
  } else if constexpr (ST == FC_E1) {
    a.out[j] = dtL;
  } else if constexpr (ST == FC_RK3B) {
    a.out[j] = 0.25f * (dv + dtL);
  } else {
    float inc;
    if constexpr (ST == FC_RK1) {
      inc = dtL;
    } else if constexpr (ST == FC_RK2B) {
      inc = 0.5f * (dv + dtL);
    } else if constexpr (ST == FC_RK3C) {
      inc = (2.f / 3.f) * (dv + dtL);
    } else {  // FC_MS: u' = u + (7 (u4 - u) + 50 dt L + 10 dt L4) / 32
      const float du4 = (h4 - h) + (l4v - l);
      const float dtl4 = fmaf(a.dt_hi, L4v, a.dt_lo * L4v);
      inc = fmaf(7.f / 32.f, du4, fmaf(50.f / 32.f, dtL, (10.f / 32.f) * dtl4));
      a.lout[j] = Lv;
    }
    acc_add(h, l, inc);
    a.hi_out[j] = h;
    a.lo_out[j] = l;
  }
}

template <int ST>
__device__ __forceinline__ void f32c_update(const F32CArgs& a, int64_t j, float h, float l,
                                            float dv, float dtL, float Lv) {
  if constexpr (ST == FC_MS) f32c_update_h<ST>(a, j, h, l, dv, dtL, Lv, a.hi4[j], a.lo4[j], a.l4[j]);
  else f32c_update_h<ST>(a, j, h, l, dv, dtL, Lv, 0.f, 0.f, 0.f);
}

// Warp-synchronous layout (no shared memory): each thread owns C consecutive cells and keeps
// the stencil window of its cells in registers; the k cells on either side come from the
// neighbouring lanes by shuffles, and only lanes 0 and 31 load the warp's halo from memory.
// Own cells are read with float4 loads and written with float4 stores when the thread's
// cells are inside the line (the float buffers are padded to 16-byte aligned slices).
template <int C>
__device__ __forceinline__ void load_cells(const float* __restrict__ p, int j0, int nc, float* out) {
  if (j0 + C <= nc) {
#pragma unroll
    for (int c = 0; c < C; c += 4) {
      const float4 v = *reinterpret_cast<const float4*>(p + j0 + c);
      out[c] = v.x, out[c + 1] = v.y, out[c + 2] = v.z, out[c + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) out[c] = p[j0 + c < nc ? j0 + c : nc - 1];
  }
}

template <int C>
__device__ __forceinline__ void store_cells(float* __restrict__ p, int j0, int nc, const float* v) {
  if (j0 + C <= nc) {
#pragma unroll
    for (int c = 0; c < C; c += 4)
      *reinterpret_cast<float4*>(p + j0 + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c)
      if (j0 + c < nc) p[j0 + c] = v[c];
  }
}

// One warp-pass: lane `lane` handles cells j0 .. j0 + C - 1 of the line a.L (all 32 lanes of
// the warp call it with consecutive j0 = base + lane * C).  FK: the flux kind when known at
// compile time, or -1.  Cell indices are 32-bit (lines of < 2^31 cells).
// ST = -1: the stage kind is the run-time (warp-uniform) `st`, one of the rktvd stages
// FC_RK1 .. FC_RK3C; one copy of the pass then serves every stage of a step (the batched
// kernel runs all stages of a problem in one launch, and per-stage copies would not fit the
// instruction cache).  The per-stage arithmetic is the same as with ST fixed.
// MSR (run-time stage kind only): the run-time path also takes FC_RHS and FC_MS (an mstvd
// batch); without it the code of those two stages stays out of the pass
template <int K, int ST, int C, int FK = -1, bool NU = false, bool MSR = false>
__device__ __forceinline__ void f32c_pass(const F32CArgs& a, int64_t j0l, int lane, int st_rt = ST) {
  static_assert(!NU || FK < 0, "non-uniform lines take the general flux path");
  static_assert(ST != FC_MS || ST >= 0, "");
  const int st = ST >= 0 ? ST : st_rt;
  // the stage writes a.out (the first stages) or the state pair (the last stage)
  const bool to_out = st == FC_RHS || st == FC_E1 || st == FC_RK3B;
  static_assert(C % 4 == 0 && C >= K, "float4 cells and a K-cell shuffle halo");
  const LineF& L = a.L;
  const int nc = L.nc;
  const int j0 = (int)j0l;
  constexpr unsigned FULL = 0xffffffffu;

  // ---- state window: w = cells j0 - K .. j0 + C + K - 1 -----------------------------------------
  float hi[C], lo[C], dv[C];
  load_cells<C>(a.hi, j0, nc, hi);
  load_cells<C>(a.lo, j0, nc, lo);
  if (a.dv) load_cells<C>(a.dv, j0, nc, dv);
  else {
#pragma unroll
    for (int c = 0; c < C; ++c) dv[c] = 0.f;
  }
  float wh[C + 2 * K], wm[C + 2 * K];  // hi and lo + dv of the window
#pragma unroll
  for (int c = 0; c < C; ++c) {
    wh[K + c] = hi[c];
    wm[K + c] = lo[c] + dv[c];
  }
#pragma unroll
  for (int q = 0; q < K; ++q) {
    wh[q] = __shfl_up_sync(FULL, hi[C - K + q], 1);
    wm[q] = __shfl_up_sync(FULL, wm[K + C - K + q], 1);
    wh[K + C + q] = __shfl_down_sync(FULL, hi[q], 1);
    wm[K + C + q] = __shfl_down_sync(FULL, wm[K + q], 1);
  }
  if (lane == 0 || lane == 31) {  // the warp's halo, ghosts replicating v(1) and v(nc)
#pragma unroll
    for (int q = 0; q < K; ++q) {
      int g = lane == 0 ? j0 - K + q : j0 + C + q;
      g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
      const float m = a.dv ? a.lo[g] + a.dv[g] : a.lo[g];
      if (lane == 0) wh[q] = a.hi[g], wm[q] = m;
      else wh[K + C + q] = a.hi[g], wm[K + C + q] = m;
    }
  }

  // ---- compensated differences d[q] = d_{j0 - K + q} and the cells' offsets ----------------------
  float d[C + 2 * K - 1];
#pragma unroll
  for (int q = 0; q < C + 2 * K - 1; ++q) d[q] = (wh[q + 1] - wh[q]) + (wm[q + 1] - wm[q]);
  float rl[C], rr[C];
  constexpr int NCF = K * (K + 1);  // coefficients per cell of a non-uniform line
  if constexpr (NU) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int jc = j0 + c < nc ? j0 + c : nc - 1;
      recon_diff_nu<K>(&d[c + 1], L.cnu + (int64_t)NCF * jc, a.eps, rl[c], rr[c]);
    }
  } else if constexpr (K == 3) {
    // eps + 13/12 (d_m - d_{m-1})^2 once per window position.  Cell c reads d[c+1 .. c+4]
    // (d_{j-2} .. d_{j+1}): its beta0, beta1, beta2 take t[c+4], t[c+3], t[c+2]
    float t[C + 4];
#pragma unroll
    for (int m = 2; m < C + 4; ++m) {
      t[m] = shared_t(d[m - 1], d[m], a.eps);
    }
#pragma unroll
    for (int c = 0; c < C; ++c)
      recon_diff3_shared(&d[c + 1], t[c + 4], t[c + 3], t[c + 2], rl[c], rr[c]);
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) recon_diff<K>(&d[c + 1], a.eps, rl[c], rr[c]);
  }
  // the cells next to the thread's ends: from the neighbouring lanes, or (lanes 0 / 31)
  // reconstructed here: cell j0-1 uses d[0 .. 2K-3], cell j0+C uses d[C+1 .. C+2K-2]
  float ed[2 * K];
#pragma unroll
  for (int q = 0; q < 2 * K - 2; ++q) ed[q] = lane == 31 ? d[C + 1 + q] : d[q];
  float el, er;
  if constexpr (NU) {
    int je = lane == 31 ? j0 + C : j0 - 1;
    je = je < 0 ? 0 : (je >= nc ? nc - 1 : je);
    recon_diff_nu<K>(ed, L.cnu + (int64_t)NCF * je, a.eps, el, er);
  } else if constexpr (K == 3) {
    float te[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) te[q] = shared_t(ed[q], ed[q + 1], a.eps);
    recon_diff3_shared(ed, te[2], te[1], te[0], el, er);
  } else {
    recon_diff<K>(ed, a.eps, el, er);
  }
  const float rr_left = __shfl_up_sync(FULL, rr[C - 1], 1);
  const float rl_right = __shfl_down_sync(FULL, rl[0], 1);
  const float rr_m0 = lane == 0 ? er : rr_left;
  const float rl_pC = lane == 31 ? el : rl_right;

  // ---- flux differences and the stage update -------------------------------------------------------
  const bool interior = j0 > 0 && j0 + C < nc;  // no boundary cell among the thread's cells
  const float* rw = L.rw;
  float o1[C], o2[C], lq[C];  // outputs; lq = L(v) for the multistep history
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int j = j0 + c;
    const float v = wh[K + c] + wm[K + c];
    const float rr_m = c == 0 ? rr_m0 : rr[c - 1];
    const float rl_p = c == C - 1 ? rl_pC : rl[c + 1];
    float dF;
    if constexpr (FK >= 4) {  // the batched kernel: the boundary path out of line
      if (interior)
        dF = flux_diff_interior<FK>(L, j, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p);
      else
        dF = j < nc ? flux_diff_f32c_call(L, j, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p) : 0.f;
    } else if constexpr (FK >= 0) {  // the single-line kernel: inline (a call costs registers)
      if (interior)
        dF = flux_diff_interior<(FK >= 0 ? FK : 0)>(L, j, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p);
      else
        dF = j < nc ? flux_diff_f32c(L, j, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p) : 0.f;
    } else {
      dF = j < nc ? flux_diff_f32c<NU>(L, j, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p) : 0.f;
    }
    const float qj = rw ? -dF * rw[j < nc ? j : nc - 1] : -dF;
    const float dtL = fmaf(a.c_hi, qj, a.c_lo * qj);  // dt L(v)_j
    lq[c] = qj * a.lscale;
    if constexpr (ST >= 0) {
      if constexpr (ST == FC_RHS) {
        o1[c] = lq[c];
      } else if constexpr (ST == FC_E1) {
        o1[c] = dtL;
      } else if constexpr (ST == FC_RK3B) {
        o1[c] = 0.25f * (dv[c] + dtL);
      } else {
        o1[c] = hi[c];
        o2[c] = lo[c];
        if constexpr (ST == FC_RK1) dv[c] = dtL;
        else if constexpr (ST == FC_RK2B) dv[c] = 0.5f * (dv[c] + dtL);
        else if constexpr (ST == FC_RK3C) dv[c] = (2.f / 3.f) * (dv[c] + dtL);
        else dv[c] = dtL;  // FC_MS: completed with the history below
      }
    } else {
      float r;  // the same expressions as the fixed-stage branches above
      if (MSR && st == FC_RHS) r = lq[c];
      else if (st == FC_E1 || st == FC_RK1 || (MSR && st == FC_MS)) r = dtL;  // FC_MS: completed below
      else if (st == FC_RK3B) r = 0.25f * (dv[c] + dtL);
      else if (st == FC_RK2B) r = 0.5f * (dv[c] + dtL);
      else r = (2.f / 3.f) * (dv[c] + dtL);  // FC_RK3C
      if (to_out) {
        o1[c] = r;
      } else {
        o1[c] = hi[c];
        o2[c] = lo[c];
        dv[c] = r;
      }
    }
  }
  if (to_out) {
    store_cells<C>(a.out, j0, nc, o1);
  } else {
    if (ST == FC_MS || (MSR && ST < 0 && st == FC_MS)) {  // u' = u + (7 (u4 - u) + 50 dt L + 10 dt L4) / 32
      float h4[C], l4[C], L4[C];
      load_cells<C>(a.hi4, j0, nc, h4);
      load_cells<C>(a.lo4, j0, nc, l4);
      load_cells<C>(a.l4, j0, nc, L4);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const float du4 = (h4[c] - o1[c]) + (l4[c] - o2[c]);
        const float dtl4 = fmaf(a.dt_hi, L4[c], a.dt_lo * L4[c]);
        dv[c] = fmaf(7.f / 32.f, du4, fmaf(50.f / 32.f, dv[c], (10.f / 32.f) * dtl4));
      }
      store_cells<C>(a.lout, j0, nc, lq);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) acc_add(o1[c], o2[c], dv[c]);
    store_cells<C>(a.hi_out, j0, nc, o1);
    store_cells<C>(a.lo_out, j0, nc, o2);
  }
}

}  // namespace hrw
