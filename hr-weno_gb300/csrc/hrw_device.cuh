// hrw_device.cuh - device building blocks of the fused WENO / flux / TVD stage kernels.
//
// Two numerics modes share every kernel:
//  * FAST (default): the FP64 method with the fewest FP64 instructions.  On GB300 the FP64
//    pipe retires about 2 DFMA per SM-clock, 1/62 of the FP32 rate, so the stage kernels are
//    bound by the count of FP64 instructions, not by HBM.  The WENO weights are evaluated in
//    product form (one reciprocal per cell instead of the twelve divisions of the reference),
//    candidates use integer-scaled stencils, and values shared by neighbouring cells (second
//    differences, candidate stencils) are computed once.  Results agree with the reference
//    to rounding level (a few ulp per stage).
//  * STRICT: the reference's operation order, one IEEE operation at a time with no fused
//    multiply-add, true divisions (src/hrweno_weno.f90:178-214, src/hrweno_fluxes.f90:43,67-74,
//    src/hrweno_tvdode.f90:139-167,257).  Bit-identical to a non-fused CPU build.
#pragma once
#include <cstdint>
#include <type_traits>

#include <cuda_runtime.h>

namespace hrw {

// ------------------------------------------------------------------------------------------
// Reciprocal: PTX rcp.approx.ftz.f64 seed, then one cubic Newton-Raphson step
//   e = 1 - x r,  r' = r (1 + e + e^2)
// (the order-3 member of the Newton iteration family for 1/x; error e^3 of the seed's e).
// Valid for normal x; callers keep x inside [2^-1000, 2^1000].
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double rcp_fast(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  return fma(r, fma(e, e, e), r);
}

// positive doubles order like their high words
__device__ __forceinline__ int hiword(double x) { return __double2hiint(x); }

// ------------------------------------------------------------------------------------------
// One IEEE operation, round to nearest, never fused: the reference-order (STRICT and REAL32)
// arithmetic in either precision.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }

// ------------------------------------------------------------------------------------------
// Reference tables (src/hrweno_weno.f90:11-21) in the real type T: each entry is the quotient
// of two small integers rounded once to T, as the Fortran constant expressions (3._rk/10 ...)
// give.  c(j, r) at [j + k*(r+1)].
// ------------------------------------------------------------------------------------------
template <int K, class T = double> struct Tab;
template <class T> struct Tab<1, T> {
  __device__ static T d(int) { return T(1); }
  __device__ static T c(int, int) { return T(1); }
};
template <class T> struct Tab<2, T> {
  __device__ static T d(int r) { return r == 0 ? T(2) / T(3) : T(1) / T(3); }
  __device__ static T c(int j, int r) {
    const T t[6] = {T(3) / T(2), T(-1) / T(2), T(1) / T(2), T(1) / T(2), T(-1) / T(2), T(3) / T(2)};
    return t[j + 2 * (r + 1)];
  }
};
template <class T> struct Tab<3, T> {
  __device__ static T d(int r) { return r == 0 ? T(3) / T(10) : (r == 1 ? T(6) / T(10) : T(1) / T(10)); }
  __device__ static T c(int j, int r) {
    const T t[12] = {T(11) / T(6), T(-7) / T(6), T(1) / T(3),  T(1) / T(3),  T(5) / T(6),  T(-1) / T(6),
                     T(-1) / T(6), T(5) / T(6),  T(1) / T(3),  T(1) / T(3),  T(-7) / T(6), T(11) / T(6)};
    return t[j + 3 * (r + 1)];
  }
};

// ------------------------------------------------------------------------------------------
// Reference-order reconstruction of one cell (src/hrweno_weno.f90:175-214), in double (STRICT)
// or float (REAL32).  p points at v(i); p[-(K-1)] .. p[K-1] must be valid (ghosts already
// substituted).
// ------------------------------------------------------------------------------------------
template <int K, class T>
__device__ __forceinline__ void recon_strict(const T* p, T eps, T& vl, T& vr) {
  T vrr[K], vlr[K], beta[K];
#pragma unroll
  for (int r = 0; r < K; ++r) {
    T sr = T(0), sl = T(0);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      sr = rn_add(sr, rn_mul(Tab<K, T>::c(j, r), p[j - r]));
      sl = rn_add(sl, rn_mul(Tab<K, T>::c(j, r - 1), p[j - r]));
    }
    vrr[r] = sr;
    vlr[r] = sl;
  }
  if constexpr (K == 1) {
    beta[0] = T(0);
  } else if constexpr (K == 2) {  // (src/hrweno_weno.f90:189-191)
    T a = rn_sub(p[1], p[0]), b = rn_sub(p[0], p[-1]);
    beta[0] = rn_mul(a, a);
    beta[1] = rn_mul(b, b);
  } else {  // (src/hrweno_weno.f90:194-202)
    const T c13 = T(13) / T(12), c14 = T(1) / T(4);
    T a, b;
    a = rn_add(rn_sub(p[0], rn_mul(T(2), p[1])), p[2]);
    b = rn_add(rn_sub(rn_mul(T(3), p[0]), rn_mul(T(4), p[1])), p[2]);
    beta[0] = rn_add(rn_mul(c13, rn_mul(a, a)), rn_mul(c14, rn_mul(b, b)));
    a = rn_add(rn_sub(p[-1], rn_mul(T(2), p[0])), p[1]);
    b = rn_sub(p[-1], p[1]);
    beta[1] = rn_add(rn_mul(c13, rn_mul(a, a)), rn_mul(c14, rn_mul(b, b)));
    a = rn_add(rn_sub(p[-2], rn_mul(T(2), p[-1])), p[0]);
    b = rn_add(rn_sub(p[-2], rn_mul(T(4), p[-1])), rn_mul(T(3), p[0]));
    beta[2] = rn_add(rn_mul(c13, rn_mul(a, a)), rn_mul(c14, rn_mul(b, b)));
  }
  T alfa[K], alfat[K];  // (src/hrweno_weno.f90:207-210)
  T sa = T(0), sat = T(0);
#pragma unroll
  for (int r = 0; r < K; ++r) {
    T e = rn_add(eps, beta[r]);
    T e2 = rn_mul(e, e);
    alfa[r] = rn_div(Tab<K, T>::d(r), e2);
    alfat[r] = rn_div(Tab<K, T>::d(K - 1 - r), e2);
  }
#pragma unroll
  for (int r = 0; r < K; ++r) { sa = rn_add(sa, alfa[r]); sat = rn_add(sat, alfat[r]); }
  T ar = T(0), al = T(0);  // (src/hrweno_weno.f90:213-214)
#pragma unroll
  for (int r = 0; r < K; ++r) {
    ar = rn_add(ar, rn_mul(rn_div(alfa[r], sa), vrr[r]));
    al = rn_add(al, rn_mul(rn_div(alfat[r], sat), vlr[r]));
  }
  vr = ar;
  vl = al;
}

// Out-of-line reference-order path for the rare cells that fail the FAST range guard.
template <int K>
__device__ __noinline__ double2 recon_guarded(double vm2, double vm1, double v0, double vp1,
                                              double vp2, double eps) {
  const double p[5] = {vm2, vm1, v0, vp1, vp2};
  double2 out;
  recon_strict<K>(p + 2, eps, out.x, out.y);  // x = vl, y = vr
  return out;
}

// ------------------------------------------------------------------------------------------
// FAST reconstruction of C consecutive cells held in a register window.
//   w[q] = v(j0 - K + q), q = 0 .. C+2K-1;  cell c (0..C-1) is centred at w[K + c].
// Out: vl[c] = v^+_{j-1/2}, vr[c] = v^-_{j+1/2} of cell j0 + c.
//
// Algebra (k = 3; k = 2 is analogous):
//   s_r = (eps + beta_r)^2,  P_0 = s_1 s_2,  P_1 = s_0 s_2,  P_2 = s_0 s_1
//   alfa_r = d_r / s_r  =>  w_r = d_r P_r / sum_q d_q P_q       (same weights, no division)
//   vr = sum_r d_r P_r vrr_r / sum_r d_r P_r,   vl likewise with d mirrored
// with d = (3, 6, 1)/10 scaled to integers and candidates scaled by 6 (integer stencils).
// Both quotients share one reciprocal of their denominators' product.
// Guard: the product form squares the range of s; cells whose s would overflow it take the
// reference-order path (only for |v| of order 1e18 and above).
// ------------------------------------------------------------------------------------------
template <int K> struct FastGuard;
// products reach ~600 s_max^4 (k=3) and ~18 s_max^2 (k=2): keep s_max below 2^240 / 2^480
template <> struct FastGuard<3> { static constexpr int hi_max = (1023 + 240) << 20; };
template <> struct FastGuard<2> { static constexpr int hi_max = (1023 + 480) << 20; };

// Intermediates of one FAST cell, handed to a tap (the discrete adjoint records what its
// reverse pass needs from them).  k = 3: e_r = eps + beta_r, the weight numerators
// (T0, Q1, P2) of vr and (P0, Q1, T2) of vl, ir = 1/(6 den), il = 1/(6 dent), the x6
// candidates V (vr) and W (vl), the second differences D at centres j+1, j, j-1 and the
// half-B terms E of beta_0..2.  k = 2: e0 = eps + (v1 - v0)^2, e1 = eps + (v0 - v-1)^2,
// s = e^2, ir = 1/(2 den), il = 1/(2 dent), x2 candidates, d0 = v1 - v0, d1 = v0 - v-1.
struct NoTap {};
struct FastCell3 {
  double vr, vl, e0, e1, e2, T0, Q1, P2, P0, T2, ir, il, V0, V1, V2, W0, W1, W2, D0, D1, D2, E0, E1, E2;
};
struct FastCell2 {
  double vr, vl, e0, e1, s0, s1, ir, il, V0, V1, W0, W1, d0, d1;
};

// WL = false computes vr only (vl is left untouched): the upwind flux of a positive velocity
// needs the left state of each interface alone.  A tap other than NoTap (WL = true only) is
// called once per cell: tap.cell(c, FastCell{K}) for FAST cells, tap.guarded(c, v-2, v-1, v0,
// v1, v2, vl, vr) for the cells that took the reference-order path (k = 2: v-2 = v2 = 0).
template <int K, int C, bool WL = true, class Tap = NoTap>
__device__ __forceinline__ void recon_fast(const double* w, double eps, double* vl, double* vr,
                                           const Tap& tap = Tap{}) {
  constexpr bool TAP = !std::is_same<Tap, NoTap>::value;
  if constexpr (K == 1) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      if constexpr (WL) vl[c] = w[1 + c];
      vr[c] = w[1 + c];
    }
  } else if constexpr (K == 2) {
    // V0 = 2 vrr0 = v0 + v1, V1 = 2 vrr1 = 3 v0 - v-1, W0 = 2 vlr0 = 3 v0 - v1,
    // W1 = 2 vlr1 = v-1 + v0 = V0 of the previous cell; beta1 = beta0 of the previous cell.
    double V0p = w[1] + w[2];  // V0 of cell c = -1 (centre q = 1)
    double dp = w[2] - w[1];
    double ep = eps + dp * dp;
    double s0p = ep * ep;  // s0 of cell -1
    double e0p = ep;       // (taps) e0 and d0 of the previous cell
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int q = 2 + c;
      const double V0 = w[q] + w[q + 1];
      const double V1 = fma(3.0, w[q], -w[q - 1]);
      const double W0 = fma(3.0, w[q], -w[q + 1]);
      const double W1 = V0p;
      const double d0 = w[q + 1] - w[q];
      const double e0 = fma(d0, d0, eps);
      const double s0 = e0 * e0, s1 = s0p;
      const double s1x2 = s1 + s1, s0x2 = s0 + s0;
      const double den = s1x2 + s0;    // 2 s1 + s0  (d = (2, 1)/3)
      const double dent = s1 + s0x2;   // s1 + 2 s0  (d mirrored)
      const double num = fma(s1x2, V0, s0 * V1);
      const double numt = fma(s1, W0, s0x2 * W1);
      if (max(hiword(s0), hiword(s1)) < FastGuard<2>::hi_max) {
        if constexpr (WL) {
          const double R = rcp_fast((den + den) * dent);
          vr[c] = num * (dent * R);
          vl[c] = numt * (den * R);
          if constexpr (TAP)
            tap.cell(c, FastCell2{vr[c], vl[c], e0, e0p, s0, s1, dent * R, den * R, V0, V1, W0, W1,
                                  d0, dp});
        } else {
          vr[c] = num * rcp_fast(den + den);
        }
      } else {
        const double2 g = recon_guarded<2>(0.0, w[q - 1], w[q], w[q + 1], 0.0, eps);
        if constexpr (WL) vl[c] = g.x;
        vr[c] = g.y;
        if constexpr (TAP) tap.guarded(c, 0.0, w[q - 1], w[q], w[q + 1], 0.0, g.x, g.y);
      }
      V0p = V0;
      s0p = s0;
      if constexpr (TAP) {
        e0p = e0;
        dp = d0;
      }
    }
  } else {
    // Per centre q, shared by the three cells whose indicators use it:
    //   D(q) = v(q-1) - 2 v(q) + v(q+1),  Ae(q) = eps + 13/12 D(q)^2,  H(q) = (v(q-1) - v(q+1))/2.
    // The indicators' B/2 terms follow from them: E1(j) = H(j), E0(j) = D(j+1) + H(j+1) and
    // E2(j) = D(j-1) - H(j-1), so that eps + beta_r = E_r^2 + Ae(centre of r).
    double A[C + 2], Dm[C + 2], Hm[C + 2];
    const double c13 = 13.0 / 12;
#pragma unroll
    for (int m = 0; m < C + 2; ++m) {  // centre q = m + 2 (cells -1 .. C)
      const int q = m + 2;
      const double D = fma(-2.0, w[q], w[q - 1] + w[q + 1]);
      Dm[m] = D;
      A[m] = fma(c13 * D, D, eps);
      Hm[m] = 0.5 * (w[q - 1] - w[q + 1]);
    }
    // candidates x6: V0 = 2v0 + 5v1 - v2, V1 = -v-1 + 5v0 + 2v1, V2 = 2v-2 - 7v-1 + 11v0,
    // W0 = 11v0 - 7v1 + 2v2, W1 = V0 of previous cell, W2 = V1 of previous cell.
    double V0p = fma(5.0, w[3], fma(2.0, w[2], -w[4]));  // cell -1: centre q = 2
    double V1p = fma(5.0, w[2], fma(2.0, w[3], -w[1]));
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int q = 3 + c;
      const double V0 = fma(5.0, w[q + 1], fma(2.0, w[q], -w[q + 2]));
      const double V1 = fma(5.0, w[q], fma(2.0, w[q + 1], -w[q - 1]));
      const double V2 = fma(11.0, w[q], fma(-7.0, w[q - 1], 2.0 * w[q - 2]));
      const double W0 = fma(11.0, w[q], fma(-7.0, w[q + 1], 2.0 * w[q + 2]));
      const double W1 = V0p, W2 = V1p;
      const double E0 = Dm[c + 2] + Hm[c + 2];  // centre j+1
      const double E1 = Hm[c + 1];               // centre j
      const double E2 = Dm[c] - Hm[c];           // centre j-1
      const double e0 = fma(E0, E0, A[c + 2]);   // eps + beta0
      const double e1 = fma(E1, E1, A[c + 1]);
      const double e2 = fma(E2, E2, A[c]);
      const double s0 = e0 * e0, s1 = e1 * e1, s2 = e2 * e2;
      if (max(max(hiword(s0), hiword(s1)), hiword(s2)) < FastGuard<3>::hi_max) {
        const double P0 = s1 * s2, P1 = s0 * s2, P2 = s0 * s1;
        const double Q1 = 6.0 * P1, T0 = 3.0 * P0, T2 = 3.0 * P2;
        // the sums as explicit fused multiply-adds: no rounding left to the compiler's choice
        // of contraction, so that every kernel that inlines this gets the same bits
        const double den = fma(3.0, P0, fma(6.0, P1, P2));   // d = (3, 6, 1)/10
        const double dent = fma(3.0, P2, fma(6.0, P1, P0));  // d mirrored = (1, 6, 3)/10
        const double num = fma(T0, V0, fma(Q1, V1, P2 * V2));
        if constexpr (WL) {
          const double numt = fma(T2, W2, fma(Q1, W1, P0 * W0));
          const double R = rcp_fast((6.0 * den) * dent);
          vr[c] = num * (dent * R);
          vl[c] = numt * (den * R);
          if constexpr (TAP)
            tap.cell(c, FastCell3{vr[c], vl[c], e0, e1, e2, T0, Q1, P2, P0, T2, dent * R, den * R,
                                  V0, V1, V2, W0, W1, W2, Dm[c + 2], Dm[c + 1], Dm[c], E0, E1, E2});
        } else {
          vr[c] = num * rcp_fast(6.0 * den);
        }
      } else {
        const double2 g = recon_guarded<3>(w[q - 2], w[q - 1], w[q], w[q + 1], w[q + 2], eps);
        if constexpr (WL) vl[c] = g.x;
        vr[c] = g.y;
        if constexpr (TAP) tap.guarded(c, w[q - 2], w[q - 1], w[q], w[q + 1], w[q + 2], g.x, g.y);
      }
      V0p = V0;
      V1p = V1;
    }
  }
}

// single cell, no neighbour sharing (block-edge cells).  Reads p[o * stride] for
// o = -(K-1) .. K-1 only; the two outermost window slots, which a single cell does not use,
// repeat the nearest value.
template <int K>
__device__ __forceinline__ void recon_fast_one(const double* p, double eps, double& vl, double& vr,
                                               int stride = 1) {
  double w[1 + 2 * K];
#pragma unroll
  for (int q = 0; q < 1 + 2 * K; ++q) {
    int o = q - K;
    o = o < -(K - 1) ? -(K - 1) : (o > K - 1 ? K - 1 : o);
    w[q] = p[o * stride];
  }
  double l[1], r[1];
  recon_fast<K, 1>(w, eps, l, r);
  vl = l[0];
  vr = r[0];
}

// Reference-order single cell with a stride: gathers p[o * stride].
template <int K, class T>
__device__ __forceinline__ void recon_strict_strided(const T* p, int stride, T eps, T& vl, T& vr) {
  T w[2 * K - 1];
#pragma unroll
  for (int q = 0; q < 2 * K - 1; ++q) w[q] = p[(q - (K - 1)) * stride];
  recon_strict<K>(w + (K - 1), eps, vl, vr);
}

// ------------------------------------------------------------------------------------------
// Reconstruction of one cell of a non-uniform grid with its coefficients ci(j, r) at
// [j + K*(r+1)] (cnu of src/hrweno_weno.f90:221-297; candidates :177-181).  c0 points at v(i),
// c0[-(K-1)] .. c0[K-1] valid.  FAST: product-form weights as the uniform kernels; STRICT:
// reference order.
// ------------------------------------------------------------------------------------------
template <int K, bool STRICT, class T>
__device__ __forceinline__ void recon_nu(const T* c0, const T* ci, T eps, T& vl, T& vr) {
  T vrr[K], vlr[K], beta[K];
#pragma unroll
  for (int r = 0; r < K; ++r) {
    T sr = T(0), sl = T(0);
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if constexpr (STRICT) {
        sr = rn_add(sr, rn_mul(ci[j + K * (r + 1)], c0[j - r]));
        sl = rn_add(sl, rn_mul(ci[j + K * r], c0[j - r]));
      } else {
        sr = fma(ci[j + K * (r + 1)], c0[j - r], sr);
        sl = fma(ci[j + K * r], c0[j - r], sl);
      }
    }
    vrr[r] = sr;
    vlr[r] = sl;
  }
  if constexpr (STRICT) {
    // beta and the weights do not depend on the grid (src/hrweno_weno.f90:183-214)
    if constexpr (K == 1) {
      beta[0] = T(0);
    } else if constexpr (K == 2) {
      T a = rn_sub(c0[1], c0[0]), b = rn_sub(c0[0], c0[-1]);
      beta[0] = rn_mul(a, a);
      beta[1] = rn_mul(b, b);
    } else {
      const T c13 = T(13) / T(12), c14 = T(1) / T(4);
      T a, b;
      a = rn_add(rn_sub(c0[0], rn_mul(T(2), c0[1])), c0[2]);
      b = rn_add(rn_sub(rn_mul(T(3), c0[0]), rn_mul(T(4), c0[1])), c0[2]);
      beta[0] = rn_add(rn_mul(c13, rn_mul(a, a)), rn_mul(c14, rn_mul(b, b)));
      a = rn_add(rn_sub(c0[-1], rn_mul(T(2), c0[0])), c0[1]);
      b = rn_sub(c0[-1], c0[1]);
      beta[1] = rn_add(rn_mul(c13, rn_mul(a, a)), rn_mul(c14, rn_mul(b, b)));
      a = rn_add(rn_sub(c0[-2], rn_mul(T(2), c0[-1])), c0[0]);
      b = rn_add(rn_sub(c0[-2], rn_mul(T(4), c0[-1])), rn_mul(T(3), c0[0]));
      beta[2] = rn_add(rn_mul(c13, rn_mul(a, a)), rn_mul(c14, rn_mul(b, b)));
    }
    T alfa[K], alfat[K], sa = T(0), sat = T(0);
#pragma unroll
    for (int r = 0; r < K; ++r) {
      const T e = rn_add(eps, beta[r]);
      const T e2 = rn_mul(e, e);
      alfa[r] = rn_div(Tab<K, T>::d(r), e2);
      alfat[r] = rn_div(Tab<K, T>::d(K - 1 - r), e2);
    }
#pragma unroll
    for (int r = 0; r < K; ++r) { sa = rn_add(sa, alfa[r]); sat = rn_add(sat, alfat[r]); }
    T ar = T(0), al = T(0);
#pragma unroll
    for (int r = 0; r < K; ++r) {
      ar = rn_add(ar, rn_mul(rn_div(alfa[r], sa), vrr[r]));
      al = rn_add(al, rn_mul(rn_div(alfat[r], sat), vlr[r]));
    }
    vr = ar;
    vl = al;
  } else {
    if constexpr (K == 1) {
      vr = vrr[0];
      vl = vlr[0];
    } else {
      if constexpr (K == 2) {
        const double a = c0[1] - c0[0], b = c0[0] - c0[-1];
        beta[0] = a * a;
        beta[1] = b * b;
      } else {
        const double c13 = 13.0 / 12;
        double a, b;
        a = fma(-2.0, c0[1], c0[0] + c0[2]);
        b = fma(3.0, c0[0], fma(-4.0, c0[1], c0[2]));
        beta[0] = fma(c13 * a, a, 0.25 * (b * b));
        a = fma(-2.0, c0[0], c0[-1] + c0[1]);
        b = c0[-1] - c0[1];
        beta[1] = fma(c13 * a, a, 0.25 * (b * b));
        a = fma(-2.0, c0[-1], c0[-2] + c0[0]);
        b = fma(3.0, c0[0], fma(-4.0, c0[-1], c0[-2]));
        beta[2] = fma(c13 * a, a, 0.25 * (b * b));
      }
      // product-form weights: w_r = d_r P_r / sum d_q P_q, P_r = prod_{q != r} s_q
      double sq[K], P[K];
      int hmax = 0;
#pragma unroll
      for (int r = 0; r < K; ++r) {
        const double e = eps + beta[r];
        sq[r] = e * e;
        hmax = max(hmax, hiword(sq[r]));
      }
      if (hmax < FastGuard<K>::hi_max) {
#pragma unroll
        for (int r = 0; r < K; ++r) {
          double pr = 1.0;
#pragma unroll
          for (int q = 0; q < K; ++q)
            if (q != r) pr *= sq[q];
          P[r] = pr;
        }
        double den = 0.0, dent = 0.0, num = 0.0, numt = 0.0;
#pragma unroll
        for (int r = 0; r < K; ++r) {
          const double qr = Tab<K>::d(r) * P[r], qt = Tab<K>::d(K - 1 - r) * P[r];
          den += qr;
          dent += qt;
          num = fma(qr, vrr[r], num);
          numt = fma(qt, vlr[r], numt);
        }
        const double R = rcp_fast(den * dent);
        vr = num * (dent * R);
        vl = numt * (den * R);
      } else {
        double alfa[K], alfat[K], sa = 0.0, sat = 0.0, ar = 0.0, al = 0.0;
#pragma unroll
        for (int r = 0; r < K; ++r) {
          alfa[r] = Tab<K>::d(r) / sq[r];
          alfat[r] = Tab<K>::d(K - 1 - r) / sq[r];
          sa += alfa[r];
          sat += alfat[r];
        }
#pragma unroll
        for (int r = 0; r < K; ++r) {
          ar += alfa[r] / sa * vrr[r];
          al += alfat[r] / sat * vlr[r];
        }
        vr = ar;
        vl = al;
      }
    }
  }
}

}  // namespace hrw
