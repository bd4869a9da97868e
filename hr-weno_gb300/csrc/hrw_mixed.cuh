// hrw_mixed.cuh - device building blocks of the MIXED numerics mode of the 1D stage kernel
// (stage1d_mixed.cu).
//
// MIXED keeps the FP64 state of the method and computes each stage's right-hand side in
// *difference form* on the FP32 pipe, which on GB300 retires 64 times more instructions per
// clock than the FP64 pipe:
//
//  * neighbour differences d_q = u_{q+1} - u_q are formed in FP64 (one subtraction per cell,
//    exact whenever neighbours are within a factor of two) and split into float pairs with
//    integer operations (no FP64 arithmetic);
//  * the linear-weight part of the reconstruction enters each cell's flux difference through
//    two stencil sums S and T, carried in float-pair precision;
//  * the WENO weights enter only through their deviations from the linear weights,
//    delta_r = w_r - d_r, computed in FP32 from factored differences of the smoothness
//    indicators (src/hrweno_weno.f90:183-210 rewritten in differences, the same method);
//  * stage values are stored as float-pair increments from u; the last stage adds its
//    increment to u in FP64.
//
// Where the FP32 parts could move a result by more than 2^-53 max|u| per stage (steep or
// under-resolved data, the line ends, values outside [2^-40, 2^60]) the whole warp runs the
// FAST FP64 arithmetic instead; each warp's decision rests on a bound of its own rounding
// errors, evaluated from the data (mx_bound below).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace hrw {
namespace mx {

struct F2 {
  float h, l;
};

// ---- exact conversions by integer operations ------------------------------------------------

// d = h + l to 2^-48 |d|: h = fl32(d) (round to nearest even), l = fl32(d - h).  The residual
// d - h is read off d's low mantissa bits, so no FP64 arithmetic is spent.  |d| < 2^-126 gives
// (0, 0); |d| < 2^-74 gives l = 0 (callers keep such d below their error budget).
__device__ __forceinline__ F2 split(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const int E = (int)((hi >> 20) & 0x7FFu);
  F2 r;
  r.h = __double2float_rn(d);
  const unsigned L29 = lo & 0x1FFFFFFFu;
  // fl32 rounded the magnitude up when the dropped 29 bits exceed half an ulp, or equal it
  // with an odd kept bit (ties to even)
  const bool up = L29 > 0x10000000u || (L29 == 0x10000000u && (lo & 0x20000000u));
  const int rem = (int)L29 - (up ? 0x20000000 : 0);
  // 2^(E - 1075) as a float (normal for E >= 949)
  const float scale = __int_as_float((E - 948) << 23);
  float l = __int2float_rn(rem) * scale;
  l = __int_as_float(__float_as_int(l) ^ (int)(hi & 0x80000000u));
  r.l = E >= 949 ? l : 0.f;
  if (E < 897) r.h = 0.f;
  return r;
}

// The same split with h = d truncated to 24 significant bits, by integer operations alone
// (the FP64-to-FP32 conversion of split() shares the narrow FP64 unit's issue slots):
// h takes d's sign, exponent and top 23 stored mantissa bits; l = fl32 of the 29 bits below
// them.  d = h + l to 2^-47 |d|; |d| < 2^-126 gives (0, 0); |d| < 2^-74 gives l = 0.  Valid for
// |d| < 2^127 (callers keep |d| far below).
__device__ __forceinline__ F2 split_t(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const int E = (int)((hi >> 20) & 0x7FFu);
  // bits 30..23 of the funnel shift are E's low 8 bits; for 897 <= E <= 1150 the float's
  // exponent field E - 896 equals them with the top bit flipped
  const unsigned f = __funnelshift_l(lo, hi, 3);
  F2 r;
  r.h = __uint_as_float(((f ^ 0x40000000u) & 0x7FFFFFFFu) | (hi & 0x80000000u));
  const float scale = __int_as_float((E - 948) << 23);  // 2^(E - 1075), normal for E >= 949
  float l = __uint2float_rn(lo & 0x1FFFFFFFu) * scale;
  l = __uint_as_float(__float_as_uint(l) | (hi & 0x80000000u));
  r.l = E >= 949 ? l : 0.f;
  if (E < 897) r.h = 0.f;
  return r;
}

// The double of a normal float (or zero) by integer operations (cvt.f64.f32 runs on the
// narrow FP64 unit).  Subnormal floats give zero.
__device__ __forceinline__ double widen(float f) {
  const unsigned b = (unsigned)__float_as_int(f);
  const unsigned mag = b & 0x7FFFFFFFu;
  const unsigned hi = mag >= 0x00800000u ? ((mag >> 3) + 0x38000000u) | (b & 0x80000000u) : (b & 0x80000000u);
  const unsigned lo = mag >= 0x00800000u ? b << 29 : 0u;
  return __hiloint2double((int)hi, (int)lo);
}

// The double nearest (within 2^-52 |h + l|) to a normalised pair h + l (|l| <= ulp(h) / 2) by
// integer operations: the FP64 pattern of h, plus l counted in units of h's FP64 ulp
// 2^(e_h - 52) (at most 2^28 of them).  Below a power of two the ulp halves, so a negative step
// from a power of two counts double.  |h| < 2^-70: l is dropped.
__device__ __forceinline__ double pack(F2 p) {
  const unsigned hb = (unsigned)__float_as_int(p.h);
  const int eb = (int)((hb >> 23) & 0xFFu);  // biased exponent of h
  const float scale = __int_as_float(min(max(52 - (eb - 127) + 127, 1), 254) << 23);
  int k = __float2int_rn(p.l * scale);       // l / 2^(e_h - 52)
  k = eb >= 57 ? k : 0;
  if (hb & 0x80000000u) k = -k;               // the pattern counts magnitudes
  if ((hb & 0x7FFFFFu) == 0 && k < 0) k *= 2;
  return __longlong_as_double(__double_as_longlong(widen(p.h)) + (long long)k);
}

// ---- float-pair arithmetic -------------------------------------------------------------------

// error-free sum: s + e == a + b
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (h, l) renormalised so that |l| <= ulp(h) / 2 (|l| no larger than about ulp(h) on entry)
__device__ __forceinline__ F2 renorm(float h, float l) {
  F2 r;
  r.h = __fadd_rn(h, l);
  r.l = __fsub_rn(l, __fsub_rn(r.h, h));
  return r;
}

__device__ __forceinline__ F2 add(F2 a, F2 b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  return renorm(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}

// a * b, both pairs (the l * l term, below 2^-48 |ab|, is dropped)
__device__ __forceinline__ F2 mul(F2 a, F2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return renorm(p, e);
}

// 1/x by the MUFU approximation (about 1 ulp); x positive and normal.  The weight deviations
// need no better: their error bound carries a few ulps of relative error.
__device__ __forceinline__ float rcp(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// ---- per-cell reconstruction in difference form -----------------------------------------------

// One cell's reconstruction, relative to the cell value v_j:
//   rr = vr_j - v_j, rl = vl_j - v_j (FP32, for the quadratic flux terms),
//   rrn, rln: their nonlinear parts sum_r (w_r - d_r)(q_r - v_j) (FP32),
//   dev: sum of |w_r - d_r| over both weight sets (for the error bound).
struct Rec {
  float rr, rl, rrn, rln, dev;
};

// k = 3.  d[0..3] = d_{j-2}, d_{j-1}, d_j, d_{j+1}; D[0..2] = Dd_{j-2}, Dd_{j-1}, Dd_j (second
// differences Dd_q = d_{q+1} - d_q); tA[0..2] = eps + 13/12 Dd^2 of the same three.
// In these variables (src/hrweno_weno.f90:19-21,194-202): the candidates x6 minus 6 v_j are
//   R0 = 4 d0 - d1, R1 = 2 d0 + dm, R2 = 5 dm - 2 dmm;  L0 = 2 d1 - 5 d0, L1 = -(2 dm + d0),
//   L2 = dmm - 4 dm;  beta_r = 13/12 A_r^2 + 1/4 B_r^2 with A0 = Dd_j, A1 = Dd_{j-1},
//   A2 = Dd_{j-2}, B0 = d1 - 3 d0, B1 = dm + d0, B2 = 3 dm - dmm.
// With s_r = (eps + beta_r)^2, P_0 = s1 s2, P_1 = s0 s2, P_2 = s0 s1 and d = (3, 6, 1)/10, the
// weight deviations are exact rational functions of the indicator differences:
//   w_0 - d_0 = 3 (6 (s1 - s0) s2 + (s2 - s0) s1) / (10 Dp),  Dp = 3 P0 + 6 P1 + P2
//   w_2 - d_2 = -(3 (s2 - s0) s1 + 6 (s2 - s1) s0) / (10 Dp)
// (w_1 - d_1 = -(the other two)), and likewise for the mirrored weights d~ = (1, 6, 3)/10.
// The indicator differences factor as
//   beta1 - beta0 = (A1 - A0) (13/12 (A1 + A0) - 1/4 (dm + 3 d0 - A0))
//   beta2 - beta1 = (A2 - A1) (13/12 (A2 + A1) + 1/4 (A2 + 3 dm + d0))
// so that they come out accurate to FP32 precision relative to themselves, not to beta.
__device__ __forceinline__ Rec rec3(const float* d, const float* D, const float* tA) {
  const float dmm = d[0], dm = d[1], d0 = d[2], d1 = d[3];
  const float A2 = D[0], A1 = D[1], A0 = D[2];
  const float B0 = fmaf(-2.f, d0, A0), B1 = dm + d0, B2 = fmaf(2.f, dm, A2);
  const float e0 = fmaf(0.25f * B0, B0, tA[2]);
  const float e1 = fmaf(0.25f * B1, B1, tA[1]);
  const float e2 = fmaf(0.25f * B2, B2, tA[0]);
  const float a10 = A1 - A0, a21 = A2 - A1;
  const float b10 = a10 * fmaf(13.f / 12.f, A1 + A0, -0.25f * (fmaf(3.f, d0, dm) - A0));
  const float b21 = a21 * fmaf(13.f / 12.f, A2 + A1, 0.25f * fmaf(3.f, dm, A2 + d0));
  const float b20 = b21 + b10;
  const float s0 = e0 * e0, s1 = e1 * e1, s2 = e2 * e2;
  const float q10 = b10 * (e1 + e0), q20 = b20 * (e2 + e0), q21 = b21 * (e2 + e1);
  const float P0 = s1 * s2, P1 = s0 * s2, P2 = s0 * s1;
  const float rD = rcp(fmaf(3.f, P0, fmaf(6.f, P1, P2)));
  const float rDt = rcp(fmaf(3.f, P2, fmaf(6.f, P1, P0)));
  const float u20 = q20 * s1, u10 = q10 * s2, u21 = q21 * s0;
  const float N0 = fmaf(6.f, u10, u20), N2 = -fmaf(6.f, u21, 3.f * u20);
  const float M0 = fmaf(6.f, u10, 3.f * u20), M2 = -fmaf(6.f, u21, u20);
  Rec r;
  // rr_nl = (delta_0 (R0 - R1) + delta_2 (R2 - R1)) / 6, R0 - R1 = A1 - A0, R2 - R1 = 2 (A2 - A1)
  r.rrn = fmaf(3.f * N0, a10, 2.f * N2 * a21) * (rD * (1.f / 60.f));
  // rl_nl = (delta~_0 (L0 - L1) + delta~_2 (L2 - L1)) / 6, L0 - L1 = 2 (A0 - A1), L2 - L1 = A1 - A2
  r.rln = fmaf(-2.f * M0, a10, -3.f * M2 * a21) * (rDt * (1.f / 60.f));
  r.dev = (fmaf(3.f, fabsf(N0), fabsf(N2)) * rD + fmaf(3.f, fabsf(M2), fabsf(M0)) * rDt) * 0.2f;
  // linear weights: (24 d0 - 3 d1 + 11 dm - 2 dmm) / 60 and (2 d1 - 11 d0 - 24 dm + 3 dmm) / 60
  const float rlin = fmaf(24.f, d0, fmaf(-3.f, d1, fmaf(11.f, dm, -2.f * dmm))) * (1.f / 60.f);
  const float llin = fmaf(2.f, d1, fmaf(-11.f, d0, fmaf(-24.f, dm, 3.f * dmm))) * (1.f / 60.f);
  r.rr = rlin + r.rrn;
  r.rl = llin + r.rln;
  return r;
}

// The linear-weight parts of rr and rl alone (FP32): k = 3 (24 d0 - 3 d1 + 11 dm - 2 dmm) / 60 and
// (2 d1 - 11 d0 - 24 dm + 3 dmm) / 60 with d as in rec3; k = 2 d0/3 + dm/6 and -(d0/6 + dm/3) with
// d as in rec2.  rec3 and rec2 add the nonlinear parts to these.
template <int K>
__device__ __forceinline__ void lin(const float* d, float& rr, float& rl) {
  if constexpr (K == 3) {
    const float dmm = d[0], dm = d[1], d0 = d[2], d1 = d[3];
    rr = fmaf(24.f, d0, fmaf(-3.f, d1, fmaf(11.f, dm, -2.f * dmm))) * (1.f / 60.f);
    rl = fmaf(2.f, d1, fmaf(-11.f, d0, fmaf(-24.f, dm, 3.f * dmm))) * (1.f / 60.f);
  } else {
    const float dm = d[0], d0 = d[1];
    rr = fmaf(1.f / 3.f, d0, (1.f / 6.f) * dm);
    rl = -fmaf(1.f / 6.f, d0, (1.f / 3.f) * dm);
  }
}

// k = 2.  d[0..1] = d_{j-1}, d_j; D[0] = Dd_{j-1} = d_j - d_{j-1}.  Candidates minus v_j:
// vrr0 - v = d0/2, vrr1 - v = dm/2, vlr0 - v = -d0/2, vlr1 - v = -dm/2 (src/hrweno_weno.f90:
// 16-18); beta0 = d0^2, beta1 = dm^2 (:189-191); d = (2, 1)/3, d~ = (1, 2)/3.  With
// s_r = (eps + beta_r)^2: w0 - 2/3 = 2 (s1 - s0) / (3 (2 s1 + s0)),
// w~0 - 1/3 = 2 (s1 - s0) / (3 (s1 + 2 s0)), s1 - s0 = (dm - d0)(dm + d0)(e0 + e1).
__device__ __forceinline__ Rec rec2(const float* d, const float* D, float eps) {
  const float dm = d[0], d0 = d[1], A = D[0];
  const float e0 = fmaf(d0, d0, eps), e1 = fmaf(dm, dm, eps);
  const float s0 = e0 * e0, s1 = e1 * e1;
  const float q10 = -A * (dm + d0) * (e0 + e1);
  const float rD = rcp(fmaf(2.f, s1, s0)), rDt = rcp(fmaf(2.f, s0, s1));
  Rec r;
  // rr_nl = (w0 - 2/3)(d0 - dm)/2, rl_nl = (w~0 - 1/3)(dm - d0)/2
  r.rrn = q10 * A * rD * (1.f / 3.f);
  r.rln = -q10 * A * rDt * (1.f / 3.f);
  r.dev = fabsf(q10) * (rD + rDt) * (4.f / 3.f);
  r.rr = fmaf(1.f / 3.f, d0, (1.f / 6.f) * dm) + r.rrn;
  r.rl = -fmaf(1.f / 6.f, d0, (1.f / 3.f) * dm) + r.rln;
  return r;
}

}  // namespace mx
}  // namespace hrw
