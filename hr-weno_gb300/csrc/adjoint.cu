// adjoint.cu - discrete adjoint of WENO reconstruction + global Lax-Friedrichs flux + rktvd(3)
// for J = 0.5 ||u(T) - u_target||^2, with checkpointed recompute (hrw_adjoint_* in
// include/hrweno_gpu.h).  No counterpart in the reference, which has no derivatives.
//
// Forward map of one step (src/hrweno_tvdode.f90:161-169) with L the example1 right-hand side
// (example/example1_burgers_1d_fv.f90:72-109) and the fixed-alpha LF flux
// (src/hrweno_fluxes.f90:43):
//   u1 = u + dt L(u),  u2 = 3/4 u + 1/4 (u1 + dt L(u1)),  u' = 1/3 u + 2/3 (u2 + dt L(u2)).
// Its transpose, given lambda' = dJ/du':
//   A3: l2 = 2/3 (lambda' + dt J(u2)^T lambda'),     acc = 1/3 lambda'
//   A2: l1 = 1/4 (l2 + dt J(u1)^T l2),               acc += 3/4 l2
//   A1: lambda = acc + l1 + dt J(u)^T l1
// where J(v)^T mu is the vector-Jacobian product of L.  It is assembled per cell i from the
// adjoints of its two reconstructed states, ar_i = dF_{i+1/2}/dvr_i * phi_{i+1/2} and
// al_i = dF_{i-1/2}/dvl_i * phi_{i-1/2} (phi = the flux adjoint from mu and the boundary
// rules), pushed back through the WENO map: the candidates are linear, the weights
// w_r = alpha_r / sum(alpha) with alpha_r = d_r/(eps + beta_r)^2 give
//   d vr / d beta_s = -2 w_s (q_s - vr) / (eps + beta_s),
// and the smoothness indicators are quadratic forms.  eps > 0 keeps all of this smooth.
//
// Lines are segment-aware: the state holds nseg independent problems of `seg` cells each,
// every segment with its own boundaries and ghost cells, so one launch serves one long line
// or a batch of equal-size problems.
#include <algorithm>
#include <cmath>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"
#include "hrw_stage.cuh"

// Launch shapes (compile-time; measured on the 2^20-cell line): cells per thread of the
// forward stage without and with the WENO tape, their minimum resident blocks per SM, and the
// cells per block of the reverse stage.
#ifndef HRW_ADJ_FWD_C
#define HRW_ADJ_FWD_C 8
#endif
#ifndef HRW_ADJ_FWD_MINB
#define HRW_ADJ_FWD_MINB 1
#endif
#ifndef HRW_ADJ_TAPE_C
#define HRW_ADJ_TAPE_C 4
#endif
#ifndef HRW_ADJ_TAPE_MINB
#define HRW_ADJ_TAPE_MINB 1
#endif
#ifndef HRW_ADJ_VJP_NT
#define HRW_ADJ_VJP_NT 256
#endif

namespace hrw {

namespace {

constexpr unsigned FULL = 0xffffffffu;

struct AdjLine {
  int64_t n;    // total cells
  int64_t seg;  // cells per problem (segment)
  int k, fn, bc;
  double a, b, alpha, xmin, rx, rdx, eps;
  double rws0;  // FAST flux scale / dx (stage kernels)
  // a non-uniform line (xedges), the same for every segment, by local cell: the weno
  // coefficients cnu (k (k + 1) per cell), 1 / width, the FAST flux scale / width, and the
  // edges (seg + 1); null on a uniform line
  const double* cnu;
  const double* rdxv;
  const double* rwsv;
  const double* xe;
};

__device__ __forceinline__ LineArgs line_args(const AdjLine& A) {
  LineArgs L{};
  L.nc = (int)A.seg;
  L.fn = A.fn;
  L.bc = A.bc;
  L.flux = HRW_FLUX_LAX_FRIEDRICHS;
  L.a = A.a;
  L.b = A.b;
  L.alpha = A.alpha;
  L.xmin = A.xmin;
  L.rx = A.rx;
  L.rws0 = A.rws0;
  L.xe = A.xe;
  L.rws = A.rwsv;
  return L;
}

// --------------------------------------------------------------------------------------------
// WENO of one cell in division form with everything the reverse pass needs, then the reverse
// pass: given ar (adjoint of vr) and al (adjoint of vl), add d(ar vr + al vl)/dp into
// out[0 .. 2K-2] for the stencil p[-(K-1) .. K-1].
// --------------------------------------------------------------------------------------------
template <int K> struct WenoTape;
template <> struct WenoTape<1> {
  double vr, vl;
  __device__ void fwd(const double* p, double) { vr = vl = p[0]; }
  __device__ void rev(double ar, double al, double* out) const { out[0] += ar + al; }
};
template <> struct WenoTape<2> {
  // stencil v_{-1}, v_0, v_1; q0 = (v0 + v1)/2, q1 = (3 v0 - v_{-1})/2; vl: r0 = (3 v0 - v1)/2,
  // r1 = (v_{-1} + v0)/2; beta0 = (v1 - v0)^2, beta1 = (v0 - v_{-1})^2; d = (2, 1)/3
  double vr, vl, D0, D1, ie0, ie1, w0, w1, u0, u1, q0, q1, r0, r1;
  __device__ void fwd(const double* p, double eps) {
    const double vm = p[-1], v0 = p[0], v1 = p[1];
    D0 = v1 - v0, D1 = v0 - vm;
    ie0 = rcp_fast(fma(D0, D0, eps)), ie1 = rcp_fast(fma(D1, D1, eps));
    const double s0 = ie0 * ie0, s1 = ie1 * ie1;
    const double iS = rcp_fast(fma(2.0, s0, s1)), iT = rcp_fast(fma(2.0, s1, s0));
    w0 = 2.0 * s0 * iS, w1 = s1 * iS, u0 = s0 * iT, u1 = 2.0 * s1 * iT;
    q0 = 0.5 * (v0 + v1), q1 = 0.5 * fma(3.0, v0, -vm);
    r0 = 0.5 * fma(3.0, v0, -v1), r1 = 0.5 * (vm + v0);
    vr = fma(w0, q0, w1 * q1), vl = fma(u0, r0, u1 * r1);
  }
  __device__ void rev(double ar, double al, double* out) const {
    // dbeta_s = -2 [ar w_s (q_s - vr) + al u_s (r_s - vl)] / (eps + beta_s)
    const double db0 = -2.0 * ie0 * fma(ar * w0, q0 - vr, al * u0 * (r0 - vl));
    const double db1 = -2.0 * ie1 * fma(ar * w1, q1 - vr, al * u1 * (r1 - vl));
    const double dq0 = ar * w0, dq1 = ar * w1, dr0 = al * u0, dr1 = al * u1;
    const double g0 = 2.0 * D0 * db0, g1 = 2.0 * D1 * db1;
    out[0] += fma(-0.5, dq1, fma(0.5, dr1, -g1));
    out[1] += fma(0.5, dq0 + dr1, fma(1.5, dq1 + dr0, g1 - g0));
    out[2] += fma(0.5, dq0 - dr0, g0);
  }
};
template <> struct WenoTape<3> {
  // stencil v_{-2} .. v_2; candidates x6 (c3 table, src/hrweno_weno.f90:19-21); indicators
  // 13/12 A_s^2 + 1/4 B_s^2 (:194-202); weights d = (3, 6, 1)/10 and mirrored (:207-210)
  double vr, vl, A0, B0, A1, B1, A2, B2, ie0, ie1, ie2, w0, w1, w2, u0, u1, u2;
  double q0, q1, q2, r0, r1, r2;  // x6
  __device__ void fwd(const double* p, double eps) {
    const double vmm = p[-2], vm = p[-1], v0 = p[0], v1 = p[1], v2 = p[2];
    A0 = fma(-2.0, v1, v0 + v2), B0 = fma(3.0, v0, fma(-4.0, v1, v2));
    A1 = fma(-2.0, v0, vm + v1), B1 = vm - v1;
    A2 = fma(-2.0, vm, vmm + v0), B2 = fma(3.0, v0, fma(-4.0, vm, vmm));
    const double c13 = 13.0 / 12.0;
    ie0 = rcp_fast(eps + fma(c13 * A0, A0, 0.25 * B0 * B0));
    ie1 = rcp_fast(eps + fma(c13 * A1, A1, 0.25 * B1 * B1));
    ie2 = rcp_fast(eps + fma(c13 * A2, A2, 0.25 * B2 * B2));
    const double s0 = ie0 * ie0, s1 = ie1 * ie1, s2 = ie2 * ie2;
    const double S1 = 6.0 * s1;
    const double iS = rcp_fast(fma(3.0, s0, S1 + s2)), iT = rcp_fast(fma(3.0, s2, S1 + s0));
    w0 = 3.0 * s0 * iS, w1 = S1 * iS, w2 = s2 * iS;
    u0 = s0 * iT, u1 = S1 * iT, u2 = 3.0 * s2 * iT;
    q0 = fma(5.0, v1, fma(2.0, v0, -v2)), q1 = fma(5.0, v0, fma(2.0, v1, -vm));
    q2 = fma(11.0, v0, fma(-7.0, vm, 2.0 * vmm));
    r0 = fma(11.0, v0, fma(-7.0, v1, 2.0 * v2)), r1 = fma(5.0, v0, fma(2.0, vm, -v1));
    r2 = fma(5.0, vm, fma(2.0, v0, -vmm));
    vr = fma(w0, q0, fma(w1, q1, w2 * q2)) * (1.0 / 6.0);
    vl = fma(u0, r0, fma(u1, r1, u2 * r2)) * (1.0 / 6.0);
  }
  __device__ void rev(double ar, double al, double* out) const {
    const double vr6 = 6.0 * vr, vl6 = 6.0 * vl;
    const double arw = ar * (1.0 / 6.0), alw = al * (1.0 / 6.0);
    const double db0 = -2.0 * ie0 * fma(arw * w0, q0 - vr6, alw * u0 * (r0 - vl6));
    const double db1 = -2.0 * ie1 * fma(arw * w1, q1 - vr6, alw * u1 * (r1 - vl6));
    const double db2 = -2.0 * ie2 * fma(arw * w2, q2 - vr6, alw * u2 * (r2 - vl6));
    const double dq0 = arw * w0, dq1 = arw * w1, dq2 = arw * w2;
    const double dr0 = alw * u0, dr1 = alw * u1, dr2 = alw * u2;
    // d beta_s = 13/6 A_s grad(A_s) + 1/2 B_s grad(B_s); grad A0 = (0,0,1,-2,1),
    // B0 = (0,0,3,-4,1); A1 = (0,1,-2,1,0), B1 = (0,1,0,-1,0); A2 = (1,-2,1,0,0), B2 = (1,-4,3,0,0)
    const double gA0 = (13.0 / 6.0) * A0 * db0, gB0 = 0.5 * B0 * db0;
    const double gA1 = (13.0 / 6.0) * A1 * db1, gB1 = 0.5 * B1 * db1;
    const double gA2 = (13.0 / 6.0) * A2 * db2, gB2 = 0.5 * B2 * db2;
    out[0] += fma(2.0, dq2, gA2 + gB2 - dr2);
    out[1] += fma(-7.0, dq2, fma(2.0, dr1, fma(5.0, dr2, fma(-2.0, gA2, fma(-4.0, gB2, gA1 + gB1 - dq1)))));
    out[2] += fma(2.0, dq0, fma(5.0, dq1 + dr1, fma(11.0, dq2 + dr0, fma(2.0, dr2,
              fma(3.0, gB0 + gB2, fma(-2.0, gA1, gA0 + gA2))))));
    out[3] += fma(5.0, dq0, fma(2.0, dq1, fma(-7.0, dr0, fma(-2.0, gA0, fma(-4.0, gB0, gA1 - gB1 - dr1)))));
    out[4] += fma(2.0, dr0, gA0 + gB0 - dq0);
  }
};

// --------------------------------------------------------------------------------------------
// The same map on a non-uniform line: the candidates take the cell's own coefficients ci
// (cnu(j, r) at [j + K (r + 1)], src/hrweno_weno.f90:177-181), the indicators and weights are
// the uniform ones (:183-210).  Division form throughout; the reverse pushes the candidates'
// adjoints back through ci and the indicators' through their quadratic forms.
// --------------------------------------------------------------------------------------------
template <int K> struct WenoTapeNu {
  double vr, vl, q[K], r[K], w[K], u[K], ie[K], G[K][2];  // G: the indicators' A, B (K = 3), D (K = 2)
  const double* ci;
  __device__ void fwd(const double* p, double eps, const double* c) {
    ci = c;
#pragma unroll
    for (int s = 0; s < K; ++s) {
      double sq = 0.0, sr = 0.0;
#pragma unroll
      for (int j = 0; j < K; ++j) {
        sq = fma(ci[j + K * (s + 1)], p[j - s], sq);
        sr = fma(ci[j + K * s], p[j - s], sr);
      }
      q[s] = sq;
      r[s] = sr;
    }
    double beta[K];
    if constexpr (K == 1) {
      beta[0] = 0.0;
    } else if constexpr (K == 2) {
      G[0][0] = p[1] - p[0], G[1][0] = p[0] - p[-1];
      beta[0] = G[0][0] * G[0][0], beta[1] = G[1][0] * G[1][0];
    } else {
      const double vmm = p[-2], vm = p[-1], v0 = p[0], v1 = p[1], v2 = p[2];
      G[0][0] = fma(-2.0, v1, v0 + v2), G[0][1] = fma(3.0, v0, fma(-4.0, v1, v2));
      G[1][0] = fma(-2.0, v0, vm + v1), G[1][1] = vm - v1;
      G[2][0] = fma(-2.0, vm, vmm + v0), G[2][1] = fma(3.0, v0, fma(-4.0, vm, vmm));
#pragma unroll
      for (int s = 0; s < 3; ++s) beta[s] = fma((13.0 / 12.0) * G[s][0], G[s][0], 0.25 * G[s][1] * G[s][1]);
    }
    double sa = 0.0, st = 0.0;
#pragma unroll
    for (int s = 0; s < K; ++s) {
      ie[s] = 1.0 / (eps + beta[s]);
      w[s] = Tab<K>::d(s) * ie[s] * ie[s];
      u[s] = Tab<K>::d(K - 1 - s) * ie[s] * ie[s];
      sa += w[s];
      st += u[s];
    }
    vr = 0.0, vl = 0.0;
#pragma unroll
    for (int s = 0; s < K; ++s) {
      w[s] /= sa;
      u[s] /= st;
      vr = fma(w[s], q[s], vr);
      vl = fma(u[s], r[s], vl);
    }
  }
  // out[0 .. 2K-2] += d(ar vr + al vl)/dp for p[-(K-1) .. K-1]
  __device__ void rev(double ar, double al, double* out) const {
#pragma unroll
    for (int s = 0; s < K; ++s) {
      const double dq = ar * w[s], dr = al * u[s];
#pragma unroll
      for (int j = 0; j < K; ++j) out[K - 1 + j - s] += fma(dq, ci[j + K * (s + 1)], dr * ci[j + K * s]);
      if constexpr (K > 1) {
        // d beta_s = -2 [ar w_s (q_s - vr) + al w~_s (r_s - vl)] / (eps + beta_s)
        const double db = -2.0 * ie[s] * fma(dq, q[s] - vr, dr * (r[s] - vl));
        if constexpr (K == 2) {  // beta_s = D_s^2: D0 = p1 - p0, D1 = p0 - p_{-1}
          const double g = 2.0 * G[s][0] * db;
          out[2 - s] += g;
          out[1 - s] -= g;
        } else {  // 13/12 A_s^2 + 1/4 B_s^2 with the gradients of WenoTape<3>::rev
          const double gA = (13.0 / 6.0) * G[s][0] * db, gB = 0.5 * G[s][1] * db;
          if (s == 0) {
            out[2] += gA + 3.0 * gB, out[3] += -2.0 * gA - 4.0 * gB, out[4] += gA + gB;
          } else if (s == 1) {
            out[1] += gA + gB, out[2] += -2.0 * gA, out[3] += gA - gB;
          } else {
            out[0] += gA + gB, out[1] += -2.0 * gA - 4.0 * gB, out[2] += gA + 3.0 * gB;
          }
        }
      }
    }
  }
};

// --------------------------------------------------------------------------------------------
// WENO tape: per cell and forward stage, what the reverse pass needs of the cell's WENO map,
// so that the reverse does not recompute it.  With ar, al the adjoints of vr, vl:
//   d beta_r = ar X_r + al Y_r,   X_r = -2 w_r (q_r - vr) / (eps + beta_r),
//                                 Y_r = -2 w~_r (r_r - vl) / (eps + beta_r)
// (q, r the candidates, w, w~ the weights), then the candidates' and indicators' gradients.
// Entries, each a plane of n doubles (structure of arrays):
//   k = 3: vr, vl, X0..2, Y0..2, w0..2/6, w~0..2/6, 13/6 A0..2, B0..2/2        (20)
//   k = 2: vr, vl, X0..1, Y0..1, w0..1, w~0..1, 2 D0..1                        (12)
// with the A, B, D of WenoTape.  FAST cells take them from the product-form weights of the
// forward pass (one extra reciprocal per cell); guarded cells from WenoTape's division form.
// --------------------------------------------------------------------------------------------
template <int K> struct TapeN { static constexpr int n = 0; };
template <> struct TapeN<2> { static constexpr int n = 12; };
template <> struct TapeN<3> { static constexpr int n = 20; };

template <int K>
__device__ __noinline__ void tape_guarded(double vm2, double vm1, double v0, double vp1, double vp2,
                                          double eps, double vl, double vr, double* wt, int64_t ts,
                                          int64_t j) {
  const double p[5] = {vm2, vm1, v0, vp1, vp2};
  WenoTape<K> W;
  W.fwd(p + 2, eps);
  wt[j] = vr;
  wt[ts + j] = vl;
  if constexpr (K == 3) {
    const double q[3] = {W.q0, W.q1, W.q2}, r[3] = {W.r0, W.r1, W.r2};
    const double w[3] = {W.w0, W.w1, W.w2}, u[3] = {W.u0, W.u1, W.u2};
    const double ie[3] = {W.ie0, W.ie1, W.ie2}, A[3] = {W.A0, W.A1, W.A2}, B[3] = {W.B0, W.B1, W.B2};
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      wt[(2 + s) * ts + j] = -2.0 * ie[s] * (w[s] * (1.0 / 6.0)) * (q[s] - 6.0 * W.vr);
      wt[(5 + s) * ts + j] = -2.0 * ie[s] * (u[s] * (1.0 / 6.0)) * (r[s] - 6.0 * W.vl);
      wt[(8 + s) * ts + j] = w[s] * (1.0 / 6.0);
      wt[(11 + s) * ts + j] = u[s] * (1.0 / 6.0);
      wt[(14 + s) * ts + j] = (13.0 / 6.0) * A[s];
      wt[(17 + s) * ts + j] = 0.5 * B[s];
    }
  } else if constexpr (K == 2) {
    const double q[2] = {W.q0, W.q1}, r[2] = {W.r0, W.r1}, w[2] = {W.w0, W.w1};
    const double u[2] = {W.u0, W.u1}, ie[2] = {W.ie0, W.ie1}, D[2] = {W.D0, W.D1};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      wt[(2 + s) * ts + j] = -2.0 * ie[s] * w[s] * (q[s] - W.vr);
      wt[(4 + s) * ts + j] = -2.0 * ie[s] * u[s] * (r[s] - W.vl);
      wt[(6 + s) * ts + j] = w[s];
      wt[(8 + s) * ts + j] = u[s];
      wt[(10 + s) * ts + j] = 2.0 * D[s];
    }
  }
}

// The tap of recon_fast that writes the tape of cells j0 + c < n (nothing when wt is null).
template <int K>
struct AdjTap {
  double* wt;
  int64_t ts, j0, n;
  double eps;
  __device__ __forceinline__ void cell(int c, const FastCell3& f) const {
    const int64_t j = j0 + c;
    if (!wt || j >= n) return;
    // 1/e_r from one reciprocal of e0 e1 e2
    const double t12 = f.e1 * f.e2, t02 = f.e0 * f.e2, t01 = f.e0 * f.e1;
    const double iE = -2.0 * rcp_fast(f.e0 * t12);
    const double m0 = t12 * iE, m1 = t02 * iE, m2 = t01 * iE;  // -2/e_r
    const double w0 = f.T0 * f.ir, w1 = f.Q1 * f.ir, w2 = f.P2 * f.ir;  // w_r / 6
    const double u0 = f.P0 * f.il, u1 = f.Q1 * f.il, u2 = f.T2 * f.il;  // w~_r / 6
    const double vr6 = 6.0 * f.vr, vl6 = 6.0 * f.vl;
    double* o = wt + j;
    o[0] = f.vr;
    o[ts] = f.vl;
    o[2 * ts] = (m0 * w0) * (f.V0 - vr6);
    o[3 * ts] = (m1 * w1) * (f.V1 - vr6);
    o[4 * ts] = (m2 * w2) * (f.V2 - vr6);
    o[5 * ts] = (m0 * u0) * (f.W0 - vl6);
    o[6 * ts] = (m1 * u1) * (f.W1 - vl6);
    o[7 * ts] = (m2 * u2) * (f.W2 - vl6);
    o[8 * ts] = w0;
    o[9 * ts] = w1;
    o[10 * ts] = w2;
    o[11 * ts] = u0;
    o[12 * ts] = u1;
    o[13 * ts] = u2;
    o[14 * ts] = (13.0 / 6.0) * f.D0;
    o[15 * ts] = (13.0 / 6.0) * f.D1;
    o[16 * ts] = (13.0 / 6.0) * f.D2;
    o[17 * ts] = f.E0;
    o[18 * ts] = f.E1;
    o[19 * ts] = f.E2;
  }
  __device__ __forceinline__ void cell(int c, const FastCell2& f) const {
    const int64_t j = j0 + c;
    if (!wt || j >= n) return;
    const double iE = -2.0 * rcp_fast(f.e0 * f.e1);
    const double m0 = f.e1 * iE, m1 = f.e0 * iE;  // -2/e_r
    const double w0 = 4.0 * f.s1 * f.ir, w1 = 2.0 * f.s0 * f.ir;
    const double u0 = 2.0 * f.s1 * f.il, u1 = 4.0 * f.s0 * f.il;
    double* o = wt + j;
    o[0] = f.vr;
    o[ts] = f.vl;
    o[2 * ts] = (m0 * w0) * fma(0.5, f.V0, -f.vr);
    o[3 * ts] = (m1 * w1) * fma(0.5, f.V1, -f.vr);
    o[4 * ts] = (m0 * u0) * fma(0.5, f.W0, -f.vl);
    o[5 * ts] = (m1 * u1) * fma(0.5, f.W1, -f.vl);
    o[6 * ts] = w0;
    o[7 * ts] = w1;
    o[8 * ts] = u0;
    o[9 * ts] = u1;
    o[10 * ts] = 2.0 * f.d0;
    o[11 * ts] = 2.0 * f.d1;
  }
  __device__ __forceinline__ void guarded(int c, double vm2, double vm1, double v0, double vp1,
                                          double vp2, double vl, double vr) const {
    const int64_t j = j0 + c;
    if (!wt || j >= n) return;
    tape_guarded<K>(vm2, vm1, v0, vp1, vp2, eps, vl, vr, wt, ts, j);
  }
};

// Reverse of the WENO map from the tape: out[0 .. 2K-2] = d(ar vr + al vl)/dp, as
// WenoTape<K>::rev (which adds to out).
template <int K>
__device__ __forceinline__ void rev_tape(const double* __restrict__ wt, int64_t ts, int64_t i,
                                         double ar, double al, double* out) {
  const double* t = wt + i;
  if constexpr (K == 3) {
    const double db0 = fma(ar, t[2 * ts], al * t[5 * ts]);
    const double db1 = fma(ar, t[3 * ts], al * t[6 * ts]);
    const double db2 = fma(ar, t[4 * ts], al * t[7 * ts]);
    const double dq0 = ar * t[8 * ts], dq1 = ar * t[9 * ts], dq2 = ar * t[10 * ts];
    const double dr0 = al * t[11 * ts], dr1 = al * t[12 * ts], dr2 = al * t[13 * ts];
    const double gA0 = t[14 * ts] * db0, gA1 = t[15 * ts] * db1, gA2 = t[16 * ts] * db2;
    const double gB0 = t[17 * ts] * db0, gB1 = t[18 * ts] * db1, gB2 = t[19 * ts] * db2;
    out[0] = fma(2.0, dq2, gA2 + gB2 - dr2);
    out[1] = fma(-7.0, dq2, fma(2.0, dr1, fma(5.0, dr2, fma(-2.0, gA2, fma(-4.0, gB2, gA1 + gB1 - dq1)))));
    out[2] = fma(2.0, dq0, fma(5.0, dq1 + dr1, fma(11.0, dq2 + dr0, fma(2.0, dr2,
              fma(3.0, gB0 + gB2, fma(-2.0, gA1, gA0 + gA2))))));
    out[3] = fma(5.0, dq0, fma(2.0, dq1, fma(-7.0, dr0, fma(-2.0, gA0, fma(-4.0, gB0, gA1 - gB1 - dr1)))));
    out[4] = fma(2.0, dr0, gA0 + gB0 - dq0);
  } else if constexpr (K == 2) {
    const double db0 = fma(ar, t[2 * ts], al * t[4 * ts]);
    const double db1 = fma(ar, t[3 * ts], al * t[5 * ts]);
    const double dq0 = ar * t[6 * ts], dq1 = ar * t[7 * ts];
    const double dr0 = al * t[8 * ts], dr1 = al * t[9 * ts];
    const double g0 = t[10 * ts] * db0, g1 = t[11 * ts] * db1;
    out[0] = fma(-0.5, dq1, fma(0.5, dr1, -g1));
    out[1] = fma(0.5, dq0 + dr1, fma(1.5, dq1 + dr0, g1 - g0));
    out[2] = fma(0.5, dq0 - dr0, g0);
  } else {
    out[0] = ar + al;
  }
}

// --------------------------------------------------------------------------------------------
// Forward stage (FAST FP64), segment-aware: the warp-pass of the batched kernel with ghosts
// replicating the first and last cell of each segment.  Requires seg % C == 0 or one segment.
// TAPE: also write this stage's slice wt of the WENO tape for every cell.  The state
// arithmetic is the same in both instantiations (and in C = 4 and 8 cells per thread), so
// taped and untaped passes give the same states.
// --------------------------------------------------------------------------------------------
template <int K, int ST, int C, bool TAPE>
__global__ void __launch_bounds__(256, TAPE ? HRW_ADJ_TAPE_MINB : HRW_ADJ_FWD_MINB)
    adj_fwd_kernel(AdjLine A, StageArgs a, double* wt) {
  const LineArgs L = line_args(A);
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t wv = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; wv * 32 * C < A.n; wv += nwarps) {
    const int64_t j0 = wv * 32 * C + (int64_t)lane * C;
    const int64_t jc = j0 < A.n ? j0 : A.n - 1;
    const int64_t s0 = jc / A.seg * A.seg, s1 = s0 + A.seg - 1;
    double w[C + 2 * K];
#pragma unroll
    for (int q = 0; q < C + 2 * K; ++q) {
      int64_t g = j0 - K + q;
      g = g < s0 ? s0 : (g > s1 ? s1 : g);
      w[q] = a.v[g];
    }
    double vl[C], vr[C];
    if constexpr (TAPE) recon_fast<K, C, true, AdjTap<K>>(w, a.eps, vl, vr, AdjTap<K>{wt, A.n, j0, A.n, a.eps});
    else recon_fast<K, C>(w, a.eps, vl, vr);
    double e[2 * K - 1];
#pragma unroll
    for (int q = 0; q < 2 * K - 1; ++q) e[q] = lane == 31 ? w[C + 1 + q] : w[q];
    double el, er;
    recon_fast_one<K>(&e[K - 1], a.eps, el, er);
    const double vr_up = __shfl_up_sync(FULL, vr[C - 1], 1);
    const double vl_dn = __shfl_down_sync(FULL, vl[0], 1);
    const double vr_m = lane == 0 ? er : vr_up;  // interfaces across segments are never used:
    const double vl_p = lane == 31 ? el : vl_dn;  // the boundary rules replace them
    const int64_t l0 = j0 - s0;  // local index of the first cell
    double F[C + 1];
    F[0] = flux_fast(L, vr_m, vl[0], l0);
#pragma unroll
    for (int c = 1; c < C; ++c) F[c] = flux_fast(L, vr[c - 1], vl[c], l0 + c);
    F[C] = flux_fast(L, vr[C - 1], vl_p, l0 + C);
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t j = j0 + c;
      if (j >= A.n) break;
      const double dF = flux_diff<false>(L, l0 + c, F[c], F[c + 1], vr[c]);
      combine_fast<ST>(a, j, w[K + c], dF, L.rws0);
    }
  }
}

// --------------------------------------------------------------------------------------------
// Forward stage on a non-uniform line (FAST FP64), segment-aware, one cell per thread: the
// arithmetic of the single-line non-uniform stage (recon_nu, numflux, flux_diff, combine_fast
// with the cell's own scale), so a one-segment line gives the same states as hrw_integrate.
// --------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void recon_cell_nu(const AdjLine& A, const double* __restrict__ v, int64_t j,
                                              double& vl, double& vr) {
  j = j < 0 ? 0 : (j >= A.n ? A.n - 1 : j);
  const int64_t s0 = j / A.seg * A.seg, s1 = s0 + A.seg - 1;
  double p[2 * K - 1];
#pragma unroll
  for (int q = 0; q < 2 * K - 1; ++q) {
    int64_t g = j - (K - 1) + q;
    g = g < s0 ? s0 : (g > s1 ? s1 : g);  // ghosts replicate the segment's end cells
    p[q] = v[g];
  }
  recon_nu<K, false>(&p[K - 1], A.cnu + (int64_t)K * (K + 1) * (j - s0), A.eps, vl, vr);
}

template <int K, int ST, int NT>
__global__ void __launch_bounds__(NT) adj_fwd_nu_kernel(AdjLine A, StageArgs a) {
  __shared__ double sL[NT + 1], sR[NT + 1];  // vl of cell s+t at sL[t], vr at sR[t+1]
  const LineArgs L = line_args(A);
  const int64_t s = (int64_t)blockIdx.x * NT;
  const int t = threadIdx.x;
  const int64_t j = s + t;
  double vl, vr;
  recon_cell_nu<K>(A, a.v, j, vl, vr);
  sL[t] = vl;
  sR[t + 1] = vr;
  if (t >= NT - 2) {  // cells s - 1 (vr) and s + NT (vl); across a segment end the boundary
    double el, er;    // rules replace the interface, so their values are not used there
    recon_cell_nu<K>(A, a.v, t == NT - 2 ? s - 1 : s + NT, el, er);
    if (t == NT - 2) sR[0] = er;
    else sL[NT] = el;
  }
  __syncthreads();
  if (j >= A.n) return;
  const int64_t li = j % A.seg;
  const double FL = numflux<false>(L, sR[t], vl, li);
  const double FR = numflux<false>(L, vr, sL[t + 1], li + 1);
  const double dF = flux_diff<false>(L, li, FL, FR, vr);
  combine_fast<ST>(a, j, a.v[j], dF, A.rwsv[li]);
}

// does cell with local index lc use the interface flux on its right / left?
__device__ __forceinline__ bool uses_fr(int bc, int64_t lc, int64_t seg) {
  if (bc == HRW_BC_COPY) return lc > 0 && lc < seg - 1;
  return lc < seg - 1;  // ZERO, ZERO_INFLOW: the last cell's right flux is the boundary's
}
__device__ __forceinline__ bool uses_fl(int bc, int64_t lc, int64_t seg) {
  if (bc == HRW_BC_COPY) return lc > 0 && lc < seg - 1;
  return lc > 0;
}

__device__ __forceinline__ double dflux(const AdjLine& A, double v, int64_t e) {
  // f'(v) at interface e (local index): Burgers u, linear g(x_e)
  if (A.fn == HRW_FN_BURGERS) return v;
  const double g = fma(A.b, A.xe ? A.xe[e] : fma(A.rx, (double)e, A.xmin), A.a);
  return A.fn == HRW_FN_BURGERS_LINEAR ? v + g : g;
}

enum AdjMode : int { ADJ_A3 = 0, ADJ_A2 = 1, ADJ_A1 = 2 };

// --------------------------------------------------------------------------------------------
// VJP + stage-adjoint combine.  Block: NT cells [s, s+NT); contributors s-(K-1) .. s+NT+K-2.
//   state: v (the stage input of the forward stage), mu: adjoint of that stage's L output
//   (scaled as described in the mode), acc: the accumulated adjoint of u.
// --------------------------------------------------------------------------------------------
// NU: a non-uniform line (recomputes its WENO maps with the cells' coefficients; no tape)
template <int K, int MODE, int NT, bool TAPE, bool NU = false>
__global__ void __launch_bounds__(NT) adj_vjp_kernel(AdjLine A, const double* __restrict__ v,
                                                     const double* __restrict__ wt,
                                                     const double* __restrict__ mu,
                                                     double* __restrict__ acc,
                                                     double* __restrict__ out, double dt) {
  constexpr int NS = 2 * K - 1;             // stencil width
  constexpr int NCTR = NT + 2 * (K - 1);    // contributors
  __shared__ double sc[NCTR * NS];
  const int64_t s = (int64_t)blockIdx.x * NT;
  const double idx = A.rdx, hidx = 0.5 * A.rdx;
  for (int t = threadIdx.x; t < NCTR; t += NT) {
    const int64_t i = s - (K - 1) + t;
    double o[NS];
#pragma unroll
    for (int q = 0; q < NS; ++q) o[q] = 0.0;  // (the taped path assigns them)
    if (i >= 0 && i < A.n) {
      const int64_t s0 = i / A.seg * A.seg, s1 = s0 + A.seg - 1, li = i - s0;
      double p[NS];
      std::conditional_t<NU, WenoTapeNu<K>, WenoTape<K>> W;
      double vl, vr;
      if constexpr (TAPE) {  // the forward pass recorded the cell's WENO map
        vr = wt[i];
        vl = wt[A.n + i];
      } else {
#pragma unroll
        for (int q = 0; q < NS; ++q) {
          int64_t g = i - (K - 1) + q;
          g = g < s0 ? s0 : (g > s1 ? s1 : g);
          p[q] = v[g];
        }
        if constexpr (NU) W.fwd(&p[K - 1], A.eps, A.cnu + (int64_t)K * (K + 1) * li);
        else W.fwd(&p[K - 1], A.eps);
        vl = W.vl, vr = W.vr;
      }
      const double mi = mu[i];
      // flux adjoints of the cell's right and left interfaces; L_i = -(F_{i+1/2} - F_{i-1/2})
      // / width_i, so a flux weighs each neighbour's adjoint by that cell's 1 / width
      const double ri = NU ? A.rdxv[li] : idx;
      double ar = 0.0, al = 0.0;
      if (li < A.seg - 1) {
        const double mp = mu[i + 1];
        double phi;  // phi / 2
        if constexpr (NU)
          phi = 0.5 * ((uses_fl(A.bc, li + 1, A.seg) ? mp * A.rdxv[li + 1] : 0.0) -
                       (uses_fr(A.bc, li, A.seg) ? mi * ri : 0.0));
        else
          phi = ((uses_fl(A.bc, li + 1, A.seg) ? mp : 0.0) - (uses_fr(A.bc, li, A.seg) ? mi : 0.0)) * hidx;
        ar = phi * (dflux(A, vr, li + 1) + A.alpha);
      } else if (A.bc == HRW_BC_ZERO_INFLOW) {  // F_{nc+1/2} = f(vr(nc))
        ar = -mi * ri * dflux(A, vr, li + 1);
      }
      if (li > 0) {
        const double mm = mu[i - 1];
        double phi;
        if constexpr (NU)
          phi = 0.5 * ((uses_fl(A.bc, li, A.seg) ? mi * ri : 0.0) -
                       (uses_fr(A.bc, li - 1, A.seg) ? mm * A.rdxv[li - 1] : 0.0));
        else
          phi = ((uses_fl(A.bc, li, A.seg) ? mi : 0.0) - (uses_fr(A.bc, li - 1, A.seg) ? mm : 0.0)) * hidx;
        al = phi * (dflux(A, vl, li) - A.alpha);
      }
      if constexpr (TAPE) rev_tape<K>(wt, A.n, i, ar, al, o);
      else W.rev(ar, al, o);
    }
#pragma unroll
    for (int q = 0; q < NS; ++q) sc[t * NS + q] = o[q];
  }
  __syncthreads();
  const int64_t m = s + threadIdx.x;
  if (m >= A.n) return;
  const int64_t s0 = m / A.seg * A.seg, s1 = s0 + A.seg - 1, lm = m - s0;
  double w;
  const double* sm = sc + (m - s + (K - 1)) * NS;  // contributor m's entries
  if (lm >= K - 1 && lm <= A.seg - K) {  // every contributor inside the segment
    // contributor i = m - o sees m at offset o: sc[(i - first) * NS + o + K - 1]
    w = sm[(K - 1) * NS];
#pragma unroll
    for (int o = -(K - 2); o <= K - 1; ++o) w += sm[-o * NS + (o + K - 1)];
  } else {
    w = 0.0;
#pragma unroll
    for (int o = -(K - 1); o <= K - 1; ++o) {
      const int64_t i = m - o;
      if (i >= s0 && i <= s1) w += sc[(i - (s - (K - 1))) * NS + (o + K - 1)];
    }
  }
  // ghost positions (outside the segment) clamp onto its end cells
  if (lm == 0) {
#pragma unroll
    for (int ii = 0; ii < K - 1; ++ii) {
      const int64_t i = s0 + ii;
#pragma unroll
      for (int q = 0; q < NS; ++q)
        if (i <= s1 && i - (K - 1) + q < s0) w += sc[(i - (s - (K - 1))) * NS + q];
    }
  }
  if (lm == A.seg - 1) {
#pragma unroll
    for (int ii = 0; ii < K - 1; ++ii) {
      const int64_t i = s1 - ii;
#pragma unroll
      for (int q = 0; q < NS; ++q)
        if (i >= s0 && i - (K - 1) + q > s1) w += sc[(i - (s - (K - 1))) * NS + q];
    }
  }
  const double mum = mu[m];
  if constexpr (MODE == ADJ_A3) {
    out[m] = (2.0 / 3.0) * fma(dt, w, mum);
    acc[m] = (1.0 / 3.0) * mum;
  } else if constexpr (MODE == ADJ_A2) {
    out[m] = 0.25 * fma(dt, w, mum);
    acc[m] = fma(0.75, mum, acc[m]);
  } else {
    out[m] = acc[m] + fma(dt, w, mum);
  }
}

// J per segment and lambda_T = u - target, summed in a fixed order (the same J, bit for bit,
// on every call, so that finite differences of J see no summation noise): block b of segment
// sg sums its chunk of kMisfitChunk cells with compensated (Neumaier) sums per thread and a
// pairwise tree across the block into part[sg * P + b]; adj_misfit_final adds the P partials.
constexpr int kMisfitThreads = 256;
constexpr int64_t kMisfitChunk = 1 << 13;

__device__ __forceinline__ void neumaier(double& s, double& c, double x) {
  const double t = s + x;
  c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
  s = t;
}

__global__ void __launch_bounds__(kMisfitThreads) adj_misfit_kernel(
    AdjLine A, const double* __restrict__ u, const double* __restrict__ tgt,
    double* __restrict__ lam, double* __restrict__ part, int P) {
  __shared__ double red[kMisfitThreads];
  const int sg = blockIdx.x / P, b = blockIdx.x - sg * P;
  const int64_t lo = sg * A.seg + b * kMisfitChunk;
  const int64_t hi = min(lo + kMisfitChunk, (sg + 1) * A.seg);
  double s = 0.0, c = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += kMisfitThreads) {
    const double r = u[i] - tgt[i];
    lam[i] = r;
    neumaier(s, c, 0.5 * r * r);
  }
  red[threadIdx.x] = s + c;
  __syncthreads();
  for (int w = kMisfitThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void adj_misfit_final(const double* __restrict__ part, int nseg, int P,
                                 double* __restrict__ J) {
  const int sg = blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= nseg) return;
  double s = 0.0, c = 0.0;
  for (int b = 0; b < P; ++b) neumaier(s, c, part[(int64_t)sg * P + b]);
  J[sg] = s + c;
}

int misfit_blocks_per_seg(const AdjLine& A) { return (int)((A.seg + kMisfitChunk - 1) / kMisfitChunk); }

template <int K, int C, bool TAPE>
cudaError_t fwd_stage_kt(const AdjLine& A, const StageArgs& a, int st, double* wt, cudaStream_t s) {
  const int64_t warps = (A.n + 32 * C - 1) / (32 * C);
  const int64_t cap = (int64_t)device_sms() * 32;
  const int blocks = (int)((warps + 7) / 8 < cap ? (warps + 7) / 8 : cap);
  if (st == ST_EULER) adj_fwd_kernel<K, ST_EULER, C, TAPE><<<blocks, 256, 0, s>>>(A, a, wt);
  else if (st == ST_RK3B) adj_fwd_kernel<K, ST_RK3B, C, TAPE><<<blocks, 256, 0, s>>>(A, a, wt);
  else adj_fwd_kernel<K, ST_RK3C, C, TAPE><<<blocks, 256, 0, s>>>(A, a, wt);
  return cudaGetLastError();
}

// taped passes run fewer cells per thread (the tape's intermediates need the registers)
template <int K>
cudaError_t fwd_stage_nu(const AdjLine& A, const StageArgs& a, int st, cudaStream_t s) {
  constexpr int NT = 128;
  const unsigned blocks = (unsigned)((A.n + NT - 1) / NT);
  if (st == ST_EULER) adj_fwd_nu_kernel<K, ST_EULER, NT><<<blocks, NT, 0, s>>>(A, a);
  else if (st == ST_RK3B) adj_fwd_nu_kernel<K, ST_RK3B, NT><<<blocks, NT, 0, s>>>(A, a);
  else adj_fwd_nu_kernel<K, ST_RK3C, NT><<<blocks, NT, 0, s>>>(A, a);
  return cudaGetLastError();
}

template <int K>
cudaError_t fwd_stage_k(const AdjLine& A, const StageArgs& a, int st, double* wt, cudaStream_t s) {
  if (A.cnu) return fwd_stage_nu<K>(A, a, st, s);
  if (TapeN<K>::n > 0 && wt) return fwd_stage_kt<K, HRW_ADJ_TAPE_C, true>(A, a, st, wt, s);
  return fwd_stage_kt<K, HRW_ADJ_FWD_C, false>(A, a, st, nullptr, s);
}

template <int K, bool TAPE, bool NU = false>
cudaError_t vjp_kt(const AdjLine& A, int mode, const double* v, const double* wt, const double* mu,
                   double* acc, double* out, double dt, cudaStream_t s) {
  constexpr int NT = HRW_ADJ_VJP_NT;
  const unsigned blocks = (unsigned)((A.n + NT - 1) / NT);
  if (mode == ADJ_A3)
    adj_vjp_kernel<K, ADJ_A3, NT, TAPE, NU><<<blocks, NT, 0, s>>>(A, v, wt, mu, acc, out, dt);
  else if (mode == ADJ_A2)
    adj_vjp_kernel<K, ADJ_A2, NT, TAPE, NU><<<blocks, NT, 0, s>>>(A, v, wt, mu, acc, out, dt);
  else
    adj_vjp_kernel<K, ADJ_A1, NT, TAPE, NU><<<blocks, NT, 0, s>>>(A, v, wt, mu, acc, out, dt);
  return cudaGetLastError();
}

template <int K>
cudaError_t vjp_k(const AdjLine& A, int mode, const double* v, const double* wt, const double* mu,
                  double* acc, double* out, double dt, cudaStream_t s) {
  if (A.cnu) return vjp_kt<K, false, true>(A, mode, v, nullptr, mu, acc, out, dt, s);
  if (TapeN<K>::n > 0 && wt) return vjp_kt<K, true>(A, mode, v, wt, mu, acc, out, dt, s);
  return vjp_kt<K, false>(A, mode, v, nullptr, mu, acc, out, dt, s);
}

cudaError_t fwd_stage(const AdjLine& A, const StageArgs& a, int st, double* wt, cudaStream_t s) {
  if (A.k == 1 && A.cnu) return fwd_stage_nu<1>(A, a, st, s);
  if (A.k == 1) return fwd_stage_k<1>(A, a, st, nullptr, s);
  if (A.k == 2) return fwd_stage_k<2>(A, a, st, wt, s);
  return fwd_stage_k<3>(A, a, st, wt, s);
}

// v: the stage's input state; wt: the stage's WENO tape (null: recompute from v)
cudaError_t vjp(const AdjLine& A, int mode, const double* v, const double* wt, const double* mu,
                double* acc, double* out, double dt, cudaStream_t s) {
  if (A.k == 1) return A.cnu ? vjp_kt<1, false, true>(A, mode, v, nullptr, mu, acc, out, dt, s)
                            : vjp_k<1>(A, mode, v, nullptr, mu, acc, out, dt, s);
  if (A.k == 2) return vjp_k<2>(A, mode, v, wt, mu, acc, out, dt, s);
  return vjp_k<3>(A, mode, v, wt, mu, acc, out, dt, s);
}

// doubles per cell and stage of the WENO tape (none on a non-uniform line: its reverse pass
// recomputes the maps)
int tape_entries(const AdjLine& A) {
  if (A.cnu) return 0;
  return A.k == 3 ? TapeN<3>::n : (A.k == 2 ? TapeN<2>::n : 0);
}

}  // namespace
}  // namespace hrw

using namespace hrw;

struct hrw_adjoint {
  AdjLine line{};
  int64_t nseg = 1;
  int every = 45;
  cudaStream_t own = nullptr, stream = nullptr;
  double *u = nullptr, *w1 = nullptr, *w2 = nullptr, *tgt = nullptr;
  double *lam = nullptr, *la = nullptr, *lb = nullptr, *acc = nullptr, *J = nullptr;
  double* part = nullptr;     // partial sums of J (nseg x misfit blocks per segment)
  double* nu = nullptr;       // non-uniform line: cnu, 1 / width, scale / width, edges
  std::vector<double*> ckpt;  // checkpoints
  double* tape = nullptr;     // (E + 1) states + E u1 + E u2 of the segment being reversed
  int64_t tape_states = 0;    // capacity of the tape in states
  double* wtape = nullptr;    // WENO tape of the 3E stages of the segment being reversed
  int64_t wtape_stages = 0;   // its capacity in stages
  int64_t wtape_used = 0;     // bytes of it the last gradient call used (0: not used)
  int64_t used_every = 0;     // checkpoint interval of the last gradient call
  int64_t fwd_steps = 0;      // forward steps taken by the last gradient call (incl. recompute)
};

namespace {

int adj_fail(int code, const std::string& m) { return set_error(code, m.c_str()); }

#define HRW_ACUDA(call)                                                                 \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return adj_fail(e_ == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,         \
                      std::string(#call ": ") + cudaGetErrorString(e_));                \
  } while (0)

StageArgs base_args(const hrw_adjoint* h, double dt) {
  StageArgs a{};
  a.eps = h->line.eps;
  a.dt = dt;
  return a;
}

// J[nseg] and lambda = u - target
cudaError_t misfit(hrw_adjoint* h, const double* u) {
  const int P = misfit_blocks_per_seg(h->line);
  adj_misfit_kernel<<<(unsigned)(h->nseg * P), kMisfitThreads, 0, h->stream>>>(h->line, u, h->tgt,
                                                                               h->lam, h->part, P);
  adj_misfit_final<<<(unsigned)((h->nseg + 127) / 128), 128, 0, h->stream>>>(h->part, (int)h->nseg,
                                                                             P, h->J);
  return cudaGetLastError();
}

// one forward RK3 step from `u` to `un` with stage arrays s1, s2 (un may equal u); wt
// (nullable): the WENO tape of the step's three stages, one after the other
cudaError_t step(hrw_adjoint* h, const double* u, double* s1, double* s2, double* un, double dt,
                 double* wt = nullptr) {
  const size_t plane = (size_t)tape_entries(h->line) * (size_t)h->line.n;
  StageArgs a = base_args(h, dt);
  a.v = u, a.u = u, a.out = s1;
  cudaError_t e = fwd_stage(h->line, a, ST_EULER, wt, h->stream);
  if (e != cudaSuccess) return e;
  a.v = s1, a.u = u, a.out = s2;
  if ((e = fwd_stage(h->line, a, ST_RK3B, wt ? wt + plane : nullptr, h->stream)) != cudaSuccess)
    return e;
  a.v = s2, a.u = u, a.out = un;
  return fwd_stage(h->line, a, ST_RK3C, wt ? wt + 2 * plane : nullptr, h->stream);
}

}  // namespace

extern "C" {

int hrw_adjoint_create(const hrw_problem* p, int nseg, int checkpoint_every, hrw_adjoint** out) {
  if (!out) return adj_fail(HRW_EINVAL, "Invalid input 'out': null pointer.");
  *out = nullptr;
  if (!p) return adj_fail(HRW_EINVAL, "Invalid input 'problem': null pointer.");
  if (p->kind != HRW_PROBLEM_FV1D) return adj_fail(HRW_EINVAL, "hrw_adjoint: FV1D problems only.");
  if (p->flux != HRW_FLUX_LAX_FRIEDRICHS)
    return adj_fail(HRW_EINVAL, "hrw_adjoint: the global Lax-Friedrichs flux with fixed alpha only.");
  if (p->width[0]) return adj_fail(HRW_EINVAL, "hrw_adjoint: non-uniform lines are given as xedges.");
  if (p->ncells[0] <= 0) return adj_fail(HRW_EINVAL, "Invalid input 'ncells'. Valid range: ncells > 0.");
  if (p->xedges[0]) {
    for (int i = 0; i < p->ncells[0]; ++i)
      if (!(p->xedges[0][i + 1] > p->xedges[0][i]))
        return adj_fail(HRW_EINVAL, "Invalid input 'xedges': edges must increase.");
  } else if (!(p->xmax[0] > p->xmin[0])) {
    return adj_fail(HRW_EINVAL, "Invalid input 'xmin', 'xmax'. Valid range: xmax > xmin.");
  }
  if (p->k < 1 || p->k > 3) return adj_fail(HRW_EINVAL, "Invalid input 'k'. Valid range: 1 <= k <= 3.");
  if (!(p->eps > 2.220446049250313e-16))
    return adj_fail(HRW_EINVAL, "Invalid input 'eps'. Valid range: eps > epsilon.");
  if (p->fn[0] < HRW_FN_BURGERS || p->fn[0] > HRW_FN_BURGERS_LINEAR) return adj_fail(HRW_EINVAL, "Invalid input 'fn'.");
  if (p->bc[0] < HRW_BC_COPY || p->bc[0] > HRW_BC_ZERO_INFLOW) return adj_fail(HRW_EINVAL, "Invalid input 'bc'.");
  if (nseg < 1) return adj_fail(HRW_EINVAL, "Invalid input 'nseg': must be >= 1.");
  if (nseg > 1 && p->ncells[0] % 8 != 0)
    return adj_fail(HRW_EINVAL, "hrw_adjoint: with nseg > 1, ncells must be a multiple of 8.");
  if (checkpoint_every < 0)
    return adj_fail(HRW_EINVAL, "Invalid input 'checkpoint_every': must be >= 0 (0: automatic).");
  hrw_adjoint* h = new hrw_adjoint;
  AdjLine& L = h->line;
  L.seg = p->ncells[0];
  L.n = L.seg * nseg;
  L.k = p->k;
  L.fn = p->fn[0];
  L.bc = p->bc[0];
  L.a = p->coef_a[0];
  L.b = p->coef_b[0];
  L.alpha = p->alpha[0];
  L.xmin = p->xmin[0];
  L.rx = (p->xmax[0] - p->xmin[0]) / L.seg;
  L.rdx = 1.0 / L.rx;
  L.eps = p->eps;
  L.rws0 = fast_flux_scale(HRW_FLUX_LAX_FRIEDRICHS, L.fn) / L.rx;
  h->nseg = nseg;
  h->every = checkpoint_every;
  const size_t bytes = sizeof(double) * (size_t)L.n;
  cudaError_t e = cudaStreamCreateWithFlags(&h->own, cudaStreamDefault);
  h->stream = h->own;
  double** bufs[] = {&h->u, &h->w1, &h->w2, &h->tgt, &h->lam, &h->la, &h->lb, &h->acc};
  for (double** b : bufs)
    if (e == cudaSuccess) e = cudaMalloc(b, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&h->J, sizeof(double) * nseg);
  if (e == cudaSuccess) e = cudaMalloc(&h->part, sizeof(double) * nseg * misfit_blocks_per_seg(L));
  if (e == cudaSuccess && p->xedges[0]) {
    // weno(ncells, k, eps, xedges): the coefficients on the device (as hrw_rktvd_create builds
    // them), the widths edges(i) - edges(i-1) and the flux at the true edges
    const size_t nc = (size_t)L.seg, ncf = (size_t)L.k * (L.k + 1);
    std::vector<double> host(2 * nc + nc + 1);
    const double fs = fast_flux_scale(HRW_FLUX_LAX_FRIEDRICHS, L.fn);
    for (size_t i = 0; i < nc; ++i) {
      const double w = p->xedges[0][i + 1] - p->xedges[0][i];
      host[i] = 1.0 / w;
      host[nc + i] = fs / w;
    }
    for (size_t i = 0; i <= nc; ++i) host[2 * nc + i] = p->xedges[0][i];
    e = cudaMalloc(&h->nu, sizeof(double) * (nc * ncf + host.size()));
    if (e == cudaSuccess)
      e = cudaMemcpy(h->nu + nc * ncf, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      L.cnu = h->nu;
      L.rdxv = h->nu + nc * ncf;
      L.rwsv = L.rdxv + nc;
      L.xe = L.rwsv + nc;
      e = launch_calc_cnu(L.xe, h->nu, (int)nc, L.k, h->own);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->own);
  }
  if (e != cudaSuccess) {
    hrw_adjoint_destroy(h);
    return adj_fail(e == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,
                    std::string("hrw_adjoint_create: ") + cudaGetErrorString(e));
  }
  *out = h;
  return HRW_OK;
}

// The reverse sweep shared by hrw_adjoint_gradient (lambda(T) = u(T) - target, J computed) and
// hrw_adjoint_vjp (lambda(T) given).
static int adjoint_sweep(hrw_adjoint* h, int mem, const double* u0, const double* target,
                         const double* lambda_T, double dt, int64_t nsteps, double* J, double* grad) {
  if (!h) return adj_fail(HRW_EINVAL, "Invalid input 'adjoint': null handle.");
  if (!u0 || !(target || lambda_T) || !grad) return adj_fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (mem != HRW_MEM_HOST && mem != HRW_MEM_DEVICE) return adj_fail(HRW_EINVAL, "Invalid input 'mem'.");
  if (nsteps < 1) return adj_fail(HRW_EINVAL, "Invalid input 'nsteps': must be >= 1.");
  if (!(dt != 0.0) || !std::isfinite(dt)) return adj_fail(HRW_EINVAL, "Invalid input 'dt'.");
  const AdjLine& L = h->line;
  const size_t bytes = sizeof(double) * (size_t)L.n;
  const cudaMemcpyKind in = mem == HRW_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  // Memory budget: 80% of the free device memory plus the tapes this handle already holds.
  // A segment of E steps needs 3E + 1 states and, for the WENO tape, 3E stage planes of
  // tape_entries(k) doubles per cell.
  const int nq = tape_entries(L);
  size_t fr = 0, tot = 0;
  HRW_ACUDA(cudaMemGetInfo(&fr, &tot));
  const double budget = 0.8 * ((double)fr + (double)bytes * (double)h->tape_states +
                               (double)bytes * nq * (double)h->wtape_stages);
  auto state_need = [&](int64_t e) { return (double)bytes * (3.0 * e + 1.0); };
  auto weno_need = [&](int64_t e) { return (double)bytes * nq * 3.0 * e; };
  // checkpoint interval: as asked, or (0) the first that fits the budget of
  //   the whole trajectory with the WENO tape (no recompute; the cheapest),
  //   sqrt(nsteps) segments with the WENO tape (one recompute; the reverse reads the tape),
  //   the whole trajectory's states without it (no recompute; the reverse recomputes the WENO
  //   maps -- about as fast as the previous choice, with more memory),
  //   sqrt(nsteps) segments without it.
  int64_t E = h->every;
  if (E == 0) {
    const int64_t sq = (int64_t)std::ceil(std::sqrt((double)nsteps));
    if (nq > 0 && state_need(nsteps) + weno_need(nsteps) <= budget) E = nsteps;
    else if (nq > 0 && state_need(sq) + weno_need(sq) <= budget) E = sq;
    else if (state_need(nsteps) <= budget) E = nsteps;
    else E = sq;
  }
  const bool use_wt = nq > 0 && state_need(E) + weno_need(E) <= budget;
  if (h->tape_states < 3 * E + 1) {
    if (h->tape) cudaFree(h->tape);
    h->tape = nullptr;
    h->tape_states = 0;
    HRW_ACUDA(cudaMalloc(&h->tape, bytes * (size_t)(3 * E + 1)));
    h->tape_states = 3 * E + 1;
  }
  if (use_wt && h->wtape_stages < 3 * E) {
    if (h->wtape) cudaFree(h->wtape);
    h->wtape = nullptr;
    h->wtape_stages = 0;
    HRW_ACUDA(cudaMalloc(&h->wtape, bytes * nq * (size_t)(3 * E)));
    h->wtape_stages = 3 * E;
  }
  h->wtape_used = use_wt ? (int64_t)(bytes * nq * (size_t)(3 * E)) : 0;
  const size_t step_planes = 3 * (size_t)nq * (size_t)L.n;  // WENO tape doubles per step
  auto WT = [&](int64_t n) { return use_wt ? h->wtape + (size_t)n * step_planes : nullptr; };
  auto WS = [&](int64_t n, int st) {  // stage st (0..2) of step n
    return use_wt ? h->wtape + (size_t)n * step_planes + (size_t)st * nq * L.n : nullptr;
  };
  h->used_every = E;
  const int64_t nck = (nsteps + E - 1) / E;  // segments of the time line
  while ((int64_t)h->ckpt.size() < nck) {
    double* c = nullptr;
    HRW_ACUDA(cudaMalloc(&c, bytes));
    h->ckpt.push_back(c);
  }
  double* U = h->tape;  // U[n] = tape + n, U1[n] = tape + E+1+n, U2[n] = tape + 2E+1+n
  auto Un = [&](int64_t n) { return U + (size_t)n * L.n; };
  auto U1 = [&](int64_t n) { return U + (size_t)(E + 1 + n) * L.n; };
  auto U2 = [&](int64_t n) { return U + (size_t)(2 * E + 1 + n) * L.n; };
  // ---- forward: checkpoints, the last segment recorded on the tape ------------------------
  HRW_ACUDA(cudaMemcpyAsync(h->u, u0, bytes, in, h->stream));
  HRW_ACUDA(cudaMemcpyAsync(h->tgt, target ? target : lambda_T, bytes, in, h->stream));
  int64_t fwd = 0;
  for (int64_t c = 0; c < nck; ++c) {
    const int64_t len = std::min(E, nsteps - c * E);
    HRW_ACUDA(cudaMemcpyAsync(h->ckpt[c], h->u, bytes, cudaMemcpyDeviceToDevice, h->stream));
    if (c < nck - 1) {
      for (int64_t n = 0; n < len; ++n) HRW_ACUDA(step(h, h->u, h->w1, h->w2, h->u, dt));
    } else {
      HRW_ACUDA(cudaMemcpyAsync(Un(0), h->u, bytes, cudaMemcpyDeviceToDevice, h->stream));
      for (int64_t n = 0; n < len; ++n) HRW_ACUDA(step(h, Un(n), U1(n), U2(n), Un(n + 1), dt, WT(n)));
    }
    fwd += len;
  }
  // ---- misfit and lambda(T) -----------------------------------------------------------------
  const int64_t last_len = nsteps - (nck - 1) * E;
  if (target) {
    HRW_ACUDA(misfit(h, Un(last_len)));
  } else {
    HRW_ACUDA(cudaMemcpyAsync(h->lam, h->tgt, bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  // ---- reverse sweep ---------------------------------------------------------------------------
  for (int64_t c = nck - 1; c >= 0; --c) {
    const int64_t len = std::min(E, nsteps - c * E);
    if (c < nck - 1) {  // recompute the segment from its checkpoint, recording every stage
      HRW_ACUDA(cudaMemcpyAsync(Un(0), h->ckpt[c], bytes, cudaMemcpyDeviceToDevice, h->stream));
      for (int64_t n = 0; n < len; ++n) HRW_ACUDA(step(h, Un(n), U1(n), U2(n), Un(n + 1), dt, WT(n)));
      fwd += len;
    }
    for (int64_t n = len - 1; n >= 0; --n) {
      HRW_ACUDA(vjp(L, ADJ_A3, U2(n), WS(n, 2), h->lam, h->acc, h->la, dt, h->stream));
      HRW_ACUDA(vjp(L, ADJ_A2, U1(n), WS(n, 1), h->la, h->acc, h->lb, dt, h->stream));
      HRW_ACUDA(vjp(L, ADJ_A1, Un(n), WS(n, 0), h->lb, h->acc, h->lam, dt, h->stream));
    }
  }
  h->fwd_steps = fwd;
  const cudaMemcpyKind outk = mem == HRW_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  HRW_ACUDA(cudaMemcpyAsync(grad, h->lam, bytes, outk, h->stream));
  if (J && target)
    HRW_ACUDA(cudaMemcpyAsync(J, h->J, sizeof(double) * h->nseg, cudaMemcpyDeviceToHost, h->stream));
  HRW_ACUDA(cudaStreamSynchronize(h->stream));
  return HRW_OK;
}

int hrw_adjoint_gradient(hrw_adjoint* h, int mem, const double* u0, const double* target, double dt,
                         int64_t nsteps, double* J, double* grad) {
  if (!target) return adj_fail(HRW_EINVAL, "Invalid input 'target': null pointer.");
  return adjoint_sweep(h, mem, u0, target, nullptr, dt, nsteps, J, grad);
}

int hrw_adjoint_vjp(hrw_adjoint* h, int mem, const double* u0, const double* lambda_T, double dt,
                    int64_t nsteps, double* grad) {
  if (!lambda_T) return adj_fail(HRW_EINVAL, "Invalid input 'lambda_T': null pointer.");
  return adjoint_sweep(h, mem, u0, nullptr, lambda_T, dt, nsteps, nullptr, grad);
}

// Forward only: u(T) after nsteps steps and J (per segment); the reference point of the
// adjoint's cost and of finite-difference checks.
int hrw_adjoint_forward(hrw_adjoint* h, int mem, const double* u0, const double* target, double dt,
                        int64_t nsteps, double* J, double* uT) {
  if (!h) return adj_fail(HRW_EINVAL, "Invalid input 'adjoint': null handle.");
  if (!u0) return adj_fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (mem != HRW_MEM_HOST && mem != HRW_MEM_DEVICE) return adj_fail(HRW_EINVAL, "Invalid input 'mem'.");
  if (nsteps < 0) return adj_fail(HRW_EINVAL, "Invalid input 'nsteps': must be >= 0.");
  if (!(dt != 0.0) || !std::isfinite(dt)) return adj_fail(HRW_EINVAL, "Invalid input 'dt'.");
  const AdjLine& L = h->line;
  const size_t bytes = sizeof(double) * (size_t)L.n;
  const cudaMemcpyKind in = mem == HRW_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  HRW_ACUDA(cudaMemcpyAsync(h->u, u0, bytes, in, h->stream));
  for (int64_t n = 0; n < nsteps; ++n) HRW_ACUDA(step(h, h->u, h->w1, h->w2, h->u, dt));
  if (target) {
    HRW_ACUDA(cudaMemcpyAsync(h->tgt, target, bytes, in, h->stream));
    HRW_ACUDA(misfit(h, h->u));
  }
  if (uT)
    HRW_ACUDA(cudaMemcpyAsync(uT, h->u, bytes, mem == HRW_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                              h->stream));
  if (J && target)
    HRW_ACUDA(cudaMemcpyAsync(J, h->J, sizeof(double) * h->nseg, cudaMemcpyDeviceToHost, h->stream));
  HRW_ACUDA(cudaStreamSynchronize(h->stream));
  return HRW_OK;
}

int hrw_adjoint_set_stream(hrw_adjoint* h, void* stream) {
  if (!h) return adj_fail(HRW_EINVAL, "Invalid input 'adjoint': null handle.");
  h->stream = stream ? (cudaStream_t)stream : h->own;
  return HRW_OK;
}

int hrw_adjoint_info(const hrw_adjoint* h, int64_t* forward_steps, int64_t* checkpoint_every) {
  if (!h) return adj_fail(HRW_EINVAL, "Invalid input 'adjoint': null handle.");
  if (forward_steps) *forward_steps = h->fwd_steps;
  if (checkpoint_every) *checkpoint_every = h->used_every;
  return HRW_OK;
}

int hrw_adjoint_tape_info(const hrw_adjoint* h, int64_t* state_bytes, int64_t* weno_tape_bytes) {
  if (!h) return adj_fail(HRW_EINVAL, "Invalid input 'adjoint': null handle.");
  const int64_t bytes = (int64_t)sizeof(double) * h->line.n;
  if (state_bytes) *state_bytes = h->used_every > 0 ? bytes * (3 * h->used_every + 1) : 0;
  if (weno_tape_bytes) *weno_tape_bytes = h->wtape_used;
  return HRW_OK;
}

int hrw_adjoint_destroy(hrw_adjoint* h) {
  if (!h) return HRW_OK;
  double* bufs[] = {h->u, h->w1, h->w2, h->tgt, h->lam, h->la, h->lb, h->acc, h->J, h->tape,
                    h->wtape, h->part, h->nu};
  for (double* b : bufs)
    if (b) cudaFree(b);
  for (double* c : h->ckpt) cudaFree(c);
  if (h->own) cudaStreamDestroy(h->own);
  delete h;
  return HRW_OK;
}

}  // extern "C"
