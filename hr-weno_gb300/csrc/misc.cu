// misc.cu - the smaller kernels of the hot path:
//  * stage kernel of the linear test ODE u_i' = a_i u_i (test/test_tvdode.f90:107-111), which
//    exercises the integrators without a spatial operator;
//  * weno_calc_cnu on the device (src/hrweno_weno.f90:221-297): Shu eq. 2.20 coefficients of a
//    non-uniform grid, one thread per (cell, r, j), in the reference's operation order;
//  * reconstruction with per-cell coefficients (src/hrweno_weno.f90:170,177-181).
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"

namespace hrw {

// ---------------------------------------------------------------------------------------------
template <int ST, bool STRICT>
__global__ void stage_linear_kernel(const double* __restrict__ rates, StageArgs a, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double v = a.v[i];
    const double dt = a.dt;
    if constexpr (STRICT) {
      const double udot = __dmul_rn(rates[i], v);
      if constexpr (ST == ST_RHS) a.out[i] = udot;
      else if constexpr (ST == ST_EULER) a.out[i] = __dadd_rn(v, __dmul_rn(dt, udot));
      else if constexpr (ST == ST_RK2B)
        a.out[i] = __ddiv_rn(__dadd_rn(__dadd_rn(a.u[i], v), __dmul_rn(dt, udot)), 2.0);
      else if constexpr (ST == ST_RK3B)
        a.out[i] = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(3.0, a.u[i]), v), __dmul_rn(dt, udot)), 4.0);
      else if constexpr (ST == ST_RK3C)
        a.out[i] = __ddiv_rn(
            __dadd_rn(__dadd_rn(a.u[i], __dmul_rn(2.0, v)), __dmul_rn(__dmul_rn(2.0, dt), udot)), 3.0);
      else if constexpr (ST == ST_MS) {
        const double t1 = __dadd_rn(__dmul_rn(25.0, v), __dmul_rn(__dmul_rn(50.0, dt), udot));
        const double t2 = __dadd_rn(t1, __dmul_rn(7.0, a.uo4[i]));
        a.out[i] = __ddiv_rn(__dadd_rn(t2, __dmul_rn(__dmul_rn(10.0, dt), a.lo4[i])), 32.0);
        a.lout[i] = udot;
      }
    } else {
      const double udot = rates[i] * v;
      if constexpr (ST == ST_RHS) a.out[i] = udot;
      else if constexpr (ST == ST_EULER) a.out[i] = fma(dt, udot, v);
      else if constexpr (ST == ST_RK2B) a.out[i] = fma(0.5, a.u[i], fma(0.5, v, (0.5 * dt) * udot));
      else if constexpr (ST == ST_RK3B) a.out[i] = fma(0.75, a.u[i], fma(0.25, v, (0.25 * dt) * udot));
      else if constexpr (ST == ST_RK3C)  // u + 2/3 ((v - u) + dt udot): unbiased in u
        a.out[i] = fma(2.0 / 3.0, fma(dt, udot, v - a.u[i]), a.u[i]);
      else if constexpr (ST == ST_MS) {
        a.out[i] = fma(25.0 / 32.0, v,
                       fma((50.0 / 32.0) * dt, udot,
                           fma(7.0 / 32.0, a.uo4[i], ((10.0 / 32.0) * dt) * a.lo4[i])));
        a.lout[i] = udot;
      }
    }
  }
}

template <bool STRICT>
static cudaError_t launch_linear_st(const double* rates, const StageArgs& a, int64_t n, int stage,
                                    cudaStream_t s) {
  const int nt = 256;
  int64_t nb = (n + nt - 1) / nt;
  if (nb > 152 * 16) nb = 152 * 16;
  switch (stage) {
    case ST_RHS: stage_linear_kernel<ST_RHS, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_EULER: stage_linear_kernel<ST_EULER, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_RK2B: stage_linear_kernel<ST_RK2B, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_RK3B: stage_linear_kernel<ST_RK3B, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_RK3C: stage_linear_kernel<ST_RK3C, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_MS: stage_linear_kernel<ST_MS, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_stage_linear(const double* rates, const StageArgs& a, int64_t n, int stage,
                                bool strict, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return strict ? launch_linear_st<true>(rates, a, n, stage, s)
                : launch_linear_st<false>(rates, a, n, stage, s);
}

// ---------------------------------------------------------------------------------------------
// weno_calc_cnu.  xext(q), q = -(k+1) .. nc+(k+1): xedges inside, linear extension outside,
// built by the same running subtraction / addition as the reference (:245-255).
__device__ double xext_at(const double* xe, int nc, int k, int q) {
  if (q >= 0 && q <= nc) return xe[q];
  if (q < 0) {
    const double dx = __dsub_rn(xe[1], xe[0]);
    double x = xe[0];
    for (int p = -1; p >= q; --p) x = __dsub_rn(x, dx);
    return x;
  }
  const double dx = __dsub_rn(xe[nc], xe[nc - 1]);
  double x = xe[nc];
  for (int p = nc + 1; p <= q; ++p) x = __dadd_rn(x, dx);
  return x;
}

__global__ void calc_cnu_kernel(const double* __restrict__ xe, double* __restrict__ cnu, int nc, int k) {
  const int64_t nper = (int64_t)k * (k + 1);
  const int64_t total = nper * nc;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int j = (int)(idx % k);
  const int r = (int)((idx / k) % (k + 1)) - 1;
  const int i = (int)(idx / nper) + 1;
  // xl(q) = xext(q-1), xr(q) = xext(q)   (:257-259)
  auto xl = [&](int q) { return xext_at(xe, nc, k, q - 1); };
  auto xr = [&](int q) { return xext_at(xe, nc, k, q); };
  double sum2 = 0.0;
  for (int m = j + 1; m <= k; ++m) {  // (:263-295)
    double prod2 = 1.0;
    for (int l = 0; l <= k; ++l) {
      if (l == m) continue;
      prod2 = __dmul_rn(prod2, __dsub_rn(xl(i - r + m), xl(i - r + l)));
    }
    double sum1 = 0.0;
    for (int l = 0; l <= k; ++l) {
      if (l == m) continue;
      double prod1 = 1.0;
      for (int q = 0; q <= k; ++q) {
        if (q == m || q == l) continue;
        prod1 = __dmul_rn(prod1, __dsub_rn(xr(i), xl(i - r + q)));
      }
      sum1 = __dadd_rn(sum1, prod1);
    }
    sum2 = __dadd_rn(sum2, __ddiv_rn(sum1, prod2));
  }
  cnu[idx] = __dmul_rn(sum2, __dsub_rn(xr(i - r + j), xl(i - r + j)));
}

cudaError_t launch_calc_cnu(const double* xedges, double* cnu, int nc, int k, cudaStream_t s) {
  const int64_t total = (int64_t)k * (k + 1) * nc;
  if (total <= 0) return cudaSuccess;
  calc_cnu_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(xedges, cnu, nc, k);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Reconstruction with per-cell coefficients: one cell per thread.  FAST: product-form
// weights as the uniform kernel; STRICT: reference order.
template <int K, bool STRICT>
__global__ void recon_nonuniform_kernel(const double* __restrict__ v, const double* __restrict__ cnu,
                                        double* __restrict__ vl, double* __restrict__ vr, int nc,
                                        double eps) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  double p[2 * K - 1];  // v(i-(K-1)) .. v(i+(K-1)), ghosts = v(1), v(nc)
#pragma unroll
  for (int q = 0; q < 2 * K - 1; ++q) {
    int64_t g = i - (K - 1) + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    p[q] = v[g];
  }
  const double* ci = cnu + (int64_t)K * (K + 1) * i;  // ci(j, r) at [j + K*(r+1)]
  const double* c0 = p + (K - 1);                      // v(i)
  double vrr[K], vlr[K], beta[K];
#pragma unroll
  for (int r = 0; r < K; ++r) {
    double sr = 0.0, sl = 0.0;
#pragma unroll
    for (int j = 0; j < K; ++j) {
      if constexpr (STRICT) {
        sr = __dadd_rn(sr, __dmul_rn(ci[j + K * (r + 1)], c0[j - r]));
        sl = __dadd_rn(sl, __dmul_rn(ci[j + K * r], c0[j - r]));
      } else {
        sr = fma(ci[j + K * (r + 1)], c0[j - r], sr);
        sl = fma(ci[j + K * r], c0[j - r], sl);
      }
    }
    vrr[r] = sr;
    vlr[r] = sl;
  }
  if constexpr (STRICT) {
    // reuse the uniform strict path for beta and weights by re-deriving from the same p
    // (beta does not depend on the grid, src/hrweno_weno.f90:183-204)
    if constexpr (K == 1) {
      beta[0] = 0.0;
    } else if constexpr (K == 2) {
      double a = __dsub_rn(c0[1], c0[0]), b = __dsub_rn(c0[0], c0[-1]);
      beta[0] = __dmul_rn(a, a);
      beta[1] = __dmul_rn(b, b);
    } else {
      const double c13 = 13.0 / 12, c14 = 1.0 / 4;
      double a, b;
      a = __dadd_rn(__dsub_rn(c0[0], __dmul_rn(2.0, c0[1])), c0[2]);
      b = __dadd_rn(__dsub_rn(__dmul_rn(3.0, c0[0]), __dmul_rn(4.0, c0[1])), c0[2]);
      beta[0] = __dadd_rn(__dmul_rn(c13, __dmul_rn(a, a)), __dmul_rn(c14, __dmul_rn(b, b)));
      a = __dadd_rn(__dsub_rn(c0[-1], __dmul_rn(2.0, c0[0])), c0[1]);
      b = __dsub_rn(c0[-1], c0[1]);
      beta[1] = __dadd_rn(__dmul_rn(c13, __dmul_rn(a, a)), __dmul_rn(c14, __dmul_rn(b, b)));
      a = __dadd_rn(__dsub_rn(c0[-2], __dmul_rn(2.0, c0[-1])), c0[0]);
      b = __dadd_rn(__dsub_rn(c0[-2], __dmul_rn(4.0, c0[-1])), __dmul_rn(3.0, c0[0]));
      beta[2] = __dadd_rn(__dmul_rn(c13, __dmul_rn(a, a)), __dmul_rn(c14, __dmul_rn(b, b)));
    }
    double alfa[K], alfat[K], sa = 0.0, sat = 0.0;
#pragma unroll
    for (int r = 0; r < K; ++r) {
      const double e = __dadd_rn(eps, beta[r]);
      const double e2 = __dmul_rn(e, e);
      alfa[r] = __ddiv_rn(Tab<K>::d(r), e2);
      alfat[r] = __ddiv_rn(Tab<K>::d(K - 1 - r), e2);
    }
#pragma unroll
    for (int r = 0; r < K; ++r) { sa = __dadd_rn(sa, alfa[r]); sat = __dadd_rn(sat, alfat[r]); }
    double ar = 0.0, al = 0.0;
#pragma unroll
    for (int r = 0; r < K; ++r) {
      ar = __dadd_rn(ar, __dmul_rn(__ddiv_rn(alfa[r], sa), vrr[r]));
      al = __dadd_rn(al, __dmul_rn(__ddiv_rn(alfat[r], sat), vlr[r]));
    }
    vr[i] = ar;
    vl[i] = al;
  } else {
    if constexpr (K == 1) {
      vr[i] = vrr[0];
      vl[i] = vlr[0];
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
        vr[i] = num * (dent * R);
        vl[i] = numt * (den * R);
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
        vr[i] = ar;
        vl[i] = al;
      }
    }
  }
}

template <bool STRICT>
static cudaError_t launch_nu(const double* v, const double* cnu, double* vl, double* vr, int nc,
                             int k, double eps, cudaStream_t s) {
  const unsigned nb = (unsigned)((nc + 127) / 128);
  if (k == 1) recon_nonuniform_kernel<1, STRICT><<<nb, 128, 0, s>>>(v, cnu, vl, vr, nc, eps);
  else if (k == 2) recon_nonuniform_kernel<2, STRICT><<<nb, 128, 0, s>>>(v, cnu, vl, vr, nc, eps);
  else recon_nonuniform_kernel<3, STRICT><<<nb, 128, 0, s>>>(v, cnu, vl, vr, nc, eps);
  return cudaGetLastError();
}

cudaError_t launch_recon_nonuniform(const double* v, const double* cnu, double* vl, double* vr,
                                    int nc, int k, double eps, bool strict, cudaStream_t s) {
  if (nc <= 0) return cudaSuccess;
  return strict ? launch_nu<true>(v, cnu, vl, vr, nc, k, eps, s)
                : launch_nu<false>(v, cnu, vl, vr, nc, k, eps, s);
}

}  // namespace hrw
