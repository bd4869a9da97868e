// misc.cu - the smaller kernels of the hot path:
//  * stage kernel of the linear test ODE u_i' = a_i u_i (test/test_tvdode.f90:107-111), which
//    exercises the integrators without a spatial operator;
//  (each in double, and in float for the REAL32 handles, which take the reference order)
//  * weno_calc_cnu on the device (src/hrweno_weno.f90:221-297): Shu eq. 2.20 coefficients of a
//    non-uniform grid, one thread per (cell, r, j), in the reference's operation order;
//  * reconstruction with per-cell coefficients (src/hrweno_weno.f90:170,177-181).
#include <atomic>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"
#include "hrw_stage.cuh"

namespace hrw {

int device_sms() {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];  // 0: not looked up yet
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return 152;
  }
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n > 0) return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return 152;
  }
  cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

// ---------------------------------------------------------------------------------------------
// R = double (FAST or STRICT) or float (REAL32, reference order only)
template <class R, int ST, bool STRICT>
__global__ void stage_linear_kernel(const R* __restrict__ rates, StageArgsT<R> a, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const R v = a.v[i];
    const R dt = a.dt;
    if constexpr (STRICT) {
      combine_strict<ST>(a, i, v, rn_mul(rates[i], v));
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

template <class R, bool STRICT>
static cudaError_t launch_linear_st(const R* rates, const StageArgsT<R>& a, int64_t n, int stage,
                                    cudaStream_t s) {
  const int nt = 256;
  int64_t nb = (n + nt - 1) / nt;
  if (nb > (int64_t)device_sms() * 16) nb = (int64_t)device_sms() * 16;
  switch (stage) {
    case ST_RHS: stage_linear_kernel<R, ST_RHS, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_EULER: stage_linear_kernel<R, ST_EULER, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_RK2B: stage_linear_kernel<R, ST_RK2B, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_RK3B: stage_linear_kernel<R, ST_RK3B, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_RK3C: stage_linear_kernel<R, ST_RK3C, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    case ST_MS: stage_linear_kernel<R, ST_MS, STRICT><<<(unsigned)nb, nt, 0, s>>>(rates, a, n); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_stage_linear(const double* rates, const StageArgs& a, int64_t n, int stage,
                                bool strict, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return strict ? launch_linear_st<double, true>(rates, a, n, stage, s)
                : launch_linear_st<double, false>(rates, a, n, stage, s);
}

cudaError_t launch_stage_linear(const float* rates, const StageArgs32& a, int64_t n, int stage,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  return launch_linear_st<float, true>(rates, a, n, stage, s);
}

// ---------------------------------------------------------------------------------------------
// weno_calc_cnu in the real type R.  xext(q), q = -(k+1) .. nc+(k+1): xedges inside, linear
// extension outside, built by the same running subtraction / addition as the reference
// (:245-255).
template <class R>
__device__ R xext_at(const R* xe, int nc, int k, int q) {
  if (q >= 0 && q <= nc) return xe[q];
  if (q < 0) {
    const R dx = rn_sub(xe[1], xe[0]);
    R x = xe[0];
    for (int p = -1; p >= q; --p) x = rn_sub(x, dx);
    return x;
  }
  const R dx = rn_sub(xe[nc], xe[nc - 1]);
  R x = xe[nc];
  for (int p = nc + 1; p <= q; ++p) x = rn_add(x, dx);
  return x;
}

template <class R>
__global__ void calc_cnu_kernel(const R* __restrict__ xe, R* __restrict__ cnu, int nc, int k) {
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
  R sum2 = R(0);
  for (int m = j + 1; m <= k; ++m) {  // (:263-295)
    R prod2 = R(1);
    for (int l = 0; l <= k; ++l) {
      if (l == m) continue;
      prod2 = rn_mul(prod2, rn_sub(xl(i - r + m), xl(i - r + l)));
    }
    R sum1 = R(0);
    for (int l = 0; l <= k; ++l) {
      if (l == m) continue;
      R prod1 = R(1);
      for (int q = 0; q <= k; ++q) {
        if (q == m || q == l) continue;
        prod1 = rn_mul(prod1, rn_sub(xr(i), xl(i - r + q)));
      }
      sum1 = rn_add(sum1, prod1);
    }
    sum2 = rn_add(sum2, rn_div(sum1, prod2));
  }
  cnu[idx] = rn_mul(sum2, rn_sub(xr(i - r + j), xl(i - r + j)));
}

template <class R>
static cudaError_t launch_cnu(const R* xedges, R* cnu, int nc, int k, cudaStream_t s) {
  const int64_t total = (int64_t)k * (k + 1) * nc;
  if (total <= 0) return cudaSuccess;
  calc_cnu_kernel<R><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(xedges, cnu, nc, k);
  return cudaGetLastError();
}

cudaError_t launch_calc_cnu(const double* xedges, double* cnu, int nc, int k, cudaStream_t s) {
  return launch_cnu<double>(xedges, cnu, nc, k, s);
}
cudaError_t launch_calc_cnu(const float* xedges, float* cnu, int nc, int k, cudaStream_t s) {
  return launch_cnu<float>(xedges, cnu, nc, k, s);
}

// ---------------------------------------------------------------------------------------------
// Reconstruction with per-cell coefficients: one cell per thread.  FAST: product-form
// weights as the uniform kernel; STRICT (and every float grid): reference order.
template <class R, int K, bool STRICT>
__global__ void recon_nonuniform_kernel(const R* __restrict__ v, const R* __restrict__ cnu,
                                        R* __restrict__ vl, R* __restrict__ vr, int nc, R eps) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  R p[2 * K - 1];  // v(i-(K-1)) .. v(i+(K-1)), ghosts = v(1), v(nc)
#pragma unroll
  for (int q = 0; q < 2 * K - 1; ++q) {
    int64_t g = i - (K - 1) + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    p[q] = v[g];
  }
  const R* ci = cnu + (int64_t)K * (K + 1) * i;  // ci(j, r) at [j + K*(r+1)]
  R l, r;
  recon_nu<K, STRICT>(p + (K - 1), ci, eps, l, r);
  vl[i] = l;
  vr[i] = r;
}

template <class R, bool STRICT>
static cudaError_t launch_nu(const R* v, const R* cnu, R* vl, R* vr, int nc, int k, R eps,
                             cudaStream_t s) {
  const unsigned nb = (unsigned)((nc + 127) / 128);
  if (k == 1) recon_nonuniform_kernel<R, 1, STRICT><<<nb, 128, 0, s>>>(v, cnu, vl, vr, nc, eps);
  else if (k == 2) recon_nonuniform_kernel<R, 2, STRICT><<<nb, 128, 0, s>>>(v, cnu, vl, vr, nc, eps);
  else recon_nonuniform_kernel<R, 3, STRICT><<<nb, 128, 0, s>>>(v, cnu, vl, vr, nc, eps);
  return cudaGetLastError();
}

cudaError_t launch_recon_nonuniform(const double* v, const double* cnu, double* vl, double* vr,
                                    int nc, int k, double eps, bool strict, cudaStream_t s) {
  if (nc <= 0) return cudaSuccess;
  return strict ? launch_nu<double, true>(v, cnu, vl, vr, nc, k, eps, s)
                : launch_nu<double, false>(v, cnu, vl, vr, nc, k, eps, s);
}

cudaError_t launch_recon_nonuniform(const float* v, const float* cnu, float* vl, float* vr, int nc,
                                    int k, float eps, cudaStream_t s) {
  if (nc <= 0) return cudaSuccess;
  return launch_nu<float, true>(v, cnu, vl, vr, nc, k, eps, s);
}

}  // namespace hrw
