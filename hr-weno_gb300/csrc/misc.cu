// misc.cu - the smaller kernels of the hot path:
//  * stage kernel of the linear test ODE u_i' = a_i u_i (test/test_tvdode.f90:107-111), which
//    exercises the integrators without a spatial operator;
//  * weno_calc_cnu on the device (src/hrweno_weno.f90:221-297): Shu eq. 2.20 coefficients of a
//    non-uniform grid, one thread per (cell, r, j), in the reference's operation order;
//  * reconstruction with per-cell coefficients (src/hrweno_weno.f90:170,177-181).
#include <atomic>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"

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
  if (nb > (int64_t)device_sms() * 16) nb = (int64_t)device_sms() * 16;
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
  double l, r;
  recon_nu<K, STRICT>(p + (K - 1), ci, eps, l, r);
  vl[i] = l;
  vr[i] = r;
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
