// stage1d_f32c.cu - fused 1D stage kernel of the compensated FP32 form (hrw_f32c.cuh):
// WENO reconstruction + numerical flux + conservative difference + TVD stage combine in
// difference form, with the state u = hi + lo held as a float pair.
//
// Stage kinds, in increment form (dv is the stored stage increment, u1 = u + d1, ...):
//   FC_RHS    out = L(u + dv)
//   FC_E1     out = d1 = dt L(u)                                  (rktvd :139/:150/:163)
//   FC_RK1    u'  = u + dt L(u)                                   (rktvd :139)
//   FC_RK2B   u'  = u + (d1 + dt L(u + d1)) / 2                    (rktvd :152)
//   FC_RK3B   out = d2 = (d1 + dt L(u + d1)) / 4                   (rktvd :165)
//   FC_RK3C   u'  = u + 2/3 (d2 + dt L(u + d2))                    (rktvd :167)
//   FC_MS     u'  = u + (7 (u4 - u) + 50 dt L(u) + 10 dt L4) / 32, lout = L(u)  (mstvd :257)
// Each is the reference's formula (src/hrweno_tvdode.f90) rewritten relative to u; the new
// state is accumulated by an error-free two-sum into (hi, lo) and written to a second
// buffer (other warps still read the old state as their halo).
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_f32c.cuh"
#include "hrw_internal.h"

namespace hrw {

template <int K, int ST, int NT, int C, int FK, bool NU = false>
__global__ void __launch_bounds__(NT) stage1d_f32c_kernel(F32CArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t gt = (int64_t)blockIdx.x * NT + threadIdx.x;
  if ((gt - lane) * C >= a.L.nc) return;  // whole warp past the line (uniform across the warp)
  f32c_pass<K, ST, C, FK, NU>(a, gt * C, lane);
}

template <int K, int ST, int NT, int C>
static cudaError_t launch_shape(const F32CArgs& a, cudaStream_t s) {
  const int64_t nblk = ((int64_t)a.L.nc + NT * C - 1) / (NT * C);
  const int fk = 2 * (a.L.fn != HRW_FN_BURGERS) + (a.L.flux != HRW_FLUX_LAX_FRIEDRICHS);
  switch (fk) {  // the flux kind as a compile-time constant
    case 0: stage1d_f32c_kernel<K, ST, NT, C, 0><<<(unsigned)nblk, NT, 0, s>>>(a); break;
    case 1: stage1d_f32c_kernel<K, ST, NT, C, 1><<<(unsigned)nblk, NT, 0, s>>>(a); break;
    case 2: stage1d_f32c_kernel<K, ST, NT, C, 2><<<(unsigned)nblk, NT, 0, s>>>(a); break;
    default: stage1d_f32c_kernel<K, ST, NT, C, 3><<<(unsigned)nblk, NT, 0, s>>>(a); break;
  }
  return cudaGetLastError();
}

// 2048-cell blocks (8 warps x 256 cells) for long lines, one-warp blocks of 128 cells for
// short ones so that they still spread over the SMs
template <int K, int ST>
static cudaError_t launch_k(const F32CArgs& a, cudaStream_t s) {
  // long lines: 8 cells per thread; 256-thread blocks for k = 3, 128 for k = 2 (measured on the
  // 2^24-cell line: 0.229 vs 0.231 ms per RK3 step for k = 3, 0.184 vs 0.172 ms for k = 2)
  if (a.L.cnu) {  // a non-uniform line: per-cell coefficients, the general flux path
    const int64_t nblk = ((int64_t)a.L.nc + 127) / 128;
    stage1d_f32c_kernel<K, ST, 32, 4, -1, true><<<(unsigned)nblk, 32, 0, s>>>(a);
    return cudaGetLastError();
  }
  if (a.L.nc >= 2 * (int64_t)device_sms() * 2048)
    return K == 2 ? launch_shape<K, ST, 128, 8>(a, s) : launch_shape<K, ST, 256, 8>(a, s);
  return launch_shape<K, ST, 32, 4>(a, s);
}

template <int K>
static cudaError_t launch_st(const F32CArgs& a, int stage, cudaStream_t s) {
  switch (stage) {
    case FC_RHS: return launch_k<K, FC_RHS>(a, s);
    case FC_E1: return launch_k<K, FC_E1>(a, s);
    case FC_RK1: return launch_k<K, FC_RK1>(a, s);
    case FC_RK2B: return launch_k<K, FC_RK2B>(a, s);
    case FC_RK3B: return launch_k<K, FC_RK3B>(a, s);
    case FC_RK3C: return launch_k<K, FC_RK3C>(a, s);
    case FC_MS: return launch_k<K, FC_MS>(a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_stage1d_f32c(const F32CArgs& a, int k, int stage, cudaStream_t s) {
  if (a.L.nc <= 0) return cudaSuccess;
  if (k == 1) return launch_st<1>(a, stage, s);
  if (k == 2) return launch_st<2>(a, stage, s);
  return launch_st<3>(a, stage, s);
}

// ---- split / merge between the caller's FP64 array and the (hi, lo) state ----------------------
__global__ void split_f64_kernel(const double* __restrict__ u, float* __restrict__ hi,
                                 float* __restrict__ lo, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double x = u[i];
    const float h = __double2float_rn(x);
    hi[i] = h;
    lo[i] = __double2float_rn(x - (double)h);
  }
}
__global__ void merge_f64_kernel(const float* __restrict__ hi, const float* __restrict__ lo,
                                 double* __restrict__ u, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    u[i] = (double)hi[i] + (double)lo[i];
}

__global__ void widen_f32_kernel(const float* __restrict__ x, double* __restrict__ y, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) y[i] = x[i];
}

cudaError_t launch_widen_f32(const float* x, double* y, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + 255) / 256;
  widen_f32_kernel<<<(unsigned)(nb < device_sms() * 16 ? nb : device_sms() * 16), 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_split_f64(const double* u, float* hi, float* lo, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + 255) / 256;
  split_f64_kernel<<<(unsigned)(nb < device_sms() * 16 ? nb : device_sms() * 16), 256, 0, s>>>(u, hi, lo, n);
  return cudaGetLastError();
}
cudaError_t launch_merge_f64(const float* hi, const float* lo, double* u, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + 255) / 256;
  merge_f64_kernel<<<(unsigned)(nb < device_sms() * 16 ? nb : device_sms() * 16), 256, 0, s>>>(hi, lo, u, n);
  return cudaGetLastError();
}

}  // namespace hrw
