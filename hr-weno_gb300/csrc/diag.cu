// diag.cu - diagnostics (hrweno_diag.h): the FMA throughput of the device (the denominator of
// the FP64-pipe roofline that bounds the FP64 stage kernels on GB300), the test hook for the 2D
// kernels' bounded tile wait, and the FAST reciprocal next to IEEE division.
#include <string>

#include <atomic>

#include <cuda_runtime.h>

#include "../../include/hrweno_diag.h"
#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"

namespace {

template <typename T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
    x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int rate(int iters, double* result) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  const int blocks = sms * 8, threads = 256;
  T* buf = nullptr;
  if ((e = cudaMalloc(&buf, sizeof(T) * (size_t)blocks * threads)) != cudaSuccess)
    return hrw::set_error(HRW_ENOMEM, cudaGetErrorString(e));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
    e = cudaEventRecord(e0);
    if (e == cudaSuccess) {
      fma_chains<T><<<blocks, threads>>>(buf, iters, T(0.999999), T(1e-7));
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && ms < best) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  *result = (double)blocks * threads * iters * 16 * 8 / (best * 1e-3);
  return HRW_OK;
}

__global__ void rcp_kernel(const double* __restrict__ x, double* __restrict__ fast,
                           double* __restrict__ exact, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    fast[i] = hrw::rcp_fast(x[i]);
    exact[i] = __ddiv_rn(1.0, x[i]);
  }
}

}  // namespace

extern "C" int hrw_diag_fma_rates(double* dfma, double* ffma) {
  int rc = HRW_OK;
  if (dfma && (rc = rate<double>(256, dfma)) != HRW_OK) return rc;
  if (ffma && (rc = rate<float>(4096, ffma)) != HRW_OK) return rc;
  return HRW_OK;
}

extern "C" int hrw_diag_set_tile_wait_limit(int polls) {
  cudaError_t e = hrw::stage2d_set_tile_wait_limit(polls);
  if (e == cudaSuccess) e = hrw::stage2d_f32c_set_tile_wait_limit(polls);
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  return HRW_OK;
}

extern "C" int hrw_diag_rcp(const double* x, double* fast, double* exact, int n) {
  if (!x || !fast || !exact || n < 0) return hrw::set_error(HRW_EINVAL, "Invalid input: null pointer.");
  if (n == 0) return HRW_OK;
  rcp_kernel<<<(n + 255) / 256, 256>>>(x, fast, exact, n);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  return HRW_OK;
}

extern "C" int hrw_diag_mixed_soft(int enable) {
  const cudaError_t e = hrw::mixed_set_soft(enable);
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  return HRW_OK;
}

extern "C" int hrw_diag_mixed_hard_warps(unsigned long long* count, int reset) {
  if (!count) return hrw::set_error(HRW_EINVAL, "Invalid input: null pointer.");
  const cudaError_t e = hrw::mixed_hard_warps(count, reset != 0);
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  return HRW_OK;
}

extern "C" int hrw_diag_upwind(int enable) {
  hrw::g_upwind_enabled.store(enable != 0 ? 1 : 0, std::memory_order_relaxed);
  return HRW_OK;
}
