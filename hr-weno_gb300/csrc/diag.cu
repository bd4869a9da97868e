// diag.cu - FMA throughput of the device (hrweno_diag.h): the denominator of the FP64-pipe
// roofline that bounds the FP64 stage kernels on GB300.
#include <string>

#include <cuda_runtime.h>

#include "../../include/hrweno_diag.h"
#include "../../include/hrweno_gpu.h"

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
  if (cudaGetDevice(&dev) != cudaSuccess) return HRW_ECUDA;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  T* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(T) * (size_t)blocks * threads) != cudaSuccess) return HRW_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, threads>>>(buf, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (cudaGetLastError() != cudaSuccess) return HRW_ECUDA;
  *result = (double)blocks * threads * iters * 16 * 8 / (best * 1e-3);
  return HRW_OK;
}

}  // namespace

extern "C" int hrw_diag_fma_rates(double* dfma, double* ffma) {
  int rc = HRW_OK;
  if (dfma && (rc = rate<double>(256, dfma)) != HRW_OK) return rc;
  if (ffma && (rc = rate<float>(4096, ffma)) != HRW_OK) return rc;
  return HRW_OK;
}
