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
// buffer (other blocks still read the old state as their halo).
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_f32c.cuh"
#include "hrw_internal.h"

namespace hrw {

template <int K, int ST, int NT, int C>
__global__ void __launch_bounds__(NT) stage1d_f32c_kernel(F32CArgs a) {
  constexpr int T = NT * C;
  constexpr int H = K;
  __shared__ float sh[T + 2 * H];  // hi of cells s-H .. s+T+H-1
  __shared__ float sm[T + 2 * H];  // lo + stage increment of the same cells
  __shared__ float sRL[NT + 1];    // rl of thread t's first cell; [NT] = rl(s+T)
  __shared__ float sRR[NT + 1];    // rr of thread t's last cell at [t+1]; [0] = rr(s-1)
  const LineF& L = a.L;
  const int64_t nc = L.nc;
  const int64_t s = (int64_t)blockIdx.x * T;
  const int tid = threadIdx.x;

  for (int q = tid; q < T + 2 * H; q += NT) {
    int64_t g = s - H + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    sh[q] = a.hi[g];
    sm[q] = a.dv ? a.lo[g] + a.dv[g] : a.lo[g];
  }
  __syncthreads();

  // ---- compensated differences and offsets of the thread's cells -------------------------------
  const int l0 = tid * C;  // local index of the first cell; sh[l0 + H] is its hi
  float d[C + 2 * K - 1];  // d[q] = d_{j0 - K + q}
#pragma unroll
  for (int q = 0; q < C + 2 * K - 1; ++q)
    d[q] = (sh[l0 + q + 1] - sh[l0 + q]) + (sm[l0 + q + 1] - sm[l0 + q]);
  float rl[C], rr[C];
#pragma unroll
  for (int c = 0; c < C; ++c) recon_diff<K>(&d[c + 1], a.eps, rl[c], rr[c]);
  sRL[tid] = rl[0];
  sRR[tid + 1] = rr[C - 1];
  if (tid >= NT - 2) {  // block-edge cells s-1 (rr) and s+T (rl)
    const int which = tid - (NT - 2);
    const int lc = which == 0 ? H - 1 : H + T;  // local index of the edge cell
    float de[2 * K];
#pragma unroll
    for (int q = 0; q < 2 * K - 2; ++q) {  // d_{cell-K+1+q}
      const int m = lc - K + 1 + q;
      de[q] = (sh[m + 1] - sh[m]) + (sm[m + 1] - sm[m]);
    }
    float el, er;
    recon_diff<K>(de, a.eps, el, er);
    if (which == 0) sRR[0] = er;
    else sRL[NT] = el;
  }
  __syncthreads();

  // ---- flux differences and the stage update -----------------------------------------------------
  const int64_t j0 = s + l0;
  if (j0 >= nc) return;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int64_t j = j0 + c;
    if (j >= nc) break;
    const int lj = l0 + H + c;
    const float v = sh[lj] + sm[lj];
    const float rr_m = c == 0 ? sRR[tid] : rr[c - 1];
    const float rl_p = c == C - 1 ? sRL[tid + 1] : rl[c + 1];
    const float dF = flux_diff_f32c(L, j, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p);
    const float qj = L.rw ? -dF * L.rw[j] : -dF;
    const float dtL = fmaf(a.c_hi, qj, a.c_lo * qj);  // dt L(v)_j
    if constexpr (ST == FC_RHS) {
      a.out[j] = qj * a.lscale;
    } else if constexpr (ST == FC_E1) {
      a.out[j] = dtL;
    } else if constexpr (ST == FC_RK3B) {
      a.out[j] = 0.25f * (a.dv[j] + dtL);
    } else {
      float hi = a.hi[j], lo = a.lo[j], inc;
      if constexpr (ST == FC_RK1) {
        inc = dtL;
      } else if constexpr (ST == FC_RK2B) {
        inc = 0.5f * (a.dv[j] + dtL);
      } else if constexpr (ST == FC_RK3C) {
        inc = (2.f / 3.f) * (a.dv[j] + dtL);
      } else {  // FC_MS
        const float du4 = (a.hi4[j] - hi) + (a.lo4[j] - lo);
        const float l4 = a.l4[j];
        const float dtl4 = fmaf(a.dt_hi, l4, a.dt_lo * l4);
        inc = fmaf(7.f / 32.f, du4, fmaf(50.f / 32.f, dtL, (10.f / 32.f) * dtl4));
        a.lout[j] = qj * a.lscale;
      }
      acc_add(hi, lo, inc);
      a.hi_out[j] = hi;
      a.lo_out[j] = lo;
    }
  }
}

template <int K, int ST>
static cudaError_t launch_k(const F32CArgs& a, cudaStream_t s) {
  constexpr int NT = 128, C = 8;
  const int64_t nblk = ((int64_t)a.L.nc + NT * C - 1) / (NT * C);
  stage1d_f32c_kernel<K, ST, NT, C><<<(unsigned)nblk, NT, 0, s>>>(a);
  return cudaGetLastError();
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
  widen_f32_kernel<<<(unsigned)(nb < 152 * 16 ? nb : 152 * 16), 256, 0, s>>>(x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_split_f64(const double* u, float* hi, float* lo, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + 255) / 256;
  split_f64_kernel<<<(unsigned)(nb < 152 * 16 ? nb : 152 * 16), 256, 0, s>>>(u, hi, lo, n);
  return cudaGetLastError();
}
cudaError_t launch_merge_f64(const float* hi, const float* lo, double* u, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + 255) / 256;
  merge_f64_kernel<<<(unsigned)(nb < 152 * 16 ? nb : 152 * 16), 256, 0, s>>>(hi, lo, u, n);
  return cudaGetLastError();
}

}  // namespace hrw
