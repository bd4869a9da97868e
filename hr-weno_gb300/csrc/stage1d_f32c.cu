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

// Warp-synchronous layout (no shared memory): each thread owns C consecutive cells and keeps
// the stencil window of its cells in registers; the k cells on either side come from the
// neighbouring lanes by shuffles, and only lanes 0 and 31 load the warp's halo from memory.
// Own cells are read with float4 loads and written with float4 stores when the thread's
// cells are inside the line (the float buffers are padded to 16-byte aligned slices).
template <int C>
__device__ __forceinline__ void load_cells(const float* __restrict__ p, int64_t j0, int64_t nc,
                                           float* out) {
  if (j0 + C <= nc) {
#pragma unroll
    for (int c = 0; c < C; c += 4) {
      const float4 v = *reinterpret_cast<const float4*>(p + j0 + c);
      out[c] = v.x, out[c + 1] = v.y, out[c + 2] = v.z, out[c + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) out[c] = p[j0 + c < nc ? j0 + c : nc - 1];
  }
}

template <int C>
__device__ __forceinline__ void store_cells(float* __restrict__ p, int64_t j0, int64_t nc,
                                            const float* v) {
  if (j0 + C <= nc) {
#pragma unroll
    for (int c = 0; c < C; c += 4)
      *reinterpret_cast<float4*>(p + j0 + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c)
      if (j0 + c < nc) p[j0 + c] = v[c];
  }
}

template <int K, int ST, int NT, int C>
__global__ void __launch_bounds__(NT) stage1d_f32c_kernel(F32CArgs a) {
  static_assert(C % 4 == 0 && C >= K, "float4 cells and a K-cell shuffle halo");
  const LineF& L = a.L;
  const int64_t nc = L.nc;
  const int lane = threadIdx.x & 31;
  const int64_t gt = (int64_t)blockIdx.x * NT + threadIdx.x;
  const int64_t j0 = gt * C;
  if ((gt - lane) * C >= nc) return;  // whole warp past the line (uniform across the warp)
  constexpr unsigned FULL = 0xffffffffu;

  // ---- state window: w = cells j0 - K .. j0 + C + K - 1 -----------------------------------------
  float hi[C], lo[C], dv[C];
  load_cells<C>(a.hi, j0, nc, hi);
  load_cells<C>(a.lo, j0, nc, lo);
  if (a.dv) load_cells<C>(a.dv, j0, nc, dv);
  else {
#pragma unroll
    for (int c = 0; c < C; ++c) dv[c] = 0.f;
  }
  float wh[C + 2 * K], wm[C + 2 * K];  // hi and lo + dv of the window
#pragma unroll
  for (int c = 0; c < C; ++c) {
    wh[K + c] = hi[c];
    wm[K + c] = lo[c] + dv[c];
  }
#pragma unroll
  for (int q = 0; q < K; ++q) {
    wh[q] = __shfl_up_sync(FULL, hi[C - K + q], 1);
    wm[q] = __shfl_up_sync(FULL, wm[K + C - K + q], 1);
    wh[K + C + q] = __shfl_down_sync(FULL, hi[q], 1);
    wm[K + C + q] = __shfl_down_sync(FULL, wm[K + q], 1);
  }
  if (lane == 0 || lane == 31) {  // the warp's halo, ghosts replicating v(1) and v(nc)
#pragma unroll
    for (int q = 0; q < K; ++q) {
      int64_t g = lane == 0 ? j0 - K + q : j0 + C + q;
      g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
      const float m = a.dv ? a.lo[g] + a.dv[g] : a.lo[g];
      if (lane == 0) wh[q] = a.hi[g], wm[q] = m;
      else wh[K + C + q] = a.hi[g], wm[K + C + q] = m;
    }
  }

  // ---- compensated differences d[q] = d_{j0 - K + q} and the cells' offsets ----------------------
  float d[C + 2 * K - 1];
#pragma unroll
  for (int q = 0; q < C + 2 * K - 1; ++q) d[q] = (wh[q + 1] - wh[q]) + (wm[q + 1] - wm[q]);
  float rl[C], rr[C];
#pragma unroll
  for (int c = 0; c < C; ++c) recon_diff<K>(&d[c + 1], a.eps, rl[c], rr[c]);
  // the cells next to the thread's ends: from the neighbouring lanes, or (lanes 0 / 31)
  // reconstructed here: cell j0-1 uses d[0 .. 2K-3], cell j0+C uses d[C+1 .. C+2K-2]
  float ed[2 * K];
#pragma unroll
  for (int q = 0; q < 2 * K - 2; ++q) ed[q] = lane == 31 ? d[C + 1 + q] : d[q];
  float el, er;
  recon_diff<K>(ed, a.eps, el, er);
  const float rr_left = __shfl_up_sync(FULL, rr[C - 1], 1);
  const float rl_right = __shfl_down_sync(FULL, rl[0], 1);
  const float rr_m0 = lane == 0 ? er : rr_left;
  const float rl_pC = lane == 31 ? el : rl_right;

  // ---- flux differences and the stage update -------------------------------------------------------
  float o1[C], o2[C], lq[C];  // outputs; lq = L(v) for the multistep history
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int64_t j = j0 + c;
    const float v = wh[K + c] + wm[K + c];
    const float rr_m = c == 0 ? rr_m0 : rr[c - 1];
    const float rl_p = c == C - 1 ? rl_pC : rl[c + 1];
    const float dF = j < nc ? flux_diff_f32c(L, j, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p)
                            : 0.f;
    const float qj = L.rw ? -dF * L.rw[j < nc ? j : nc - 1] : -dF;
    const float dtL = fmaf(a.c_hi, qj, a.c_lo * qj);  // dt L(v)_j
    lq[c] = qj * a.lscale;
    if constexpr (ST == FC_RHS) {
      o1[c] = lq[c];
    } else if constexpr (ST == FC_E1) {
      o1[c] = dtL;
    } else if constexpr (ST == FC_RK3B) {
      o1[c] = 0.25f * (dv[c] + dtL);
    } else {
      o1[c] = hi[c];
      o2[c] = lo[c];
      if constexpr (ST == FC_RK1) dv[c] = dtL;
      else if constexpr (ST == FC_RK2B) dv[c] = 0.5f * (dv[c] + dtL);
      else if constexpr (ST == FC_RK3C) dv[c] = (2.f / 3.f) * (dv[c] + dtL);
      else dv[c] = dtL;  // FC_MS: completed with the history below
    }
  }
  if constexpr (ST == FC_RHS || ST == FC_E1 || ST == FC_RK3B) {
    store_cells<C>(a.out, j0, nc, o1);
  } else {
    if constexpr (ST == FC_MS) {  // u' = u + (7 (u4 - u) + 50 dt L + 10 dt L4) / 32
      float h4[C], l4[C], L4[C];
      load_cells<C>(a.hi4, j0, nc, h4);
      load_cells<C>(a.lo4, j0, nc, l4);
      load_cells<C>(a.l4, j0, nc, L4);
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const float du4 = (h4[c] - o1[c]) + (l4[c] - o2[c]);
        const float dtl4 = fmaf(a.dt_hi, L4[c], a.dt_lo * L4[c]);
        dv[c] = fmaf(7.f / 32.f, du4, fmaf(50.f / 32.f, dv[c], (10.f / 32.f) * dtl4));
      }
      store_cells<C>(a.lout, j0, nc, lq);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) acc_add(o1[c], o2[c], dv[c]);
    store_cells<C>(a.hi_out, j0, nc, o1);
    store_cells<C>(a.lo_out, j0, nc, o2);
  }
}

template <int K, int ST, int NT, int C>
static cudaError_t launch_shape(const F32CArgs& a, cudaStream_t s) {
  const int64_t nblk = ((int64_t)a.L.nc + NT * C - 1) / (NT * C);
  stage1d_f32c_kernel<K, ST, NT, C><<<(unsigned)nblk, NT, 0, s>>>(a);
  return cudaGetLastError();
}

// 2048-cell blocks (8 warps x 256 cells) for long lines, one-warp blocks of 128 cells for
// short ones so that they still spread over the SMs
template <int K, int ST>
static cudaError_t launch_k(const F32CArgs& a, cudaStream_t s) {
  if (a.L.nc >= 2 * 152 * 2048) return launch_shape<K, ST, 256, 8>(a, s);
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
