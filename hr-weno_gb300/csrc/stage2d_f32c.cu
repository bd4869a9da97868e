// stage2d_f32c.cu - fused 2D stage kernel of the compensated FP32 form (hrw_f32c.cuh): the
// dimension-by-dimension right-hand side of example/example2_pbe_2d_fv.f90:73-129 in difference
// form, one pass per stage.
//
// Tiling as the FP64 2D kernel (stage2d.cu): a 32 x 32 tile plus a k halo in shared memory,
// 128 threads; each thread reconstructs an 8-cell x1 segment (warp = segment, lane = row),
// then an 8-cell x2 segment (warp = segment, lane = column).  Every difference along a line is
// compensated, (hi diff) + ((lo + stage increment) diff); each direction's flux difference is
// formed relative to the cell's own value (flux_diff_f32c), so that
//   dt L = (dt/dx1) (-dF1) + (dt/dx2) (-dF2)
// carries no cancellation of O(1) fluxes.  Stage kinds and the two-sum state update as the 1D
// compensated kernel (f32c_update).
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_f32c.cuh"
#include "hrw_internal.h"

namespace hrw {

namespace {

constexpr int TX = 32, TY = 32, C = 8, NT = 128;

template <int K, int ST>
__global__ void __launch_bounds__(NT) stage2d_f32c_kernel(F32CArgs a) {
  constexpr int H = K;
  constexpr int RW = TX + 2 * H, SW = RW + 1, SQ = TX + 1;
  constexpr int NSX = TX / C, NSY = TY / C;
  __shared__ float sh[(TY + 2 * H) * SW];
  __shared__ float sm[(TY + 2 * H) * SW];
  __shared__ float sq[TY * SQ];                                 // x1 part of dt L
  __shared__ float sLx[TY * (NSX + 1)], sRx[TY * (NSX + 1)];  // rl / rr at segment edges
  __shared__ float sLy[(NSY + 1) * TX], sRy[(NSY + 1) * TX];
  const LineF& L1 = a.L;
  const LineF& L2 = a.L2;
  const int64_t n1 = L1.nc, n2 = L2.nc, ld = a.ld;
  const int64_t bx = (int64_t)blockIdx.x * TX, by = (int64_t)blockIdx.y * TY;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int q = tid; q < (TY + 2 * H) * RW; q += NT) {
    const int row = q / RW, col = q - row * RW;
    int64_t gy = by - H + row, gx = bx - H + col;
    gy = gy < 0 ? 0 : (gy >= n2 ? n2 - 1 : gy);
    gx = gx < 0 ? 0 : (gx >= n1 ? n1 - 1 : gx);
    const int64_t g = gy * ld + gx;
    sh[row * SW + col] = a.hi[g];
    sm[row * SW + col] = a.dv ? a.lo[g] + a.dv[g] : a.lo[g];
  }
  __syncthreads();

  // ---- x1: differences and offsets of the row segment ------------------------------------------
  const int r = lane, sg = warp;
  float d[C + 2 * K - 1], rl[C], rr[C];
  {
    const int base = (r + H) * SW + sg * C;  // local cell bx + sg*C - H + q at base + q
#pragma unroll
    for (int q = 0; q < C + 2 * K - 1; ++q)
      d[q] = (sh[base + q + 1] - sh[base + q]) + (sm[base + q + 1] - sm[base + q]);
#pragma unroll
    for (int c = 0; c < C; ++c) recon_diff<K>(&d[c + 1], a.eps, rl[c], rr[c]);
    sLx[r * (NSX + 1) + sg] = rl[0];
    sRx[r * (NSX + 1) + sg + 1] = rr[C - 1];
  }
  // tile-edge cells: warp 0 rr of x1 = bx-1, warp 1 rl of x1 = bx+TX, warp 2 rr of x2 = by-1,
  // warp 3 rl of x2 = by+TY; each needs d of its cell at offsets -(K-1) .. K-2
  {
    float de[2 * K];
    int p, stride;
    if (warp < 2) {
      p = (lane + H) * SW + (warp == 0 ? H - 1 : H + TX);
      stride = 1;
    } else {
      p = (warp == 2 ? H - 1 : H + TY) * SW + H + lane;
      stride = SW;
    }
#pragma unroll
    for (int q = 0; q < 2 * K - 2; ++q) {
      const int m0 = p + (q - (K - 1)) * stride, m1 = m0 + stride;
      de[q] = (sh[m1] - sh[m0]) + (sm[m1] - sm[m0]);
    }
    float el, er;
    recon_diff<K>(de, a.eps, el, er);
    if (warp == 0) sRx[lane * (NSX + 1)] = er;
    else if (warp == 1) sLx[lane * (NSX + 1) + NSX] = el;
    else if (warp == 2) sRy[lane] = er;
    else sLy[NSY * TX + lane] = el;
  }
  __syncthreads();

  // ---- x1 flux differences -> dt/dx1 (-dF1) in shared memory -----------------------------------
  {
    const int64_t j0 = bx + sg * C;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t gx = j0 + c;
      float t = 0.f;
      if (gx < n1) {
        const int lj = (r + H) * SW + H + sg * C + c;
        const float v = sh[lj] + sm[lj];
        const float rr_m = c == 0 ? sRx[r * (NSX + 1) + sg] : rr[c - 1];
        const float rl_p = c == C - 1 ? sLx[r * (NSX + 1) + sg + 1] : rl[c + 1];
        const float dF = flux_diff_f32c(L1, gx, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p);
        t = -dF;
      }
      sq[r * SQ + sg * C + c] = t;
    }
  }

  // ---- x2: differences and offsets of the column segment ---------------------------------------
  const int col = lane, sy = warp;
  {
    const int base = (sy * C) * SW + H + col;  // row by + sy*C - H + q at base + q*SW
#pragma unroll
    for (int q = 0; q < C + 2 * K - 1; ++q) {
      const int m0 = base + q * SW, m1 = m0 + SW;
      d[q] = (sh[m1] - sh[m0]) + (sm[m1] - sm[m0]);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) recon_diff<K>(&d[c + 1], a.eps, rl[c], rr[c]);
    sLy[sy * TX + col] = rl[0];
    sRy[(sy + 1) * TX + col] = rr[C - 1];
  }
  __syncthreads();

  // ---- x2 flux differences, dt L and the stage update ------------------------------------------
  const int64_t gx = bx + col;
  if (gx >= n1) return;
  const int64_t j0 = by + sy * C;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int64_t gy = j0 + c;
    if (gy >= n2) break;
    const int ly = sy * C + c;
    const int lj = (ly + H) * SW + H + col;
    const float v = sh[lj] + sm[lj];
    const float rr_m = c == 0 ? sRy[sy * TX + col] : rr[c - 1];
    const float rl_p = c == C - 1 ? sLy[(sy + 1) * TX + col] : rl[c + 1];
    const float dF2 = flux_diff_f32c(L2, gy, v, rr_m, d[c + K - 1], rl[c], rr[c], d[c + K], rl_p);
    const float q1 = L1.rw ? sq[ly * SQ + col] * L1.rw[gx] : sq[ly * SQ + col];
    const float q2 = L2.rw ? -dF2 * L2.rw[gy] : -dF2;
    // dt L = c1 q1 + c2 q2 with the dt/dx float pairs; L = q1/dx1 + q2/dx2
    const float dtL = fmaf(a.c_hi, q1, fmaf(a.c_lo, q1, fmaf(a.c2_hi, q2, a.c2_lo * q2)));
    const float Lv = fmaf(q1, a.lscale, q2 * a.lscale2);
    const int64_t j = gy * ld + gx;
    const float h = a.hi[j], l = a.lo[j];
    const float dv = a.dv ? a.dv[j] : 0.f;
    f32c_update<ST>(a, j, h, l, dv, dtL, Lv);
  }
}

template <int K, int ST>
cudaError_t launch_k(const F32CArgs& a, cudaStream_t s) {
  const dim3 grid((unsigned)((a.L.nc + TX - 1) / TX), (unsigned)((a.L2.nc + TY - 1) / TY));
  stage2d_f32c_kernel<K, ST><<<grid, NT, 0, s>>>(a);
  return cudaGetLastError();
}

template <int K>
cudaError_t launch_st(const F32CArgs& a, int stage, cudaStream_t s) {
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

}  // namespace

cudaError_t launch_stage2d_f32c(const F32CArgs& a, int k, int stage, cudaStream_t s) {
  if (a.L.nc <= 0 || a.L2.nc <= 0) return cudaSuccess;
  if (a.L2.nc > 65535LL * TY) return cudaErrorInvalidValue;
  if (k == 1) return launch_st<1>(a, stage, s);
  if (k == 2) return launch_st<2>(a, stage, s);
  return launch_st<3>(a, stage, s);
}

}  // namespace hrw
