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
//
// Loading.  When a row holds a multiple of 4 floats (16-byte row pitch), one thread issues TMA
// tensor copies (cp.async.bulk.tensor.2d) of the tile plus halo of hi, lo and the stage
// increment -- a 40 x 38 box at (bx - 4, by - 3), the x origin on a 16-byte boundary -- and,
// for the multistep stage, of the 32 x 32 history tiles, all completing on one mbarrier; the
// block then builds its padded compensated tile from shared memory, replicating edge cells
// into the ghosts (the box reads zeros outside the grid).  Otherwise every thread gathers the
// tile from global memory.  Both loaders feed the same arithmetic, so both give the same bits.
//
// Non-uniform grids (a line with xedges) take the gathering loader and the general flux path,
// each cell of such a line reconstructing with its own coefficients (recon_diff_nu).  Their
// kernels are compiled as part 1 of this file (HRW_PART = 1), the uniform ones as part 0.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/hrweno_gpu.h"
#include "hrw_f32c.cuh"
#include "hrw_internal.h"
#include "hrw_tma.cuh"

namespace hrw {

// part 1 (non-uniform grids)
cudaError_t launch_stage2d_f32c_nu(const F32CArgs& a, int k, int stage, cudaStream_t s);

namespace {

constexpr int TX = 32, TY = 32, C = 8, NT = 128;
constexpr int BX = 40, BY = 38;  // TMA box of the tile plus halo: x from bx - 4, y from by - 3
constexpr int BS = (BY * BX + 31) / 32 * 32;  // its shared-memory stride: 128-byte aligned boxes

// TMA descriptors of one launch: the tile plus halo of hi, lo and the stage increment, and the
// 32 x 32 history tiles of the multistep stage
struct TileMaps {
  CUtensorMap hi, lo, dv;
  CUtensorMap h4, l4, L4;
};

// poll limit of the first wait for the tile copies (stage2d_f32c_set_tile_wait_limit)
constexpr int kTileWaitPolls = 1 << 20;
__device__ int g_tile_wait_limit = kTileWaitPolls;

// WENO offsets of the C cells of a segment from its differences d[0 .. C+2K-2]; for k = 3 the
// eps + 13/12 (second difference)^2 terms are computed once per window position (as the 1D pass).
// WL = false (upwind, k = 3): rr only.  NU: on a non-uniform line (L.cnu) each cell j0 + c
// takes its own coefficients (recon_diff_nu); a uniform line of the same grid the tables.
template <int K, bool WL = true, bool NU = false>
__device__ __forceinline__ void segment_recon(const float* d, float eps, float* rl, float* rr,
                                              const LineF& L, int j0) {
  if constexpr (NU) {
    if (L.cnu) {
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const int j = j0 + c < L.nc ? j0 + c : L.nc - 1;
        recon_diff_nu<K>(&d[c + 1], L.cnu + (int64_t)K * (K + 1) * j, eps, rl[c], rr[c]);
      }
      return;
    }
  }
  if constexpr (K == 3) {
    float t[C + 4];
#pragma unroll
    for (int m = 2; m < C + 4; ++m) t[m] = shared_t(d[m - 1], d[m], eps);
#pragma unroll
    for (int c = 0; c < C; ++c)
      recon_diff3_shared<WL>(&d[c + 1], t[c + 4], t[c + 3], t[c + 2], rl[c], rr[c]);
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) recon_diff<K>(&d[c + 1], eps, rl[c], rr[c]);
  }
}

// one cell's offsets from its 2K-2 differences (tile-edge cells), the same arithmetic; NU:
// cell j of a non-uniform line with its coefficients
template <int K, bool WL = true, bool NU = false>
__device__ __forceinline__ void cell_recon(const float* de, float eps, float& el, float& er,
                                           const LineF& L, int j) {
  if constexpr (NU) {
    if (L.cnu) {
      j = j < 0 ? 0 : (j >= L.nc ? L.nc - 1 : j);
      recon_diff_nu<K>(de, L.cnu + (int64_t)K * (K + 1) * j, eps, el, er);
      return;
    }
  }
  if constexpr (K == 3) {
    float te[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) te[q] = shared_t(de[q], de[q + 1], eps);
    recon_diff3_shared<WL>(de, te[2], te[1], te[0], el, er);
  } else {
    recon_diff<K>(de, eps, el, er);
  }
}

// flux difference of cell j of a segment: `interior` (no cell of the segment on the line's
// ends) takes the path without the boundary rules when the numerical flux is known (FKI = 4
// Lax-Friedrichs, 5 Godunov; the flux function is a uniform branch), with the same arithmetic;
// UPW (upwind Godunov of g u, g > 0): the interior takes flux_diff_upwind, and the line's end
// cells the general path with any right states (rl = 0), which the upwind flux ignores
// NU: the general path, g at the true edges of a non-uniform line
template <int FKI, bool UPW = false, bool NU = false>
__device__ __forceinline__ float seg_flux(const LineF& L, bool interior, int j, float v, float rr_m,
                                          float d_m, float rl_j, float rr_j, float d_j, float rl_p) {
  if constexpr (NU) {
    static_assert(FKI < 0 && !UPW, "non-uniform grids take the general flux path");
    if (L.cnu) return flux_diff_f32c<true>(L, j, v, rr_m, d_m, rl_j, rr_j, d_j, rl_p);
    return flux_diff_f32c(L, j, v, rr_m, d_m, rl_j, rr_j, d_j, rl_p);
  } else if constexpr (UPW) {
    if (interior) return flux_diff_upwind(L, j, v, rr_m, d_m, rr_j);
    return flux_diff_f32c_call(L, j, v, rr_m, d_m, 0.f, rr_j, d_j, 0.f);
  } else if constexpr (FKI >= 0) {
    if (interior) return flux_diff_interior<FKI>(L, j, v, rr_m, d_m, rl_j, rr_j, d_j, rl_p);
    return flux_diff_f32c_call(L, j, v, rr_m, d_m, rl_j, rr_j, d_j, rl_p);
  } else {
    return flux_diff_f32c(L, j, v, rr_m, d_m, rl_j, rr_j, d_j, rl_p);
  }
}

template <int K, int ST, bool TMA, bool HAS_DV, int FKI, bool UPW = false, bool NU = false>
__global__ void __launch_bounds__(NT) stage2d_f32c_kernel(const __grid_constant__ TileMaps M,
                                                          F32CArgs a) {
  static_assert(!UPW || K == 3, "the upwind pass is written for k = 3");
  static_assert(!NU || (!TMA && FKI < 0 && !UPW), "non-uniform grids: gathered tiles, general flux");
  constexpr int H = K;
  constexpr int RW = TX + 2 * H, SW = RW + 1, SQ = TX + 1;
  constexpr int NSX = TX / C, NSY = TY / C;
  constexpr bool MS = ST == FC_MS;
  constexpr int NB = HAS_DV ? 3 : 2;  // TMA tiles: hi, lo (, increment)
  __shared__ float sh[(TY + 2 * H) * SW];
  __shared__ float sm[(TY + 2 * H) * SW];
  __shared__ float sq[TY * SQ];                                 // x1 part of dt L
  __shared__ float sLx[TY * (NSX + 1)], sRx[TY * (NSX + 1)];  // rl / rr at segment edges
  __shared__ float sLy[(NSY + 1) * TX], sRy[(NSY + 1) * TX];
  // TMA boxes; in the multistep stage the same space then takes the three 32 x 32 history
  // tiles (the padded tile holds each cell's hi and lo exactly, as there is no increment)
  static_assert(!MS || HAS_DV || 2 * BS >= 3 * TX * TY, "history tiles fit the box space");
  __shared__ alignas(128) float tb[TMA ? NB : 1][TMA ? BS : 1];
  float* const hb = &tb[0][0];
  __shared__ alignas(8) uint64_t bar;
  const LineF& L1 = a.L;
  const LineF& L2 = a.L2;
  const int n1 = L1.nc, n2 = L2.nc;
  const int64_t ld = a.ld;
  const int bx = blockIdx.x * TX, by = blockIdx.y * TY;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  if constexpr (TMA) {
    if (tid == 0) mbar_init(&bar);
    __syncthreads();
    if (tid == 0) {
      mbar_expect_tx(&bar, NB * BY * BX * 4);
      tma_load_2d(tb[0], &M.hi, bx - 4, by - 3, &bar);
      tma_load_2d(tb[1], &M.lo, bx - 4, by - 3, &bar);
      if constexpr (HAS_DV) tma_load_2d(tb[NB - 1], &M.dv, bx - 4, by - 3, &bar);
    }
    // bounded wait; on a timeout every thread of the block learns of it, the block waits
    // (bounded again) for its copies to land and leaves, and the host sees the flag
    const bool ok = mbar_wait(&bar, 0, g_tile_wait_limit);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicExch(a.timeout_flag, 1u);
      mbar_wait(&bar, 0, kTileWaitPolls);
      return;
    }
    if (bx >= H && bx + TX + H <= n1 && by >= H && by + TY + H <= n2) {
      // no ghost cell in the tile: row by row, a warp per row and a lane per column
      for (int row = warp; row < TY + 2 * H; row += NT / 32) {
        const int src = (row + 3 - H) * BX + 4 - H;
        for (int col = lane; col < RW; col += 32) {
          sh[row * SW + col] = tb[0][src + col];
          sm[row * SW + col] = HAS_DV ? tb[1][src + col] + tb[NB - 1][src + col] : tb[1][src + col];
        }
      }
    } else {
      for (int q = tid; q < (TY + 2 * H) * RW; q += NT) {
        const int row = q / RW, col = q - row * RW;
        int gy = by - H + row, gx = bx - H + col;
        gy = gy < 0 ? 0 : (gy >= n2 ? n2 - 1 : gy);
        gx = gx < 0 ? 0 : (gx >= n1 ? n1 - 1 : gx);
        const int src = (gy - (by - 3)) * BX + (gx - (bx - 4));
        sh[row * SW + col] = tb[0][src];
        sm[row * SW + col] = HAS_DV ? tb[1][src] + tb[NB - 1][src] : tb[1][src];
      }
    }
  } else {
    for (int q = tid; q < (TY + 2 * H) * RW; q += NT) {
      const int row = q / RW, col = q - row * RW;
      int gy = by - H + row, gx = bx - H + col;
      gy = gy < 0 ? 0 : (gy >= n2 ? n2 - 1 : gy);
      gx = gx < 0 ? 0 : (gx >= n1 ? n1 - 1 : gx);
      const int64_t g = gy * ld + gx;
      sh[row * SW + col] = a.hi[g];
      sm[row * SW + col] = HAS_DV ? a.lo[g] + a.dv[g] : a.lo[g];
    }
  }
  if constexpr (TMA && MS) {
    // the boxes have been read (generic proxy) before the history copies (async proxy)
    // overwrite them: fence, then the block barrier below, then the copies
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if constexpr (TMA && MS) {
    if (tid == 0) {
      mbar_expect_tx(&bar, 3 * TX * TY * 4);
      tma_load_2d(hb, &M.h4, bx, by, &bar);
      tma_load_2d(hb + TX * TY, &M.l4, bx, by, &bar);
      tma_load_2d(hb + 2 * TX * TY, &M.L4, bx, by, &bar);
    }
  }

  // ---- x1: differences and offsets of the row segment ------------------------------------------
  const int r = lane, sg = warp;
  float d[C + 2 * K - 1], rl[C], rr[C];
  {
    const int base = (r + H) * SW + sg * C;  // local cell bx + sg*C - H + q at base + q
#pragma unroll
    for (int q = 0; q < C + 2 * K - 1; ++q)
      d[q] = (sh[base + q + 1] - sh[base + q]) + (sm[base + q + 1] - sm[base + q]);
    segment_recon<K, !UPW, NU>(d, a.eps, rl, rr, L1, bx + sg * C);
    if constexpr (!UPW) sLx[r * (NSX + 1) + sg] = rl[0];
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
    if (!UPW || warp == 0 || warp == 2) {  // upwind: the right-edge cells' rl are not needed
#pragma unroll
      for (int q = 0; q < 2 * K - 2; ++q) {
        const int m0 = p + (q - (K - 1)) * stride, m1 = m0 + stride;
        de[q] = (sh[m1] - sh[m0]) + (sm[m1] - sm[m0]);
      }
      float el, er;
      const int je = warp == 0 ? bx - 1 : warp == 1 ? bx + TX : warp == 2 ? by - 1 : by + TY;
      cell_recon<K, !UPW, NU>(de, a.eps, el, er, warp < 2 ? L1 : L2, je);
      if (warp == 0) sRx[lane * (NSX + 1)] = er;
      else if (warp == 1) sLx[lane * (NSX + 1) + NSX] = el;
      else if (warp == 2) sRy[lane] = er;
      else sLy[NSY * TX + lane] = el;
    }
  }
  __syncthreads();

  // ---- x1 flux differences -> dt/dx1 (-dF1) in shared memory -----------------------------------
  {
    const int j0 = bx + sg * C;
    const bool interior = j0 > 0 && j0 + C < n1;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int gx = j0 + c;
      float t = 0.f;
      if (gx < n1) {
        const int lj = (r + H) * SW + H + sg * C + c;
        const float v = sh[lj] + sm[lj];
        const float rr_m = c == 0 ? sRx[r * (NSX + 1) + sg] : rr[c - 1];
        const float rl_j = UPW ? 0.f : rl[c];
        const float rl_p = UPW ? 0.f : (c == C - 1 ? sLx[r * (NSX + 1) + sg + 1] : rl[c + 1]);
        const float dF =
            seg_flux<FKI, UPW, NU>(L1, interior, gx, v, rr_m, d[c + K - 1], rl_j, rr[c], d[c + K], rl_p);
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
    segment_recon<K, !UPW, NU>(d, a.eps, rl, rr, L2, by + sy * C);
    if constexpr (!UPW) sLy[sy * TX + col] = rl[0];
    sRy[(sy + 1) * TX + col] = rr[C - 1];
  }
  __syncthreads();

  // ---- x2 flux differences, dt L and the stage update ------------------------------------------
  if constexpr (TMA && MS) {  // the history tiles (bounded wait, as for the boxes)
    const bool ok = mbar_wait(&bar, 1, kTileWaitPolls);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicExch(a.timeout_flag, 1u);
      mbar_wait(&bar, 1, kTileWaitPolls);
      return;
    }
  }
  const int gx = bx + col;
  if (gx >= n1) return;
  const int j0 = by + sy * C;
  const bool interior = j0 > 0 && j0 + C < n2;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int gy = j0 + c;
    if (gy >= n2) break;
    const int ly = sy * C + c;
    const int lj = (ly + H) * SW + H + col;
    const float v = sh[lj] + sm[lj];
    const float rr_m = c == 0 ? sRy[sy * TX + col] : rr[c - 1];
    const float rl_j = UPW ? 0.f : rl[c];
    const float rl_p = UPW ? 0.f : (c == C - 1 ? sLy[(sy + 1) * TX + col] : rl[c + 1]);
    const float dF2 =
        seg_flux<FKI, UPW, NU>(L2, interior, gy, v, rr_m, d[c + K - 1], rl_j, rr[c], d[c + K], rl_p);
    const float q1 = L1.rw ? sq[ly * SQ + col] * L1.rw[gx] : sq[ly * SQ + col];
    const float q2 = L2.rw ? -dF2 * L2.rw[gy] : -dF2;
    // dt L = c1 q1 + c2 q2 with the dt/dx float pairs; L = q1/dx1 + q2/dx2
    const float dtL = fmaf(a.c_hi, q1, fmaf(a.c_lo, q1, fmaf(a.c2_hi, q2, a.c2_lo * q2)));
    const float Lv = fmaf(q1, a.lscale, q2 * a.lscale2);
    const int64_t j = gy * ld + gx;
    if constexpr (TMA && MS) {  // hi, lo from the padded tile; history from the tiles
      const int q = ly * TX + col;
      f32c_update_h<ST>(a, j, sh[lj], sm[lj], 0.f, dtL, Lv, hb[q], hb[TX * TY + q], hb[2 * TX * TY + q]);
    } else if constexpr (TMA) {
      const int src = (ly + 3) * BX + col + 4;  // the cell in the halo box
      const float h = tb[0][src], l = tb[1][src];
      const float dv = HAS_DV ? tb[NB - 1][src] : 0.f;
      f32c_update_h<ST>(a, j, h, l, dv, dtL, Lv, 0.f, 0.f, 0.f);
    } else {
      const float h = a.hi[j], l = a.lo[j];
      const float dv = HAS_DV ? a.dv[j] : 0.f;
      f32c_update<ST>(a, j, h, l, dv, dtL, Lv);
    }
  }
}

#if !defined(HRW_PART) || HRW_PART == 0
template <int K, int ST, bool TMA, bool HAS_DV>
cudaError_t launch_kt(const TileMaps& M, const F32CArgs& a, cudaStream_t s) {
  const dim3 grid((unsigned)((a.L.nc + TX - 1) / TX), (unsigned)((a.L2.nc + TY - 1) / TY));
  if constexpr (K == 3 && TMA) {
    if (a.L.flux == HRW_FLUX_LAX_FRIEDRICHS)
      stage2d_f32c_kernel<K, ST, TMA, HAS_DV, 4><<<grid, NT, 0, s>>>(M, a);
    else if (a.upwind)
      stage2d_f32c_kernel<K, ST, TMA, HAS_DV, 5, true><<<grid, NT, 0, s>>>(M, a);
    else
      stage2d_f32c_kernel<K, ST, TMA, HAS_DV, 5><<<grid, NT, 0, s>>>(M, a);
  } else {
    stage2d_f32c_kernel<K, ST, TMA, HAS_DV, -1><<<grid, NT, 0, s>>>(M, a);
  }
  return cudaGetLastError();
}

template <int K, int ST>
cudaError_t launch_k(const F32CArgs& a, cudaStream_t s) {
  constexpr bool MS = ST == FC_MS;
  TileMaps M{};
  const int n1 = a.L.nc, n2 = a.L2.nc;
  const bool tma = n1 == a.ld && tile_map_2d(a.hi, 4, n1, n2, BX, BY, &M.hi) &&
                   tile_map_2d(a.lo, 4, n1, n2, BX, BY, &M.lo) &&
                   (!a.dv || tile_map_2d(a.dv, 4, n1, n2, BX, BY, &M.dv)) &&
                   (!MS || (tile_map_2d(a.hi4, 4, n1, n2, TX, TY, &M.h4) &&
                            tile_map_2d(a.lo4, 4, n1, n2, TX, TY, &M.l4) &&
                            tile_map_2d(a.l4, 4, n1, n2, TX, TY, &M.L4)));
  if constexpr (MS) {  // the multistep stage has no stage increment
    if (a.dv) return cudaErrorInvalidValue;
    return tma ? launch_kt<K, ST, true, false>(M, a, s) : launch_kt<K, ST, false, false>(M, a, s);
  } else {
    if (tma) {
      if (a.dv) return launch_kt<K, ST, true, true>(M, a, s);
      return launch_kt<K, ST, true, false>(M, a, s);
    }
    if (a.dv) return launch_kt<K, ST, false, true>(M, a, s);
    return launch_kt<K, ST, false, false>(M, a, s);
  }
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
#endif  // part 0

#if !defined(HRW_PART) || HRW_PART == 1
// Non-uniform grids: gathered tiles (each thread loads its share of the tile from global
// memory) and the general flux path; the per-cell coefficients of a non-uniform line come
// with its LineF.
template <int K, int ST, bool HAS_DV>
cudaError_t launch_nu_kt(const F32CArgs& a, cudaStream_t s) {
  const dim3 grid((unsigned)((a.L.nc + TX - 1) / TX), (unsigned)((a.L2.nc + TY - 1) / TY));
  const TileMaps M{};
  stage2d_f32c_kernel<K, ST, false, HAS_DV, -1, false, true><<<grid, NT, 0, s>>>(M, a);
  return cudaGetLastError();
}

template <int K>
cudaError_t launch_nu_k(const F32CArgs& a, int stage, cudaStream_t s) {
  const bool dv = a.dv != nullptr;
  switch (stage) {
    case FC_RHS: return dv ? launch_nu_kt<K, FC_RHS, true>(a, s) : launch_nu_kt<K, FC_RHS, false>(a, s);
    case FC_E1: return dv ? launch_nu_kt<K, FC_E1, true>(a, s) : launch_nu_kt<K, FC_E1, false>(a, s);
    case FC_RK1: return dv ? launch_nu_kt<K, FC_RK1, true>(a, s) : launch_nu_kt<K, FC_RK1, false>(a, s);
    case FC_RK2B: return dv ? launch_nu_kt<K, FC_RK2B, true>(a, s) : launch_nu_kt<K, FC_RK2B, false>(a, s);
    case FC_RK3B: return dv ? launch_nu_kt<K, FC_RK3B, true>(a, s) : launch_nu_kt<K, FC_RK3B, false>(a, s);
    case FC_RK3C: return dv ? launch_nu_kt<K, FC_RK3C, true>(a, s) : launch_nu_kt<K, FC_RK3C, false>(a, s);
    case FC_MS: return dv ? cudaErrorInvalidValue : launch_nu_kt<K, FC_MS, false>(a, s);
  }
  return cudaErrorInvalidValue;
}
#endif  // part 1

}  // namespace

#if !defined(HRW_PART) || HRW_PART == 1
cudaError_t launch_stage2d_f32c_nu(const F32CArgs& a, int k, int stage, cudaStream_t s) {
  if (k == 1) return launch_nu_k<1>(a, stage, s);
  if (k == 2) return launch_nu_k<2>(a, stage, s);
  return launch_nu_k<3>(a, stage, s);
}
#endif

#if !defined(HRW_PART) || HRW_PART == 0

// ---- TMA descriptors: cuTensorMapEncodeTiled (CUDA driver API), cached by array ---------------
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

struct MapEntry {
  const void* p;
  int elem, n1, n2, box_x, box_y;
  CUtensorMap map;
};

}  // namespace

bool tile_map_2d(const void* p, int elem_bytes, int n1, int n2, int box_x, int box_y, CUtensorMap* out) {
  static std::mutex mu;
  static std::vector<MapEntry> cache;
  if ((int64_t)n1 * elem_bytes % 16 != 0 || (reinterpret_cast<uintptr_t>(p) & 15) != 0) return false;
  std::lock_guard<std::mutex> lock(mu);
  for (const MapEntry& e : cache)
    if (e.p == p && e.elem == elem_bytes && e.n1 == n1 && e.n2 == n2 && e.box_x == box_x &&
        e.box_y == box_y) {
      *out = e.map;
      return true;
    }
  const auto fn = encode_fn();
  if (!fn) return false;
  MapEntry e{p, elem_bytes, n1, n2, box_x, box_y, {}};
  const cuuint64_t dim[2] = {(cuuint64_t)n1, (cuuint64_t)n2};
  const cuuint64_t stride[1] = {(cuuint64_t)n1 * (cuuint64_t)elem_bytes};
  const cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_y};
  const cuuint32_t estride[2] = {1, 1};
  const CUtensorMapDataType dt = elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  if (fn(&e.map, dt, 2, const_cast<void*>(p), dim, stride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  if (cache.size() >= 256) cache.erase(cache.begin());
  cache.push_back(e);
  *out = e.map;
  return true;
}

cudaError_t launch_stage2d_f32c(const F32CArgs& a, int k, int stage, cudaStream_t s) {
  if (a.L.nc <= 0 || a.L2.nc <= 0) return cudaSuccess;
  if (a.L2.nc > 65535LL * TY || !a.timeout_flag) return cudaErrorInvalidValue;
  if (a.L.cnu || a.L2.cnu) return launch_stage2d_f32c_nu(a, k, stage, s);
  if (k == 1) return launch_st<1>(a, stage, s);
  if (k == 2) return launch_st<2>(a, stage, s);
  return launch_st<3>(a, stage, s);
}

cudaError_t stage2d_f32c_set_tile_wait_limit(int polls) {
  const int v = polls < 0 ? kTileWaitPolls : polls;
  return cudaMemcpyToSymbol(g_tile_wait_limit, &v, sizeof(v));
}

#endif  // part 0

}  // namespace hrw
