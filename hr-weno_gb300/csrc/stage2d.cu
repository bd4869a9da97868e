// stage2d.cu - fused 2D stage kernel: dimension-by-dimension WENO reconstruction, numerical
// fluxes in x1 and x2, the conservative update and the TVD stage combine, one pass per stage.
//
// Follows, for one stage of the reference's time loop on the 2D population-balance example:
//   x1 sweep over contiguous rows       example/example2_pbe_2d_fv.f90:97-103
//   x2 sweep over strided columns       example/example2_pbe_2d_fv.f90:106-112
//   boundary fluxes                     example/example2_pbe_2d_fv.f90:117-120
//   update -(dF1)/dx1 - (dF2)/dx2       example/example2_pbe_2d_fv.f90:123-127
//   weno_reconstruct                    src/hrweno_weno.f90:129-219
//   godunov / lax_friedrichs            src/hrweno_fluxes.f90:22-76
//   mstvd / rktvd stage update          src/hrweno_tvdode.f90:139-167,257
//
// Layout: u((j-1)*nc1 + i), x1 fastest (example2...f90:124).  One block owns a 32 x 32 tile
// of cells; the tile plus a k-cell halo in each direction is staged in shared memory once
// (ghosts replicate the first/last cell of each row and column, src/hrweno_weno.f90:172-173).
// Each of the 128 threads reconstructs a segment of 8 cells along x1 from a register window,
// then a segment of 8 cells along x2; segment-edge states are exchanged through shared
// memory and the tile-edge states are recomputed by one lane each.  The x1 flux divergence
// is parked in shared memory; the x2 pass adds its own and writes each cell once.
//
// Upwind specialisation (UPW): for the Godunov flux of f = g(x) u with g > 0 on the whole
// domain in both directions, F = g vm exactly (hrw_stage.cuh: upwind_flux), so only the left
// state vr of every interface is reconstructed.
//
// Non-uniform lines (NU): a line with xedges reconstructs every cell with its own coefficients
// cnu (src/hrweno_weno.f90:170,177-181; "any smooth grid can be used",
// example/example2_pbe_2d_fv.f90:36-39), divides by its cells' widths and evaluates the flux
// function at its true interface coordinates; a uniform line of the same problem keeps the
// tables.
#include <atomic>
#include <type_traits>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"
#include "hrw_stage.cuh"
#include "hrw_tma.cuh"

namespace hrw {

namespace {

constexpr int TX = 32, TY = 32, C = 8, NT = 128;
static_assert(TX * TY == NT * C, "one segment of C cells per thread and direction");
static_assert(TX == 32 && TY / C == NT / 32 && TX / C == NT / 32, "warp-per-segment mapping");

// default poll limit of the first wait for the tile copies (stage2d_set_tile_wait_limit
// changes it per device; the launch passes it in the arguments), and the limit of the wait that
// drains the copies after a timeout
constexpr int kTileWaitPolls = 1 << 20;
constexpr int BX = 40, BY = 38;  // TMA box of the tile plus halo: x from bx - 4, y from by - 3

// Reconstruction of C consecutive cells g0 .. g0 + C - 1 of a non-uniform line of n cells, with
// p[q * stride] = v(g0 - K + q) and cell g's coefficients at cnu + K(K+1) g (cells past the
// line's end, whose results are not used, read the last cell's).
template <class R, int K, bool STRICT>
__device__ __forceinline__ void recon_nu_seg(const R* p, int stride, const R* cnu, int64_t g0,
                                             int64_t n, R eps, R* vl, R* vr) {
#pragma unroll
  for (int c = 0; c < C; ++c) {
    R w[2 * K - 1];  // v(g0 + c - (K-1)) .. v(g0 + c + (K-1))
#pragma unroll
    for (int q = 0; q < 2 * K - 1; ++q) w[q] = p[(c + 1 + q) * stride];
    const int64_t g = g0 + c < n ? g0 + c : n - 1;
    recon_nu<K, STRICT>(w + (K - 1), cnu + (int64_t)K * (K + 1) * g, eps, vl[c], vr[c]);
  }
}

// TMA: the tile plus halo of the stage input comes in as one 40 x 38 box at (bx - 4, by - 3)
// (x on a 16-byte boundary for doubles and floats alike), completing on a block mbarrier; the
// block then builds its padded tile from shared memory, replicating edge cells into the ghosts (the box
// reads zeros outside the grid).  Otherwise every thread gathers the tile from global memory.
// Both give the same tile, so the same bits.
// R = double (HRW_F64, FAST or STRICT) or float (HRW_F32, reference order only).
template <class R, int K, int ST, bool STRICT, bool UPW, bool TMA, bool NU>
__global__ void __launch_bounds__(NT) stage2d_kernel(const __grid_constant__ CUtensorMap Mv, StageArgsT<R> a) {
  static_assert(STRICT || std::is_same<R, double>::value, "float grids take the reference order");
  constexpr int H = K;
  constexpr int RW = TX + 2 * H;      // loaded row width
  constexpr int SW = RW + 1;          // odd row stride: the x1 pass reads 32 rows per warp
  constexpr int SQ = TX + 1;          // odd stride of the parked x1 divergence
  constexpr int NSX = TX / C, NSY = TY / C;
  __shared__ R sv[(TY + 2 * H) * SW];
  __shared__ R sq[TY * SQ];
  __shared__ R sLx[TY * (NSX + 1)], sRx[TY * (NSX + 1)];  // [row][segment edge]
  __shared__ R sLy[(NSY + 1) * TX], sRy[(NSY + 1) * TX];  // [segment edge][column]
  __shared__ alignas(128) R tbox[TMA ? BY * BX : 1];
  __shared__ alignas(8) uint64_t bar;

  const LineArgsT<R>& L1 = a.L;
  const LineArgsT<R>& L2 = a.L2;
  const int64_t n1 = L1.nc, n2 = L2.nc, ld = a.ld;
  const int64_t bx = (int64_t)blockIdx.x * TX, by = (int64_t)blockIdx.y * TY;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  // ---- stage the tile and its halo ------------------------------------------------------------
  if constexpr (TMA) {
    if (tid == 0) mbar_init(&bar);
    __syncthreads();
    if (tid == 0) {
      mbar_expect_tx(&bar, BY * BX * (uint32_t)sizeof(R));
      tma_load_2d(tbox, &Mv, (int)bx - 4, (int)by - 3, &bar);
    }
    // bounded wait; on a timeout every thread of the block learns of it, the block waits
    // (with the default bound) for its copy to land and leaves, and the host sees the flag
    const bool ok = mbar_wait(&bar, 0, a.tile_wait_polls);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicExch(a.timeout_flag, 1u);
      mbar_wait(&bar, 0, kTileWaitPolls);
      return;
    }
    const int ibx = (int)bx, iby = (int)by, in1 = (int)n1, in2 = (int)n2;
    for (int q = tid; q < (TY + 2 * H) * RW; q += NT) {
      const int row = q / RW, col = q - row * RW;
      int gy = iby - H + row, gx = ibx - H + col;
      gy = gy < 0 ? 0 : (gy >= in2 ? in2 - 1 : gy);
      gx = gx < 0 ? 0 : (gx >= in1 ? in1 - 1 : gx);
      sv[row * SW + col] = tbox[(gy - (iby - 3)) * BX + (gx - (ibx - 4))];
    }
  } else {
    for (int q = tid; q < (TY + 2 * H) * RW; q += NT) {
      const int row = q / RW, col = q - row * RW;
      int64_t gy = by - H + row, gx = bx - H + col;
      gy = gy < 0 ? 0 : (gy >= n2 ? n2 - 1 : gy);
      gx = gx < 0 ? 0 : (gx >= n1 ? n1 - 1 : gx);
      sv[row * SW + col] = a.v[gy * ld + gx];
    }
  }
  __syncthreads();

  // ---- x1 reconstruction: row r = lane, segment sg = warp ------------------------------------
  const int r = lane, sg = warp;
  R vl[C], vr[C];
  {
    const R* row = &sv[(r + H) * SW + sg * C];  // row[q] = v(bx + sg*C - H + q)
    auto uniform = [&]() {
      if constexpr (STRICT) {
#pragma unroll
        for (int c = 0; c < C; ++c) recon_strict<K>(row + H + c, a.eps, vl[c], vr[c]);
      } else {
        R w[C + 2 * K];
#pragma unroll
        for (int q = 0; q < C + 2 * K; ++q) w[q] = row[q];
        recon_fast<K, C, !UPW>(w, a.eps, vl, vr);
      }
    };
    if constexpr (NU) {
      if (a.cnu) recon_nu_seg<R, K, STRICT>(row, 1, a.cnu, bx + sg * C, n1, a.eps, vl, vr);
      else uniform();
    } else {
      uniform();
    }
    if constexpr (!UPW) sLx[r * (NSX + 1) + sg] = vl[0];
    sRx[r * (NSX + 1) + sg + 1] = vr[C - 1];
  }
  // tile-edge cells: warp 0 the left column (vr of x1 = bx-1), warp 1 the right column (vl of
  // x1 = bx+TX); warp 2 the row above (vr of x2 = by-1), warp 3 the row below (vl of by+TY)
  {
    R el, er;
    const R* p;
    int stride;
    if (warp < 2) {
      p = &sv[(lane + H) * SW + (warp == 0 ? H - 1 : H + TX)];
      stride = 1;
    } else {
      p = &sv[(warp == 2 ? H - 1 : H + TY) * SW + H + lane];
      stride = SW;
    }
    const bool need = !UPW || warp == 0 || warp == 2;
    bool done = false;
    if constexpr (NU) {
      const R* ci = warp < 2 ? a.cnu : a.cnu2;
      if (need && ci) {
        const int64_t n = warp < 2 ? n1 : n2;
        int64_t g = warp == 0 ? bx - 1 : (warp == 1 ? bx + TX : (warp == 2 ? by - 1 : by + TY));
        g = g < 0 ? 0 : (g >= n ? n - 1 : g);
        R w[2 * K - 1];
#pragma unroll
        for (int q = 0; q < 2 * K - 1; ++q) w[q] = p[(q - (K - 1)) * stride];
        recon_nu<K, STRICT>(w + (K - 1), ci + (int64_t)K * (K + 1) * g, a.eps, el, er);
        done = true;
      }
    }
    if (need && !done) {
      if constexpr (STRICT) recon_strict_strided<K>(p, stride, a.eps, el, er);
      else recon_fast_one<K>(p, a.eps, el, er, stride);
    }
    if (need) {
      if (warp == 0) sRx[lane * (NSX + 1)] = er;
      else if (warp == 1) sLx[lane * (NSX + 1) + NSX] = el;
      else if (warp == 2) sRy[lane] = er;
      else sLy[NSY * TX + lane] = el;
    }
  }
  __syncthreads();

  // ---- x1 fluxes of the segment; park the x1 divergence --------------------------------------
  {
    const int64_t j0 = bx + sg * C;
    R F[C + 1];
    if constexpr (UPW) {
      F[0] = upwind_flux<STRICT>(L1, sRx[r * (NSX + 1) + sg], j0);
#pragma unroll
      for (int c = 1; c <= C; ++c) F[c] = upwind_flux<STRICT>(L1, vr[c - 1], j0 + c);
    } else {
      F[0] = numflux<STRICT>(L1, sRx[r * (NSX + 1) + sg], vl[0], j0);
#pragma unroll
      for (int c = 1; c < C; ++c) F[c] = numflux<STRICT>(L1, vr[c - 1], vl[c], j0 + c);
      F[C] = numflux<STRICT>(L1, vr[C - 1], sLx[r * (NSX + 1) + sg + 1], j0 + C);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t gx = j0 + c;
      R t = R(0);
      if (gx < n1) {
        const R dF = flux_diff<STRICT>(L1, gx, F[c], F[c + 1], vr[c]);
        if constexpr (STRICT) t = rn_div(dF, L1.width ? L1.width[gx] : L1.rx);
        else t = (L1.rws ? L1.rws[gx] : L1.rws0) * dF;
      }
      sq[r * SQ + sg * C + c] = t;
    }
  }

  // ---- x2 reconstruction: column = lane, segment sy = warp -----------------------------------
  const int col = lane, sy = warp;
  {
    const R* cp = &sv[(sy * C) * SW + H + col];  // cp[q*SW] = v(x2 = by + sy*C - H + q)
    auto uniform = [&]() {
      if constexpr (STRICT) {
#pragma unroll
        for (int c = 0; c < C; ++c) recon_strict_strided<K>(cp + (H + c) * SW, SW, a.eps, vl[c], vr[c]);
      } else {
        R w[C + 2 * K];
#pragma unroll
        for (int q = 0; q < C + 2 * K; ++q) w[q] = cp[q * SW];
        recon_fast<K, C, !UPW>(w, a.eps, vl, vr);
      }
    };
    if constexpr (NU) {
      if (a.cnu2) recon_nu_seg<R, K, STRICT>(cp, SW, a.cnu2, by + sy * C, n2, a.eps, vl, vr);
      else uniform();
    } else {
      uniform();
    }
    if constexpr (!UPW) sLy[sy * TX + col] = vl[0];
    sRy[(sy + 1) * TX + col] = vr[C - 1];
  }
  __syncthreads();

  // ---- x2 fluxes, the update and the stage combine -------------------------------------------
  {
    const int64_t gx = bx + col;
    const int64_t j0 = by + sy * C;
    R F[C + 1];
    if constexpr (UPW) {
      F[0] = upwind_flux<STRICT>(L2, sRy[sy * TX + col], j0);
#pragma unroll
      for (int c = 1; c <= C; ++c) F[c] = upwind_flux<STRICT>(L2, vr[c - 1], j0 + c);
    } else {
      F[0] = numflux<STRICT>(L2, sRy[sy * TX + col], vl[0], j0);
#pragma unroll
      for (int c = 1; c < C; ++c) F[c] = numflux<STRICT>(L2, vr[c - 1], vl[c], j0 + c);
      F[C] = numflux<STRICT>(L2, vr[C - 1], sLy[(sy + 1) * TX + col], j0 + C);
    }
    if (gx < n1) {
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const int64_t gy = j0 + c;
        if (gy >= n2) break;
        const R dF = flux_diff<STRICT>(L2, gy, F[c], F[c + 1], vr[c]);
        const int ly = sy * C + c;
        const R v = sv[(ly + H) * SW + H + col];
        const R t1 = sq[ly * SQ + col];
        const int64_t j = gy * ld + gx;
        if constexpr (STRICT) {
          // vdot = -((f1(i)-f1(i-1))/dx1) - (f2(j)-f2(j-1))/dx2   (example2...f90:123-127)
          const R t2 = rn_div(dF, L2.width ? L2.width[gy] : L2.rx);
          combine_strict<ST>(a, j, v, rn_sub(-t1, t2));
        } else {
          const double q = fma(L2.rws ? L2.rws[gy] : L2.rws0, dF, t1);
          combine_fast<ST>(a, j, v, q, 1.0);
        }
      }
    }
  }
}

template <class R, int K, int ST, bool STRICT, bool UPW>
cudaError_t launch_k(const StageArgsT<R>& a, cudaStream_t s) {
  const dim3 grid((unsigned)((a.L.nc + TX - 1) / TX), (unsigned)((a.L2.nc + TY - 1) / TY));
  CUtensorMap mv{};
  if (a.cnu || a.cnu2)  // non-uniform lines: the general flux path (upwind is only a shortcut)
    stage2d_kernel<R, K, ST, STRICT, false, false, true><<<grid, NT, 0, s>>>(mv, a);
  else if (a.ld == a.L.nc && tile_map_2d(a.v, (int)sizeof(R), (int)a.L.nc, (int)a.L2.nc, BX, BY, &mv))
    stage2d_kernel<R, K, ST, STRICT, UPW, true, false><<<grid, NT, 0, s>>>(mv, a);
  else
    stage2d_kernel<R, K, ST, STRICT, UPW, false, false><<<grid, NT, 0, s>>>(mv, a);
  return cudaGetLastError();
}

template <class R, int K, bool STRICT, bool UPW>
cudaError_t launch_st(const StageArgsT<R>& a, int stage, cudaStream_t s) {
  switch (stage) {
    case ST_RHS: return launch_k<R, K, ST_RHS, STRICT, UPW>(a, s);
    case ST_EULER: return launch_k<R, K, ST_EULER, STRICT, UPW>(a, s);
    case ST_RK2B: return launch_k<R, K, ST_RK2B, STRICT, UPW>(a, s);
    case ST_RK3B: return launch_k<R, K, ST_RK3B, STRICT, UPW>(a, s);
    case ST_RK3C: return launch_k<R, K, ST_RK3C, STRICT, UPW>(a, s);
    case ST_MS: return launch_k<R, K, ST_MS, STRICT, UPW>(a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

// Every stage kind of one (real type, numerics, k).  The nine combinations compile as separate
// objects, HRW_PART = 0 .. 8 in the order below (the build compiles this file once per part,
// in parallel); part 0 also holds the dispatch.  Built without HRW_PART, the file holds all.
template <class R, bool STRICT, int K>
cudaError_t stage2d_launch(const StageArgsT<R>& a, int stage, cudaStream_t s) {
  return a.upwind ? launch_st<R, K, STRICT, true>(a, stage, s) : launch_st<R, K, STRICT, false>(a, stage, s);
}
extern template cudaError_t stage2d_launch<double, false, 1>(const StageArgsT<double>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<double, false, 2>(const StageArgsT<double>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<double, false, 3>(const StageArgsT<double>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<double, true, 1>(const StageArgsT<double>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<double, true, 2>(const StageArgsT<double>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<double, true, 3>(const StageArgsT<double>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<float, true, 1>(const StageArgsT<float>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<float, true, 2>(const StageArgsT<float>&, int, cudaStream_t);
extern template cudaError_t stage2d_launch<float, true, 3>(const StageArgsT<float>&, int, cudaStream_t);
#if !defined(HRW_PART) || HRW_PART == 0
template cudaError_t stage2d_launch<double, false, 1>(const StageArgsT<double>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 1
template cudaError_t stage2d_launch<double, false, 2>(const StageArgsT<double>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 2
template cudaError_t stage2d_launch<double, false, 3>(const StageArgsT<double>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 3
template cudaError_t stage2d_launch<double, true, 1>(const StageArgsT<double>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 4
template cudaError_t stage2d_launch<double, true, 2>(const StageArgsT<double>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 5
template cudaError_t stage2d_launch<double, true, 3>(const StageArgsT<double>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 6
template cudaError_t stage2d_launch<float, true, 1>(const StageArgsT<float>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 7
template cudaError_t stage2d_launch<float, true, 2>(const StageArgsT<float>&, int, cudaStream_t);
#endif
#if !defined(HRW_PART) || HRW_PART == 8
template cudaError_t stage2d_launch<float, true, 3>(const StageArgsT<float>&, int, cudaStream_t);
#endif

#if !defined(HRW_PART) || HRW_PART == 0
namespace {
// poll limit of the first wait for the tile copies, per device (stage2d_set_tile_wait_limit);
// stored + 1, so that 0 reads as the default
constexpr int kMaxDevices = 64;
std::atomic<int> g_tile_wait[kMaxDevices];

int tile_wait_polls() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return kTileWaitPolls;
  }
  const int v = g_tile_wait[dev].load(std::memory_order_relaxed);
  return v > 0 ? v - 1 : kTileWaitPolls;
}
}  // namespace

cudaError_t stage2d_set_tile_wait_limit(int polls) {
  int dev = 0;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  g_tile_wait[dev].store(polls < 0 ? 0 : polls + 1, std::memory_order_relaxed);
  return cudaSuccess;
}

template <class R>
static cudaError_t dispatch(StageArgsT<R> a, int k, int stage, bool strict, cudaStream_t s) {
  if (a.L.nc <= 0 || a.L2.nc <= 0) return cudaSuccess;
  if (a.L2.nc > 65535LL * TY || !a.timeout_flag) return cudaErrorInvalidValue;
  a.tile_wait_polls = tile_wait_polls();
  if constexpr (std::is_same<R, float>::value) {
    (void)strict;
    return k == 1 ? stage2d_launch<R, true, 1>(a, stage, s)
                  : (k == 2 ? stage2d_launch<R, true, 2>(a, stage, s) : stage2d_launch<R, true, 3>(a, stage, s));
  } else if (strict) {
    return k == 1 ? stage2d_launch<R, true, 1>(a, stage, s)
                  : (k == 2 ? stage2d_launch<R, true, 2>(a, stage, s) : stage2d_launch<R, true, 3>(a, stage, s));
  } else {
    return k == 1 ? stage2d_launch<R, false, 1>(a, stage, s)
                  : (k == 2 ? stage2d_launch<R, false, 2>(a, stage, s) : stage2d_launch<R, false, 3>(a, stage, s));
  }
}

cudaError_t launch_stage2d(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s) {
  return dispatch(a, k, stage, strict, s);
}

cudaError_t launch_stage2d(const StageArgs32& a, int k, int stage, cudaStream_t s) {
  return dispatch(a, k, stage, true, s);
}
#endif

}  // namespace hrw
