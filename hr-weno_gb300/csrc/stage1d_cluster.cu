// stage1d_cluster.cu - every step of an rktvd integrate call of a short uniform 1D line in one
// launch of one thread-block cluster.
//
// A short line (the reference's example 1 has 500 cells) is bound by latency, not by
// bandwidth or arithmetic: launched stage by stage, each of its 3 x 1201 stages waits for the
// previous kernel to drain and the next to start.  Here the line lives in the distributed
// shared memory of one cluster of up to 16 CTAs for the whole call:
//   * CTA r owns cells [r NT, r NT + NT), one per thread, and holds them, with a k-cell halo on
//     each side, in three shared buffers: U (u^n), A (the first stage's output) and B (the
//     second's);
//   * a stage computes the CTA's own cells from the halo-extended stencil input (the same
//     reconstruction, flux and combine code as stage1d_kernel, so the same bits), then one
//     cluster barrier (release / acquire) publishes them, and each CTA copies the k cells it
//     needs from each neighbour's buffer over DSMEM into its halo;
//   * a buffer is overwritten only one cluster barrier after the neighbours last read it, so
//     one barrier per stage suffices.  Ghost cells outside the line replicate v(1) and v(nc)
//     (src/hrweno_weno.f90:172-173).
// The time loop is the reference's (src/hrweno_tvdode.f90:136-171); t is advanced on the host.
//
// Shape.  On GB300 a warp's FP64 instruction holds its SM sub-partition's FP64 unit for about
// 66 clocks whatever its active lanes, and a warp's independent FP64 instructions do not
// overlap, so a stage takes (FP64 instructions per thread) x 66 clocks for any count of cells
// per warp, up to one warp per sub-partition.  Hence one cell per thread, up to 4 cell warps
// per CTA, and the two block-edge reconstructions (cells s - 1 and s + NT, recomputed from the
// halo) on a fifth warp of their own, which runs beside the cell warps instead of after them
// (3.3 instead of 5.3 us per stage on the 500-cell line).
#include <cooperative_groups.h>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"
#include "hrw_stage.cuh"

namespace hrw {

namespace {

namespace cg = cooperative_groups;

constexpr int kMaxCluster = 16;

// One stage of the CTA's own cells: out = stage(in), stencil input `in` (halo-extended, in[0]
// is cell s - K), `u` the state u^n (own cells at u[K ..]).  Threads 0 .. NT-1 take one cell
// each; lanes 0 and 1 of the warp after them reconstruct cells s - 1 and s + NT.  The last CTA
// of the line also fills its ghost cells (positions K + owned .. NT + 2K - 1 replicate cell
// nc - 1) before the barrier, since its neighbour reads some of them when the last CTA owns
// fewer than K cells.
template <int K, int ST, bool STRICT, int NT>
__device__ __forceinline__ void cluster_stage(const StageArgs& a, const double* in, const double* u,
                                              double* out, double* sL, double* sR, int64_t s,
                                              int owned, bool last) {
  const LineArgs& L = a.L;
  const int tid = threadIdx.x;
  double vl[1], vr[1];
  if (tid < NT) {
    double w[1 + 2 * K];
#pragma unroll
    for (int q = 0; q < 1 + 2 * K; ++q) w[q] = in[tid + q];  // v(s + tid - K + q)
    if constexpr (STRICT) recon_strict<K>(&w[K], a.eps, vl[0], vr[0]);
    else recon_fast<K, 1>(w, a.eps, vl, vr);
    sL[tid] = vl[0];
    sR[tid + 1] = vr[0];
  } else if (tid < NT + 2) {  // cells s - 1 (vr) and s + NT (vl)
    const int which = tid - NT;
    const double* p = in + (which == 0 ? K - 1 : K + NT);
    double el, er;
    if constexpr (STRICT) recon_strict<K>(p, a.eps, el, er);
    else recon_fast_one<K>(p, a.eps, el, er);
    if (which == 0) sR[0] = er;
    else sL[NT] = el;
  }
  __syncthreads();
  if (tid >= owned) return;  // also every thread of the edge warp (owned <= NT)
  const int64_t j = s + tid;
  const double FL = numflux<STRICT>(L, sR[tid], vl[0], j);
  const double FR = numflux<STRICT>(L, vr[0], sL[tid + 1], j + 1);
  const double dF = flux_diff<STRICT>(L, j, FL, FR, vr[0]);
  // the combines index the CTA's buffers by the local cell (uniform line: no per-cell widths)
  StageArgs b = a;
  b.u = u + K;
  b.out = out + K;
  const double v = in[K + tid];
  if constexpr (STRICT) combine_strict<ST>(b, tid, v, rn_div(-dF, L.rx));
  else combine_fast<ST>(b, tid, v, dF, L.rws0);
  if (last && tid == owned - 1) {  // the thread of cell nc - 1
    const double g = out[K + owned - 1];
    for (int q = K + owned; q < NT + 2 * K; ++q) out[q] = g;
  }
}

// After a cluster barrier: the halo of `buf` from the neighbours' copies of the same buffer
// (the left ghosts of the first CTA replicate cell 0; the last CTA's right ghosts are written
// by its stage), then a block barrier.
template <int K, int NT>
__device__ __forceinline__ void fill_halo(cg::cluster_group& cl, double* buf, int rank, int nrank) {
  const int tid = threadIdx.x;
  if (tid < K) {  // cells s - K + tid
    buf[tid] = rank == 0 ? buf[K] : cl.map_shared_rank(buf, rank - 1)[tid + NT];
  } else if (tid < 2 * K && rank < nrank - 1) {  // cells s + NT + (tid - K)
    buf[NT + tid] = cl.map_shared_rank(buf, rank + 1)[tid];
  }
  __syncthreads();
}

template <int K, bool STRICT, int ORDER, int NT>
__global__ void __launch_bounds__(NT + 32) rk_cluster_kernel(StageArgs a, double* u_io, int64_t nsteps) {
  static_assert(NT >= 2 * K && NT % 32 == 0, "the halo lanes and whole cell warps");
  __shared__ double U[NT + 2 * K], A[NT + 2 * K], B[NT + 2 * K];
  __shared__ double sL[NT + 1], sR[NT + 1];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank(), nrank = (int)cl.num_blocks();
  const bool last = rank == nrank - 1;
  const int64_t nc = a.L.nc, s = (int64_t)rank * NT;
  const int owned = (int)(nc - s < NT ? nc - s : NT);
  const int tid = threadIdx.x;
  // own cells; the last CTA also its ghosts (cell nc - 1 repeated)
  for (int q = tid; q < (last ? NT + K : NT); q += NT + 32) U[K + q] = u_io[s + (q < owned ? q : owned - 1)];
  cl.sync();
  fill_halo<K, NT>(cl, U, rank, nrank);
  double* cur = U;  // order 1 alternates between U and A
  double* nxt = A;
  for (int64_t n = 0; n < nsteps; ++n) {
    if constexpr (ORDER == 1) {
      cluster_stage<K, ST_EULER, STRICT, NT>(a, cur, cur, nxt, sL, sR, s, owned, last);
      cl.sync();
      fill_halo<K, NT>(cl, nxt, rank, nrank);
      double* t = cur;
      cur = nxt;
      nxt = t;
    } else {
      cluster_stage<K, ST_EULER, STRICT, NT>(a, U, U, A, sL, sR, s, owned, last);
      cl.sync();
      fill_halo<K, NT>(cl, A, rank, nrank);
      if constexpr (ORDER == 2) {
        cluster_stage<K, ST_RK2B, STRICT, NT>(a, A, U, U, sL, sR, s, owned, last);
      } else {
        cluster_stage<K, ST_RK3B, STRICT, NT>(a, A, U, B, sL, sR, s, owned, last);
        cl.sync();
        fill_halo<K, NT>(cl, B, rank, nrank);
        cluster_stage<K, ST_RK3C, STRICT, NT>(a, B, U, U, sL, sR, s, owned, last);
      }
      cl.sync();
      fill_halo<K, NT>(cl, U, rank, nrank);
    }
  }
  for (int q = tid; q < owned; q += NT + 32) u_io[s + q] = cur[K + q];
  // no CTA leaves while a neighbour may still read its buffers
  cl.sync();
}

template <int K, bool STRICT, int ORDER, int NT>
cudaError_t launch_shape(const StageArgs& a, double* u, int64_t nsteps, cudaStream_t s) {
  const int nrank = (int)((a.L.nc + NT - 1) / NT);
  auto kern = rk_cluster_kernel<K, STRICT, ORDER, NT>;
  if (nrank > 8) {
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)nrank);
  cfg.blockDim = dim3(NT + 32);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)nrank;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a, u, nsteps);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

// Cells per CTA: the fewest cell warps that spread the line over at most 16 CTAs (up to 4
// warps, one per sub-partition, cost no extra time per stage; 8 take about twice as long).
template <int K, bool STRICT, int ORDER>
cudaError_t launch_order(const StageArgs& a, double* u, int64_t nsteps, cudaStream_t s) {
  const int64_t nc = a.L.nc;
  if (nc <= kMaxCluster * 32) return launch_shape<K, STRICT, ORDER, 32>(a, u, nsteps, s);
  if (nc <= kMaxCluster * 64) return launch_shape<K, STRICT, ORDER, 64>(a, u, nsteps, s);
  if (nc <= kMaxCluster * 128) return launch_shape<K, STRICT, ORDER, 128>(a, u, nsteps, s);
  return launch_shape<K, STRICT, ORDER, 256>(a, u, nsteps, s);
}

template <int K, bool STRICT>
cudaError_t launch_k(const StageArgs& a, int order, double* u, int64_t nsteps, cudaStream_t s) {
  if (order == 1) return launch_order<K, STRICT, 1>(a, u, nsteps, s);
  if (order == 2) return launch_order<K, STRICT, 2>(a, u, nsteps, s);
  return launch_order<K, STRICT, 3>(a, u, nsteps, s);
}

}  // namespace

bool cluster_line_ok(const StageArgs& a) {
  const LineArgs& L = a.L;
  // at least 6 cells (the last CTA's ghosts and the halo lanes assume a line longer than the
  // stencil); uniform grids only (the combines index the CTA's buffers, not per-cell widths)
  if (L.nc < 6 || L.nc > kMaxCluster * 256 || L.width || L.xe || a.cnu) return false;
  int dev = 0, major = 0;  // clusters of 16 CTAs: sm_90 and later
  const bool ok = cudaGetDevice(&dev) == cudaSuccess &&
                  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) == cudaSuccess &&
                  major >= 9;
  if (!ok) cudaGetLastError();
  return ok;
}

cudaError_t launch_rk_cluster(const StageArgs& a, int k, int order, bool strict, double* u,
                              int64_t nsteps, cudaStream_t s) {
  if (nsteps <= 0) return cudaSuccess;
  if (k == 1) return strict ? launch_k<1, true>(a, order, u, nsteps, s) : launch_k<1, false>(a, order, u, nsteps, s);
  if (k == 2) return strict ? launch_k<2, true>(a, order, u, nsteps, s) : launch_k<2, false>(a, order, u, nsteps, s);
  return strict ? launch_k<3, true>(a, order, u, nsteps, s) : launch_k<3, false>(a, order, u, nsteps, s);
}

}  // namespace hrw
