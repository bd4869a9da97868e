// stage1d_nu.cu - fused 1D stage kernel on a non-uniform line: the reconstruction uses the
// per-cell coefficients cnu(0:k-1,-1:k-1,1:nc) that weno(ncells, k, eps, xedges) builds
// (src/hrweno_weno.f90:100-104,170,177-181,221-297), the conservative difference divides by
// the cells' own widths (example/example1_burgers_1d_fv.f90:107) and the flux functions see
// the true interface coordinates.
//
// One cell per thread (the coefficients differ from cell to cell, so neighbouring cells share
// no candidate sums); a block owns NT cells plus a k-cell halo in shared memory, the two
// block-edge reconstructions are done by two lanes, and interface states pass between
// threads through shared memory.
#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_device.cuh"
#include "hrw_internal.h"
#include "hrw_stage.cuh"

namespace hrw {

namespace {

template <class R, int K, int ST, bool STRICT, int NT>
__global__ void __launch_bounds__(NT) stage1d_nu_kernel(StageArgsT<R> a) {
  constexpr int H = K;
  constexpr int NC = K * (K + 1);  // coefficients per cell
  __shared__ R sv[NT + 2 * H];
  __shared__ R sL[NT + 1], sR[NT + 1];  // vl of cell s+t at sL[t], vr at sR[t+1]
  const LineArgsT<R>& L = a.L;
  const int64_t nc = L.nc;
  const int64_t s = (int64_t)blockIdx.x * NT;
  const int t = threadIdx.x;
  for (int q = t; q < NT + 2 * H; q += NT) {
    int64_t g = s - H + q;
    g = g < 0 ? 0 : (g >= nc ? nc - 1 : g);
    sv[q] = a.v[g];
  }
  __syncthreads();
  const int64_t j = s + t;
  const int64_t jc = j < nc ? j : nc - 1;
  R vl, vr;
  recon_nu<K, STRICT>(&sv[H + t], a.cnu + NC * jc, a.eps, vl, vr);
  sL[t] = vl;
  sR[t + 1] = vr;
  if (t >= NT - 2) {  // block-edge cells s-1 (vr) and s+NT (vl), when they exist
    const int which = t - (NT - 2);
    int64_t e = which == 0 ? s - 1 : s + NT;
    e = e < 0 ? 0 : (e >= nc ? nc - 1 : e);
    R el, er;
    recon_nu<K, STRICT>(&sv[which == 0 ? H - 1 : H + NT], a.cnu + NC * e, a.eps, el, er);
    if (which == 0) sR[0] = er;
    else sL[NT] = el;
  }
  __syncthreads();
  if (j >= nc) return;
  const R FL = numflux<STRICT>(L, sR[t], vl, j);
  const R FR = numflux<STRICT>(L, vr, sL[t + 1], j + 1);
  const R dF = flux_diff<STRICT>(L, j, FL, FR, vr);
  const R v = sv[H + t];
  if constexpr (STRICT) combine_strict<ST>(a, j, v, rn_div(-dF, L.width[j]));
  else combine_fast<ST>(a, j, v, dF, L.rws[j]);
}

template <class R, int K, int ST, bool STRICT>
cudaError_t launch_k(const StageArgsT<R>& a, cudaStream_t s) {
  constexpr int NT = 128;
  const int64_t nblk = ((int64_t)a.L.nc + NT - 1) / NT;
  stage1d_nu_kernel<R, K, ST, STRICT, NT><<<(unsigned)nblk, NT, 0, s>>>(a);
  return cudaGetLastError();
}

template <class R, int K, bool STRICT>
cudaError_t launch_st(const StageArgsT<R>& a, int stage, cudaStream_t s) {
  switch (stage) {
    case ST_RHS: return launch_k<R, K, ST_RHS, STRICT>(a, s);
    case ST_EULER: return launch_k<R, K, ST_EULER, STRICT>(a, s);
    case ST_RK2B: return launch_k<R, K, ST_RK2B, STRICT>(a, s);
    case ST_RK3B: return launch_k<R, K, ST_RK3B, STRICT>(a, s);
    case ST_RK3C: return launch_k<R, K, ST_RK3C, STRICT>(a, s);
    case ST_MS: return launch_k<R, K, ST_MS, STRICT>(a, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_stage1d_nu(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s) {
  if (a.L.nc <= 0) return cudaSuccess;
  if (!a.cnu || !a.L.xe || !a.L.width || !a.L.rws) return cudaErrorInvalidValue;
  using D = double;
  if (k == 1) return strict ? launch_st<D, 1, true>(a, stage, s) : launch_st<D, 1, false>(a, stage, s);
  if (k == 2) return strict ? launch_st<D, 2, true>(a, stage, s) : launch_st<D, 2, false>(a, stage, s);
  return strict ? launch_st<D, 3, true>(a, stage, s) : launch_st<D, 3, false>(a, stage, s);
}

// REAL32: the reference order only, so no FAST per-cell scale (rws) is needed
cudaError_t launch_stage1d_nu(const StageArgs32& a, int k, int stage, cudaStream_t s) {
  if (a.L.nc <= 0) return cudaSuccess;
  if (!a.cnu || !a.L.xe || !a.L.width) return cudaErrorInvalidValue;
  if (k == 1) return launch_st<float, 1, true>(a, stage, s);
  if (k == 2) return launch_st<float, 2, true>(a, stage, s);
  return launch_st<float, 3, true>(a, stage, s);
}

}  // namespace hrw
