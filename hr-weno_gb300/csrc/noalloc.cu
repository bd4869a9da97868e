// noalloc.cu - rktvd order-3 steps of a 1D line that allocate no device memory
// (hrw_rktvd3_steps_noalloc in include/hrweno_gpu.h).
//
// The two RK stage arrays of an rktvd(order 3) handle normally come from cudaMalloc when the
// handle is created.  Here they live in one file-scope device array of fixed size, so a call
// performs no allocation at all: it validates the problem on the host, looks up the array's
// device address (on every call made outside stream capture, so that a device reset, which
// reloads the module, cannot leave a stale address behind; a captured call uses the address
// the last uncaptured call on that device found), and launches the same three fused stage
// kernels, in the same order, as hrw_integrate does for one RK3 step.
#include <cmath>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_internal.h"

namespace {

constexpr int64_t kMaxCells = HRW_NOALLOC_MAX_CELLS;
constexpr int kMaxDevices = 64;

// u1 at [0, kMaxCells), u2 at [kMaxCells, 2 kMaxCells).  Host code must not use this name as
// an address (it is a host-side stand-in); the device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) double g_stage_scratch[2 * kMaxCells];

std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

// Device address of g_stage_scratch on the current device.  Looked up again on every call
// whose stream is not capturing (cheap once the module is loaded); a capturing call reuses the
// address of the last uncaptured call on the device and fails if there was none.
int scratch_address(cudaStream_t s, double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return hrw::set_error(HRW_EINVAL, "device ordinal too large");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(s, &cs);
  if (e != cudaSuccess) return hrw::set_error(HRW_ECUDA, cudaGetErrorString(e));
  std::lock_guard<std::mutex> lock(g_mu);
  if (cs == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_stage_scratch);
    if (e != cudaSuccess || !p)
      return hrw::set_error(HRW_ECUDA, "hrw_rktvd3_steps_noalloc: cudaGetSymbolAddress failed");
    g_addr[dev] = static_cast<double*>(p);
  } else if (!g_addr[dev]) {
    return hrw::set_error(HRW_ECUDA,
                          "hrw_rktvd3_steps_noalloc: the first call on a device must not be captured");
  }
  *out = g_addr[dev];
  return HRW_OK;
}

}  // namespace

extern "C" int hrw_rktvd3_steps_noalloc(const hrw_problem* p, double* u, double dt, int nsteps,
                                        void* stream) {
  using namespace hrw;
  if (!p || !u) return set_error(HRW_EINVAL, "Invalid input: null pointer.");
  if (p->kind != HRW_PROBLEM_FV1D)
    return set_error(HRW_EINVAL, "hrw_rktvd3_steps_noalloc: only HRW_PROBLEM_FV1D problems.");
  if (p->width[0] || p->xedges[0])
    return set_error(HRW_EINVAL, "hrw_rktvd3_steps_noalloc: only uniform grids (width[0] = NULL).");
  const int64_t nc = p->ncells[0];
  if (nc <= 0) return set_error(HRW_EINVAL, "Invalid input 'ncells'. Valid range: ncells > 0.");
  if (nc > kMaxCells)
    return set_error(HRW_EINVAL,
                     "hrw_rktvd3_steps_noalloc: ncells exceeds HRW_NOALLOC_MAX_CELLS (1048576).");
  if (p->k < 1 || p->k > 3) return set_error(HRW_EINVAL, "Invalid input 'k'. Valid range: 1 <= k <= 3.");
  if (!(p->eps > 2.220446049250313e-16))
    return set_error(HRW_EINVAL, "Invalid input 'eps'. Valid range: eps > epsilon.");
  if (p->flux != HRW_FLUX_LAX_FRIEDRICHS && p->flux != HRW_FLUX_GODUNOV)
    return set_error(HRW_EINVAL, "Invalid input 'flux'.");
  if (p->fn[0] < HRW_FN_BURGERS || p->fn[0] > HRW_FN_BURGERS_LINEAR)
    return set_error(HRW_EINVAL, "Invalid input 'fn'.");
  if (p->bc[0] < HRW_BC_COPY || p->bc[0] > HRW_BC_ZERO_INFLOW)
    return set_error(HRW_EINVAL, "Invalid input 'bc'.");
  if (p->numerics != HRW_NUMERICS_FAST && p->numerics != HRW_NUMERICS_STRICT)
    return set_error(HRW_EINVAL, "Invalid input 'numerics'.");
  if (!(p->xmax[0] > p->xmin[0]))
    return set_error(HRW_EINVAL, "Invalid input 'xmin', 'xmax'. Valid range: xmax > xmin.");
  if (nsteps < 0) return set_error(HRW_EINVAL, "Invalid input 'nsteps': must be >= 0.");
  if (!(dt != 0.0) || !std::isfinite(dt))
    return set_error(HRW_EINVAL, "Invalid input 'dt': must be finite and nonzero.");

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // an error left by earlier, unrelated work is not this call's: clear it before launching
  cudaGetLastError();
  double* scratch = nullptr;
  int rc = scratch_address(s, &scratch);
  if (rc != HRW_OK) return rc;
  double* u1 = scratch;
  double* u2 = scratch + kMaxCells;

  // the line as ode_create sets it up for a uniform grid
  StageArgs b{};
  b.eps = p->eps;
  b.dt = dt;
  LineArgs& L = b.L;
  L.nc = (int)nc;
  L.fn = p->fn[0];
  L.bc = p->bc[0];
  L.flux = p->flux;
  L.a = p->coef_a[0];
  L.b = p->coef_b[0];
  L.alpha = p->alpha[0];
  L.xmin = p->xmin[0];
  L.rx = (p->xmax[0] - p->xmin[0]) / L.nc;
  L.rws0 = fast_flux_scale(p->flux, p->fn[0]) / L.rx;
  b.ld = nc;
  const bool strict = p->numerics == HRW_NUMERICS_STRICT;

  for (int n = 0; n < nsteps; ++n) {  // rktvd order 3 (src/hrweno_tvdode.f90:161-169)
    StageArgs a = b;
    a.v = u, a.u = u, a.out = u1;
    cudaError_t e = launch_stage1d(a, p->k, ST_EULER, strict, s);
    a = b;
    a.v = u1, a.u = u, a.out = u2;
    if (e == cudaSuccess) e = launch_stage1d(a, p->k, ST_RK3B, strict, s);
    a = b;
    a.v = u2, a.u = u, a.out = u;
    if (e == cudaSuccess) e = launch_stage1d(a, p->k, ST_RK3C, strict, s);
    if (e != cudaSuccess) return set_error(HRW_ECUDA, cudaGetErrorString(e));
  }
  return HRW_OK;
}
