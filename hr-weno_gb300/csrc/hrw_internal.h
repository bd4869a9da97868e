// hrw_internal.h - host-side declarations shared by the C-ABI and the kernel launchers.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace hrw {

// Kind of stage a launch performs: what it combines with L(v).
enum StageKind : int {
  ST_RHS = 0,    // out = L(v)
  ST_EULER = 1,  // out = v + dt L(v)                      (rktvd :139,150,163)
  ST_RK2B = 2,   // out = (u + v + dt L(v)) / 2            (rktvd :152)
  ST_RK3B = 3,   // out = (3u + v + dt L(v)) / 4           (rktvd :165)
  ST_RK3C = 4,   // out = (u + 2v + 2dt L(v)) / 3          (rktvd :167)
  ST_MS = 5,     // out = (25v + 50dt L(v) + 7uo4 + 10dt lo4)/32, lout = L(v)  (mstvd :257)
  ST_RECON = 6   // out = vl, lout = vr                    (weno%reconstruct)
};

// One dimension of the problem as the kernels see it.
struct LineArgs {
  int nc;
  int fn;        // HRW_FN_*
  int bc;        // HRW_BC_*
  int flux;      // HRW_FLUX_*
  double a, b;   // LINEAR: g(x) = a + b x
  double alpha;  // Lax-Friedrichs alpha
  double xmin, rx;
  // STRICT: divide by width (width[] or rx); FAST: multiply by rws (rws[] or rws0), which
  // already carries the flux scaling of the FAST flux form.
  const double* width;
  const double* rws;
  double rws0;
  const double* xe;  // non-uniform line: edges(0:nc) (x of interface e = xe[e]); null: uniform
};

struct StageArgs {
  const double* v;    // stencil input
  const double* u;    // u^n for RK2B / RK3B / RK3C
  double* out;
  double* lout;       // ST_MS: L(v); ST_RECON: vr
  const double* uo4;  // ST_MS: u^{n-4}
  const double* lo4;  // ST_MS: L(u^{n-4})
  double eps, dt;
  LineArgs L;
  // 2D only
  LineArgs L2;
  int64_t ld;         // row stride (nc1) of the 2D layout
  int upwind;         // Godunov flux of g(x) u with g > 0 everywhere: F = g vm (2D kernel)
  const double* cnu;  // non-uniform 1D line: weno coefficients cnu(0:k-1,-1:k-1,1:nc)
  // uniform 1D line (stage1d_kernel): update only cells cell0 .. cell0 + ncell - 1 (ncell = 0:
  // the whole line); cell0 and ncell are multiples of the launch's tile (1024 cells for lines
  // of at least 2 x SMs x 1024 cells), so that ranges launched side by side write disjoint cells
  int64_t cell0, ncell;
  // set by the launcher: grids of at most this many blocks are one wave (4 blocks per SM of the
  // current device) and release their programmatic dependents at once
  int wave_blocks;
  // 2D stages: the handle's word that a block sets when its bounded wait for its tile copies
  // runs out (zero-initialised device memory; checked and cleared by the host after the call)
  unsigned int* timeout_flag;
};

// ---- compensated FP32 form (hrw_f32c.cuh, stage1d_f32c.cu) ---------------------------------
enum F32CStage : int {
  FC_RHS = 0,   // out = L(u + dv)
  FC_E1 = 1,    // out = dt L(u)
  FC_RK1 = 2,   // u' = u + dt L(u)
  FC_RK2B = 3,  // u' = u + (d1 + dt L(u + d1)) / 2
  FC_RK3B = 4,  // out = (d1 + dt L(u + d1)) / 4
  FC_RK3C = 5,  // u' = u + 2/3 (d2 + dt L(u + d2))
  FC_MS = 6     // u' = u + (7 (u4 - u) + 50 dt L(u) + 10 dt L4) / 32, lout = L(u)
};

// One dimension of a compensated-FP32 problem as the kernels see it.
struct LineF {
  int nc;
  int fn, bc, flux;
  float a, b, alpha;  // g(x) = a + b x; LF alpha
  float xmin, rx;
  float gstep;        // g(x_{e+1}) - g(x_e) = b * rx
  const float* rw;    // per-cell 1 / width, or null (uniform grid)
};

struct F32CArgs {
  const float* hi;    // state u = hi + lo
  const float* lo;
  const float* dv;    // stored stage increment added to the stencil input, or null
  float* out;         // increment or L(u) output
  float* hi_out;      // new state (a buffer other than hi/lo)
  float* lo_out;
  const float* hi4;   // FC_MS: u^{n-4}
  const float* lo4;
  const float* l4;    // FC_MS: L(u^{n-4})
  float* lout;        // FC_MS: L(u^n)
  // scalars as float pairs so that no rounding of dt or dx biases every increment alike:
  //   q_j = -dF_j (uniform grid) or -dF_j / width_j;  L_j = q_j * lscale;
  //   dt L_j = (c_hi + c_lo) q_j;  dt x = (dt_hi + dt_lo) x
  float c_hi, c_lo;   // dt / dx (uniform) or dt (per-cell widths)
  float dt_hi, dt_lo;
  float lscale;       // 1 / dx (uniform) or 1
  float eps;
  LineF L;
  // 2D (x1 fastest, row stride ld): the x2 line and its dt/dx2 pair and 1/dx2
  LineF L2;
  float c2_hi, c2_lo;
  float lscale2;
  int64_t ld;
  unsigned int* timeout_flag;  // 2D stages: as StageArgs::timeout_flag
};

cudaError_t launch_stage1d_f32c(const F32CArgs& a, int k, int stage, cudaStream_t s);
cudaError_t launch_stage2d_f32c(const F32CArgs& a, int k, int stage, cudaStream_t s);
// Poll limit of the 2D stage kernels' first wait for their TMA tile copies (both the FP64 and
// the compensated kernels; the wait that drains the copies after a timeout keeps its own
// bound).  polls < 0 restores the default, 2^20.
cudaError_t stage2d_set_tile_wait_limit(int polls);
cudaError_t stage2d_f32c_set_tile_wait_limit(int polls);
cudaError_t launch_split_f64(const double* u, float* hi, float* lo, int64_t n, cudaStream_t s);
cudaError_t launch_merge_f64(const float* hi, const float* lo, double* u, int64_t n, cudaStream_t s);
cudaError_t launch_widen_f32(const float* x, double* y, int64_t n, cudaStream_t s);

// Multiprocessor count of the current device (cached per device; 152 on GB300).
int device_sms();

// FAST flux form: the kernels evaluate F / fscale, fscale folded into rws.
double fast_flux_scale(int flux, int fn);
// Record msg as the calling thread's last error (hrw_last_error) and return code.
int set_error(int code, const char* msg);
// True when the line's flux is g(x) u with g > 0 at every interface (upwind Godunov).
bool positive_velocity(const LineArgs& L);

// 1D fused stage over nc cells; k in 1..3; strict selects the reference-order numerics.
cudaError_t launch_stage1d(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s);
// 2D fused stage (x1 fastest), dimension by dimension.
cudaError_t launch_stage2d(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s);
// 1D fused stage on a non-uniform line (a.cnu, a.L.xe, a.L.width / a.L.rws set).
cudaError_t launch_stage1d_nu(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s);
// Linear ODE u' = a u stage (test problem of the reference's integrator tests).
cudaError_t launch_stage_linear(const double* rates, const StageArgs& a, int64_t n, int stage,
                                bool strict, cudaStream_t s);
// Non-uniform WENO: coefficients cnu(0:k-1,-1:k-1,1:nc) from xedges(0:nc), on the device.
cudaError_t launch_calc_cnu(const double* xedges, double* cnu, int nc, int k, cudaStream_t s);
// Reconstruction with per-cell coefficients (non-uniform grid).
cudaError_t launch_recon_nonuniform(const double* v, const double* cnu, double* vl, double* vr,
                                    int nc, int k, double eps, bool strict, cudaStream_t s);

}  // namespace hrw
