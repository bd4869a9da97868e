// hrw_internal.h - host-side declarations shared by the C-ABI and the kernel launchers.
#pragma once
#include <atomic>
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

// One dimension of the problem as the kernels see it.  T is the real type of the problem: double
// for HRW_F64 handles, float for HRW_F32 handles (the REAL32 build of the reference; those run
// the reference-order arithmetic only, so the FAST-only fields stay unset).
template <class T>
struct LineArgsT {
  int nc;
  int fn;        // HRW_FN_*
  int bc;        // HRW_BC_*
  int flux;      // HRW_FLUX_*
  T a, b;        // LINEAR: g(x) = a + b x
  T alpha;       // Lax-Friedrichs alpha
  T xmin, rx;
  // STRICT: divide by width (width[] or rx); FAST: multiply by rws (rws[] or rws0), which
  // already carries the flux scaling of the FAST flux form.
  const T* width;
  const T* rws;
  T rws0;
  const T* xe;  // non-uniform line: edges(0:nc) (x of interface e = xe[e]); null: uniform
};
using LineArgs = LineArgsT<double>;

template <class T>
struct StageArgsT {
  const T* v;    // stencil input
  const T* u;    // u^n for RK2B / RK3B / RK3C
  T* out;
  T* lout;       // ST_MS: L(v); ST_RECON: vr
  const T* uo4;  // ST_MS: u^{n-4}
  const T* lo4;  // ST_MS: L(u^{n-4})
  T eps, dt;
  LineArgsT<T> L;
  // 2D only
  LineArgsT<T> L2;
  int64_t ld;    // row stride (nc1) of the 2D layout
  int upwind;    // Godunov flux of g(x) u with g > 0 everywhere: F = g vm (2D kernel)
  const T* cnu;   // non-uniform line (1D, or x1 of 2D): weno coefficients cnu(0:k-1,-1:k-1,1:nc)
  const T* cnu2;  // 2D: the x2 line's coefficients when it is non-uniform
  // uniform 1D line (stage1d_kernel): update only cells cell0 .. cell0 + ncell - 1 (ncell = 0:
  // the whole line); cell0 and ncell are multiples of the launch's tile (1024 cells for lines
  // of at least 2 x SMs x 1024 cells), so that ranges launched side by side write disjoint cells
  int64_t cell0, ncell;
  // set by the launcher: grids of at most this many blocks are one wave (4 blocks per SM of the
  // current device) and release their programmatic dependents at once
  int wave_blocks;
  // 2D stages: the handle's word that a block sets when its bounded wait for its tile copies
  // runs out (zero-initialised device memory; checked and cleared by the host after the call),
  // and the poll limit of that wait (set by the launcher)
  unsigned int* timeout_flag;
  int tile_wait_polls;
};
using StageArgs = StageArgsT<double>;
using StageArgs32 = StageArgsT<float>;

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
  // non-uniform line (1D): per-cell weno coefficients cnu(0:k-1,-1:k-1) rounded from FP64,
  // the edges x_e, and per-cell g(x_{j+1}) - g(x_j) = b width_j (from FP64 widths); null: uniform
  const float* cnu;
  const float* xe;
  const float* gst;
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
  // 2D: Godunov's flux of linear fluxes g(x) u with g > 0 at every interface of both lines in
  // FP32: only the left state of each interface is reconstructed (stage2d_f32c.cu)
  int upwind;
};

// ---- MIXED numerics (hrw_mixed.cuh, stage1d_mixed.cu) --------------------------------------
enum MixedStage : int {
  MX_E1 = 0,    // dout = d1 = dt L(u)
  MX_RK1 = 1,   // uout = u + dt L(u)
  MX_RK2B = 2,  // uout = u + (d1 + dt L(u + d1)) / 2
  MX_RK3B = 3,  // dout = d2 = (d1 + dt L(u + d1)) / 4
  MX_RK3C = 4   // uout = u + 2/3 (d2 + dt L(u + d2))
};

struct MixedArgs {
  const double* u;       // u^n (FP64)
  const float2* dv;      // stage increment of the stencil input (u + dv), float pairs; or null
  float2* dout;          // increment output (MX_E1, MX_RK3B)
  double* uout;          // new state (MX_RK1, MX_RK2B, MX_RK3C); never u itself
  const unsigned* scale; // high word of max|u| over the line (launch_mixed_scale)
  double eps, dt;        // the FP64 path's scalars
  LineArgs L;            // the line as the FAST kernels see it
  // the FP32 path's scalars (mixed_fill)
  float epsf, inv_eps, alpha_f;
  float c_h, c_l;        // dt / (4 dx) as a pair: dt L = -c (4 dF)
  float g_h, g_l;        // linear flux: the velocity g = a as a pair
  float two3_h, two3_l;  // 2/3 as a pair
  // update only cells cell0 .. cell0 + ncell - 1 (ncell = 0: the whole line); cell0 a multiple of
  // the kernel's 1024-cell block tile (kMixedTile), so that ranges side by side write disjoint cells
  int64_t cell0, ncell;
};
constexpr int64_t kMixedTile = 1024;

// Whether the MIXED kernel covers a line: k = 2 or 3, Lax-Friedrichs, uniform grid, Burgers or
// linear advection at constant speed.  Other lines run the FAST kernels.
bool mixed_supported(const LineArgs& L, int k);
// The FP32 scalars of a from its line, eps and dt.
void mixed_fill(MixedArgs& a, double eps, double dt);
cudaError_t launch_stage1d_mixed(const MixedArgs& a, int k, int stage, cudaStream_t s);
// *word = high word of max |u_i| (reset first; asynchronous on s).
cudaError_t launch_mixed_scale(const double* u, int64_t n, unsigned* word, cudaStream_t s);
// Test hooks: every warp through the FP64 path (enable = 0), and the count of warps away from
// the line ends that took it (optionally reset).
cudaError_t mixed_set_soft(int enable);
cudaError_t mixed_hard_warps(unsigned long long* count, bool reset);

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
// True when the line's flux is g(x) u with g > 0 at every interface (upwind Godunov), with g
// at the line ends above rel_margin (|a| + |b x|).
bool positive_velocity(const LineArgs& L, double rel_margin = 1e-12);
// 0 turns the upwind specialisation of the 2D kernels off for handles created afterwards (a
// test hook, hrw_diag_upwind: the general flux path gives the same bits)
// The compensated FP32 kernels' copy of a non-uniform line (LineF's rw, xe, gst, cnu): 1/width,
// the edges and b width from the FP64 edges (host), and the FP64 weno coefficients (device,
// k (k + 1) per cell) rounded once; one block of nu_line_f32_floats(nc, k) floats at dst, the
// four arrays 256-byte aligned.
struct NuLineF32 {
  float *rw, *xe, *gst, *cnu;
};
size_t nu_line_f32_floats(int nc, int k);
cudaError_t build_nu_line_f32(const double* xedges, int nc, int k, double b, const double* cnu64,
                              float* dst, NuLineF32* out);

extern std::atomic<int> g_upwind_enabled;

// 1D fused stage over nc cells; k in 1..3; strict selects the reference-order numerics.
cudaError_t launch_stage1d(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s);
// 2D fused stage (x1 fastest), dimension by dimension.
cudaError_t launch_stage2d(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s);
// 1D fused stage on a non-uniform line (a.cnu, a.L.xe, a.L.width / a.L.rws set).
cudaError_t launch_stage1d_nu(const StageArgs& a, int k, int stage, bool strict, cudaStream_t s);
// Every step of an rktvd integrate call of a short uniform FV1D line (6 .. 4096 cells) in one
// launch of one thread-block cluster holding the line in shared memory (stage1d_cluster.cu);
// the same bits as the stage-by-stage launches.  cluster_line_ok: whether a line qualifies.
bool cluster_line_ok(const StageArgs& a);
cudaError_t launch_rk_cluster(const StageArgs& a, int k, int order, bool strict, double* u,
                              int64_t nsteps, cudaStream_t s);
// Linear ODE u' = a u stage (test problem of the reference's integrator tests).
cudaError_t launch_stage_linear(const double* rates, const StageArgs& a, int64_t n, int stage,
                                bool strict, cudaStream_t s);
// Non-uniform WENO: coefficients cnu(0:k-1,-1:k-1,1:nc) from xedges(0:nc), on the device.
cudaError_t launch_calc_cnu(const double* xedges, double* cnu, int nc, int k, cudaStream_t s);
// Reconstruction with per-cell coefficients (non-uniform grid).
cudaError_t launch_recon_nonuniform(const double* v, const double* cnu, double* vl, double* vr,
                                    int nc, int k, double eps, bool strict, cudaStream_t s);

// REAL32 (HRW_F32): the same kernels instantiated on float, always in the reference's operation
// order (what a REAL32 build of the reference computes, src/hrweno_kinds.F90:9-10).
cudaError_t launch_stage1d(const StageArgs32& a, int k, int stage, cudaStream_t s);
cudaError_t launch_stage2d(const StageArgs32& a, int k, int stage, cudaStream_t s);
cudaError_t launch_stage1d_nu(const StageArgs32& a, int k, int stage, cudaStream_t s);
cudaError_t launch_stage_linear(const float* rates, const StageArgs32& a, int64_t n, int stage,
                                cudaStream_t s);
cudaError_t launch_calc_cnu(const float* xedges, float* cnu, int nc, int k, cudaStream_t s);
cudaError_t launch_recon_nonuniform(const float* v, const float* cnu, float* vl, float* vr, int nc,
                                    int k, float eps, cudaStream_t s);

}  // namespace hrw
