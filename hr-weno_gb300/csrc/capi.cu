// capi.cu - the C ABI (include/hrweno_gpu.h): handles, validation with the reference's
// messages, and the host time loops that reproduce the reference's step sequence exactly.
//
//   weno_init            src/hrweno_weno.f90:54-127
//   rktvd_init/integrate src/hrweno_tvdode.f90:69-178
//   mstvd_init/integrate src/hrweno_tvdode.f90:180-271
//   is_done              src/hrweno_tvdode.f90:273-284
//
// The time t stays on the host in the handle's real type (FP64, or FP32 for the REAL32 handles
// of HRW_F32) and is advanced by the same `t = t + dt` sequence as the reference, so the step
// count of every integrate call is known before the first launch; the kernels themselves do not
// depend on t (every flux of the problem descriptor is autonomous).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_internal.h"

using namespace hrw;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define HRW_CUDA(call)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,               \
                  std::string(#call ": ") + cudaGetErrorString(e_));                      \
  } while (0)

// is_done (src/hrweno_tvdode.f90:282), in the handle's real type
template <class R>
inline bool is_done(R t, R tout, R dt) {
  return (t - tout) * std::copysign(R(1), dt) > R(0);
}

// epsilon(1.0_rk) of the eps check (src/hrweno_weno.f90:92) for rk = real64 and real32
constexpr double kEps64 = 2.220446049250313e-16;
constexpr float kEps32 = 1.1920928955078125e-07f;

constexpr int64_t kMaxSteps = int64_t(1) << 40;
// MIXED numerics take the MIXED kernel on lines of at least this many cells (shorter lines are
// launch-bound, and the FAST kernel's shared-memory tile serves them better)
constexpr int kMixedMinCells = 1 << 16;

struct DevLine {
  double* width = nullptr;  // device copy of the user's widths (STRICT)
  double* rws = nullptr;    // device fscale/width (FAST)
  double* xe = nullptr;     // non-uniform line: edges(0:nc)
  double* cnu = nullptr;    // non-uniform line: weno coefficients
};

// Validate the problem descriptor against the same rules the reference's constructors apply,
// plus the descriptor's own fields.
int validate_problem(const hrw_problem* p, int neq) {
  if (!p) return fail(HRW_EINVAL, "Invalid input 'problem': null pointer.");
  if (neq <= 0) return fail(HRW_EINVAL, "Invalid input 'neq'. Valid range: neq >= 1.");
  if (p->kind == HRW_PROBLEM_LINEAR_ODE) {
    if (!p->rates) return fail(HRW_EINVAL, "Invalid input 'rates': null pointer.");
    return HRW_OK;
  }
  if (p->kind != HRW_PROBLEM_FV1D && p->kind != HRW_PROBLEM_FV2D)
    return fail(HRW_EINVAL, "Invalid input 'kind'.");
  const int nd = p->kind == HRW_PROBLEM_FV2D ? 2 : 1;
  int64_t cells = 1;
  for (int d = 0; d < nd; ++d) {
    if (p->ncells[d] <= 0) return fail(HRW_EINVAL, "Invalid input 'ncells'. Valid range: ncells > 0.");
    if (!(p->xmax[d] > p->xmin[d]))
      return fail(HRW_EINVAL, "Invalid input 'xmin', 'xmax'. Valid range: xmax > xmin.");
    if (p->fn[d] < HRW_FN_BURGERS || p->fn[d] > HRW_FN_BURGERS_LINEAR)
      return fail(HRW_EINVAL, "Invalid input 'fn'.");
    if (p->bc[d] < HRW_BC_COPY || p->bc[d] > HRW_BC_ZERO_INFLOW)
      return fail(HRW_EINVAL, "Invalid input 'bc'.");
    if (p->xedges[d]) {
      if (p->width[d]) return fail(HRW_EINVAL, "Invalid input: give either 'xedges' or 'width'.");
      for (int i = 0; i < p->ncells[d]; ++i)
        if (!(p->xedges[d][i + 1] > p->xedges[d][i]))
          return fail(HRW_EINVAL, "Invalid input 'xedges': edges must increase.");
    }
    cells *= p->ncells[d];
  }
  if (p->k < 1 || p->k > 3) return fail(HRW_EINVAL, "Invalid input 'k'. Valid range: 1 <= k <= 3.");
  if (!(p->eps > kEps64))
    return fail(HRW_EINVAL, "Invalid input 'eps'. Valid range: eps > epsilon.");
  if (p->flux != HRW_FLUX_LAX_FRIEDRICHS && p->flux != HRW_FLUX_GODUNOV)
    return fail(HRW_EINVAL, "Invalid input 'flux'.");
  if (p->numerics != HRW_NUMERICS_FAST && p->numerics != HRW_NUMERICS_STRICT &&
      p->numerics != HRW_NUMERICS_MIXED)
    return fail(HRW_EINVAL, "Invalid input 'numerics'.");
  if (p->numerics == HRW_NUMERICS_MIXED && !(p->eps >= 1e-8))
    return fail(HRW_EINVAL, "Invalid input 'eps': HRW_NUMERICS_MIXED needs eps >= 1e-8.");
  if (cells != neq) return fail(HRW_EINVAL, "Invalid input 'neq': neq /= product of ncells.");
  return HRW_OK;
}

// The checks of a REAL32 build on top of validate_problem: its epsilon is FP32's, and the
// grid's values must stay valid once rounded to FP32 (the values that build would hold).
int validate_problem_f32(const hrw_problem* p) {
  if (!((float)p->eps > kEps32)) return fail(HRW_EINVAL, "Invalid input 'eps'. Valid range: eps > epsilon.");
  if (p->kind == HRW_PROBLEM_LINEAR_ODE) return HRW_OK;
  for (int d = 0; d < (p->kind == HRW_PROBLEM_FV2D ? 2 : 1); ++d) {
    if (!((float)p->xmax[d] > (float)p->xmin[d]))
      return fail(HRW_EINVAL, "Invalid input 'xmin', 'xmax': xmax > xmin must hold in REAL32.");
    if (p->xedges[d])
      for (int i = 0; i < p->ncells[d]; ++i)
        if (!((float)p->xedges[d][i + 1] > (float)p->xedges[d][i]))
          return fail(HRW_EINVAL, "Invalid input 'xedges': edges must increase in REAL32.");
    if (p->width[d])
      for (int i = 0; i < p->ncells[d]; ++i)
        if (!((float)p->width[d][i] > 0.0f))
          return fail(HRW_EINVAL, "Invalid input 'width': widths must be > 0 in REAL32.");
  }
  return HRW_OK;
}

// The number of steps n of an integrate call from t and the time it ends at (*tend), by the
// reference's sequence t = t + dt (src/hrweno_tvdode.f90:137-143,170-171) in real type R: one
// step for itask = 2, else until is_done.  A step that leaves t unchanged would never reach
// tout and is refused.
template <class R>
int count_steps(R t, R tout, R dt, int itask, int64_t* n, R* tend) {
  int64_t k = 0;
  do {
    const R t1 = t + dt;
    if (t1 == t) return fail(HRW_EINVAL, "Invalid input 'dt': t + dt == t, so tout is never reached.");
    t = t1;
    if (++k > kMaxSteps) return fail(HRW_EINVAL, "Invalid input 'dt': too many steps to reach tout.");
  } while (!(is_done(t, tout, dt) || itask == 2));
  *n = k;
  *tend = t;
  return HRW_OK;
}

// The number of mstvd steps from t (src/hrweno_tvdode.f90:252-268: is_done is tested before
// each step, so n may be 0), with the same refusal of steps that leave t unchanged.
template <class R>
int count_ms_steps(R t, R tout, R dt, int64_t* n) {
  int64_t k = 0;
  while (!is_done(t, tout, dt)) {
    const R t1 = t + dt;
    if (t1 == t) return fail(HRW_EINVAL, "Invalid input 'dt': t + dt == t, so tout is never reached.");
    t = t1;
    if (++k > kMaxSteps) return fail(HRW_EINVAL, "Invalid input 'dt': too many steps to reach tout.");
  }
  *n = k;
  return HRW_OK;
}

}  // namespace

namespace hrw {
// Record msg as this host thread's last error (read by hrw_last_error) and return code.
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace hrw

// -------------------------------------------------------------------------------------------
// Handles
// -------------------------------------------------------------------------------------------
struct hrw_weno {
  int nc = 0, k = 3;
  double eps = 1e-6;
  int numerics = HRW_NUMERICS_FAST;
  bool uniform = true;
  double* cnu = nullptr;  // device cnu(0:k-1,-1:k-1,1:nc)
  double* buf = nullptr;  // device v, vl, vr for host-memory calls (3 nc)
  cudaStream_t stream = nullptr;
  // REAL32 calls on a non-uniform grid: the edges, and cnu computed from them in FP32 at the
  // first such call
  std::vector<double> xedges;
  float* cnu32 = nullptr;
};

struct hrw_ode {
  hrw_problem prob{};
  int neq = 0, order = 3, method = 0, dtype = HRW_F64;
  int fevals = 0, istate = 0;
  int64_t nsteps = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  DevLine line[2];
  double* rates = nullptr;
  double* u = nullptr;   // device state for host-memory calls (rktvd)
  double* w1 = nullptr;  // stage buffers
  double* w2 = nullptr;
  double* ring_u[5] = {};  // mstvd: u^m at slot m % 5
  double* ring_l[4] = {};  // mstvd: L(u^m) at slot m % 4
  int64_t level = 0;       // mstvd: m of the current solution
  StageArgs base{};
  // compensated FP32 form (HRW_F32C): state slots as float pairs; rktvd ping-pongs between
  // slots 0 and 1, mstvd keeps u^m in slot m % 5 and L(u^m) in fl[m % 4]
  float* fmem = nullptr;
  float* fhi[5] = {};
  float* flo[5] = {};
  float* fl[4] = {};
  float* fd1 = nullptr;  // stage increments
  float* fd2 = nullptr;
  float* frw = nullptr;  // per-cell 1/width
  int fslot = 0;
  F32CArgs fbase{};
  // CUDA graphs of kGraphSteps consecutive steps, replayed for long integrate calls
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    const void* ptr = nullptr;
    double dt = 0.0;
    cudaStream_t stream = nullptr;
    int64_t phase = -1;
    int64_t steps = 0;
  } graph;
  bool use_graphs = true;
  // short uniform 1D lines: all steps of an integrate call in one cluster launch
  bool use_cluster = true;
  // host lines with the copies overlapped (rk3_integrate_host): two compute streams and a copy
  // stream beside `stream`, and their events
  cudaStream_t pipe[2] = {}, copy = nullptr;
  cudaEvent_t ev_start = nullptr, ev_in[16] = {}, ev_s3[16] = {}, ev_join[3] = {};
  // MIXED host lines: a third compute stream, a stream for the copies back, the events of the
  // first and second stages' chunks, and whether mscale[2] holds the exponent of the last
  // output (the guess of the next call)
  cudaStream_t pipe3 = nullptr, copy_out = nullptr;
  cudaEvent_t ev_s1[16] = {}, ev_s2[16] = {}, ev_end[2] = {};
  bool mguess = false;
  // 2D problems: the word a stage block sets when its bounded wait for its tile copies ran out
  unsigned int* tflag = nullptr;
  // MIXED numerics on a line the MIXED kernel covers: its arguments and the words holding the
  // high word of max|u|: [0] the one the stages use (max|u| at the start of each integrate
  // call), [1] and [2] those of a host line's input and output (rk3_integrate_host_mixed)
  bool mixed = false;
  MixedArgs mbase{};
  unsigned int* mscale = nullptr;
  // REAL32 (HRW_F32): the problem in FP32 as a REAL32 build holds it, the state and stage
  // buffers in FP32 (rktvd: su, sw1, sw2; mstvd also the rings), every allocation in sallocs
  StageArgs32 sbase{};
  float* su = nullptr;
  float* sw1 = nullptr;
  float* sw2 = nullptr;
  float* sring_u[5] = {};
  float* sring_l[4] = {};
  float* srates = nullptr;
  std::vector<void*> sallocs;
};

// weno%reconstruct of a REAL32 build: float arrays, FP32 eps, FP32 tables or FP32 cnu, in the
// reference's operation order.
static int weno_reconstruct_f32(hrw_weno* w, int mem, const void* v, void* vl, void* vr) {
  if (!((float)w->eps > kEps32)) return fail(HRW_EINVAL, "Invalid input 'eps'. Valid range: eps > epsilon.");
  if (!w->uniform && !w->cnu32) {
    const int nc = w->nc;
    std::vector<float> xe(nc + 1);
    for (int i = 0; i <= nc; ++i) xe[i] = (float)w->xedges[i];
    for (int i = 0; i < nc; ++i)
      if (!(xe[i + 1] > xe[i])) return fail(HRW_EINVAL, "Invalid input 'xedges': edges must increase in REAL32.");
    float* dx = nullptr;
    float* cnu = nullptr;
    cudaError_t e = cudaMalloc(&cnu, sizeof(float) * (size_t)w->k * (w->k + 1) * nc);
    if (e == cudaSuccess) e = cudaMalloc(&dx, sizeof(float) * ((size_t)nc + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, xe.data(), sizeof(float) * ((size_t)nc + 1), cudaMemcpyHostToDevice, w->stream);
    if (e == cudaSuccess) e = launch_calc_cnu(dx, cnu, nc, w->k, w->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
    if (dx) cudaFree(dx);
    if (e != cudaSuccess) {
      if (cnu) cudaFree(cnu);
      return fail(e == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,
                  std::string("hrw_weno_reconstruct: ") + cudaGetErrorString(e));
    }
    w->cnu32 = cnu;
  }
  const size_t bytes = sizeof(float) * (size_t)w->nc;
  const float* dv = (const float*)v;
  float* dl = (float*)vl;
  float* dr = (float*)vr;
  if (mem == HRW_MEM_HOST) {  // the 3 nc doubles of buf hold 3 nc floats
    float* b = (float*)w->buf;
    dv = b;
    dl = b + w->nc;
    dr = b + 2 * (size_t)w->nc;
    HRW_CUDA(cudaMemcpyAsync((void*)dv, v, bytes, cudaMemcpyHostToDevice, w->stream));
  }
  if (w->uniform) {
    StageArgs32 a{};
    a.v = dv;
    a.out = dl;
    a.lout = dr;
    a.eps = (float)w->eps;
    a.L.nc = w->nc;
    a.L.rx = 1.0f;
    HRW_CUDA(launch_stage1d(a, w->k, ST_RECON, w->stream));
  } else {
    HRW_CUDA(launch_recon_nonuniform(dv, w->cnu32, dl, dr, w->nc, w->k, (float)w->eps, w->stream));
  }
  if (mem == HRW_MEM_HOST) {
    HRW_CUDA(cudaMemcpyAsync(vl, dl, bytes, cudaMemcpyDeviceToHost, w->stream));
    HRW_CUDA(cudaMemcpyAsync(vr, dr, bytes, cudaMemcpyDeviceToHost, w->stream));
  }
  HRW_CUDA(cudaStreamSynchronize(w->stream));
  return HRW_OK;
}

// The REAL32 problem on the device: lines, widths, edges and cnu in FP32 as a REAL32 build
// computes them (grid1%linear: dx = (xmax - xmin)/nc in FP32, src/hrweno_grids.f90:72; widths
// edges(i) - edges(i-1); cnu by weno_calc_cnu in FP32), and the state and stage buffers.
static cudaError_t setup_f32(hrw_ode* o, const hrw_problem* p) {
  auto alloc = [&](size_t n, float** out) {
    const cudaError_t e = cudaMalloc(out, sizeof(float) * (n ? n : 1));
    if (e == cudaSuccess) o->sallocs.push_back(*out);
    return e;
  };
  auto upload = [&](const std::vector<float>& h, float** out) {
    cudaError_t e = alloc(h.size(), out);
    if (e == cudaSuccess) e = cudaMemcpy(*out, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice);
    return e;
  };
  cudaError_t e;
  StageArgs32& b = o->sbase;
  b.eps = (float)p->eps;
  const size_t n = (size_t)o->neq;
  if (p->kind == HRW_PROBLEM_LINEAR_ODE) {
    std::vector<float> r(n);
    for (size_t i = 0; i < n; ++i) r[i] = (float)p->rates[i];
    if ((e = upload(r, &o->srates)) != cudaSuccess) return e;
  } else {
    const int nd = p->kind == HRW_PROBLEM_FV2D ? 2 : 1;
    for (int d = 0; d < nd; ++d) {
      LineArgsT<float>& L = d == 0 ? b.L : b.L2;
      L.nc = p->ncells[d];
      L.fn = p->fn[d];
      L.bc = p->bc[d];
      L.flux = p->flux;
      L.a = (float)p->coef_a[d];
      L.b = (float)p->coef_b[d];
      L.alpha = (float)p->alpha[d];
      L.xmin = (float)p->xmin[d];
      const float span = (float)p->xmax[d] - (float)p->xmin[d];
      L.rx = span / (float)L.nc;
      if (p->width[d]) {
        std::vector<float> w(L.nc);
        for (int i = 0; i < L.nc; ++i) w[i] = (float)p->width[d][i];
        float* dw = nullptr;
        if ((e = upload(w, &dw)) != cudaSuccess) return e;
        L.width = dw;
      }
      if (p->xedges[d]) {
        std::vector<float> xe(L.nc + 1), w(L.nc);
        for (int i = 0; i <= L.nc; ++i) xe[i] = (float)p->xedges[d][i];
        for (int i = 0; i < L.nc; ++i) w[i] = xe[i + 1] - xe[i];
        float *dxe = nullptr, *dw = nullptr, *cnu = nullptr;
        if ((e = upload(xe, &dxe)) != cudaSuccess) return e;
        if ((e = upload(w, &dw)) != cudaSuccess) return e;
        if ((e = alloc((size_t)p->k * (p->k + 1) * L.nc, &cnu)) != cudaSuccess) return e;
        if ((e = launch_calc_cnu(dxe, cnu, L.nc, p->k, o->own)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(o->own)) != cudaSuccess) return e;
        L.xe = dxe;
        L.width = dw;
        (d == 0 ? b.cnu : b.cnu2) = cnu;
      }
    }
    b.ld = p->ncells[0];
    if (nd == 2) {
      // upwind when g > 0 at every interface in FP32: the FP32 evaluation of g at the line ends
      // differs from the FP64 one by a few FP32 rounding errors, far inside a 1e-5 margin
      LineArgs g1{}, g2{};
      for (int d = 0; d < 2; ++d) {
        const LineArgsT<float>& F = d == 0 ? b.L : b.L2;
        LineArgs& G = d == 0 ? g1 : g2;
        G.nc = F.nc, G.fn = F.fn, G.a = F.a, G.b = F.b, G.xmin = F.xmin, G.rx = F.rx;
      }
      b.upwind = p->flux == HRW_FLUX_GODUNOV && positive_velocity(g1, 1e-5) && positive_velocity(g2, 1e-5);
      if ((e = cudaMalloc(&o->tflag, sizeof(unsigned int))) != cudaSuccess) return e;
      if ((e = cudaMemset(o->tflag, 0, sizeof(unsigned int))) != cudaSuccess) return e;
      b.timeout_flag = o->tflag;
    }
  }
  if ((e = alloc(n, &o->su)) != cudaSuccess) return e;
  if ((e = alloc(n, &o->sw1)) != cudaSuccess) return e;
  if ((e = alloc(n, &o->sw2)) != cudaSuccess) return e;
  if (o->method == 1) {
    for (float*& q : o->sring_u)
      if ((e = alloc(n, &q)) != cudaSuccess) return e;
    for (float*& q : o->sring_l)
      if ((e = alloc(n, &q)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

extern "C" {

const char* hrw_last_error(void) { return g_err.c_str(); }

void hrw_problem_init(hrw_problem* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->kind = HRW_PROBLEM_FV1D;
  p->k = 3;
  p->eps = 1e-6;
  p->flux = HRW_FLUX_LAX_FRIEDRICHS;
  p->fn[0] = p->fn[1] = HRW_FN_BURGERS;
  p->coef_a[0] = p->coef_a[1] = 1.0;
  p->alpha[0] = p->alpha[1] = 1.0;
  p->bc[0] = p->bc[1] = HRW_BC_COPY;
  p->xmin[0] = p->xmin[1] = 0.0;
  p->xmax[0] = p->xmax[1] = 1.0;
  p->numerics = HRW_NUMERICS_FAST;
}

// ---- weno ------------------------------------------------------------------------------------
int hrw_weno_create(int ncells, int k, double eps, const double* xedges, hrw_weno** out) {
  if (!out) return fail(HRW_EINVAL, "Invalid input 'out': null pointer.");
  *out = nullptr;
  // weno_init validation (src/hrweno_weno.f90:72-98); k <= 0 / eps <= 0 mean "not present"
  if (ncells <= 0) return fail(HRW_EINVAL, "Invalid input 'ncells'. Valid range: ncells > 0.");
  if (k > 0 && k > 3) return fail(HRW_EINVAL, "Invalid input 'k'. Valid range: 1 <= k <= 3.");
  if (k == 0 || k < 0) k = 3;
  if (eps <= 0.0 && eps == eps) eps = 1e-6;
  if (!(eps > kEps64))
    return fail(HRW_EINVAL, "Invalid input 'eps'. Valid range: eps > epsilon.");
  hrw_weno* w = new hrw_weno;
  w->nc = ncells;
  w->k = k;
  w->eps = eps;
  cudaError_t e = cudaStreamCreateWithFlags(&w->stream, cudaStreamDefault);
  if (e == cudaSuccess) e = cudaMalloc(&w->buf, sizeof(double) * 3 * (size_t)ncells);
  if (e == cudaSuccess && xedges) {
    w->uniform = false;
    w->xedges.assign(xedges, xedges + (size_t)ncells + 1);
    double* dx = nullptr;
    e = cudaMalloc(&w->cnu, sizeof(double) * (size_t)k * (k + 1) * ncells);
    if (e == cudaSuccess) e = cudaMalloc(&dx, sizeof(double) * ((size_t)ncells + 1));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dx, xedges, sizeof(double) * ((size_t)ncells + 1), cudaMemcpyHostToDevice, w->stream);
    if (e == cudaSuccess) e = launch_calc_cnu(dx, w->cnu, ncells, k, w->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
    if (dx) cudaFree(dx);
  }
  if (e != cudaSuccess) {
    hrw_weno_destroy(w);
    return fail(e == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,
                std::string("hrw_weno_create: ") + cudaGetErrorString(e));
  }
  *out = w;
  return HRW_OK;
}

int hrw_weno_set_numerics(hrw_weno* w, int numerics) {
  if (!w) return fail(HRW_EINVAL, "Invalid input 'w': null handle.");
  if (numerics != HRW_NUMERICS_FAST && numerics != HRW_NUMERICS_STRICT)
    return fail(HRW_EINVAL, "Invalid input 'numerics'.");
  w->numerics = numerics;
  return HRW_OK;
}

int hrw_weno_reconstruct(hrw_weno* w, int dtype, int mem, const void* v, void* vl, void* vr) {
  if (!w) return fail(HRW_EINVAL, "Invalid input 'w': null handle.");
  if (!v || !vl || !vr) return fail(HRW_EINVAL, "Invalid input: null array.");
  if (dtype != HRW_F64 && dtype != HRW_F32)
    return fail(HRW_EINVAL, "Invalid input 'dtype': reconstruct supports HRW_F64 and HRW_F32.");
  if (mem != HRW_MEM_HOST && mem != HRW_MEM_DEVICE) return fail(HRW_EINVAL, "Invalid input 'mem'.");
  if (dtype == HRW_F32) return weno_reconstruct_f32(w, mem, v, vl, vr);
  const size_t bytes = sizeof(double) * (size_t)w->nc;
  const double* dv = (const double*)v;
  double* dl = (double*)vl;
  double* dr = (double*)vr;
  if (mem == HRW_MEM_HOST) {
    dv = w->buf;
    dl = w->buf + w->nc;
    dr = w->buf + 2 * (size_t)w->nc;
    HRW_CUDA(cudaMemcpyAsync((void*)dv, v, bytes, cudaMemcpyHostToDevice, w->stream));
  }
  const bool strict = w->numerics == HRW_NUMERICS_STRICT;
  if (w->uniform) {
    StageArgs a{};
    a.v = dv;
    a.out = dl;
    a.lout = dr;
    a.eps = w->eps;
    a.L.nc = w->nc;
    a.L.rx = 1.0;
    HRW_CUDA(launch_stage1d(a, w->k, ST_RECON, strict, w->stream));
  } else {
    HRW_CUDA(launch_recon_nonuniform(dv, w->cnu, dl, dr, w->nc, w->k, w->eps, strict, w->stream));
  }
  if (mem == HRW_MEM_HOST) {
    HRW_CUDA(cudaMemcpyAsync(vl, dl, bytes, cudaMemcpyDeviceToHost, w->stream));
    HRW_CUDA(cudaMemcpyAsync(vr, dr, bytes, cudaMemcpyDeviceToHost, w->stream));
  }
  HRW_CUDA(cudaStreamSynchronize(w->stream));
  return HRW_OK;
}

int hrw_weno_cnu(const hrw_weno* w, double* cnu_host) {
  if (!w || !cnu_host) return fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (w->uniform) return fail(HRW_EINVAL, "hrw_weno_cnu: the grid is uniform (no xedges).");
  HRW_CUDA(cudaMemcpy(cnu_host, w->cnu, sizeof(double) * (size_t)w->k * (w->k + 1) * w->nc,
                      cudaMemcpyDeviceToHost));
  return HRW_OK;
}

int hrw_weno_destroy(hrw_weno* w) {
  if (!w) return HRW_OK;
  if (w->cnu) cudaFree(w->cnu);
  if (w->cnu32) cudaFree(w->cnu32);
  if (w->buf) cudaFree(w->buf);
  if (w->stream) cudaStreamDestroy(w->stream);
  delete w;
  return HRW_OK;
}

// ---- ode -------------------------------------------------------------------------------------
static int ode_create(const hrw_problem* p, int neq, int order, int method, int dtype, hrw_ode** out) {
  if (!out) return fail(HRW_EINVAL, "Invalid input 'out': null pointer.");
  *out = nullptr;
  // rktvd_init / mstvd_init validation (src/hrweno_tvdode.f90:80-90,190-194)
  if (neq <= 0) return fail(HRW_EINVAL, "Invalid input 'neq'. Valid range: neq >= 1.");
  if (method == 0 && (order < 1 || order > 3))
    return fail(HRW_EINVAL, "Invalid input 'order' in 'rktvd'. Valid range: 1 <= k <= 3.");
  if (dtype != HRW_F64 && dtype != HRW_F32C && dtype != HRW_F32) return fail(HRW_EINVAL, "Invalid input 'dtype'.");
  int rc = validate_problem(p, neq);
  if (rc != HRW_OK) return rc;
  if (dtype == HRW_F32 && (rc = validate_problem_f32(p)) != HRW_OK) return rc;
  if (dtype == HRW_F32C) {
    if (p->kind != HRW_PROBLEM_FV1D && p->kind != HRW_PROBLEM_FV2D)
      return fail(HRW_EINVAL, "Invalid input 'dtype': HRW_F32C supports FV1D and FV2D problems.");
    if (!(p->eps > 1.1920928955078125e-07))  // epsilon(1.0_real32), src/hrweno_weno.f90:92
      return fail(HRW_EINVAL, "Invalid input 'eps'. Valid range: eps > epsilon.");
    for (int d = 0; d < (p->kind == HRW_PROBLEM_FV2D ? 2 : 1); ++d)
      if (p->fn[d] == HRW_FN_BURGERS_LINEAR)  // its difference-form algebra is not written
        return fail(HRW_EINVAL, "Invalid input 'fn': HRW_F32C supports BURGERS and LINEAR.");
  }
  hrw_ode* o = new hrw_ode;
  o->prob = *p;
  o->neq = neq;
  o->order = method == 1 ? 3 : order;
  o->method = method;
  o->dtype = dtype;
  o->prob.width[0] = o->prob.width[1] = nullptr;  // host pointers are not kept
  o->prob.xedges[0] = o->prob.xedges[1] = nullptr;
  o->prob.rates = nullptr;
  auto cleanup = [&](cudaError_t e) {
    hrw_ode_destroy(o);
    return fail(e == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,
                std::string("hrw_ode_create: ") + cudaGetErrorString(e));
  };
  cudaError_t e = cudaStreamCreateWithFlags(&o->own, cudaStreamDefault);
  if (e != cudaSuccess) return cleanup(e);
  o->stream = o->own;
  if (dtype == HRW_F32) {
    if ((e = setup_f32(o, p)) != cudaSuccess) return cleanup(e);
    o->istate = 1;
    *out = o;
    return HRW_OK;
  }
  const size_t bytes = sizeof(double) * (size_t)neq;
  StageArgs& b = o->base;
  b.eps = p->eps;
  const bool strict = p->numerics == HRW_NUMERICS_STRICT;
  if (p->kind == HRW_PROBLEM_LINEAR_ODE) {
    if ((e = cudaMalloc(&o->rates, bytes)) != cudaSuccess) return cleanup(e);
    if ((e = cudaMemcpy(o->rates, p->rates, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) return cleanup(e);
  } else {
    const int nd = p->kind == HRW_PROBLEM_FV2D ? 2 : 1;
    for (int d = 0; d < nd; ++d) {
      LineArgs& L = d == 0 ? b.L : b.L2;
      L.nc = p->ncells[d];
      L.fn = p->fn[d];
      L.bc = p->bc[d];
      L.flux = p->flux;
      L.a = p->coef_a[d];
      L.b = p->coef_b[d];
      L.alpha = p->alpha[d];
      L.xmin = p->xmin[d];
      L.rx = (p->xmax[d] - p->xmin[d]) / L.nc;  // grid1%linear (src/hrweno_grids.f90:72)
      const double fs = fast_flux_scale(p->flux, p->fn[d]);
      L.rws0 = fs / L.rx;
      if (p->width[d]) {
        const size_t wb = sizeof(double) * (size_t)L.nc;
        std::vector<double> rws(L.nc);
        for (int i = 0; i < L.nc; ++i) {
          if (!(p->width[d][i] > 0.0)) {
            hrw_ode_destroy(o);
            return fail(HRW_EINVAL, "Invalid input 'width': widths must be > 0.");
          }
          rws[i] = fs / p->width[d][i];
        }
        if ((e = cudaMalloc(&o->line[d].width, wb)) != cudaSuccess) return cleanup(e);
        if ((e = cudaMalloc(&o->line[d].rws, wb)) != cudaSuccess) return cleanup(e);
        if ((e = cudaMemcpy(o->line[d].width, p->width[d], wb, cudaMemcpyHostToDevice)) != cudaSuccess)
          return cleanup(e);
        if ((e = cudaMemcpy(o->line[d].rws, rws.data(), wb, cudaMemcpyHostToDevice)) != cudaSuccess)
          return cleanup(e);
        L.width = o->line[d].width;
        L.rws = strict ? nullptr : o->line[d].rws;
        if (strict) L.rws = nullptr;
      }
      if (p->xedges[d]) {  // weno(ncells, k, eps, xedges): cnu on the device, widths, edges
        const size_t nb = sizeof(double) * (size_t)L.nc;
        std::vector<double> w(L.nc), rws(L.nc);
        for (int i = 0; i < L.nc; ++i) {
          w[i] = p->xedges[d][i + 1] - p->xedges[d][i];
          rws[i] = fs / w[i];
        }
        DevLine& D = o->line[d];
        if ((e = cudaMalloc(&D.width, nb)) != cudaSuccess) return cleanup(e);
        if ((e = cudaMalloc(&D.rws, nb)) != cudaSuccess) return cleanup(e);
        if ((e = cudaMalloc(&D.xe, nb + sizeof(double))) != cudaSuccess) return cleanup(e);
        if ((e = cudaMalloc(&D.cnu, nb * (size_t)p->k * (p->k + 1))) != cudaSuccess) return cleanup(e);
        if ((e = cudaMemcpy(D.width, w.data(), nb, cudaMemcpyHostToDevice)) != cudaSuccess) return cleanup(e);
        if ((e = cudaMemcpy(D.rws, rws.data(), nb, cudaMemcpyHostToDevice)) != cudaSuccess) return cleanup(e);
        if ((e = cudaMemcpy(D.xe, p->xedges[d], nb + sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
          return cleanup(e);
        if ((e = launch_calc_cnu(D.xe, D.cnu, L.nc, p->k, o->own)) != cudaSuccess) return cleanup(e);
        if ((e = cudaStreamSynchronize(o->own)) != cudaSuccess) return cleanup(e);
        L.width = D.width;
        L.rws = D.rws;
        L.xe = D.xe;
        (d == 0 ? b.cnu : b.cnu2) = D.cnu;
      }
    }
    b.ld = p->ncells[0];
    b.upwind = nd == 2 && p->flux == HRW_FLUX_GODUNOV && positive_velocity(b.L) &&
               positive_velocity(b.L2);
    if (nd == 2) {
      if ((e = cudaMalloc(&o->tflag, sizeof(unsigned int))) != cudaSuccess) return cleanup(e);
      if ((e = cudaMemset(o->tflag, 0, sizeof(unsigned int))) != cudaSuccess) return cleanup(e);
      b.timeout_flag = o->tflag;
    }
  }
  if ((e = cudaMalloc(&o->u, bytes)) != cudaSuccess) return cleanup(e);
  if (dtype == HRW_F32C) {
    // float buffers: rktvd 2 slots (hi, lo) + 2 increments; mstvd 5 slots + 4 L + 2 increments
    // each array starts on a 256-byte boundary: the stage kernel reads and writes float4
    const int slots = method == 1 ? 5 : 2;
    const size_t n = (size_t)neq, sn = (n + 63) / 64 * 64;
    const int nd = p->kind == HRW_PROBLEM_FV2D ? 2 : 1;
    size_t nw = 0;  // per-cell 1/width entries of the lines that have widths
    for (int d = 0; d < nd; ++d)
      if (p->width[d]) nw += (size_t)(p->ncells[d] + 63) / 64 * 64;
    // a non-uniform line: 1/width, the edges, b width and k (k + 1) coefficients per cell
    for (int d = 0; d < nd; ++d)
      if (p->xedges[d]) nw += nu_line_f32_floats(p->ncells[d], p->k);
    const size_t nf = sn * (2 * slots + (method == 1 ? 4 : 0) + 2) + nw;
    if ((e = cudaMalloc(&o->fmem, sizeof(float) * nf)) != cudaSuccess) return cleanup(e);
    float* q = o->fmem;
    for (int k = 0; k < slots; ++k) { o->fhi[k] = q; q += sn; o->flo[k] = q; q += sn; }
    if (method == 1)
      for (int k = 0; k < 4; ++k) { o->fl[k] = q; q += sn; }
    o->fd1 = q; q += sn;
    o->fd2 = q; q += sn;
    F32CArgs& f = o->fbase;
    f.eps = (float)p->eps;
    f.ld = p->ncells[0];
    f.timeout_flag = o->tflag;
    for (int d = 0; d < nd; ++d) {
      const LineArgs& L = d == 0 ? b.L : b.L2;
      LineF& F = d == 0 ? f.L : f.L2;
      F.nc = L.nc;
      F.fn = L.fn;
      F.bc = L.bc;
      F.flux = L.flux;
      F.a = (float)L.a;
      F.b = (float)L.b;
      F.alpha = (float)L.alpha;
      F.xmin = (float)L.xmin;
      F.rx = (float)L.rx;
      F.gstep = (float)(L.b * L.rx);
      if (p->width[d]) {
        std::vector<float> rw(L.nc);
        for (int i = 0; i < L.nc; ++i) rw[i] = (float)(1.0 / p->width[d][i]);
        if ((e = cudaMemcpy(q, rw.data(), sizeof(float) * L.nc, cudaMemcpyHostToDevice)) != cudaSuccess)
          return cleanup(e);
        F.rw = q;
        if (d == 0) o->frw = q;
        q += (size_t)(L.nc + 63) / 64 * 64;
      } else if (p->xedges[d]) {
        // the FP64 coefficients of the line (computed above on the device) and its FP64 widths,
        // rounded once to FP32; g at the edges from the rounded edges
        NuLineF32 nl{};
        if ((e = build_nu_line_f32(p->xedges[d], L.nc, p->k, L.b, o->line[d].cnu, q, &nl)) != cudaSuccess)
          return cleanup(e);
        F.rw = nl.rw;
        F.xe = nl.xe;
        F.gst = nl.gst;
        F.cnu = nl.cnu;
        if (d == 0) o->frw = nl.rw;
        q += nu_line_f32_floats(L.nc, p->k);
      }
    }
    if (nd == 2 && p->flux == HRW_FLUX_GODUNOV && !p->xedges[0] && !p->xedges[1]) {
      // upwind when g > 0 at every interface in FP32: the kernels evaluate g(x_e) from the float
      // a, b, rx, xmin, which differs from this FP64 evaluation of the same floats by a few FP32
      // roundings, far inside a 1e-5 margin (non-uniform grids take the general flux path)
      bool up = true;
      for (int d = 0; d < 2; ++d) {
        const LineF& F = d == 0 ? f.L : f.L2;
        LineArgs G{};
        G.nc = F.nc, G.fn = F.fn, G.a = F.a, G.b = F.b, G.xmin = F.xmin, G.rx = F.rx;
        up = up && positive_velocity(G, 1e-5);
      }
      f.upwind = up;
    }
    o->istate = 1;
    *out = o;
    return HRW_OK;
  }
  if ((e = cudaMalloc(&o->w1, bytes)) != cudaSuccess) return cleanup(e);
  if ((e = cudaMalloc(&o->w2, bytes)) != cudaSuccess) return cleanup(e);
  // MIXED numerics: lines of at least kMixedMinCells cells that the MIXED kernel covers take it
  // (shorter lines, and everything else, run the FAST kernels)
  if (p->numerics == HRW_NUMERICS_MIXED && p->kind == HRW_PROBLEM_FV1D && method == 0 &&
      !p->xedges[0] && !p->width[0] && neq >= kMixedMinCells && mixed_supported(b.L, p->k)) {
    if ((e = cudaMalloc(&o->mscale, 3 * sizeof(unsigned int))) != cudaSuccess) return cleanup(e);
    o->mixed = true;
    o->mbase.L = b.L;
    o->mbase.eps = p->eps;
  }
  if (method == 1) {
    for (int q = 0; q < 5; ++q)
      if ((e = cudaMalloc(&o->ring_u[q], bytes)) != cudaSuccess) return cleanup(e);
    for (int q = 0; q < 4; ++q)
      if ((e = cudaMalloc(&o->ring_l[q], bytes)) != cudaSuccess) return cleanup(e);
  }
  o->istate = 1;
  *out = o;
  return HRW_OK;
}

int hrw_rktvd_create(const hrw_problem* p, int neq, int order, int dtype, hrw_ode** out) {
  return ode_create(p, neq, order, 0, dtype, out);
}

int hrw_mstvd_create(const hrw_problem* p, int neq, int dtype, hrw_ode** out) {
  return ode_create(p, neq, 3, 1, dtype, out);
}

int hrw_ode_set_stream(hrw_ode* o, void* stream) {
  if (!o) return fail(HRW_EINVAL, "Invalid input 'ode': null handle.");
  o->stream = stream ? (cudaStream_t)stream : o->own;
  return HRW_OK;
}

int hrw_ode_set_graphs(hrw_ode* o, int enable) {
  if (!o) return fail(HRW_EINVAL, "Invalid input 'ode': null handle.");
  o->use_graphs = enable != 0;
  return HRW_OK;
}

int hrw_ode_set_cluster(hrw_ode* o, int enable) {
  if (!o) return fail(HRW_EINVAL, "Invalid input 'ode': null handle.");
  o->use_cluster = enable != 0;
  return HRW_OK;
}

int hrw_ode_info(const hrw_ode* o, int* fevals, int* istate, int64_t* nsteps) {
  if (!o) return fail(HRW_EINVAL, "Invalid input 'ode': null handle.");
  if (fevals) *fevals = o->fevals;
  if (istate) *istate = o->istate;
  if (nsteps) *nsteps = o->nsteps;
  return HRW_OK;
}

int hrw_ode_destroy(hrw_ode* o) {
  if (!o) return HRW_OK;
  for (int d = 0; d < 2; ++d) {
    if (o->line[d].width) cudaFree(o->line[d].width);
    if (o->line[d].rws) cudaFree(o->line[d].rws);
    if (o->line[d].xe) cudaFree(o->line[d].xe);
    if (o->line[d].cnu) cudaFree(o->line[d].cnu);
  }
  double* bufs[] = {o->rates, o->u, o->w1, o->w2};
  for (double* p : bufs)
    if (p) cudaFree(p);
  for (double* p : o->ring_u)
    if (p) cudaFree(p);
  for (double* p : o->ring_l)
    if (p) cudaFree(p);
  if (o->fmem) cudaFree(o->fmem);
  for (void* q : o->sallocs) cudaFree(q);
  if (o->tflag) cudaFree(o->tflag);
  if (o->mscale) cudaFree(o->mscale);
  if (o->graph.exec) cudaGraphExecDestroy(o->graph.exec);
  for (cudaStream_t st : {o->pipe[0], o->pipe[1], o->copy, o->pipe3, o->copy_out})
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t ev : o->ev_in)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : o->ev_s3)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : o->ev_s1)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : o->ev_s2)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : o->ev_end)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : o->ev_join)
    if (ev) cudaEventDestroy(ev);
  if (o->ev_start) cudaEventDestroy(o->ev_start);
  if (o->own) cudaStreamDestroy(o->own);
  delete o;
  return HRW_OK;
}

}  // extern "C"

// -------------------------------------------------------------------------------------------
// Stage dispatch and time loops
// -------------------------------------------------------------------------------------------
static cudaError_t run_stage(hrw_ode* o, int stage, const double* v, const double* u, double* out,
                             double* lout, const double* uo4, const double* lo4, double dt) {
  StageArgs a = o->base;
  a.v = v;
  a.u = u;
  a.out = out;
  a.lout = lout;
  a.uo4 = uo4;
  a.lo4 = lo4;
  a.dt = dt;
  const bool strict = o->prob.numerics == HRW_NUMERICS_STRICT;
  switch (o->prob.kind) {
    case HRW_PROBLEM_LINEAR_ODE: return launch_stage_linear(o->rates, a, o->neq, stage, strict, o->stream);
    case HRW_PROBLEM_FV1D:
      if (a.cnu) return launch_stage1d_nu(a, o->prob.k, stage, strict, o->stream);
      return launch_stage1d(a, o->prob.k, stage, strict, o->stream);
    default: return launch_stage2d(a, o->prob.k, stage, strict, o->stream);
  }
}

// A stage of a uniform 1D line over cells cell0 .. cell0 + ncell - 1 on stream `st`.
static cudaError_t run_stage_range(hrw_ode* o, int stage, const double* v, const double* u, double* out,
                                   int64_t cell0, int64_t ncell, double dt, cudaStream_t st) {
  StageArgs a = o->base;
  a.v = v;
  a.u = u;
  a.out = out;
  a.dt = dt;
  a.cell0 = cell0;
  a.ncell = ncell;
  return launch_stage1d(a, o->prob.k, stage, o->prob.numerics == HRW_NUMERICS_STRICT, st);
}

// One rktvd step from u (in place for orders 2 and 3); order 1 writes into `out1`.
static cudaError_t rk_step(hrw_ode* o, double* u, double* out1, double dt) {
  cudaError_t e;
  if (o->order == 1) return run_stage(o, ST_EULER, u, u, out1, nullptr, nullptr, nullptr, dt);
  if ((e = run_stage(o, ST_EULER, u, u, o->w1, nullptr, nullptr, nullptr, dt)) != cudaSuccess) return e;
  if (o->order == 2) return run_stage(o, ST_RK2B, o->w1, u, u, nullptr, nullptr, nullptr, dt);
  if ((e = run_stage(o, ST_RK3B, o->w1, u, o->w2, nullptr, nullptr, nullptr, dt)) != cudaSuccess) return e;
  return run_stage(o, ST_RK3C, o->w2, u, u, nullptr, nullptr, nullptr, dt);
}

// One rktvd step of the MIXED kernel from `cur` into `other` (the state ping-pongs between
// them: a stage's stencil reads u, so the last stage cannot write u in place).  Order 3:
//   d1 -> other (float pairs), d2 -> w2 (float pairs), u' -> other (over d1).
static cudaError_t rk_step_mixed(hrw_ode* o, const double* cur, double* other, double dt) {
  MixedArgs a = o->mbase;
  mixed_fill(a, o->prob.eps, dt);
  a.u = cur;
  a.scale = o->mscale;
  const int k = o->prob.k;
  cudaError_t e;
  float2* d1 = reinterpret_cast<float2*>(o->order == 2 ? o->w2 : other);
  float2* d2 = reinterpret_cast<float2*>(o->w2);
  if (o->order == 1) {
    a.uout = other;
    return launch_stage1d_mixed(a, k, MX_RK1, o->stream);
  }
  a.dout = d1;
  if ((e = launch_stage1d_mixed(a, k, MX_E1, o->stream)) != cudaSuccess) return e;
  a.dout = nullptr;
  a.dv = d1;
  if (o->order == 2) {
    a.uout = other;
    return launch_stage1d_mixed(a, k, MX_RK2B, o->stream);
  }
  a.dout = d2;
  if ((e = launch_stage1d_mixed(a, k, MX_RK3B, o->stream)) != cudaSuccess) return e;
  a.dout = nullptr;
  a.dv = d2;
  a.uout = other;
  return launch_stage1d_mixed(a, k, MX_RK3C, o->stream);
}

// Captured graphs hold up to kGraphMax consecutive steps (rktvd; an even count for order 1,
// which ping-pongs between two arrays) or a multiple of kMsPeriod steps (mstvd rotates a
// 5-slot and a 4-slot ring, so its launch pattern repeats every 20 steps).  A driver loop that
// integrates the same number of steps per call (the reference's output-time loops) captures
// one graph and replays it on every later call.
constexpr int64_t kGraphMax = 64;
constexpr int64_t kMsPeriod = 20;

// Replay `reps` times a graph of `steps` steps recorded by `record` (which launches them on
// o->stream).  The graph is captured once and reused while the device array, dt, stream, ring
// phase and step count stay the same.  *replayed = false (nothing launched, cudaSuccess) when
// capture is not possible on this stream; the caller then launches the steps one by one.  A
// replay that fails returns its error: the replays before it have run, so the steps cannot be
// launched again from the start.
template <class Record>
static cudaError_t run_graph(hrw_ode* o, const void* ptr, double dt, int64_t phase, int64_t steps,
                             int64_t reps, bool* replayed, Record record) {
  *replayed = false;
  auto& g = o->graph;
  if (!g.exec || g.ptr != ptr || g.dt != dt || g.stream != o->stream || g.phase != phase ||
      g.steps != steps) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
    cudaStreamCaptureStatus st;
    if (cudaStreamIsCapturing(o->stream, &st) != cudaSuccess || st != cudaStreamCaptureStatusNone) {
      cudaGetLastError();
      return cudaSuccess;
    }
    if (cudaStreamBeginCapture(o->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return cudaSuccess;
    }
    const cudaError_t rec = record();
    cudaGraph_t graph = nullptr;
    const cudaError_t end = cudaStreamEndCapture(o->stream, &graph);
    if (rec != cudaSuccess || end != cudaSuccess || !graph ||
        cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      g.exec = nullptr;
      cudaGetLastError();
      return cudaSuccess;
    }
    cudaGraphDestroy(graph);
    g.ptr = ptr, g.dt = dt, g.stream = o->stream, g.phase = phase, g.steps = steps;
  }
  for (int64_t r = 0; r < reps; ++r) {
    const cudaError_t e = cudaGraphLaunch(g.exec, o->stream);
    if (e != cudaSuccess) return e;
  }
  *replayed = true;
  return cudaSuccess;
}

// steps per graph of an rktvd integration of n steps (0: no graph)
static int64_t rk_graph_steps(const hrw_ode* o, int64_t n) {
  if (!o->use_graphs || n < 4) return 0;
  int64_t G = n < kGraphMax ? n : kGraphMax;
  if (o->order == 1 || o->mixed) G &= ~int64_t(1);  // the state ping-pongs between two arrays
  return G;
}

// rktvd_integrate of the MIXED kernel: n steps from du (the state alternates between du and w1)
// n MIXED steps from du (after the scale), leaving the state in *where (du or w1)
static int mixed_steps(hrw_ode* o, double* du, int64_t n, double dt, double** where) {
  double* cur = du;
  double* other = o->w1;
  int64_t s0 = 0;
  if (const int64_t G = rk_graph_steps(o, n)) {
    bool ok = false;
    HRW_CUDA(run_graph(o, du, dt, 1, G, n / G, &ok, [&]() {
      double* c = du;
      double* w = o->w1;
      for (int64_t s = 0; s < G; ++s) {
        const cudaError_t e = rk_step_mixed(o, c, w, dt);
        if (e != cudaSuccess) return e;
        std::swap(c, w);
      }
      return cudaSuccess;
    }));
    if (ok) s0 = n / G * G;
  }
  for (int64_t s = s0; s < n; ++s) {
    HRW_CUDA(rk_step_mixed(o, cur, other, dt));
    std::swap(cur, other);
  }
  *where = cur;
  return HRW_OK;
}

static int rk_integrate_mixed(hrw_ode* o, double* du, int64_t n, double dt) {
  HRW_CUDA(launch_mixed_scale(du, o->neq, o->mscale, o->stream));
  double* cur = du;
  if (const int rc = mixed_steps(o, du, n, dt, &cur)) return rc;
  if (cur != du)
    HRW_CUDA(cudaMemcpyAsync(du, cur, sizeof(double) * (size_t)o->neq, cudaMemcpyDeviceToDevice, o->stream));
  return HRW_OK;
}

// rktvd_integrate (src/hrweno_tvdode.f90:97-178) on device array du.
static int rk_integrate(hrw_ode* o, double* du, double* t, double tout, double dt, int itask) {
  // replay the reference's time sequence (:137-143) to count the steps
  double tt;
  int64_t n;
  if (const int rc = count_steps(*t, tout, dt, itask, &n, &tt)) return rc;
  // the MIXED kernel moves 16-byte vectors: a device array that is not 16-byte aligned (a view
  // at an odd offset) runs the FAST kernels
  if (o->mixed && ((uintptr_t)du & 15) == 0) {
    const int rc = rk_integrate_mixed(o, du, n, dt);
    if (rc != HRW_OK) return rc;
    *t = tt;
    o->fevals += (int)(o->order * n);
    o->nsteps += n;
    if (o->istate == 1) o->istate = 2;
    return HRW_OK;
  }
  if (o->use_cluster && o->prob.kind == HRW_PROBLEM_FV1D && cluster_line_ok(o->base)) {
    StageArgs a = o->base;
    a.dt = dt;
    const cudaError_t e = launch_rk_cluster(a, o->prob.k, o->order, o->prob.numerics == HRW_NUMERICS_STRICT,
                                            du, n, o->stream);
    if (e == cudaSuccess) {
      *t = tt;
      o->fevals += (int)(o->order * n);
      o->nsteps += n;
      if (o->istate == 1) o->istate = 2;
      return HRW_OK;
    }
    // a device that cannot schedule the cluster: the stage-by-stage launches from now on
    if (e != cudaErrorInvalidClusterSize && e != cudaErrorNotSupported && e != cudaErrorLaunchOutOfResources)
      return fail(HRW_ECUDA, std::string("launch_rk_cluster: ") + cudaGetErrorString(e));
    cudaGetLastError();
    o->use_cluster = false;
  }
  double* cur = du;
  double* other = o->w2;
  int64_t s0 = 0;
  if (const int64_t G = rk_graph_steps(o, n)) {
    bool ok = false;
    HRW_CUDA(run_graph(o, du, dt, 0, G, n / G, &ok, [&]() {
      double* c = du;
      double* w = o->w2;
      for (int64_t s = 0; s < G; ++s) {
        const cudaError_t e = rk_step(o, c, w, dt);
        if (e != cudaSuccess) return e;
        if (o->order == 1) std::swap(c, w);
      }
      return cudaSuccess;
    }));
    if (ok) s0 = n / G * G;
  }
  for (int64_t s = s0; s < n; ++s) {
    HRW_CUDA(rk_step(o, cur, other, dt));
    if (o->order == 1) std::swap(cur, other);
  }
  if (cur != du)
    HRW_CUDA(cudaMemcpyAsync(du, cur, sizeof(double) * (size_t)o->neq, cudaMemcpyDeviceToDevice, o->stream));
  *t = tt;
  o->fevals += (int)(o->order * n);
  o->nsteps += n;
  if (o->istate == 1) o->istate = 2;  // (:176)
  return HRW_OK;
}

// mstvd_integrate (src/hrweno_tvdode.f90:203-271) on device array du.
static int ms_integrate(hrw_ode* o, double* du, double* t, double tout, double dt) {
  const size_t bytes = sizeof(double) * (size_t)o->neq;
  double tt = *t;
  if (o->istate == 1) {
    // RK3 start (:236-249): u^m -> slot m % 5, L(u^m) -> slot m % 4, m = 0..3
    o->level = 0;
    HRW_CUDA(cudaMemcpyAsync(o->ring_u[0], du, bytes, cudaMemcpyDeviceToDevice, o->stream));
    for (int m = 0; m < 4; ++m) {
      double* um = o->ring_u[m % 5];
      double* un = o->ring_u[(m + 1) % 5];
      HRW_CUDA(run_stage(o, ST_RHS, um, um, o->ring_l[m % 4], nullptr, nullptr, nullptr, dt));
      HRW_CUDA(run_stage(o, ST_EULER, um, um, o->w1, nullptr, nullptr, nullptr, dt));
      HRW_CUDA(run_stage(o, ST_RK3B, o->w1, um, o->w2, nullptr, nullptr, nullptr, dt));
      HRW_CUDA(run_stage(o, ST_RK3C, o->w2, um, un, nullptr, nullptr, nullptr, dt));
      tt = tt + dt;  // ode_start%integrate(u, t, t + 2*dt, dt, itask=2): one step
    }
    o->level = 4;
    o->fevals = 12;  // (:246) the start's RK3 evaluations; the 4 extra rhs calls are not counted
    o->nsteps += 4;
    o->istate = 2;
  } else {
    HRW_CUDA(cudaMemcpyAsync(o->ring_u[o->level % 5], du, bytes, cudaMemcpyDeviceToDevice, o->stream));
  }
  int64_t n;
  if (const int rc = count_ms_steps(tt, tout, dt, &n)) return rc;
  auto ms_step = [&](int64_t m) {  // (:252-268)
    double* um = o->ring_u[m % 5];
    double* un = o->ring_u[(m + 1) % 5];  // holds u^{m-4}, overwritten in place
    double* lm = o->ring_l[m % 4];        // holds L(u^{m-4}), overwritten in place
    return run_stage(o, ST_MS, um, um, un, lm, un, lm, dt);
  };
  int64_t s0 = 0;
  if (o->use_graphs && n >= kMsPeriod) {
    const int64_t m0 = o->level;
    const int64_t G = n < 3 * kMsPeriod ? kMsPeriod : 3 * kMsPeriod;
    bool ok = false;
    HRW_CUDA(run_graph(o, o->ring_u[0], dt, m0 % kMsPeriod, G, n / G, &ok, [&]() {
      for (int64_t s = 0; s < G; ++s) {
        const cudaError_t e = ms_step(m0 + s);
        if (e != cudaSuccess) return e;
      }
      return cudaSuccess;
    }));
    if (ok) {
      s0 = n / G * G;
      for (int64_t s = 0; s < s0; ++s) tt = tt + dt;
      o->level = m0 + s0;
    }
  }
  for (int64_t s = s0; s < n; ++s) {
    HRW_CUDA(ms_step(o->level));
    tt = tt + dt;
    o->level = o->level + 1;
  }
  HRW_CUDA(cudaMemcpyAsync(du, o->ring_u[o->level % 5], bytes, cudaMemcpyDeviceToDevice, o->stream));
  *t = tt;
  o->fevals += (int)n;
  o->nsteps += n;
  return HRW_OK;
}

// ---- compensated FP32 form ---------------------------------------------------------------------
namespace hrw {

size_t nu_line_f32_floats(int nc, int k) {
  return ((size_t)nc + 64) / 64 * 64 * (3 + (size_t)k * (k + 1));
}

cudaError_t build_nu_line_f32(const double* xedges, int nc, int k, double b, const double* cnu64,
                              float* dst, NuLineF32* out) {
  const size_t n = (size_t)nc, ncf = (size_t)k * (k + 1), seg = (n + 64) / 64 * 64;
  std::vector<double> c64(n * ncf);
  cudaError_t e = cudaMemcpy(c64.data(), cnu64, sizeof(double) * c64.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  std::vector<float> host(seg * (3 + ncf), 0.f);  // rw | xe | gst | cnu
  for (size_t j = 0; j < n; ++j) {
    const double w = xedges[j + 1] - xedges[j];
    host[j] = (float)(1.0 / w);
    host[2 * seg + j] = (float)(b * w);
  }
  for (size_t j = 0; j <= n; ++j) host[seg + j] = (float)xedges[j];
  for (size_t j = 0; j < c64.size(); ++j) host[3 * seg + j] = (float)c64[j];
  if ((e = cudaMemcpy(dst, host.data(), sizeof(float) * host.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
    return e;
  *out = NuLineF32{dst, dst + seg, dst + 2 * seg, dst + 3 * seg};
  return cudaSuccess;
}

}  // namespace hrw

static void split_pair(double x, float& hi, float& lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

static cudaError_t run_f32c(hrw_ode* o, int stage, int slot, const float* dv, float* out, int slot_out,
                            const float* hi4, const float* lo4, const float* l4, float* lout, double dt) {
  F32CArgs a = o->fbase;
  a.hi = o->fhi[slot];
  a.lo = o->flo[slot];
  a.dv = dv;
  a.out = out;
  a.hi_out = slot_out >= 0 ? o->fhi[slot_out] : nullptr;
  a.lo_out = slot_out >= 0 ? o->flo[slot_out] : nullptr;
  a.hi4 = hi4;
  a.lo4 = lo4;
  a.l4 = l4;
  a.lout = lout;
  const LineArgs& L = o->base.L;
  const bool widths = a.L.rw != nullptr;
  split_pair(widths ? dt : dt / L.rx, a.c_hi, a.c_lo);
  split_pair(dt, a.dt_hi, a.dt_lo);
  a.lscale = widths ? 1.0f : (float)(1.0 / L.rx);
  if (o->prob.kind == HRW_PROBLEM_FV2D) {
    const LineArgs& L2 = o->base.L2;
    const bool w2 = a.L2.rw != nullptr;
    split_pair(w2 ? dt : dt / L2.rx, a.c2_hi, a.c2_lo);
    a.lscale2 = w2 ? 1.0f : (float)(1.0 / L2.rx);
    return launch_stage2d_f32c(a, o->prob.k, stage, o->stream);
  }
  return launch_stage1d_f32c(a, o->prob.k, stage, o->stream);
}

// one rktvd step from slot `from` into slot `to`
static cudaError_t rk_step_f32c(hrw_ode* o, int from, int to, double dt) {
  cudaError_t e;
  if (o->order == 1) return run_f32c(o, FC_RK1, from, nullptr, nullptr, to, nullptr, nullptr, nullptr, nullptr, dt);
  if ((e = run_f32c(o, FC_E1, from, nullptr, o->fd1, -1, nullptr, nullptr, nullptr, nullptr, dt)) != cudaSuccess)
    return e;
  if (o->order == 2) return run_f32c(o, FC_RK2B, from, o->fd1, nullptr, to, nullptr, nullptr, nullptr, nullptr, dt);
  if ((e = run_f32c(o, FC_RK3B, from, o->fd1, o->fd2, -1, nullptr, nullptr, nullptr, nullptr, dt)) != cudaSuccess)
    return e;
  return run_f32c(o, FC_RK3C, from, o->fd2, nullptr, to, nullptr, nullptr, nullptr, nullptr, dt);
}

static int rk_integrate_f32c(hrw_ode* o, double* du, double* t, double tout, double dt, int itask) {
  double tt;
  int64_t n;
  if (const int rc = count_steps(*t, tout, dt, itask, &n, &tt)) return rc;
  int slot = 0;
  HRW_CUDA(launch_split_f64(du, o->fhi[0], o->flo[0], o->neq, o->stream));
  int64_t s0 = 0;
  int64_t G = rk_graph_steps(o, n);
  G &= ~int64_t(1);  // the compensated form always ping-pongs its (hi, lo) slots
  if (G) {
    bool ok = false;
    HRW_CUDA(run_graph(o, o->fhi[0], dt, 0, G, n / G, &ok, [&]() {
      for (int64_t s = 0; s < G; ++s) {
        const cudaError_t e = rk_step_f32c(o, (int)(s & 1), (int)(1 - (s & 1)), dt);
        if (e != cudaSuccess) return e;
      }
      return cudaSuccess;
    }));
    if (ok) s0 = n / G * G;
  }
  for (int64_t s = s0; s < n; ++s) {
    HRW_CUDA(rk_step_f32c(o, slot, 1 - slot, dt));
    slot = 1 - slot;
  }
  HRW_CUDA(launch_merge_f64(o->fhi[slot], o->flo[slot], du, o->neq, o->stream));
  *t = tt;
  o->fevals += (int)(o->order * n);
  o->nsteps += n;
  if (o->istate == 1) o->istate = 2;
  return HRW_OK;
}

static int ms_integrate_f32c(hrw_ode* o, double* du, double* t, double tout, double dt) {
  double tt = *t;
  if (o->istate == 1) {  // RK3 start (src/hrweno_tvdode.f90:236-249)
    o->level = 0;
    HRW_CUDA(launch_split_f64(du, o->fhi[0], o->flo[0], o->neq, o->stream));
    for (int m = 0; m < 4; ++m) {
      HRW_CUDA(run_f32c(o, FC_RHS, m % 5, nullptr, o->fl[m % 4], -1, nullptr, nullptr, nullptr, nullptr, dt));
      HRW_CUDA(rk_step_f32c(o, m % 5, (m + 1) % 5, dt));
      tt = tt + dt;
    }
    o->level = 4;
    o->fevals = 12;
    o->nsteps += 4;
    o->istate = 2;
  } else {
    HRW_CUDA(launch_split_f64(du, o->fhi[o->level % 5], o->flo[o->level % 5], o->neq, o->stream));
  }
  int64_t n;
  if (const int rc = count_ms_steps(tt, tout, dt, &n)) return rc;
  for (int64_t s = 0; s < n; ++s) {  // (:252-268)
    const int64_t m = o->level;
    const int cur = (int)(m % 5), nxt = (int)((m + 1) % 5);  // nxt holds u^{m-4}
    float* lm = o->fl[m % 4];                                 // holds L(u^{m-4})
    HRW_CUDA(run_f32c(o, FC_MS, cur, nullptr, nullptr, nxt, o->fhi[nxt], o->flo[nxt], lm, lm, dt));
    tt = tt + dt;
    o->level = m + 1;
  }
  HRW_CUDA(launch_merge_f64(o->fhi[o->level % 5], o->flo[o->level % 5], du, o->neq, o->stream));
  *t = tt;
  o->fevals += (int)n;
  o->nsteps += n;
  return HRW_OK;
}

// ---- REAL32 (HRW_F32) ---------------------------------------------------------------------------
// The time loops of a REAL32 build: t, tout and dt in FP32, the state and every stage in FP32
// in the reference's operation order.
static cudaError_t run_stage32(hrw_ode* o, int stage, const float* v, const float* u, float* out,
                               float* lout, const float* uo4, const float* lo4, float dt) {
  StageArgs32 a = o->sbase;
  a.v = v;
  a.u = u;
  a.out = out;
  a.lout = lout;
  a.uo4 = uo4;
  a.lo4 = lo4;
  a.dt = dt;
  const int k = o->prob.k;
  switch (o->prob.kind) {
    case HRW_PROBLEM_LINEAR_ODE: return launch_stage_linear(o->srates, a, o->neq, stage, o->stream);
    case HRW_PROBLEM_FV1D:
      return a.cnu ? launch_stage1d_nu(a, k, stage, o->stream) : launch_stage1d(a, k, stage, o->stream);
    default: return launch_stage2d(a, k, stage, o->stream);
  }
}

// one rktvd step (src/hrweno_tvdode.f90:136-171) from u, in place for orders 2 and 3
static cudaError_t rk_step32(hrw_ode* o, float* u, float* out1, float dt) {
  cudaError_t e;
  if (o->order == 1) return run_stage32(o, ST_EULER, u, u, out1, nullptr, nullptr, nullptr, dt);
  if ((e = run_stage32(o, ST_EULER, u, u, o->sw1, nullptr, nullptr, nullptr, dt)) != cudaSuccess) return e;
  if (o->order == 2) return run_stage32(o, ST_RK2B, o->sw1, u, u, nullptr, nullptr, nullptr, dt);
  if ((e = run_stage32(o, ST_RK3B, o->sw1, u, o->sw2, nullptr, nullptr, nullptr, dt)) != cudaSuccess) return e;
  return run_stage32(o, ST_RK3C, o->sw2, u, u, nullptr, nullptr, nullptr, dt);
}

static int rk_integrate32(hrw_ode* o, float* du, float* t, float tout, float dt, int itask) {
  float tt;
  int64_t n;
  if (const int rc = count_steps(*t, tout, dt, itask, &n, &tt)) return rc;
  float* cur = du;
  float* other = o->sw2;
  int64_t s0 = 0;
  if (const int64_t G = rk_graph_steps(o, n)) {
    bool ok = false;
    HRW_CUDA(run_graph(o, du, dt, 0, G, n / G, &ok, [&]() {
      float* c = du;
      float* w = o->sw2;
      for (int64_t s = 0; s < G; ++s) {
        const cudaError_t e = rk_step32(o, c, w, dt);
        if (e != cudaSuccess) return e;
        if (o->order == 1) std::swap(c, w);
      }
      return cudaSuccess;
    }));
    if (ok) s0 = n / G * G;
  }
  for (int64_t s = s0; s < n; ++s) {
    HRW_CUDA(rk_step32(o, cur, other, dt));
    if (o->order == 1) std::swap(cur, other);
  }
  if (cur != du)
    HRW_CUDA(cudaMemcpyAsync(du, cur, sizeof(float) * (size_t)o->neq, cudaMemcpyDeviceToDevice, o->stream));
  *t = tt;
  o->fevals += (int)(o->order * n);
  o->nsteps += n;
  if (o->istate == 1) o->istate = 2;  // (:176)
  return HRW_OK;
}

// mstvd_integrate (src/hrweno_tvdode.f90:203-271): u^m in sring_u[m % 5], L(u^m) in sring_l[m % 4]
static int ms_integrate32(hrw_ode* o, float* du, float* t, float tout, float dt) {
  const size_t bytes = sizeof(float) * (size_t)o->neq;
  float tt = *t;
  if (o->istate == 1) {  // RK3 start (:236-249)
    o->level = 0;
    HRW_CUDA(cudaMemcpyAsync(o->sring_u[0], du, bytes, cudaMemcpyDeviceToDevice, o->stream));
    for (int m = 0; m < 4; ++m) {
      float* um = o->sring_u[m % 5];
      float* un = o->sring_u[(m + 1) % 5];
      HRW_CUDA(run_stage32(o, ST_RHS, um, um, o->sring_l[m % 4], nullptr, nullptr, nullptr, dt));
      HRW_CUDA(run_stage32(o, ST_EULER, um, um, o->sw1, nullptr, nullptr, nullptr, dt));
      HRW_CUDA(run_stage32(o, ST_RK3B, o->sw1, um, o->sw2, nullptr, nullptr, nullptr, dt));
      HRW_CUDA(run_stage32(o, ST_RK3C, o->sw2, um, un, nullptr, nullptr, nullptr, dt));
      tt = tt + dt;  // ode_start%integrate(u, t, t + 2*dt, dt, itask=2): one step
    }
    o->level = 4;
    o->fevals = 12;  // (:246)
    o->nsteps += 4;
    o->istate = 2;
  } else {
    HRW_CUDA(cudaMemcpyAsync(o->sring_u[o->level % 5], du, bytes, cudaMemcpyDeviceToDevice, o->stream));
  }
  int64_t n;
  if (const int rc = count_ms_steps(tt, tout, dt, &n)) return rc;
  auto ms_step = [&](int64_t m) {  // (:252-268)
    float* um = o->sring_u[m % 5];
    float* un = o->sring_u[(m + 1) % 5];  // holds u^{m-4}, overwritten in place
    float* lm = o->sring_l[m % 4];        // holds L(u^{m-4}), overwritten in place
    return run_stage32(o, ST_MS, um, um, un, lm, un, lm, dt);
  };
  int64_t s0 = 0;
  if (o->use_graphs && n >= kMsPeriod) {
    const int64_t m0 = o->level;
    const int64_t G = n < 3 * kMsPeriod ? kMsPeriod : 3 * kMsPeriod;
    bool ok = false;
    HRW_CUDA(run_graph(o, o->sring_u[0], dt, m0 % kMsPeriod, G, n / G, &ok, [&]() {
      for (int64_t s = 0; s < G; ++s) {
        const cudaError_t e = ms_step(m0 + s);
        if (e != cudaSuccess) return e;
      }
      return cudaSuccess;
    }));
    if (ok) {
      s0 = n / G * G;
      for (int64_t s = 0; s < s0; ++s) tt = tt + dt;
      o->level = m0 + s0;
    }
  }
  for (int64_t s = s0; s < n; ++s) {
    HRW_CUDA(ms_step(o->level));
    tt = tt + dt;
    o->level = o->level + 1;
  }
  HRW_CUDA(cudaMemcpyAsync(du, o->sring_u[o->level % 5], bytes, cudaMemcpyDeviceToDevice, o->stream));
  *t = tt;
  o->fevals += (int)n;
  o->nsteps += n;
  return HRW_OK;
}

// rktvd(3) of a uniform FP64 line on a page-locked host array, with the copies overlapped:
// the line is copied in by 16 chunks of whole 1024-cell tiles (measured: 4 and 8 chunks leave
// more of the first and last copies exposed), and stage 1 of the first step runs
// on each chunk as soon as it and its right neighbour (the halo) have landed; stage 3 of the
// last step runs by chunks, each chunk's copy back following it.  Chunks alternate between two
// streams, so the tail of one overlaps the next.  The arithmetic is that of rk_integrate.
constexpr int kPipeChunks = 16;
constexpr int64_t kPipeTile = 1024;
static_assert(kPipeChunks <= (int)(sizeof(hrw_ode::ev_in) / sizeof(cudaEvent_t)), "one event per chunk");

static bool host_pipeline_ok(const hrw_ode* o, const void* u) {
  if (o->mixed || o->dtype != HRW_F64 || o->prob.kind != HRW_PROBLEM_FV1D || o->method != 0 || o->order != 3 ||
      o->line[0].xe || (int64_t)o->neq < 2 * (int64_t)device_sms() * kPipeTile)
    return false;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, u) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;  // page-locked: asynchronous copies
}

static int rk3_integrate_host(hrw_ode* o, double* uh, double* t, double tout, double dt, int itask) {
  double tt;
  int64_t n;
  if (const int rc = count_steps(*t, tout, dt, itask, &n, &tt)) return rc;
  if (!o->copy) {
    for (cudaStream_t* st : {&o->pipe[0], &o->pipe[1], &o->copy})
      HRW_CUDA(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
    HRW_CUDA(cudaEventCreateWithFlags(&o->ev_start, cudaEventDisableTiming));
    for (int i = 0; i < kPipeChunks; ++i) {
      HRW_CUDA(cudaEventCreateWithFlags(&o->ev_in[i], cudaEventDisableTiming));
      HRW_CUDA(cudaEventCreateWithFlags(&o->ev_s3[i], cudaEventDisableTiming));
    }
    for (cudaEvent_t& ev : o->ev_join) HRW_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  const int64_t nc = o->neq;
  const int64_t chunk = ((nc + kPipeChunks - 1) / kPipeChunks + kPipeTile - 1) / kPipeTile * kPipeTile;
  const int nch = (int)((nc + chunk - 1) / chunk);
  double* du = o->u;
  cudaStream_t ms = o->stream;
  // every side stream starts after the work already queued on the handle's stream
  HRW_CUDA(cudaEventRecord(o->ev_start, ms));
  for (cudaStream_t st : {o->pipe[0], o->pipe[1], o->copy}) HRW_CUDA(cudaStreamWaitEvent(st, o->ev_start, 0));
  for (int i = 0; i < nch; ++i) {
    const int64_t off = i * chunk, len = std::min(chunk, nc - off);
    HRW_CUDA(cudaMemcpyAsync(du + off, uh + off, sizeof(double) * (size_t)len, cudaMemcpyHostToDevice, o->copy));
    HRW_CUDA(cudaEventRecord(o->ev_in[i], o->copy));
  }
  // stage 1 of the first step, per chunk: its cells and the right neighbour's halo have arrived
  for (int i = 0; i < nch; ++i) {
    const int64_t off = i * chunk, len = std::min(chunk, nc - off);
    cudaStream_t st = o->pipe[i & 1];
    HRW_CUDA(cudaStreamWaitEvent(st, o->ev_in[std::min(i + 1, nch - 1)], 0));
    HRW_CUDA(run_stage_range(o, ST_EULER, du, du, o->w1, off, len, dt, st));
  }
  for (int p = 0; p < 2; ++p) {
    HRW_CUDA(cudaEventRecord(o->ev_join[p], o->pipe[p]));
    HRW_CUDA(cudaStreamWaitEvent(ms, o->ev_join[p], 0));
  }
  for (int64_t s = 0; s < n; ++s) {
    if (s > 0) HRW_CUDA(run_stage(o, ST_EULER, du, du, o->w1, nullptr, nullptr, nullptr, dt));
    HRW_CUDA(run_stage(o, ST_RK3B, o->w1, du, o->w2, nullptr, nullptr, nullptr, dt));
    if (s < n - 1) HRW_CUDA(run_stage(o, ST_RK3C, o->w2, du, du, nullptr, nullptr, nullptr, dt));
  }
  // stage 3 of the last step, per chunk, each chunk copied back behind it
  HRW_CUDA(cudaEventRecord(o->ev_join[2], ms));
  for (int p = 0; p < 2; ++p) HRW_CUDA(cudaStreamWaitEvent(o->pipe[p], o->ev_join[2], 0));
  for (int i = 0; i < nch; ++i) {
    const int64_t off = i * chunk, len = std::min(chunk, nc - off);
    cudaStream_t st = o->pipe[i & 1];
    HRW_CUDA(run_stage_range(o, ST_RK3C, o->w2, du, du, off, len, dt, st));
    HRW_CUDA(cudaEventRecord(o->ev_s3[i], st));
    HRW_CUDA(cudaStreamWaitEvent(o->copy, o->ev_s3[i], 0));
    HRW_CUDA(cudaMemcpyAsync(uh + off, du + off, sizeof(double) * (size_t)len, cudaMemcpyDeviceToHost, o->copy));
  }
  HRW_CUDA(cudaEventRecord(o->ev_join[0], o->copy));
  HRW_CUDA(cudaStreamWaitEvent(ms, o->ev_join[0], 0));  // later work on the handle's stream
  *t = tt;
  o->fevals += (int)(3 * n);
  o->nsteps += n;
  if (o->istate == 1) o->istate = 2;
  return HRW_OK;
}

// MIXED rktvd(3) of a uniform line on a page-locked host array, with the copies overlapped.
//
// Every stage of a call takes its error budget from the line's largest |u| at the start of the
// call (its exponent, mscale[0]), a reduction over the whole input.  A call of one step whose
// handle knows the exponent of its previous output (mscale[2]) guesses that the input is that
// output, as in a driver loop, and pipelines the whole step by 16 chunks of whole 1024-cell
// tiles: chunk i is copied in, its first stage runs once chunk i + 1 (its halo) has landed,
// its second stage once the first has passed chunk i + 1, its third stage once the second has,
// and it is copied back behind its third stage, so that the copies in and back overlap each
// other and the stages.  The input's true exponent (mscale[1]) is reduced beside; if it differs
// from the guess the step is taken again from the device copy of the input (which no stage
// overwrites) with the true exponent, and the host line is written again.  Either way the
// results are those of rk_integrate_mixed, bit for bit.
//
// Without a guess (the first call, or several steps) the line comes in whole, the steps before
// the last run as on a device array, and the last step's second and third stages run by
// chunks, each chunk copied back behind its third stage.  The third stage writes u' over the
// first stage's increment, which the second stage has finished reading in chunk i once it has
// passed chunk i + 1.
static bool host_pipeline_mixed_ok(const hrw_ode* o, const void* u) {
  if (!o->mixed || o->order != 3 || (int64_t)o->neq < 2 * (int64_t)device_sms() * kMixedTile) return false;
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, u) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

static cudaError_t mixed_pipe_init(hrw_ode* o) {
  if (o->copy_out) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  for (cudaStream_t* st : {&o->pipe[0], &o->pipe[1], &o->copy, &o->pipe3, &o->copy_out})
    if (!*st && e == cudaSuccess) e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
  auto ev = [&](cudaEvent_t& x) {
    if (!x && e == cudaSuccess) e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
  };
  ev(o->ev_start);
  for (int i = 0; i < kPipeChunks; ++i) {
    ev(o->ev_in[i]);
    ev(o->ev_s1[i]);
    ev(o->ev_s2[i]);
    ev(o->ev_s3[i]);
  }
  for (cudaEvent_t& x : o->ev_join) ev(x);
  for (cudaEvent_t& x : o->ev_end) ev(x);
  return e;
}

// The last step of a MIXED host call from `cur` (state of level n-1 on the device), u^n into
// `other`: the first stage whole on the handle's stream (or, with `chunked_in`, chunk by chunk
// behind the copy in of uh), the second and third stages chunk by chunk, each chunk copied back
// to uh.  mscale[2] receives the exponent of the output.  Every stream joins the handle's
// stream at the end.
static int mixed_last_step(hrw_ode* o, double* uh, const double* cur, double* other, double dt,
                           bool chunked_in) {
  const int64_t nc = o->neq;
  cudaStream_t ms = o->stream;
  MixedArgs a = o->mbase;
  mixed_fill(a, o->prob.eps, dt);
  a.u = cur;
  a.scale = o->mscale;
  const int k = o->prob.k;
  float2* d1 = reinterpret_cast<float2*>(other);
  float2* d2 = reinterpret_cast<float2*>(o->w2);
  const int64_t chunk = ((nc + kPipeChunks - 1) / kPipeChunks + kMixedTile - 1) / kMixedTile * kMixedTile;
  const int nch = (int)((nc + chunk - 1) / chunk);
  auto range = [&](MixedArgs b, int i) {
    b.cell0 = i * chunk;
    b.ncell = std::min(chunk, nc - b.cell0);
    return b;
  };
  if (!chunked_in) {
    MixedArgs b = a;
    b.dout = d1;
    HRW_CUDA(launch_stage1d_mixed(b, k, MX_E1, ms));
  }
  HRW_CUDA(cudaEventRecord(o->ev_start, ms));
  for (cudaStream_t st : {o->pipe[0], o->pipe[1], o->pipe3, o->copy, o->copy_out})
    HRW_CUDA(cudaStreamWaitEvent(st, o->ev_start, 0));
  // issued in waves, so that chunk i's copy back is queued early: wave w issues the copy in of
  // chunk w, the first stage of chunk w - 1, the second of w - 2, and the third and the copy back
  // of w - 3 (without chunked_in, the second of w and the third of w - 1); every event is
  // recorded before a wait on it is issued
  const int lag = chunked_in ? 3 : 1;
  for (int w = 0; w < nch + lag; ++w) {
    if (chunked_in && w < nch) {  // the copy in
      const int64_t off = w * chunk, len = std::min(chunk, nc - off);
      HRW_CUDA(cudaMemcpyAsync(const_cast<double*>(cur) + off, uh + off, sizeof(double) * (size_t)len,
                               cudaMemcpyHostToDevice, o->copy));
      HRW_CUDA(cudaEventRecord(o->ev_in[w], o->copy));
      if (w == nch - 1)  // the input's true exponent, beside the stages
        HRW_CUDA(launch_mixed_scale(cur, nc, o->mscale + 1, o->copy));
    }
    if (const int i = w - (lag - 2); chunked_in && i >= 0 && i < nch) {  // the first stage
      MixedArgs b = range(a, i);
      b.dout = d1;
      HRW_CUDA(cudaStreamWaitEvent(o->pipe[0], o->ev_in[std::min(i + 1, nch - 1)], 0));
      HRW_CUDA(launch_stage1d_mixed(b, k, MX_E1, o->pipe[0]));
      HRW_CUDA(cudaEventRecord(o->ev_s1[i], o->pipe[0]));
    }
    if (const int i = w - (lag - 1); i >= 0 && i < nch) {  // the second stage
      MixedArgs b = range(a, i);
      b.dv = d1;
      b.dout = d2;
      if (chunked_in) HRW_CUDA(cudaStreamWaitEvent(o->pipe[1], o->ev_s1[std::min(i + 1, nch - 1)], 0));
      HRW_CUDA(launch_stage1d_mixed(b, k, MX_RK3B, o->pipe[1]));
      HRW_CUDA(cudaEventRecord(o->ev_s2[i], o->pipe[1]));
    }
    if (const int i = w - lag; i >= 0 && i < nch) {  // the third stage and the copy back
      MixedArgs b = range(a, i);
      b.dv = d2;
      b.uout = other;
      HRW_CUDA(cudaStreamWaitEvent(o->pipe3, o->ev_s2[std::min(i + 1, nch - 1)], 0));
      HRW_CUDA(launch_stage1d_mixed(b, k, MX_RK3C, o->pipe3));
      HRW_CUDA(cudaEventRecord(o->ev_s3[i], o->pipe3));
      HRW_CUDA(cudaStreamWaitEvent(o->copy_out, o->ev_s3[i], 0));
      HRW_CUDA(cudaMemcpyAsync(uh + b.cell0, other + b.cell0, sizeof(double) * (size_t)b.ncell,
                               cudaMemcpyDeviceToHost, o->copy_out));
    }
  }
  // the output's exponent: the next call's guess
  HRW_CUDA(launch_mixed_scale(other, nc, o->mscale + 2, o->pipe3));
  int q = 0;
  for (cudaStream_t st : {o->pipe[0], o->pipe[1], o->pipe3, o->copy, o->copy_out}) {
    cudaEvent_t ev = q < 3 ? o->ev_join[q] : o->ev_end[q - 3];
    HRW_CUDA(cudaEventRecord(ev, st));
    HRW_CUDA(cudaStreamWaitEvent(ms, ev, 0));
    ++q;
  }
  return HRW_OK;
}

static int rk3_integrate_host_mixed(hrw_ode* o, double* uh, double* t, double tout, double dt, int itask) {
  double tt;
  int64_t n;
  if (const int rc = count_steps(*t, tout, dt, itask, &n, &tt)) return rc;
  HRW_CUDA(mixed_pipe_init(o));
  const int64_t nc = o->neq;
  const size_t bytes = sizeof(double) * (size_t)nc;
  double* du = o->u;
  cudaStream_t ms = o->stream;
  bool done = false;
  if (n == 1 && o->mguess) {  // the guess: this input is the previous output
    // launched directly: replayed as a CUDA graph the same work measured slower (1.25e10
    // against 1.48e10 cell-updates/s end to end on the 2^24-cell line)
    HRW_CUDA(cudaMemcpyAsync(o->mscale, o->mscale + 2, sizeof(unsigned), cudaMemcpyDeviceToDevice, ms));
    if (const int rc = mixed_last_step(o, uh, du, o->w1, dt, true)) return rc;
    unsigned w[2] = {0, 0};
    HRW_CUDA(cudaStreamSynchronize(ms));
    HRW_CUDA(cudaMemcpy(w, o->mscale, sizeof(w), cudaMemcpyDeviceToHost));
    done = (w[0] >> 20) == (w[1] >> 20);  // the stages read the exponent only
    if (!done)  // taken again from the input on the device, with its true exponent
      HRW_CUDA(cudaMemcpyAsync(o->mscale, o->mscale + 1, sizeof(unsigned), cudaMemcpyDeviceToDevice, ms));
  } else {
    HRW_CUDA(cudaMemcpyAsync(du, uh, bytes, cudaMemcpyHostToDevice, ms));
    HRW_CUDA(launch_mixed_scale(du, nc, o->mscale, ms));
  }
  if (!done) {
    double* cur = du;
    if (const int rc = mixed_steps(o, du, n - 1, dt, &cur)) return rc;
    if (const int rc = mixed_last_step(o, uh, cur, cur == du ? o->w1 : du, dt, false)) return rc;
  }
  o->mguess = true;
  *t = tt;
  o->fevals += (int)(3 * n);
  o->nsteps += n;
  if (o->istate == 1) o->istate = 2;
  return HRW_OK;
}

// Whether a 2D stage block of this handle gave up waiting for its tile copies since the last
// check; clears the handle's flag.  Waits for the handle's stream.
static cudaError_t take_timeout(hrw_ode* o, bool* timed_out) {
  *timed_out = false;
  if (!o->tflag) return cudaSuccess;
  unsigned int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, o->tflag, sizeof(v), cudaMemcpyDeviceToHost, o->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(o->stream);
  if (e == cudaSuccess && v) e = cudaMemsetAsync(o->tflag, 0, sizeof(v), o->stream);
  if (e == cudaSuccess && v) e = cudaStreamSynchronize(o->stream);
  *timed_out = v != 0;
  return e;
}

static int integrate_on(hrw_ode* o, int mem, void* u, double* t, double tout, double dt, int itask);

extern "C" int hrw_integrate(hrw_ode* o, int mem, void* u, double* t, double tout, double dt, int itask) {
  if (!o) return fail(HRW_EINVAL, "Invalid input 'ode': null handle.");
  if (!u || !t) return fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (mem != HRW_MEM_HOST && mem != HRW_MEM_DEVICE) return fail(HRW_EINVAL, "Invalid input 'mem'.");
  if (o->istate < 1) return fail(HRW_ESTATE, "ode is in an error state.");  // (:126,228)
  if (o->dtype == HRW_F32) {  // a REAL32 build holds t, tout and dt in FP32
    const float tf = (float)*t, toutf = (float)tout, dtf = (float)dt;
    if (is_done(tf, toutf, dtf)) return HRW_OK;  // (:127,229)
    if (!(dtf != 0.0f) || !std::isfinite(dtf) || !std::isfinite(tf) || !std::isfinite(toutf))
      return fail(HRW_EINVAL, "Invalid input 'dt': must be finite and nonzero.");
  } else {
    if (is_done(*t, tout, dt)) return HRW_OK;  // (:127,229)
    if (!(dt != 0.0) || !std::isfinite(dt) || !std::isfinite(*t) || !std::isfinite(tout))
      return fail(HRW_EINVAL, "Invalid input 'dt': must be finite and nonzero.");
  }
  if (itask != 1 && itask != 2) itask = 1;
  const int rc = integrate_on(o, mem, u, t, tout, dt, itask);
  // a CUDA failure part-way leaves u (and the mstvd history) undefined: later calls refuse
  if (rc == HRW_ECUDA || rc == HRW_ENOMEM) o->istate = -1;
  return rc;
}

static int integrate_on32(hrw_ode* o, int mem, void* u, double* t, double tout, double dt, int itask) {
  const size_t bytes = sizeof(float) * (size_t)o->neq;
  float* du = (float*)u;
  if (mem == HRW_MEM_HOST) {
    du = o->su;
    HRW_CUDA(cudaMemcpyAsync(du, u, bytes, cudaMemcpyHostToDevice, o->stream));
  }
  float tf = (float)*t;
  const int rc = o->method == 0 ? rk_integrate32(o, du, &tf, (float)tout, (float)dt, itask)
                                : ms_integrate32(o, du, &tf, (float)tout, (float)dt);
  if (rc != HRW_OK) return rc;
  *t = tf;
  if (mem == HRW_MEM_HOST) HRW_CUDA(cudaMemcpyAsync(u, du, bytes, cudaMemcpyDeviceToHost, o->stream));
  HRW_CUDA(cudaStreamSynchronize(o->stream));
  return HRW_OK;
}

static int integrate_on(hrw_ode* o, int mem, void* u, double* t, double tout, double dt, int itask) {
  const size_t bytes = sizeof(double) * (size_t)o->neq;
  double* du = (double*)u;
  if (mem == HRW_MEM_HOST && host_pipeline_ok(o, u)) {
    const int rc = rk3_integrate_host(o, (double*)u, t, tout, dt, itask);
    if (rc != HRW_OK) return rc;
    HRW_CUDA(cudaStreamSynchronize(o->stream));
    return HRW_OK;
  }
  if (mem == HRW_MEM_HOST && host_pipeline_mixed_ok(o, u)) {
    const int rc = rk3_integrate_host_mixed(o, (double*)u, t, tout, dt, itask);
    if (rc != HRW_OK) return rc;
    HRW_CUDA(cudaStreamSynchronize(o->stream));
    return HRW_OK;
  }
  if (mem == HRW_MEM_HOST && o->dtype != HRW_F32) {
    du = o->u;
    HRW_CUDA(cudaMemcpyAsync(du, u, bytes, cudaMemcpyHostToDevice, o->stream));
  }
  int rc;
  if (o->dtype == HRW_F32)
    rc = integrate_on32(o, mem, u, t, tout, dt, itask);
  else if (o->dtype == HRW_F32C)
    rc = o->method == 0 ? rk_integrate_f32c(o, du, t, tout, dt, itask) : ms_integrate_f32c(o, du, t, tout, dt);
  else
    rc = o->method == 0 ? rk_integrate(o, du, t, tout, dt, itask) : ms_integrate(o, du, t, tout, dt);
  if (rc != HRW_OK) return rc;
  if (mem == HRW_MEM_HOST && o->dtype != HRW_F32)
    HRW_CUDA(cudaMemcpyAsync(u, du, bytes, cudaMemcpyDeviceToHost, o->stream));
  HRW_CUDA(cudaStreamSynchronize(o->stream));
  if (o->prob.kind == HRW_PROBLEM_FV2D) {
    bool timed_out = false;
    HRW_CUDA(take_timeout(o, &timed_out));
    if (timed_out) {
      o->istate = -1;
      return fail(HRW_ETIMEOUT, "hrw_integrate: a 2D stage block's bounded wait for its tile copies ran out.");
    }
  }
  return HRW_OK;
}

extern "C" int hrw_rhs(const hrw_problem* p, int dtype, double t, const void* v, void* vdot, void* stream) {
  (void)t;
  if (!v || !vdot) return fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (dtype != HRW_F64 && dtype != HRW_F32C && dtype != HRW_F32) return fail(HRW_EINVAL, "Invalid input 'dtype'.");
  // cells in 64 bits: the arrays hold at most 2^31 - 1 elements (neq is an int in the ABI)
  const int64_t cells = !p ? 0
                        : p->kind == HRW_PROBLEM_FV2D ? (int64_t)p->ncells[0] * p->ncells[1]
                                                      : (int64_t)p->ncells[0];
  if (p && p->ncells[0] > 0 && p->ncells[1] > 0 && cells > INT32_MAX)
    return fail(HRW_EINVAL, "Invalid input 'ncells': more than 2^31 - 1 cells.");
  const int neq = (int)cells;
  hrw_ode* o = nullptr;
  int rc = ode_create(p, neq, 1, 0, dtype, &o);
  if (rc != HRW_OK) return rc;
  if (stream) o->stream = (cudaStream_t)stream;
  cudaError_t e;
  if (dtype == HRW_F32) {
    e = run_stage32(o, ST_RHS, (const float*)v, (const float*)v, (float*)vdot, nullptr, nullptr, nullptr, 0.0f);
  } else if (dtype == HRW_F32C) {
    e = launch_split_f64((const double*)v, o->fhi[0], o->flo[0], neq, o->stream);
    if (e == cudaSuccess)
      e = run_f32c(o, FC_RHS, 0, nullptr, o->fd1, -1, nullptr, nullptr, nullptr, nullptr, 1.0);
    if (e == cudaSuccess) e = launch_widen_f32(o->fd1, (double*)vdot, neq, o->stream);
  } else {
    e = run_stage(o, ST_RHS, (const double*)v, (const double*)v, (double*)vdot, nullptr, nullptr,
                  nullptr, 0.0);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(o->stream);
  bool timed_out = false;
  if (e == cudaSuccess && p->kind == HRW_PROBLEM_FV2D) e = take_timeout(o, &timed_out);
  hrw_ode_destroy(o);
  if (e != cudaSuccess) return fail(HRW_ECUDA, std::string("hrw_rhs: ") + cudaGetErrorString(e));
  if (timed_out) return fail(HRW_ETIMEOUT, "hrw_rhs: a 2D stage block's bounded wait for its tile copies ran out.");
  return HRW_OK;
}
