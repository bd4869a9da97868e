// capi_batch.cu - the batch handle (hrw_batch_* in include/hrweno_gpu.h): validation, packed
// layout, per-problem step counts, size classes, the shape autotuner and the launches.
//
// Every problem follows the reference's integrate contract on its own: its step count comes
// from replaying `t = t + dt` until is_done (src/hrweno_tvdode.f90:137-143,273-284) with its
// own t and dt, so a batched solve takes exactly the steps of a loop of single solves.  An
// mstvd batch (hrw_batch_create_mstvd) keeps each problem's multistep history between calls and
// runs its RK3 start on its first call that takes a step (src/hrweno_tvdode.f90:203-271).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hrweno_gpu.h"
#include "hrw_batch.h"
#include "hrw_internal.h"

using namespace hrw;

namespace {

constexpr int kClasses = 3;
// size classes by cells: [0, 512), [512, 4096), [4096, inf)
constexpr int64_t kClassHi[kClasses] = {512, 4096, INT64_MAX};
// shapes used before (or without) tuning: one warp with 4 cells per thread for short lines,
// one warp with 8 for medium ones, a 256-thread block with 8 for long ones
constexpr int kDefaultShape[kClasses] = {1, 2, 5};
// compensated FP32 (kBatchShapesF32): 128 threads x 4 cells for short lines, 256 x 4 otherwise
constexpr int kDefaultShapeF32[kClasses] = {1, 2, 2};

bool is_done(double t, double tout, double dt) { return (t - tout) * std::copysign(1.0, dt) > 0.0; }

int cls_of(int64_t nc) {
  for (int c = 0; c < kClasses; ++c)
    if (nc < kClassHi[c]) return c;
  return kClasses - 1;
}

}  // namespace

struct hrw_batch {
  int nprob = 0, order = 3, dtype = HRW_F64;
  int method = 0;  // 0 rktvd, 1 mstvd
  double* ring = nullptr;     // mstvd: 5 packed states u^m and 4 packed L(u^m)
  bool nu = false;            // some problem has a non-uniform line (xedges)
  double* nu_mem = nullptr;   // their edges, widths, FAST scales and weno coefficients
  float* nu_fmem = nullptr;   // HRW_F32C: the same lines in FP32 (coefficients, 1/width, b width, edges)
  std::vector<char> started;  // mstvd: the problem's RK3 start has run
  std::vector<int64_t> level; // mstvd: m of the problem's current state
  bool strict = false;
  std::vector<BatchProblem> probs;
  std::vector<int64_t> off;  // nprob + 1
  int64_t total = 0;
  std::vector<int> members[kClasses + 1];  // + the non-uniform lines, launched on their own
  int shape[kClasses] = {kDefaultShape[0], kDefaultShape[1], kDefaultShape[2]};
  bool tuned = false;
  BatchProblem* d_probs = nullptr;
  int* d_order = nullptr;
  int* d_counter = nullptr;
  double* u = nullptr;  // device state for host-memory calls
  double* u1 = nullptr;
  double* u2 = nullptr;
  float* fmem = nullptr;  // HRW_F32C: hi/lo slots x 2, d1, d2 (packed like u)
  cudaStream_t own = nullptr, main = nullptr;
  cudaStream_t side[kClasses + 1] = {};
  cudaEvent_t fork = nullptr, join[kClasses + 1] = {};
  int sms = 0;
  std::vector<int64_t> steps_done;  // per problem, all calls
  std::string dev_name;
};

namespace {

int batch_fail(int code, const std::string& m) { return set_error(code, m.c_str()); }

#define HRW_BCUDA(call)                                                                  \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return batch_fail(e_ == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,        \
                        std::string(#call ": ") + cudaGetErrorString(e_));               \
  } while (0)

// Launch every class of the batch for the step counts already in b->probs (uploaded) on the
// state `u`: the classes run concurrently on their own streams, each one persistent launch; the
// non-uniform lines (class kClasses) have one launch of their own.
int launch_all(hrw_batch* b, double* u, const int* shapes) {
  std::vector<int> order;
  std::vector<int> start(kClasses + 2, 0);
  for (int c = 0; c <= kClasses; ++c) {
    std::vector<int> m = b->members[c];
    std::stable_sort(m.begin(), m.end(), [&](int x, int y) {
      return (double)b->probs[x].nc * b->probs[x].nsteps > (double)b->probs[y].nc * b->probs[y].nsteps;
    });
    start[c] = (int)order.size();
    order.insert(order.end(), m.begin(), m.end());
  }
  start[kClasses + 1] = (int)order.size();
  HRW_BCUDA(cudaMemcpyAsync(b->d_probs, b->probs.data(), sizeof(BatchProblem) * b->nprob,
                            cudaMemcpyHostToDevice, b->main));
  HRW_BCUDA(cudaMemcpyAsync(b->d_order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice,
                            b->main));
  HRW_BCUDA(cudaMemsetAsync(b->d_counter, 0, sizeof(int) * (kClasses + 1), b->main));
  HRW_BCUDA(cudaEventRecord(b->fork, b->main));
  for (int c = 0; c <= kClasses; ++c) {
    const int n = start[c + 1] - start[c];
    HRW_BCUDA(cudaStreamWaitEvent(b->side[c], b->fork, 0));
    if (n > 0) {
      BatchArgs A{};
      A.probs = b->d_probs;
      A.order_idx = b->d_order + start[c];
      A.nprob = n;
      A.counter = b->d_counter + c;
      A.u = u;
      A.u1 = b->u1;
      A.u2 = b->u2;
      A.order = b->order;
      A.method = b->method;
      if (b->ring) {
        for (int q = 0; q < 5; ++q) A.ring_u[q] = b->ring + (size_t)q * b->total;
        for (int q = 0; q < 4; ++q) A.ring_l[q] = b->ring + (size_t)(5 + q) * b->total;
      }
      const bool f32 = b->dtype == HRW_F32C;
      if (f32) {
        float* q = b->fmem;
        for (int k = 0; k < 2; ++k) {
          A.fhi[k] = q, q += b->total;
          A.flo[k] = q, q += b->total;
        }
        A.fd1 = q, q += b->total;
        A.fd2 = q, q += b->total;
        if (b->method == 1) {
          for (int k = 0; k < 5; ++k) A.fring_h[k] = q, q += b->total;
          for (int k = 0; k < 5; ++k) A.fring_lo[k] = q, q += b->total;
          for (int k = 0; k < 4; ++k) A.fring_L[k] = q, q += b->total;
        }
      }
      const bool nu = c == kClasses;
      const bool ms = A.method == 1;
      const int per_sm = std::max(1, nu    ? (f32 ? batch_f32c_nu_blocks_per_sm(ms) : batch_nu_blocks_per_sm(b->strict))
                                     : f32 ? batch_f32_blocks_per_sm(shapes[c], ms)
                                           : batch_blocks_per_sm(shapes[c], b->strict));
      const int group = nu ? kBatchNuGroup : f32 ? kBatchShapesF32[shapes[c]].group : kBatchShapes[shapes[c]].group;
      const int groups_per_block = 256 / group;
      int blocks = per_sm * b->sms;
      blocks = std::min<int64_t>(blocks, (n + groups_per_block - 1) / groups_per_block);
      if (nu && f32) HRW_BCUDA(launch_batch_f32c_nu(A, std::max(blocks, 1), b->side[c]));
      else if (nu) HRW_BCUDA(launch_batch_nu(A, b->strict, std::max(blocks, 1), b->side[c]));
      else if (f32) HRW_BCUDA(launch_batch_f32c(A, shapes[c], std::max(blocks, 1), b->side[c]));
      else HRW_BCUDA(launch_batch(A, shapes[c], b->strict, std::max(blocks, 1), b->side[c]));
    }
    HRW_BCUDA(cudaEventRecord(b->join[c], b->side[c]));
    HRW_BCUDA(cudaStreamWaitEvent(b->main, b->join[c], 0));
  }
  return HRW_OK;
}

// launch_all on the packed FP64 state du; compensated FP32 batches split it into their
// (hi, lo) slot 0 first and merge the result back
int run_all(hrw_batch* b, double* du) {
  // (compensated mstvd: each problem splits its lines into its ring slot and merges them back
  // in the kernel)
  if (b->dtype == HRW_F32C && b->method == 0) {
    float* hi = b->fmem;
    float* lo = b->fmem + b->total;
    HRW_BCUDA(launch_split_f64(du, hi, lo, b->total, b->main));
    int rc = launch_all(b, du, b->shape);
    if (rc != HRW_OK) return rc;
    HRW_BCUDA(launch_merge_f64(hi, lo, du, b->total, b->main));
    return HRW_OK;
  }
  return launch_all(b, du, b->shape);
}

std::string tune_key(const hrw_batch* b, int c) {
  int64_t cells = 0;
  int mix = 0;
  for (int p : b->members[c]) {
    cells += b->probs[p].nc;
    mix |= 1 << b->probs[p].k;
  }
  std::ostringstream s;
  s << b->dev_name << "|class" << c << "|n" << b->members[c].size() << "|cells" << cells << "|k" << mix
    << "|order" << b->order << "|" << (b->strict ? "strict" : "fast") << (b->method ? "|ms" : "")
    << (b->nu ? "|nu" : "")
    << (b->dtype == HRW_F32C ? "|f32c" : "|f64");
  std::string k = s.str();
  std::replace(k.begin(), k.end(), ' ', '_');
  return k;
}

// After a call: problem i's steps (the mstvd start counts its 4), its level and start flag.
void note_steps(hrw_batch* b, int i) {
  const BatchProblem& q = b->probs[i];
  b->steps_done[i] += q.nsteps + (q.start ? 4 : 0);
  if (b->method == 1 && (q.start || q.nsteps > 0)) {
    b->level[i] = (q.start ? 4 : b->level[i]) + q.nsteps;
    b->started[i] = 1;
  }
}

}  // namespace

static int batch_create(const hrw_problem* probs, int nprob, int order, int dtype, int method,
                        hrw_batch** out) {
  if (!out) return batch_fail(HRW_EINVAL, "Invalid input 'out': null pointer.");
  *out = nullptr;
  if (!probs || nprob <= 0) return batch_fail(HRW_EINVAL, "Invalid input 'nprob': must be >= 1.");
  if (order < 1 || order > 3)
    return batch_fail(HRW_EINVAL, "Invalid input 'order' in 'rktvd'. Valid range: 1 <= k <= 3.");
  if (dtype != HRW_F64 && dtype != HRW_F32C)
    return batch_fail(HRW_EINVAL, "Invalid input 'dtype': batches support HRW_F64 and HRW_F32C.");
  hrw_batch* b = new hrw_batch;
  b->nprob = nprob;
  b->order = order;
  b->dtype = dtype;
  b->method = method;
  if (dtype == HRW_F32C)
    for (int c = 0; c < kClasses; ++c) b->shape[c] = kDefaultShapeF32[c];
  b->strict = probs[0].numerics == HRW_NUMERICS_STRICT;
  b->off.resize(nprob + 1);
  int64_t off = 0;
  for (int i = 0; i < nprob; ++i) {
    const hrw_problem& p = probs[i];
    std::string where = " (problem " + std::to_string(i) + ")";
    auto bad = [&](const char* m) {
      delete b;
      return batch_fail(HRW_EINVAL, std::string(m) + where);
    };
    if (p.kind != HRW_PROBLEM_FV1D) return bad("Invalid input 'kind': batches hold FV1D problems.");
    if (p.ncells[0] <= 0) return bad("Invalid input 'ncells'. Valid range: ncells > 0.");
    if (p.width[0]) return bad("Invalid input 'width': batches take non-uniform lines as xedges.");
    if (p.xedges[0]) {
      for (int q = 0; q < p.ncells[0]; ++q)
        if (!(p.xedges[0][q + 1] > p.xedges[0][q])) return bad("Invalid input 'xedges': edges must increase.");
    }
    if (p.k < 1 || p.k > 3) return bad("Invalid input 'k'. Valid range: 1 <= k <= 3.");
    if (!(p.eps > 2.220446049250313e-16)) return bad("Invalid input 'eps'. Valid range: eps > epsilon.");
    if (p.flux != HRW_FLUX_LAX_FRIEDRICHS && p.flux != HRW_FLUX_GODUNOV) return bad("Invalid input 'flux'.");
    if (p.fn[0] < HRW_FN_BURGERS || p.fn[0] > HRW_FN_BURGERS_LINEAR) return bad("Invalid input 'fn'.");
    if (p.fn[0] == HRW_FN_BURGERS_LINEAR && b->dtype == HRW_F32C)
      return bad("Invalid input 'fn': HRW_F32C supports BURGERS and LINEAR.");
    if (p.bc[0] < HRW_BC_COPY || p.bc[0] > HRW_BC_ZERO_INFLOW) return bad("Invalid input 'bc'.");
    if (!(p.xmax[0] > p.xmin[0])) return bad("Invalid input 'xmin', 'xmax'. Valid range: xmax > xmin.");
    if ((p.numerics == HRW_NUMERICS_STRICT) != b->strict)
      return bad("Invalid input 'numerics': all problems of a batch share one numerics mode.");
    BatchProblem q{};
    q.off = off;
    q.nc = p.ncells[0];
    q.k = p.k;
    q.fn = p.fn[0];
    q.flux = p.flux;
    q.bc = p.bc[0];
    q.a = p.coef_a[0];
    q.b = p.coef_b[0];
    q.alpha = p.alpha[0];
    q.xmin = p.xmin[0];
    q.rx = (p.xmax[0] - p.xmin[0]) / q.nc;  // grid1%linear (src/hrweno_grids.f90:72)
    q.rws0 = fast_flux_scale(p.flux, p.fn[0]) / q.rx;
    q.eps = p.eps;
    b->probs.push_back(q);
    b->off[i] = off;
    off += (q.nc + 63) / 64 * 64;
    b->members[p.xedges[0] ? kClasses : cls_of(q.nc)].push_back(i);
  }
  b->off[nprob] = off;
  b->total = off;
  b->steps_done.assign(nprob, 0);
  b->started.assign(nprob, 0);
  b->level.assign(nprob, 0);
  auto cleanup = [&](cudaError_t e) {
    hrw_batch_destroy(b);
    return batch_fail(e == cudaErrorMemoryAllocation ? HRW_ENOMEM : HRW_ECUDA,
                      std::string("hrw_batch_create: ") + cudaGetErrorString(e));
  };
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceProp prop{};
  if (e == cudaSuccess) e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return cleanup(e);
  b->dev_name = prop.name;
  const size_t bytes = sizeof(double) * (size_t)off;
  if ((e = cudaStreamCreateWithFlags(&b->own, cudaStreamDefault)) != cudaSuccess) return cleanup(e);
  b->main = b->own;
  for (int c = 0; c <= kClasses; ++c) {
    if ((e = cudaStreamCreateWithFlags(&b->side[c], cudaStreamNonBlocking)) != cudaSuccess) return cleanup(e);
    if ((e = cudaEventCreateWithFlags(&b->join[c], cudaEventDisableTiming)) != cudaSuccess) return cleanup(e);
  }
  if ((e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess) return cleanup(e);
  if ((e = cudaMalloc(&b->d_probs, sizeof(BatchProblem) * nprob)) != cudaSuccess) return cleanup(e);
  if ((e = cudaMalloc(&b->d_order, sizeof(int) * nprob)) != cudaSuccess) return cleanup(e);
  if ((e = cudaMalloc(&b->d_counter, sizeof(int) * (kClasses + 1))) != cudaSuccess) return cleanup(e);
  if ((e = cudaMalloc(&b->u, bytes)) != cudaSuccess) return cleanup(e);
  if (dtype == HRW_F32C) {
    // slots (hi, lo) x 2, d1, d2; mstvd adds the ring: u^m (hi, lo) x 5 and L(u^m) x 4
    const size_t per_cell = method == 1 ? 6 + 14 : 6;
    if ((e = cudaMalloc(&b->fmem, sizeof(float) * (size_t)off * per_cell)) != cudaSuccess) return cleanup(e);
  } else {
    if ((e = cudaMalloc(&b->u1, bytes)) != cudaSuccess) return cleanup(e);
    if ((e = cudaMalloc(&b->u2, bytes)) != cudaSuccess) return cleanup(e);
  }
  if (method == 1 && (e = cudaMalloc(&b->ring, bytes * 9)) != cudaSuccess) return cleanup(e);
  // non-uniform lines: per problem edges(0:nc), widths edges(i) - edges(i-1), FAST scales
  // fs / width and cnu(0:k-1,-1:k-1,1:nc) by weno_calc_cnu on the device (src/hrweno_weno.f90:221-297)
  size_t nu_len = 0;
  for (int i = 0; i < nprob; ++i)
    if (probs[i].xedges[0]) nu_len += (size_t)(probs[i].ncells[0] + 1) + 2 * (size_t)probs[i].ncells[0] +
                                      (size_t)probs[i].k * (probs[i].k + 1) * probs[i].ncells[0];
  if (nu_len) {
    b->nu = true;
    if ((e = cudaMalloc(&b->nu_mem, sizeof(double) * nu_len)) != cudaSuccess) return cleanup(e);
    double* q = b->nu_mem;
    for (int i = 0; i < nprob; ++i) {
      const hrw_problem& p = probs[i];
      if (!p.xedges[0]) continue;
      BatchProblem& bp = b->probs[i];
      const int nc = p.ncells[0];
      const double fs = fast_flux_scale(p.flux, p.fn[0]);
      std::vector<double> host((size_t)3 * nc + 1);
      for (int j = 0; j <= nc; ++j) host[j] = p.xedges[0][j];
      for (int j = 0; j < nc; ++j) {
        host[nc + 1 + j] = p.xedges[0][j + 1] - p.xedges[0][j];
        host[2 * nc + 1 + j] = fs / host[nc + 1 + j];
      }
      if ((e = cudaMemcpy(q, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cleanup(e);
      bp.xe = q;
      bp.width = q + nc + 1;
      bp.rws = q + 2 * nc + 1;
      bp.cnu = q + 3 * nc + 1;
      if ((e = launch_calc_cnu(bp.xe, q + 3 * nc + 1, nc, p.k, b->own)) != cudaSuccess) return cleanup(e);
      q += host.size() + (size_t)p.k * (p.k + 1) * nc;
    }
    if ((e = cudaStreamSynchronize(b->own)) != cudaSuccess) return cleanup(e);
    if (dtype == HRW_F32C) {
      // the compensated pass's copy of each line, as a single-line handle builds it: the FP64
      // coefficients rounded once, 1/width and b width from the FP64 widths, the edges rounded
      size_t nf = 0;
      for (int i = 0; i < nprob; ++i)
        if (probs[i].xedges[0]) nf += nu_line_f32_floats(probs[i].ncells[0], probs[i].k);
      if ((e = cudaMalloc(&b->nu_fmem, sizeof(float) * nf)) != cudaSuccess) return cleanup(e);
      float* f = b->nu_fmem;
      for (int i = 0; i < nprob; ++i) {
        const hrw_problem& p = probs[i];
        if (!p.xedges[0]) continue;
        BatchProblem& bp = b->probs[i];
        NuLineF32 nl{};
        if ((e = build_nu_line_f32(p.xedges[0], p.ncells[0], p.k, p.coef_b[0], bp.cnu, f, &nl)) != cudaSuccess)
          return cleanup(e);
        bp.frw = nl.rw;
        bp.fxe = nl.xe;
        bp.fgst = nl.gst;
        bp.fcnu = nl.cnu;
        f += nu_line_f32_floats(p.ncells[0], p.k);
      }
    }
  }
  *out = b;
  return HRW_OK;
}

extern "C" {

int hrw_batch_create(const hrw_problem* probs, int nprob, int order, int dtype, hrw_batch** out) {
  return batch_create(probs, nprob, order, dtype, 0, out);
}

int hrw_batch_create_mstvd(const hrw_problem* probs, int nprob, int dtype, hrw_batch** out) {
  return batch_create(probs, nprob, 3, dtype, 1, out);
}

int hrw_batch_layout(const hrw_batch* b, int64_t* offsets) {
  if (!b || !offsets) return batch_fail(HRW_EINVAL, "Invalid input: null pointer.");
  std::memcpy(offsets, b->off.data(), sizeof(int64_t) * (b->nprob + 1));
  return HRW_OK;
}

int hrw_batch_info(const hrw_batch* b, int* shapes, int64_t* steps_done) {
  if (!b) return batch_fail(HRW_EINVAL, "Invalid input 'batch': null handle.");
  if (shapes)
    for (int c = 0; c < kClasses; ++c) {
      const BatchShape& sh = b->dtype == HRW_F32C ? kBatchShapesF32[b->shape[c]] : kBatchShapes[b->shape[c]];
      shapes[2 * c] = sh.group;
      shapes[2 * c + 1] = sh.cells;
    }
  if (steps_done) std::memcpy(steps_done, b->steps_done.data(), sizeof(int64_t) * b->nprob);
  return HRW_OK;
}

int hrw_batch_set_stream(hrw_batch* b, void* stream) {
  if (!b) return batch_fail(HRW_EINVAL, "Invalid input 'batch': null handle.");
  b->main = stream ? (cudaStream_t)stream : b->own;
  return HRW_OK;
}

// Advance problem i from t[i] to the first t > tout with its own dt[i] (itask = 1), or by
// exactly one step when itask = 2; t[] is updated.  u is the packed state (layout from
// hrw_batch_layout) in memory space `mem`.
int hrw_batch_integrate(hrw_batch* b, int mem, double* u, double* t, double tout, const double* dt,
                        int itask) {
  if (!b) return batch_fail(HRW_EINVAL, "Invalid input 'batch': null handle.");
  if (!u || !t || !dt) return batch_fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (mem != HRW_MEM_HOST && mem != HRW_MEM_DEVICE) return batch_fail(HRW_EINVAL, "Invalid input 'mem'.");
  std::vector<double> tnew(b->nprob);
  for (int i = 0; i < b->nprob; ++i) {
    const double h = dt[i];
    if (!(h != 0.0) || !std::isfinite(h) || !std::isfinite(t[i]))
      return batch_fail(HRW_EINVAL, "Invalid input 'dt': must be finite and nonzero (problem " +
                                        std::to_string(i) + ").");
    double tt = t[i];
    int64_t n = 0;
    BatchProblem& q = b->probs[i];
    q.start = 0;
    q.level = b->level[i];
    if (!is_done(tt, tout, h)) {
      if (b->method == 1) {  // mstvd_integrate: the RK3 start once, then until is_done (:236-268)
        if (!b->started[i]) {
          q.start = 1;
          for (int m = 0; m < 4; ++m) tt = tt + h;
        }
        while (!is_done(tt, tout, h)) {
          const double t1 = tt + h;
          if (t1 == tt) return batch_fail(HRW_EINVAL, "Invalid input 'dt': t + dt == t, so tout is never reached.");
          tt = t1;
          if (++n > (int64_t(1) << 40))
            return batch_fail(HRW_EINVAL, "Invalid input 'dt': too many steps to reach tout.");
        }
      } else {
        do {  // (src/hrweno_tvdode.f90:137-143)
          const double t1 = tt + h;
          if (t1 == tt) return batch_fail(HRW_EINVAL, "Invalid input 'dt': t + dt == t, so tout is never reached.");
          tt = t1;
          if (++n > (int64_t(1) << 40))
            return batch_fail(HRW_EINVAL, "Invalid input 'dt': too many steps to reach tout.");
        } while (!(is_done(tt, tout, h) || itask == 2));
      }
    }
    q.dt = h;
    q.nsteps = n;
    tnew[i] = tt;
  }
  double* du = u;
  const size_t bytes = sizeof(double) * (size_t)b->total;
  if (mem == HRW_MEM_HOST) {
    du = b->u;
    HRW_BCUDA(cudaMemcpyAsync(du, u, bytes, cudaMemcpyHostToDevice, b->main));
  }
  int rc = run_all(b, du);
  if (rc != HRW_OK) return rc;
  if (mem == HRW_MEM_HOST) HRW_BCUDA(cudaMemcpyAsync(u, du, bytes, cudaMemcpyDeviceToHost, b->main));
  HRW_BCUDA(cudaStreamSynchronize(b->main));
  for (int i = 0; i < b->nprob; ++i) {
    t[i] = tnew[i];
    note_steps(b, i);
  }
  return HRW_OK;
}

// nsteps steps of every problem (nsteps calls of integrate(itask = 2) each), one launch per
// size class; t[] is updated with the reference's t = t + dt sequence.
int hrw_batch_advance(hrw_batch* b, int mem, double* u, double* t, const double* dt, int64_t nsteps) {
  if (!b) return batch_fail(HRW_EINVAL, "Invalid input 'batch': null handle.");
  if (!u || !t || !dt) return batch_fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (mem != HRW_MEM_HOST && mem != HRW_MEM_DEVICE) return batch_fail(HRW_EINVAL, "Invalid input 'mem'.");
  if (nsteps < 0) return batch_fail(HRW_EINVAL, "Invalid input 'nsteps': must be >= 0.");
  for (int i = 0; i < b->nprob; ++i) {
    if (!(dt[i] != 0.0) || !std::isfinite(dt[i]) || !std::isfinite(t[i]))
      return batch_fail(HRW_EINVAL, "Invalid input 'dt': must be finite and nonzero (problem " +
                                        std::to_string(i) + ").");
    BatchProblem& q = b->probs[i];
    q.dt = dt[i];
    q.nsteps = nsteps;
    q.start = b->method == 1 && !b->started[i];
    q.level = b->level[i];
  }
  double* du = u;
  const size_t bytes = sizeof(double) * (size_t)b->total;
  if (mem == HRW_MEM_HOST) {
    du = b->u;
    HRW_BCUDA(cudaMemcpyAsync(du, u, bytes, cudaMemcpyHostToDevice, b->main));
  }
  int rc = run_all(b, du);
  if (rc != HRW_OK) return rc;
  if (mem == HRW_MEM_HOST) HRW_BCUDA(cudaMemcpyAsync(u, du, bytes, cudaMemcpyDeviceToHost, b->main));
  HRW_BCUDA(cudaStreamSynchronize(b->main));
  for (int i = 0; i < b->nprob; ++i) {
    const int64_t n = nsteps + (b->probs[i].start ? 4 : 0);
    for (int64_t s = 0; s < n; ++s) t[i] = t[i] + dt[i];
    note_steps(b, i);
  }
  return HRW_OK;
}

// Autotuner: for every size class, time `probe_steps` steps of that class alone with each
// candidate shape, and keep the fastest.  The probes run on the handle's scratch copy of the
// state u (memory space `mem`), which they advance; u itself is not changed.  Results are
// cached in the text file cache_path (one "key shape" line per class; NULL: no cache), keyed
// by the device name and the class's problem count, total cells, k mix, order and numerics.
int hrw_batch_tune(hrw_batch* b, int mem, const double* u, const double* dt, int probe_steps,
                   const char* cache_path) {
  if (!b || !u || !dt) return batch_fail(HRW_EINVAL, "Invalid input: null pointer.");
  if (mem != HRW_MEM_HOST && mem != HRW_MEM_DEVICE) return batch_fail(HRW_EINVAL, "Invalid input 'mem'.");
  if (probe_steps < 1) probe_steps = 1;
  std::vector<std::pair<std::string, int>> cache;
  if (cache_path) {
    std::ifstream in(cache_path);
    std::string k;
    int s;
    while (in >> k >> s)
      if (s >= 0 && s < (b->dtype == HRW_F32C ? kNumBatchShapesF32 : kNumBatchShapes)) cache.emplace_back(k, s);
  }
  const size_t bytes = sizeof(double) * (size_t)b->total;
  HRW_BCUDA(cudaMemcpyAsync(b->u, u, bytes,
                            mem == HRW_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                            b->main));
  if (b->dtype == HRW_F32C)
    HRW_BCUDA(launch_split_f64(b->u, b->fmem, b->fmem + b->total, b->total, b->main));
  struct Events {  // destroyed on every return, early ones included
    cudaEvent_t e[2] = {};
    ~Events() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } ev;
  cudaEvent_t& e0 = ev.e[0];
  cudaEvent_t& e1 = ev.e[1];
  HRW_BCUDA(cudaEventCreate(&e0));
  HRW_BCUDA(cudaEventCreate(&e1));
  bool wrote = false;
  for (int c = 0; c < kClasses; ++c) {
    if (b->members[c].empty()) continue;
    const std::string key = tune_key(b, c);
    auto hit = std::find_if(cache.begin(), cache.end(), [&](auto& kv) { return kv.first == key; });
    if (hit != cache.end()) {
      b->shape[c] = hit->second;
      continue;
    }
    // only this class advances during its probe
    for (int i = 0; i < b->nprob; ++i) {
      b->probs[i].dt = dt[i];
      b->probs[i].nsteps = 0;
    }
    for (int p : b->members[c]) b->probs[p].nsteps = probe_steps;
    for (int i = 0; i < b->nprob; ++i) b->probs[i].start = 0;
    float best = 1e30f;
    const bool f32 = b->dtype == HRW_F32C;
    int best_s = f32 ? kDefaultShapeF32[c] : kDefaultShape[c];
    for (int s = 0; s < (f32 ? kNumBatchShapesF32 : kNumBatchShapes); ++s) {
      int shapes[kClasses] = {b->shape[0], b->shape[1], b->shape[2]};
      shapes[c] = s;
      float ms = 0.f;
      for (int rep = 0; rep < 2; ++rep) {  // first run warms up
        HRW_BCUDA(cudaEventRecord(e0, b->main));
        // an mstvd batch probes RK3 steps of the same stage code, leaving its history as it is
        const int method = b->method;
        b->method = 0;
        int rc = launch_all(b, b->u, shapes);
        b->method = method;
        if (rc != HRW_OK) return rc;
        HRW_BCUDA(cudaEventRecord(e1, b->main));
        HRW_BCUDA(cudaEventSynchronize(e1));
        HRW_BCUDA(cudaEventElapsedTime(&ms, e0, e1));
      }
      if (ms < best) best = ms, best_s = s;
    }
    b->shape[c] = best_s;
    cache.emplace_back(key, best_s);
    wrote = true;
  }
  b->tuned = true;
  if (wrote && cache_path) {
    std::ofstream outf(cache_path);
    for (auto& kv : cache) outf << kv.first << " " << kv.second << "\n";
  }
  return HRW_OK;
}

int hrw_batch_destroy(hrw_batch* b) {
  if (!b) return HRW_OK;
  if (b->d_probs) cudaFree(b->d_probs);
  if (b->d_order) cudaFree(b->d_order);
  if (b->d_counter) cudaFree(b->d_counter);
  if (b->u) cudaFree(b->u);
  if (b->u1) cudaFree(b->u1);
  if (b->u2) cudaFree(b->u2);
  if (b->fmem) cudaFree(b->fmem);
  if (b->ring) cudaFree(b->ring);
  if (b->nu_mem) cudaFree(b->nu_mem);
  if (b->nu_fmem) cudaFree(b->nu_fmem);
  for (int c = 0; c <= kClasses; ++c) {
    if (b->side[c]) cudaStreamDestroy(b->side[c]);
    if (b->join[c]) cudaEventDestroy(b->join[c]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
  return HRW_OK;
}

}  // extern "C"
