// hrw_batch.h - device-side layout of a batch of independent 1D problems (batch.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace hrw {

// One problem of the batch: the example1 right-hand side on its own uniform line, with its own
// time step and number of steps for the current integrate call.
struct BatchProblem {
  int64_t off;     // first cell in the packed arrays (a multiple of 64)
  int nc, k, fn, flux, bc;
  double a, b, alpha, xmin, rx, rws0, eps;
  double dt;
  int64_t nsteps;  // rktvd: steps; mstvd: multistep steps after the start
  // mstvd: run the RK3 start first (the problem's first call), and the level m of the state
  // u^m when the call begins (after the start: 4)
  int start;
  int64_t level;
  // non-uniform line (xedges): its weno coefficients cnu, widths, FAST 1/width scales and edges
  // (device arrays of the batch); null for a uniform line
  const double* cnu;
  const double* width;
  const double* rws;
  const double* xe;
  // the same line for compensated FP32 batches: cnu rounded to FP32, 1/width and b width from
  // the FP64 widths, the edges in FP32 (LineF's cnu, rw, gst, xe)
  const float* fcnu;
  const float* frw;
  const float* fgst;
  const float* fxe;
};

struct BatchArgs {
  const BatchProblem* probs;
  const int* order_idx;  // problems of this launch, most expensive first
  int nprob;
  int* counter;          // next entry of order_idx to claim
  double* u;             // packed state
  double* u1;            // packed stage arrays
  double* u2;
  int order;             // rktvd order 1..3
  // mstvd batches (method 1): u^m in ring_u[m % 5], L(u^m) in ring_l[m % 4], packed
  int method;
  double* ring_u[5];
  double* ring_l[4];
  // compensated FP32 batches: state slots (hi, lo) x 2 and the stage increments, packed;
  // mstvd: the ring of u^m (hi, lo) [m % 5] and L(u^m) [m % 4] instead of the two slots
  float* fhi[2];
  float* flo[2];
  float* fd1;
  float* fd2;
  float* fring_h[5];
  float* fring_lo[5];
  float* fring_L[4];
};

struct BatchShape {
  int group;  // threads that share one problem (whole warps)
  int cells;  // consecutive cells per thread and pass
};

constexpr int kNumBatchShapes = 6;
extern const BatchShape kBatchShapes[kNumBatchShapes];

int batch_blocks_per_sm(int shape, bool strict);
cudaError_t launch_batch(const BatchArgs& B, int shape, bool strict, int blocks, cudaStream_t s);
// the non-uniform lines of a batch: one launch of 128-thread groups, 4 cells per thread
constexpr int kBatchNuGroup = 128;
int batch_nu_blocks_per_sm(bool strict);
cudaError_t launch_batch_nu(const BatchArgs& B, bool strict, int blocks, cudaStream_t s);

// compensated FP32 batches: their own shapes (cells per thread a multiple of 4)
constexpr int kNumBatchShapesF32 = 3;
extern const BatchShape kBatchShapesF32[kNumBatchShapesF32];
int batch_f32_blocks_per_sm(int shape, bool ms);  // ms: the mstvd batches' kernel
cudaError_t launch_batch_f32c(const BatchArgs& B, int shape, int blocks, cudaStream_t s);
// their non-uniform lines: one launch of 128-thread groups, 4 cells per thread
int batch_f32c_nu_blocks_per_sm(bool ms);
cudaError_t launch_batch_f32c_nu(const BatchArgs& B, int blocks, cudaStream_t s);

}  // namespace hrw
