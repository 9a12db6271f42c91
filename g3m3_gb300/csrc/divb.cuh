// divb.cuh -- state and arguments of the div B conjugate-gradient solver.
#pragma once

#include <map>
#include <string>

#include "kargs.cuh"

namespace g3m3 {

enum CgStatus : int { CG_RUNNING = 0, CG_CONVERGED = 1, CG_RESTART = 2, CG_MAXIT = 3, CG_GAVE_UP = 4 };

struct CgState {          // lives in device memory
  double anum, aden, r2, rsq, bsq, gg, dgg, errlim2, r2_last;
  float gam, pad;
  int status, iters, maxit, redos;
};

struct DivbArgs {
  float *bx, *by, *bz;    // box slices, updated in place
  float *rhs, *x, *xs, *g, *h, *xi, *xj;   // scratch vectors of one box
  CgState* st;
  Dims d;
  float rx, ry, rz;
  // explicit banded operator (sparse_solver): band(nbands, n) column-major,
  // product out(i) = sum_b band(b, i+pos[b]) x(i+pos[b]) (banded_tpose);
  // null: the matrix-free 7-point Laplacian of d
  const float* band;
  int nbands;
  int pos[16];
};

// CUDA graphs of solver iterations.  A chunk of n iterations is 7n small
// kernels whose launches, not their work, bound a solve on a box that fits
// in L2; replaying captured graphs of 64, 32, ..., 1 iterations (captured on
// first use for each argument block) issues a chunk in at most a few graph
// launches.  The kernels and their order are those of
// divb_launch_iterations, so the results are the same.
class CgGraphs {
 public:
  CgGraphs() = default;
  CgGraphs(const CgGraphs&) = delete;
  CgGraphs& operator=(const CgGraphs&) = delete;
  ~CgGraphs() { clear(); }
  // queue n iterations on s; falls back to plain launches where a graph
  // cannot be captured (s already capturing)
  cudaError_t iterations(const DivbArgs& a, int n, cudaStream_t s);
  void clear();

 private:
  cudaGraphExec_t get(const DivbArgs& a, int m, cudaStream_t s);
  std::map<std::string, cudaGraphExec_t> execs_;
};

// one CG solve in flight (the host side of cg_begin / cg_step)
struct CgRun {
  DivbArgs a;
  CgState* host_st = nullptr;   // pinned read-back of a.st
  cudaStream_t s = nullptr;
  int chunk = 8;
  bool first = true;
  int status = 0;
  CgGraphs* graphs = nullptr;   // null: iterations as plain launches
};

void divb_launch_init(const DivbArgs& a, cudaStream_t s);
void divb_launch_init_given(const DivbArgs& a, cudaStream_t s);
void divb_launch_restart(const DivbArgs& a, cudaStream_t s);
void divb_launch_restore(const DivbArgs& a, cudaStream_t s);
void divb_launch_iterations(const DivbArgs& a, int n, cudaStream_t s);
void divb_launch_apply(const DivbArgs& a, cudaStream_t s);

}  // namespace g3m3
