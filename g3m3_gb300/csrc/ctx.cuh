// ctx.cuh -- the library context: stream, host-array mirrors, scratch.
#pragma once

#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#include "bndry.cuh"
#include "divb.cuh"
#include "launch.cuh"

struct g3m3_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  struct Mirror {
    void* dev;
    size_t bytes;
    bool floats;                      // FP32 data (checked for NaN/Inf when checks are on)
  };
  std::unordered_map<const void*, Mirror> mirrors;
  std::string err;
  float iso_flag = 1.0f;   // set_speed_agrd's SAVEd iso_flag
  bool check_finite = false;          // reject host-staged FP32 inputs holding NaN or Inf
  size_t alloc_limit = 0;             // device bytes this context may allocate (0: no limit)
  size_t alloc_used = 0;              // device bytes allocated so far (never decremented)
  // scratch for the drop-in routines, grown on demand
  float* guard_list = nullptr;
  size_t guard_cap = 0;    // entries
  int cg_hint = 0;                    // iterations of the last converged CG solve (graph-replayed)
  int cg_hint_plain = 0;              // the same for solves issued as plain launches
  int cg_maxit = 0;                   // iteration cap of every solve (0: the reference's 10 npts)
  unsigned* words = nullptr;          // [0] list count, [1..5] maxima, [8..13] set_speed_agrd results, [16..27] GuardArgs::fold
  unsigned* host_words = nullptr;     // pinned
  g3m3::CgState* cg = nullptr;
  g3m3::CgState* host_cg = nullptr;   // pinned
  float* cgvec = nullptr;
  size_t cgvec_cells = 0;
  g3m3::CgGraphs cg_graphs;           // solver iterations as replayed graphs
};

namespace g3m3 {

int set_err(g3m3_ctx* c, int code, const char* fmt, ...);
int cuda_check(g3m3_ctx* c, cudaError_t e, const char* what);

// Device address for an array argument of `bytes` bytes: device and managed
// pointers pass through; a host array gets (or reuses) its mirror.
void* resolve(g3m3_ctx* c, const void* p, size_t bytes, int* status, bool floats = false);

// cudaMalloc charged to the context's allocation budget (g3m3_ctx_set_alloc_limit):
// over the budget it fails as cudaMalloc does when the device is full.
cudaError_t dev_alloc(g3m3_ctx* c, void** p, size_t bytes);

// Host FP32 data free of NaN and Inf (always true while checks are off).
bool finite_ok(const g3m3_ctx* c, const float* p, size_t n);

// Small host copies of parameter arrays (grd_*, xspac) that may live on
// either side.
bool host_floats(g3m3_ctx* c, const float* p, int n, float* out);
int host_ints(g3m3_ctx* c, const int* p, int n, int* out);

int ensure_guard_scratch(g3m3_ctx* c, size_t cells);
int ensure_cg_scratch(g3m3_ctx* c, size_t cells);

}  // namespace g3m3

#define G3M3_CUDA(ctx, call)                                  \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return g3m3::cuda_check(ctx, e_, #call); \
  } while (0)
