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
  };
  std::unordered_map<const void*, Mirror> mirrors;
  std::string err;
  float iso_flag = 1.0f;   // set_speed_agrd's SAVEd iso_flag
  // scratch for the drop-in routines, grown on demand
  float* guard_list = nullptr;
  size_t guard_cap = 0;    // entries
  int cg_hint = 0;                    // iterations of the last converged CG solve
  unsigned* words = nullptr;          // [0] list count, [1..5] maxima
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
void* resolve(g3m3_ctx* c, const void* p, size_t bytes, int* status);

// Small host copies of parameter arrays (grd_*, xspac) that may live on
// either side.
bool host_floats(g3m3_ctx* c, const float* p, int n, float* out);

int ensure_guard_scratch(g3m3_ctx* c, size_t cells);
int ensure_cg_scratch(g3m3_ctx* c, size_t cells);

}  // namespace g3m3

#define G3M3_CUDA(ctx, call)                                  \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return g3m3::cuda_check(ctx, e_, #call); \
  } while (0)
