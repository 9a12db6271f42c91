// k_divb.cu -- div B cleaning: divB_correct (sub_divB_correct.f90:25-175)
// with the conjugate-gradient normal-equation solver sparse_solver
// (sub_sparse_solver.f90:19-159) and its banded product banded_tpose
// (sub_banded_tpose.f90:6-33).
//
// The 7-band matrix of the reference is the 7-point Laplacian with zero
// Dirichlet values outside the box; it is applied matrix-free, adding the
// bands in the reference's band order (k+1, j+1, i+1, diagonal, i-1, j-1,
// k-1).  Vectors stay FP32 as in the reference; every dot product and the
// residual norm accumulate the FP32 products in FP64 (warp shuffle, block
// reduction, one FP64 atomic per block).  The iteration control of one CG
// step is taken on the device, so the host only polls a status word once
// per chunk of iterations; no kernel waits on another.
#include "divb.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

constexpr int TPB = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;   // valid in thread 0
}

__device__ __forceinline__ float amul(const float* __restrict__ x, const Dims& d, size_t c, int i, int j, int k) {
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  float r = 0.0f;
  if (k < d.nz) r = r + __ldg(x + c + sz);
  if (j < d.ny) r = r + __ldg(x + c + sy);
  if (i < d.nx) r = r + __ldg(x + c + 1);
  r = r + -6.0f * __ldg(x + c);
  if (i > 1) r = r + __ldg(x + c - 1);
  if (j > 1) r = r + __ldg(x + c - sy);
  if (k > 1) r = r + __ldg(x + c - sz);
  return r;
}

// the solver's matrix product (banded_tpose, sub_banded_tpose.f90:20-30)
__device__ __forceinline__ float op(const DivbArgs& a, const float* __restrict__ x, size_t c, int i, int j, int k) {
  if (a.band == nullptr) return amul(x, a.d, c, i, j, k);
  const long long n = (long long)a.d.cells();
  float r = 0.0f;
  for (int b = 0; b < a.nbands; b++) {
    const long long ii = (long long)c + a.pos[b];
    if (ii >= 0 && ii < n) r = r + __ldg(a.band + (size_t)b + (size_t)a.nbands * (size_t)ii) * __ldg(x + ii);
  }
  return r;
}

// grid indices of cell c (a box holds fewer than 2^31 cells: 32-bit
// division, far cheaper than the 64-bit one)
__device__ __forceinline__ void ijk(size_t c, const Dims& d, int& i, int& j, int& k) {
  const unsigned cu = (unsigned)c, nx = (unsigned)d.nx, ny = (unsigned)d.ny;
  const unsigned r = cu / nx;
  i = (int)(cu - r * nx) + 1;
  const unsigned q = r / ny;
  j = (int)(r - q * ny) + 1;
  k = (int)q + 1;
}

#define GRID_LOOP(c, n) \
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < (n); c += (size_t)gridDim.x * blockDim.x)

// divB = div(b)/(2 rx) on the interior, 0 elsewhere; x = 0; xi = A x - b;
// rsq = |xi|^2, bsq = |b|^2  (:88-141, sparse_solver :61-71)
__global__ void __launch_bounds__(TPB) k_cg_init(DivbArgs a) {
  __shared__ double sh[TPB / 32];
  const Dims d = a.d;
  const size_t n = d.cells();
  double bsq = 0.0, rsq = 0.0;
  const float twor = 2.0f * a.rx;
  GRID_LOOP(c, n) {
    int i, j, k;
    ijk(c, d, i, j, k);
    float b = 0.0f;
    if (i > 1 && j > 1 && k > 1 && i < d.nx && j < d.ny && k < d.nz) {
      const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
      b = ((__ldg(a.bx + c + 1) - __ldg(a.bx + c - 1)) + (__ldg(a.by + c + sy) - __ldg(a.by + c - sy))
           + (__ldg(a.bz + c + sz) - __ldg(a.bz + c - sz))) / twor;
    }
    a.rhs[c] = b;
    a.x[c] = 0.0f;
    const float xi = 0.0f - b;   // A*0 - b
    a.xi[c] = xi;
    bsq += (double)(b * b);
    rsq += (double)(xi * xi);
  }
  bsq = block_sum(bsq, sh);
  rsq = block_sum(rsq, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&a.st->bsq, bsq);
    atomicAdd(&a.st->rsq, rsq);
  }
}

// caller's iterate and right-hand side: xi = A x - b, bsq = |b|^2,
// rsq = |xi|^2  (sub_sparse_solver.f90:61-71)
__global__ void __launch_bounds__(TPB) k_cg_init_given(DivbArgs a) {
  __shared__ double sh[TPB / 32];
  const Dims d = a.d;
  double bsq = 0.0, rsq = 0.0;
  GRID_LOOP(c, d.cells()) {
    int i, j, k;
    ijk(c, d, i, j, k);
    const float b = __ldg(a.rhs + c);
    const float xi = op(a, a.x, c, i, j, k) - b;
    a.xi[c] = xi;
    bsq += (double)(b * b);
    rsq += (double)(xi * xi);
  }
  bsq = block_sum(bsq, sh);
  rsq = block_sum(rsq, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&a.st->bsq, bsq);
    atomicAdd(&a.st->rsq, rsq);
  }
}

// g = -A xi ; h = g   (:73-75); also used after a restart
__global__ void __launch_bounds__(TPB) k_cg_grad(DivbArgs a) {
  const Dims d = a.d;
  GRID_LOOP(c, d.cells()) {
    int i, j, k;
    ijk(c, d, i, j, k);
    const float g = -op(a, a.xi, c, i, j, k);
    a.g[c] = g;
    a.h[c] = g;
  }
}

// restart from the restored iterate: xi = A x - b, rsq = |xi|^2
__global__ void __launch_bounds__(TPB) k_cg_resid(DivbArgs a) {
  __shared__ double sh[TPB / 32];
  const Dims d = a.d;
  double rsq = 0.0;
  GRID_LOOP(c, d.cells()) {
    int i, j, k;
    ijk(c, d, i, j, k);
    const float xi = op(a, a.x, c, i, j, k) - __ldg(a.rhs + c);
    a.xi[c] = xi;
    rsq += (double)(xi * xi);
  }
  rsq = block_sum(rsq, sh);
  if (threadIdx.x == 0) atomicAdd(&a.st->rsq, rsq);
}

// (:82-92) xi = A h ; anum = g.h ; aden = |xi|^2
__global__ void __launch_bounds__(TPB) k_cg_a(DivbArgs a) {
  if (a.st->status != CG_RUNNING) return;
  __shared__ double sh[TPB / 32];
  const Dims d = a.d;
  double an = 0.0, ad = 0.0;
  GRID_LOOP(c, d.cells()) {
    int i, j, k;
    ijk(c, d, i, j, k);
    const float xi = op(a, a.h, c, i, j, k);
    a.xi[c] = xi;
    an += (double)(__ldg(a.g + c) * __ldg(a.h + c));
    ad += (double)(xi * xi);
  }
  an = block_sum(an, sh);
  ad = block_sum(ad, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&a.st->anum, an);
    atomicAdd(&a.st->aden, ad);
  }
}

// (:95-99) save x, x = x + alpha h
__global__ void __launch_bounds__(TPB) k_cg_b(DivbArgs a) {
  if (a.st->status != CG_RUNNING) return;
  const float alpha = (float)(a.st->anum / a.st->aden);
  GRID_LOOP(c, a.d.cells()) {
    const float x = a.x[c];
    a.xs[c] = x;
    a.x[c] = x + alpha * __ldg(a.h + c);
  }
}

// (:101-107) xj = A x - b ; r2 = |xj|^2
__global__ void __launch_bounds__(TPB) k_cg_c(DivbArgs a) {
  if (a.st->status != CG_RUNNING) return;
  __shared__ double sh[TPB / 32];
  const Dims d = a.d;
  double r2 = 0.0;
  GRID_LOOP(c, d.cells()) {
    int i, j, k;
    ijk(c, d, i, j, k);
    const float xj = op(a, a.x, c, i, j, k) - __ldg(a.rhs + c);
    a.xj[c] = xj;
    r2 += (double)(xj * xj);
  }
  r2 = block_sum(r2, sh);
  if (threadIdx.x == 0) atomicAdd(&a.st->r2, r2);
}

// (:111-133) convergence, stagnation and divergence tests
__global__ void k_cg_control(DivbArgs a) {
  CgState* s = a.st;
  if (s->status != CG_RUNNING) return;
  s->iters += 1;
  const double r2 = s->r2;
  if (r2 == s->rsq || r2 <= s->bsq * s->errlim2) {
    s->status = CG_CONVERGED;
  } else if (r2 > s->rsq) {
    s->status = CG_RESTART;            // the host restores x and restarts
  } else if (s->iters >= s->maxit) {
    s->status = CG_MAXIT;
  } else {
    s->rsq = r2;
  }
  s->r2_last = r2;
  s->anum = 0.0; s->aden = 0.0; s->r2 = 0.0;
}

// (:134-141) xi = A xj ; gg = |g|^2 ; dgg = (xi+g).xi
__global__ void __launch_bounds__(TPB) k_cg_e(DivbArgs a) {
  if (a.st->status != CG_RUNNING) return;
  __shared__ double sh[TPB / 32];
  const Dims d = a.d;
  double gg = 0.0, dgg = 0.0;
  GRID_LOOP(c, d.cells()) {
    int i, j, k;
    ijk(c, d, i, j, k);
    const float xi = op(a, a.xj, c, i, j, k);
    a.xi[c] = xi;
    const float g = __ldg(a.g + c);
    gg += (double)(g * g);
    dgg += (double)((xi + g) * xi);
  }
  gg = block_sum(gg, sh);
  dgg = block_sum(dgg, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&a.st->gg, gg);
    atomicAdd(&a.st->dgg, dgg);
  }
}

__global__ void k_cg_control2(DivbArgs a) {
  CgState* s = a.st;
  if (s->status != CG_RUNNING) return;
  if (s->gg == 0.0) {
    s->status = CG_CONVERGED;          // the reference's return at gg = 0 (:142)
  } else if (s->r2_last != s->r2_last) {
    // a NaN residual never passes a test again: the reference iterates on
    // to 10*npts with x already NaN; stop now with the same result and the
    // same not-converged status.  (An exactly divergence-free B gives NaN
    // from 0/0 with g = 0, and returns through the test above, as the
    // reference does after its first iteration.)
    s->status = CG_MAXIT;
  } else {
    s->gam = (float)(s->dgg / s->gg);
  }
  s->gg = 0.0; s->dgg = 0.0;
}

// (:147-151) g = -xi ; h = g + gam h
__global__ void __launch_bounds__(TPB) k_cg_f(DivbArgs a) {
  if (a.st->status != CG_RUNNING) return;
  const float gam = a.st->gam;
  GRID_LOOP(c, a.d.cells()) {
    const float g = -__ldg(a.xi + c);
    a.g[c] = g;
    a.h[c] = g + gam * a.h[c];
  }
}

__global__ void __launch_bounds__(TPB) k_cg_restore(DivbArgs a) {
  GRID_LOOP(c, a.d.cells()) a.x[c] = a.xs[c];
}

// (:147-172) poten = rx^2 x ; b -= grad(poten) on the interior
__global__ void __launch_bounds__(TPB) k_cg_apply(DivbArgs a) {
  const Dims d = a.d;
  const float scale = a.rx * a.rx;
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  GRID_LOOP(c, d.cells()) {
    int i, j, k;
    ijk(c, d, i, j, k);
    if (!(i > 1 && j > 1 && k > 1 && i < d.nx && j < d.ny && k < d.nz)) continue;
    auto P = [&](size_t q) { return scale * __ldg(a.x + q); };
    const float dbx = (P(c + 1) - P(c - 1)) / (2.0f * a.rx);
    const float dby = (P(c + sy) - P(c - sy)) / (2.0f * a.ry);
    const float dbz = (P(c + sz) - P(c - sz)) / (2.0f * a.rz);
    a.bx[c] = a.bx[c] - dbx;
    a.by[c] = a.by[c] - dby;
    a.bz[c] = a.bz[c] - dbz;
  }
}

unsigned cg_blocks(const Dims& d) {
  const size_t n = d.cells();
  size_t b = (n + TPB - 1) / TPB;
  if (b > 4 * (size_t)sm_count()) b = 4 * (size_t)sm_count();   // 4 blocks per SM: fewer FP64 atomics per dot product (timed against 2 and 8)
  return (unsigned)b;
}

}  // namespace

void divb_launch_init(const DivbArgs& a, cudaStream_t s) {
  const unsigned nb = cg_blocks(a.d);
  k_cg_init<<<nb, TPB, 0, s>>>(a);
  k_cg_grad<<<nb, TPB, 0, s>>>(a);
}

void divb_launch_init_given(const DivbArgs& a, cudaStream_t s) {
  const unsigned nb = cg_blocks(a.d);
  k_cg_init_given<<<nb, TPB, 0, s>>>(a);
  k_cg_grad<<<nb, TPB, 0, s>>>(a);
}

void divb_launch_restart(const DivbArgs& a, cudaStream_t s) {
  const unsigned nb = cg_blocks(a.d);
  k_cg_restore<<<nb, TPB, 0, s>>>(a);
  k_cg_resid<<<nb, TPB, 0, s>>>(a);
  k_cg_grad<<<nb, TPB, 0, s>>>(a);
}

void divb_launch_restore(const DivbArgs& a, cudaStream_t s) {
  k_cg_restore<<<cg_blocks(a.d), TPB, 0, s>>>(a);
}

void divb_launch_iterations(const DivbArgs& a, int n, cudaStream_t s) {
  const unsigned nb = cg_blocks(a.d);
  for (int it = 0; it < n; it++) {
    k_cg_a<<<nb, TPB, 0, s>>>(a);
    k_cg_b<<<nb, TPB, 0, s>>>(a);
    k_cg_c<<<nb, TPB, 0, s>>>(a);
    k_cg_control<<<1, 1, 0, s>>>(a);
    k_cg_e<<<nb, TPB, 0, s>>>(a);
    k_cg_control2<<<1, 1, 0, s>>>(a);
    k_cg_f<<<nb, TPB, 0, s>>>(a);
  }
}

void divb_launch_apply(const DivbArgs& a, cudaStream_t s) {
  k_cg_apply<<<cg_blocks(a.d), TPB, 0, s>>>(a);
}

namespace {
// the fields of an argument block that the iteration kernels read (not the
// field arrays bx, by, bz: only the set-up and the correction touch them,
// and the engine's buffer roles alternate which arrays those are)
std::string graph_key(const DivbArgs& a, int m) {
  const void* ptrs[8] = {a.rhs, a.x, a.xs, a.g, a.h, a.xi, a.xj, a.st};
  std::string k(reinterpret_cast<const char*>(ptrs), sizeof ptrs);
  const int ints[5] = {a.d.nx, a.d.ny, a.d.nz, a.nbands, m};
  k.append(reinterpret_cast<const char*>(ints), sizeof ints);
  const float fl[3] = {a.rx, a.ry, a.rz};
  k.append(reinterpret_cast<const char*>(fl), sizeof fl);
  k.append(reinterpret_cast<const char*>(&a.band), sizeof a.band);
  if (a.band && a.nbands > 0) k.append(reinterpret_cast<const char*>(a.pos), sizeof(int) * (size_t)a.nbands);
  return k;
}
constexpr int kMaxGraphIters = 64;
constexpr size_t kMaxGraphs = 2048;  // a bound on the cache (16 members x 5 boxes x 7 lengths fit)
}  // namespace

cudaGraphExec_t CgGraphs::get(const DivbArgs& a, int m, cudaStream_t s) {
  const std::string key = graph_key(a, m);
  auto it = execs_.find(key);
  if (it != execs_.end()) return it->second;
  if (execs_.size() >= kMaxGraphs) clear();
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  DivbArgs ai = a;
  ai.bx = ai.by = ai.bz = nullptr;   // never read by the iteration kernels
  divb_launch_iterations(ai, m, s);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  cudaGraphExec_t ex = nullptr;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  execs_.emplace(key, ex);
  return ex;
}

cudaError_t CgGraphs::iterations(const DivbArgs& a, int n, cudaStream_t s) {
  // an argument block seen for the first time gets all seven lengths, so
  // later chunk lengths never capture in the middle of a run
  if (!execs_.count(graph_key(a, kMaxGraphIters)))
    for (int m = kMaxGraphIters; m >= 1; m >>= 1) get(a, m, s);
  while (n > 0) {
    int m = kMaxGraphIters;
    while (m > n) m >>= 1;
    cudaGraphExec_t ex = get(a, m, s);
    if (ex) {
      const cudaError_t e = cudaGraphLaunch(ex, s);
      if (e != cudaSuccess) return e;
    } else {
      divb_launch_iterations(a, m, s);
    }
    n -= m;
  }
  return cudaGetLastError();
}

void CgGraphs::clear() {
  for (auto& kv : execs_) cudaGraphExecDestroy(kv.second);
  execs_.clear();
}

}  // namespace g3m3
