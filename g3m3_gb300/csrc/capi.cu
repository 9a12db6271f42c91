// capi.cu -- the drop-in C ABI (include/g3m3.h): context, host-array
// mirrors and one entry point per reference routine.
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <vector>

#include "ctx.cuh"

namespace g3m3 {

void launch_sample(const SampleArgs& a, cudaStream_t s);
void launch_bande_interior(const BandEArgs& a, cudaStream_t s);

int set_err(g3m3_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int cuda_check(g3m3_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return G3M3_OK;
  return set_err(c, e == cudaErrorMemoryAllocation ? G3M3_ERR_ALLOC : G3M3_ERR_CUDA, "%s: %s", what,
                 cudaGetErrorString(e));
}

static bool is_device_ptr(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

cudaError_t dev_alloc(g3m3_ctx* c, void** p, size_t bytes) {
  *p = nullptr;
  if (c && c->alloc_limit && c->alloc_used + bytes > c->alloc_limit) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess && c) c->alloc_used += bytes;
  return e;
}

bool finite_ok(const g3m3_ctx* c, const float* p, size_t n) {
  if (!c || !c->check_finite || !p) return true;
  for (size_t i = 0; i < n; i++)
    if (!std::isfinite(p[i])) return false;
  return true;
}

void* resolve(g3m3_ctx* c, const void* p, size_t bytes, int* status, bool floats) {
  if (*status) return nullptr;
  if (!p) {
    *status = set_err(c, G3M3_ERR_ARG, "null array argument");
    return nullptr;
  }
  if (is_device_ptr(p)) return const_cast<void*>(p);
  auto it = c->mirrors.find(p);
  if (it != c->mirrors.end()) {
    if (it->second.bytes < bytes) {
      *status = set_err(c, G3M3_ERR_ARG, "host array %p was mirrored with %zu bytes, call needs %zu", p,
                        it->second.bytes, bytes);
      return nullptr;
    }
    return it->second.dev;
  }
  if (floats && !finite_ok(c, static_cast<const float*>(p), bytes / sizeof(float))) {
    *status = set_err(c, G3M3_ERR_NONFINITE, "host array %p holds NaN or Inf", p);
    return nullptr;
  }
  void* d = nullptr;
  cudaError_t e = dev_alloc(c, (void**)&d, bytes);
  if (e != cudaSuccess) {
    *status = cuda_check(c, e, "cudaMalloc(mirror)");
    return nullptr;
  }
  e = cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    *status = cuda_check(c, e, "cudaMemcpyAsync(mirror upload)");
    return nullptr;
  }
  c->mirrors[p] = {d, bytes, floats};
  return d;
}

// Small host copies of integer parameter arrays (the band layout), read on
// the context's stream so that they follow the caller's earlier work there.
int host_ints(g3m3_ctx* c, const int* p, int n, int* out) {
  if (!p) return set_err(c, G3M3_ERR_ARG, "null integer array");
  if (is_device_ptr(p)) {
    G3M3_CUDA(c, cudaMemcpyAsync(out, p, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    G3M3_CUDA(c, cudaStreamSynchronize(c->stream));
    return G3M3_OK;
  }
  std::memcpy(out, p, n * sizeof(int));
  return G3M3_OK;
}

bool host_floats(g3m3_ctx* c, const float* p, int n, float* out) {
  if (!p) return false;
  if (is_device_ptr(p)) {
    if (cudaMemcpyAsync(out, p, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return false;
    return cudaStreamSynchronize(c->stream) == cudaSuccess;
  }
  auto it = c->mirrors.find(p);
  if (it != c->mirrors.end()) {   // the library may have written the mirror
    if (cudaMemcpyAsync(out, it->second.dev, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
      return false;
    return cudaStreamSynchronize(c->stream) == cudaSuccess;
  }
  std::memcpy(out, p, n * sizeof(float));
  return true;
}

int ensure_guard_scratch(g3m3_ctx* c, size_t cells) {
  const size_t need = 3 * cells;
  if (!c->words) {
    G3M3_CUDA(c, dev_alloc(c, (void**)&c->words, 32 * sizeof(unsigned)));
    G3M3_CUDA(c, cudaMallocHost(&c->host_words, 16 * sizeof(unsigned)));
  }
  if (c->guard_cap >= need) return G3M3_OK;
  if (c->guard_list) cudaFree(c->guard_list);
  c->guard_list = nullptr;
  c->guard_cap = 0;
  G3M3_CUDA(c, dev_alloc(c, (void**)&c->guard_list, need * 11 * sizeof(float)));
  c->guard_cap = need;
  return G3M3_OK;
}

int ensure_words(g3m3_ctx* c) {
  if (!c->words) {
    G3M3_CUDA(c, dev_alloc(c, (void**)&c->words, 32 * sizeof(unsigned)));
    G3M3_CUDA(c, cudaMallocHost(&c->host_words, 16 * sizeof(unsigned)));
  }
  return G3M3_OK;
}

int ensure_cg_scratch(g3m3_ctx* c, size_t cells) {
  if (!c->cg) {
    G3M3_CUDA(c, dev_alloc(c, (void**)&c->cg, sizeof(CgState)));
    G3M3_CUDA(c, cudaMallocHost(&c->host_cg, sizeof(CgState)));
  }
  if (c->cgvec_cells >= cells) return G3M3_OK;
  if (c->cgvec) cudaFree(c->cgvec);
  c->cgvec = nullptr;
  c->cgvec_cells = 0;
  G3M3_CUDA(c, dev_alloc(c, (void**)&c->cgvec, 7 * cells * sizeof(float)));
  c->cgvec_cells = cells;
  return G3M3_OK;
}

// --------------------------------------------------------------------------
// Shared pieces of the drop-in routines and the engine
// --------------------------------------------------------------------------
// The CG loop of sparse_solver (sub_sparse_solver.f90:19-159) on a prepared
// argument block: initialise (from b = div B with x = 0, or from the
// caller's x and b), iterate in chunks with the control decided on the
// device, restart after a growing residual (the reference's recursive call,
// :112-125) until the SAVEd restart count reaches 3.
// One solve as a resumable object: cg_begin queues the initialisation and
// the first chunk of iterations with a read-back of the status word;
// cg_step waits for that read-back and queues what the status asks for
// (the next chunk, a restart, or nothing when the solve has ended), so a
// caller can keep several solves on separate streams in flight.
static cudaError_t launch_iterations(CgRun& r) {
  if (r.graphs) return r.graphs->iterations(r.a, r.chunk, r.s);
  divb_launch_iterations(r.a, r.chunk, r.s);
  return cudaSuccess;
}

int cg_begin(g3m3_ctx* c, CgRun& r, float errlim, bool given, int redos0, int hint) {
  const size_t n = r.a.d.cells();
  CgState init{};
  const float e2 = (float)n * (errlim * errlim);   // sub_sparse_solver.f90:53 in FP32
  init.errlim2 = (double)e2;
  init.status = CG_RUNNING;
  init.maxit = (int)((10L * (long)n) > 2000000000L ? 2000000000L : 10L * (long)n);   // :80
  if (c->cg_maxit > 0 && c->cg_maxit < init.maxit) init.maxit = c->cg_maxit;
  init.redos = redos0;
  *r.host_st = init;
  G3M3_CUDA(c, cudaMemcpyAsync(r.a.st, r.host_st, sizeof(CgState), cudaMemcpyHostToDevice, r.s));
  if (given) divb_launch_init_given(r.a, r.s);
  else divb_launch_init(r.a, r.s);
  // iterations run in chunks between polls of the device-held status; the
  // first chunk is the iteration count of an earlier solve of the same kind
  // (solves of one run converge alike), the later ones grow from 2, so few
  // iterations are launched past convergence
  r.chunk = hint > 0 ? hint : 8;
  r.first = true;
  r.status = CG_RUNNING;
  G3M3_CUDA(c, launch_iterations(r));
  G3M3_CUDA(c, cudaMemcpyAsync(r.host_st, r.a.st, sizeof(CgState), cudaMemcpyDeviceToHost, r.s));
  return G3M3_OK;
}

int cg_step(g3m3_ctx* c, CgRun& r, bool* done) {
  *done = false;
  G3M3_CUDA(c, cudaStreamSynchronize(r.s));
  r.status = r.host_st->status;
  if (r.status == CG_RUNNING) {
    r.chunk = r.first ? 2 : (r.chunk < 64 ? 2 * r.chunk : 64);
    r.first = false;
  } else if (r.status == CG_RESTART) {
    // the residual grew: restore the previous iterate (:118-121); after
    // three restarts give up (:125), else restart the solver from it
    if (r.host_st->redos >= 3) {
      divb_launch_restore(r.a, r.s);
      r.status = CG_GAVE_UP;
      *done = true;
      G3M3_CUDA(c, cudaGetLastError());
      return G3M3_OK;
    }
    CgState& h = *r.host_st;
    h.redos += 1;
    h.status = CG_RUNNING;
    h.rsq = 0.0; h.anum = 0.0; h.aden = 0.0; h.r2 = 0.0; h.gg = 0.0; h.dgg = 0.0;
    G3M3_CUDA(c, cudaMemcpyAsync(r.a.st, r.host_st, sizeof(CgState), cudaMemcpyHostToDevice, r.s));
    divb_launch_restart(r.a, r.s);
  } else {
    *done = true;
    G3M3_CUDA(c, cudaGetLastError());
    return G3M3_OK;
  }
  G3M3_CUDA(c, launch_iterations(r));
  G3M3_CUDA(c, cudaMemcpyAsync(r.host_st, r.a.st, sizeof(CgState), cudaMemcpyDeviceToHost, r.s));
  return G3M3_OK;
}

// The CG loop of sparse_solver (sub_sparse_solver.f90:19-159) on a prepared
// argument block: initialise (from b = div B with x = 0, or from the
// caller's x and b), iterate in chunks with the control decided on the
// device, restart after a growing residual (the reference's recursive call,
// :112-125) until the SAVEd restart count reaches 3.
int run_cg(g3m3_ctx* c, const DivbArgs& a, float errlim, bool given, int redos0, CgState* host_st,
           cudaStream_t s, int* iters_out, float* residual2_out, int* status_out, CgGraphs* graphs = nullptr) {
  CgRun r;
  r.a = a; r.host_st = host_st; r.s = s; r.graphs = graphs;
  // replayed graphs make a long first chunk cheap to issue; plain launches
  // (the no-allocation entry) keep their own hint, capped, so that a hint
  // from a larger box cannot queue thousands of launches before the first poll
  int& hint = graphs ? c->cg_hint : c->cg_hint_plain;
  int rc = cg_begin(c, r, errlim, given, redos0, graphs ? hint : (hint < 64 ? hint : 64));
  bool done = false;
  while (rc == G3M3_OK && !done) rc = cg_step(c, r, &done);
  if (rc) return rc;
  if (iters_out) *iters_out = host_st->iters;
  if (r.status == CG_CONVERGED && host_st->iters > 0 && host_st->iters <= 4096) hint = host_st->iters;
  if (residual2_out) *residual2_out = (float)host_st->r2_last;
  if (status_out) *status_out = r.status;
  return G3M3_OK;
}

// div B projection of one box.  With graphs (the context's cache), the
// solver's iterations are replayed graphs; without (the no-allocation entry,
// which must not create any), plain launches.
int run_divb_with(g3m3_ctx* c, float* bx, float* by, float* bz, const Dims& d, float rx, float errlim,
                  CgState* st, CgState* host_st, float* vec, cudaStream_t s, int* iters_out, CgGraphs* graphs) {
  DivbArgs a{};
  a.bx = bx; a.by = by; a.bz = bz;
  const size_t n = d.cells();
  a.rhs = vec; a.x = vec + n; a.xs = vec + 2 * n; a.g = vec + 3 * n; a.h = vec + 4 * n;
  a.xi = vec + 5 * n; a.xj = vec + 6 * n;
  a.st = st; a.d = d; a.rx = rx; a.ry = rx; a.rz = rx;
  int status = CG_RUNNING;
  int rc = run_cg(c, a, errlim, false, 1, host_st, s, iters_out, nullptr, &status, graphs);
  if (rc) return rc;
  divb_launch_apply(a, s);
  G3M3_CUDA(c, cudaGetLastError());
  if (status == CG_MAXIT) return set_err(c, G3M3_ERR_NOCONV, "div B solver: too many iterations (%d)", host_st->iters);
  return G3M3_OK;
}

int run_divb(g3m3_ctx* c, float* bx, float* by, float* bz, const Dims& d, float rx, float errlim,
             CgState* st, CgState* host_st, float* vec, cudaStream_t s, int* iters_out) {
  return run_divb_with(c, bx, by, bz, d, rx, errlim, st, host_st, vec, s, iters_out, nullptr);
}

}  // namespace g3m3

using namespace g3m3;

namespace {

struct Res {
  g3m3_ctx* c;
  int st = 0;
  explicit Res(g3m3_ctx* cc) : c(cc) {}
  float* f(const float* p, size_t n) { return static_cast<float*>(resolve(c, p, n * sizeof(float), &st, true)); }
  int* i(const int* p, size_t n) { return static_cast<int*>(resolve(c, p, n * sizeof(int), &st)); }
};

int check_dims(g3m3_ctx* c, int nx, int ny, int nz, int n_grids, int box) {
  if (!c) return G3M3_ERR_ARG;
  if (nx < 4 || ny < 4 || nz < 4 || n_grids < 1 || box < 1 || box > n_grids)
    return set_err(c, G3M3_ERR_ARG, "bad dimensions nx=%d ny=%d nz=%d n_grids=%d box=%d", nx, ny, nz, n_grids, box);
  return G3M3_OK;
}

int finish(g3m3_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_check(c, e, what);
  return G3M3_OK;
}

inline size_t off(int nx, int ny, int nz, int box) { return (size_t)(box - 1) * nx * ny * nz; }

__global__ void k_velocity(const float* __restrict__ rho, const float* __restrict__ px, const float* __restrict__ py,
                           const float* __restrict__ pz, float* vx, float* vy, float* vz, float floor_,
                           size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const float r = amax1(rho[c], floor_);
    vx[c] = px[c] / r;
    vy[c] = py[c] / r;
    vz[c] = pz[c] / r;
  }
}

// the six results of set_speed_agrd; a word that met a NaN takes its
// refolded value (the maximum after the last NaN, or NaN)
__global__ void k_fastest(const unsigned* w, const unsigned* fold, float* out6) {
  float m[5];
  for (int q = 0; q < 5; q++) {
    unsigned bits = w[1 + q];
    if ((fold[0] >> q) & 1u) bits = ((fold[11] >> q) & 1u) ? fold[6 + q] : 0x7fc00000u;
    m[q] = __uint_as_float(bits);
  }
  const float px = m[0], py = m[1], pz = m[2], cs = m[3], al = m[4];
  out6[0] = px; out6[1] = py; out6[2] = pz; out6[3] = cs; out6[4] = al;
  out6[5] = amax1(0.0f, sqrtf(px * px + py * py + pz * pz + cs * cs + al * al));
}

}  // namespace

extern "C" {

const char* g3m3_version(void) {
  return "g3m3_gpu sm_103a; FP32 state, IEEE div/sqrt, no FMA contraction; FP64 CG reductions";
}

void* g3m3_ctx_stream(g3m3_ctx* c) { return c ? (void*)c->stream : nullptr; }

int g3m3_ctx_create(g3m3_ctx** out, int device) {
  if (!out) return G3M3_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) {
    cudaGetLastError();
    return G3M3_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) return G3M3_ERR_CUDA;
  // kernels that stage more than 48 KB get their shared-memory limit on
  // this device now, before any stream capture
  if (prepare_device_kernels() != cudaSuccess) {
    cudaGetLastError();
    return G3M3_ERR_CUDA;
  }
  g3m3_ctx* c = new g3m3_ctx();
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return G3M3_ERR_CUDA;
  }
  *out = c;
  return G3M3_OK;
}

int g3m3_ctx_destroy(g3m3_ctx* c) {
  if (!c) return G3M3_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& kv : c->mirrors) cudaFree(kv.second.dev);
  if (c->guard_list) cudaFree(c->guard_list);
  if (c->words) cudaFree(c->words);
  if (c->host_words) cudaFreeHost(c->host_words);
  if (c->cg) cudaFree(c->cg);
  if (c->host_cg) cudaFreeHost(c->host_cg);
  if (c->cgvec) cudaFree(c->cgvec);
  cudaStreamDestroy(c->stream);
  delete c;
  return G3M3_OK;
}

const char* g3m3_last_error(g3m3_ctx* c) { return c ? c->err.c_str() : "no context"; }

int g3m3_ctx_set_cg_maxit(g3m3_ctx* c, int maxit) {
  if (!c || maxit < 0) return G3M3_ERR_ARG;
  c->cg_maxit = maxit;
  return G3M3_OK;
}

int g3m3_ctx_set_finite_check(g3m3_ctx* c, int on) {
  if (!c) return G3M3_ERR_ARG;
  c->check_finite = on != 0;
  return G3M3_OK;
}

int g3m3_ctx_set_alloc_limit(g3m3_ctx* c, size_t bytes) {
  if (!c) return G3M3_ERR_ARG;
  c->alloc_limit = bytes;
  return G3M3_OK;
}

size_t g3m3_ctx_allocated(g3m3_ctx* c) { return c ? c->alloc_used : 0; }

int g3m3_synchronize(g3m3_ctx* c) {
  if (!c) return G3M3_ERR_ARG;
  G3M3_CUDA(c, cudaStreamSynchronize(c->stream));
  return G3M3_OK;
}

int g3m3_sync_to_host(g3m3_ctx* c, void* p) {
  if (!c || !p) return G3M3_ERR_ARG;
  auto it = c->mirrors.find(p);
  if (it == c->mirrors.end()) return G3M3_OK;
  G3M3_CUDA(c, cudaMemcpyAsync(p, it->second.dev, it->second.bytes, cudaMemcpyDeviceToHost, c->stream));
  G3M3_CUDA(c, cudaStreamSynchronize(c->stream));
  return G3M3_OK;
}

int g3m3_sync_to_device(g3m3_ctx* c, const void* p) {
  if (!c || !p) return G3M3_ERR_ARG;
  auto it = c->mirrors.find(p);
  if (it == c->mirrors.end()) return G3M3_OK;
  if (it->second.floats && !finite_ok(c, static_cast<const float*>(p), it->second.bytes / sizeof(float)))
    return set_err(c, G3M3_ERR_NONFINITE, "host array %p holds NaN or Inf", p);
  G3M3_CUDA(c, cudaMemcpyAsync(it->second.dev, p, it->second.bytes, cudaMemcpyHostToDevice, c->stream));
  G3M3_CUDA(c, cudaStreamSynchronize(c->stream));
  return G3M3_OK;
}

int g3m3_release_mirrors(g3m3_ctx* c) {
  if (!c) return G3M3_ERR_ARG;
  G3M3_CUDA(c, cudaStreamSynchronize(c->stream));
  for (auto& kv : c->mirrors) cudaFree(kv.second.dev);
  c->mirrors.clear();
  return G3M3_OK;
}

int g3m3_push_ion(g3m3_ctx* ctx, float* qrho, float* qpresx, float* qpresy, float* qpresz, float* qpx,
                  float* qpy, float* qpz, const float* oldqrho, const float* oldqpresx, const float* oldqpresy,
                  const float* oldqpresz, const float* oldqpx, const float* oldqpy, const float* oldqpz,
                  const float* wrkqrho, const float* wrkqpresx, const float* wrkqpresy, const float* wrkqpresz,
                  const float* wrkqpx, const float* wrkqpy, const float* wrkqpz, float* qpresxy, float* qpresxz,
                  float* qpresyz, const float* oldqpresxy, const float* oldqpresxz, const float* oldqpresyz,
                  const float* wrkqpresxy, const float* wrkqpresxz, const float* wrkqpresyz, const float* bsx,
                  const float* bsy, const float* bsz, const float* btot, const float* efldx,
                  const float* efldy, const float* efldz, float rmassq, float* qvx, float* qvy, float* qvz,
                  const float* tvx, const float* tvy, const float* tvz, float gamma, float gamma1, int nx,
                  int ny, int nz, int n_grids, int box, float delt, float grav, float re_equiv, float reynolds,
                  const float* grd_xmin, const float* grd_xmax, const float* grd_ymin, const float* grd_ymax,
                  const float* grd_zmin, const float* grd_zmax, int isotropic) {
  (void)gamma; (void)gamma1; (void)isotropic;
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  PushIonArgs a{};
  float* outs[10] = {qrho, qpx, qpy, qpz, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz};
  const float* olds[10] = {oldqrho, oldqpx, oldqpy, oldqpz, oldqpresx, oldqpresy, oldqpresz, oldqpresxy,
                           oldqpresxz, oldqpresyz};
  const float* srcs[10] = {wrkqrho, wrkqpx, wrkqpy, wrkqpz, wrkqpresx, wrkqpresy, wrkqpresz, wrkqpresxy,
                           wrkqpresxz, wrkqpresyz};
  for (int f = 0; f < 10; f++) {
    a.out[f] = r.f(outs[f], n4) + o;
    a.old[f] = r.f(olds[f], n4) + o;
    a.src[f] = r.f(srcs[f], n4) + o;
  }
  const float* bs[3] = {bsx, bsy, bsz};
  const float* ef[3] = {efldx, efldy, efldz};
  const float* tv[3] = {tvx, tvy, tvz};
  float* qv[3] = {qvx, qvy, qvz};
  float* dqv[3];
  for (int q = 0; q < 3; q++) {
    a.bs[q] = r.f(bs[q], n3);
    a.efld[q] = r.f(ef[q], n3);
    a.tv[q] = r.f(tv[q], n3);
    dqv[q] = r.f(qv[q], n3);
  }
  a.btot = r.f(btot, n3);
  if (r.st) return r.st;
  float g[6][G3M3_MAX_GRIDS];
  const float* gp[6] = {grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax};
  for (int q = 0; q < 6; q++)
    if (!host_floats(ctx, gp[q], n_grids, g[q])) return set_err(ctx, G3M3_ERR_ARG, "grid extents unreadable");
  a.d = Dims{nx, ny, nz};
  a.g.dx = (g[1][box - 1] - g[0][box - 1]) / (float)(nx - 1);
  a.g.dy = (g[3][box - 1] - g[2][box - 1]) / (float)(ny - 1);
  a.g.dz = (g[5][box - 1] - g[4][box - 1]) / (float)(nz - 1);
  a.g.xmin = g[0][box - 1]; a.g.ymin = g[2][box - 1]; a.g.zmin = g[4][box - 1];
  a.rmass = rmassq; a.grav = grav; a.re_equiv = re_equiv; a.reynolds = reynolds;
  a.delt = ScalarRef{delt, nullptr};
  a.boundary_from_old = 0;
  // the reference's velocity pre-pass output (sub_push_ion.f90:67-81)
  k_velocity<<<blocks_for(n3, 256), 256, 0, ctx->stream>>>(a.src[0], a.src[1], a.src[2], a.src[3], dqv[0], dqv[1],
                                                          dqv[2], 1.e-6f, n3);
  launch_push_ion(a, ctx->stream);
  return finish(ctx, "push_ion");
}

int g3m3_push_elec(g3m3_ctx* ctx, const float* wrkepres, const float* oldepres, float* epres, const float* evx,
                   const float* evy, const float* evz, float gamma, float gamma1, int nx, int ny, int nz,
                   int n_grids, int box, float delt, float rx, float ry, float rz) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  PushFieldArgs a{};
  a.wrkepres = r.f(wrkepres, n4) + o;
  a.oldepres = r.f(oldepres, n4) + o;
  a.epres = r.f(epres, n4) + o;
  a.ev[0] = r.f(evx, n3); a.ev[1] = r.f(evy, n3); a.ev[2] = r.f(evz, n3);
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.rx = rx; a.ry = ry; a.rz = rz; a.gamma = gamma; a.gamma1 = gamma1;
  a.delt = ScalarRef{delt, nullptr};
  a.do_elec = 1;
  launch_push_field(a, ctx->stream);
  return finish(ctx, "push_elec");
}

int g3m3_push_bfld(g3m3_ctx* ctx, float* bx, float* by, float* bz, const float* oldbx, const float* oldby,
                   const float* oldbz, const float* efldx, const float* efldy, const float* efldz, int nx, int ny,
                   int nz, int n_grids, int box, float delt, float rx, float ry, float rz) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  PushFieldArgs a{};
  a.b[0] = r.f(bx, n4) + o; a.b[1] = r.f(by, n4) + o; a.b[2] = r.f(bz, n4) + o;
  a.oldb[0] = r.f(oldbx, n4) + o; a.oldb[1] = r.f(oldby, n4) + o; a.oldb[2] = r.f(oldbz, n4) + o;
  a.efld[0] = r.f(efldx, n3); a.efld[1] = r.f(efldy, n3); a.efld[2] = r.f(efldz, n3);
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.rx = rx; a.ry = ry; a.rz = rz;
  a.delt = ScalarRef{delt, nullptr};
  a.do_bfld = 1;
  launch_push_field(a, ctx->stream);
  return finish(ctx, "push_bfld");
}

int g3m3_calcur(g3m3_ctx* ctx, const float* bx, const float* by, const float* bz, int nx, int ny, int nz,
                int n_grids, int box, float* curx, float* cury, float* curz, float rx, float ry, float rz) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  CurrentArgs a{};
  a.b[0] = r.f(bx, n4) + o; a.b[1] = r.f(by, n4) + o; a.b[2] = r.f(bz, n4) + o;
  a.cur[0] = r.f(curx, n3); a.cur[1] = r.f(cury, n3); a.cur[2] = r.f(curz, n3);
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.rx = rx; a.ry = ry; a.rz = rz;
  launch_current(a, ctx->stream);
  return finish(ctx, "calcur");
}

int g3m3_total_b(g3m3_ctx* ctx, const float* bx, const float* by, const float* bz, const float* bx0,
                 const float* by0, const float* bz0, int nx, int ny, int nz, int n_grids, int box,
                 float smallbit, float* bsx, float* bsy, float* bsz, float* btot) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  const float* b[3] = {r.f(bx, n4) + o, r.f(by, n4) + o, r.f(bz, n4) + o};
  const float* b0[3] = {r.f(bx0, n4) + o, r.f(by0, n4) + o, r.f(bz0, n4) + o};
  float* bs[3] = {r.f(bsx, n3), r.f(bsy, n3), r.f(bsz, n3)};
  float* bt = r.f(btot, n3);
  if (r.st) return r.st;
  launch_total_b(b, b0, bs, bt, smallbit, Dims{nx, ny, nz}, ctx->stream);
  return finish(ctx, "total_b");
}

static int evel_common(g3m3_ctx* ctx, const float* P[3][3], const float* R[3], const float* cur[3], float* ev[3],
                       float* tv[3], int nx, int ny, int nz, int n_grids, int box, const float m[3], float rey) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  EvelArgs a{};
  for (int sp = 0; sp < 3; sp++) {
    for (int q = 0; q < 3; q++) a.p[sp][q] = r.f(P[sp][q], n4) + o;
    a.rho[sp] = r.f(R[sp], n4) + o;
    a.rmass[sp] = m[sp];
  }
  for (int q = 0; q < 3; q++) {
    a.tv[q] = r.f(tv[q], n3);
    if (ev) {
      a.cur[q] = r.f(cur[q], n3);
      a.ev[q] = r.f(ev[q], n3);
    }
  }
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.reynolds = rey;
  launch_evel(a, ctx->stream);
  return finish(ctx, "fnd_evel");
}

int g3m3_fnd_evel(g3m3_ctx* ctx, const float* qpx, const float* qpy, const float* qpz, const float* qrho,
                  const float* hpx, const float* hpy, const float* hpz, const float* hrho, const float* opx,
                  const float* opy, const float* opz, const float* orho, const float* curx, const float* cury,
                  const float* curz, float* evx, float* evy, float* evz, float* tvx, float* tvy, float* tvz,
                  int nx, int ny, int nz, int n_grids, int box, float rmassq, float rmassh, float rmasso,
                  float reynolds) {
  const float* P[3][3] = {{qpx, qpy, qpz}, {hpx, hpy, hpz}, {opx, opy, opz}};
  const float* R[3] = {qrho, hrho, orho};
  const float* cur[3] = {curx, cury, curz};
  float* ev[3] = {evx, evy, evz};
  float* tv[3] = {tvx, tvy, tvz};
  const float m[3] = {rmassq, rmassh, rmasso};
  return evel_common(ctx, P, R, cur, ev, tv, nx, ny, nz, n_grids, box, m, reynolds);
}

int g3m3_fnd_vtot(g3m3_ctx* ctx, const float* qpx, const float* qpy, const float* qpz, const float* qrho,
                  const float* hpx, const float* hpy, const float* hpz, const float* hrho, const float* opx,
                  const float* opy, const float* opz, const float* orho, float* vx, float* vy, float* vz, int nx,
                  int ny, int nz, int n_grids, int box, float rmassq, float rmassh, float rmasso) {
  const float* P[3][3] = {{qpx, qpy, qpz}, {hpx, hpy, hpz}, {opx, opy, opz}};
  const float* R[3] = {qrho, hrho, orho};
  float* tv[3] = {vx, vy, vz};
  const float m[3] = {rmassq, rmassh, rmasso};
  return evel_common(ctx, P, R, nullptr, nullptr, tv, nx, ny, nz, n_grids, box, m, 1.0f);
}

int g3m3_bande(g3m3_ctx* ctx, float* efldx, float* efldy, float* efldz, const float* bsx, const float* bsy,
               const float* bsz, const float* curx, const float* cury, const float* curz, const float* evx,
               const float* evy, const float* evz, const float* btot, const float* epres, const float* qrho,
               const float* hrho, const float* orho, const float* rst, float resist, float reynolds, int nx,
               int ny, int nz, int n_grids, int box, float rmassq, float rmassh, float rmasso, const int* ijmid,
               const int* nummid, const int* ijzero, int mbndry, const int* numzero, int mmid, int mzero,
               float rx, float ry, float rz) {
  (void)btot;
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  BandEArgs a{};
  a.efld[0] = r.f(efldx, n3); a.efld[1] = r.f(efldy, n3); a.efld[2] = r.f(efldz, n3);
  a.bs[0] = r.f(bsx, n3); a.bs[1] = r.f(bsy, n3); a.bs[2] = r.f(bsz, n3);
  a.cur[0] = r.f(curx, n3); a.cur[1] = r.f(cury, n3); a.cur[2] = r.f(curz, n3);
  a.ev[0] = r.f(evx, n3); a.ev[1] = r.f(evy, n3); a.ev[2] = r.f(evz, n3);
  a.epres = r.f(epres, n4) + o;
  a.rho[0] = r.f(qrho, n4) + o; a.rho[1] = r.f(hrho, n4) + o; a.rho[2] = r.f(orho, n4) + o;
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.rmass[0] = rmassq; a.rmass[1] = rmassh; a.rmass[2] = rmasso;
  a.reynolds = reynolds; a.rx = rx; a.ry = ry; a.rz = rz;
  launch_bande_interior(a, ctx->stream);
  if (box <= mbndry && resist < 5000.0f) {
    int nm[G3M3_MAX_GRIDS * 4], nzr[G3M3_MAX_GRIDS * 4];
    if (mbndry > (int)(sizeof nm / sizeof nm[0])) return set_err(ctx, G3M3_ERR_ARG, "mbndry too large");
    // the counts are host integers in the reference; read them on the host
    // (device arrays on the context's stream, after the work queued on it)
    int st;
    if ((st = host_ints(ctx, nummid, mbndry, nm)) || (st = host_ints(ctx, numzero, mbndry, nzr))) return st;
    BandEListArgs l{};
    for (int q = 0; q < 3; q++) {
      l.efld[q] = a.efld[q];
      l.cur[q] = a.cur[q];
      l.rho[q] = a.rho[q];
      l.rmass[q] = a.rmass[q];
    }
    l.rst = r.f(rst, n3 * mbndry) + o;
    l.mbndry = mbndry; l.box = box; l.d = a.d;
    const int* lists[2] = {r.i(ijmid, (size_t)mbndry * 3 * mmid), r.i(ijzero, (size_t)mbndry * 3 * mzero)};
    if (r.st) return r.st;
    const int counts[2] = {nm[box - 1], nzr[box - 1]};
    const int caps[2] = {mmid, mzero};
    // a list naming a cell twice adds to it twice, in order: find those on the host
    const int* lp[2] = {ijmid, ijzero};
    std::vector<int> hl[2];
    for (int q = 0; q < 2; q++) {
      if (counts[q] < 0 || counts[q] > caps[q]) return set_err(ctx, G3M3_ERR_ARG, "list count out of range");
      hl[q].resize((size_t)mbndry * 3 * counts[q] + 1);
      if (counts[q] > 0 && (st = host_ints(ctx, lp[q], mbndry * 3 * counts[q], hl[q].data()))) return st;
    }
    const int* hp[3] = {nullptr, hl[0].data(), hl[1].data()};
    const int num3[3] = {0, counts[0], counts[1]};
    const InnerOrder order = inner_order(hp, num3, mbndry, box, a.d);
    for (int q = 0; q < 2; q++) {
      l.ij = lists[q];
      l.count = counts[q];
      l.serial = order.repeat[1 + q] ? 1 : 0;
      launch_bande_list(l, ctx->stream);   // the two lists run in order
    }
  }
  launch_bande_faces(a.efld, a.d, ctx->stream);
  return finish(ctx, "BandE");
}

int g3m3_fnd_pres(g3m3_ctx* ctx, const float* px, const float* py, const float* pz, const float* pxy,
                  const float* pxz, const float* pyz, float* p_para, float* p_perp, float* p_cross,
                  const float* vvx, const float* vvy, const float* vvz, const float* bxt, const float* byt,
                  const float* bzt, int nx, int ny, int nz, int n_grids, int box) {
  (void)pxy; (void)pxz; (void)pyz;
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  const float* pr[3] = {r.f(px, n4) + o, r.f(py, n4) + o, r.f(pz, n4) + o};
  float* pa = r.f(p_para, n4) + o;
  float* pp = r.f(p_perp, n4) + o;
  float* pc = r.f(p_cross, n4) + o;
  const float* v[3] = {r.f(vvx, n3), r.f(vvy, n3), r.f(vvz, n3)};
  const float* b[3] = {r.f(bxt, n3), r.f(byt, n3), r.f(bzt, n3)};
  if (r.st) return r.st;
  launch_fnd_pres(pr, pa, pp, pc, v, b, Dims{nx, ny, nz}, ctx->stream);
  return finish(ctx, "fnd_pres");
}

static int lap_common(g3m3_ctx* ctx, const float* const* in, float* const* out, const float* chi, int nf,
                      const float* vx, const float* vy, const float* vz, int nx, int ny, int nz, int n_grids,
                      int box, float delt) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  LapArgs a{};
  for (int f = 0; f < nf; f++) {
    a.in[f] = r.f(in[f], n4) + o;
    a.out[f] = r.f(out[f], n4) + o;
    a.chi[f] = chi[f];
  }
  a.nf = nf;
  a.v[0] = r.f(vx, n3); a.v[1] = r.f(vy, n3); a.v[2] = r.f(vz, n3);
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.delt = ScalarRef{delt, nullptr};
  launch_lap(a, ctx->stream);
  return finish(ctx, "lapidus");
}

int g3m3_lap_plasma(g3m3_ctx* ctx, const float* rho, const float* px, const float* py, const float* pz,
                    const float* presx, const float* presy, const float* presz, const float* presxy,
                    const float* presxz, const float* presyz, float* wrkrho, float* wrkpx, float* wrkpy,
                    float* wrkpz, float* wrkpresx, float* wrkpresy, float* wrkpresz, float* wrkpresxy,
                    float* wrkpresxz, float* wrkpresyz, const float* vx, const float* vy, const float* vz, int nx,
                    int ny, int nz, int n_grids, int box, float chirho, float chipxyz, float chierg, float delt,
                    int isotropic) {
  (void)chierg; (void)isotropic;
  const float* in[10] = {rho, px, py, pz, presx, presy, presz, presxy, presxz, presyz};
  float* out[10] = {wrkrho, wrkpx, wrkpy, wrkpz, wrkpresx, wrkpresy, wrkpresz, wrkpresxy, wrkpresxz, wrkpresyz};
  float chi[10];
  for (int f = 0; f < 10; f++) chi[f] = f == 0 ? chirho : chipxyz;
  return lap_common(ctx, in, out, chi, 10, vx, vy, vz, nx, ny, nz, n_grids, box, delt);
}

int g3m3_lap_elec(g3m3_ctx* ctx, const float* ppres, float* wrkppres, const float* vx, const float* vy,
                  const float* vz, int nx, int ny, int nz, int n_grids, int box, float chirho, float chipxyz,
                  float chierg, float delt) {
  (void)chirho; (void)chierg;
  const float* in[1] = {ppres};
  float* out[1] = {wrkppres};
  const float chi[1] = {chipxyz};
  return lap_common(ctx, in, out, chi, 1, vx, vy, vz, nx, ny, nz, n_grids, box, delt);
}

int g3m3_lap_bfld(g3m3_ctx* ctx, const float* bx, const float* by, const float* bz, float* wrkbx, float* wrkby,
                  float* wrkbz, const float* vx, const float* vy, const float* vz, int nx, int ny, int nz,
                  int n_grids, int box, float chirho, float chipxyz, float chierg, float delt) {
  (void)chirho; (void)chipxyz;
  const float* in[3] = {bx, by, bz};
  float* out[3] = {wrkbx, wrkby, wrkbz};
  const float chi[3] = {chierg, chierg, chierg};
  return lap_common(ctx, in, out, chi, 3, vx, vy, vz, nx, ny, nz, n_grids, box, delt);
}

int g3m3_fcsmooth(g3m3_ctx* ctx, float* px, const float* oldpx, const float* wrkpx, int nx, int ny, int nz,
                  int n_grids, int box, float chipx, float* tempx, float* tempy, float* tempz) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  FcsArgs a{};
  a.px[0] = r.f(px, n4) + o;
  a.old[0] = r.f(oldpx, n4) + o;
  a.wrk[0] = r.f(wrkpx, n4) + o;
  a.chi[0] = chipx;
  a.nf = 1;
  // tempx..tempz are the reference's work arrays; this implementation keeps
  // its intermediates in registers and leaves them untouched
  (void)tempx; (void)tempy; (void)tempz; (void)n3;
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  launch_fcsmooth(a, ctx->stream);
  return finish(ctx, "fcsmooth");
}

int g3m3_flux_correct(g3m3_ctx* ctx, float* const cur[G3M3_NFIELDS], const float* const wrk[G3M3_NFIELDS],
                      const float* const old[G3M3_NFIELDS], int nx, int ny, int nz, int n_grids, int box,
                      float difrho, float diferg) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  FcsArgs a{};
  for (int f = 0; f < G3M3_NFIELDS; f++) {
    a.px[f] = r.f(cur[f], n4) + o;
    a.old[f] = r.f(old[f], n4) + o;
    a.wrk[f] = r.f(wrk[f], n4) + o;
    a.chi[f] = f >= G3M3_F_BX ? diferg : difrho;
  }
  if (r.st) return r.st;
  a.nf = G3M3_NFIELDS;
  a.d = Dims{nx, ny, nz};
  launch_fcsmooth(a, ctx->stream);
  return finish(ctx, "flux_correct");
}

int g3m3_set_rho(g3m3_ctx* ctx, float* qrho, float* qpresx, float* qpresy, float* qpresz, float* qpresxy,
                 float* qpresxz, float* qpresyz, float rmassq, float* hrho, float* hpresx, float* hpresy,
                 float* hpresz, float* hpresxy, float* hpresxz, float* hpresyz, float rmassh, float* orho,
                 float* opresx, float* opresy, float* opresz, float* opresxy, float* opresxz, float* opresyz,
                 float rmasso, float* epres, int nx, int ny, int nz, int n_grids, int box, float o_conc) {
  (void)rmassq; (void)rmassh; (void)rmasso; (void)o_conc;
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  GuardArgs a{};
  float* sp[3][7] = {{qrho, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz},
                     {hrho, hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz},
                     {orho, opresx, opresy, opresz, opresxy, opresxz, opresyz}};
  const int slot[7] = {0, 4, 5, 6, 7, 8, 9};
  for (int q = 0; q < 3; q++)
    for (int m = 0; m < 7; m++) a.f[10 * q + slot[m]] = r.f(sp[q][m], n4) + o;
  // set_rho does not touch the momenta; point them at rho so loads are valid
  for (int q = 0; q < 3; q++)
    for (int m = 1; m <= 3; m++) a.f[10 * q + m] = a.f[10 * q];
  a.f[G3M3_F_EPRES] = r.f(epres, n4) + o;
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.do_set_rho = 1;
  a.do_speed = 0;
  launch_guards(a, ctx->stream);
  return finish(ctx, "set_rho");
}

int g3m3_set_speed_agrd(g3m3_ctx* ctx, int nx, int ny, int nz, int n_grids, int box, float rmassq, float rmassh,
                        float rmasso, int isotropic, float smallbit, float aniso_limit, float vlim, float qvlim,
                        float hvlim, float ovlim, float qclim, float hclim, float oclim, float cslim,
                        const float* bx, const float* by, const float* bz, const float* bx0, const float* by0,
                        const float* bz0, float* qrho, float* qpx, float* qpy, float* qpz, float* qpresx,
                        float* qpresy, float* qpresz, float* qpresxy, float* qpresxz, float* qpresyz, float* hrho,
                        float* hpx, float* hpy, float* hpz, float* hpresx, float* hpresy, float* hpresz,
                        float* hpresxy, float* hpresxz, float* hpresyz, float* orho, float* opx, float* opy,
                        float* opz, float* opresx, float* opresy, float* opresz, float* opresxy, float* opresxz,
                        float* opresyz, float* epres, float* btot, float* pxmax, float* pymax, float* pzmax,
                        float* csmax, float* alfmax, float* fastest) {
  (void)rmassq; (void)rmassh; (void)rmasso;
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  if ((s = ensure_guard_scratch(ctx, n3))) return s;
  Res r(ctx);
  GuardArgs a{};
  float* fl[30] = {qrho, qpx, qpy, qpz, qpresx, qpresy, qpresz, qpresxy, qpresxz, qpresyz,
                   hrho, hpx, hpy, hpz, hpresx, hpresy, hpresz, hpresxy, hpresxz, hpresyz,
                   orho, opx, opy, opz, opresx, opresy, opresz, opresxy, opresxz, opresyz};
  for (int f = 0; f < 30; f++) a.f[f] = r.f(fl[f], n4) + o;
  a.f[G3M3_F_EPRES] = r.f(epres, n4) + o;
  a.f[G3M3_F_BX] = r.f(bx, n4) + o; a.f[G3M3_F_BY] = r.f(by, n4) + o; a.f[G3M3_F_BZ] = r.f(bz, n4) + o;
  a.b0[0] = r.f(bx0, n4) + o; a.b0[1] = r.f(by0, n4) + o; a.b0[2] = r.f(bz0, n4) + o;
  a.btot = r.f(btot, n3);
  if (r.st) return r.st;
  if (isotropic) ctx->iso_flag = 0.0f;   // SAVEd (sub_set_speed_agrd.f90:68-75)
  a.d = Dims{nx, ny, nz};
  a.smallbit = smallbit; a.aniso_limit = aniso_limit; a.vlim = vlim;
  a.svlim[0] = qvlim; a.svlim[1] = hvlim; a.svlim[2] = ovlim;
  a.sclim[0] = qclim; a.sclim[1] = hclim; a.sclim[2] = oclim;
  a.cslim = cslim; a.iso_flag = ctx->iso_flag; a.isotropic = isotropic != 0;
  a.do_set_rho = 0; a.do_speed = 1;
  a.list = ctx->guard_list; a.list_cap = (unsigned)ctx->guard_cap;
  a.list_count = ctx->words; a.maxbits = ctx->words + 1; a.fold = ctx->words + 16;
  G3M3_CUDA(ctx, cudaMemsetAsync(ctx->words, 0, 32 * sizeof(unsigned), ctx->stream));
  launch_guards(a, ctx->stream);
  launch_guard_fold_species(a, ctx->stream);
  ScatterArgs sa{};
  for (int f = 0; f < G3M3_NFIELDS; f++) sa.f[f] = a.f[f];
  sa.list = a.list; sa.list_count = a.list_count; sa.list_cap = a.list_cap;
  launch_guard_scatter(sa, ctx->stream);
  launch_guard_fold_alf(a, ctx->stream);
  k_fastest<<<1, 1, 0, ctx->stream>>>(ctx->words, ctx->words + 16, reinterpret_cast<float*>(ctx->words + 8));
  G3M3_CUDA(ctx, cudaMemcpyAsync(ctx->host_words, ctx->words, 16 * sizeof(unsigned), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  G3M3_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const float* h6 = reinterpret_cast<const float*>(ctx->host_words + 8);
  if (ctx->host_words[0] > a.list_cap) return set_err(ctx, G3M3_ERR_STATE, "limiter list overflow");
  if (pxmax) *pxmax = h6[0];
  if (pymax) *pymax = h6[1];
  if (pzmax) *pzmax = h6[2];
  if (csmax) *csmax = h6[3];
  if (alfmax) *alfmax = h6[4];
  if (fastest) *fastest = h6[5];
  return finish(ctx, "set_speed_agrd");
}

int g3m3_store_array(g3m3_ctx* ctx, float* bx, const float* bx0, int nx, int ny, int nz, int n_grids, int box) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  float* d = r.f(bx, n4) + o;
  const float* src = r.f(bx0, n4) + o;
  if (r.st) return r.st;
  G3M3_CUDA(ctx, cudaMemcpyAsync(d, src, n3 * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
  return G3M3_OK;
}

int g3m3_bndry_outer(g3m3_ctx* ctx, float* const f[G3M3_NFIELDS], const float* bx0, const float* by0,
                     const float* bz0, const g3m3_params* p) {
  if (!ctx || !p) return G3M3_ERR_ARG;
  int s = check_dims(ctx, p->nx, p->ny, p->nz, p->n_grids, p->n_grids);
  if (s) return s;
  const size_t n3 = (size_t)p->nx * p->ny * p->nz, n4 = n3 * p->n_grids;
  const size_t o = off(p->nx, p->ny, p->nz, p->n_grids);
  Res r(ctx);
  OuterArgs a{};
  for (int q = 0; q < G3M3_NFIELDS; q++) a.f[q] = r.f(f[q], n4) + o;
  a.b0[0] = r.f(bx0, n4) + o; a.b0[1] = r.f(by0, n4) + o; a.b0[2] = r.f(bz0, n4) + o;
  if (r.st) return r.st;
  a.d = Dims{p->nx, p->ny, p->nz};
  a.rmassq = p->rmassq; a.rmassh = p->rmassh; a.rmasso = p->rmasso;
  a.srho = p->srho; a.rho_frac = p->rho_frac; a.o_conc = p->o_conc; a.spress = p->spress;
  a.spx = p->spx; a.spy = p->spy; a.spz = p->spz;
  a.sbx_wind = p->sbx_wind; a.sby_wind = p->sby_wind; a.sbz_wind = p->sbz_wind; a.ti_te = p->ti_te;
  launch_bndry_outer(a, ctx->stream);
  return finish(ctx, "bndry_outer");
}

int g3m3_bndry_inner(g3m3_ctx* ctx, float* const f[G3M3_NFIELDS], const float* parm_srf, const float* parm_mid,
                     const float* parm_zero, const int* ijsrf, const int* numsrf, const int* ijmid,
                     const int* nummid, const int* ijzero, const int* numzero, int msrf, int mmid, int mzero,
                     const g3m3_params* p) {
  if (!ctx || !p) return G3M3_ERR_ARG;
  const int mb = p->mbndry;
  int s = check_dims(ctx, p->nx, p->ny, p->nz, p->n_grids, mb);
  if (s) return s;
  const size_t n3 = (size_t)p->nx * p->ny * p->nz, n4 = n3 * p->n_grids, o = off(p->nx, p->ny, p->nz, mb);
  Res r(ctx);
  InnerArgs a{};
  for (int q = 0; q < G3M3_NFIELDS; q++) a.f[q] = r.f(f[q], n4) + o;
  a.ij[0] = r.i(ijsrf, (size_t)mb * 3 * msrf);
  a.ij[1] = r.i(ijmid, (size_t)mb * 3 * mmid);
  a.ij[2] = r.i(ijzero, (size_t)mb * 3 * mzero);
  a.parm[0] = r.f(parm_srf, (size_t)mb * 7 * msrf);
  a.parm[1] = r.f(parm_mid, (size_t)mb * 7 * mmid);
  a.parm[2] = r.f(parm_zero, (size_t)mb * 7 * mzero);
  if (r.st) return r.st;
  int cnt[3][G3M3_MAX_GRIDS];
  const int* cp[3] = {numsrf, nummid, numzero};
  for (int q = 0; q < 3; q++) {
    if (mb > G3M3_MAX_GRIDS) return set_err(ctx, G3M3_ERR_ARG, "mbndry too large");
    const int st = host_ints(ctx, cp[q], mb, cnt[q]);
    if (st) return st;
  }
  const int caps[3] = {msrf, mmid, mzero};
  for (int q = 0; q < 3; q++) {
    a.num[q] = cnt[q][mb - 1];
    if (a.num[q] < 0 || a.num[q] > caps[q]) return set_err(ctx, G3M3_ERR_ARG, "inner list count out of range");
  }
  a.mbndry = mb; a.box = mb;
  a.d = Dims{p->nx, p->ny, p->nz};
  a.dx = (p->grd_xmax[mb - 1] - p->grd_xmin[mb - 1]) / ((float)p->nx - 1.0f);
  a.dy = (p->grd_ymax[mb - 1] - p->grd_ymin[mb - 1]) / ((float)p->ny - 1.0f);
  a.xmin = p->grd_xmin[mb - 1]; a.ymin = p->grd_ymin[mb - 1];
  a.re_equiv = p->re_equiv; a.v_rot = p->v_rot;
  // the lists on the host, to find cells they name twice
  const int* lp[3] = {ijsrf, ijmid, ijzero};
  std::vector<int> hl[3];
  const int* hp[3];
  for (int q = 0; q < 3; q++) {
    hl[q].resize((size_t)mb * 3 * a.num[q] + 1);
    if (a.num[q] > 0 && (s = host_ints(ctx, lp[q], mb * 3 * a.num[q], hl[q].data()))) return s;
    hp[q] = hl[q].data();
  }
  launch_bndry_inner(a, inner_order(hp, a.num, mb, mb, a.d), ctx->stream);
  return finish(ctx, "bndry_inner");
}

}  // extern "C"

namespace g3m3 {

void fill_flanks_geometry(FlanksArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                          const float* gymin, const float* gymax, const float* gzmin, const float* gzmax) {
  const int mb = box + 1, ms = box;
  a.d = Dims{nx, ny, nz};
  a.delx = (gxmax[mb - 1] - gxmin[mb - 1]) / ((float)nx - 1.0f);
  a.dely = (gymax[mb - 1] - gymin[mb - 1]) / ((float)ny - 1.0f);
  a.delz = (gzmax[mb - 1] - gzmin[mb - 1]) / ((float)nz - 1.0f);
  a.sx = (gxmax[ms - 1] - gxmin[ms - 1]) / ((float)nx - 1.0f);
  a.sy = (gymax[ms - 1] - gymin[ms - 1]) / ((float)ny - 1.0f);
  a.sz = (gzmax[ms - 1] - gzmin[ms - 1]) / ((float)nz - 1.0f);
  a.sxmin = gxmin[ms - 1]; a.symin = gymin[ms - 1]; a.szmin = gzmin[ms - 1];
  a.bxmin = gxmin[mb - 1]; a.bymin = gymin[mb - 1]; a.bzmin = gzmin[mb - 1];
}

void fill_corer_geometry(CorerArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                         const float* gymin, const float* gymax, const float* gzmin, const float* gzmax) {
  const int mb = box + 1, ms = box;
  a.d = Dims{nx, ny, nz};
  const float sx = (gxmax[ms - 1] - gxmin[ms - 1]) / ((float)nx - 1.0f);
  const float dx = (gxmax[mb - 1] - gxmin[mb - 1]) / ((float)nx - 1.0f);
  const float dy = (gymax[mb - 1] - gymin[mb - 1]) / ((float)ny - 1.0f);
  const float dz = (gzmax[mb - 1] - gzmin[mb - 1]) / ((float)nz - 1.0f);
  a.nskip = (int)(dx / sx);
  a.nbx1 = (int)(1.0f + (gxmin[ms - 1] - gxmin[mb - 1]) / dx + 0.5f);
  a.nby1 = (int)(1.0f + (gymin[ms - 1] - gymin[mb - 1]) / dy + 0.5f);
  a.nbz1 = (int)(1.0f + (gzmin[ms - 1] - gzmin[mb - 1]) / dz + 0.5f);
  const int ns = a.nskip > 0 ? a.nskip : 1;
  a.ni = nx - 2 * a.nskip >= 1 ? (nx - 1 - 2 * a.nskip) / ns + 1 : 0;
  a.nj = ny - 2 * a.nskip >= 1 ? (ny - 1 - 2 * a.nskip) / ns + 1 : 0;
  a.nk = nz - 2 * a.nskip >= 1 ? (nz - 1 - 2 * a.nskip) / ns + 1 : 0;
}

void fill_synced_geometry(SyncedArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                          const float* gymin, const float* gymax, const float* gzmin, const float* gzmax) {
  const int mb = box + 1, ms = box;
  a.d = Dims{nx, ny, nz};
  a.delx = (gxmax[mb - 1] - gxmin[mb - 1]) / ((float)nx - 1.0f);
  a.dely = (gymax[mb - 1] - gymin[mb - 1]) / ((float)ny - 1.0f);
  a.delz = (gzmax[mb - 1] - gzmin[mb - 1]) / ((float)nz - 1.0f);
  a.sx = (gxmax[ms - 1] - gxmin[ms - 1]) / ((float)nx - 1.0f);
  a.sy = (gymax[ms - 1] - gymin[ms - 1]) / ((float)ny - 1.0f);
  a.sz = (gzmax[ms - 1] - gzmin[ms - 1]) / ((float)nz - 1.0f);
  a.sxmin = gxmin[ms - 1]; a.symin = gymin[ms - 1]; a.szmin = gzmin[ms - 1];
  a.bxmin = gxmin[mb - 1]; a.bymin = gymin[mb - 1]; a.bzmin = gzmin[mb - 1];
  a.kb_top = (int)(1.0f + (gzmax[ms - 1] - gzmin[mb - 1]) / a.delz);
  a.kb_bot = (int)(1.0f + (gzmin[ms - 1] - gzmin[mb - 1]) / a.delz);
  a.jb_top = (int)(1.0f + (gymax[ms - 1] - gymin[mb - 1]) / a.dely);
  a.jb_bot = (int)(1.0f + (gymin[ms - 1] - gymin[mb - 1]) / a.dely);
  a.ib_top = (int)(1.0f + (gxmax[ms - 1] - gxmin[mb - 1]) / a.delx);
  a.ib_bot = (int)(1.0f + (gxmin[ms - 1] - gxmin[mb - 1]) / a.delx);
}

}  // namespace g3m3

extern "C" {

static int read_grid(g3m3_ctx* ctx, int n_grids, const float* gp[6], float g[6][G3M3_MAX_GRIDS]) {
  if (n_grids > G3M3_MAX_GRIDS) return set_err(ctx, G3M3_ERR_ARG, "n_grids > %d", G3M3_MAX_GRIDS);
  for (int q = 0; q < 6; q++)
    if (!host_floats(ctx, gp[q], n_grids, g[q])) return set_err(ctx, G3M3_ERR_ARG, "grid extents unreadable");
  return G3M3_OK;
}

int g3m3_bndry_flanks(g3m3_ctx* ctx, float* const target[G3M3_NFIELDS], const float* const cur[G3M3_NFIELDS],
                      const float* const old[G3M3_NFIELDS], int nx, int ny, int nz, int n_grids, int box,
                      const double* t_old, const double* t_new, double t, const float* grd_xmin,
                      const float* grd_xmax, const float* grd_ymin, const float* grd_ymax, const float* grd_zmin,
                      const float* grd_zmax) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  if (box >= n_grids) return set_err(ctx, G3M3_ERR_ARG, "flanks need a coarser box above box %d", box);
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids;
  const size_t os = off(nx, ny, nz, box), ob = off(nx, ny, nz, box + 1);
  float g[6][G3M3_MAX_GRIDS];
  const float* gp[6] = {grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax};
  if ((s = read_grid(ctx, n_grids, gp, g))) return s;
  Res r(ctx);
  FlanksArgs a{};
  int nf = 0;
  for (int q = 0; q < G3M3_NFIELDS; q++) {
    if (!target[q]) continue;
    a.target[nf] = r.f(target[q], n4) + os;
    a.curc[nf] = r.f(cur[q], n4) + ob;
    a.oldc[nf] = r.f(old[q], n4) + ob;
    nf++;
  }
  if (r.st) return r.st;
  a.nf = nf;
  fill_flanks_geometry(a, nx, ny, nz, box, g[0], g[1], g[2], g[3], g[4], g[5]);
  const int mb = box + 1;
  a.t1 = ScalarRef{(float)((t_new[mb - 1] - t) / (t_new[mb - 1] - t_old[mb - 1])), nullptr};
  launch_flanks(a, ctx->stream);
  return finish(ctx, "bndry_flanks");
}

int g3m3_flanks(g3m3_ctx* ctx, float* wrkrho, const float* rho, const float* oldrho, int nx, int ny, int nz,
                int n_grids, int box, const double* t_new, const double* t_old, double t, float* work,
                const float* grd_xmin, const float* grd_xmax, const float* grd_ymin, const float* grd_ymax,
                const float* grd_zmin, const float* grd_zmax) {
  (void)work;
  float* tg[G3M3_NFIELDS] = {};
  const float* cu[G3M3_NFIELDS] = {};
  const float* od[G3M3_NFIELDS] = {};
  tg[0] = wrkrho; cu[0] = rho; od[0] = oldrho;
  return g3m3_bndry_flanks(ctx, tg, cu, od, nx, ny, nz, n_grids, box, t_old, t_new, t, grd_xmin, grd_xmax,
                           grd_ymin, grd_ymax, grd_zmin, grd_zmax);
}

int g3m3_bndry_corer(g3m3_ctx* ctx, float* const f[G3M3_NFIELDS], int nx, int ny, int nz, int n_grids, int box,
                     const float* grd_xmin, const float* grd_xmax, const float* grd_ymin, const float* grd_ymax,
                     const float* grd_zmin, const float* grd_zmax) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  if (box >= n_grids) return set_err(ctx, G3M3_ERR_ARG, "corer needs a coarser box above box %d", box);
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids;
  float g[6][G3M3_MAX_GRIDS];
  const float* gp[6] = {grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax};
  if ((s = read_grid(ctx, n_grids, gp, g))) return s;
  Res r(ctx);
  CorerArgs a{};
  int nf = 0;
  for (int q = 0; q < G3M3_NFIELDS; q++) {
    if (!f[q]) continue;
    float* base = r.f(f[q], n4);
    if (r.st) return r.st;
    a.fine[nf] = base + off(nx, ny, nz, box);
    a.coarse[nf] = base + off(nx, ny, nz, box + 1);
    nf++;
  }
  a.nf = nf;
  fill_corer_geometry(a, nx, ny, nz, box, g[0], g[1], g[2], g[3], g[4], g[5]);
  launch_corer(a, ctx->stream);
  return finish(ctx, "bndry_corer");
}

int g3m3_corer(g3m3_ctx* ctx, float* rho, int nx, int ny, int nz, int n_grids, int box, const float* grd_xmin,
               const float* grd_xmax, const float* grd_ymin, const float* grd_ymax, const float* grd_zmin,
               const float* grd_zmax) {
  float* f[G3M3_NFIELDS] = {};
  f[0] = rho;
  return g3m3_bndry_corer(ctx, f, nx, ny, nz, n_grids, box, grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin,
                          grd_zmax);
}

int g3m3_flanks_synced(g3m3_ctx* ctx, float* rho, int nx, int ny, int nz, int n_grids, int box,
                       const float* grd_xmin, const float* grd_xmax, const float* grd_ymin, const float* grd_ymax,
                       const float* grd_zmin, const float* grd_zmax) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  if (box >= n_grids) return set_err(ctx, G3M3_ERR_ARG, "flanks_synced needs a coarser box above box %d", box);
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids;
  float g[6][G3M3_MAX_GRIDS];
  const float* gp[6] = {grd_xmin, grd_xmax, grd_ymin, grd_ymax, grd_zmin, grd_zmax};
  if ((s = read_grid(ctx, n_grids, gp, g))) return s;
  Res r(ctx);
  float* base = r.f(rho, n4);
  if (r.st) return r.st;
  SyncedArgs a{};
  a.fine[0] = base + off(nx, ny, nz, box);
  a.coarse[0] = base + off(nx, ny, nz, box + 1);
  a.nf = 1;
  fill_synced_geometry(a, nx, ny, nz, box, g[0], g[1], g[2], g[3], g[4], g[5]);
  launch_flanks_synced(a, ctx->stream);
  return finish(ctx, "flanks_synced");
}

int g3m3_divb_correct(g3m3_ctx* ctx, int nx, int ny, int nz, int n_grids, int box, int nbands,
                      const int* divb_band_pos, const float* xspac, float divb_errlim, float* bx, float* by,
                      float* bz, int* iters) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  if (nbands != 7) return set_err(ctx, G3M3_ERR_ARG, "divB_correct supports the 7-band Laplacian only");
  if (divb_band_pos) {
    int pos[7];
    if ((s = host_ints(ctx, divb_band_pos, 7, pos))) return s;
    const int want[7] = {nx * ny, nx, 1, 0, -1, -nx, -nx * ny};
    for (int q = 0; q < 7; q++)
      if (pos[q] != want[q]) return set_err(ctx, G3M3_ERR_ARG, "unexpected band layout");
  }
  float xs[G3M3_MAX_GRIDS];
  if (n_grids > G3M3_MAX_GRIDS || !host_floats(ctx, xspac, n_grids, xs))
    return set_err(ctx, G3M3_ERR_ARG, "xspac unreadable");
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  if ((s = ensure_cg_scratch(ctx, n3))) return s;
  Res r(ctx);
  float* dbx = r.f(bx, n4) + o;
  float* dby = r.f(by, n4) + o;
  float* dbz = r.f(bz, n4) + o;
  if (r.st) return r.st;
  return run_divb_with(ctx, dbx, dby, dbz, Dims{nx, ny, nz}, xs[box - 1], divb_errlim, ctx->cg, ctx->host_cg,
                       ctx->cgvec, ctx->stream, iters, &ctx->cg_graphs);
}

int g3m3_flux_counter(g3m3_ctx* ctx, const float* qpx, const float* qpy, const float* qpz, const float* hpx,
                      const float* hpy, const float* hpz, const float* opx, const float* opy, const float* opz,
                      int nx, int ny, int nz, int n_grids, int box, float rmassq, float rmassh, float rmasso,
                      float grid_spacing, float* qflux_in, float* qflux_out, float* hflux_in, float* hflux_out,
                      float* oflux_in, float* oflux_out) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, box);
  if (s) return s;
  if ((s = ensure_words(ctx))) return s;
  const size_t n3 = (size_t)nx * ny * nz, n4 = n3 * n_grids, o = off(nx, ny, nz, box);
  Res r(ctx);
  FluxArgs a{};
  const float* p[3][3] = {{qpx, qpy, qpz}, {hpx, hpy, hpz}, {opx, opy, opz}};
  for (int sp = 0; sp < 3; sp++)
    for (int q = 0; q < 3; q++) a.p[sp][q] = r.f(p[sp][q], n4) + o;
  if (r.st) return r.st;
  a.d = Dims{nx, ny, nz};
  a.rmass[0] = rmassq; a.rmass[1] = rmassh; a.rmass[2] = rmasso;
  a.grid_spacing = grid_spacing;
  a.out = reinterpret_cast<float*>(ctx->words);
  a.n_grids = n_grids; a.box = box;
  launch_flux_counter(a, ctx->stream);
  G3M3_CUDA(ctx, cudaMemcpyAsync(ctx->host_words, ctx->words, 6 * sizeof(float), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  G3M3_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const float* h = reinterpret_cast<const float*>(ctx->host_words);
  float* outs[6] = {qflux_in, qflux_out, hflux_in, hflux_out, oflux_in, oflux_out};
  for (int q = 0; q < 6; q++)
    if (outs[q]) *outs[q] = h[q];
  return finish(ctx, "flux_counter");
}

int g3m3_sparse_solver(g3m3_ctx* ctx, int nbands, int npts, const int* divb_band_pos, float divb_errlim,
                       int recurse, int redo_lim, const float* divb, float* soln_vec, float* residual2,
                       const float* banded_matrix) {
  if (!ctx) return G3M3_ERR_ARG;
  if (nbands < 1 || nbands > 16 || npts < 1 || !divb_band_pos)
    return set_err(ctx, G3M3_ERR_ARG, "sparse_solver: nbands=%d (1..16), npts=%d", nbands, npts);
  DivbArgs a{};
  int s = host_ints(ctx, divb_band_pos, nbands, a.pos);
  if (s) return s;
  s = ensure_cg_scratch(ctx, (size_t)npts);
  if (s) return s;
  Res r(ctx);
  const size_t n = (size_t)npts;
  a.rhs = r.f(divb, n);
  a.x = r.f(soln_vec, n);
  a.band = r.f(banded_matrix, (size_t)nbands * n);
  if (r.st) return r.st;
  float* vec = ctx->cgvec;
  a.xs = vec; a.g = vec + n; a.h = vec + 2 * n; a.xi = vec + 3 * n; a.xj = vec + 4 * n;
  a.st = ctx->cg;
  a.d = Dims{npts, 1, 1};
  a.nbands = nbands;
  int status = CG_RUNNING;
  // the SAVEd restart count starts at redo_lim for a recursive call (:55-60)
  const int redos0 = (recurse ? redo_lim : 0) + 1;
  float r2 = 0.0f;
  s = run_cg(ctx, a, divb_errlim, true, redos0, ctx->host_cg, ctx->stream, nullptr, &r2, &status, &ctx->cg_graphs);
  if (s) return s;
  if (residual2) *residual2 = r2;
  if (status == CG_MAXIT) return set_err(ctx, G3M3_ERR_NOCONV, "sparse_solver: too many iterations");
  return G3M3_OK;
}

int g3m3_sample_points(g3m3_ctx* ctx, const float* field, int nx, int ny, int nz, int n_grids,
                       const float* grid_minvals, const float* grid_maxvals, const float* xspac, float re_equiv,
                       const float* xyz, int n, float* out) {
  int s = check_dims(ctx, nx, ny, nz, n_grids, 1);
  if (s) return s;
  if (n < 0 || n_grids > G3M3_MAX_GRIDS) return set_err(ctx, G3M3_ERR_ARG, "bad sample count");
  if (n == 0) return G3M3_OK;
  SampleArgs a{};
  if (!host_floats(ctx, grid_minvals, 3 * n_grids, a.gmin) || !host_floats(ctx, grid_maxvals, 3 * n_grids, a.gmax) ||
      !host_floats(ctx, xspac, n_grids, a.xspac))
    return set_err(ctx, G3M3_ERR_ARG, "grid description unreadable");
  const size_t n4 = (size_t)nx * ny * nz * n_grids;
  Res r(ctx);
  a.field = r.f(field, n4);
  a.xyz = r.f(xyz, 3 * (size_t)n);
  a.out = r.f(out, (size_t)n);
  if (r.st) return r.st;
  a.n = n; a.n_grids = n_grids; a.d = Dims{nx, ny, nz}; a.re_equiv = re_equiv;
  launch_sample(a, ctx->stream);
  return finish(ctx, "sample_points");
}

}  // extern "C"
