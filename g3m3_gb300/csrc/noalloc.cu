// noalloc.cu -- g3m3_divb_correct_noalloc: the div B correction of
// g3m3_divb_correct (sub_divb_correct.f90:4-57 with the CG solver of
// sub_sparse_solver.f90:10-140) for callers that must not allocate device
// memory while they run.
//
// Who needs it: a host code that hands the whole device to its own memory
// pool at start-up (so a later cudaMalloc fails or steals from the pool), or
// one that keeps other streams busy and cannot afford the device-wide
// synchronisation that cudaMalloc/cudaFree may bring.  g3m3_divb_correct
// grows per-context scratch with cudaMalloc and mirrors host arrays into new
// device buffers; this variant does neither.
//
// The solver's state and its seven vectors live in one file-scope device
// array, sized for boxes of up to G3M3_NOALLOC_DIVB_MAX_CELLS cells.  Every
// call looks up the array's address on the context's device (with that
// device current); the lookup allocates nothing, so a device reset between
// calls leaves no stale address behind.  The array is shared by every call
// on the device and keeps the last call's contents: each call rewrites the
// solver state from the host and its first kernel zeroes the iterate; every
// other vector is written before it is read.  Two calls that overlap in
// time race on the array.
#include <cstring>
#include <mutex>

#include "ctx.cuh"

namespace g3m3 {
int run_divb(g3m3_ctx* c, float* bx, float* by, float* bz, const Dims& d, float rx, float errlim, CgState* st,
             CgState* host_st, float* vec, cudaStream_t s, int* iters_out);
}  // namespace g3m3

using namespace g3m3;

namespace {

constexpr size_t kMaxCells = G3M3_NOALLOC_DIVB_MAX_CELLS;
constexpr size_t kStateBytes = 256;   // CgState, padded so the vectors start 256-byte aligned
constexpr size_t kScratchBytes = kStateBytes + 7 * kMaxCells * sizeof(float);
static_assert(sizeof(CgState) <= kStateBytes, "solver state does not fit its slot");
constexpr int kMaxDevices = 64;

}  // namespace

// 256 B of solver state followed by the 7 CG vectors of the largest box: 28 MiB
static __device__ __align__(256) unsigned char divb_noalloc_scratch[kScratchBytes];

namespace {

std::mutex setup_mutex;

// Device address of the scratch array on the context's device, looked up
// with that device current.
int scratch_for(g3m3_ctx* c, void** out) {
  if (c->device < 0 || c->device >= kMaxDevices)
    return set_err(c, G3M3_ERR_ARG, "divb_correct_noalloc: device %d out of range", c->device);
  std::lock_guard<std::mutex> lock(setup_mutex);
  int prev = -1;
  G3M3_CUDA(c, cudaGetDevice(&prev));
  if (prev != c->device) G3M3_CUDA(c, cudaSetDevice(c->device));
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, divb_noalloc_scratch);
  if (prev != c->device) cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_check(c, e, "cudaGetSymbolAddress(div B scratch)");
  *out = p;
  return G3M3_OK;
}

// Device (or managed) memory that the context's device can use directly.
bool on_device(const g3m3_ctx* c, const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == c->device;
}

}  // namespace

extern "C" int g3m3_divb_correct_noalloc(g3m3_ctx* ctx, int nx, int ny, int nz, int n_grids, int box, int nbands,
                                         const int* divb_band_pos, const float* xspac, float divb_errlim,
                                         float* bx, float* by, float* bz, int* iters) {
  if (!ctx) return G3M3_ERR_ARG;
  if (nx < 4 || ny < 4 || nz < 4 || n_grids < 1 || box < 1 || box > n_grids || n_grids > G3M3_MAX_GRIDS)
    return set_err(ctx, G3M3_ERR_ARG, "bad dimensions nx=%d ny=%d nz=%d n_grids=%d box=%d", nx, ny, nz, n_grids,
                   box);
  const size_t n3 = (size_t)nx * ny * nz;
  if (n3 > kMaxCells)
    return set_err(ctx, G3M3_ERR_ARG,
                   "divb_correct_noalloc: a %dx%dx%d box has %zu cells, more than the %zu its fixed scratch holds; "
                   "use g3m3_divb_correct",
                   nx, ny, nz, n3, kMaxCells);
  if (nbands != 7) return set_err(ctx, G3M3_ERR_ARG, "divB_correct supports the 7-band Laplacian only");
  if (divb_band_pos) {
    int pos[7];
    const int rc = host_ints(ctx, divb_band_pos, 7, pos);   // ordered on the context's stream
    if (rc) return rc;
    const int want[7] = {nx * ny, nx, 1, 0, -1, -nx, -nx * ny};
    for (int q = 0; q < 7; q++)
      if (pos[q] != want[q]) return set_err(ctx, G3M3_ERR_ARG, "unexpected band layout");
  }
  float xs[G3M3_MAX_GRIDS];
  if (!host_floats(ctx, xspac, n_grids, xs)) return set_err(ctx, G3M3_ERR_ARG, "xspac unreadable");
  if (!bx || !by || !bz || !on_device(ctx, bx) || !on_device(ctx, by) || !on_device(ctx, bz))
    return set_err(ctx, G3M3_ERR_ARG,
                   "divb_correct_noalloc: bx, by, bz must be device memory of the context's device %d (a host "
                   "array would need a device copy)",
                   ctx->device);
  void* scratch = nullptr;
  int s = scratch_for(ctx, &scratch);
  if (s) return s;
  CgState host_state;
  const size_t o = (size_t)(box - 1) * n3;
  float* vec = reinterpret_cast<float*>(static_cast<unsigned char*>(scratch) + kStateBytes);
  return run_divb(ctx, bx + o, by + o, bz + o, Dims{nx, ny, nz}, xs[box - 1], divb_errlim,
                  static_cast<CgState*>(scratch), &host_state, vec, ctx->stream, iters);
}
