// fluidfile.cu -- the reference's fluid (restart) file and a device-side
// comparison of two states.
//
// File layout (3d_main.f90:3305-3349 writes it, compare_fluids.f90 and the
// restart read it): Fortran unformatted sequential records, each framed by
// a 4-byte little-endian byte count before and after it:
//   t                                  real(dp)
//   qrho qpx qpy qpz qpresx qpresy qpresz qpresxy qpresxz qpresyz
//   hrho ... hpresyz, orho ... opresyz (30 records, (nx,ny,nz,n_grids) each)
//   bx by bz epres bx0 by0 bz0         (7 records)
//   parm_srf parm_mid parm_zero ijzero numzero ijmid nummid ijsrf numsrf
//                                      (one record)
// The state arrays handed over here are the library's 34-field order
// (g3m3_types.h: species, then epres, then bx, by, bz).
#include <cstdio>
#include <cstring>
#include <vector>

#include "ctx.cuh"

namespace g3m3 {
namespace {

// file record index of each library field
const int kFileOrder[G3M3_NFIELDS] = {
    0,  1,  2,  3,  4,  5,  6,  7,  8,  9,    // q
    10, 11, 12, 13, 14, 15, 16, 17, 18, 19,   // h
    20, 21, 22, 23, 24, 25, 26, 27, 28, 29,   // o
    33,                                        // epres is written after bz
    30, 31, 32};                               // bx, by, bz

struct Part {
  const void* p;
  size_t bytes;
};

bool put_record(FILE* f, const std::vector<Part>& parts) {
  size_t n = 0;
  for (const Part& q : parts) n += q.bytes;
  if (n > 0x7fffffffu) return false;   // larger records need subrecord markers
  const uint32_t m = (uint32_t)n;
  unsigned char b[4] = {(unsigned char)(m & 0xff), (unsigned char)((m >> 8) & 0xff), (unsigned char)((m >> 16) & 0xff),
                        (unsigned char)((m >> 24) & 0xff)};
  if (fwrite(b, 1, 4, f) != 4) return false;
  for (const Part& q : parts)
    if (q.bytes && fwrite(q.p, 1, q.bytes, f) != q.bytes) return false;
  return fwrite(b, 1, 4, f) == 4;
}

bool get_marker(FILE* f, uint32_t* m) {
  unsigned char b[4];
  if (fread(b, 1, 4, f) != 4) return false;
  *m = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
  return true;
}

// reads one record into parts; the record must hold at least their bytes
// (a Fortran read may take a prefix of a record)
bool get_record(FILE* f, const std::vector<std::pair<void*, size_t>>& parts) {
  uint32_t m = 0, m2 = 0;
  if (!get_marker(f, &m)) return false;
  size_t want = 0;
  for (auto& q : parts) want += q.second;
  if (want > m) return false;
  for (auto& q : parts)
    if (q.second && fread(q.first, 1, q.second, f) != q.second) return false;
  if (m > want && fseek(f, (long)(m - want), SEEK_CUR) != 0) return false;
  return get_marker(f, &m2) && m2 == m;
}

int fail(g3m3_ctx* c, int code, const char* what, const char* path) {
  if (c) return set_err(c, code, "%s: %s", what, path);
  return code;
}

__device__ __forceinline__ bool differ(float a, float b) {
  if (a == b) return false;                  // includes +0 == -0
  return !(isnan(a) && isnan(b));
}

__global__ void __launch_bounds__(256) k_diff(const float* const* a, const float* const* b, size_t n, int n_grids,
                                              double* stats) {
  // blockIdx.y = field * n_grids + box; stats[.][4] = max|a-b|, sum (a-b)^2, sum a^2, count differing
  const int fb = blockIdx.y;
  const int f = fb / n_grids, box = fb % n_grids;
  const float* pa = a[f] + (size_t)box * n;
  const float* pb = b[f] + (size_t)box * n;
  double mx = 0.0, s2 = 0.0, a2 = 0.0, cnt = 0.0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const float x = __ldg(pa + c), y = __ldg(pb + c);
    if (differ(x, y)) {
      const double d = (double)x - (double)y;
      mx = fmax(mx, fabs(d));
      s2 += d * d;
      cnt += 1.0;
    }
    a2 += (double)x * (double)x;
  }
  __shared__ double sh[4][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double v[4] = {mx, s2, a2, cnt};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_xor_sync(0xffffffffu, v[q], o);
      v[q] = q == 0 ? fmax(v[q], t) : v[q] + t;
    }
    if (lane == 0) sh[q][w] = v[q];
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    const int q = threadIdx.x;
    double r = sh[q][0];
    for (int i = 1; i < 8; i++) r = q == 0 ? fmax(r, sh[q][i]) : r + sh[q][i];
    double* out = stats + (size_t)fb * 4 + q;
    if (q == 0) {
      // non-negative doubles order like their bit patterns
      atomicMax(reinterpret_cast<unsigned long long*>(out), (unsigned long long)__double_as_longlong(r));
    } else {
      atomicAdd(out, r);
    }
  }
}

}  // namespace
}  // namespace g3m3

using namespace g3m3;

extern "C" {

int g3m3_fluid_write(g3m3_ctx* ctx, const char* path, const g3m3_params* p, double t, const float* state,
                     const float* b0, const float* parm_srf, const float* parm_mid, const float* parm_zero,
                     const int* ijzero, const int* numzero, const int* ijmid, const int* nummid, const int* ijsrf,
                     const int* numsrf, int msrf, int mmid, int mzero) {
  if (!path || !p || !state || !b0) return G3M3_ERR_ARG;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1 || p->n_grids < 1 || p->mbndry < 0 || p->mbndry > p->n_grids)
    return fail(ctx, G3M3_ERR_ARG, "bad dimensions for", path);
  const size_t n4 = (size_t)p->nx * p->ny * p->nz * p->n_grids;
  const size_t mb = (size_t)p->mbndry;
  FILE* f = fopen(path, "wb");
  if (!f) return fail(ctx, G3M3_ERR_ARG, "cannot open for writing", path);
  bool ok = put_record(f, {{&t, sizeof t}});
  const float* rec[37];
  for (int q = 0; q < G3M3_NFIELDS; q++) rec[kFileOrder[q]] = state + (size_t)q * n4;
  for (int q = 0; q < 3; q++) rec[34 + q] = b0 + (size_t)q * n4;
  for (int r = 0; r < 37 && ok; r++) ok = put_record(f, {{rec[r], n4 * sizeof(float)}});
  if (ok)
    ok = put_record(f, {{parm_srf, mb * 7 * msrf * sizeof(float)}, {parm_mid, mb * 7 * mmid * sizeof(float)},
                        {parm_zero, mb * 7 * mzero * sizeof(float)}, {ijzero, mb * 3 * mzero * sizeof(int)},
                        {numzero, mb * sizeof(int)}, {ijmid, mb * 3 * mmid * sizeof(int)}, {nummid, mb * sizeof(int)},
                        {ijsrf, mb * 3 * msrf * sizeof(int)}, {numsrf, mb * sizeof(int)}});
  ok = (fclose(f) == 0) && ok;
  return ok ? G3M3_OK : fail(ctx, G3M3_ERR_STATE, "write failed", path);
}

int g3m3_fluid_read(g3m3_ctx* ctx, const char* path, const g3m3_params* p, double* t, float* state, float* b0,
                    float* parm_srf, float* parm_mid, float* parm_zero, int* ijzero, int* numzero, int* ijmid,
                    int* nummid, int* ijsrf, int* numsrf, int msrf, int mmid, int mzero) {
  if (!path || !p || !state || !b0 || !t) return G3M3_ERR_ARG;
  if (p->nx < 1 || p->ny < 1 || p->nz < 1 || p->n_grids < 1 || p->mbndry < 0 || p->mbndry > p->n_grids)
    return fail(ctx, G3M3_ERR_ARG, "bad dimensions for", path);
  const size_t n4 = (size_t)p->nx * p->ny * p->nz * p->n_grids;
  const size_t mb = (size_t)p->mbndry;
  FILE* f = fopen(path, "rb");
  if (!f) return fail(ctx, G3M3_ERR_ARG, "cannot open for reading", path);
  bool ok = get_record(f, {{t, sizeof(double)}});
  float* rec[37];
  for (int q = 0; q < G3M3_NFIELDS; q++) rec[kFileOrder[q]] = state + (size_t)q * n4;
  for (int q = 0; q < 3; q++) rec[34 + q] = b0 + (size_t)q * n4;
  for (int r = 0; r < 37 && ok; r++) ok = get_record(f, {{rec[r], n4 * sizeof(float)}});
  if (ok && parm_srf)
    ok = get_record(f, {{parm_srf, mb * 7 * msrf * sizeof(float)}, {parm_mid, mb * 7 * mmid * sizeof(float)},
                        {parm_zero, mb * 7 * mzero * sizeof(float)}, {ijzero, mb * 3 * mzero * sizeof(int)},
                        {numzero, mb * sizeof(int)}, {ijmid, mb * 3 * mmid * sizeof(int)}, {nummid, mb * sizeof(int)},
                        {ijsrf, mb * 3 * msrf * sizeof(int)}, {numsrf, mb * sizeof(int)}});
  fclose(f);
  return ok ? G3M3_OK : fail(ctx, G3M3_ERR_STATE, "not a fluid file of these dimensions", path);
}

int g3m3_diff_fields(g3m3_ctx* ctx, int nfields, const float* const* a, const float* const* b, int nx, int ny,
                     int nz, int n_grids, double* stats) {
  if (!ctx || nfields < 1 || nfields > 64 || !a || !b || !stats || nx < 1 || ny < 1 || nz < 1 || n_grids < 1)
    return G3M3_ERR_ARG;
  const size_t n = (size_t)nx * ny * nz, n4 = n * n_grids;
  std::vector<const float*> da(nfields), db(nfields);
  int st = 0;
  for (int q = 0; q < nfields; q++) {
    da[q] = static_cast<const float*>(resolve(ctx, a[q], n4 * sizeof(float), &st));
    db[q] = static_cast<const float*>(resolve(ctx, b[q], n4 * sizeof(float), &st));
  }
  if (st) return st;
  const size_t nstat = (size_t)nfields * n_grids * 4;
  // pointer tables and the statistics in one scratch block
  const size_t bytes = 2 * nfields * sizeof(float*) + nstat * sizeof(double);
  void* scratch = nullptr;
  G3M3_CUDA(ctx, dev_alloc(ctx, (void**)&scratch, bytes));
  const float** tab = static_cast<const float**>(scratch);
  double* dstat = reinterpret_cast<double*>(static_cast<char*>(scratch) + 2 * nfields * sizeof(float*));
  std::vector<const float*> host_tab(2 * nfields);
  for (int q = 0; q < nfields; q++) { host_tab[q] = da[q]; host_tab[nfields + q] = db[q]; }
  cudaError_t e = cudaMemcpyAsync(tab, host_tab.data(), 2 * nfields * sizeof(float*), cudaMemcpyHostToDevice,
                                  ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(dstat, 0, nstat * sizeof(double), ctx->stream);
  if (e == cudaSuccess) {
    unsigned bx = (unsigned)((n + 255) / 256);
    if (bx > (unsigned)sm_count()) bx = (unsigned)sm_count();
    k_diff<<<dim3(bx, (unsigned)(nfields * n_grids)), 256, 0, ctx->stream>>>(tab, tab + nfields, n, n_grids, dstat);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(stats, dstat, nstat * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(scratch);
  return e == cudaSuccess ? G3M3_OK : cuda_check(ctx, e, "diff_fields");
}

}  // extern "C"
