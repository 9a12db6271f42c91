// k_guards.cu -- positivity floors and the speed limiter:
//   set_rho         sub_set_rho.f90:5-104
//   set_speed_agrd  sub_set_speed_agrd.f90:6-435
//
// The reference limiter replaces a cell by the mean of its six neighbours'
// snapshot values (taken before the limiter loop, after set_rho).  A cell
// only ever reads its own current values and its neighbours' snapshot, so
// cells are independent; the in-place update is made race-free by
// (a) evaluating set_rho on the fly for every value read, and
// (b) deferring every species store (set_rho repairs and limiter
//     replacements alike): a changed cell appends (cell, species, 10
//     values) to a scratch list that a second launch scatters once every
//     thread has read its neighbours.  During the first launch the species
//     arrays are read only, so no thread can see another's half-written
//     update.  Electron pressure and btot are never read at a neighbour
//     and are stored in place.
// Both routines therefore run as one pass over the box plus a scatter of
// the (rare) flagged cells.  Max-speed reductions are warp-shuffle maxima
// folded into 5 device words with atomicMax on the (non-negative) float bits.
#include <cooperative_groups.h>

#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

struct Sp {   // one species at one cell
  float r, px, py, pz, xx, yy, zz, xy, xz, yz;
};

__device__ __forceinline__ Sp load_sp(const GuardArgs& a, int s, size_t c) {
  const int b = 10 * s;
  Sp v;
  v.r = a.f[b + 0][c]; v.px = a.f[b + 1][c]; v.py = a.f[b + 2][c]; v.pz = a.f[b + 3][c];
  v.xx = a.f[b + 4][c]; v.yy = a.f[b + 5][c]; v.zz = a.f[b + 6][c];
  v.xy = a.f[b + 7][c]; v.xz = a.f[b + 8][c]; v.yz = a.f[b + 9][c];
  return v;
}

// the seven values the checks read; the off-diagonal pressures are loaded
// only for a cell whose values are rewritten
__device__ __forceinline__ Sp load_diag(const GuardArgs& a, int s, size_t c) {
  const int b = 10 * s;
  Sp v;
  v.r = a.f[b + 0][c]; v.px = a.f[b + 1][c]; v.py = a.f[b + 2][c]; v.pz = a.f[b + 3][c];
  v.xx = a.f[b + 4][c]; v.yy = a.f[b + 5][c]; v.zz = a.f[b + 6][c];
  v.xy = 0.0f; v.xz = 0.0f; v.yz = 0.0f;
  return v;
}

// The limiter's speeds of one species at one cell
// (sub_set_speed_agrd.f90:135-141): |p|/(rho + smallbit) per component and
// the sound speed
struct Speeds {
  float vx, vy, vz, cq;
};

__device__ __forceinline__ Speeds speeds(const Sp& v, float smallbit) {
  const float arho = v.r + smallbit;
  Speeds o;
  o.vx = fabsf(v.px / arho);
  o.vy = fabsf(v.py / arho);
  o.vz = fabsf(v.pz / arho);
  o.cq = sqrtf(0.33f * (v.xx + v.yy + v.zz) / arho);
  return o;
}

__device__ __forceinline__ float rho_min(int s) { return s == 0 ? 2.e-4f : (s == 1 ? 1.e-4f : 2.e-5f); }

// set_rho for one species; returns true when the values changed
__device__ __forceinline__ bool floor_sp(Sp& v, float rmin) {
  if (v.r < rmin || v.xx < 0.0f || v.yy < 0.0f || v.zz < 0.0f) {
    v.r = amax1(fabsf(v.r), 1.05f * rmin);
    const float ap = (fabsf(v.xx) + fabsf(v.yy) + fabsf(v.zz)) / 3.0f;
    v.xx = ap; v.yy = ap; v.zz = ap;
    v.xy = 0.0f; v.xz = 0.0f; v.yz = 0.0f;
    return true;
  }
  return false;
}

// deferred store of a species' ten values at cell c; the threads of a warp
// that append together take consecutive slots with one counter update
__device__ __forceinline__ void append(const GuardArgs& a, size_t c, int s, const Sp& v) {
  const cooperative_groups::coalesced_group g = cooperative_groups::coalesced_threads();
  unsigned base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(a.list_count, g.size());
  const unsigned slot = g.shfl(base, 0) + g.thread_rank();
  if (slot >= a.list_cap) return;   // counted: the host reports the overflow
  float* e = a.list + (size_t)slot * 11;
  e[0] = __uint_as_float((unsigned)(c * 4 + (size_t)s));
  e[1] = v.r; e[2] = v.px; e[3] = v.py; e[4] = v.pz; e[5] = v.xx; e[6] = v.yy;
  e[7] = v.zz; e[8] = v.xy; e[9] = v.xz; e[10] = v.yz;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = amax1(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__global__ void __launch_bounds__(256, 4) k_guards(const __grid_constant__ GuardArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  const bool inside = i <= d.nx && j <= d.ny && k <= d.nz;
  float mx = 0.0f, my = 0.0f, mz = 0.0f, mc = 0.0f, ma = 0.0f;
  if (inside) {
    const size_t c = d.at(i, j, k);
    const bool interior = i > 1 && j > 1 && k > 1 && i < d.nx && j < d.ny && k < d.nz;
    float newr[3];
    Sp sp3[3];   // every species value of this cell, loaded before any store
#pragma unroll
    for (int s = 0; s < 3; s++) sp3[s] = load_diag(a, s, c);
    float bsum[3] = {0.0f, 0.0f, 0.0f};
    if (a.do_speed) {
      bsum[0] = __ldg(a.b0[0] + c) + a.f[G3M3_F_BX][c];
      bsum[1] = __ldg(a.b0[1] + c) + a.f[G3M3_F_BY][c];
      bsum[2] = __ldg(a.b0[2] + c) + a.f[G3M3_F_BZ][c];
    }
    float ep = a.f[G3M3_F_EPRES][c];
    if (a.do_set_rho) ep = fabsf(ep);
    bool ep_changed = a.do_set_rho;
#pragma unroll
    for (int s = 0; s < 3; s++) {
      Sp v = sp3[s];
      // set_rho zeroes the off-diagonal terms of a repaired cell, so they
      // matter only when the cell is limited without being repaired
      const bool floored = a.do_set_rho && floor_sp(v, rho_min(s));
      newr[s] = v.r;
      if (floored && !a.do_speed) {   // no neighbour reads: store in place
        const int b = 10 * s;         // (set_rho leaves the momenta alone)
        a.f[b + 0][c] = v.r;
        a.f[b + 4][c] = v.xx; a.f[b + 5][c] = v.yy; a.f[b + 6][c] = v.zz;
        a.f[b + 7][c] = 0.0f; a.f[b + 8][c] = 0.0f; a.f[b + 9][c] = 0.0f;
        continue;
      }
      if (!(a.do_speed && interior)) {
        if (floored) append(a, c, s, v);   // deferred: neighbours still read this cell
        continue;
      }
      const Speeds sv = speeds(v, a.smallbit);
      const float avx = sv.vx, avy = sv.vy, avz = sv.vz, cq = sv.cq;
      const float vq = sqrtf(avx * avx + avy * avy + avz * avz);
      if (a.fold) {
        const unsigned nan_bits = (isnan(avx) ? 1u : 0u) | (isnan(avy) ? 2u : 0u) | (isnan(avz) ? 4u : 0u) |
                                  (isnan(cq) ? 8u : 0u);
        if (nan_bits) atomicOr(a.fold, nan_bits);
      }
      const float vl = a.vlim * a.svlim[s];
      const float cl = a.vlim * a.svlim[s] * a.sclim[s];
      if ((vq > vl) || (cq > cl)) {
        // neighbour means of the snapshot (anisotropy-limited pressures)
        const size_t nb[6] = {c + 1, c - 1, c + (size_t)d.nx, c - (size_t)d.nx,
                              c + (size_t)d.nx * d.ny, c - (size_t)d.nx * d.ny};
        float acc[10];
#pragma unroll
        for (int q = 0; q < 10; q++) acc[q] = 0.0f;
        for (int m = 0; m < 6; m++) {
          Sp u = load_sp(a, s, nb[m]);
          if (a.do_set_rho) floor_sp(u, rho_min(s));
          float sx, sy, sz, sxy, sxz, syz;
          if (a.isotropic) {
            sx = u.xx; sy = u.xx; sz = u.xx; sxy = 0.0f; sxz = 0.0f; syz = 0.0f;
          } else {
            const float ap = (u.xx + u.yy + u.zz) / 3.0f;
            sx = a.aniso_limit * u.xx + (1.0f - a.aniso_limit) * ap;
            sy = a.aniso_limit * u.yy + (1.0f - a.aniso_limit) * ap;
            sz = a.aniso_limit * u.zz + (1.0f - a.aniso_limit) * ap;
            sxy = a.aniso_limit * u.xy; sxz = a.aniso_limit * u.xz; syz = a.aniso_limit * u.yz;
          }
          if (m == 0) {
            acc[0] = u.r; acc[1] = u.px; acc[2] = u.py; acc[3] = u.pz;
            acc[4] = sx; acc[5] = sy; acc[6] = sz; acc[7] = sxy; acc[8] = sxz; acc[9] = syz;
          } else {
            acc[0] = acc[0] + u.r; acc[1] = acc[1] + u.px; acc[2] = acc[2] + u.py; acc[3] = acc[3] + u.pz;
            acc[4] = acc[4] + sx; acc[5] = acc[5] + sy; acc[6] = acc[6] + sz;
            acc[7] = acc[7] + sxy; acc[8] = acc[8] + sxz; acc[9] = acc[9] + syz;
          }
        }
        float nv[10];
#pragma unroll
        for (int q = 0; q < 7; q++) nv[q] = acc[q] / 6.0f;
#pragma unroll
        for (int q = 7; q < 10; q++) nv[q] = a.iso_flag * acc[q] / 6.0f;
        newr[s] = nv[0];
        Sp r;
        r.r = nv[0]; r.px = nv[1]; r.py = nv[2]; r.pz = nv[3]; r.xx = nv[4]; r.yy = nv[5];
        r.zz = nv[6]; r.xy = nv[7]; r.xz = nv[8]; r.yz = nv[9];
        append(a, c, s, r);
      } else if (floored) {
        append(a, c, s, v);
      }
      mx = amax1(mx, avx); my = amax1(my, avy); mz = amax1(mz, avz); mc = amax1(mc, cq);
    }
    if (a.do_speed) {
      const float sx = bsum[0], sy = bsum[1], sz = bsum[2];
      const float bt = amax1(sqrtf(sx * sx + sy * sy + sz * sz), a.smallbit);
      a.btot[c] = bt;
      if (interior) {
        const float arho = newr[0] + newr[1] + newr[2] + a.smallbit;
        const float cs = sqrtf(ep / arho);
        if (cs > a.cslim) { ep = ep * a.cslim / cs; ep_changed = true; }
        const float alf = bt / sqrtf(arho);
        if (a.fold && isnan(alf)) atomicOr(a.fold, 16u);
        ma = amax1(ma, alf);
      }
    }
    if (ep_changed) a.f[G3M3_F_EPRES][c] = ep;
  }
  if (a.do_speed) {
    // warp maxima, then block maxima, then one atomic per block and word
    __shared__ float wmax[5][8];
    mx = warp_max(mx); my = warp_max(my); mz = warp_max(mz); mc = warp_max(mc); ma = warp_max(ma);
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    if (lane == 0) {
      wmax[0][warp] = mx; wmax[1][warp] = my; wmax[2][warp] = mz; wmax[3][warp] = mc; wmax[4][warp] = ma;
    }
    __syncthreads();
    if (tid < 5) {
      float m = wmax[tid][0];
#pragma unroll
      for (int w = 1; w < 8; w++) m = amax1(m, wmax[tid][w]);
      if (m > 0.0f) atomicMax(a.maxbits + tid, __float_as_uint(m));
    }
  }
}

// The reference folds its maxima in loop order with amax1 (a > b ? a : b):
// a NaN replaces the running value and the next element replaces the NaN,
// so the result is the maximum of the elements after the last NaN (NaN when
// the NaN is the last element).  The words that met a NaN in k_guards are
// refolded here, in two passes: the last NaN's position, then the maximum
// after it.  Species words (pxmax..csmax) run over the species loops
// (species, then k, j, i over interior cells) on the values k_guards read,
// so before the scatter; alfmax over interior cells on the densities after
// the limiter, so after it.
__device__ __forceinline__ bool interior_cell(const Dims& d, long t, int& i, int& j, int& k) {
  const long ix = d.nx - 2, iy = d.ny - 2;
  if (t >= ix * iy * (d.nz - 2)) return false;
  i = (int)(t % ix) + 2;
  j = (int)((t / ix) % iy) + 2;
  k = (int)(t / (ix * iy)) + 2;
  return true;
}

template <int PASS>
__global__ void __launch_bounds__(256) k_fold_species(const __grid_constant__ GuardArgs a) {
  const unsigned flag = *(volatile unsigned*)a.fold & 15u;
  if (!flag) return;
  const Dims d = a.d;
  const long nint = (long)(d.nx - 2) * (d.ny - 2) * (d.nz - 2);
  int i, j, k;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; interior_cell(d, t, i, j, k);
       t += (long)gridDim.x * blockDim.x) {
    const size_t c = d.at(i, j, k);
    for (int s = 0; s < 3; s++) {
      const Speeds sv = speeds(load_diag(a, s, c), a.smallbit);
      const float x[4] = {sv.vx, sv.vy, sv.vz, sv.cq};
      const unsigned pos = (unsigned)(s * nint + t + 1);
#pragma unroll
      for (int w = 0; w < 4; w++) {
        if (!((flag >> w) & 1u)) continue;
        if (PASS == 0) {
          if (isnan(x[w])) atomicMax(a.fold + 1 + w, pos);
        } else if (pos > *(volatile unsigned*)(a.fold + 1 + w)) {
          atomicMax(a.fold + 6 + w, x[w] == 0.0f ? 0u : __float_as_uint(x[w]));
          atomicOr(a.fold + 11, 1u << w);
        }
      }
    }
  }
}

template <int PASS>
__global__ void __launch_bounds__(256) k_fold_alf(const __grid_constant__ GuardArgs a) {
  if (!(*(volatile unsigned*)a.fold & 16u)) return;
  const Dims d = a.d;
  int i, j, k;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; interior_cell(d, t, i, j, k);
       t += (long)gridDim.x * blockDim.x) {
    const size_t c = d.at(i, j, k);
    const float arho = a.f[0][c] + a.f[10][c] + a.f[20][c] + a.smallbit;
    const float x = a.btot[c] / sqrtf(arho);
    const unsigned pos = (unsigned)(t + 1);
    if (PASS == 0) {
      if (isnan(x)) atomicMax(a.fold + 5, pos);
    } else if (pos > *(volatile unsigned*)(a.fold + 5)) {
      atomicMax(a.fold + 10, x == 0.0f ? 0u : __float_as_uint(x));
      atomicOr(a.fold + 11, 16u);
    }
  }
}

__global__ void __launch_bounds__(256) k_guard_scatter(const __grid_constant__ ScatterArgs a) {
  const unsigned n = min(*a.list_count, a.list_cap);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const float* v = a.list + (size_t)e * 11;
    const unsigned w = __float_as_uint(v[0]);
    const size_t c = w >> 2;
    const int b = 10 * (int)(w & 3u);
#pragma unroll
    for (int q = 0; q < 10; q++) a.f[b + q][c] = v[1 + q];
  }
}

__global__ void __launch_bounds__(256) k_copy(float* __restrict__ dst, const float* __restrict__ src, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    dst[c] = src[c];
}

}  // namespace

void launch_guards(const GuardArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2), grd = grid3(a.d, blk);
  k_guards<<<grd, blk, 0, s>>>(a);
}

void launch_guard_fold_species(const GuardArgs& a, cudaStream_t s) {
  k_fold_species<0><<<sm_count(), 256, 0, s>>>(a);
  k_fold_species<1><<<sm_count(), 256, 0, s>>>(a);
}

void launch_guard_fold_alf(const GuardArgs& a, cudaStream_t s) {
  k_fold_alf<0><<<sm_count(), 256, 0, s>>>(a);
  k_fold_alf<1><<<sm_count(), 256, 0, s>>>(a);
}

void launch_guard_scatter(const ScatterArgs& a, cudaStream_t s) {
  k_guard_scatter<<<sm_count(), 256, 0, s>>>(a);
}

void launch_copy(float* dst, const float* src, size_t n, cudaStream_t s) {
  const unsigned cap = 8u * sm_count();
  k_copy<<<blocks_for(n, 256) < cap ? blocks_for(n, 256) : cap, 256, 0, s>>>(dst, src, n);
}

}  // namespace g3m3
