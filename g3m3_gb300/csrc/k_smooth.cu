// k_smooth.cu -- Lapidus smoothing and flux correction:
//   lap_plasma  sub_lap_plasma.f90:4-147   lap_elec  sub_lap_elec.f90:4-51
//   lap_bfld    sub_lap_bfld.f90:4-67      fnd_vtot  sub_fnd_vtot.f90:4-41
//   fcsmooth    sub_fcsmooth.f90:7-242     (flux_correct: sub_flux_correct.f90)
//
// fcsmooth: the reference makes ~20 full-array passes per field (diffused
// copy, three difference arrays, three limiter arrays, the running temp).
// Each output value depends only on a radius-2 cross of the diffused field
// P1 = wrk + chi*Lap7(old) and a radius-1 cross of wrk, so one thread
// evaluates the whole chain for its cell, with the reference's edge rules
// (copied end differences and end fluxes) applied per axis.
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

__device__ __forceinline__ float lap_one(const float* __restrict__ f, size_t c, size_t sy, size_t sz,
                                         float chi, float delt, float uxp1, float uxm1, float uyp1,
                                         float uym1, float uzp1, float uzm1) {
  const float f0 = __ldg(f + c);
  return f0 + chi * (delt * (uxp1 * (__ldg(f + c + 1) - f0) - uxm1 * (f0 - __ldg(f + c - 1)))
                     + delt * (uyp1 * (__ldg(f + c + sy) - f0) - uym1 * (f0 - __ldg(f + c - sy)))
                     + delt * (uzp1 * (__ldg(f + c + sz) - f0) - uzm1 * (f0 - __ldg(f + c - sz))));
}

__global__ void __launch_bounds__(256) k_lap(const __grid_constant__ LapArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 2;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 2;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 2;
  if (i > d.nx - 1 || j > d.ny - 1 || k > d.nz - 1) return;
  const size_t c = d.at(i, j, k);
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * (size_t)d.ny;
  float vx0, vxp, vxm, vy0, vyp, vym, vz0, vzp, vzm;
  if (a.vrho) {
    // v = p / max(rho, floor) (3d_main.f90:2698-2748), evaluated where needed
    const float* __restrict__ r = a.vrho;
    auto inv = [&](size_t q) { return amax1(__ldg(r + q), a.vfloor); };
    const float r0 = inv(c);
    vx0 = __ldg(a.vp[0] + c) / r0; vy0 = __ldg(a.vp[1] + c) / r0; vz0 = __ldg(a.vp[2] + c) / r0;
    vxp = __ldg(a.vp[0] + c + 1) / inv(c + 1);
    vxm = __ldg(a.vp[0] + c - 1) / inv(c - 1);
    vyp = __ldg(a.vp[1] + c + sy) / inv(c + sy);
    vym = __ldg(a.vp[1] + c - sy) / inv(c - sy);
    vzp = __ldg(a.vp[2] + c + sz) / inv(c + sz);
    vzm = __ldg(a.vp[2] + c - sz) / inv(c - sz);
  } else {
    vx0 = __ldg(a.v[0] + c); vxp = __ldg(a.v[0] + c + 1); vxm = __ldg(a.v[0] + c - 1);
    vy0 = __ldg(a.v[1] + c); vyp = __ldg(a.v[1] + c + sy); vym = __ldg(a.v[1] + c - sy);
    vz0 = __ldg(a.v[2] + c); vzp = __ldg(a.v[2] + c + sz); vzm = __ldg(a.v[2] + c - sz);
  }
  const float uxp1 = fabsf(vxp - vx0), uxm1 = fabsf(vx0 - vxm);
  const float uyp1 = fabsf(vyp - vy0), uym1 = fabsf(vy0 - vym);
  const float uzp1 = fabsf(vzp - vz0), uzm1 = fabsf(vz0 - vzm);
  const float delt = a.delt.get();
  for (int f = 0; f < a.nf; f++)
    a.out[f][c] = lap_one(a.in[f], c, sy, sz, a.chi[f], delt, uxp1, uxm1, uyp1, uym1, uzp1, uzm1);
}

__global__ void __launch_bounds__(256) k_vtot(const __grid_constant__ VtotArgs a) {
  const size_t n = a.d.cells();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const float tden = __ldg(a.rho[0] + c) + __ldg(a.rho[1] + c) + __ldg(a.rho[2] + c);
#pragma unroll
    for (int q = 0; q < 3; q++)
      a.v[q][c] = (__ldg(a.p[0][q] + c) + __ldg(a.p[1][q] + c) + __ldg(a.p[2][q] + c)) / tden;
  }
}

// ---------------------------------------------------------------- fcsmooth
struct Fcs {
  const float* __restrict__ W;
  const float* __restrict__ O;
  float chi;
  Dims d;
  size_t sy, sz;

  // P1 = W + chi*Lap7(O) in the interior, W on the boundary (:226-275)
  __device__ __forceinline__ float p1(int i, int j, int k) const {
    const size_t c = d.at(i, j, k);
    if (i == 1 || j == 1 || k == 1 || i == d.nx || j == d.ny || k == d.nz) return __ldg(W + c);
    return __ldg(W + c) + chi * (__ldg(O + c + 1) + __ldg(O + c - 1) + __ldg(O + c + sy) + __ldg(O + c - sy)
                                 + __ldg(O + c + sz) + __ldg(O + c - sz) - 6.0f * __ldg(O + c));
  }
  __device__ __forceinline__ float w(int i, int j, int k) const { return __ldg(W + d.at(i, j, k)); }
};

// limiter flux along one axis at index m (1..n) of the line through (i,j,k)
template <int AX>
__device__ __forceinline__ float fn_axis(const Fcs& s, int i, int j, int k, int m) {
  const int n = AX == 0 ? s.d.nx : (AX == 1 ? s.d.ny : s.d.nz);
  if (m < 2) m = 2;
  if (m > n - 1) m = n - 1;
  auto P = [&](int q) { return AX == 0 ? s.p1(q, j, k) : (AX == 1 ? s.p1(i, q, k) : s.p1(i, j, q)); };
  auto Wl = [&](int q) { return AX == 0 ? s.w(q, j, k) : (AX == 1 ? s.w(i, q, k) : s.w(i, j, q)); };
  auto d1 = [&](int q) { if (q > n - 1) q = n - 1; return P(q + 1) - P(q); };
  const float dw = Wl(m + 1) - Wl(m);
  const float sg = sign1(dw);
  return sg * amax1(0.0f, amin1(amin1(sg * d1(m - 1), s.chi * fabsf(dw)), sg * d1(m + 1)));
}

__global__ void __launch_bounds__(256) k_fcsmooth(const __grid_constant__ FcsArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int kz = blockIdx.z * blockDim.z + threadIdx.z;
  const int kt = (d.nz + blockDim.z - 1) / blockDim.z * blockDim.z;  // threads per field along z
  const int f = kz / kt;
  const int k = kz % kt + 1;
  if (f >= a.nf || i > d.nx || j > d.ny || k > d.nz) return;
  Fcs s;
  s.W = a.wrk[f]; s.O = a.old[f]; s.chi = a.chi[f]; s.d = d;
  s.sy = (size_t)d.nx; s.sz = (size_t)d.nx * (size_t)d.ny;
  const size_t c = d.at(i, j, k);
  if (k == 1 || k == d.nz) {
    a.px[f][c] = __ldg(s.W + c);
    return;
  }
  // x pass (:279-327)
  float t;
  if (i == 1 || i == d.nx) t = s.w(i, j, k);
  else t = s.p1(i, j, k) - fn_axis<0>(s, i, j, k, i) + fn_axis<0>(s, i, j, k, i - 1);
  // y pass (:331-381)
  if (j != 1 && j != d.ny) t = t - fn_axis<1>(s, i, j, k, j) + fn_axis<1>(s, i, j, k, j - 1);
  // z pass (:385-431)
  a.px[f][c] = t - fn_axis<2>(s, i, j, k, k) + fn_axis<2>(s, i, j, k, k - 1);
}

}  // namespace

void launch_lap(const LapArgs& a, cudaStream_t s) {
  Dims in{a.d.nx - 2, a.d.ny - 2, a.d.nz - 2};
  const dim3 blk(32, 4, 2), grd = grid3(in, blk);
  k_lap<<<grd, blk, 0, s>>>(a);
}

void launch_vtot(const VtotArgs& a, cudaStream_t s) {
  k_vtot<<<blocks_for(a.d.cells(), 256), 256, 0, s>>>(a);
}

void launch_fcsmooth_tiled(const FcsArgs& a, cudaStream_t s, int variant);

void launch_fcsmooth(const FcsArgs& a, cudaStream_t s) { launch_fcsmooth_tiled(a, s, a.variant); }

// One thread per cell re-deriving every intermediate: kept as the simple
// statement of the algorithm (not launched by the library).
void launch_fcsmooth_percell(const FcsArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2);
  const unsigned kt = (unsigned)((a.d.nz + blk.z - 1) / blk.z);
  const dim3 grd((unsigned)((a.d.nx + blk.x - 1) / blk.x), (unsigned)((a.d.ny + blk.y - 1) / blk.y),
                 kt * (unsigned)a.nf);
  k_fcsmooth<<<grd, blk, 0, s>>>(a);
}

}  // namespace g3m3
