// k_fields.cu -- current, velocities and Ohm's-law E:
//   calcur      sub_calcur.f90:5-189  (+ bs = b0 + b, btot, 3d_main.f90:2248-2254)
//   fnd_evel    sub_fnd_evel.f90:4-57
//   BandE       sub_BandE.f90:5-162
//   fnd_pres    sub_fnd_pres.f90:5-67
//
// The reference fills the faces, edges and corners of curx/efld by a chain
// of copies (faces from the interior, edges from faces, corners from edges).
// Followed through, every boundary value is the interior value at the
// clamped index (min(max(i,2),n-1) per axis); the six curx corners that the
// reference averages are averages of equal values, evaluated here in the
// same order.  A boundary thread therefore evaluates the interior formula at
// its clamped source point, and one launch fills the whole array.
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

template <bool POW2>
__device__ __forceinline__ void curl_at(const CurrentArgs& a, int i, int j, int k, float& cx,
                                        float& cy, float& cz) {
  const Dims d = a.d;
  const size_t c = d.at(i, j, k);
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * (size_t)d.ny;
  const float dxt = 2.0f * a.rx, dyt = 2.0f * a.ry, dzt = 2.0f * a.rz;
  const float* __restrict__ bx = a.b[0];
  const float* __restrict__ by = a.b[1];
  const float* __restrict__ bz = a.b[2];
  cx = dvd<POW2>(__ldg(bz + c + sy) - __ldg(bz + c - sy), dyt, 1.0f / dyt)
       - dvd<POW2>(__ldg(by + c + sz) - __ldg(by + c - sz), dzt, 1.0f / dzt);
  cy = dvd<POW2>(__ldg(bx + c + sz) - __ldg(bx + c - sz), dzt, 1.0f / dzt)
       - dvd<POW2>(__ldg(bz + c + 1) - __ldg(bz + c - 1), dxt, 1.0f / dxt);
  cz = dvd<POW2>(__ldg(by + c + 1) - __ldg(by + c - 1), dxt, 1.0f / dxt)
       - dvd<POW2>(__ldg(bx + c + sy) - __ldg(bx + c - sy), dyt, 1.0f / dyt);
}

template <bool POW2>
__global__ void __launch_bounds__(256) k_current(const __grid_constant__ CurrentArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.at(i, j, k);
  const int si = clampi(i, 2, d.nx - 1), sj = clampi(j, 2, d.ny - 1), sk = clampi(k, 2, d.nz - 1);
  float cx, cy, cz;
  curl_at<POW2>(a, si, sj, sk, cx, cy, cz);
  // corner averages (sub_calcur.f90:326-351)
  const bool xl = i == 1, xh = i == d.nx, yl = j == 1, yh = j == d.ny, zl = k == 1, zh = k == d.nz;
  if (xl && zh && (yl || yh)) {
    cx = (cx + cx) / 2.0f; cy = (cy + cy) / 2.0f; cz = (cz + cz) / 2.0f;
  } else if (xh && (yl || yh) && (zl || zh)) {
    cx = (cx + cx + cx) / 3.0f; cy = (cy + cy + cy) / 3.0f; cz = (cz + cz + cz) / 3.0f;
  }
  a.cur[0][c] = cx;
  a.cur[1][c] = cy;
  a.cur[2][c] = cz;
  if (a.b0[0]) {
    const float sx = __ldg(a.b0[0] + c) + __ldg(a.b[0] + c);
    const float sy = __ldg(a.b0[1] + c) + __ldg(a.b[1] + c);
    const float sz = __ldg(a.b0[2] + c) + __ldg(a.b[2] + c);
    a.bs[0][c] = sx;
    a.bs[1][c] = sy;
    a.bs[2][c] = sz;
    a.btot[c] = amax1(sqrtf(sx * sx + sy * sy + sz * sz), a.smallbit);
  }
}

__global__ void __launch_bounds__(256) k_total_b(const float* __restrict__ bx, const float* __restrict__ by,
                                                 const float* __restrict__ bz, const float* __restrict__ b0x,
                                                 const float* __restrict__ b0y, const float* __restrict__ b0z,
                                                 float* bsx, float* bsy, float* bsz, float* btot, float smallbit,
                                                 size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const float sx = __ldg(b0x + c) + __ldg(bx + c);
    const float sy = __ldg(b0y + c) + __ldg(by + c);
    const float sz = __ldg(b0z + c) + __ldg(bz + c);
    bsx[c] = sx; bsy[c] = sy; bsz[c] = sz;
    btot[c] = amax1(sqrtf(sx * sx + sy * sy + sz * sz), smallbit);
  }
}

__global__ void __launch_bounds__(256) k_evel(const __grid_constant__ EvelArgs a) {
  const size_t n = a.d.cells();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const float rq = __ldg(a.rho[0] + c), rh = __ldg(a.rho[1] + c), ro = __ldg(a.rho[2] + c);
    const float tden = rq + rh + ro;
    float tv[3];
#pragma unroll
    for (int q = 0; q < 3; q++)
      tv[q] = (__ldg(a.p[0][q] + c) + __ldg(a.p[1][q] + c) + __ldg(a.p[2][q] + c)) / tden;
    if (a.ev[0]) {
      const float qden = (rq + 0.000001f) / a.rmass[0];
      const float hden = (rh + 0.000001f) / a.rmass[1];
      const float oden = (ro + 0.000001f) / a.rmass[2];
      const float tot = qden + hden + oden;
#pragma unroll
      for (int q = 0; q < 3; q++) a.ev[q][c] = tv[q] - __ldg(a.cur[q] + c) / tot / a.reynolds;
    }
#pragma unroll
    for (int q = 0; q < 3; q++) a.tv[q][c] = tv[q];
  }
}

// E at an interior point: Ohm's law, grad p_e, and the resistive term where
// rst_e is nonzero.
template <bool POW2>
__device__ __forceinline__ void efield_at(const BandEArgs& a, int i, int j, int k, float& ex, float& ey,
                                          float& ez) {
  const Dims d = a.d;
  const size_t c = d.at(i, j, k);
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * (size_t)d.ny;
  const float avx = __ldg(a.ev[0] + c), avy = __ldg(a.ev[1] + c), avz = __ldg(a.ev[2] + c);
  const float abx = __ldg(a.bs[0] + c), aby = __ldg(a.bs[1] + c), abz = __ldg(a.bs[2] + c);
  ex = -(avy * abz - avz * aby);
  ey = -(avz * abx - avx * abz);
  ez = -(avx * aby - avy * abx);
  const float rq = __ldg(a.rho[0] + c), rh = __ldg(a.rho[1] + c), ro = __ldg(a.rho[2] + c);
  const float arho = (rq / a.rmass[0] + rh / a.rmass[1] + ro / a.rmass[2]) * a.reynolds;
  const float dxt = 2.0f * a.rx, dyt = 2.0f * a.ry, dzt = 2.0f * a.rz;
  const float* __restrict__ ep = a.epres;
  ex = ex - dvd<POW2>(__ldg(ep + c + 1) - __ldg(ep + c - 1), dxt, 1.0f / dxt) / arho;
  ey = ey - dvd<POW2>(__ldg(ep + c + sy) - __ldg(ep + c - sy), dyt, 1.0f / dyt) / arho;
  ez = ez - dvd<POW2>(__ldg(ep + c + sz) - __ldg(ep + c - sz), dzt, 1.0f / dzt) / arho;
  if (a.rst_e) {
    const float r = __ldg(a.rst_e + c);
    if (r != 0.0f) {
      const float eden = (rq / a.rmass[0] + rh / a.rmass[1] + ro / a.rmass[2]);
      ex = ex + r * __ldg(a.cur[0] + c) / eden;
      ey = ey + r * __ldg(a.cur[1] + c) / eden;
      ez = ez + r * __ldg(a.cur[2] + c) / eden;
    }
  }
}

template <bool POW2>
__global__ void __launch_bounds__(256) k_bande(const __grid_constant__ BandEArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  float ex, ey, ez;
  efield_at<POW2>(a, clampi(i, 2, d.nx - 1), clampi(j, 2, d.ny - 1), clampi(k, 2, d.nz - 1), ex, ey, ez);
  const size_t c = d.at(i, j, k);
  a.efld[0][c] = ex;
  a.efld[1][c] = ey;
  a.efld[2][c] = ez;
}

// Interior-only E (no face copies): used by the per-routine entry point,
// which then applies the list scatter and the face copies like the reference.
template <bool POW2>
__global__ void __launch_bounds__(256) k_bande_interior(const __grid_constant__ BandEArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.at(i, j, k);
  if (i == 1 || j == 1 || k == 1 || i == d.nx || j == d.ny || k == d.nz) {
    const float avx = __ldg(a.ev[0] + c), avy = __ldg(a.ev[1] + c), avz = __ldg(a.ev[2] + c);
    const float abx = __ldg(a.bs[0] + c), aby = __ldg(a.bs[1] + c), abz = __ldg(a.bs[2] + c);
    a.efld[0][c] = -(avy * abz - avz * aby);
    a.efld[1][c] = -(avz * abx - avx * abz);
    a.efld[2][c] = -(avx * aby - avy * abx);
    return;
  }
  float ex, ey, ez;
  efield_at<POW2>(a, i, j, k, ex, ey, ez);
  a.efld[0][c] = ex;
  a.efld[1][c] = ey;
  a.efld[2][c] = ez;
}

// Entry m of a list: E += rst J / n at its cell (sub_BandE.f90:88-116).
__device__ void bande_entry(const BandEListArgs& a, int m) {
  const int i = a.ij[(a.box - 1) + (size_t)a.mbndry * (0 + 3 * (size_t)m)];
  const int j = a.ij[(a.box - 1) + (size_t)a.mbndry * (1 + 3 * (size_t)m)];
  const int k = a.ij[(a.box - 1) + (size_t)a.mbndry * (2 + 3 * (size_t)m)];
  if (i < 1 || j < 1 || k < 1 || i > a.d.nx || j > a.d.ny || k > a.d.nz) return;
  const size_t c = a.d.at(i, j, k);
  const float eden = (__ldg(a.rho[0] + c) / a.rmass[0] + __ldg(a.rho[1] + c) / a.rmass[1]
                      + __ldg(a.rho[2] + c) / a.rmass[2]);
  const float r = __ldg(a.rst + c);
  a.efld[0][c] = a.efld[0][c] + r * __ldg(a.cur[0] + c) / eden;
  a.efld[1][c] = a.efld[1][c] + r * __ldg(a.cur[1] + c) / eden;
  a.efld[2][c] = a.efld[2][c] + r * __ldg(a.cur[2] + c) / eden;
}

// One thread per entry when the list names each cell once; otherwise one
// thread walks the list in order, as the reference does.
__global__ void k_bande_list(const __grid_constant__ BandEListArgs a) {
  if (a.serial) {
    if (blockIdx.x == 0 && threadIdx.x == 0)
      for (int m = 0; m < a.count; m++) bande_entry(a, m);
    return;
  }
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < a.count) bande_entry(a, m);
}

// Face copies of sub_BandE.f90:124-159: boundary = value at the clamped index.
__global__ void __launch_bounds__(256) k_clamp_faces(float* ex, float* ey, float* ez, Dims d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  if (!(i == 1 || j == 1 || k == 1 || i == d.nx || j == d.ny || k == d.nz)) return;
  const size_t c = d.at(i, j, k);
  const size_t s = d.at(clampi(i, 2, d.nx - 1), clampi(j, 2, d.ny - 1), clampi(k, 2, d.nz - 1));
  ex[c] = ex[s];
  ey[c] = ey[s];
  ez[c] = ez[s];
}

__global__ void __launch_bounds__(256) k_fnd_pres(const float* __restrict__ px, const float* __restrict__ py,
                                                  const float* __restrict__ pz, float* p_para, float* p_perp,
                                                  float* p_cross, const float* __restrict__ vx,
                                                  const float* __restrict__ vy, const float* __restrict__ vz,
                                                  const float* __restrict__ bx, const float* __restrict__ by,
                                                  const float* __restrict__ bz, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const float presx = px[c], presy = py[c], presz = pz[c];
    const float presmag = sqrtf(presx * presx + presy * presy + presz * presz) + 1.e-11f;
    const float abx = bx[c], aby = by[c], abz = bz[c];
    const float bmag = sqrtf(abx * abx + aby * aby + abz * abz) + 1.e-12f;
    const float avx = vx[c], avy = vy[c], avz = vz[c];
    const float vcbx = (avy * abz - avz * aby) / bmag;
    const float vcby = -(avx * abz - avz * abx) / bmag;
    const float vcbz = (avx * aby - avy * abx) / bmag;
    const float vcmag = sqrtf(vcbx * vcbx + vcby * vcby + vcbz * vcbz) + 1.e-12f;
    const float a1 = abx * presx, a2 = aby * presy, a3 = abz * presz;
    const float para = sqrtf(a1 * a1 + a2 * a2 + a3 * a3) / bmag;
    const float b1 = vcbx * presx, b2 = vcby * presy, b3 = vcbz * presz;
    const float cross = sqrtf(b1 * b1 + b2 * b2 + b3 * b3) / vcmag;
    p_para[c] = para;
    p_cross[c] = cross;
    p_perp[c] = sqrtf(fabsf(presmag * presmag - (para * para + cross * cross)));
  }
}

}  // namespace

void launch_current(const CurrentArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2), grd = grid3(a.d, blk);
  if (is_pow2(2.0f * a.rx) && is_pow2(2.0f * a.ry) && is_pow2(2.0f * a.rz))
    k_current<true><<<grd, blk, 0, s>>>(a);
  else
    k_current<false><<<grd, blk, 0, s>>>(a);
}

void launch_total_b(const float* const b[3], const float* const b0[3], float* const bs[3], float* btot,
                    float smallbit, const Dims& d, cudaStream_t s) {
  const size_t n = d.cells();
  k_total_b<<<blocks_for(n, 256), 256, 0, s>>>(b[0], b[1], b[2], b0[0], b0[1], b0[2], bs[0], bs[1], bs[2],
                                               btot, smallbit, n);
}

void launch_evel(const EvelArgs& a, cudaStream_t s) {
  k_evel<<<blocks_for(a.d.cells(), 256), 256, 0, s>>>(a);
}

void launch_bande(const BandEArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2), grd = grid3(a.d, blk);
  const bool p2 = is_pow2(2.0f * a.rx) && is_pow2(2.0f * a.ry) && is_pow2(2.0f * a.rz);
  if (p2) k_bande<true><<<grd, blk, 0, s>>>(a);
  else k_bande<false><<<grd, blk, 0, s>>>(a);
}

void launch_bande_interior(const BandEArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2), grd = grid3(a.d, blk);
  const bool p2 = is_pow2(2.0f * a.rx) && is_pow2(2.0f * a.ry) && is_pow2(2.0f * a.rz);
  if (p2) k_bande_interior<true><<<grd, blk, 0, s>>>(a);
  else k_bande_interior<false><<<grd, blk, 0, s>>>(a);
}

void launch_bande_list(const BandEListArgs& a, cudaStream_t s) {
  if (a.count <= 0) return;
  if (a.serial) k_bande_list<<<1, 1, 0, s>>>(a);
  else k_bande_list<<<blocks_for((size_t)a.count, 128), 128, 0, s>>>(a);
}

void launch_bande_faces(float* const efld[3], const Dims& d, cudaStream_t s) {
  const dim3 blk(32, 4, 2), grd = grid3(d, blk);
  k_clamp_faces<<<grd, blk, 0, s>>>(efld[0], efld[1], efld[2], d);
}

void launch_fnd_pres(const float* const pr[3], float* p_para, float* p_perp, float* p_cross,
                     const float* const v[3], const float* const b[3], const Dims& d, cudaStream_t s) {
  const size_t n = d.cells();
  k_fnd_pres<<<blocks_for(n, 256), 256, 0, s>>>(pr[0], pr[1], pr[2], p_para, p_perp, p_cross, v[0], v[1],
                                                v[2], b[0], b[1], b[2], n);
}

}  // namespace g3m3
