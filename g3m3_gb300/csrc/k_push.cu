// k_push.cu -- Lax-Wendroff pushes: push_ion (sub_push_ion.f90:4-362),
// push_elec (sub_push_elec.f90:4-53) and push_bfld (sub_push_bfld.f90:4-50).
//
// One thread per cell.  push_ion recomputes the species velocity
// v = p / max(rho, 1e-6) at the seven stencil points instead of storing the
// reference's qvx/qvy/qvz pre-pass arrays (same divisions, same bits, no
// extra HBM round trip).
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

struct V3 { float x, y, z; };

__device__ __forceinline__ V3 vel(const float* __restrict__ rho, const float* __restrict__ px,
                                  const float* __restrict__ py, const float* __restrict__ pz,
                                  size_t c) {
  const float r = amax1(__ldg(rho + c), 1.e-6f);
  return V3{__ldg(px + c) / r, __ldg(py + c) / r, __ldg(pz + c) / r};
}

template <bool POW2>
__global__ void __launch_bounds__(256) k_push_ion(const __grid_constant__ PushIonArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.at(i, j, k);
  if (i == 1 || j == 1 || k == 1 || i == d.nx || j == d.ny || k == d.nz) {
    if (a.boundary_from_old)
#pragma unroll
      for (int f = 0; f < 10; f++) a.out[f][c] = __ldg(a.old[f] + c);
    return;
  }
  const float delt = a.delt.get();
  const float dxt = 2.0f * a.g.dx, dyt = 2.0f * a.g.dy, dzt = 2.0f * a.g.dz;
  const float rdx = 1.0f / dxt, rdy = 1.0f / dyt, rdz = 1.0f / dzt;
  const float bmax = 0.20f * a.rmass / delt / a.reynolds;
  const size_t sx = 1, sy = (size_t)d.nx, sz = (size_t)d.nx * (size_t)d.ny;
  const size_t xp = c + sx, xm = c - sx, yp = c + sy, ym = c - sy, zp = c + sz, zm = c - sz;

  const float* __restrict__ rho = a.src[0];
  const float* __restrict__ Px = a.src[1];
  const float* __restrict__ Py = a.src[2];
  const float* __restrict__ Pz = a.src[3];
  const V3 v0 = vel(rho, Px, Py, Pz, c);
  const V3 vxp = vel(rho, Px, Py, Pz, xp), vxm = vel(rho, Px, Py, Pz, xm);
  const V3 vyp = vel(rho, Px, Py, Pz, yp), vym = vel(rho, Px, Py, Pz, ym);
  const V3 vzp = vel(rho, Px, Py, Pz, zp), vzm = vel(rho, Px, Py, Pz, zm);

#define DV(a_, d_, rd_) dvd<POW2>((a_), (d_), (rd_))
  // flux divergence of field f with the species velocity
  auto fluxdiv = [&](const float* __restrict__ f) -> float {
    return (DV(__ldg(f + xp) * vxp.x - __ldg(f + xm) * vxm.x, dxt, rdx)
            + DV(__ldg(f + yp) * vyp.y - __ldg(f + ym) * vym.y, dyt, rdy))
           + DV(__ldg(f + zp) * vzp.z - __ldg(f + zm) * vzm.z, dzt, rdz);
  };

  // continuity
  const float o_rho = __ldg(a.old[0] + c) - delt * ((DV(__ldg(Px + xp) - __ldg(Px + xm), dxt, rdx)
                                               + DV(__ldg(Py + yp) - __ldg(Py + ym), dyt, rdy))
                                              + DV(__ldg(Pz + zp) - __ldg(Pz + zm), dzt, rdz));
  const float aqpx = __ldg(a.old[1] + c) - delt * fluxdiv(Px);
  const float aqpy = __ldg(a.old[2] + c) - delt * fluxdiv(Py);
  const float aqpz = __ldg(a.old[3] + c) - delt * fluxdiv(Pz);

  const float* __restrict__ Wx = a.src[4];
  const float* __restrict__ Wy = a.src[5];
  const float* __restrict__ Wz = a.src[6];
  const float* __restrict__ Wxy = a.src[7];
  const float* __restrict__ Wxz = a.src[8];
  const float* __restrict__ Wyz = a.src[9];
  const float* __restrict__ Bx = a.bs[0];
  const float* __restrict__ By = a.bs[1];
  const float* __restrict__ Bz = a.bs[2];

  float abx = __ldg(Bx + c), aby = __ldg(By + c), abz = __ldg(Bz + c);
  float bmag = __ldg(a.btot + c);
  const float weight = amax1(1.0f, bmag / bmax);
  const float skin_depth = a.reynolds / weight;
  const float tvx = __ldg(a.tv[0] + c), tvy = __ldg(a.tv[1] + c), tvz = __ldg(a.tv[2] + c);
  const float tcx = (tvy * abz - tvz * aby);
  const float tcy = -(tvx * abz - tvz * abx);
  const float tcz = (tvx * aby - tvy * abx);
  const float qcx = (v0.y * abz - v0.z * aby);
  const float qcy = -(v0.x * abz - v0.z * abx);
  const float qcz = (v0.x * aby - v0.y * abx);
  // the reference divides the y/z derivatives of the off-diagonal terms by
  // dxt here; the spacings are equal within a box
  const float gpx = DV(__ldg(Wx + xp) - __ldg(Wx + xm), dxt, rdx)
                    + DV(__ldg(Wxy + yp) - __ldg(Wxy + ym), dxt, rdx)
                    + DV(__ldg(Wxz + zp) - __ldg(Wxz + zm), dxt, rdx);
  const float gpy = DV(__ldg(Wxy + xp) - __ldg(Wxy + xm), dxt, rdx)
                    + DV(__ldg(Wy + yp) - __ldg(Wy + ym), dyt, rdy)
                    + DV(__ldg(Wyz + zp) - __ldg(Wyz + zm), dxt, rdx);
  const float gpz = DV(__ldg(Wxz + xp) - __ldg(Wxz + xm), dxt, rdx)
                    + DV(__ldg(Wyz + yp) - __ldg(Wyz + ym), dyt, rdy)
                    + DV(__ldg(Wz + zp) - __ldg(Wz + zm), dzt, rdz);
  const float rey = a.reynolds;
  const float dex = (__ldg(a.efld[0] + c) + tcx) * rey;
  const float dey = (__ldg(a.efld[1] + c) + tcy) * rey;
  const float dez = (__ldg(a.efld[2] + c) + tcz) * rey;
  const float dvx = (qcx - tcx) * skin_depth;
  const float dvy = (qcy - tcy) * skin_depth;
  const float dvz = (qcz - tcz) * skin_depth;
  const float rho_c = __ldg(rho + c);
  const float qden = rho_c / a.rmass;
  const float npx = aqpx + delt * (qden * (dex + dvx) - gpx);
  const float npy = aqpy + delt * (qden * (dey + dvy) - gpy);
  const float npz = aqpz + delt * (qden * (dez + dvz) - gpz);
  // gravity
  const float ax = a.g.xmin + a.g.dx * (float)(i - 1);
  const float ay = a.g.ymin + a.g.dy * (float)(j - 1);
  const float az = a.g.zmin + a.g.dz * (float)(k - 1);
  const float radius = sqrtf(ax * ax + ay * ay + az * az) + 0.0000001f;
  const float rr = a.re_equiv * radius;
  const float g = delt * rho_c * a.grav / (rr * rr);
  const float o_px = npx - g * ax / radius;
  const float o_py = npy - g * ay / radius;
  const float o_pz = npz - g * az / radius;

  const float wx = __ldg(Wx + c), wy = __ldg(Wy + c), wz = __ldg(Wz + c);
  const float wxy = __ldg(Wxy + c), wxz = __ldg(Wxz + c), wyz = __ldg(Wyz + c);
  const float t2 = 2.0f * delt;
  const float px_ = __ldg(a.old[4] + c) - delt * fluxdiv(Wx) - DV(t2 * wx * (vxp.x - vxm.x), dxt, rdx);
  const float py_ = __ldg(a.old[5] + c) - delt * fluxdiv(Wy) - DV(t2 * wy * (vyp.y - vym.y), dyt, rdy);
  const float pz_ = __ldg(a.old[6] + c) - delt * fluxdiv(Wz) - DV(t2 * wz * (vzp.z - vzm.z), dzt, rdz);

  // gyro term with the 12-point smoothed field
  abx = (6.0f * abx + __ldg(Bx + xp) + __ldg(Bx + xm) + __ldg(Bx + yp) + __ldg(Bx + ym)
         + __ldg(Bx + zp) + __ldg(Bx + zm)) / 12.0f;
  aby = (6.0f * aby + __ldg(By + xp) + __ldg(By + xm) + __ldg(By + yp) + __ldg(By + ym)
         + __ldg(By + zp) + __ldg(By + zm)) / 12.0f;
  abz = (6.0f * abz + __ldg(Bz + xp) + __ldg(Bz + xm) + __ldg(Bz + yp) + __ldg(Bz + ym)
         + __ldg(Bz + zp) + __ldg(Bz + zm)) / 12.0f;
  bmag = sqrtf(abx * abx + aby * aby + abz * abz);
  float skin = rey;
  if (bmag > bmax) skin = rey * (bmax / bmag);
  const float gy2 = t2 * skin / a.rmass;
  const float o_xx = px_ - DV(t2 * wxy * (vyp.x - vym.x), dyt, rdy) - DV(t2 * wxz * (vzp.x - vzm.x), dzt, rdz)
                + gy2 * (wxy * abz - wxz * aby);
  const float o_yy = py_ - DV(t2 * wxy * (vxp.y - vxm.y), dxt, rdx) - DV(t2 * wyz * (vzp.y - vzm.y), dzt, rdz)
                + gy2 * (wyz * abx - wxy * abz);
  const float o_zz = pz_ - DV(t2 * wxz * (vxp.z - vxm.z), dxt, rdx) - DV(t2 * wyz * (vyp.z - vym.z), dyt, rdy)
                + gy2 * (wxz * aby - wyz * abx);

  const float gy1 = delt * skin / a.rmass;
  float o_xy, o_xz, o_yz;
  {
    const float p0 = __ldg(a.old[7] + c) - delt * fluxdiv(Wxy);
    o_xy = p0 - delt * wxy * (DV(vxp.x - vxm.x, dxt, rdx) + DV(vyp.y - vym.y, dyt, rdy))
                  - DV(delt * wy * (vyp.x - vym.x), dyt, rdy)
                  - DV(delt * wx * (vxp.y - vxm.y), dxt, rdx)
                  - DV(delt * wyz * (vzp.x - vzm.x), dzt, rdz)
                  - DV(delt * wxz * (vzp.y - vzm.y), dzt, rdz)
                  + gy1 * (abz * (wy - wx) - aby * wyz + abx * wxz);
  }
  {
    const float p0 = __ldg(a.old[8] + c) - delt * fluxdiv(Wxz);
    o_xz = p0 - delt * wxz * (DV(vxp.x - vxm.x, dxt, rdx) + DV(vzp.z - vzm.z, dzt, rdz))
                  - DV(delt * wz * (vzp.x - vzm.x), dzt, rdz)
                  - DV(delt * wx * (vxp.z - vxm.z), dxt, rdx)
                  - DV(delt * wyz * (vyp.x - vym.x), dyt, rdy)
                  - DV(delt * wxy * (vyp.z - vym.z), dyt, rdy)
                  + gy1 * (aby * (wx - wz) - abx * wxy + abz * wyz);
  }
  {
    const float p0 = __ldg(a.old[9] + c) - delt * fluxdiv(Wyz);
    o_yz = p0 - delt * wyz * (DV(vyp.y - vym.y, dyt, rdy) + DV(vzp.z - vzm.z, dzt, rdz))
                  - DV(delt * wy * (vyp.z - vym.z), dyt, rdy)
                  - DV(delt * wz * (vzp.y - vzm.y), dzt, rdz)
                  - DV(delt * wxy * (vxp.z - vxm.z), dxt, rdx)
                  - DV(delt * wxz * (vxp.y - vxm.y), dxt, rdx)
                  + gy1 * (abx * (wz - wy) - abz * wxz + aby * wxy);
  }
  // every load above precedes every store: the output arrays are distinct
  // from the inputs, but the compiler cannot know it through the tables
  a.out[0][c] = o_rho; a.out[1][c] = o_px; a.out[2][c] = o_py; a.out[3][c] = o_pz;
  a.out[4][c] = o_xx; a.out[5][c] = o_yy; a.out[6][c] = o_zz;
  a.out[7][c] = o_xy; a.out[8][c] = o_xz; a.out[9][c] = o_yz;
#undef DV
}

template <bool POW2>
__global__ void __launch_bounds__(256) k_push_field(const __grid_constant__ PushFieldArgs a) {
  const Dims d = a.d;
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y * blockDim.y + threadIdx.y + 1;
  const int k = blockIdx.z * blockDim.z + threadIdx.z + 1;
  if (i > d.nx || j > d.ny || k > d.nz) return;
  const size_t c = d.at(i, j, k);
  if (i == 1 || j == 1 || k == 1 || i == d.nx || j == d.ny || k == d.nz) {
    if (a.boundary_from_old) {
      if (a.do_elec) a.epres[c] = __ldg(a.oldepres + c);
      if (a.do_bfld)
        for (int q = 0; q < 3; q++) a.b[q][c] = __ldg(a.oldb[q] + c);
    }
    return;
  }
  const float delt = a.delt.get();
  const float dxt = 2.0f * a.rx, dyt = 2.0f * a.ry, dzt = 2.0f * a.rz;
  const float rdx = 1.0f / dxt, rdy = 1.0f / dyt, rdz = 1.0f / dzt;
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * (size_t)d.ny;
  const size_t xp = c + 1, xm = c - 1, yp = c + sy, ym = c - sy, zp = c + sz, zm = c - sz;
#define DV(a_, d_, rd_) dvd<POW2>((a_), (d_), (rd_))
  if (a.do_elec) {
    const float* __restrict__ w = a.wrkepres;
    const float* __restrict__ ex = a.ev[0];
    const float* __restrict__ ey = a.ev[1];
    const float* __restrict__ ez = a.ev[2];
    const float gx = DV(__ldg(w + xp) - __ldg(w + xm), dxt, rdx);
    const float gy = DV(__ldg(w + yp) - __ldg(w + ym), dyt, rdy);
    const float gz = DV(__ldg(w + zp) - __ldg(w + zm), dzt, rdz);
    const float e = __ldg(a.oldepres + c)
                    - delt * a.gamma * ((DV(__ldg(w + xp) * __ldg(ex + xp) - __ldg(w + xm) * __ldg(ex + xm), dxt, rdx)
                                         + DV(__ldg(w + yp) * __ldg(ey + yp) - __ldg(w + ym) * __ldg(ey + ym), dyt, rdy))
                                        + DV(__ldg(w + zp) * __ldg(ez + zp) - __ldg(w + zm) * __ldg(ez + zm), dzt, rdz));
    a.epres[c] = e + delt * a.gamma1 * (__ldg(ex + c) * gx + __ldg(ey + c) * gy + __ldg(ez + c) * gz);
  }
  if (a.do_bfld) {
    const float* __restrict__ Ex = a.efld[0];
    const float* __restrict__ Ey = a.efld[1];
    const float* __restrict__ Ez = a.efld[2];
    a.b[0][c] = __ldg(a.oldb[0] + c) - delt * (DV(__ldg(Ez + yp) - __ldg(Ez + ym), dyt, rdy)
                                               - DV(__ldg(Ey + zp) - __ldg(Ey + zm), dzt, rdz));
    a.b[1][c] = __ldg(a.oldb[1] + c) + delt * (DV(__ldg(Ez + xp) - __ldg(Ez + xm), dxt, rdx)
                                               - DV(__ldg(Ex + zp) - __ldg(Ex + zm), dzt, rdz));
    a.b[2][c] = __ldg(a.oldb[2] + c) - delt * (DV(__ldg(Ey + xp) - __ldg(Ey + xm), dxt, rdx)
                                               - DV(__ldg(Ex + yp) - __ldg(Ex + ym), dyt, rdy));
  }
#undef DV
}

}  // namespace

void launch_push_ion_tiled(const PushIonArgs& a, cudaStream_t s);
namespace contracted {
void launch_push_ion_tiled(const PushIonArgs& a, cudaStream_t s);
}

void launch_push_ion(const PushIonArgs& a, cudaStream_t s) {
  if (a.contracted) contracted::launch_push_ion_tiled(a, s);
  else launch_push_ion_tiled(a, s);
}

// The per-cell form (every neighbour through the L1 cache): the direct
// statement of the stencil, kept for reference; the tiled kernel replaces it.
void launch_push_ion_percell(const PushIonArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2);
  const dim3 grd = grid3(a.d, blk);
  if (is_pow2(2.0f * a.g.dx) && is_pow2(2.0f * a.g.dy) && is_pow2(2.0f * a.g.dz))
    k_push_ion<true><<<grd, blk, 0, s>>>(a);
  else
    k_push_ion<false><<<grd, blk, 0, s>>>(a);
}

void launch_push_field(const PushFieldArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2);
  const dim3 grd = grid3(a.d, blk);
  if (is_pow2(2.0f * a.rx) && is_pow2(2.0f * a.ry) && is_pow2(2.0f * a.rz))
    k_push_field<true><<<grd, blk, 0, s>>>(a);
  else
    k_push_field<false><<<grd, blk, 0, s>>>(a);
}

}  // namespace g3m3
