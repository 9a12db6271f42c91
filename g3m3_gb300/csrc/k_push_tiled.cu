// k_push_tiled.cu -- push_ion (sub_push_ion.f90:4-362) staged through
// shared memory.
//
// A block owns a TX x TY tile and marches along z.  For every plane it
// stages the 13 fields that push_ion differentiates (the source state's
// rho, px, py, pz and six pressures, and bs) together with the species
// velocity v = p / max(rho, 1e-6) -- computed once per cell, as the
// reference's pre-pass does (:67-81) -- in a 3-plane ring with a halo of
// one cell.  The seven-point neighbours then come from shared memory and
// the centre-only inputs (old state, btot, efld, tv) straight from HBM, so
// each input is read from HBM about once.  The arithmetic is the per-cell
// kernel's (k_push.cu), operation for operation.
#include "device.cuh"
#include "kargs.cuh"
#include "launch.cuh"

// Built twice.  The default object keeps the reference's FP32 operation
// order bit for bit (no contraction, quotients correctly rounded).  With
// G3M3_CONTRACTED (and -fmad=true) the same kernel goes to the namespace
// g3m3::contracted: products and sums contract to fused multiply-adds and a
// quotient by a shared denominator is a product with its reciprocal
// (within 1.5 ulp); the engine runs it when the model's contracted flavour
// is on (g3m3_model_set_contracted).
#ifdef G3M3_CONTRACTED
#define QUOT(x_, d_, r_) ((x_) * (r_))
#else
#define QUOT(x_, d_, r_) div_by((x_), (d_), (r_))
#endif

namespace g3m3 {
#ifdef G3M3_CONTRACTED
namespace contracted {
#endif

namespace {

constexpr int TX = 32, TY = 8;
constexpr int HX = TX + 2, HY = TY + 2;

constexpr int NLOAD = 13;           // src 0..9, bs 0..2
constexpr int NF = NLOAD + 3;       // + velocity x, y, z
constexpr int VX = 13, VY = 14, VZ = 15;
constexpr size_t SMEM = sizeof(float) * 3 * NF * HY * HX;

__device__ __forceinline__ float& S(float* sm, int slot, int f, int ly, int lx) {
  return sm[((slot * NF + f) * HY + ly) * HX + lx];
}

// Centre-only inputs of one cell.
struct PushCentre {
  float old[10], bt, e[3], tv[3];
};

__device__ __forceinline__ void load_centre(const PushIonArgs& a, size_t c, PushCentre& cin) {
#pragma unroll
  for (int f = 0; f < 10; f++) cin.old[f] = __ldg(a.old[f] + c);
  cin.bt = __ldg(a.btot + c);
#pragma unroll
  for (int q = 0; q < 3; q++) cin.e[q] = __ldg(a.efld[q] + c);
#pragma unroll
  for (int q = 0; q < 3; q++) cin.tv[q] = __ldg(a.tv[q] + c);
}

// Scalars of one launch.
struct PushConst {
  float delt, dxt, dyt, dzt, rdx, rdy, rdz, bmax, rey, r_bmax, r_rmass;
};

__device__ __forceinline__ PushConst push_const(const PushIonArgs& a) {
  PushConst q;
  q.delt = a.delt.get();
  q.dxt = 2.0f * a.g.dx; q.dyt = 2.0f * a.g.dy; q.dzt = 2.0f * a.g.dz;
  q.rdx = 1.0f / q.dxt; q.rdy = 1.0f / q.dyt; q.rdz = 1.0f / q.dzt;
  q.bmax = 0.20f * a.rmass / q.delt / a.reynolds;
  q.rey = a.reynolds;
  q.r_bmax = 1.0f / q.bmax; q.r_rmass = 1.0f / a.rmass;
  return q;
}

// The push of one interior cell (sub_push_ion.f90:107-356) from three
// staged planes [NF][HY][HX] (below, own, above) and the centre-only
// inputs; the ten results in the reference's field order.
template <bool POW2>
__device__ __forceinline__ void push_cell(const float* __restrict__ Plm, const float* __restrict__ Pl0,
                                          const float* __restrict__ Plp, int tx, int ty, int gi, int gj, int k,
                                          const PushCentre& cin, const PushIonArgs& a, const PushConst& q,
                                          float* o) {
  const float delt = q.delt;
  const float dxt = q.dxt, dyt = q.dyt, dzt = q.dzt, rdx = q.rdx, rdy = q.rdy, rdz = q.rdz;
  const float bmax = q.bmax, rey = q.rey, r_bmax = q.r_bmax, r_rmass = q.r_rmass;
  constexpr float r12 = 1.0f / 12.0f;
#define DV(a_, d_, rd_) dvd<POW2>((a_), (d_), (rd_))
  const int ly = ty + 1, lx = tx + 1;
  // field f at the centre and the six neighbours
  auto C0 = [&](int f) { return Pl0[(f * HY + ly) * HX + lx]; };
  auto XP = [&](int f) { return Pl0[(f * HY + ly) * HX + lx + 1]; };
  auto XM = [&](int f) { return Pl0[(f * HY + ly) * HX + lx - 1]; };
  auto YP = [&](int f) { return Pl0[(f * HY + ly + 1) * HX + lx]; };
  auto YM = [&](int f) { return Pl0[(f * HY + ly - 1) * HX + lx]; };
  auto ZP = [&](int f) { return Plp[(f * HY + ly) * HX + lx]; };
  auto ZM = [&](int f) { return Plm[(f * HY + ly) * HX + lx]; };
  auto fluxdiv = [&](int f) -> float {
    return (DV(XP(f) * XP(VX) - XM(f) * XM(VX), dxt, rdx) + DV(YP(f) * YP(VY) - YM(f) * YM(VY), dyt, rdy))
           + DV(ZP(f) * ZP(VZ) - ZM(f) * ZM(VZ), dzt, rdz);
  };
  const float old0 = cin.old[0], old1 = cin.old[1], old2 = cin.old[2], old3 = cin.old[3], old4 = cin.old[4];
  const float old5 = cin.old[5], old6 = cin.old[6], old7 = cin.old[7], old8 = cin.old[8], old9 = cin.old[9];
  const float bt = cin.bt;
  const float e0 = cin.e[0], e1 = cin.e[1], e2 = cin.e[2];
  const float tvx = cin.tv[0], tvy = cin.tv[1], tvz = cin.tv[2];

  const float o_rho = old0 - delt * ((DV(XP(1) - XM(1), dxt, rdx) + DV(YP(2) - YM(2), dyt, rdy))
                                     + DV(ZP(3) - ZM(3), dzt, rdz));
  const float aqpx = old1 - delt * fluxdiv(1);
  const float aqpy = old2 - delt * fluxdiv(2);
  const float aqpz = old3 - delt * fluxdiv(3);
  float abx = C0(10), aby = C0(11), abz = C0(12);
  float bmag = bt;
  const float weight = amax1(1.0f, QUOT(bmag, bmax, r_bmax));
  const float skin_depth = rey / weight;
  const float tcx = (tvy * abz - tvz * aby);
  const float tcy = -(tvx * abz - tvz * abx);
  const float tcz = (tvx * aby - tvy * abx);
  const float v0x = C0(VX), v0y = C0(VY), v0z = C0(VZ);
  const float qcx = (v0y * abz - v0z * aby);
  const float qcy = -(v0x * abz - v0z * abx);
  const float qcz = (v0x * aby - v0y * abx);
  const float gpx = DV(XP(4) - XM(4), dxt, rdx) + DV(YP(7) - YM(7), dxt, rdx) + DV(ZP(8) - ZM(8), dxt, rdx);
  const float gpy = DV(XP(7) - XM(7), dxt, rdx) + DV(YP(5) - YM(5), dyt, rdy) + DV(ZP(9) - ZM(9), dxt, rdx);
  const float gpz = DV(XP(8) - XM(8), dxt, rdx) + DV(YP(9) - YM(9), dyt, rdy) + DV(ZP(6) - ZM(6), dzt, rdz);
  const float dex = (e0 + tcx) * rey;
  const float dey = (e1 + tcy) * rey;
  const float dez = (e2 + tcz) * rey;
  const float dvx = (qcx - tcx) * skin_depth;
  const float dvy = (qcy - tcy) * skin_depth;
  const float dvz = (qcz - tcz) * skin_depth;
  const float rho_c = C0(0);
  const float qden = QUOT(rho_c, a.rmass, r_rmass);
  const float npx = aqpx + delt * (qden * (dex + dvx) - gpx);
  const float npy = aqpy + delt * (qden * (dey + dvy) - gpy);
  const float npz = aqpz + delt * (qden * (dez + dvz) - gpz);
  const float ax = a.g.xmin + a.g.dx * (float)(gi - 1);
  const float ay = a.g.ymin + a.g.dy * (float)(gj - 1);
  const float az = a.g.zmin + a.g.dz * (float)(k - 1);
  const float radius = sqrtf(ax * ax + ay * ay + az * az) + 0.0000001f;
  const float rr = a.re_equiv * radius;
  const float g = delt * rho_c * a.grav / (rr * rr);
  const float r_radius = 1.0f / radius;
  const float o_px = npx - QUOT(g * ax, radius, r_radius);
  const float o_py = npy - QUOT(g * ay, radius, r_radius);
  const float o_pz = npz - QUOT(g * az, radius, r_radius);

  const float wx = C0(4), wy = C0(5), wz = C0(6), wxy = C0(7), wxz = C0(8), wyz = C0(9);
  const float t2 = 2.0f * delt;
  const float px_ = old4 - delt * fluxdiv(4) - DV(t2 * wx * (XP(VX) - XM(VX)), dxt, rdx);
  const float py_ = old5 - delt * fluxdiv(5) - DV(t2 * wy * (YP(VY) - YM(VY)), dyt, rdy);
  const float pz_ = old6 - delt * fluxdiv(6) - DV(t2 * wz * (ZP(VZ) - ZM(VZ)), dzt, rdz);
  abx = QUOT(6.0f * abx + XP(10) + XM(10) + YP(10) + YM(10) + ZP(10) + ZM(10), 12.0f, r12);
  aby = QUOT(6.0f * aby + XP(11) + XM(11) + YP(11) + YM(11) + ZP(11) + ZM(11), 12.0f, r12);
  abz = QUOT(6.0f * abz + XP(12) + XM(12) + YP(12) + YM(12) + ZP(12) + ZM(12), 12.0f, r12);
  bmag = sqrtf(abx * abx + aby * aby + abz * abz);
  float skin = rey;
  if (bmag > bmax) skin = rey * (bmax / bmag);
  const float gy2 = QUOT(t2 * skin, a.rmass, r_rmass);
  const float o_xx = px_ - DV(t2 * wxy * (YP(VX) - YM(VX)), dyt, rdy) - DV(t2 * wxz * (ZP(VX) - ZM(VX)), dzt, rdz)
                     + gy2 * (wxy * abz - wxz * aby);
  const float o_yy = py_ - DV(t2 * wxy * (XP(VY) - XM(VY)), dxt, rdx) - DV(t2 * wyz * (ZP(VY) - ZM(VY)), dzt, rdz)
                     + gy2 * (wyz * abx - wxy * abz);
  const float o_zz = pz_ - DV(t2 * wxz * (XP(VZ) - XM(VZ)), dxt, rdx) - DV(t2 * wyz * (YP(VZ) - YM(VZ)), dyt, rdy)
                     + gy2 * (wxz * aby - wyz * abx);
  const float gy1 = QUOT(delt * skin, a.rmass, r_rmass);
  const float o_xy = old7 - delt * fluxdiv(7)
                     - delt * wxy * (DV(XP(VX) - XM(VX), dxt, rdx) + DV(YP(VY) - YM(VY), dyt, rdy))
                     - DV(delt * wy * (YP(VX) - YM(VX)), dyt, rdy)
                     - DV(delt * wx * (XP(VY) - XM(VY)), dxt, rdx)
                     - DV(delt * wyz * (ZP(VX) - ZM(VX)), dzt, rdz)
                     - DV(delt * wxz * (ZP(VY) - ZM(VY)), dzt, rdz)
                     + gy1 * (abz * (wy - wx) - aby * wyz + abx * wxz);
  const float o_xz = old8 - delt * fluxdiv(8)
                     - delt * wxz * (DV(XP(VX) - XM(VX), dxt, rdx) + DV(ZP(VZ) - ZM(VZ), dzt, rdz))
                     - DV(delt * wz * (ZP(VX) - ZM(VX)), dzt, rdz)
                     - DV(delt * wx * (XP(VZ) - XM(VZ)), dxt, rdx)
                     - DV(delt * wyz * (YP(VX) - YM(VX)), dyt, rdy)
                     - DV(delt * wxy * (YP(VZ) - YM(VZ)), dyt, rdy)
                     + gy1 * (aby * (wx - wz) - abx * wxy + abz * wyz);
  const float o_yz = old9 - delt * fluxdiv(9)
                     - delt * wyz * (DV(YP(VY) - YM(VY), dyt, rdy) + DV(ZP(VZ) - ZM(VZ), dzt, rdz))
                     - DV(delt * wy * (YP(VZ) - YM(VZ)), dyt, rdy)
                     - DV(delt * wz * (ZP(VY) - ZM(VY)), dzt, rdz)
                     - DV(delt * wxy * (XP(VZ) - XM(VZ)), dxt, rdx)
                     - DV(delt * wxz * (XP(VY) - XM(VY)), dxt, rdx)
                     + gy1 * (abx * (wz - wy) - abz * wxz + aby * wxy);
  o[0] = o_rho; o[1] = o_px; o[2] = o_py; o[3] = o_pz;
  o[4] = o_xx; o[5] = o_yy; o[6] = o_zz;
  o[7] = o_xy; o[8] = o_xz; o[9] = o_yz;
#undef DV
}

template <bool POW2>
__global__ void __launch_bounds__(TX* TY, 3) k_push_ion_tiled(const __grid_constant__ PushIonArgs a, int kchunk) {
  extern __shared__ float sm[];
  const Dims d = a.d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX + 1, j0 = blockIdx.y * TY + 1;
  const int gi = i0 + tx, gj = j0 + ty;
  const bool mine = gi <= nx && gj <= ny;
  const bool inner_col = gi >= 2 && gi <= nx - 1 && gj >= 2 && gj <= ny - 1;
  const size_t plane = (size_t)nx * ny;

  const float* src[NLOAD];
#pragma unroll
  for (int f = 0; f < 10; f++) src[f] = a.src[f];
  src[10] = a.bs[0]; src[11] = a.bs[1]; src[12] = a.bs[2];

  auto load_plane = [&](int kp) {
    const int slot = kp % 3;
    for (int t = tid; t < HX * HY; t += TX * TY) {
      const int ly = t / HX, lx = t % HX;
      const int i = i0 - 1 + lx, j = j0 - 1 + ly;
      float v[NLOAD];
      if (kp >= 1 && kp <= nz && i >= 1 && i <= nx && j >= 1 && j <= ny) {
        const size_t c = (size_t)(kp - 1) * plane + (size_t)(j - 1) * nx + (i - 1);
#pragma unroll
        for (int f = 0; f < NLOAD; f++) v[f] = __ldg(src[f] + c);
        const float r = amax1(v[0], 1.e-6f);
        const float rr = 1.0f / r;
        S(sm, slot, VX, ly, lx) = QUOT(v[1], r, rr);
        S(sm, slot, VY, ly, lx) = QUOT(v[2], r, rr);
        S(sm, slot, VZ, ly, lx) = QUOT(v[3], r, rr);
      } else {
#pragma unroll
        for (int f = 0; f < NLOAD; f++) v[f] = 0.0f;
        S(sm, slot, VX, ly, lx) = 0.0f;
        S(sm, slot, VY, ly, lx) = 0.0f;
        S(sm, slot, VZ, ly, lx) = 0.0f;
      }
#pragma unroll
      for (int f = 0; f < NLOAD; f++) S(sm, slot, f, ly, lx) = v[f];
    }
  };

  auto copy_old = [&](int k) {   // boundary cells of cur take the start-of-step state
    if (!a.boundary_from_old || !mine) return;
    const size_t c = (size_t)(k - 1) * plane + (size_t)(gj - 1) * nx + (gi - 1);
#pragma unroll
    for (int f = 0; f < 10; f++) a.out[f][c] = __ldg(a.old[f] + c);
  };

  // this block's planes: [k_lo, k_hi] of the interior 2..nz-1
  const int k_lo = 2 + (int)blockIdx.z * kchunk;
  const int k_hi = min(nz - 1, k_lo + kchunk - 1);
  if (k_lo > k_hi) return;
  if (blockIdx.z == 0) copy_old(1);
  if (k_hi == nz - 1) copy_old(nz);
  load_plane(k_lo - 1);
  load_plane(k_lo);
  const PushConst q = push_const(a);
  for (int k = k_lo; k <= k_hi; k++) {
    load_plane(k + 1);
    __syncthreads();
    if (mine && !inner_col) {
      copy_old(k);
    } else if (inner_col) {
      const size_t c = (size_t)(k - 1) * plane + (size_t)(gj - 1) * nx + (gi - 1);
      PushCentre cin;
      load_centre(a, c, cin);
      float o[10];
      push_cell<POW2>(sm + (size_t)((k - 1) % 3) * NF * HY * HX, sm + (size_t)(k % 3) * NF * HY * HX,
                      sm + (size_t)((k + 1) % 3) * NF * HY * HX, tx, ty, gi, gj, k, cin, a, q, o);
#pragma unroll
      for (int f = 0; f < 10; f++) a.out[f][c] = o[f];
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t prepare_push_ion() {
  cudaError_t e = prepare_smem((const void*)k_push_ion_tiled<true>, (int)SMEM);
  if (e == cudaSuccess) e = prepare_smem((const void*)k_push_ion_tiled<false>, (int)SMEM);
  return e;
}

void launch_push_ion_tiled(const PushIonArgs& a, cudaStream_t s) {
  const dim3 blk(TX, TY, 1);
  const int tiles = ((a.d.nx + TX - 1) / TX) * ((a.d.ny + TY - 1) / TY);
  const int interior = a.d.nz - 2;
  // about one resident wave: every SM x 3 blocks (65 KB of shared memory each)
  int chunks = (3 * sm_count() + tiles - 1) / tiles;
  if (chunks > interior) chunks = interior;
  if (chunks < 1) chunks = 1;
  const int kchunk = (interior + chunks - 1) / chunks;
  chunks = (interior + kchunk - 1) / kchunk;
  const dim3 grd((unsigned)((a.d.nx + TX - 1) / TX), (unsigned)((a.d.ny + TY - 1) / TY), (unsigned)chunks);
  // if preparing failed, the launch fails and the caller's check reports it
  prepare_push_ion();
  if (is_pow2(2.0f * a.g.dx) && is_pow2(2.0f * a.g.dy) && is_pow2(2.0f * a.g.dz)) {
    k_push_ion_tiled<true><<<grd, blk, SMEM, s>>>(a, kchunk);
  } else {
    k_push_ion_tiled<false><<<grd, blk, SMEM, s>>>(a, kchunk);
  }
}

#ifdef G3M3_CONTRACTED
}  // namespace contracted
#endif
}  // namespace g3m3
