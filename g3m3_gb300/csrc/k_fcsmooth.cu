// k_fcsmooth.cu -- flux correction, fcsmooth (sub_fcsmooth.f90:7-242),
// staged through shared memory.
//
// A block owns a TX x TY tile of one field and marches along z.  Shared
// memory holds rings of old planes (halo 3, 4 slots), wrk planes (halo 2, 4
// slots) and diffused planes P1 = wrk + chi*Lap7(old) (halo 2, 3 slots).  At
// front plane kf a block computes P1(kf), the x and y limiter fluxes of
// plane kf-1 and the output plane k = kf-2.  Each face flux is evaluated
// once: a thread computes the flux on its own +x and +y faces; the -x face
// comes from the neighbouring lane (a tile row is one warp), the -y face
// from the row above through shared memory, and the tile's left and top
// edge faces from two extra passes.  The z flux of the face below is the
// previous plane's upper flux, kept in a register, and the z terms read
// register windows P1(k-2..k+2), wrk(k-1..k+1).  The global loads of
// old(kf+2) and wrk(kf+1) are issued into registers at the top of the
// iteration and stored into their ring slots after the compute.  Each cell
// of wrk and old is read from HBM once and each output written once (12
// bytes per cell per field).  The arithmetic is the reference's, operation
// for operation, including its end rules (copied end differences and end
// fluxes).
#include <type_traits>

#include "device.cuh"
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

constexpr int TX = 32;   // one warp per tile row

__device__ __forceinline__ float limiter(float dw, float d1m, float d1p, float chi) {
  const float s = sign1(dw);
  return s * amax1(0.0f, amin1(amin1(s * d1m, chi * fabsf(dw)), s * d1p));
}

// flux at face m (between m and m+1) along a line of n cells; o is the
// shared-memory index of cell m and st the stride along the line
__device__ __forceinline__ float face_flux(const float* P, const float* Wp, int o, int st, int m, int n, float chi) {
  const float dw = Wp[o + st] - Wp[o];
  const float d1m = P[o] - P[o - st];
  const float d1p = (m + 1 <= n - 1) ? P[o + 2 * st] - P[o + st] : P[o + st] - P[o];
  return limiter(dw, d1m, d1p, chi);
}

template <int TY>
__global__ void __launch_bounds__(TX * TY) k_fcsmooth_tiled(const __grid_constant__ FcsArgs a) {
  constexpr int NT = TX * TY;
  constexpr int OX = TX + 6, OY = TY + 6;   // old, halo 3
  constexpr int PX = TX + 4, PY = TY + 4;   // P1 and wrk, halo 2
  constexpr int NO = OX * OY, NP = PX * PY;
  constexpr int RO = (NO + NT - 1) / NT;    // old elements per thread and plane
  constexpr int RP = (NP + NT - 1) / NT;    // wrk / P1 elements per thread and plane
  __shared__ float sO[4][NO];
  __shared__ float sW[4][NP];
  __shared__ float sP[3][NP];
  __shared__ float sFy[2][TY + 1][TX];   // y fluxes: row 0 the tile's top edge face, row r+1 row r's +y face
  __shared__ float sFx[2][TY];           // x flux of each row's left edge face
  const Dims d = a.d;
  const int f = blockIdx.z;
  const float* __restrict__ W = a.wrk[f];
  const float* __restrict__ O = a.old[f];
  float* __restrict__ out = a.px[f];
  const float chi = a.chi[f];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX + 1, j0 = blockIdx.y * TY + 1;   // global index of tile cell (0,0)
  const int gi = i0 + tx, gj = j0 + ty;
  const bool mine = gi <= d.nx && gj <= d.ny;
  const size_t plane = (size_t)d.nx * d.ny;
  const int nx = d.nx, ny = d.ny, nz = d.nz;

  // per-thread element tables, the same for every plane: in-plane offset of
  // each staged cell (-1: outside the box or the tile frame)
  int oofs[RO];
#pragma unroll
  for (int r = 0; r < RO; r++) {
    const int t = tid + r * NT;
    const int i = i0 - 3 + t % OX, j = j0 - 3 + t / OX;
    oofs[r] = (t < NO && i >= 1 && i <= nx && j >= 1 && j <= ny) ? (j - 1) * nx + (i - 1) : -1;
  }
  int wofs[RP], pO[RP];
  bool pedge[RP];
#pragma unroll
  for (int r = 0; r < RP; r++) {
    const int t = tid + r * NT;
    const int lx = t % PX, ly = t / PX;
    const int i = i0 - 2 + lx, j = j0 - 2 + ly;
    wofs[r] = (t < NP && i >= 1 && i <= nx && j >= 1 && j <= ny) ? (j - 1) * nx + (i - 1) : -1;
    pO[r] = (ly + 1) * OX + lx + 1;   // the same cell in the halo-3 frame
    pedge[r] = i == 1 || i == nx || j == 1 || j == ny;
  }
  auto fetch_O = [&](int kp, float* v) {
#pragma unroll
    for (int r = 0; r < RO; r++)
      v[r] = (kp >= 1 && kp <= nz && oofs[r] >= 0) ? __ldg(O + (size_t)(kp - 1) * plane + oofs[r]) : 0.0f;
  };
  auto fetch_W = [&](int kp, float* v) {
#pragma unroll
    for (int r = 0; r < RP; r++)
      v[r] = (kp >= 1 && kp <= nz && wofs[r] >= 0) ? __ldg(W + (size_t)(kp - 1) * plane + wofs[r]) : 0.0f;
  };
  auto store_O = [&](int kp, const float* v) {
#pragma unroll
    for (int r = 0; r < RO; r++)
      if (tid + r * NT < NO) sO[kp & 3][tid + r * NT] = v[r];
  };
  auto store_W = [&](int kp, const float* v) {
#pragma unroll
    for (int r = 0; r < RP; r++)
      if (tid + r * NT < NP) sW[kp & 3][tid + r * NT] = v[r];
  };

  const int cc = (ty + 2) * PX + tx + 2;   // this thread's cell in the halo-2 frame
  // register windows of this thread's column
  float p_m2 = 0.0f, p_m1 = 0.0f, p_0 = 0.0f, p_p1 = 0.0f, p_p2 = 0.0f;   // P1(k-2..k+2)
  float w_m1 = 0.0f, w_0 = 0.0f, w_p1 = 0.0f;                            // wrk(k-1..k+1)
  float fx_cur = 0.0f, fy_cur = 0.0f;   // own +x / +y face fluxes of the output plane
  float fz_prev = 0.0f;                 // z flux of the face below the output cell
  float rO[RO], rW[RP];

  // prologue: old planes 1 and 2, wrk plane 1
  fetch_O(1, rO); store_O(1, rO);
  fetch_O(2, rO); store_O(2, rO);
  fetch_W(1, rW); store_W(1, rW);
  __syncthreads();
  for (int kf = 1; kf <= nz + 2; kf++) {
    // next planes in flight while this one is computed
    fetch_O(kf + 2, rO);
    fetch_W(kf + 1, rW);
    // P1 of the front plane kf on the tile plus a halo of 2
    if (kf <= nz) {
      float* dP = sP[kf % 3];
      const float* Wk = sW[kf & 3];
      const float* Om = sO[(kf - 1) & 3];
      const float* Oc = sO[kf & 3];
      const float* Op = sO[(kf + 1) & 3];
      const bool zb = kf == 1 || kf == nz;
#pragma unroll
      for (int r = 0; r < RP; r++) {
        const int t = tid + r * NT;
        if (t < NP) {
          float v = 0.0f;
          if (wofs[r] >= 0) {
            const float w = Wk[t];
            if (zb || pedge[r]) {
              v = w;
            } else {
              const int q = pO[r];
              v = w + chi * (Oc[q + 1] + Oc[q - 1] + Oc[q + OX] + Oc[q - OX] + Op[q] + Om[q] - 6.0f * Oc[q]);
            }
          }
          dP[t] = v;
        }
      }
    }
    // x and y face fluxes of plane kx = kf-1 (sub_fcsmooth.f90:279-381);
    // faces outside 2..n-1 give values nobody reads
    const int kx = kf - 1;
    float fx_next = 0.0f, fy_next = 0.0f;
    if (kx >= 2 && kx <= nz - 1) {
      const float* P = sP[kx % 3];
      const float* Wp = sW[kx & 3];
      fx_next = face_flux(P, Wp, cc, 1, gi, nx, chi);
      fy_next = face_flux(P, Wp, cc, PX, gj, ny, chi);
      sFy[kx & 1][ty + 1][tx] = fy_next;
      if (ty == 0) {            // the tile's top edge faces, j0-1
        sFy[kx & 1][0][tx] = face_flux(P, Wp, cc - PX, PX, j0 - 1, ny, chi);
      } else if (ty == 1 && tx < TY) {   // the left edge face i0-1 of row tx
        const int o = (tx + 2) * PX + 1;
        sFx[kx & 1][tx] = face_flux(P, Wp, o, 1, i0 - 1, nx, chi);
      }
    }
    __syncthreads();
    // slide the column windows: P1(kf) and wrk(k+1) enter
    const int k = kf - 2;
    p_m2 = p_m1; p_m1 = p_0; p_0 = p_p1; p_p1 = p_p2;
    p_p2 = (kf <= nz) ? sP[kf % 3][cc] : 0.0f;
    w_m1 = w_0; w_0 = w_p1;
    w_p1 = (k + 1 >= 1 && k + 1 <= nz) ? sW[(k + 1) & 3][cc] : 0.0f;
    // -x face flux from the lane on the left (every lane takes part)
    const float fx_left_lane = __shfl_up_sync(0xffffffffu, fx_cur, 1);
    if (mine && k >= 1) {
      const size_t c = (size_t)(k - 1) * plane + (size_t)(gj - 1) * nx + (gi - 1);
      if (k == 1 || k == nz) {
        out[c] = w_0;
      } else {
        const float* P = sP[k % 3];
        const float* Wp = sW[k & 3];
        // x pass: px - fnx(i) + fnx(i-1), fnx(1) = fnx(2)
        float tv;
        if (gi == 1 || gi == nx) {
          tv = Wp[cc];
        } else {
          const float f0 = fx_cur;
          const float f1 = gi == 2 ? f0 : (tx == 0 ? sFx[k & 1][ty] : fx_left_lane);
          tv = P[cc] - f0 + f1;
        }
        // y pass
        if (gj != 1 && gj != ny) {
          const float f0 = fy_cur;
          const float f1 = gj == 2 ? f0 : sFy[k & 1][ty][tx];
          tv = tv - f0 + f1;
        }
        // z pass (:385-431) from the column windows; the flux of the face
        // below is the previous plane's upper flux (fnz(1) = fnz(2))
        const float d1p_k = (k + 1 <= nz - 1) ? p_p2 - p_p1 : p_p1 - p_0;
        const float fz0 = limiter(w_p1 - w_0, p_0 - p_m1, d1p_k, chi);
        const float fz1 = k == 2 ? fz0 : fz_prev;
        fz_prev = fz0;
        out[c] = tv - fz0 + fz1;
      }
    }
    fx_cur = fx_next;
    fy_cur = fy_next;
    // the prefetched planes go to slots no reader of this iteration uses
    store_O(kf + 2, rO);
    store_W(kf + 1, rW);
    __syncthreads();
  }
}

// ---- two fields per block, packed FP32x2 arithmetic -----------------
// The same algorithm on a pair of fields: shared memory holds the two
// fields' values interleaved, and the pair's FP32 adds and subtracts are
// add/sub.rn.f32x2 (per-lane IEEE round-to-nearest, the scalar code's
// operations in the same order).  Products that feed an add or subtract are
// formed per lane with scalar mul.rn.f32: the code generator may contract a
// packed multiply and a dependent packed add into one fused operation,
// which would change the rounding.  Products that only feed the limiter's
// min/max stay packed.  The limiter's sign, min and max act per lane.
// Fewer FP32 instructions and half the shared-memory loads of the one-field
// form for the same arithmetic.
typedef unsigned long long f2x;

__device__ __forceinline__ f2x pk(float a, float b) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk(f2x v, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
__device__ __forceinline__ f2x add2(f2x a, f2x b) {
  f2x r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2x sub2(f2x a, f2x b) {
  f2x r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
  f2x r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// per-lane scalar products (never contracted with a following add)
__device__ __forceinline__ f2x mul2s(f2x a, f2x b) {
  float a0, a1, b0, b1;
  upk(a, a0, a1);
  upk(b, b0, b1);
  return pk(a0 * b0, a1 * b1);
}
__device__ __forceinline__ f2x ld2(const float2* p) {
  const float2 v = *p;
  return pk(v.x, v.y);
}

__device__ __forceinline__ f2x limiter2(f2x dw, f2x d1m, f2x d1p, f2x chi) {
  float dw0, dw1;
  upk(dw, dw0, dw1);
  const f2x s = pk(sign1(dw0), sign1(dw1));
  float a0, a1, c0, c1, b0, b1;
  upk(mul2(s, d1m), a0, a1);
  upk(mul2(chi, pk(fabsf(dw0), fabsf(dw1))), c0, c1);
  upk(mul2(s, d1p), b0, b1);
  return mul2s(s, pk(amax1(0.0f, amin1(amin1(a0, c0), b0)), amax1(0.0f, amin1(amin1(a1, c1), b1))));
}

__device__ __forceinline__ f2x face_flux2(const float2* P, const float2* Wp, int o, int st, int m, int n, f2x chi) {
  const f2x dw = sub2(ld2(Wp + o + st), ld2(Wp + o));
  const f2x d1m = sub2(ld2(P + o), ld2(P + o - st));
  const f2x d1p = (m + 1 <= n - 1) ? sub2(ld2(P + o + 2 * st), ld2(P + o + st)) : sub2(ld2(P + o + st), ld2(P + o));
  return limiter2(dw, d1m, d1p, chi);
}

template <int TY, int MINB>
__global__ void __launch_bounds__(TX * TY, MINB) k_fcsmooth_pair(const __grid_constant__ FcsArgs a) {
  constexpr int NT = TX * TY;
  constexpr int OX = TX + 6, OY = TY + 6;
  constexpr int PX = TX + 4, PY = TY + 4;
  constexpr int NO = OX * OY, NP = PX * PY;
  constexpr int RO = (NO + NT - 1) / NT;
  constexpr int RP = (NP + NT - 1) / NT;
  __shared__ float2 sO[4][NO];
  __shared__ float2 sW[4][NP];
  __shared__ float2 sP[3][NP];
  __shared__ float2 sFy[2][TY + 1][TX];
  __shared__ float2 sFx[2][TY];
  const Dims d = a.d;
  const int f0 = 2 * blockIdx.z;
  const bool two = f0 + 1 < a.nf;
  const int f1 = two ? f0 + 1 : f0;
  const float* __restrict__ W0 = a.wrk[f0];
  const float* __restrict__ W1 = a.wrk[f1];
  const float* __restrict__ O0 = a.old[f0];
  const float* __restrict__ O1 = a.old[f1];
  const f2x chi = pk(a.chi[f0], a.chi[f1]);
  const f2x six = pk(6.0f, 6.0f);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX + 1, j0 = blockIdx.y * TY + 1;
  const int gi = i0 + tx, gj = j0 + ty;
  const bool mine = gi <= d.nx && gj <= d.ny;
  const size_t plane = (size_t)d.nx * d.ny;
  const int nx = d.nx, ny = d.ny, nz = d.nz;

  int oofs[RO];
#pragma unroll
  for (int r = 0; r < RO; r++) {
    const int t = tid + r * NT;
    const int i = i0 - 3 + t % OX, j = j0 - 3 + t / OX;
    oofs[r] = (t < NO && i >= 1 && i <= nx && j >= 1 && j <= ny) ? (j - 1) * nx + (i - 1) : -1;
  }
  int wofs[RP], pO[RP];
  bool pedge[RP];
#pragma unroll
  for (int r = 0; r < RP; r++) {
    const int t = tid + r * NT;
    const int lx = t % PX, ly = t / PX;
    const int i = i0 - 2 + lx, j = j0 - 2 + ly;
    wofs[r] = (t < NP && i >= 1 && i <= nx && j >= 1 && j <= ny) ? (j - 1) * nx + (i - 1) : -1;
    pO[r] = (ly + 1) * OX + lx + 1;
    pedge[r] = i == 1 || i == nx || j == 1 || j == ny;
  }
  auto fetch_O = [&](int kp, float2* v) {
#pragma unroll
    for (int r = 0; r < RO; r++) {
      v[r] = make_float2(0.0f, 0.0f);
      if (kp >= 1 && kp <= nz && oofs[r] >= 0) {
        const size_t c = (size_t)(kp - 1) * plane + oofs[r];
        v[r] = make_float2(__ldg(O0 + c), __ldg(O1 + c));
      }
    }
  };
  auto fetch_W = [&](int kp, float2* v) {
#pragma unroll
    for (int r = 0; r < RP; r++) {
      v[r] = make_float2(0.0f, 0.0f);
      if (kp >= 1 && kp <= nz && wofs[r] >= 0) {
        const size_t c = (size_t)(kp - 1) * plane + wofs[r];
        v[r] = make_float2(__ldg(W0 + c), __ldg(W1 + c));
      }
    }
  };
  auto store_O = [&](int kp, const float2* v) {
#pragma unroll
    for (int r = 0; r < RO; r++)
      if (tid + r * NT < NO) sO[kp & 3][tid + r * NT] = v[r];
  };
  auto store_W = [&](int kp, const float2* v) {
#pragma unroll
    for (int r = 0; r < RP; r++)
      if (tid + r * NT < NP) sW[kp & 3][tid + r * NT] = v[r];
  };

  const int cc = (ty + 2) * PX + tx + 2;
  const f2x z2 = pk(0.0f, 0.0f);
  f2x p_m2 = z2, p_m1 = z2, p_0 = z2, p_p1 = z2, p_p2 = z2;
  f2x w_m1 = z2, w_0 = z2, w_p1 = z2;
  f2x fx_cur = z2, fy_cur = z2, fz_prev = z2;
  float2 rO[RO], rW[RP];

  fetch_O(1, rO); store_O(1, rO);
  fetch_O(2, rO); store_O(2, rO);
  fetch_W(1, rW); store_W(1, rW);
  __syncthreads();
  for (int kf = 1; kf <= nz + 2; kf++) {
    fetch_O(kf + 2, rO);
    fetch_W(kf + 1, rW);
    if (kf <= nz) {
      float2* dP = sP[kf % 3];
      const float2* Wk = sW[kf & 3];
      const float2* Om = sO[(kf - 1) & 3];
      const float2* Oc = sO[kf & 3];
      const float2* Op = sO[(kf + 1) & 3];
      const bool zb = kf == 1 || kf == nz;
#pragma unroll
      for (int r = 0; r < RP; r++) {
        const int t = tid + r * NT;
        if (t < NP) {
          f2x v = z2;
          if (wofs[r] >= 0) {
            const f2x w = ld2(Wk + t);
            if (zb || pedge[r]) {
              v = w;
            } else {
              const int q = pO[r];
              const f2x sum = add2(add2(add2(add2(add2(ld2(Oc + q + 1), ld2(Oc + q - 1)), ld2(Oc + q + OX)),
                                                ld2(Oc + q - OX)),
                                           ld2(Op + q)),
                                      ld2(Om + q));
              v = add2(w, mul2s(chi, sub2(sum, mul2s(six, ld2(Oc + q)))));
            }
          }
          float lo, hi;
          upk(v, lo, hi);
          dP[t] = make_float2(lo, hi);
        }
      }
    }
    const int kx = kf - 1;
    f2x fx_next = z2, fy_next = z2;
    if (kx >= 2 && kx <= nz - 1) {
      const float2* P = sP[kx % 3];
      const float2* Wp = sW[kx & 3];
      fx_next = face_flux2(P, Wp, cc, 1, gi, nx, chi);
      fy_next = face_flux2(P, Wp, cc, PX, gj, ny, chi);
      float lo, hi;
      upk(fy_next, lo, hi);
      sFy[kx & 1][ty + 1][tx] = make_float2(lo, hi);
      if (ty == 0) {
        upk(face_flux2(P, Wp, cc - PX, PX, j0 - 1, ny, chi), lo, hi);
        sFy[kx & 1][0][tx] = make_float2(lo, hi);
      } else if (ty == 1 && tx < TY) {
        upk(face_flux2(P, Wp, (tx + 2) * PX + 1, 1, i0 - 1, nx, chi), lo, hi);
        sFx[kx & 1][tx] = make_float2(lo, hi);
      }
    }
    __syncthreads();
    const int k = kf - 2;
    p_m2 = p_m1; p_m1 = p_0; p_0 = p_p1; p_p1 = p_p2;
    p_p2 = (kf <= nz) ? ld2(sP[kf % 3] + cc) : z2;
    w_m1 = w_0; w_0 = w_p1;
    w_p1 = (k + 1 >= 1 && k + 1 <= nz) ? ld2(sW[(k + 1) & 3] + cc) : z2;
    const f2x fx_left_lane = __shfl_up_sync(0xffffffffu, fx_cur, 1);
    if (mine && k >= 1) {
      const size_t c = (size_t)(k - 1) * plane + (size_t)(gj - 1) * nx + (gi - 1);
      f2x res;
      if (k == 1 || k == nz) {
        res = w_0;
      } else {
        const float2* P = sP[k % 3];
        const float2* Wp = sW[k & 3];
        f2x tv;
        if (gi == 1 || gi == nx) {
          tv = ld2(Wp + cc);
        } else {
          const f2x fl = gi == 2 ? fx_cur : (tx == 0 ? ld2(&sFx[k & 1][ty]) : fx_left_lane);
          tv = add2(sub2(ld2(P + cc), fx_cur), fl);
        }
        if (gj != 1 && gj != ny) {
          const f2x fl = gj == 2 ? fy_cur : ld2(&sFy[k & 1][ty][tx]);
          tv = add2(sub2(tv, fy_cur), fl);
        }
        const f2x d1p_k = (k + 1 <= nz - 1) ? sub2(p_p2, p_p1) : sub2(p_p1, p_0);
        const f2x fz0 = limiter2(sub2(w_p1, w_0), sub2(p_0, p_m1), d1p_k, chi);
        const f2x fz1 = k == 2 ? fz0 : fz_prev;
        fz_prev = fz0;
        res = add2(sub2(tv, fz0), fz1);
      }
      float lo, hi;
      upk(res, lo, hi);
      a.px[f0][c] = lo;
      if (two) a.px[f1][c] = hi;
    }
    fx_cur = fx_next;
    fy_cur = fy_next;
    store_O(kf + 2, rO);
    store_W(kf + 1, rW);
    __syncthreads();
  }
}

__device__ __forceinline__ void st2(float2* p, f2x v) {
  float lo, hi;
  upk(v, lo, hi);
  *p = make_float2(lo, hi);
}

// face flux with the end rule decided by the caller (inner = m+1 <= n-1)
__device__ __forceinline__ f2x face_flux2i(const float2* P, const float2* Wp, int o, int st, bool inner, f2x chi) {
  const f2x dw = sub2(ld2(Wp + o + st), ld2(Wp + o));
  const f2x d1m = sub2(ld2(P + o), ld2(P + o - st));
  const f2x d1p = inner ? sub2(ld2(P + o + 2 * st), ld2(P + o + st)) : sub2(ld2(P + o + st), ld2(P + o));
  return limiter2(dw, d1m, d1p, chi);
}

// ---- two fields per block, planes copied asynchronously ---------------
// The pair form above, arranged so the march neither waits for a global
// load round trip every plane nor spends its instructions on addresses:
//  * global reads are asynchronous copies into shared memory (cp.async, 4
//    bytes per field and cell, no register staging) issued two plane steps
//    ahead of their first reader: step kf issues old kf+3 and wrk kf+2 as one
//    copy group and, before its barrier, waits for the group of step kf-1
//    (old kf+2, wrk kf+1), which step kf+1's P1 reads;
//  * one barrier per plane: the edge fluxes have four slots (plane mod 4,
//    fixed at compile time, the march being unrolled over the four phases),
//    P1 four or two (its readers -- the next step's fluxes and this step's
//    window load after the barrier -- are done one barrier interval after
//    it is written), old and wrk six or five (plane mod NS, rotated at run
//    time), so no slot is written in the barrier interval in which another
//    step reads it, and a copy into a slot starts at least one barrier after
//    the last read of the plane it held (with five slots: old kf-2, last
//    read by P1(kf-1); wrk kf-3, last read by the output of plane kf-4
//    before step kf-1's barrier);
//  * shared-memory offsets and edge tests are per-thread constants computed
//    before the march; halo cells outside the box are zeroed once in every
//    slot and never copied; the output takes P1(k) and wrk(k) of its own
//    cell from the register windows.
// The arithmetic is the pair form's, operation for operation.
// (The global planes cannot be staged by TMA tensor copies: a row of nx =
// 121 floats is 484 bytes, and tensor strides must be multiples of 16.)
__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

template <int TY, int NS_, int NPS_>
struct PcLayout {
  static constexpr int NT = TX * TY;
  static constexpr int OX = TX + 6, OY = TY + 6;
  static constexpr int PX = TX + 4, PY = TY + 4;
  static constexpr int NO = OX * OY, NP = PX * PY;
  static constexpr int RO = (NO + NT - 1) / NT, RP = (NP + NT - 1) / NT;
  static constexpr int NS = NS_;                             // old / wrk ring slots
  static constexpr int NPS = NPS_;                           // P1 ring slots (2 or 4)
  static constexpr int O_OFF = 0;                            // float2 offsets
  static constexpr int W_OFF = O_OFF + NS * NO;
  static constexpr int P_OFF = W_OFF + NS * NP;
  static constexpr int FY_OFF = P_OFF + NPS * NP;            // [4][TY+1][TX]
  static constexpr int FX_OFF = FY_OFF + 4 * (TY + 1) * TX;  // [4][TY]
  static constexpr size_t BYTES = (size_t)(FX_OFF + 4 * TY) * sizeof(float2);
};

template <int TY, int MINB, int NS_, int NPS_>
__global__ void __launch_bounds__(TX * TY, MINB) k_fcsmooth_pc(const __grid_constant__ FcsArgs a) {
  using L = PcLayout<TY, NS_, NPS_>;
  constexpr int NT = L::NT, OX = L::OX, PX = L::PX, NO = L::NO, NP = L::NP, RO = L::RO, RP = L::RP, NS = L::NS;
  extern __shared__ float2 smem[];
  float2* const sO = smem + L::O_OFF;
  float2* const sW = smem + L::W_OFF;
  float2* const sP = smem + L::P_OFF;
  float2* const sFy = smem + L::FY_OFF;
  float2* const sFx = smem + L::FX_OFF;
  const Dims d = a.d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int f0 = 2 * blockIdx.z;
  const bool two = f0 + 1 < a.nf;
  const int f1 = two ? f0 + 1 : f0;
  const float* __restrict__ W0 = a.wrk[f0];
  const float* __restrict__ W1 = a.wrk[f1];
  const float* __restrict__ O0 = a.old[f0];
  const float* __restrict__ O1 = a.old[f1];
  float* __restrict__ X0 = a.px[f0];
  float* __restrict__ X1 = a.px[f1];
  const f2x chi = pk(a.chi[f0], a.chi[f1]);
  const f2x six = pk(6.0f, 6.0f);
  const f2x z2 = pk(0.0f, 0.0f);
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int i0 = blockIdx.x * TX + 1, j0 = blockIdx.y * TY + 1;
  const int gi = i0 + tx, gj = j0 + ty;
  const bool mine = gi <= nx && gj <= ny;
  const size_t plane = (size_t)nx * ny;
  const uint32_t sO_a = (uint32_t)__cvta_generic_to_shared(sO);
  const uint32_t sW_a = (uint32_t)__cvta_generic_to_shared(sW);

  int oofs[RO];
  bool oin[RO];
#pragma unroll
  for (int r = 0; r < RO; r++) {
    const int t = tid + r * NT;
    const int i = i0 - 3 + t % OX, j = j0 - 3 + t / OX;
    const bool inbox = i >= 1 && i <= nx && j >= 1 && j <= ny;
    oin[r] = t < NO && inbox;
    oofs[r] = (j - 1) * nx + (i - 1);
    if (t < NO && !inbox) {
#pragma unroll
      for (int sl = 0; sl < NS; sl++) sO[sl * NO + t] = make_float2(0.0f, 0.0f);
    }
  }
  int wofs[RP], pO[RP];
  bool win[RP], pint[RP];
#pragma unroll
  for (int r = 0; r < RP; r++) {
    const int t = tid + r * NT;
    const int lx = t % PX, ly = t / PX;
    const int i = i0 - 2 + lx, j = j0 - 2 + ly;
    const bool inbox = i >= 1 && i <= nx && j >= 1 && j <= ny;
    win[r] = t < NP && inbox;
    wofs[r] = (j - 1) * nx + (i - 1);
    pO[r] = (ly + 1) * OX + lx + 1;
    pint[r] = !(i == 1 || i == nx || j == 1 || j == ny);
    if (t < NP && !inbox) {
#pragma unroll
      for (int sl = 0; sl < NS; sl++) sW[sl * NP + t] = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int sl = 0; sl < L::NPS; sl++) sP[sl * NP + t] = make_float2(0.0f, 0.0f);
    }
  }
  const int cc = (ty + 2) * PX + tx + 2;
  const bool xin = gi + 1 <= nx - 1, yin = gj + 1 <= ny - 1;
  const bool xedge = gi == 1 || gi == nx, x2 = gi == 2;
  const bool yint = gj != 1 && gj != ny, y2 = gj == 2;
  const int rowoff = (gj - 1) * nx + (gi - 1);

  // asynchronous copies of one plane into a ring slot (both fields of a cell
  // into the two halves of its float2)
  auto copy_O = [&](int kp, int slot) {
    const float* o0 = O0 + (size_t)(kp - 1) * plane;
    const float* o1 = O1 + (size_t)(kp - 1) * plane;
    const uint32_t base = sO_a + (uint32_t)(slot * NO + tid) * 8u;
#pragma unroll
    for (int r = 0; r < RO; r++)
      if (oin[r]) {
        cp_async4(base + r * NT * 8, o0 + oofs[r]);
        cp_async4(base + r * NT * 8 + 4, o1 + oofs[r]);
      }
  };
  auto copy_W = [&](int kp, int slot) {
    const float* w0 = W0 + (size_t)(kp - 1) * plane;
    const float* w1 = W1 + (size_t)(kp - 1) * plane;
    const uint32_t base = sW_a + (uint32_t)(slot * NP + tid) * 8u;
#pragma unroll
    for (int r = 0; r < RP; r++)
      if (win[r]) {
        cp_async4(base + r * NT * 8, w0 + wofs[r]);
        cp_async4(base + r * NT * 8 + 4, w1 + wofs[r]);
      }
  };

  // prologue: group 1 = old 1, 2 and wrk 1; group 2 = old 3 and wrk 2 (the
  // group a step 0 would have issued); wait for group 1
  copy_O(1, 1 % NS);
  if (2 <= nz) copy_O(2, 2 % NS);
  copy_W(1, 1 % NS);
  cp_async_commit();
  if (3 <= nz) copy_O(3, 3 % NS);
  if (2 <= nz) copy_W(2, 2 % NS);
  cp_async_commit();
  cp_async_wait1();
  __syncthreads();

  f2x p_m1 = z2, p_0 = z2, p_p1 = z2, p_p2 = z2;
  f2x w_0 = z2, w_p1 = z2;
  f2x fx_cur = z2, fy_cur = z2, fz_prev = z2;
  int m6 = 1 % NS;   // kf mod NS

  auto step = [&](auto phase, const int kf) {
    constexpr int PH = decltype(phase)::value;   // kf mod 4: edge-flux slots (and P1 slots mod NPS)
    constexpr int S2 = (PH + 2) & 3, S3 = (PH + 3) & 3;
    constexpr int P0 = PH % L::NPS, P3 = (PH + 3) % L::NPS;   // P1 of planes kf, kf-1
    const int om = m6 == 0 ? NS - 1 : m6 - 1;                 // old kf-1, wrk kf-1
    const int op = m6 == NS - 1 ? 0 : m6 + 1;                 // old kf+1
    const int o3 = m6 + 3 >= NS ? m6 + 3 - NS : m6 + 3;       // old kf+3
    const int w2 = m6 + 2 >= NS ? m6 + 2 - NS : m6 + 2;       // wrk kf+2
    if (kf + 3 <= nz) copy_O(kf + 3, o3);
    if (kf + 2 <= nz) copy_W(kf + 2, w2);
    cp_async_commit();
    if (kf <= nz) {
      const bool zb = kf == 1 || kf == nz;
      const float2* Om = sO + om * NO;
      const float2* Oc = sO + m6 * NO;
      const float2* Op = sO + op * NO;
      const float2* Wk = sW + m6 * NP;
#pragma unroll
      for (int r = 0; r < RP; r++) {
        if (win[r]) {
          const int t = tid + r * NT;
          const f2x w = ld2(Wk + t);
          f2x v = w;
          if (!zb && pint[r]) {
            const int q = pO[r];
            const f2x sum = add2(add2(add2(add2(add2(ld2(Oc + q + 1), ld2(Oc + q - 1)), ld2(Oc + q + OX)),
                                              ld2(Oc + q - OX)),
                                         ld2(Op + q)),
                                    ld2(Om + q));
            v = add2(w, mul2s(chi, sub2(sum, mul2s(six, ld2(Oc + q)))));
          }
          st2(sP + P0 * NP + t, v);
        }
      }
    }
    const int kx = kf - 1;
    const float2* Wx = sW + om * NP;
    f2x fx_next = z2, fy_next = z2;
    if (kx >= 2 && kx <= nz - 1) {
      const float2* P = sP + P3 * NP;
      fx_next = face_flux2i(P, Wx, cc, 1, xin, chi);
      fy_next = face_flux2i(P, Wx, cc, PX, yin, chi);
      st2(sFy + (S3 * (TY + 1) + ty + 1) * TX + tx, fy_next);
      if (ty == 0) {
        st2(sFy + (S3 * (TY + 1)) * TX + tx, face_flux2i(P, Wx, cc - PX, PX, j0 <= ny - 1, chi));
      } else if (ty == 1 && tx < TY) {
        st2(sFx + S3 * TY + tx, face_flux2i(P, Wx, (tx + 2) * PX + 1, 1, i0 <= nx - 1, chi));
      }
    }
    cp_async_wait1();   // the group of step kf-1: old kf+2, wrk kf+1
    __syncthreads();
    const int k = kf - 2;
    p_m1 = p_0; p_0 = p_p1; p_p1 = p_p2;
    p_p2 = (kf <= nz) ? ld2(sP + P0 * NP + cc) : z2;
    w_0 = w_p1;
    w_p1 = (kx >= 1 && kx <= nz) ? ld2(Wx + cc) : z2;
    const f2x fx_left_lane = __shfl_up_sync(0xffffffffu, fx_cur, 1);
    if (mine && k >= 1) {
      f2x res;
      if (k == 1 || k == nz) {
        res = w_0;
      } else {
        f2x tv;
        if (xedge) {
          tv = w_0;
        } else {
          const f2x fl = x2 ? fx_cur : (tx == 0 ? ld2(sFx + S2 * TY + ty) : fx_left_lane);
          tv = add2(sub2(p_0, fx_cur), fl);
        }
        if (yint) {
          const f2x fl = y2 ? fy_cur : ld2(sFy + (S2 * (TY + 1) + ty) * TX + tx);
          tv = add2(sub2(tv, fy_cur), fl);
        }
        const f2x d1p_k = (k + 1 <= nz - 1) ? sub2(p_p2, p_p1) : sub2(p_p1, p_0);
        const f2x fz0 = limiter2(sub2(w_p1, w_0), sub2(p_0, p_m1), d1p_k, chi);
        const f2x fz1 = k == 2 ? fz0 : fz_prev;
        fz_prev = fz0;
        res = add2(sub2(tv, fz0), fz1);
      }
      const size_t c = (size_t)(k - 1) * plane + rowoff;
      float lo, hi;
      upk(res, lo, hi);
      X0[c] = lo;
      if (two) X1[c] = hi;
    }
    fx_cur = fx_next;
    fy_cur = fy_next;
    m6 = op;
  };
  for (int kf = 1; kf <= nz + 2; kf += 4) {
    step(std::integral_constant<int, 1>{}, kf);
    if (kf + 1 <= nz + 2) step(std::integral_constant<int, 2>{}, kf + 1);
    if (kf + 2 <= nz + 2) step(std::integral_constant<int, 3>{}, kf + 2);
    if (kf + 3 <= nz + 2) step(std::integral_constant<int, 0>{}, kf + 3);
  }
  cp_async_wait0();   // no copy outlives the block (all groups past the march are empty)
}

}  // namespace

template <int TY>
static void launch_ty(const FcsArgs& a, cudaStream_t s) {
  const dim3 blk(TX, TY, 1);
  const dim3 grd((unsigned)((a.d.nx + TX - 1) / TX), (unsigned)((a.d.ny + TY - 1) / TY), (unsigned)a.nf);
  k_fcsmooth_tiled<TY><<<grd, blk, 0, s>>>(a);
}

template <int TY, int MINB>
static void launch_pair(const FcsArgs& a, cudaStream_t s) {
  const dim3 blk(TX, TY, 1);
  const dim3 grd((unsigned)((a.d.nx + TX - 1) / TX), (unsigned)((a.d.ny + TY - 1) / TY),
                 (unsigned)((a.nf + 1) / 2));
  k_fcsmooth_pair<TY, MINB><<<grd, blk, 0, s>>>(a);
}

template <int TY, int MINB, int NS_, int NPS_>
static cudaError_t prepare_pc() {
  return prepare_smem((const void*)k_fcsmooth_pc<TY, MINB, NS_, NPS_>, (int)PcLayout<TY, NS_, NPS_>::BYTES);
}

template <int TY, int MINB, int NS_, int NPS_>
static void launch_pc(const FcsArgs& a, cudaStream_t s) {
  prepare_pc<TY, MINB, NS_, NPS_>();   // if it failed, the launch below fails and the caller's check reports it
  const dim3 blk(TX, TY, 1);
  const dim3 grd((unsigned)((a.d.nx + TX - 1) / TX), (unsigned)((a.d.ny + TY - 1) / TY),
                 (unsigned)((a.nf + 1) / 2));
  k_fcsmooth_pc<TY, MINB, NS_, NPS_><<<grd, blk, PcLayout<TY, NS_, NPS_>::BYTES, s>>>(a);
}

// Dynamic shared-memory limits of the forms that need them on the current
// device (contexts call this at creation, the engine when a variant is
// chosen).
cudaError_t prepare_fcsmooth() {
  cudaError_t e = prepare_pc<8, 3, 6, 4>();
  if (e == cudaSuccess) e = prepare_pc<8, 2, 6, 4>();
  if (e == cudaSuccess) e = prepare_pc<8, 4, 5, 2>();
  if (e == cudaSuccess) e = prepare_pc<16, 2, 5, 2>();
  return e;
}

// variant 0: 32x8 tiles, 1: 32x16 tiles, 2 and 3: 32x8 tiles with two
// fields per block in packed FP32x2 arithmetic, registers bounded for 3 or
// 4 resident blocks per SM; 4 and 5: the two-field form with asynchronous
// plane copies and one barrier per plane, registers bounded for 3 or 2
// blocks per SM (shared memory admits 3); 6: the same with 5-slot old/wrk
// rings and a 2-slot P1 ring (55 KB), 4 blocks per SM; 7: variant 6 on
// 32x16 tiles (fewer halo cells per output, 92 KB, 2 blocks of 512 per SM)
void launch_fcsmooth_tiled(const FcsArgs& a, cudaStream_t s, int variant) {
  if (variant == 1) launch_ty<16>(a, s);
  else if (variant == 2) launch_pair<8, 3>(a, s);
  else if (variant == 3) launch_pair<8, 4>(a, s);
  else if (variant == 4) launch_pc<8, 3, 6, 4>(a, s);
  else if (variant == 5) launch_pc<8, 2, 6, 4>(a, s);
  else if (variant == 6) launch_pc<8, 4, 5, 2>(a, s);
  else if (variant == 7) launch_pc<16, 2, 5, 2>(a, s);
  else launch_ty<8>(a, s);
}

}  // namespace g3m3
