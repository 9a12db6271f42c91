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

}  // namespace

template <int TY>
static void launch_ty(const FcsArgs& a, cudaStream_t s) {
  const dim3 blk(TX, TY, 1);
  const dim3 grd((unsigned)((a.d.nx + TX - 1) / TX), (unsigned)((a.d.ny + TY - 1) / TY), (unsigned)a.nf);
  k_fcsmooth_tiled<TY><<<grd, blk, 0, s>>>(a);
}

// variant 0: 32x8 tiles, 1: 32x16 tiles
void launch_fcsmooth_tiled(const FcsArgs& a, cudaStream_t s, int variant) {
  if (variant == 1) launch_ty<16>(a, s);
  else launch_ty<8>(a, s);
}

}  // namespace g3m3
