// k_fcsmooth.cu -- flux correction, fcsmooth (sub_fcsmooth.f90:7-242),
// staged through shared memory.
//
// A block owns a TX x TY tile of one field and marches along z.  Shared
// memory holds rings of old planes (halo 3, 4 slots), wrk planes (halo 2, 4
// slots) and diffused planes P1 = wrk + chi*Lap7(old) (halo 2, 3 slots).  At
// front plane kf a block computes P1(kf) and emits output plane k = kf-2:
// the x and y limiter fluxes read P1 and wrk of plane k from the rings, the
// z fluxes read per-thread register windows P1(k-2..k+2), wrk(k-1..k+1).
// The global loads of old(kf+2) and wrk(kf+1) are issued into registers at
// the top of the iteration and stored into their ring slots after the
// compute, so their latency overlaps a whole plane of work; each cell of
// wrk and old is read from HBM once and each output written once (12 bytes
// per cell per field).  The arithmetic is the reference's, operation for
// operation, including its end rules (copied end differences and end
// fluxes).
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

constexpr int TX = 32, TY = 8, NT = TX * TY;
constexpr int OX = TX + 6, OY = TY + 6;   // old, halo 3
constexpr int PX = TX + 4, PY = TY + 4;   // P1 and wrk, halo 2
constexpr int NO = OX * OY, NP = PX * PY;
constexpr int RO = (NO + NT - 1) / NT;   // old elements per thread and plane
constexpr int RP = (NP + NT - 1) / NT;   // wrk / P1 elements per thread and plane

__device__ __forceinline__ float limiter(float dw, float d1m, float d1p, float chi) {
  const float s = sign1(dw);
  return s * amax1(0.0f, amin1(amin1(s * d1m, chi * fabsf(dw)), s * d1p));
}

__global__ void __launch_bounds__(NT) k_fcsmooth_tiled(const __grid_constant__ FcsArgs a) {
  __shared__ float sO[4][NO];
  __shared__ float sW[4][NP];
  __shared__ float sP[3][NP];
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

  // register windows of this thread's column
  float p_m2 = 0.0f, p_m1 = 0.0f, p_0 = 0.0f, p_p1 = 0.0f, p_p2 = 0.0f;   // P1(k-2..k+2)
  float w_m1 = 0.0f, w_0 = 0.0f, w_p1 = 0.0f;                            // wrk(k-1..k+1)
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
    __syncthreads();
    // slide the column windows: P1(kf) and wrk(k+1) enter
    const int k = kf - 2;
    const int cc = (ty + 2) * PX + tx + 2;   // this thread's cell in the halo-2 frame
    p_m2 = p_m1; p_m1 = p_0; p_0 = p_p1; p_p1 = p_p2;
    p_p2 = (kf <= nz) ? sP[kf % 3][cc] : 0.0f;
    w_m1 = w_0; w_0 = w_p1;
    w_p1 = (k + 1 >= 1 && k + 1 <= nz) ? sW[(k + 1) & 3][cc] : 0.0f;
    if (mine && k >= 1) {
      const size_t c = (size_t)(k - 1) * plane + (size_t)(gj - 1) * nx + (gi - 1);
      if (k == 1 || k == nz) {
        out[c] = w_0;
      } else {
        const float* P = sP[k % 3];
        const float* Wp = sW[k & 3];
        // x pass (sub_fcsmooth.f90:279-327)
        float tv;
        if (gi == 1 || gi == nx) {
          tv = Wp[cc];
        } else {
          // limiter flux at index m (2..nx-1) of this row; P1 and wrk offsets
          // relative to the output cell
          auto fx = [&](int m) {
            const int o = cc + (m - gi);
            const float dw = Wp[o + 1] - Wp[o];
            const float d1m = P[o] - P[o - 1];
            const float d1p = (m + 1 <= nx - 1) ? P[o + 2] - P[o + 1] : P[o + 1] - P[o];
            return limiter(dw, d1m, d1p, chi);
          };
          const float f0 = fx(gi);
          const float f1 = fx(gi - 1 < 2 ? 2 : gi - 1);
          tv = P[cc] - f0 + f1;
        }
        // y pass (:331-381)
        if (gj != 1 && gj != ny) {
          auto fy = [&](int m) {
            const int o = cc + (m - gj) * PX;
            const float dw = Wp[o + PX] - Wp[o];
            const float d1m = P[o] - P[o - PX];
            const float d1p = (m + 1 <= ny - 1) ? P[o + 2 * PX] - P[o + PX] : P[o + PX] - P[o];
            return limiter(dw, d1m, d1p, chi);
          };
          const float f0 = fy(gj);
          const float f1 = fy(gj - 1 < 2 ? 2 : gj - 1);
          tv = tv - f0 + f1;
        }
        // z pass (:385-431) from the column windows
        const float d1p_k = (k + 1 <= nz - 1) ? p_p2 - p_p1 : p_p1 - p_0;
        const float fz0 = limiter(w_p1 - w_0, p_0 - p_m1, d1p_k, chi);
        float fz1;
        if (k - 1 >= 2) fz1 = limiter(w_0 - w_m1, p_m1 - p_m2, p_p1 - p_0, chi);
        else fz1 = fz0;   // fnz(1) = fnz(2)
        out[c] = tv - fz0 + fz1;
      }
    }
    // the prefetched planes go to slots no reader of this iteration uses
    store_O(kf + 2, rO);
    store_W(kf + 1, rW);
    __syncthreads();
  }
}

}  // namespace

void launch_fcsmooth_tiled(const FcsArgs& a, cudaStream_t s) {
  const dim3 blk(TX, TY, 1);
  const dim3 grd((unsigned)((a.d.nx + TX - 1) / TX), (unsigned)((a.d.ny + TY - 1) / TY), (unsigned)a.nf);
  k_fcsmooth_tiled<<<grd, blk, 0, s>>>(a);
}

}  // namespace g3m3
