// k_fcsmooth.cu -- flux correction, fcsmooth (sub_fcsmooth.f90:7-242),
// staged through shared memory.
//
// A block owns a TX x TY tile of one field and marches along z.  For the
// front plane kf it stages old(kf+1) (halo 3) in a 3-plane ring, evaluates
// the diffused field P1 = wrk + chi*Lap7(old) once per cell of the tile and
// a halo of 2 (another 3-plane ring), and two planes later emits the output
// plane k = kf-2: the x and y limiter fluxes read P1 and wrk of plane k from
// shared memory, the z fluxes read the per-thread register windows
// P1(k-2..k+2) and wrk(k-1..k+1).  Every cell of wrk and old is read from
// HBM about once and every output written once (12 bytes per cell per
// field); the arithmetic is the reference's, operation for operation,
// including its end rules (copied end differences and end fluxes).
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

constexpr int TX = 32, TY = 8;
constexpr int OX = TX + 6, OY = TY + 6;   // old, halo 3
constexpr int PX = TX + 4, PY = TY + 4;   // P1, halo 2
constexpr int WX = TX + 2, WY = TY + 2;   // wrk, halo 1

__device__ __forceinline__ float limiter(float dw, float d1m, float d1p, float chi) {
  const float s = sign1(dw);
  return s * amax1(0.0f, amin1(amin1(s * d1m, chi * fabsf(dw)), s * d1p));
}

__global__ void __launch_bounds__(TX* TY) k_fcsmooth_tiled(const __grid_constant__ FcsArgs a) {
  __shared__ float sO[3][OY][OX];
  __shared__ float sP[3][PY][PX];
  __shared__ float sW[WY][WX];
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

  auto load_O = [&](int kp) {   // old plane kp into ring slot kp%3, halo 3
    float(*dst)[OX] = sO[(kp + 3) % 3];
    for (int t = tid; t < OX * OY; t += TX * TY) {
      const int ly = t / OX, lx = t % OX;
      const int i = i0 - 3 + lx, j = j0 - 3 + ly;
      float v = 0.0f;
      if (kp >= 1 && kp <= nz && i >= 1 && i <= nx && j >= 1 && j <= ny)
        v = __ldg(O + (size_t)(kp - 1) * plane + (size_t)(j - 1) * nx + (i - 1));
      dst[ly][lx] = v;
    }
  };

  // register windows of this thread's column
  float p_m2 = 0.0f, p_m1 = 0.0f, p_0 = 0.0f, p_p1 = 0.0f, p_p2 = 0.0f;   // P1(k-2..k+2)
  float w_m1 = 0.0f, w_0 = 0.0f, w_p1 = 0.0f;                            // wrk(k-1..k+1)

  load_O(0);   // planes -1..0 do not exist; ring slots start as zeros
  load_O(1);
  for (int kf = 1; kf <= nz + 2; kf++) {
    load_O(kf + 1);
    __syncthreads();
    // P1 of the front plane kf on the tile plus a halo of 2
    if (kf <= nz) {
      float(*dP)[PX] = sP[kf % 3];
      const float(*Om)[OX] = sO[(kf - 1 + 3) % 3];
      const float(*Oc)[OX] = sO[kf % 3];
      const float(*Op)[OX] = sO[(kf + 1) % 3];
      const bool zb = kf == 1 || kf == nz;
      for (int t = tid; t < PX * PY; t += TX * TY) {
        const int ly = t / PX, lx = t % PX;
        const int i = i0 - 2 + lx, j = j0 - 2 + ly;
        float v = 0.0f;
        if (i >= 1 && i <= nx && j >= 1 && j <= ny) {
          const float w = __ldg(W + (size_t)(kf - 1) * plane + (size_t)(j - 1) * nx + (i - 1));
          if (zb || i == 1 || i == nx || j == 1 || j == ny) {
            v = w;
          } else {
            const int oy = ly + 1, ox = lx + 1;   // same cell in the halo-3 frame
            v = w + chi * (Oc[oy][ox + 1] + Oc[oy][ox - 1] + Oc[oy + 1][ox] + Oc[oy - 1][ox]
                           + Op[oy][ox] + Om[oy][ox] - 6.0f * Oc[oy][ox]);
          }
        }
        dP[ly][lx] = v;
      }
    }
    // wrk of the output plane k = kf-2 with a halo of 1
    const int k = kf - 2;
    if (k >= 1) {
      for (int t = tid; t < WX * WY; t += TX * TY) {
        const int ly = t / WX, lx = t % WX;
        const int i = i0 - 1 + lx, j = j0 - 1 + ly;
        float v = 0.0f;
        if (i >= 1 && i <= nx && j >= 1 && j <= ny) v = __ldg(W + (size_t)(k - 1) * plane + (size_t)(j - 1) * nx + (i - 1));
        sW[ly][lx] = v;
      }
    }
    __syncthreads();
    // slide the column windows: P1(kf) and wrk(k+1) enter
    p_m2 = p_m1; p_m1 = p_0; p_0 = p_p1; p_p1 = p_p2;
    p_p2 = (kf <= nz) ? sP[kf % 3][ty + 2][tx + 2] : 0.0f;
    w_m1 = w_0; w_0 = w_p1;
    w_p1 = (mine && k + 1 >= 1 && k + 1 <= nz) ? __ldg(W + (size_t)k * plane + (size_t)(gj - 1) * nx + (gi - 1)) : 0.0f;
    if (mine && k >= 1) {
      const size_t c = (size_t)(k - 1) * plane + (size_t)(gj - 1) * nx + (gi - 1);
      if (k == 1 || k == nz) {
        out[c] = w_0;
      } else {
        const float(*P)[PX] = sP[k % 3];
        const int py = ty + 2, px = tx + 2, wy = ty + 1, wx = tx + 1;
        // x pass (sub_fcsmooth.f90:279-327)
        float tv;
        if (gi == 1 || gi == nx) {
          tv = sW[wy][wx];
        } else {
          // limiter flux at index m (2..nx-1) of this row; P1 and wrk offsets
          // relative to the output cell
          auto fx = [&](int m) {
            const int o = m - gi;
            const float dw = sW[wy][wx + o + 1] - sW[wy][wx + o];
            const float d1m = P[py][px + o] - P[py][px + o - 1];
            const float d1p = (m + 1 <= nx - 1) ? P[py][px + o + 2] - P[py][px + o + 1] : P[py][px + o + 1] - P[py][px + o];
            return limiter(dw, d1m, d1p, chi);
          };
          const float f0 = fx(gi);
          const float f1 = fx(gi - 1 < 2 ? 2 : gi - 1);
          tv = P[py][px] - f0 + f1;
        }
        // y pass (:331-381)
        if (gj != 1 && gj != ny) {
          auto fy = [&](int m) {
            const int o = m - gj;
            const float dw = sW[wy + o + 1][wx] - sW[wy + o][wx];
            const float d1m = P[py + o][px] - P[py + o - 1][px];
            const float d1p = (m + 1 <= ny - 1) ? P[py + o + 2][px] - P[py + o + 1][px] : P[py + o + 1][px] - P[py + o][px];
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
