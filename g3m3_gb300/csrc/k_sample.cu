// k_sample.cu -- virtual-spacecraft sampling: findgrid (cft_findgrid.f90:
// 70-126), the cube of find_aux_cube (cft_find_aux_cube.f90:37-65), the
// 2x2x2 gather of cft_craft_handling.f90:178-189 and trilin_interp
// (cft_trilin_interp.f90:10-66).  One thread per trajectory point.
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

__global__ void k_sample(const __grid_constant__ SampleArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  const float abit = 0.001f;
  const float xyz[3] = {a.xyz[3 * p], a.xyz[3 * p + 1], a.xyz[3 * p + 2]};
  float v[3] = {xyz[0] / a.re_equiv, xyz[1] / a.re_equiv, xyz[2] / a.re_equiv};
  int box = 0;
  for (int b = 1; b <= a.n_grids; b++) {
    const float* mn = a.gmin + 3 * (b - 1);
    const float* mx = a.gmax + 3 * (b - 1);
    if (v[0] > mn[0] && v[1] > mn[1] && v[2] > mn[2] && v[0] < mx[0] && v[1] < mx[1] && v[2] < mx[2]) {
      box = b;
      break;
    }
  }
  if (box == 0) {
    box = a.n_grids;
    for (int q = 0; q < 3; q++) {
      v[q] = amax1(v[q], a.gmin[3 * (box - 1) + q] + abit);
      v[q] = amin1(v[q], a.gmax[3 * (box - 1) + q] - abit);
    }
  }
  int g[3];
  for (int q = 0; q < 3; q++) g[q] = 1 + (int)((v[q] - a.gmin[3 * (box - 1) + q]) / a.xspac[box - 1]);
  if (g[0] <= 0 || g[1] <= 0 || g[2] <= 0 || g[0] >= a.d.nx || g[1] >= a.d.ny || g[2] >= a.d.nz) {
    a.out[p] = __int_as_float(0x7fc00000);   // the reference stops recording this craft
    return;
  }
  float cv0[3], cv1[3];
  for (int q = 0; q < 3; q++) {
    cv0[q] = (a.gmin[3 * (box - 1) + q] + ((float)g[q] - 1.0f) * a.xspac[box - 1]) * a.re_equiv;
    cv1[q] = cv0[q] + a.xspac[box - 1] * a.re_equiv;
  }
  const float* f = a.field + (size_t)(box - 1) * a.d.cells();
  auto Q = [&](int di, int dj, int dk) { return __ldg(f + a.d.at(g[0] + di, g[1] + dj, g[2] + dk)); };
  // with a point outside every box the reference interpolates at the
  // original (unclamped) position between the clamped cube's vertices
  const float xd = (xyz[0] - cv0[0]) / (cv1[0] - cv0[0]);
  const float yd = (xyz[1] - cv0[1]) / (cv1[1] - cv0[1]);
  const float zd = (xyz[2] - cv0[2]) / (cv1[2] - cv0[2]);
  const float e00 = Q(0, 0, 0) * (1.0f - xd) + Q(1, 0, 0) * xd;
  const float e01 = Q(0, 0, 1) * (1.0f - xd) + Q(1, 0, 1) * xd;
  const float e10 = Q(0, 1, 0) * (1.0f - xd) + Q(1, 1, 0) * xd;
  const float e11 = Q(0, 1, 1) * (1.0f - xd) + Q(1, 1, 1) * xd;
  const float f0 = e00 * (1.0f - yd) + e10 * yd;
  const float f1 = e01 * (1.0f - yd) + e11 * yd;
  a.out[p] = f0 * (1.0f - zd) + f1 * zd;
}

}  // namespace

void launch_sample(const SampleArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  k_sample<<<(a.n + 127) / 128, 128, 0, s>>>(a);
}

}  // namespace g3m3
