// k_sample.cu -- virtual-spacecraft sampling: findgrid (cft_findgrid.f90:
// 70-126), the cube of find_aux_cube (cft_find_aux_cube.f90:37-65), the
// 2x2x2 gather of cft_craft_handling.f90:178-189 and trilin_interp
// (cft_trilin_interp.f90:10-66); one thread per trajectory point.  Also the
// engine's per-step craft recorder (k_craft).
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

// Trilinear value at xyz (planet radii) in the smallest box that holds it;
// slice(b) gives box b's slice of the sampled field.  NaN where the
// reference stops recording (no cube inside the box).
template <class Slice>
__device__ float sample_at(const SampleArgs& a, Slice slice, const float xyz[3]) {
  const float abit = 0.001f;
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
  if (g[0] <= 0 || g[1] <= 0 || g[2] <= 0 || g[0] >= a.d.nx || g[1] >= a.d.ny || g[2] >= a.d.nz)
    return __int_as_float(0x7fc00000);
  float cv0[3], cv1[3];
  for (int q = 0; q < 3; q++) {
    cv0[q] = (a.gmin[3 * (box - 1) + q] + ((float)g[q] - 1.0f) * a.xspac[box - 1]) * a.re_equiv;
    cv1[q] = cv0[q] + a.xspac[box - 1] * a.re_equiv;
  }
  const float* f = slice(box);
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
  return f0 * (1.0f - zd) + f1 * zd;
}

__global__ void k_sample(const __grid_constant__ SampleArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n) return;
  const float xyz[3] = {a.xyz[3 * p], a.xyz[3 * p + 1], a.xyz[3 * p + 2]};
  const size_t n3 = a.d.cells();
  a.out[p] = sample_at(a, [&](int box) { return a.field + (size_t)(box - 1) * n3; }, xyz);
}

// Virtual spacecraft at the model's time (cft_craft_handling.f90:120-200):
// the position between the trajectory samples around t (linterp,
// cft_linterp.f90:17-27; find_aux_cube, cft_find_aux_cube.f90:37-41), then
// each recorded field sampled there.  One thread per craft; the record of
// a craft whose trajectory does not cover t holds NaN.
__global__ void k_craft(const __grid_constant__ CraftArgs a) {
  const unsigned step = *a.count;
  const int c = threadIdx.x;
  if (step < a.capacity && c < a.ncraft) {
    float* rec = a.out + ((size_t)step * a.ncraft + c) * (4 + a.nf);
    const float t = a.t.get();
    const int lo = a.start[c], hi = a.start[c + 1];   // samples of this craft, sorted by time
    const float* T = a.traj;
    int i = -1;
    for (int s = lo; s + 1 < hi; s++)
      if (t >= T[4 * s + 3] && t < T[4 * (s + 1) + 3]) { i = s; break; }
    rec[0] = t;
    if (i < 0) {
      for (int q = 1; q < 4 + a.nf; q++) rec[q] = __int_as_float(0x7fc00000);
    } else {
      const float* x1 = T + 4 * i;
      const float* x2 = T + 4 * (i + 1);
      float xyz[3];
      if (x1[3] == x2[3]) {
        xyz[0] = x1[0]; xyz[1] = x1[1]; xyz[2] = x1[2];
      } else {
        for (int q = 0; q < 3; q++) xyz[q] = x1[q] + (x2[q] - x1[q]) / (x2[3] - x1[3]) * (t - x1[3]);
      }
      rec[1] = xyz[0]; rec[2] = xyz[1]; rec[3] = xyz[2];
      for (int f = 0; f < a.nf; f++)
        rec[4 + f] = sample_at(a.geo, [&](int box) { return a.fld[f][box - 1]; }, xyz);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && step < a.capacity) *a.count = step + 1;
}

}  // namespace

void launch_sample(const SampleArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  k_sample<<<(a.n + 127) / 128, 128, 0, s>>>(a);
}

void launch_craft(const CraftArgs& a, cudaStream_t s) { k_craft<<<1, 128, 0, s>>>(a); }

}  // namespace g3m3
