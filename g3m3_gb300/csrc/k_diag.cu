// k_diag.cu -- diagnostics on the device.
//
// flux_counter (sub_flux_counter.f90:5-158): the momentum of
// each ion species summed over the six walls one cell inside the box faces
// (index 2 and n-1), counted as inflow or outflow by the sign of the
// ionospheric-H+ sum, and scaled by grid_spacing / mass.
//
// The reference sums each wall serially in FP32; the result depends on that
// order, so each of the 18 sums (3 walls x 2 sides x 3 species) is one
// thread adding in the reference's order (loads issued eight ahead), and
// one thread then combines them exactly as the reference does.
//
// Graphing planes (sub_write_graphing_data.f90:340-420): species velocity
// with a density floor, and the gather of one grid plane of many arrays.
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

__device__ __forceinline__ float wall_sum(const float* __restrict__ p, size_t base, size_t s_in, int n_in,
                                          size_t s_out, int n_out) {
  float acc = 0.0f;
  for (int o = 0; o < n_out; o++) {
    const float* row = p + base + (size_t)o * s_out;
    int i = 0;
    for (; i + 8 <= n_in; i += 8) {
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; u++) v[u] = __ldg(row + (size_t)(i + u) * s_in);
#pragma unroll
      for (int u = 0; u < 8; u++) acc = acc + v[u];
    }
    for (; i < n_in; i++) acc = acc + __ldg(row + (size_t)i * s_in);
  }
  return acc;
}

__global__ void __launch_bounds__(32) k_flux_counter(const __grid_constant__ FluxArgs a) {
  __shared__ float sums[3][2][3];   // wall, side, species
  const int t = threadIdx.x;
  const Dims d = a.d;
  const size_t sx = 1, sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  if (t < 18) {
    const int wall = t / 6, side = (t / 3) % 2, s = t % 3;
    const float* p = a.p[s][wall];
    float v;
    if (wall == 0) {        // i = 2 / nx-1: k outer, j inner (:38-46)
      const int i = side == 0 ? 2 : d.nx - 1;
      v = wall_sum(p, (size_t)(i - 1), sy, d.ny, sz, d.nz);
    } else if (wall == 1) { // j = 2 / ny-1: k outer, i inner (:80-88)
      const int j = side == 0 ? 2 : d.ny - 1;
      v = wall_sum(p, (size_t)(j - 1) * sy, sx, d.nx, sz, d.nz);
    } else {                // k = 2 / nz-1: j outer, i inner (:122-130)
      const int k = side == 0 ? 2 : d.nz - 1;
      v = wall_sum(p, (size_t)(k - 1) * sz, sx, d.nx, sy, d.ny);
    }
    sums[wall][side][s] = v;
  }
  __syncwarp();
  if (t == 0) {
    float in[3] = {0.0f, 0.0f, 0.0f}, out[3] = {0.0f, 0.0f, 0.0f};
    const float gs = a.grid_spacing;
    for (int w = 0; w < 3; w++) {
      const float* f1 = sums[w][0];
      const float* f2 = sums[w][1];
      if (f1[1] > 0.0f) {
        for (int s = 0; s < 3; s++) in[s] = in[s] + f1[s] * gs / a.rmass[s];
      } else {
        for (int s = 0; s < 3; s++) out[s] = out[s] - f1[s] * gs / a.rmass[s];
      }
      if (f2[1] < 0.0f) {
        for (int s = 0; s < 3; s++) in[s] = in[s] - f2[s] * gs / a.rmass[s];
      } else {
        for (int s = 0; s < 3; s++) out[s] = out[s] + f2[s] * gs / a.rmass[s];
      }
    }
    float* o = a.out;
    if (a.count) {   // history mode: the slot of the current main step
      const unsigned step = *a.count;
      if (step >= a.capacity) return;
      o = a.out + ((size_t)step * a.n_grids + (a.box - 1)) * 6;
      if (a.advance) *a.count = step + 1;
    }
    o[0] = in[0]; o[1] = out[0]; o[2] = in[1]; o[3] = out[1]; o[4] = in[2]; o[5] = out[2];
  }
}

// v = p / max(rho, floor) (sub_write_graphing_data.f90:376-378)
__global__ void __launch_bounds__(256) k_velocity_floor(const float* __restrict__ rho, const float* __restrict__ px,
                                                        const float* __restrict__ py, const float* __restrict__ pz,
                                                        float* vx, float* vy, float* vz, float floor_, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const float r = amax1(__ldg(rho + c), floor_);
    vx[c] = __ldg(px + c) / r;
    vy[c] = __ldg(py + c) / r;
    vz[c] = __ldg(pz + c) / r;
  }
}

// one plane of nq box arrays: plane 0 = z index, 1 = y index, 2 = x index;
// out[q][a][b] with the faster grid axis last
__global__ void __launch_bounds__(256) k_cut(const __grid_constant__ CutArgs a) {
  const Dims d = a.d;
  const int na = a.plane == 0 ? d.ny : d.nz;
  const int nb = a.plane == 2 ? d.ny : d.nx;
  const int total = a.nq * na * nb;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int q = t / (na * nb), r = t % (na * nb), ia = r / nb, ib = r % nb;
    int i, j, k;
    if (a.plane == 0) { i = ib + 1; j = ia + 1; k = a.index; }
    else if (a.plane == 1) { i = ib + 1; j = a.index; k = ia + 1; }
    else { i = a.index; j = ib + 1; k = ia + 1; }
    a.out[(size_t)(a.q0 + q) * na * nb + r] = __ldg(a.src[q] + d.at(i, j, k));
  }
}

}  // namespace

void launch_flux_counter(const FluxArgs& a, cudaStream_t s) { k_flux_counter<<<1, 32, 0, s>>>(a); }

void launch_velocity_floor(const float* rho, const float* const p[3], float* const v[3], float floor_, size_t n,
                           cudaStream_t s) {
  unsigned b = (unsigned)((n + 255) / 256);
  if (b > 8u * sm_count()) b = 8u * sm_count();
  k_velocity_floor<<<b, 256, 0, s>>>(rho, p[0], p[1], p[2], v[0], v[1], v[2], floor_, n);
}

void launch_cut(const CutArgs& a, cudaStream_t s) {
  const int na = a.plane == 0 ? a.d.ny : a.d.nz;
  const int nb = a.plane == 2 ? a.d.ny : a.d.nx;
  const int total = a.nq * na * nb;
  k_cut<<<(total + 255) / 256, 256, 0, s>>>(a);
}

}  // namespace g3m3
