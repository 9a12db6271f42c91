// k_adj.cu -- reverse-mode kernels of the step (the adjoint of every
// forward kernel the engine launches in a main step).
//
// Each kernel reads the adjoint of what its forward kernel wrote, clears it
// where the forward kernel overwrote a value, and adds J^T times it to the
// adjoints of the forward kernel's inputs.  A cell's stencil inputs are
// shared with its neighbours, so those additions are atomic (fire-and-
// forget reductions in L2; the order of the FP32 sums is not fixed, which
// changes gradients by rounding only), except in the Lapidus and
// flux-correction reverses, which gather each input's shares in the
// input's own thread.  The per-cell arithmetic of the
// pushes, fields, Lapidus and flux-correction kernels comes from the
// reverse sweeps in adj_cells.cuh; the boundary, nested-grid, guard and
// div B reverses are written out here.
#include "adj_cells.cuh"
#include "adjoint.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

__device__ __forceinline__ void red(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ float sgn(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

struct Cell3 {
  int i, j, k;
  size_t c;
  bool ok, interior;
};

__device__ __forceinline__ Cell3 cell3(const Dims& d) {   // one thread per cell, x fastest, 1D blocks
  Cell3 r;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  r.ok = t < (long)d.nx * d.ny * d.nz;
  const long tt = r.ok ? t : 0;
  const long u = tt / d.nx;
  r.i = (int)(tt - u * d.nx) + 1;
  r.j = (int)(u % d.ny) + 1;
  r.k = (int)(u / d.ny) + 1;
  r.interior = r.i > 1 && r.j > 1 && r.k > 1 && r.i < d.nx && r.j < d.ny && r.k < d.nz;
  r.c = (size_t)tt;
  return r;
}

// the cells of the one-deep outer shell: x faces, then y faces (x
// interior), then z faces (x and y interior)
__device__ bool shell1_cell(long t, const Dims& d, int& i, int& j, int& k) {
  const long nyz = (long)d.ny * d.nz;
  if (t < 2 * nyz) {
    i = t < nyz ? 1 : d.nx;
    const long r = t % nyz;
    j = (int)(r % d.ny) + 1;
    k = (int)(r / d.ny) + 1;
    return true;
  }
  t -= 2 * nyz;
  const int ix = d.nx - 2;
  const long nxz = (long)ix * d.nz;
  if (t < 2 * nxz) {
    j = t < nxz ? 1 : d.ny;
    const long r = t % nxz;
    i = (int)(r % ix) + 2;
    k = (int)(r / ix) + 1;
    return true;
  }
  t -= 2 * nxz;
  const int iy = d.ny - 2;
  const long nxy = (long)ix * iy;
  if (t < 2 * nxy) {
    k = t < nxy ? 1 : d.nz;
    const long r = t % nxy;
    i = (int)(r % ix) + 2;
    j = (int)(r / ix) + 2;
    return true;
  }
  return false;
}

// offsets of the 7-point stencil in the order c, xp, xm, yp, ym, zp, zm
struct Off7 {
  long o[7];
  __device__ __forceinline__ explicit Off7(const Dims& d) {
    const long sy = d.nx, sz = (long)d.nx * d.ny;
    o[0] = 0; o[1] = 1; o[2] = -1; o[3] = sy; o[4] = -sy; o[5] = sz; o[6] = -sz;
  }
};

// ------------------------------------------------------------------ push_ion
// 168 registers (three blocks of 128 per SM; a small spill) timed fastest
// against the unbounded 255, 128 and 80.  Also slower, per launch on a
// 97x97x49 box: a form that sums the stencil contributions of a tile in a
// shared-memory ring with shared atomics before adding them to global
// memory (289 against 226 us, both with IEEE division); a tile marching
// along z with the 13 stencil fields of three planes staged in shared
// memory (350 against 215 us: two barriers per plane); each thread's 108
// inputs copied into its own shared-memory column by asynchronous copies
// issued at once (238 against 215 us: the sweep still holds 168 registers);
// the reverse split into launches over subsets of the ten outputs, each
// with the sweep of its outputs only (generated per subset; the subsets'
// gradients sum to the whole cell's): density and momenta, then the six
// pressures, 9 % slower at 128 registers and 13 % at 168; three parts
// (momenta, diagonal, off-diagonal pressures) 25 % slower at 128 or 80,
// since the stencil loads and atomics the parts share are repeated.
__global__ void __launch_bounds__(128, 3) k_adj_push_ion(const __grid_constant__ AdjPushIonArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok || !p.interior) return;   // the boundary: k_adj_push_ion_shell
  const size_t c = p.c;
  float ob[10];
  bool any = false;
#pragma unroll
  for (int f = 0; f < 10; f++) {
    ob[f] = a.a_out[f][c];
    any |= ob[f] != 0.0f;
    a.a_out[f][c] = 0.0f;
  }
  if (!any) return;
  const Off7 o(d);
  using Cellf = adj::push_ion_cell<float>;
  float in[Cellf::NIN];
#pragma unroll
  for (int f = 0; f < 13; f++) {
    const float* base = f < 10 ? a.src[f] : a.bs[f - 10];
#pragma unroll
    for (int q = 0; q < 7; q++) in[f * 7 + q] = __ldg(base + c + o.o[q]);
  }
#pragma unroll
  for (int f = 0; f < 10; f++) in[91 + f] = __ldg(a.old[f] + c);
  in[101] = __ldg(a.btot + c);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    in[102 + q] = __ldg(a.efld[q] + c);
    in[105 + q] = __ldg(a.tv[q] + c);
  }
  const float delt = a.delt;
  const float ax = a.g.xmin + a.g.dx * (float)(p.i - 1);
  const float ay = a.g.ymin + a.g.dy * (float)(p.j - 1);
  const float az = a.g.zmin + a.g.dz * (float)(p.k - 1);
  const float radius = sqrtf(ax * ax + ay * ay + az * az) + 0.0000001f;
  const float rr = a.re_equiv * radius;
  const float par[Cellf::NPAR] = {delt, 2.0f * a.g.dx, 2.0f * a.g.dy, 2.0f * a.g.dz, a.rmass, a.reynolds,
                                  0.20f * a.rmass / delt / a.reynolds, a.grav, rr * rr, radius, ax, ay, az};
  Cellf::adj(in, par, ob, [&](int s, float v) {
    if (s < 91) {
      const int f = s / 7, q = s % 7;
      red((f < 10 ? a.a_src[f] : a.a_bs[f - 10]) + c + o.o[q], v);
    } else if (s < 101) {
      red(a.a_old[s - 91] + c, v);
    } else if (s == 101) {
      red(a.a_btot + c, v);
    } else if (s < 105) {
      red(a.a_efld[s - 102] + c, v);
    } else {
      red(a.a_tv[s - 105] + c, v);
    }
  });
}

// the boundary cells of out: copies of old when the push wrote them
__global__ void __launch_bounds__(256) k_adj_push_ion_shell(const __grid_constant__ AdjPushIonArgs a) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int i, j, k;
  if (!shell1_cell(t, a.d, i, j, k)) return;
  const size_t c = a.d.at(i, j, k);
#pragma unroll
  for (int f = 0; f < 10; f++) {
    const float g = a.a_out[f][c];
    if (g != 0.0f) red(a.a_old[f] + c, g);
    a.a_out[f][c] = 0.0f;
  }
}

// ---------------------------------------------------- push_elec, push_bfld
__global__ void __launch_bounds__(256) k_adj_push_field(const __grid_constant__ AdjPushFieldArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok) return;
  const size_t c = p.c;
  if (!p.interior) {
    if (a.boundary_from_old) {
      if (a.do_elec) {
        const float g = a.a_epres[c];
        if (g != 0.0f) red(a.a_oldepres + c, g);
        a.a_epres[c] = 0.0f;
      }
      if (a.do_bfld)
        for (int q = 0; q < 3; q++) {
          const float g = a.a_b[q][c];
          if (g != 0.0f) red(a.a_oldb[q] + c, g);
          a.a_b[q][c] = 0.0f;
        }
    }
    return;
  }
  const Off7 o(d);
  const float dxt = 2.0f * a.rx, dyt = 2.0f * a.ry, dzt = 2.0f * a.rz;
  if (a.do_elec) {
    const float g = a.a_epres[c];
    a.a_epres[c] = 0.0f;
    if (g != 0.0f) {
      using Ce = adj::push_elec_cell<float>;
      const float* w = a.wrkepres;
      float in[Ce::NIN];
      for (int q = 0; q < 6; q++) in[q] = __ldg(w + c + o.o[1 + q]);
      in[6] = __ldg(a.ev[0] + c + o.o[1]); in[7] = __ldg(a.ev[0] + c + o.o[2]);
      in[8] = __ldg(a.ev[1] + c + o.o[3]); in[9] = __ldg(a.ev[1] + c + o.o[4]);
      in[10] = __ldg(a.ev[2] + c + o.o[5]); in[11] = __ldg(a.ev[2] + c + o.o[6]);
      in[12] = __ldg(a.ev[0] + c); in[13] = __ldg(a.ev[1] + c); in[14] = __ldg(a.ev[2] + c);
      in[15] = 0.0f;   // the old value enters linearly
      const float par[Ce::NPAR] = {a.delt, a.gamma, a.gamma1, dxt, dyt, dzt};
      Ce::adj(in, par, &g, [&](int s, float v) {
        if (s < 6) red(a.a_wrkepres + c + o.o[1 + s], v);
        else if (s < 8) red(a.a_ev[0] + c + o.o[1 + (s - 6)], v);
        else if (s < 10) red(a.a_ev[1] + c + o.o[3 + (s - 8)], v);
        else if (s < 12) red(a.a_ev[2] + c + o.o[5 + (s - 10)], v);
        else if (s < 15) red(a.a_ev[s - 12] + c, v);
        else red(a.a_oldepres + c, v);
      });
    }
  }
  if (a.do_bfld) {
    float g[3];
    bool any = false;
    for (int q = 0; q < 3; q++) {
      g[q] = a.a_b[q][c];
      any |= g[q] != 0.0f;
      a.a_b[q][c] = 0.0f;
    }
    if (any) {
      using Cb = adj::push_bfld_cell<float>;
      float in[Cb::NIN] = {};   // linear: the derivatives do not depend on the values
      const float par[Cb::NPAR] = {a.delt, dxt, dyt, dzt};
      // inputs: obx oby obz, ex(yp ym zp zm), ey(xp xm zp zm), ez(xp xm yp ym)
      Cb::adj(in, par, g, [&](int s, float v) {
        if (s < 3) red(a.a_oldb[s] + c, v);
        else if (s < 7) red(a.a_efld[0] + c + o.o[3 + (s - 3)], v);
        else if (s < 9) red(a.a_efld[1] + c + o.o[1 + (s - 7)], v);
        else if (s < 11) red(a.a_efld[1] + c + o.o[5 + (s - 9)], v);
        else red(a.a_efld[2] + c + o.o[1 + (s - 11)], v);
      });
    }
  }
}

// -------------------------------------------------------------- fields
// BandE (every cell takes E at its clamped interior point)
__global__ void __launch_bounds__(256) k_adj_bande(const __grid_constant__ AdjFieldsArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok) return;
  float g[3];
  bool any = false;
  for (int q = 0; q < 3; q++) {
    g[q] = a.a_efld[q][p.c];
    any |= g[q] != 0.0f;
    a.a_efld[q][p.c] = 0.0f;
  }
  if (!any) return;
  const size_t s = d.at(clampi(p.i, 2, d.nx - 1), clampi(p.j, 2, d.ny - 1), clampi(p.k, 2, d.nz - 1));
  const Off7 o(d);
  using Cb = adj::bande_cell<float>;
  float in[Cb::NIN];
  for (int q = 0; q < 3; q++) {
    in[q] = __ldg(a.ev[q] + s);
    in[3 + q] = __ldg(a.bs[q] + s);
    in[6 + q] = __ldg(a.rho[q] + s);
    in[15 + q] = __ldg(a.cur[q] + s);
  }
  for (int q = 0; q < 6; q++) in[9 + q] = __ldg(a.epres + s + o.o[1 + q]);
  const float rst = a.rst_e ? __ldg(a.rst_e + s) : 0.0f;
  const float par[Cb::NPAR] = {a.rmass[0], a.rmass[1], a.rmass[2], a.reynolds,
                               2.0f * a.rx, 2.0f * a.ry, 2.0f * a.rz, rst};
  Cb::adj(in, par, g, [&](int q, float v) {
    if (q < 3) red(a.a_ev[q] + s, v);
    else if (q < 6) red(a.a_bs[q - 3] + s, v);
    else if (q < 9) red(a.a_rho[q - 6] + s, v);
    else if (q < 15) red(a.a_epres + s + o.o[1 + (q - 9)], v);
    else red(a.a_cur[q - 15] + s, v);
  });
}

// fnd_evel (pointwise)
__global__ void __launch_bounds__(256) k_adj_evel(const __grid_constant__ AdjFieldsArgs a) {
  const size_t n = a.d.cells();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    float g[6];
    bool any = false;
    for (int q = 0; q < 3; q++) {
      g[q] = a.a_ev[q][c];
      g[3 + q] = a.a_tv[q][c];
      a.a_ev[q][c] = 0.0f;
      a.a_tv[q][c] = 0.0f;
    }
    for (int q = 0; q < 6; q++) any |= g[q] != 0.0f;
    if (!any) continue;
    using Ce = adj::evel_cell<float>;
    float in[Ce::NIN];
    for (int s = 0; s < 3; s++) {
      in[s] = __ldg(a.rho[s] + c);
      for (int q = 0; q < 3; q++) in[3 + 3 * s + q] = __ldg(a.p[s][q] + c);
      in[12 + s] = __ldg(a.cur[s] + c);
    }
    const float par[Ce::NPAR] = {a.rmass[0], a.rmass[1], a.rmass[2], a.reynolds};
    Ce::adj(in, par, g, [&](int q, float v) {
      if (q < 3) red(a.a_rho[q] + c, v);
      else if (q < 12) red(a.a_p[(q - 3) / 3][(q - 3) % 3] + c, v);
      else red(a.a_cur[q - 12] + c, v);
    });
  }
}

// bs = b0 + b, btot (pointwise)
__global__ void __launch_bounds__(256) k_adj_total_b(const __grid_constant__ AdjFieldsArgs a) {
  const size_t n = a.d.cells();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    float g[4];
    for (int q = 0; q < 3; q++) {
      g[q] = a.a_bs[q][c];
      a.a_bs[q][c] = 0.0f;
    }
    g[3] = a.a_btot[c];
    a.a_btot[c] = 0.0f;
    if (g[0] == 0.0f && g[1] == 0.0f && g[2] == 0.0f && g[3] == 0.0f) continue;
    using Ct = adj::total_b_cell<float>;
    const float in[3] = {__ldg(a.b[0] + c), __ldg(a.b[1] + c), __ldg(a.b[2] + c)};
    const float par[4] = {__ldg(a.b0[0] + c), __ldg(a.b0[1] + c), __ldg(a.b0[2] + c), a.smallbit};
    Ct::adj(in, par, g, [&](int q, float v) { red(a.a_b[q] + c, v); });
  }
}

// calcur (every cell takes the curl at its clamped interior point)
__global__ void __launch_bounds__(256) k_adj_curl(const __grid_constant__ AdjFieldsArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok) return;
  float g[3];
  bool any = false;
  for (int q = 0; q < 3; q++) {
    g[q] = a.a_cur[q][p.c];
    any |= g[q] != 0.0f;
    a.a_cur[q][p.c] = 0.0f;
  }
  if (!any) return;
  const size_t s = d.at(clampi(p.i, 2, d.nx - 1), clampi(p.j, 2, d.ny - 1), clampi(p.k, 2, d.nz - 1));
  const Off7 o(d);
  using Cc = adj::curl_cell<float>;
  float in[Cc::NIN] = {};
  const float par[3] = {2.0f * a.rx, 2.0f * a.ry, 2.0f * a.rz};
  // inputs: bx(yp ym zp zm) by(xp xm zp zm) bz(xp xm yp ym)
  Cc::adj(in, par, g, [&](int q, float v) {
    if (q < 4) red(a.a_b[0] + s + o.o[3 + q], v);
    else if (q < 6) red(a.a_b[1] + s + o.o[1 + (q - 4)], v);
    else if (q < 8) red(a.a_b[1] + s + o.o[5 + (q - 6)], v);
    else red(a.a_b[2] + s + o.o[1 + (q - 8)], v);
  });
}

// ------------------------------------------------------------ Lapidus
// The smoothing of a field f at an interior cell c (sub_lap_plasma.f90:
// 50-140, sub_lap_elec.f90:33-48) is
//   out(c) = f(c) + chi delt sum_e [U(c,c+e) (f(c+e) - f(c)) - U(c-e,c) (f(c) - f(c-e))],
// U(a,b) = |v_e(b) - v_e(a)| the jump of the velocity component e across
// the face (a, b) (lap_speed_cell / lap_jump_cell: the same value from both
// sides).  A face (a, b = a + e) adds k F to out(a) and -k F to out(b),
// F = U (f(b) - f(a)), k = chi delt, where those cells are interior.  Its
// adjoint is Fbar = k (I(a) abar(a) - I(b) abar(b)) (I: interior), passing
// -U Fbar to fbar(a), U Fbar to fbar(b) and Fbar (f(b) - f(a)) to U; seen
// from a cell c and a neighbour n across either face this is the same
// expression, D = I(c) abar(c) - I(n) abar(n): fbar(c) -= U k D,
// Ubar += k D (f(n) - f(c)), vbar_e(c) += sign(v_e(c) - v_e(n)) Ubar.  So
// every cell gathers its six faces' shares and its own identity term, with
// no atomics, and turns its velocity adjoint into the adjoints of its own
// rho and p (v = p / max(rho, floor)) or adds it to the given velocity's.
// The output adjoints are only read: the caller clears them afterwards.
template <int NF>   // fields of the call at most (10: a species, 4: epres and B)
__global__ void __launch_bounds__(128) k_adj_lap(const __grid_constant__ AdjLapArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok) return;
  const size_t c = p.c;
  const int idx[3] = {p.i, p.j, p.k};
  const int nn[3] = {d.nx, d.ny, d.nz};
  const long st[3] = {1, (long)d.nx, (long)d.nx * d.ny};
  bool in[3];
  for (int e = 0; e < 3; e++) in[e] = idx[e] > 1 && idx[e] < nn[e];
  const bool ic = in[0] && in[1] && in[2];
  const bool species = a.vrho != nullptr;
  // velocity at c (all components) and of a neighbour (one component)
  float r0 = 0.0f, v0[3];
  if (species) {
    r0 = amax1(__ldg(a.vrho + c), a.vfloor);
    for (int e = 0; e < 3; e++) v0[e] = __ldg(a.vp[e] + c) / r0;
  } else {
    for (int e = 0; e < 3; e++) v0[e] = __ldg(a.v[e] + c);
  }
  auto vel = [&](int e, size_t q) {
    return species ? __ldg(a.vp[e] + q) / amax1(__ldg(a.vrho + q), a.vfloor) : __ldg(a.v[e] + q);
  };
  float ga[NF], fc[NF], acc[NF];
#pragma unroll
  for (int f = 0; f < NF; f++) {
    const bool on = f < a.nf;
    ga[f] = on && ic ? __ldg(a.a_out[f] + c) : 0.0f;
    fc[f] = on ? __ldg(a.in[f] + c) : 0.0f;
    acc[f] = ga[f];
  }
  float vb[3] = {0.0f, 0.0f, 0.0f};
  for (int e = 0; e < 3; e++) {
    const bool others = (e == 0 || in[0]) && (e == 1 || in[1]) && (e == 2 || in[2]);
    for (int dir = -1; dir <= 1; dir += 2) {
      const int t = idx[e] + dir;
      if (t < 1 || t > nn[e]) continue;
      const bool inb = others && t > 1 && t < nn[e];
      if (!ic && !inb) continue;
      const size_t q = (size_t)((long)c + dir * st[e]);
      const float vn = vel(e, q);
      const float u = fabsf(v0[e] - vn);
      float ub = 0.0f;
#pragma unroll
      for (int f = 0; f < NF; f++) {
        if (f >= a.nf) continue;
        const float dd = ga[f] - (inb ? __ldg(a.a_out[f] + q) : 0.0f);
        if (dd == 0.0f) continue;
        const float kd = a.chi[f] * a.delt * dd;
        acc[f] -= u * kd;
        ub += kd * (__ldg(a.in[f] + q) - fc[f]);
      }
      vb[e] += sgn(v0[e] - vn) * ub;
    }
  }
#pragma unroll
  for (int f = 0; f < NF; f++)
    if (f < a.nf && acc[f] != 0.0f) a.a_in[f][c] += acc[f];
  if (species) {
    float rb = 0.0f;
    for (int e = 0; e < 3; e++) {
      if (vb[e] == 0.0f) continue;
      a.a_vp[e][c] += vb[e] / r0;
      rb -= vb[e] * v0[e] / r0;
    }
    if (rb != 0.0f && __ldg(a.vrho + c) > a.vfloor) a.a_vrho[c] += rb;
  } else {
    for (int e = 0; e < 3; e++)
      if (vb[e] != 0.0f) a.a_v[e][c] += vb[e];
  }
}

__global__ void __launch_bounds__(256) k_adj_vtot(const __grid_constant__ AdjVtotArgs a) {
  const size_t n = a.d.cells();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    float g[3];
    for (int q = 0; q < 3; q++) {
      g[q] = a.a_v[q][c];
      a.a_v[q][c] = 0.0f;
    }
    if (g[0] == 0.0f && g[1] == 0.0f && g[2] == 0.0f) continue;
    using Cv = adj::vtot_cell<float>;
    float in[Cv::NIN];
    for (int s = 0; s < 3; s++) {
      in[s] = __ldg(a.rho[s] + c);
      for (int q = 0; q < 3; q++) in[3 + 3 * s + q] = __ldg(a.p[s][q] + c);
    }
    Cv::adj(in, nullptr, g, [&](int q, float v) {
      if (q < 3) red(a.a_rho[q] + c, v);
      else red(a.a_p[(q - 3) / 3][(q - 3) % 3] + c, v);
    });
  }
}

// ---------------------------------------------------------- flux correction
__global__ void __launch_bounds__(256) k_fcs_p1(const __grid_constant__ AdjFcsArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  const int f = blockIdx.y;
  if (!p.ok || f >= a.nf) return;
  const int k = p.k;
  const size_t c = p.c;
  const size_t n = d.cells();
  const float* W = a.wrk[f];
  const float* O = a.old[f];
  float v = __ldg(W + c);
  if (!(p.i == 1 || p.j == 1 || k == 1 || p.i == d.nx || p.j == d.ny || k == d.nz)) {
    const size_t sy = d.nx, sz = (size_t)d.nx * d.ny;
    v = v + a.chi[f] * (__ldg(O + c + 1) + __ldg(O + c - 1) + __ldg(O + c + sy) + __ldg(O + c - sy)
                        + __ldg(O + c + sz) + __ldg(O + c - sz) - 6.0f * __ldg(O + c));
  }
  a.p1[(size_t)f * n + c] = v;
}

// The flux-correction reverse in two passes, without atomics.  Along an
// axis, the limiter flux of face m (2 <= m <= n-1; the reference clamps the
// end faces onto these, sub_fcsmooth.f90:87-239)
//   fn = s max(0, min(s d1m, chi |dw|, s d1p)),  s = sign(dw),
//   d1m = P1(m) - P1(m-1), d1p = P1(q+1) - P1(q), dw = W(m+1) - W(m),
//   q = min(m+1, n-1),
// enters output cell m with -1, cell m+1 with +1 (m+1 <= n-1) and, for
// m = 2, cell 2 once more with +1 (cell 2's lower face is clamped onto face
// 2); on x and y only in interior k planes.  So its adjoint is
// g = -A(m) + A(m+1) [m+1 <= n-1] + A(2) [m = 2], A the output's adjoint,
// and the limiter passes g to exactly one of the three differences, the one
// the min/max chose (none where 0 won; the ties as the forward breaks them,
// amin1/amax1).  k_adj_fcs_faces evaluates every face once and stores the
// passed value in one of three arrays, by the difference it goes to (d1m,
// dw, d1p; zeros elsewhere and at positions that are no face);
// k_adj_fcs_gather then adds to each point, with loads that do not depend
// on the limiter's choices, the shares of the four faces along each axis
// whose differences hold it, plus the output's own adjoint (to P1 where the
// output is P1 - fluxes, to W where it is W).
template <int AX>
__device__ __forceinline__ void fcs_face(const AdjFcsArgs& a, int f, int i, int j, int k) {
  const Dims& d = a.d;
  const int n = AX == 0 ? d.nx : (AX == 1 ? d.ny : d.nz);
  const int m = AX == 0 ? i : (AX == 1 ? j : k);
  auto at = [&](int t) { return AX == 0 ? d.at(t, j, k) : (AX == 1 ? d.at(i, t, k) : d.at(i, j, t)); };
  const size_t cells = d.cells();
  const size_t slot = ((size_t)AX * a.nf + f) * cells + at(m);
  float vm = 0.0f, vw = 0.0f, vp = 0.0f;   // to d1m, dw, d1p
  if (m >= 2 && m <= n - 1 && (AX == 2 || (k != 1 && k != d.nz))) {
    const float* Apx = a.a_px[f];
    float g = -__ldg(Apx + at(m));
    if (m + 1 <= n - 1) g += __ldg(Apx + at(m + 1));
    if (m == 2) g += __ldg(Apx + at(2));
    if (g != 0.0f) {
      const float* P = a.p1 + (size_t)f * cells;
      const float* W = a.wrk[f];
      const int q = m + 1 > n - 1 ? n - 1 : m + 1;
      const float chi = a.chi[f];
      const float dw = __ldg(W + at(m + 1)) - __ldg(W + at(m));
      const float sg = dw >= 0.0f ? 1.0f : -1.0f;
      const float tm = sg * (__ldg(P + at(m)) - __ldg(P + at(m - 1)));
      const float tw = chi * fabsf(dw);
      const float tp = sg * (__ldg(P + at(q + 1)) - __ldg(P + at(q)));
      const bool c1m = tm < tw;                 // amin1(s d1m, chi |dw|)
      const float v1 = c1m ? tm : tw;
      const bool c2p = !(v1 < tp);              // amin1(., s d1p)
      const float v2 = c2p ? tp : v1;
      if (!(0.0f > v2)) {                       // amax1(0, .): the zero passes nothing
        if (c2p) vp = g;                        // d(s s d1p)/d(d1p) = 1
        else if (c1m) vm = g;
        else vw = g * chi * sg * sgn(dw);
      }
    }
  }
  a.fm[slot] = vm;
  a.fw[slot] = vw;
  a.fp[slot] = vp;
}

__global__ void __launch_bounds__(256) k_adj_fcs_faces(const __grid_constant__ AdjFcsArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  const int f = blockIdx.y;
  if (!p.ok || f >= a.nf) return;
  const int i = p.i, j = p.j, k = p.k;
  fcs_face<0>(a, f, i, j, k);
  fcs_face<1>(a, f, i, j, k);
  fcs_face<2>(a, f, i, j, k);
}

// The shares at point p of one axis: d1m of face m adds to P(m), subtracts
// from P(m-1); d1p of face m adds to P(q+1), subtracts from P(q) (q = m+1,
// or m for the clamped face m = n-1); dw adds to W(m+1), subtracts from
// W(m).  Faces that do not exist hold zeros.
template <int AX>
__device__ __forceinline__ void fcs_gather_axis(const AdjFcsArgs& a, int f, int i, int j, int k, float& accP,
                                                float& accW) {
  const Dims& d = a.d;
  const int n = AX == 0 ? d.nx : (AX == 1 ? d.ny : d.nz);
  const int p = AX == 0 ? i : (AX == 1 ? j : k);
  if (AX != 2 && (k == 1 || k == d.nz)) return;
  auto at = [&](int t) { return AX == 0 ? d.at(t, j, k) : (AX == 1 ? d.at(i, t, k) : d.at(i, j, t)); };
  const size_t base = ((size_t)AX * a.nf + f) * d.cells();
  const float* FM = a.fm + base;
  const float* FW = a.fw + base;
  const float* FP = a.fp + base;
  const size_t c = at(p);
  const long st = AX == 0 ? 1L : (AX == 1 ? (long)d.nx : (long)d.nx * d.ny);
  const float m0 = FM[c];
  const float m1 = p + 1 <= n ? FM[c + st] : 0.0f;
  const float w0 = FW[c];
  const float w1 = p >= 2 ? FW[c - st] : 0.0f;
  const float p2 = p >= 3 ? FP[c - 2 * st] : 0.0f;             // face p-2 (q + 1 = p)
  const float p1 = p >= 2 && p <= n - 1 ? FP[c - st] : 0.0f;    // face p-1 (q = p)
  float pe = 0.0f;                                               // the clamped face n-1
  if (p == n) pe = FP[c - st];
  else if (p == n - 1) pe = -FP[c];
  accP += m0 - m1 + p2 - p1 + pe;
  accW += w1 - w0;
}

__global__ void __launch_bounds__(256) k_adj_fcs_gather(const __grid_constant__ AdjFcsArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  const int f = blockIdx.y;
  if (!p.ok || f >= a.nf) return;
  const int i = p.i, j = p.j, k = p.k;
  const size_t c = d.at(i, j, k);
  float accP = 0.0f, accW = 0.0f;
  const float g = __ldg(a.a_px[f] + c);
  if (k == 1 || k == d.nz || i == 1 || i == d.nx) accW += g;   // px = wrk there (x pass: t = wrk)
  else accP += g;                                              // t = P1
  // every point gathers along every axis: a boundary point is read by the
  // faces next to it even where its own cell takes no flux
  fcs_gather_axis<0>(a, f, i, j, k, accP, accW);
  fcs_gather_axis<1>(a, f, i, j, k, accP, accW);
  fcs_gather_axis<2>(a, f, i, j, k, accP, accW);
  a.a_p1[(size_t)f * d.cells() + c] = accP;
  if (accW != 0.0f) a.a_wrk[f][c] += accW;
}

// P1 = W + chi Lap7(O) in the interior, W on the boundary: gathered
__global__ void __launch_bounds__(256) k_adj_p1(const __grid_constant__ AdjFcsArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  const int f = blockIdx.y;
  if (!p.ok || f >= a.nf) return;
  const int i = p.i, j = p.j, k = p.k;
  const size_t c = d.at(i, j, k);
  const float* G = a.a_p1 + (size_t)f * d.cells();
  const float g = G[c];
  if (g != 0.0f) a.a_wrk[f][c] += g;
  auto inner = [&](int ii, int jj, int kk) {
    return ii > 1 && jj > 1 && kk > 1 && ii < d.nx && jj < d.ny && kk < d.nz;
  };
  float s = 0.0f;
  if (inner(i + 1, j, k)) s += G[c + 1];
  if (inner(i - 1, j, k)) s += G[c - 1];
  if (inner(i, j + 1, k)) s += G[c + d.nx];
  if (inner(i, j - 1, k)) s += G[c - d.nx];
  if (inner(i, j, k + 1)) s += G[c + (size_t)d.nx * d.ny];
  if (inner(i, j, k - 1)) s += G[c - (size_t)d.nx * d.ny];
  if (inner(i, j, k)) s -= 6.0f * g;
  if (s != 0.0f) a.a_old[f][c] += a.chi[f] * s;
  if (a.clear_px) a.a_px[f][c] = 0.0f;   // px was overwritten: its adjoint before is zero
}

// ---------------------------------------------------------------- guards
__device__ __forceinline__ float rho_min(int s) { return s == 0 ? 2.e-4f : (s == 1 ? 1.e-4f : 2.e-5f); }

struct Sp10 {
  float v[10];
};

__device__ __forceinline__ bool floored_sp(const Sp10& u, float rmin) {
  return u.v[0] < rmin || u.v[4] < 0.0f || u.v[5] < 0.0f || u.v[6] < 0.0f;
}

// set_rho's repair of one species' values (forward)
__device__ __forceinline__ void floor_fwd(Sp10& u, float rmin) {
  u.v[0] = amax1(fabsf(u.v[0]), 1.05f * rmin);
  const float ap = (fabsf(u.v[4]) + fabsf(u.v[5]) + fabsf(u.v[6])) / 3.0f;
  u.v[4] = ap; u.v[5] = ap; u.v[6] = ap;
  u.v[7] = 0.0f; u.v[8] = 0.0f; u.v[9] = 0.0f;
}

// its reverse: g holds the adjoint of the repaired values, u the values before
__device__ __forceinline__ void floor_adj(float g[10], const Sp10& u, float rmin) {
  g[0] = fabsf(u.v[0]) > 1.05f * rmin ? g[0] * sgn(u.v[0]) : 0.0f;
  const float gs = (g[4] + g[5] + g[6]) / 3.0f;
  g[4] = gs * sgn(u.v[4]); g[5] = gs * sgn(u.v[5]); g[6] = gs * sgn(u.v[6]);
  g[7] = 0.0f; g[8] = 0.0f; g[9] = 0.0f;
}

__device__ __forceinline__ Sp10 load10(const float* const* f, int s, size_t c) {
  Sp10 u;
  for (int q = 0; q < 10; q++) u.v[q] = __ldg(f[10 * s + q] + c);
  return u;
}

__global__ void __launch_bounds__(128) k_adj_guard_a(const __grid_constant__ AdjGuardArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok) return;
  const size_t c = p.c;
  const bool speed = a.do_speed && p.interior;
  bool floored[3], replaced[3];
  Sp10 u[3];
  float newr[3];
  for (int s = 0; s < 3; s++) {
    u[s] = load10(a.pre, s, c);
    Sp10 v = u[s];
    floored[s] = floored_sp(v, rho_min(s));
    if (floored[s]) floor_fwd(v, rho_min(s));
    newr[s] = v.v[0];
    replaced[s] = false;
    if (speed) {
      const float arho = v.v[0] + a.smallbit;
      const float avx = fabsf(v.v[1] / arho), avy = fabsf(v.v[2] / arho), avz = fabsf(v.v[3] / arho);
      const float vq = sqrtf(avx * avx + avy * avy + avz * avz);
      const float cq = sqrtf(0.33f * (v.v[4] + v.v[5] + v.v[6]) / arho);
      const float vl = a.vlim * a.svlim[s];
      const float cl = a.vlim * a.svlim[s] * a.sclim[s];
      if ((vq > vl) || (cq > cl)) {
        replaced[s] = true;
        const size_t nb[6] = {c + 1, c - 1, c + (size_t)d.nx, c - (size_t)d.nx, c + (size_t)d.nx * d.ny,
                              c - (size_t)d.nx * d.ny};
        float acc = 0.0f;
        for (int m = 0; m < 6; m++) {
          Sp10 w = load10(a.pre, s, nb[m]);
          if (floored_sp(w, rho_min(s))) floor_fwd(w, rho_min(s));
          acc = m == 0 ? w.v[0] : acc + w.v[0];
        }
        newr[s] = acc / 6.0f;
      }
    }
  }
  // electron pressure: |ep|, capped where the sound speed exceeds cslim
  const float ep0 = __ldg(a.pre[G3M3_F_EPRES] + c);
  const float e1 = fabsf(ep0);
  float ge = a.a[G3M3_F_EPRES][c];
  float gnewr = 0.0f;
  if (speed) {
    const float arho = newr[0] + newr[1] + newr[2] + a.smallbit;
    const float cs = sqrtf(e1 / arho);
    if (cs > a.cslim) {
      const float e2 = e1 * a.cslim / cs;
      gnewr = ge * 0.5f * e2 / arho;
      ge = ge * 0.5f * a.cslim / cs;
    }
  }
  a.a[G3M3_F_EPRES][c] = ge * sgn(ep0);
  for (int s = 0; s < 3; s++) {
    float g[10];
    for (int q = 0; q < 10; q++) g[q] = a.a[10 * s + q][c];
    g[0] += gnewr;
    if (replaced[s]) {
      bool any = false;
      for (int q = 0; q < 10; q++) any |= g[q] != 0.0f;
      for (int q = 0; q < 10; q++) a.a[10 * s + q][c] = 0.0f;
      if (any) {
        const unsigned slot = atomicAdd(a.list_count, 1u);
        if (slot < a.list_cap) {
          float* e = a.list + (size_t)slot * 11;
          e[0] = __uint_as_float((unsigned)(c * 4 + (size_t)s));
          for (int q = 0; q < 10; q++) e[1 + q] = g[q];
        }
      }
      continue;
    }
    if (floored[s]) floor_adj(g, u[s], rho_min(s));
    for (int q = 0; q < 10; q++) a.a[10 * s + q][c] = g[q];
  }
}

// the replaced cells' adjoints go to the neighbours whose snapshot values
// they were made of (mean of six, anisotropy limiting, set_rho repair)
__global__ void __launch_bounds__(128) k_adj_guard_b(const __grid_constant__ AdjGuardArgs a) {
  const unsigned n = min(*a.list_count, a.list_cap);
  const Dims d = a.d;
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const float* E = a.list + (size_t)e * 11;
    const unsigned w = __float_as_uint(E[0]);
    const size_t c = w >> 2;
    const int s = (int)(w & 3u);
    float gacc[10];
    for (int q = 0; q < 7; q++) gacc[q] = E[1 + q] / 6.0f;
    for (int q = 7; q < 10; q++) gacc[q] = a.iso_flag * E[1 + q] / 6.0f;
    float gu[10];
    gu[0] = gacc[0]; gu[1] = gacc[1]; gu[2] = gacc[2]; gu[3] = gacc[3];
    if (a.isotropic) {
      gu[4] = gacc[4] + gacc[5] + gacc[6]; gu[5] = 0.0f; gu[6] = 0.0f;
      gu[7] = 0.0f; gu[8] = 0.0f; gu[9] = 0.0f;
    } else {
      const float al = a.aniso_limit;
      const float gap = (gacc[4] + gacc[5] + gacc[6]) * (1.0f - al) / 3.0f;
      gu[4] = al * gacc[4] + gap; gu[5] = al * gacc[5] + gap; gu[6] = al * gacc[6] + gap;
      gu[7] = al * gacc[7]; gu[8] = al * gacc[8]; gu[9] = al * gacc[9];
    }
    const size_t nb[6] = {c + 1, c - 1, c + (size_t)d.nx, c - (size_t)d.nx, c + (size_t)d.nx * d.ny,
                          c - (size_t)d.nx * d.ny};
    for (int m = 0; m < 6; m++) {
      const Sp10 u = load10(a.pre, s, nb[m]);
      float g[10];
      for (int q = 0; q < 10; q++) g[q] = gu[q];
      if (floored_sp(u, rho_min(s))) floor_adj(g, u, rho_min(s));
      for (int q = 0; q < 10; q++)
        if (g[q] != 0.0f) red(a.a[10 * s + q] + nb[m], g[q]);
    }
  }
}

// ------------------------------------------------------------ bndry_outer
struct OuterA {
  const AdjOuterArgs* a;
  int f, comp;
  double gp;   // this thread's share of the adjoint of the field's wind parameter
  bool hit;    // the thread reached the wind face
};

// The wind parameter a field's wind-face value depends on (k_bndry.cu
// wind_value): 0 srho, 1-3 the velocity, 4 spress, 5-7 the IMF; -1 none.
__device__ __forceinline__ int wind_param(int f) {
  if (f >= 30) return f == G3M3_F_EPRES ? 4 : 5 + (f - G3M3_F_BX);
  const int q = f % 10;
  return q == 0 ? 0 : (q <= 3 ? q : (q < 7 ? 4 : -1));
}

template <int S>
__device__ float outer_val_a(const OuterA& o, int i, int j, int k) {
  // the forward value chain (k_bndry.cu outer_val) evaluated on the state
  // after the boundary, whose interior is the boundary's input
  const Dims& d = o.a->d;
  const int nx = d.nx, ny = d.ny, nz = d.nz, nx1 = nx - 1, ny1 = ny - 1, nz1 = nz - 1;
  if constexpr (S == 0) {
    return __ldg(o.a->post[o.f] + d.at(i, j, k));
  } else {
    if constexpr (S == 8) {
      if (i >= 2 && (j == 1 || j == ny) && (k == 1 || k == nz)) return outer_val_a<7>(o, i, j, k == 1 ? 2 : nz1);
    }
    if constexpr (S == 7) {
      if (i == nx && j >= 2 && j <= ny - 1) {
        if (k == 1) return outer_val_a<6>(o, nx, j, 2);
        if (k == nz && o.f != G3M3_F_EPRES) return outer_val_a<6>(o, nx1, j, nz);
      }
    }
    if constexpr (S == 6) {
      if (i == nx && (j == 1 || j == ny) && k >= 2 && k <= nz - 1) {
        const int jn = j == 1 ? 2 : ny1;
        if (o.f == G3M3_F_BX) return outer_val_a<5>(o, nx1, j, k);
        return (outer_val_a<5>(o, nx1, j, k) + outer_val_a<5>(o, nx, jn, k)) / 2.0f;
      }
    }
    if constexpr (S == 5) {
      if (k == 1 && i >= 2) {
        const float v = outer_val_a<4>(o, i, j, 2);
        return o.comp == 3 ? -fabsf(v) : v;
      }
    }
    if constexpr (S == 4) {
      if (k == nz && i >= 2) {
        const float v = outer_val_a<3>(o, i, j, nz1);
        return o.comp == 3 ? fabsf(v) : v;
      }
    }
    if constexpr (S == 3) {
      if (i >= 2 && (j == 1 || j == ny)) {
        const float v = outer_val_a<2>(o, i, j == 1 ? 2 : ny1, k);
        if (o.comp == 2) return j == 1 ? -fabsf(v) : fabsf(v);
        return v;
      }
    }
    if constexpr (S == 2) {
      if (i == nx) {
        const float v = outer_val_a<1>(o, nx1, j, k);
        return o.comp == 1 ? fabsf(v) : v;
      }
    }
    if constexpr (S == 1) {
      if (i == 1) return 0.0f;   // the wind value: only its derivative is used
    }
    return outer_val_a<S - 1>(o, i, j, k);
  }
}

// the wind face's dependence on the upstream parameters (k_bndry.cu wind_value)
__device__ void wind_adj(OuterA& o, float g) {
  const AdjOuterArgs& a = *o.a;
  const int f = o.f;
  if (f >= 30) {
    o.gp += f == G3M3_F_EPRES ? (double)g * 0.5 / (double)a.ti_te : (double)g;
    o.hit = true;
    return;
  }
  const int s = f / 10, q = f % 10;
  if (q >= 7) return;
  double w = 1.0;
  if (s > 0) {
    const float fr = s == 1 ? a.rho_frac : a.rho_frac * a.o_conc;
    const float mf = s == 1 ? a.rmassh / a.rmassq : a.rmasso / a.rmassq;
    w = q <= 3 ? (double)fr * (double)mf : (double)fr;
  }
  o.gp += q <= 3 ? w * g : 0.5 * w * g;
  o.hit = true;
}

template <int S>
__device__ void outer_adj(OuterA& o, int i, int j, int k, float g) {
  if (g == 0.0f) return;
  const Dims& d = o.a->d;
  const int nx = d.nx, ny = d.ny, nz = d.nz, nx1 = nx - 1, ny1 = ny - 1, nz1 = nz - 1;
  if constexpr (S == 0) {
    red(o.a->a[o.f] + d.at(i, j, k), g);
  } else {
    if constexpr (S == 8) {
      if (i >= 2 && (j == 1 || j == ny) && (k == 1 || k == nz)) {
        outer_adj<7>(o, i, j, k == 1 ? 2 : nz1, g);
        return;
      }
    }
    if constexpr (S == 7) {
      if (i == nx && j >= 2 && j <= ny - 1) {
        if (k == 1) { outer_adj<6>(o, nx, j, 2, g); return; }
        if (k == nz && o.f != G3M3_F_EPRES) { outer_adj<6>(o, nx1, j, nz, g); return; }
      }
    }
    if constexpr (S == 6) {
      if (i == nx && (j == 1 || j == ny) && k >= 2 && k <= nz - 1) {
        const int jn = j == 1 ? 2 : ny1;
        if (o.f == G3M3_F_BX) {
          outer_adj<5>(o, nx1, j, k, g);
        } else {
          outer_adj<5>(o, nx1, j, k, g / 2.0f);
          outer_adj<5>(o, nx, jn, k, g / 2.0f);
        }
        return;
      }
    }
    if constexpr (S == 5) {
      if (k == 1 && i >= 2) {
        float gg = g;
        if (o.comp == 3) gg = -g * sgn(outer_val_a<4>(o, i, j, 2));
        outer_adj<4>(o, i, j, 2, gg);
        return;
      }
    }
    if constexpr (S == 4) {
      if (k == nz && i >= 2) {
        float gg = g;
        if (o.comp == 3) gg = g * sgn(outer_val_a<3>(o, i, j, nz1));
        outer_adj<3>(o, i, j, nz1, gg);
        return;
      }
    }
    if constexpr (S == 3) {
      if (i >= 2 && (j == 1 || j == ny)) {
        const int js = j == 1 ? 2 : ny1;
        float gg = g;
        if (o.comp == 2) gg = (j == 1 ? -g : g) * sgn(outer_val_a<2>(o, i, js, k));
        outer_adj<2>(o, i, js, k, gg);
        return;
      }
    }
    if constexpr (S == 2) {
      if (i == nx) {
        float gg = g;
        if (o.comp == 1) gg = g * sgn(outer_val_a<1>(o, nx1, j, k));
        outer_adj<1>(o, nx1, j, k, gg);
        return;
      }
    }
    if constexpr (S == 1) {
      if (i == 1) {
        wind_adj(o, g);
        return;
      }
    }
    outer_adj<S - 1>(o, i, j, k, g);
  }
}

__global__ void __launch_bounds__(256) k_adj_outer(const __grid_constant__ AdjOuterArgs a) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int f = blockIdx.y;
  OuterA o;
  o.a = &a;
  o.f = f;
  o.comp = f < 30 ? ((f % 10) >= 1 && (f % 10) <= 3 ? f % 10 : 0) : 0;
  o.gp = 0.0;
  o.hit = false;
  int i, j, k;
  if (shell1_cell(t, a.d, i, j, k)) {
    const size_t c = a.d.at(i, j, k);
    const float g = a.a[f][c];
    a.a[f][c] = 0.0f;   // every shell value was overwritten
    outer_adj<8>(o, i, j, k, g);
  }
  // block sum of the field's wind-parameter adjoint, one atomic per block;
  // FP64 is slow on this GPU, so only warps that reached the wind face
  // reduce
  const int pidx = wind_param(f);
  if (pidx < 0) return;   // block-uniform: f is the block's field
  __shared__ double part[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double v = 0.0;
  if (__any_sync(0xffffffffu, o.hit)) {
    v = o.gp;
    for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
  }
  if (lane == 0) part[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) sum += part[w];
    if (sum != 0.0) atomicAdd(a.a_param + pidx, sum);
  }
}

// ------------------------------------------------------------ bndry_inner
__global__ void __launch_bounds__(128) k_adj_inner(const __grid_constant__ AdjInnerArgs a) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  int l;
  if (m < a.num[0]) l = 0;
  else if ((m -= a.num[0]) < a.num[1]) l = 1;
  else if ((m -= a.num[1]) < a.num[2]) l = 2;
  else return;
  const int* ij = a.ij[l];
  const float* parm = a.parm[l];
  const int mb = a.mbndry, b = a.box - 1;
  const int i = ij[b + (size_t)mb * (0 + 3 * (size_t)m)];
  const int j = ij[b + (size_t)mb * (1 + 3 * (size_t)m)];
  const int k = ij[b + (size_t)mb * (2 + 3 * (size_t)m)];
  if (i < 1 || j < 1 || k < 1 || i > a.d.nx || j > a.d.ny || k > a.d.nz) return;
  auto P = [&](int q) { return parm[b + (size_t)mb * ((q - 1) + 7 * (size_t)m)]; };
  const size_t c = a.d.at(i, j, k);
  const float ay = a.ymin + a.dy * (float)(j - 1);
  const float ax = a.xmin + a.dx * (float)(i - 1);
  const float rvy = ax * a.re_equiv * a.v_rot;
  const float rvx = -(ay * a.re_equiv) * a.v_rot;
  for (int s = 0; s < 3; s++) {
    float* const* F = a.a + 10 * s;
    const float gden = F[0][c] + F[1][c] * rvx + F[2][c] * rvy;
    for (int q = 0; q < 10; q++) F[q][c] = 0.0f;
    // surface cells keep max(parm, density): the density's adjoint passes
    // where the density won
    if (l == 0 && __ldg(a.post[10 * s] + c) > P(1 + s)) F[0][c] = gden;
  }
  a.a[G3M3_F_EPRES][c] = 0.0f;
  if (l == 2) {
    a.a[G3M3_F_BX][c] = 0.0f; a.a[G3M3_F_BY][c] = 0.0f; a.a[G3M3_F_BZ][c] = 0.0f;
  }
}

// ------------------------------------------------------------ flanks
struct AxisA { int b, b1; float d, dd; };

__device__ __forceinline__ AxisA axis_a(float smin, float sp, int idx, float bmin, float del) {
  const float av = smin + sp * (float)(idx - 1);
  const float ai = 1.0f + (av - bmin) / del;
  AxisA r;
  r.b = (int)ai;
  r.b1 = r.b + 1;
  r.d = ai - (float)r.b;
  r.dd = 1.0f - r.d;
  return r;
}

__device__ bool shell2(long t, const Dims& d, int& i, int& j, int& k) {
  const int D = 2;
  const long nyz = (long)d.ny * d.nz;
  const long xs = 2L * D * nyz;
  if (t < xs) {
    const long half = (long)D * nyz;
    const int side = (int)(t / half);
    const long r = t % half;
    const int ii = (int)(r % D);
    const long rr = r / D;
    i = side == 0 ? ii + 1 : d.nx - D + 1 + ii;
    j = (int)(rr % d.ny) + 1;
    k = (int)(rr / d.ny) + 1;
    return true;
  }
  t -= xs;
  const int ix = d.nx - 2 * D;
  const long nxz = (long)ix * d.nz;
  const long ys = 2L * D * nxz;
  if (t < ys) {
    const int s = (int)(t / nxz);
    const long r = t % nxz;
    j = s < D ? s + 1 : d.ny - (2 * D - 1 - s);
    i = (int)(r % ix) + D + 1;
    k = (int)(r / ix) + 1;
    return true;
  }
  t -= ys;
  const int iy = d.ny - 2 * D;
  const long nxy = (long)ix * iy;
  if (t < 2L * D * nxy) {
    const int s = (int)(t / nxy);
    const long r = t % nxy;
    k = s < D ? s + 1 : d.nz - (2 * D - 1 - s);
    i = (int)(r % ix) + D + 1;
    j = (int)(r / ix) + D + 1;
    return true;
  }
  return false;
}

__global__ void __launch_bounds__(256) k_adj_flanks(const __grid_constant__ AdjFlanksArgs a) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int f = blockIdx.y;
  int is, js, ks;
  const Dims d = a.d;
  if (!shell2(t, d, is, js, ks)) return;
  const AxisA X = axis_a(a.sxmin, a.sx, is, a.bxmin, a.delx);
  const AxisA Y = axis_a(a.symin, a.sy, js, a.bymin, a.dely);
  const AxisA Z = axis_a(a.szmin, a.sz, ks, a.bzmin, a.delz);
  if (X.b < 1 || Y.b < 1 || Z.b < 1 || X.b1 > d.nx || Y.b1 > d.ny || Z.b1 > d.nz) return;   // left unchanged
  const size_t c = d.at(is, js, ks);
  const float g = a.a_target[f][c];
  if (g == 0.0f) return;
  float alpha = 1.0f;
  auto apply = [&](int layer) { alpha *= (float)(layer - 1) / 2.0f; };
  if (ks <= 2) apply(ks);
  if (ks >= d.nz - 1) apply(d.nz - ks + 1);
  if (js <= 2) apply(js);
  if (js >= d.ny - 1) apply(d.ny - js + 1);
  if (is <= 2) apply(is);
  if (is >= d.nx - 1) apply(d.nx - is + 1);
  a.a_target[f][c] = alpha * g;
  const float gi = (1.0f - alpha) * g;
  const float t1 = a.t1, t2 = 1.0f - t1;
  const size_t c000 = d.at(X.b, Y.b, Z.b);
  const size_t sx = 1, sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  const size_t off[8] = {0, sz, sy, sy + sz, sx, sx + sz, sx + sy, sx + sy + sz};
  const float w[8] = {X.dd * Y.dd * Z.dd, X.dd * Y.dd * Z.d, X.dd * Y.d * Z.dd, X.dd * Y.d * Z.d,
                      X.d * Y.dd * Z.dd,  X.d * Y.dd * Z.d,  X.d * Y.d * Z.dd,  X.d * Y.d * Z.d};
  for (int q = 0; q < 8; q++) {
    const float v = gi * w[q];
    red(a.a_oldc[f] + c000 + off[q], v * t1);
    red(a.a_curc[f] + c000 + off[q], v * t2);
  }
}

// ------------------------------------------------------------ corer
__global__ void __launch_bounds__(256) k_adj_corer(const __grid_constant__ AdjCorerArgs a) {
  const int q = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.ni * a.nj * a.nk) return;
  const int ks = 1 + a.nskip * (1 + t / (a.ni * a.nj));
  const int js = 1 + a.nskip * (1 + (t / a.ni) % a.nj);
  const int is = 1 + a.nskip * (1 + t % a.ni);
  const int kb = a.nbz1 + (ks - 1) / a.nskip;
  const int jb = a.nby1 + (js - 1) / a.nskip;
  const int ib = a.nbx1 + (is - 1) / a.nskip;
  const Dims d = a.d;
  if (ib < 1 || jb < 1 || kb < 1 || ib > d.nx || jb > d.ny || kb > d.nz) return;
  const size_t cc = d.at(ib, jb, kb);
  const float g = a.a_coarse[q][cc];
  a.a_coarse[q][cc] = 0.0f;
  if (g == 0.0f) return;
  float* F = a.a_fine[q];
  const size_t c = d.at(is, js, ks);
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  const float g1 = g / 12.0f;
  red(F + c, 6.0f * g1);
  red(F + c + 1, g1); red(F + c - 1, g1);
  red(F + c + sy, g1); red(F + c - sy, g1);
  red(F + c + sz, g1); red(F + c - sz, g1);
}

// ------------------------------------------------------------ flanks_synced
__global__ void __launch_bounds__(256) k_adj_synced(const __grid_constant__ AdjSyncedArgs a) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  int is, js, ks;
  const Dims d = a.d;
  if (!shell1_cell(t, d, is, js, ks)) return;
  const size_t c = d.at(is, js, ks);
  const float g = a.a_fine[q][c];
  a.a_fine[q][c] = 0.0f;
  if (g == 0.0f) return;
  float* Fb = a.a_coarse[q];
  auto A = [&](int i, int j, int k, float v) {
    i = i < 1 ? 1 : (i > d.nx ? d.nx : i);
    j = j < 1 ? 1 : (j > d.ny ? d.ny : j);
    k = k < 1 ? 1 : (k > d.nz ? d.nz : k);
    red(Fb + d.at(i, j, k), v);
  };
  if (is == 1 || is == d.nx) {
    const AxisA Y = axis_a(a.symin, a.sy, js, a.bymin, a.dely);
    const AxisA Z = axis_a(a.szmin, a.sz, ks, a.bzmin, a.delz);
    const int ib = is == 1 ? a.ib_bot : a.ib_top;
    A(ib, Y.b, Z.b, g * Y.dd * Z.dd); A(ib, Y.b1, Z.b, g * Y.d * Z.dd);
    A(ib, Y.b, Z.b1, g * Y.dd * Z.d); A(ib, Y.b1, Z.b1, g * Y.d * Z.d);
  } else if (js == 1 || js == d.ny) {
    const AxisA X = axis_a(a.sxmin, a.sx, is, a.bxmin, a.delx);
    const AxisA Z = axis_a(a.szmin, a.sz, ks, a.bzmin, a.delz);
    const int jb = js == 1 ? a.jb_bot : a.jb_top;
    A(X.b, jb, Z.b, g * X.dd * Z.dd); A(X.b, jb, Z.b1, g * X.dd * Z.d);
    A(X.b1, jb, Z.b, g * X.d * Z.dd); A(X.b1, jb, Z.b1, g * X.d * Z.d);
  } else {
    const AxisA X = axis_a(a.sxmin, a.sx, is, a.bxmin, a.delx);
    const AxisA Y = axis_a(a.symin, a.sy, js, a.bymin, a.dely);
    const int kb = ks == 1 ? a.kb_bot : a.kb_top;
    A(X.b, Y.b, kb, g * X.dd * Y.dd); A(X.b, Y.b1, kb, g * X.dd * Y.d);
    A(X.b1, Y.b, kb, g * X.d * Y.dd); A(X.b1, Y.b1, kb, g * X.d * Y.d);
  }
}

// ------------------------------------------------------------ div B
// The projection B' = B - G(s A^-1 D B) (s = rx^2; D the central
// divergence and G the central gradient, both on the interior; A the
// symmetric 7-point Laplacian the CG inverts).  Its reverse: rhs =
// -s G^T a_b, z = A^-1 rhs (solved by the caller), a_b += D^T z.
__global__ void __launch_bounds__(256) k_adj_divb_rhs(const __grid_constant__ AdjDivbArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok) return;
  const size_t c = p.c;
  const size_t sy = d.nx, sz = (size_t)d.nx * d.ny;
  auto inner = [&](int i, int j, int k) { return i > 1 && j > 1 && k > 1 && i < d.nx && j < d.ny && k < d.nz; };
  float v = 0.0f;
  if (inner(p.i + 1, p.j, p.k)) v += a.a_b[0][c + 1];
  if (inner(p.i - 1, p.j, p.k)) v -= a.a_b[0][c - 1];
  if (inner(p.i, p.j + 1, p.k)) v += a.a_b[1][c + sy];
  if (inner(p.i, p.j - 1, p.k)) v -= a.a_b[1][c - sy];
  if (inner(p.i, p.j, p.k + 1)) v += a.a_b[2][c + sz];
  if (inner(p.i, p.j, p.k - 1)) v -= a.a_b[2][c - sz];
  a.rhs[c] = (a.rx * a.rx) * (v / (2.0f * a.rx));
}

__global__ void __launch_bounds__(256) k_adj_divb_apply(const __grid_constant__ AdjDivbArgs a) {
  const Dims d = a.d;
  const Cell3 p = cell3(d);
  if (!p.ok) return;
  const size_t c = p.c;
  const size_t sy = d.nx, sz = (size_t)d.nx * d.ny;
  auto inner = [&](int i, int j, int k) { return i > 1 && j > 1 && k > 1 && i < d.nx && j < d.ny && k < d.nz; };
  const float r = 1.0f / (2.0f * a.rx);
  float gx = 0.0f, gy = 0.0f, gz = 0.0f;
  if (inner(p.i - 1, p.j, p.k)) gx += a.z[c - 1];
  if (inner(p.i + 1, p.j, p.k)) gx -= a.z[c + 1];
  if (inner(p.i, p.j - 1, p.k)) gy += a.z[c - sy];
  if (inner(p.i, p.j + 1, p.k)) gy -= a.z[c + sy];
  if (inner(p.i, p.j, p.k - 1)) gz += a.z[c - sz];
  if (inner(p.i, p.j, p.k + 1)) gz -= a.z[c + sz];
  a.a_b[0][c] += gx * r;
  a.a_b[1][c] += gy * r;
  a.a_b[2][c] += gz * r;
}

// ------------------------------------------------------------ the loss
// Trilinear samples of bx, by, bz and the total density at the sample
// positions in the smallest box holding each (findgrid, cft_findgrid.f90:
// 70-126; trilin_interp, cft_trilin_interp.f90:34-54); forward: residuals
// and the summed squared misfit; reverse: 2 r times the weights into the
// adjoints of the eight corner cells.
__global__ void k_loss(const __grid_constant__ LossArgs a, int reverse) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  double part = 0.0;
  if (n < a.n) {
    const float* X = a.xyz + 3 * n;
    float v[3] = {X[0] / a.re_equiv, X[1] / a.re_equiv, X[2] / a.re_equiv};
    int box = 0;
    for (int b = 1; b <= a.n_grids; b++) {
      const float* mn = a.gmin + 3 * (b - 1);
      const float* mx = a.gmax + 3 * (b - 1);
      if (v[0] > mn[0] && v[1] > mn[1] && v[2] > mn[2] && v[0] < mx[0] && v[1] < mx[1] && v[2] < mx[2]) {
        box = b;
        break;
      }
    }
    bool inside = box > 0;
    int g[3] = {0, 0, 0};
    float w[3] = {0.0f, 0.0f, 0.0f};
    if (inside) {
      for (int q = 0; q < 3; q++) {
        const float lo = a.gmin[3 * (box - 1) + q];
        g[q] = 1 + (int)((v[q] - lo) / a.xspac[box - 1]);
        const float c0 = (lo + ((float)g[q] - 1.0f) * a.xspac[box - 1]) * a.re_equiv;
        w[q] = (X[q] - c0) / (a.xspac[box - 1] * a.re_equiv);
      }
      const int lim[3] = {a.d.nx, a.d.ny, a.d.nz};
      for (int q = 0; q < 3; q++) inside &= g[q] >= 1 && g[q] < lim[q];
    }
    if (inside) {
      const int b = box - 1;
      size_t idx[8];
      float wt[8];
      int t = 0;
      for (int dk = 0; dk < 2; dk++)
        for (int dj = 0; dj < 2; dj++)
          for (int di = 0; di < 2; di++) {
            idx[t] = a.d.at(g[0] + di, g[1] + dj, g[2] + dk);
            wt[t] = (di ? w[0] : 1.0f - w[0]) * (dj ? w[1] : 1.0f - w[1]) * (dk ? w[2] : 1.0f - w[2]);
            t++;
          }
      float* R = a.resid + 4 * n;
      if (!reverse) {
        for (int q = 0; q < 4; q++) {
          float val = 0.0f;
          for (int u = 0; u < 8; u++) {
            const float fv = q < 3 ? __ldg(a.f[b][q] + idx[u])
                                   : __ldg(a.rho[b][0] + idx[u]) + __ldg(a.rho[b][1] + idx[u]) +
                                         __ldg(a.rho[b][2] + idx[u]);
            val += wt[u] * fv;
          }
          R[q] = val - a.target[4 * n + q];
          part += (double)R[q] * (double)R[q];
        }
      } else {
        for (int q = 0; q < 4; q++) {
          const float gq = 2.0f * R[q];
          for (int u = 0; u < 8; u++) {
            if (q < 3) {
              red(a.a_f[b][q] + idx[u], gq * wt[u]);
            } else {
              for (int s = 0; s < 3; s++) red(a.a_rho[b][s] + idx[u], gq * wt[u]);
            }
          }
        }
      }
    } else if (!reverse) {
      for (int q = 0; q < 4; q++) a.resid[4 * n + q] = 0.0f;
    }
  }
  if (!reverse) {
    for (int s = 16; s > 0; s >>= 1) part += __shfl_xor_sync(0xffffffffu, part, s);
    if ((threadIdx.x & 31) == 0 && part != 0.0) atomicAdd(a.loss, part);
  }
}

// ------------------------------------------------------------ helpers
struct FieldPtrs {
  const float* p[G3M3_NFIELDS];
};
struct FieldPtrsW {
  float* p[G3M3_NFIELDS];
};

__global__ void k_copy_fields(float* __restrict__ dst, const __grid_constant__ FieldPtrs src, int nf, size_t n) {
  const int f = blockIdx.y;
  if (f >= nf) return;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    dst[(size_t)f * n + c] = __ldg(src.p[f] + c);
}

// the fields into a block, each source cleared behind the copy
__global__ void k_move_fields(float* __restrict__ dst, const __grid_constant__ FieldPtrsW src, int nf, size_t n) {
  const int f = blockIdx.y;
  if (f >= nf) return;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    dst[(size_t)f * n + c] = src.p[f][c];
    src.p[f][c] = 0.0f;
  }
}

__global__ void k_copy_fields_out(const __grid_constant__ FieldPtrsW dst, const float* __restrict__ src, int nf,
                                  size_t n) {
  const int f = blockIdx.y;
  if (f >= nf) return;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    dst.p[f][c] = __ldg(src + (size_t)f * n + c);
}

__global__ void k_zero(float* p, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    p[c] = 0.0f;
}

__global__ void k_axpy(float* y, const float* __restrict__ x, size_t n) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    y[c] += x[c];
}

inline dim3 cells_grid(const Dims& d, const dim3& b) { return dim3(blocks_for(d.cells(), b.x * b.y * b.z)); }
inline unsigned tcount(const dim3& b) { return b.x * b.y * b.z; }

}  // namespace

void launch_adj_push_ion(const AdjPushIonArgs& a, cudaStream_t s) {
  if (a.boundary_from_old) {
    const long n = shell_count(a.d, 1);
    k_adj_push_ion_shell<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
  }
  const dim3 blk(32, 2, 2);
  k_adj_push_ion<<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
}

void launch_adj_push_field(const AdjPushFieldArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2);
  k_adj_push_field<<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
}

void launch_adj_fields(const AdjFieldsArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2);
  const unsigned pw = blocks_for(a.d.cells(), 256) < 8u * sm_count() ? blocks_for(a.d.cells(), 256) : 8u * sm_count();
  k_adj_bande<<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
  k_adj_evel<<<pw, 256, 0, s>>>(a);
  k_adj_total_b<<<pw, 256, 0, s>>>(a);
  k_adj_curl<<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
}

void launch_adj_lap(const AdjLapArgs& a, cudaStream_t s) {
  const dim3 blk(32, 2, 2);
  if (a.nf <= 4) k_adj_lap<4><<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
  else k_adj_lap<10><<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
}

void launch_adj_vtot(const AdjVtotArgs& a, cudaStream_t s) {
  const unsigned pw = blocks_for(a.d.cells(), 256) < 8u * sm_count() ? blocks_for(a.d.cells(), 256) : 8u * sm_count();
  k_adj_vtot<<<pw, 256, 0, s>>>(a);
}

void launch_adj_fcs(const AdjFcsArgs& a, cudaStream_t s) {
  const unsigned blk = 256;
  const dim3 grd(blocks_for(a.d.cells(), blk), (unsigned)a.nf);
  k_fcs_p1<<<grd, blk, 0, s>>>(a);
  k_adj_fcs_faces<<<grd, blk, 0, s>>>(a);
  AdjFcsArgs b = a;
  b.clear_px = 1;
  k_adj_fcs_gather<<<grd, blk, 0, s>>>(b);
  k_adj_p1<<<grd, blk, 0, s>>>(b);
}

void launch_adj_guard(const AdjGuardArgs& a, cudaStream_t s) {
  const dim3 blk(32, 2, 2);
  cudaMemsetAsync(a.list_count, 0, sizeof(unsigned), s);
  k_adj_guard_a<<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
  k_adj_guard_b<<<sm_count(), 128, 0, s>>>(a);
}

void launch_adj_outer(const AdjOuterArgs& a, cudaStream_t s) {
  const long n = shell_count(a.d, 1);
  k_adj_outer<<<dim3((unsigned)((n + 255) / 256), G3M3_NFIELDS), 256, 0, s>>>(a);
}

void launch_adj_inner(const AdjInnerArgs& a, cudaStream_t s) {
  const int n = a.num[0] + a.num[1] + a.num[2];
  if (n <= 0) return;
  k_adj_inner<<<(n + 127) / 128, 128, 0, s>>>(a);
}

void launch_adj_flanks(const AdjFlanksArgs& a, cudaStream_t s) {
  const long n = shell_count(a.d, 2);
  k_adj_flanks<<<dim3((unsigned)((n + 255) / 256), (unsigned)a.nf), 256, 0, s>>>(a);
}

void launch_adj_corer(const AdjCorerArgs& a, cudaStream_t s) {
  const int n = a.ni * a.nj * a.nk;
  if (n <= 0) return;
  k_adj_corer<<<dim3((unsigned)((n + 255) / 256), (unsigned)a.nf), 256, 0, s>>>(a);
}

void launch_adj_synced(const AdjSyncedArgs& a, cudaStream_t s) {
  const long n = shell_count(a.d, 1);
  k_adj_synced<<<dim3((unsigned)((n + 255) / 256), (unsigned)a.nf), 256, 0, s>>>(a);
}

void launch_adj_divb_rhs(const AdjDivbArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2);
  k_adj_divb_rhs<<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
}

void launch_adj_divb_apply(const AdjDivbArgs& a, cudaStream_t s) {
  const dim3 blk(32, 4, 2);
  k_adj_divb_apply<<<cells_grid(a.d, blk), tcount(blk), 0, s>>>(a);
}

void launch_loss(const LossArgs& a, cudaStream_t s, bool reverse) {
  if (a.n <= 0) return;
  k_loss<<<(a.n + 127) / 128, 128, 0, s>>>(a, reverse ? 1 : 0);
}

void launch_copy_fields(float* dst, const float* const src[], int nf, size_t n, cudaStream_t s) {
  FieldPtrs p{};
  for (int f = 0; f < nf; f++) p.p[f] = src[f];
  const unsigned bx = blocks_for(n, 256) < 4u * sm_count() ? blocks_for(n, 256) : 4u * sm_count();
  k_copy_fields<<<dim3(bx, (unsigned)nf), 256, 0, s>>>(dst, p, nf, n);
}

void launch_move_fields(float* dst, float* const src[], int nf, size_t n, cudaStream_t s) {
  FieldPtrsW p{};
  for (int f = 0; f < nf; f++) p.p[f] = src[f];
  const unsigned bx = blocks_for(n, 256) < 4u * sm_count() ? blocks_for(n, 256) : 4u * sm_count();
  k_move_fields<<<dim3(bx, (unsigned)nf), 256, 0, s>>>(dst, p, nf, n);
}

void launch_copy_fields_out(float* const dst[], const float* src, int nf, size_t n, cudaStream_t s) {
  FieldPtrsW p{};
  for (int f = 0; f < nf; f++) p.p[f] = dst[f];
  const unsigned bx = blocks_for(n, 256) < 4u * sm_count() ? blocks_for(n, 256) : 4u * sm_count();
  k_copy_fields_out<<<dim3(bx, (unsigned)nf), 256, 0, s>>>(p, src, nf, n);
}

void launch_zero(float* p, size_t n, cudaStream_t s) {
  const unsigned b = blocks_for(n, 256) < 8u * sm_count() ? blocks_for(n, 256) : 8u * sm_count();
  k_zero<<<b, 256, 0, s>>>(p, n);
}

void launch_axpy(float* y, const float* x, size_t n, cudaStream_t s) {
  const unsigned b = blocks_for(n, 256) < 8u * sm_count() ? blocks_for(n, 256) : 8u * sm_count();
  k_axpy<<<b, 256, 0, s>>>(y, x, n);
}

}  // namespace g3m3
