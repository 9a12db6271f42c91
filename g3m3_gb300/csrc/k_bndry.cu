// k_bndry.cu -- boundaries and nested-grid coupling:
//   bndry_outer    sub_bndry_outer.f90:5-731
//   bndry_inner    sub_bndry_inner.f90:5-268
//   flanks         sub_flanks.f90:5-303 (via sub_bndry_flanks.f90:105-209)
//   corer          sub_corer.f90:5-55 (via sub_bndry_corer.f90:42-111)
//   flanks_synced  sub_flanks_synced.f90:5-141
#include <unordered_map>
#include <unordered_set>

#include "bndry.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

// Cells of the D-deep outer shell of a box, enumerated as x slabs, then y
// slabs (x interior), then z slabs (x and y interior).  In the x slabs the
// D cells of one side of a grid row are neighbours in the enumeration
// (i fastest, then j, then k), so that adjacent threads touch the same
// 32-byte sectors of the row.
__device__ __forceinline__ bool shell_cell(long t, int D, const Dims& d, int& i, int& j, int& k) {
  const long nyz = (long)d.ny * d.nz;
  const long xs = 2L * D * nyz;
  if (t < xs) {
    const long half = (long)D * nyz;
    const int side = (int)(t / half);      // 0: i = 1..D, 1: i = nx-D+1..nx
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

// ------------------------------------------------------------ bndry_outer
// Value of field f at (i,j,k) after the first S statements groups of
// bndry_outer, following the reference's copy chain:
//   1 wind face i=1        2 back wall i=nx        3 y faces (i>=2)
//   4 top face k=nz (i>=2) 5 bottom face k=1 (i>=2)
//   6 back-wall corner lines (nx,1|ny,k)           7 (nx,j,1|nz)
//   8 edge lines (i,1|ny,1|nz), i>=2
// Every chain ends in an interior cell or the wind face.
struct Outer {
  const OuterArgs* a;
  int f, comp;   // comp: 1,2,3 for the momentum components px,py,pz, else 0
};

__device__ float wind_value(const Outer& o, int j, int k) {
  const OuterArgs& a = *o.a;
  const int f = o.f;
  const float ofrac = a.rho_frac * a.o_conc;
  const float frac_h = a.rmassh / a.rmassq;
  const float frac_o = a.rmasso / a.rmassq;
  if (f >= 30) {
    if (f == G3M3_F_EPRES) return 0.5f * a.spress / a.ti_te;
    const size_t c = o.a->d.at(1, j, k);
    if (f == G3M3_F_BX) return a.sbx_wind - __ldg(a.b0[0] + c);
    if (f == G3M3_F_BY) return a.sby_wind - __ldg(a.b0[1] + c);
    return a.sbz_wind - __ldg(a.b0[2] + c);
  }
  const int s = f / 10, q = f % 10;
  if (q >= 7) return 0.0f;
  if (s == 0) {
    switch (q) {
      case 0: return a.srho;
      case 1: return a.spx;
      case 2: return a.spy;
      case 3: return a.spz;
      default: return 0.5f * a.spress;
    }
  }
  const float fr = s == 1 ? a.rho_frac : ofrac;
  const float mf = s == 1 ? frac_h : frac_o;
  switch (q) {
    case 0: return a.srho * fr * mf;
    case 1: return a.spx * fr * mf;
    case 2: return a.spy * fr * mf;
    case 3: return a.spz * fr * mf;
    default: return 0.5f * a.spress * fr;
  }
}

template <int S>
__device__ float outer_val(const Outer& o, int i, int j, int k) {
  const Dims& d = o.a->d;
  const int nx = d.nx, ny = d.ny, nz = d.nz, nx1 = nx - 1, ny1 = ny - 1, nz1 = nz - 1;
  if constexpr (S == 0) {
    return o.a->f[o.f][d.at(i, j, k)];
  } else {
    if constexpr (S == 8) {
      if (i >= 2 && (j == 1 || j == ny) && (k == 1 || k == nz))
        return outer_val<7>(o, i, j, k == 1 ? 2 : nz1);
    }
    if constexpr (S == 7) {
      if (i == nx && j >= 2 && j <= ny - 1) {
        if (k == 1) return outer_val<6>(o, nx, j, 2);
        if (k == nz && o.f != G3M3_F_EPRES) return outer_val<6>(o, nx1, j, nz);
      }
    }
    if constexpr (S == 6) {
      if (i == nx && (j == 1 || j == ny) && k >= 2 && k <= nz - 1) {
        const int jn = j == 1 ? 2 : ny1;
        if (o.f == G3M3_F_BX) return outer_val<5>(o, nx1, j, k);
        return (outer_val<5>(o, nx1, j, k) + outer_val<5>(o, nx, jn, k)) / 2.0f;
      }
    }
    if constexpr (S == 5) {
      if (k == 1 && i >= 2) {
        const float v = outer_val<4>(o, i, j, 2);
        return o.comp == 3 ? -fabsf(v) : v;
      }
    }
    if constexpr (S == 4) {
      if (k == nz && i >= 2) {
        const float v = outer_val<3>(o, i, j, nz1);
        return o.comp == 3 ? fabsf(v) : v;
      }
    }
    if constexpr (S == 3) {
      if (i >= 2 && (j == 1 || j == ny)) {
        const float v = outer_val<2>(o, i, j == 1 ? 2 : ny1, k);
        if (o.comp == 2) return j == 1 ? -fabsf(v) : fabsf(v);
        return v;
      }
    }
    if constexpr (S == 2) {
      if (i == nx) {
        const float v = outer_val<1>(o, nx1, j, k);
        return o.comp == 1 ? fabsf(v) : v;
      }
    }
    if constexpr (S == 1) {
      if (i == 1) return wind_value(o, j, k);
    }
    return outer_val<S - 1>(o, i, j, k);
  }
}

__global__ void __launch_bounds__(256) k_bndry_outer(const __grid_constant__ OuterArgs a) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int f = blockIdx.y;
  int i, j, k;
  if (!shell_cell(t, 1, a.d, i, j, k)) return;
  Outer o{&a, f, f < 30 ? ((f % 10) >= 1 && (f % 10) <= 3 ? f % 10 : 0) : 0};
  const float v = outer_val<8>(o, i, j, k);
  // all reads above are of interior cells or of b0; no other thread writes them
  a.f[f][a.d.at(i, j, k)] = v;
}

// ------------------------------------------------------------ bndry_inner
// entry m of list l (sub_bndry_inner.f90:81-265)
__device__ void inner_entry(const InnerArgs& a, int l, int m) {
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
  const float rx = ax * a.re_equiv, ry = ay * a.re_equiv;
  const float vfrac = 1.0f;
  const float rvy = rx * a.v_rot * vfrac;
  const float rvx = -ry * a.v_rot * vfrac;
  const float rvz = 0.0f;
  float den[3];
  if (l == 0) {
    den[0] = amax1(P(1), a.f[0][c]);
    den[1] = amax1(P(2), a.f[10][c]);
    den[2] = amax1(P(3), a.f[20][c]);
  } else {
    den[0] = P(1); den[1] = P(2); den[2] = P(3);
  }
#pragma unroll
  for (int s = 0; s < 3; s++) {
    float* const* F = a.f + 10 * s;
    const float pr = P(4 + s);
    F[0][c] = den[s];
    F[4][c] = pr; F[5][c] = pr; F[6][c] = pr;
    F[1][c] = den[s] * rvx; F[2][c] = den[s] * rvy; F[3][c] = den[s] * rvz;
    F[7][c] = 0.0f; F[8][c] = 0.0f; F[9][c] = 0.0f;
  }
  a.f[G3M3_F_EPRES][c] = P(7);
  if (l == 2) {
    a.f[G3M3_F_BX][c] = 0.0f; a.f[G3M3_F_BY][c] = 0.0f; a.f[G3M3_F_BZ][c] = 0.0f;
  }
}

__global__ void __launch_bounds__(128) k_bndry_inner(const __grid_constant__ InnerArgs a) {
  if (a.serial) {   // a list naming a cell twice: its entries in order
    if (blockIdx.x == 0 && threadIdx.x == 0)
      for (int m = 0; m < a.num[a.only - 1]; m++) inner_entry(a, a.only - 1, m);
    return;
  }
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  int l;
  if (a.only) {
    l = a.only - 1;
    if (m >= a.num[l]) return;
  } else if (m < a.num[0]) {
    l = 0;
  } else if ((m -= a.num[0]) < a.num[1]) {
    l = 1;
  } else if ((m -= a.num[1]) < a.num[2]) {
    l = 2;
  } else {
    return;
  }
  inner_entry(a, l, m);
}

// ------------------------------------------------------------ flanks
struct Axis { int b, b1; float d, dd; };

__device__ __forceinline__ Axis flank_axis(float smin, float sp, int idx, float bmin, float del) {
  const float av = smin + sp * (float)(idx - 1);
  const float ai = 1.0f + (av - bmin) / del;
  Axis r;
  r.b = (int)ai;
  r.b1 = r.b + 1;
  r.d = ai - (float)r.b;
  r.dd = 1.0f - r.d;
  return r;
}

template <int MODE>
__global__ void __launch_bounds__(256) k_flanks(const __grid_constant__ FlanksArgs a) {
  // one thread per shell cell; the interpolation geometry is shared by all
  // fields, which the thread then walks (blockIdx.y splits the field list).
  // FLANKS_KEEP also stores each interpolated value I in ibuf; FLANKS_REUSE
  // takes I from there (same coarse data and time weight) and only blends.
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  int is, js, ks;
  const Dims d = a.d;
  if (!shell_cell(t, 2, d, is, js, ks)) return;
  const Axis X = flank_axis(a.sxmin, a.sx, is, a.bxmin, a.delx);
  const Axis Y = flank_axis(a.symin, a.sy, js, a.bymin, a.dely);
  const Axis Z = flank_axis(a.szmin, a.sz, ks, a.bzmin, a.delz);
  // coarse indices outside the coarse box mean the boxes do not nest; the
  // reference would read out of bounds -- leave the cell unchanged instead
  if (X.b < 1 || Y.b < 1 || Z.b < 1 || X.b1 > d.nx || Y.b1 > d.ny || Z.b1 > d.nz) return;
  const float t1 = a.t1.get();
  const float t2 = 1.0f - t1;
  const size_t c000 = d.at(X.b, Y.b, Z.b);
  const size_t sx = 1, sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  const size_t off[8] = {0, sz, sy, sy + sz, sx, sx + sz, sx + sy, sx + sy + sz};
  // trilinear weights in the reference's term order (sub_flanks.f90:75-83)
  const float wgt[8][3] = {{X.dd, Y.dd, Z.dd}, {X.dd, Y.dd, Z.d}, {X.dd, Y.d, Z.dd}, {X.dd, Y.d, Z.d},
                           {X.d, Y.dd, Z.dd},  {X.d, Y.dd, Z.d},  {X.d, Y.d, Z.dd},  {X.d, Y.d, Z.d}};
  const size_t c = d.at(is, js, ks);
  const int f_lo = blockIdx.y * a.fields_per_block;
  const int f_hi = min(a.nf, f_lo + a.fields_per_block);
  const size_t nshell = (size_t)a.nshell;
  // fields in groups of G: every load of a group is issued before its
  // stores, so the loads of a group overlap one another
  constexpr int G = 3;
  for (int f0 = f_lo; f0 < f_hi; f0 += G) {
    float wo[G][8], wc[G][8], tw[G], Ig[G];
#pragma unroll
    for (int g = 0; g < G; g++) {
      if (f0 + g >= f_hi) break;
      if constexpr (MODE == FLANKS_REUSE) {
        Ig[g] = __ldg(a.ibuf + (size_t)(f0 + g) * nshell + t);
      } else {
        const float* __restrict__ oc = a.oldc[f0 + g];
        const float* __restrict__ cc = a.curc[f0 + g];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          wo[g][q] = __ldg(oc + c000 + off[q]);
          wc[g][q] = __ldg(cc + c000 + off[q]);
        }
      }
      tw[g] = a.target[f0 + g][c];
    }
#pragma unroll
    for (int g = 0; g < G; g++) {
      if (f0 + g >= f_hi) break;
      float I;
      if constexpr (MODE == FLANKS_REUSE) {
        I = Ig[g];
      } else {
        float wk[8];
#pragma unroll
        for (int q = 0; q < 8; q++) wk[q] = wo[g][q] * t1 + wc[g][q] * t2;
        I = wk[0] * wgt[0][0] * wgt[0][1] * wgt[0][2];
#pragma unroll
        for (int q = 1; q < 8; q++) I = I + wk[q] * wgt[q][0] * wgt[q][1] * wgt[q][2];
        if constexpr (MODE == FLANKS_KEEP) a.ibuf[(size_t)(f0 + g) * nshell + t] = I;
      }
      float w = tw[g];
      // panels in the reference's order: bottom, top, front, back, left,
      // right; the inner layer blends half and half, the outer layer takes I
      auto apply = [&](int layer) {
        const float frac = (float)(layer - 1) / 2.0f;
        const float frac1 = 1.0f - frac;
        w = frac * w + frac1 * I;
      };
      if (ks <= 2) apply(ks);
      if (ks >= d.nz - 1) apply(d.nz - ks + 1);
      if (js <= 2) apply(js);
      if (js >= d.ny - 1) apply(d.ny - js + 1);
      if (is <= 2) apply(is);
      if (is >= d.nx - 1) apply(d.nx - is + 1);
      a.target[f0 + g][c] = w;
    }
  }
}

// ------------------------------------------------------------ corer
__global__ void __launch_bounds__(256) k_corer(const __grid_constant__ CorerArgs a) {
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
  if (ib < 1 || jb < 1 || kb < 1 || ib > d.nx || jb > d.ny || kb > d.nz) return;   // boxes do not nest
  const float* __restrict__ f = a.fine[q];
  const size_t c = d.at(is, js, ks);
  const size_t sy = (size_t)d.nx, sz = (size_t)d.nx * d.ny;
  a.coarse[q][d.at(ib, jb, kb)] = (6.0f * __ldg(f + c) + __ldg(f + c + 1) + __ldg(f + c - 1)
                                   + __ldg(f + c + sy) + __ldg(f + c - sy)
                                   + __ldg(f + c + sz) + __ldg(f + c - sz)) / 12.0f;
}

// ------------------------------------------------------------ flanks_synced
__global__ void __launch_bounds__(256) k_flanks_synced(const __grid_constant__ SyncedArgs a) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  int is, js, ks;
  const Dims d = a.d;
  if (!shell_cell(t, 1, d, is, js, ks)) return;
  const float* __restrict__ fb = a.coarse[q];
  auto F = [&](int i, int j, int k) {
    // indices outside the coarse box (boxes that do not nest) read the
    // nearest coarse cell instead of out-of-bounds memory
    i = i < 1 ? 1 : (i > d.nx ? d.nx : i);
    j = j < 1 ? 1 : (j > d.ny ? d.ny : j);
    k = k < 1 ? 1 : (k > d.nz ? d.nz : k);
    return __ldg(fb + d.at(i, j, k));
  };
  float v;
  if (is == 1 || is == d.nx) {          // left/right panels are written last
    const Axis Y = flank_axis(a.symin, a.sy, js, a.bymin, a.dely);
    const Axis Z = flank_axis(a.szmin, a.sz, ks, a.bzmin, a.delz);
    const int ib = is == 1 ? a.ib_bot : a.ib_top;
    v = F(ib, Y.b, Z.b) * Y.dd * Z.dd + F(ib, Y.b1, Z.b) * Y.d * Z.dd + F(ib, Y.b, Z.b1) * Y.dd * Z.d
        + F(ib, Y.b1, Z.b1) * Y.d * Z.d;
  } else if (js == 1 || js == d.ny) {
    const Axis X = flank_axis(a.sxmin, a.sx, is, a.bxmin, a.delx);
    const Axis Z = flank_axis(a.szmin, a.sz, ks, a.bzmin, a.delz);
    const int jb = js == 1 ? a.jb_bot : a.jb_top;
    v = F(X.b, jb, Z.b) * X.dd * Z.dd + F(X.b, jb, Z.b1) * X.dd * Z.d + F(X.b1, jb, Z.b) * X.d * Z.dd
        + F(X.b1, jb, Z.b1) * X.d * Z.d;
  } else {
    const Axis X = flank_axis(a.sxmin, a.sx, is, a.bxmin, a.delx);
    const Axis Y = flank_axis(a.symin, a.sy, js, a.bymin, a.dely);
    const int kb = ks == 1 ? a.kb_bot : a.kb_top;
    v = F(X.b, Y.b, kb) * X.dd * Y.dd + F(X.b, Y.b1, kb) * X.dd * Y.d + F(X.b1, Y.b, kb) * X.d * Y.dd
        + F(X.b1, Y.b1, kb) * X.d * Y.d;
  }
  a.fine[q][d.at(is, js, ks)] = v;
}

}  // namespace

long shell_count(const Dims& d, int D) {
  return 2L * D * d.ny * d.nz + 2L * D * (d.nx - 2 * D) * d.nz + 2L * D * (d.nx - 2 * D) * (d.ny - 2 * D);
}

void launch_bndry_outer(const OuterArgs& a, cudaStream_t s) {
  const long n = shell_count(a.d, 1);
  k_bndry_outer<<<dim3((unsigned)((n + 255) / 256), G3M3_NFIELDS), 256, 0, s>>>(a);
}

int launch_bndry_inner(const InnerArgs& a, const InnerOrder& o, cudaStream_t s) {
  if (!o.any()) {
    const int n = a.num[0] + a.num[1] + a.num[2];
    if (n <= 0) return 0;
    k_bndry_inner<<<(n + 127) / 128, 128, 0, s>>>(a);
    return 1;
  }
  int launches = 0;
  for (int l = 0; l < 3; l++) {
    if (a.num[l] <= 0) continue;
    InnerArgs b = a;
    b.only = l + 1;
    b.serial = o.repeat[l] ? 1 : 0;
    if (b.serial) k_bndry_inner<<<1, 1, 0, s>>>(b);
    else k_bndry_inner<<<(a.num[l] + 127) / 128, 128, 0, s>>>(b);
    launches += 1;
  }
  return launches;
}

InnerOrder inner_order(const int* const ij[3], const int num[3], int mbndry, int box, const Dims& d) {
  InnerOrder o;
  std::unordered_map<size_t, int> owner;   // cell -> the list that named it first
  for (int l = 0; l < 3; l++) {
    std::unordered_set<size_t> mine;
    for (int n = 0; n < num[l]; n++) {
      const int i = ij[l][(box - 1) + (size_t)mbndry * (0 + 3 * (size_t)n)];
      const int j = ij[l][(box - 1) + (size_t)mbndry * (1 + 3 * (size_t)n)];
      const int k = ij[l][(box - 1) + (size_t)mbndry * (2 + 3 * (size_t)n)];
      if (i < 1 || j < 1 || k < 1 || i > d.nx || j > d.ny || k > d.nz) continue;
      const size_t c = d.at(i, j, k);
      if (!mine.insert(c).second) o.repeat[l] = true;
      const auto it = owner.emplace(c, l).first;
      if (it->second != l) o.overlap = true;
    }
  }
  return o;
}

void launch_flanks(const FlanksArgs& a, cudaStream_t s) {
  const long n = shell_count(a.d, 2);
  FlanksArgs b = a;
  b.nshell = n;
  b.fields_per_block = 12;   // 34 fields over 3 rows of blocks (12 timed fastest of 3..34 on 121x121x61)
  const unsigned fy = (unsigned)((a.nf + b.fields_per_block - 1) / b.fields_per_block);
  const dim3 grd((unsigned)((n + 255) / 256), fy);
  if (a.mode == FLANKS_KEEP) k_flanks<FLANKS_KEEP><<<grd, 256, 0, s>>>(b);
  else if (a.mode == FLANKS_REUSE) k_flanks<FLANKS_REUSE><<<grd, 256, 0, s>>>(b);
  else k_flanks<FLANKS_PLAIN><<<grd, 256, 0, s>>>(b);
}

void launch_corer(const CorerArgs& a, cudaStream_t s) {
  const int n = a.ni * a.nj * a.nk;
  if (n <= 0) return;
  k_corer<<<dim3((unsigned)((n + 255) / 256), (unsigned)a.nf), 256, 0, s>>>(a);
}

void launch_flanks_synced(const SyncedArgs& a, cudaStream_t s) {
  const long n = shell_count(a.d, 1);
  k_flanks_synced<<<dim3((unsigned)((n + 255) / 256), (unsigned)a.nf), 256, 0, s>>>(a);
}

}  // namespace g3m3
