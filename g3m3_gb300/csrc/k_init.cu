// k_init.cu -- the fresh-start state on the device: dipole background
// (sub_dipole.f90:4-52, no rotation or tilt), corotating ionospheric plasma
// (3d_main.f90:1291-1367), the solar-wind fill with its ramp (:1466-1585),
// the speed clip (:1589-1625) and a seeded perturbation of density and
// diagonal pressures.  Arithmetic in FP64, rounded to FP32 once per value,
// as the host restatement (g3m3_gb300/state.py) does.
#include "kargs.cuh"
#include "launch.cuh"

namespace g3m3 {

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  // SplitMix64 finaliser (Steele, Lea, Flood 2014)
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// standard normal from a counter (Box-Muller on two 53-bit uniforms)
__device__ double normal_at(unsigned long long seed, unsigned long long counter) {
  const unsigned long long a = mix64(seed ^ mix64(2 * counter));
  const unsigned long long b = mix64(seed ^ mix64(2 * counter + 1));
  const double u1 = ((double)(a >> 11) + 1.0) * 0x1p-53;   // (0, 1]
  const double u2 = (double)(b >> 11) * 0x1p-53;           // [0, 1)
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

__global__ void __launch_bounds__(256) k_init(const __grid_constant__ InitArgs a) {
  const Dims d = a.d;
  const size_t n = d.cells();
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.nx), j = (int)((c / d.nx) % d.ny), k = (int)(c / ((size_t)d.nx * d.ny));
    const double xdip = 0.00001;
    const double ax = (double)a.xmin + a.dx * i - xdip;
    const double ay = (double)a.ymin + a.dy * j;
    const double az = (double)a.zmin + a.dz * k;
    const double ar = sqrt(ax * ax + ay * ay + az * az);
    // dipole (sub_dipole.f90:30-40) about x = xdip
    {
      const double x1 = (ax + xdip) - xdip, y1 = ay, z1 = az;
      const double x2 = x1 * x1, y2 = y1 * y1, z2 = z1 * z1;
      const double r = sqrt(x2 + y2 + z2);
      const double bmag = -a.b0c / pow(r, 5.0);
      const bool inside = ar < a.zero_b;
      a.b0[0][c] = inside ? 0.0f : (float)(-3.0 * bmag * x1 * z1);
      a.b0[1][c] = inside ? 0.0f : (float)(-3.0 * bmag * y1 * z1);
      a.b0[2][c] = inside ? 0.0f : (float)(bmag * (x2 + y2 - 2.0 * z2));
    }
    // corotation (3d_main.f90:1296-1308)
    const double rx = ax * a.re_equiv, ry = ay * a.re_equiv;
    const double rd = sqrt(rx * rx + ry * ry);
    const double rr2 = a.r_rot * a.r_rot;
    const double vq = (2.0 * rr2) / (rr2 + rd * rd);
    const double vfrac = rd < a.r_rot ? 1.0 : vq * vq;
    const double rvy = rx * a.v_rot * vfrac, rvx = -ry * a.v_rot * vfrac;
    // ionospheric plasma (3d_main.f90:1310-1367)
    const double ar_iono = fmax(sqrt(ax * ax + ay * ay + 1.25 * az * az), 0.0001);
    double ra = pow((ar_iono + 0.5 * a.r_inner) / (1.5 * a.r_inner), -a.alpha_e);
    const double h15 = 1.5 * a.r_inner, h30 = 3.0 * a.r_inner;
    const double zheight = fmax(1.0, (az * az + h15 * h15) / (h30 * h30));
    ra = ra / (zheight * zheight);
    const double rho_iono = fmax(a.erho * ra, a.d_min);
    const double arho = fmax(rho_iono, a.d_min);
    const double vt = fmax(sqrt(rvy * rvy + rvx * rvx), a.cs_inner);
    const double qrho = arho * a.rmass[0] / zheight;
    const double qpres = arho * vt;
    const double hrho = 0.05 * qrho * a.rmass[1] / a.rmass[0];
    const double hpres = 0.05 * qpres;
    const double orho = qrho * a.rmass[2] / a.rmass[0];
    const double opres = qpres;
    double sp[3][5] = {{qrho, qrho * rvx, qrho * rvy, 0.0 * qrho, qpres},
                       {hrho, hrho * rvx, hrho * rvy, 0.0 * hrho, hpres},
                       {orho, orho * rvx, orho * rvy, 0.0 * orho, opres}};
    double epres = (qpres + hpres + opres) / a.ti_te;
    // solar wind (3d_main.f90:1466-1585)
    const double wind_bnd = a.r_rot / a.re_equiv;
    const double ar0 = sqrt(ax * ax + ay * ay + az * az);
    const bool full = ar0 >= 1.5 * wind_bnd && ax < 0.0;
    const bool ramp = ar0 > wind_bnd && ar0 < 1.5 * wind_bnd && ax < 0.0;
    const double dfrac = full ? 1.0 : (ramp ? (ar0 - wind_bnd) / (0.5 * wind_bnd) : 0.0);
    const double g = a.gamma;
    const double cs_wind2 = a.spress * (g - 1.0) * g / a.srho;
    const double qr = sp[0][0] + a.srho * dfrac;
    const double qpx = sp[0][1] + a.spx * dfrac;
    const double qpy = sp[0][2] + a.spy * dfrac;
    const double qpz = sp[0][3] + a.spz * dfrac;
    const double avx = qpx / qr, avy = qpy / qr, avz = qpz / qr;
    const double apres = cs_wind2 * qr / g;
    const bool wind = dfrac > 0.0;
    sp[0][0] = qr; sp[0][1] = qpx; sp[0][2] = qpy; sp[0][3] = qpz;
    sp[0][4] = wind ? 0.5 * apres * dfrac + qpres : qpres;
    epres = wind ? 0.5 * apres / a.ti_te * dfrac + epres : epres;
    const double hr = hrho + a.srho * a.rho_frac * a.rmass[1] / a.rmass[0] * dfrac;
    sp[1][0] = hr;
    sp[1][1] = wind ? avx * hr : sp[1][1];
    sp[1][2] = wind ? avy * hr : sp[1][2];
    sp[1][3] = wind ? avz * hr : 0.0 * hr;
    sp[1][4] = hpres + 0.5 * a.spress * a.rho_frac * dfrac;
    const double orr = orho + a.srho * a.rho_frac * a.rmass[2] / a.rmass[0] * dfrac;
    sp[2][0] = orr;
    sp[2][1] = wind ? avx * orr : sp[2][1];
    sp[2][2] = wind ? avy * orr : sp[2][2];
    sp[2][3] = wind ? avz * orr : 0.0 * orr;
    sp[2][4] = opres + 0.5 * a.spress * a.rho_frac * dfrac;
    // speed clip (3d_main.f90:1589-1625)
    for (int s = 0; s < 3; s++) {
      const double r = sp[s][0];
      const double vx = sp[s][1] / r, vy = sp[s][2] / r, vz = sp[s][3] / r;
      if (sqrt(vx * vx + vy * vy + vz * vz) > 1.0) { sp[s][1] = 0.0; sp[s][2] = 0.0; sp[s][3] = 0.0; }
    }
    // seeded multiplicative perturbation of density and diagonal pressures
    const unsigned long long base = ((unsigned long long)a.box << 40) + (unsigned long long)c * 16;
    for (int s = 0; s < 3; s++) {
      const double nr = a.noise > 0.0f ? 1.0 + a.noise * normal_at(a.seed, base + 4 * s) : 1.0;
      a.f[10 * s + 0][c] = (float)(sp[s][0] * nr);
      a.f[10 * s + 1][c] = (float)sp[s][1];
      a.f[10 * s + 2][c] = (float)sp[s][2];
      a.f[10 * s + 3][c] = (float)sp[s][3];
      for (int q = 0; q < 3; q++) {
        const double np = a.noise > 0.0f ? 1.0 + a.noise * normal_at(a.seed, base + 4 * s + 1 + q) : 1.0;
        a.f[10 * s + 4 + q][c] = (float)(sp[s][4] * np);
      }
      for (int q = 7; q < 10; q++) a.f[10 * s + q][c] = 0.0f;
    }
    a.f[G3M3_F_EPRES][c] = (float)epres;
    a.f[G3M3_F_BX][c] = 0.0f;
    a.f[G3M3_F_BY][c] = 0.0f;
    a.f[G3M3_F_BZ][c] = 0.0f;
  }
}

}  // namespace

void launch_init(const InitArgs& a, cudaStream_t s) {
  const size_t n = a.d.cells();
  unsigned blocks = (unsigned)((n + 255) / 256);
  if (blocks > 16u * sm_count()) blocks = 16u * sm_count();
  k_init<<<blocks, 256, 0, s>>>(a);
}

}  // namespace g3m3
