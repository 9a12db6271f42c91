/*
 * dual.h -- TEST INFRASTRUCTURE: forced in front of the oracle's sources
 * (g++ -x c++ -include dual.h) to build liboracle_dual.so, the FP64 build
 * (real8.h) differentiated in forward mode: every REAL of the restatement
 * is a dual number (value, tangent) of doubles, each operation carries the
 * tangent by its derivative (the rules below), and the wind-face
 * parameters that bndry_outer reads take their tangents from
 * oracle_wind_tangent[8] (srho, spx, spy, spz, spress, sbx/sby/sbz_wind).
 * One run gives the misfit's exact directional derivative along the FP64
 * trajectory: a gradient reference without a difference quotient's step.
 *
 * Branches (max, min, sign, the guards' and limiters' comparisons) compare
 * values only and pass the tangent of the operand they chose, as the
 * library's reverse does.  The arrays hold (value, tangent) pairs, the
 * layout of complex128 with the value as the real part.
 */
#ifndef G3M3_ORACLE_DUAL_H
#define G3M3_ORACLE_DUAL_H
#include <math.h>

#include "../include/g3m3_types.h"

struct Dual {
  double v, d;
  Dual() = default;
  constexpr Dual(double x) : v(x), d(0.0) {}
  constexpr Dual(double x, double t) : v(x), d(t) {}
  explicit operator double() const { return v; }
  explicit operator int() const { return (int)v; }
  Dual& operator+=(const Dual& b) { v += b.v; d += b.d; return *this; }
  Dual& operator-=(const Dual& b) { v -= b.v; d -= b.d; return *this; }
  Dual& operator*=(const Dual& b) { d = d * b.v + v * b.d; v *= b.v; return *this; }
  Dual& operator/=(const Dual& b) { const double q = v / b.v; d = (d - q * b.d) / b.v; v = q; return *this; }
};

inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
inline Dual operator+(const Dual& a) { return a; }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
inline bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }

inline Dual sqrt(const Dual& a) {
  const double r = sqrt(a.v);
  return Dual(r, r > 0.0 ? a.d / (2.0 * r) : 0.0);
}
inline Dual fabs(const Dual& a) {
  return Dual(fabs(a.v), a.v > 0.0 ? a.d : (a.v < 0.0 ? -a.d : 0.0));
}
inline Dual floor(const Dual& a) { return Dual(floor(a.v), 0.0); }

// the OpenMP reductions the restatement uses, on dual numbers
#pragma omp declare reduction(max : Dual : omp_out = (omp_in > omp_out ? omp_in : omp_out)) \
    initializer(omp_priv = Dual(-HUGE_VAL))
#pragma omp declare reduction(min : Dual : omp_out = (omp_in < omp_out ? omp_in : omp_out)) \
    initializer(omp_priv = Dual(HUGE_VAL))
#pragma omp declare reduction(+ : Dual : omp_out += omp_in) initializer(omp_priv = Dual(0.0))

extern "C" {
inline double oracle_wind_tangent[8] = {};   // one definition across the build
}

#define ORACLE_WIND(k, val) Dual((double)(val), oracle_wind_tangent[k])
#define float Dual
#define sqrtf sqrt
#define fabsf fabs
#define floorf floor
#endif
