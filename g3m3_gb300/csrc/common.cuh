// common.cuh -- device helpers shared by every G3M^3 kernel.
//
// Arithmetic contract: the library is compiled with -fmad=false and IEEE
// division/sqrt (no fast-math), and every expression keeps the operand order
// of the reference Fortran, so a kernel's FP32 result is bit-for-bit the
// serial CPU restatement's.  Multiplication by the reciprocal is used in
// place of a division only where the divisor is a power of two (grid
// spacings of 2^n), where both give the identical correctly rounded value.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/g3m3.h"

namespace g3m3 {

// Fortran column-major index of (i,j,k), 1-based, inside one box.
struct Dims {
  int nx, ny, nz;
  __host__ __device__ __forceinline__ size_t cells() const {
    return (size_t)nx * (size_t)ny * (size_t)nz;
  }
  __host__ __device__ __forceinline__ size_t at(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
  }
};

// amax1/amin1 as x86 MAXSS/MINSS evaluate them (second operand on ties and
// unordered compares); SIGN(1.,x) with ifort's default treatment of -0.
__device__ __forceinline__ float amax1(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float amin1(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float sign1(float x) { return x >= 0.0f ? 1.0f : -1.0f; }

// A time-dependent scalar: either a value fixed at launch, or a pointer into
// a device table that a captured CUDA graph re-reads on every replay.
struct ScalarRef {
  float v;
  const float* p;
  __device__ __forceinline__ float get() const { return p ? __ldg(p) : v; }
};

__host__ __device__ inline bool is_pow2(float x) {
  if (!(x > 0.0f)) return false;
  // frexp is not available on the device in all modes; use the bits.
  union { float f; uint32_t u; } c{x};
  return (c.u & 0x007fffffu) == 0u && ((c.u >> 23) & 0xffu) != 0u && ((c.u >> 23) & 0xffu) != 0xffu;
}

// x / d, correctly rounded, given r = RN(1/d) (an IEEE division done once
// per denominator): Markstein's correction of the reciprocal product.  For
// q = RN(x r) the residual x - q d is exact in one FMA, and RN(q + rem r)
// is the correctly rounded quotient while nothing under- or overflows: the
// quotient within [2^-124, 2^124] and |x| >= 2^-100, so that the residual is
// a normal number (P. Markstein, "Computation of elementary functions on the
// IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  Outside
// that range the IEEE division is used.  Results are bit-identical to x / d.
__device__ __forceinline__ float div_by(float x, float d, float r) {
  const float q = x * r;
  const float aq = fabsf(q);
  if (aq >= 0x1p-124f && aq <= 0x1p+124f && fabsf(x) >= 0x1p-100f) {
    const float rem = __fmaf_rn(-q, d, x);
    return __fmaf_rn(rem, r, q);
  }
  if (x == 0.0f) return q;   // +-0 with the quotient's sign
  return x / d;
}

// Divide by a grid spacing.  POW2 selects reciprocal multiplication, which is
// exact for power-of-two spacings.
template <bool POW2>
__device__ __forceinline__ float dvd(float a, float d, float rd) {
  if constexpr (POW2) return a * rd; else return a / d;
}

__device__ __forceinline__ float ldg(const float* p) { return __ldg(p); }

}  // namespace g3m3

