// divide.cuh -- FP64 division from a precomputed reciprocal, correctly
// rounded (the quotient the division operator gives), for divisors that
// stay fixed over many divisions: the reference SOR's diagonal, the plain
// path's metric factors and implicit-damping factors.  GB300's FP64 rate is
// low; the division operator takes about twice the FP64 operations of the
// sequence below.
#pragma once
#include <cuda_runtime.h>

namespace swm {

// a / b rounded to nearest from y = 1/b rounded to nearest, by Markstein's
// theorem (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34, 1990; also Muller et
// al., Handbook of Floating-Point Arithmetic, the FMA-based division
// section): if y is within half an ulp of 1/b and q within one ulp of a/b,
// then q + (a - b q) y, each operation rounded to nearest and the remainder
// taken with one FMA, is a/b rounded to nearest.  q = a y can be up to 1.5
// ulp off, so a first correction brings it within an ulp and the second
// gives the rounded quotient.  Valid while no step underflows or overflows:
// for a and b with binary exponents in [-500, 500] (div_rn_range).
__device__ __forceinline__ double div_rn(double a, double b, double y) {
  double q = __dmul_rn(a, y);
  double r = __fma_rn(-q, b, a);
  q = __fma_rn(r, y, q);
  r = __fma_rn(-q, b, a);
  return __fma_rn(r, y, q);
}

// x is finite, nonzero, normal and of binary exponent in [-500, 500]
__device__ __forceinline__ bool div_rn_range(double x) {
  const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
  return e - 523u <= 1000u;
}

// a / b given y = 1/b rounded to nearest, with b of binary exponent in
// [-500, 500]: div_rn where a is in its range, a * y for a zero numerator
// (the zero of the quotient's sign), the division operator otherwise
__device__ __forceinline__ double div_fast(double a, double b, double y) {
  if (div_rn_range(a)) return div_rn(a, b, y);
  return a == 0. ? a * y : a / b;
}

// the host's check of a divisor for div_fast
inline bool div_host_range(double x) {
  if (!(x - x == 0.) || x == 0.) return false;  // infinite, NaN or zero
  int e = 0;
  const double m = __builtin_frexp(x < 0 ? -x : x, &e);
  (void)m;
  return e - 1 >= -500 && e - 1 <= 500;
}

}  // namespace swm
