// exc_divrn.cuh -- the correctly rounded double quotient by a divisor whose correctly
// rounded reciprocal is known (shared by the tracer builds and the division probe).
#pragma once

// x / c correctly rounded, from the correctly rounded reciprocal r_c = RN(1/c) of a divisor
// known at launch: Markstein's quotient correction (P. Markstein, IBM J. Res. Develop. 34
// (1990) 111-119; J.-M. Muller et al., Handbook of Floating-Point Arithmetic, the theorem on
// division with a correctly rounded reciprocal). q = RN(x r_c) is within one ulp of x/c, the
// remainder x - c q is exact in one FMA, and RN(q + (x - c q) r_c) = RN(x/c) -- the IEEE
// quotient, in three FP64 pipe slots where a division takes about eight. It holds while x/c
// and the remainder stay normal (the tracer's operands are far from that range). A zero or
// non-finite x, or an overflowing q, returns q itself, which has the IEEE quotient's sign and
// infinity; the tests are on the bit patterns (integer pipe).
static __device__ __forceinline__ double div_rn(double x, double c, double r_c) {
  const double q = x * r_c;
  const double rem = fma(-c, q, x);
  const double qc = fma(rem, r_c, q);
  const unsigned long long xb = (unsigned long long)__double_as_longlong(x);
  const unsigned long long qb = (unsigned long long)__double_as_longlong(q);
  const bool pass = ((xb << 1) == 0ull) || ((qb & 0x7ff0000000000000ull) == 0x7ff0000000000000ull);
  return pass ? q : qc;
}

