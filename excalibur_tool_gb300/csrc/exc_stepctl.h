/* exc_stepctl.h -- the adaptive RK45 controller's step-size factors err**-0.2
 * and err**-0.25 (integrator.py:147-152), from IEEE-754 basic operations only.
 *
 * The reference evaluates them with libm's pow. GPU and host libm differ in the
 * last ulp, and the controller amplifies that: err is a ratio of the small
 * difference y5 - y4, so one ulp in a step size becomes ~1e-9 in the next error
 * estimate and the two step sequences part. Written once here for the device
 * tracers and the C oracle alike, with only +, -, *, /, sqrt, floor, frexp and
 * ldexp (all exact or correctly rounded in both), the factors are bit-identical
 * on both sides and within ~2e-16 relative of the exact powers.
 *
 * Method: x = m 2^e with m in [1/sqrt(2), sqrt(2)); ln m = 2 atanh(s),
 * s = (m - 1) / (m + 1), |s| <= 0.1716, by its odd series to s^23; exp(t) =
 * 2^k exp(r) with k = round(t / ln 2) (ln 2 split Cody-Waite style into a
 * 32-bit head and a tail), |r| <= ln(2)/2, exp(r) by its Taylor series to r^17.
 */
#ifndef EXC_STEPCTL_H
#define EXC_STEPCTL_H

#include <math.h>

#ifdef __CUDACC__
#define EXC_STEPCTL_FN __host__ __device__ __forceinline__
#else
#define EXC_STEPCTL_FN static inline
#endif

#define EXC_LN2_HI 6.93147180369123816490e-01 /* ln 2 rounded to 32 significant bits */
#define EXC_LN2_LO 1.90821492927058770002e-10 /* ln 2 - EXC_LN2_HI */

/* ln x for finite x > 0 (absolute error a few ulp of max(|ln x|, 1)) */
EXC_STEPCTL_FN double exc_ctl_ln(double x) {
  int e;
  double m = frexp(x, &e); /* x = m 2^e, m in [0.5, 1) */
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e = e - 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double p = 1.0 / 23.0;
  p = p * s2 + 1.0 / 21.0;
  p = p * s2 + 1.0 / 19.0;
  p = p * s2 + 1.0 / 17.0;
  p = p * s2 + 1.0 / 15.0;
  p = p * s2 + 1.0 / 13.0;
  p = p * s2 + 1.0 / 11.0;
  p = p * s2 + 1.0 / 9.0;
  p = p * s2 + 1.0 / 7.0;
  p = p * s2 + 1.0 / 5.0;
  p = p * s2 + 1.0 / 3.0;
  p = p * s2 + 1.0;
  const double lnm = 2.0 * s * p;
  const double de = (double)e;
  return de * EXC_LN2_HI + (de * EXC_LN2_LO + lnm);
}

/* exp t for |t| below ~700 */
EXC_STEPCTL_FN double exc_ctl_exp(double t) {
  const double k = floor(t * 1.44269504088896338700 + 0.5);
  const double r = (t - k * EXC_LN2_HI) - k * EXC_LN2_LO;
  double p = 1.0 / 355687428096000.0; /* 1/17! */
  p = p * r + 1.0 / 20922789888000.0;
  p = p * r + 1.0 / 1307674368000.0;
  p = p * r + 1.0 / 87178291200.0;
  p = p * r + 1.0 / 6227020800.0;
  p = p * r + 1.0 / 479001600.0;
  p = p * r + 1.0 / 39916800.0;
  p = p * r + 1.0 / 3628800.0;
  p = p * r + 1.0 / 362880.0;
  p = p * r + 1.0 / 40320.0;
  p = p * r + 1.0 / 5040.0;
  p = p * r + 1.0 / 720.0;
  p = p * r + 1.0 / 120.0;
  p = p * r + 1.0 / 24.0;
  p = p * r + 1.0 / 6.0;
  p = p * r + 0.5;
  p = p * r + 1.0;
  p = p * r + 1.0;
  return ldexp(p, (int)k);
}

/* x^p for p = -0.2 as the reference writes it (the double nearest -1/5, which
 * is -1/5 - d with d = 2^-54 / 5 exactly), x > 0 (inf -> 0, NaN -> NaN). With
 * x = m 2^e and e = 5 q + r (0 <= r < 5): x^p = 2^-q 2^(-r/5) exp(p ln m - d e ln 2);
 * the exponent part is exact scaling times one of five constants, and only the
 * small argument p ln m - d e ln 2 (|.| <= 0.08) goes through the series, so the
 * result stays within a few ulp of pow(x, -0.2) for every x. */
EXC_STEPCTL_FN double exc_ctl_pow_m1_5(double x) {
  if (x != x) return x;
  if (x > 1.79769313486231570815e+308) return 0.0;
  int e;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e = e - 1;
  }
  const int q = (e >= 0) ? e / 5 : -((-e + 4) / 5);
  const int r = e - 5 * q;
  const double c = r == 0 ? 1.0 : r == 1 ? 0.87055056329612413914 : r == 2 ? 0.75785828325519904117
                 : r == 3 ? 0.65975395538644712969 : 0.57434917749851750340; /* 2^(-r/5) */
  /* d ln 2 = (2^-54 / 5) ln 2 */
  return ldexp(c * exc_ctl_exp(-0.2 * exc_ctl_ln(m) - (double)e * 7.6954795931166199e-18), -q);
}

/* x^(-1/4) for x > 0: two correctly rounded square roots and a division */
EXC_STEPCTL_FN double exc_ctl_pow_m1_4(double x) { return 1.0 / sqrt(sqrt(x)); }

#endif /* EXC_STEPCTL_H */
