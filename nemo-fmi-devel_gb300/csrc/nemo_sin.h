/* nemo_sin.h -- sine and cosine in FP64, one evaluation shared by the CUDA kernels
 * and the test oracle (C), so that both give the same values. nemo_sin_0pi(x), x in
 * [0, pi]: the Langmuir-cell source of the TKE closure (zdftke.F90:300, SIN( rpi * pdepw / zhlc ) with
 * 0 <= pdepw < zhlc). Library sines differ between each other by an ulp (a CPU libm
 * against the GPU's), and the closure carries such a difference into en, the mixing
 * lengths and the coefficients within a few steps; one shared evaluation keeps the
 * FP64 device results equal to the oracle's.
 *
 * Method: x in (pi/2, pi] is reflected, sin(x) = sin(pi - x), with pi - x formed as
 * (PI_HI - x) + PI_LO, pi split into the double nearest it and the remainder (Cody and
 * Waite's additive reduction; PI_HI - x is exact for x in [pi/2, pi] by Sterbenz's
 * lemma). On [0, pi/2] the Taylor series r - r^3/3! + ... - r^23/23! is summed by
 * Horner's rule in r^2 (the first omitted term is below 6e-21 there). Every operation
 * is a separate IEEE double operation: compile without contraction (gcc
 * -ffp-contract=off, nvcc --fmad=false). Accurate to about one ulp; a test checks it
 * against the host's sin. */
#ifndef NEMO_SIN_H
#define NEMO_SIN_H

#if defined(__CUDACC__)
#define NEMO_SIN_FN __host__ __device__ __forceinline__
#else
#include <math.h>
#define NEMO_SIN_FN static inline
#endif

NEMO_SIN_FN double nemo_sin_0pi(double x) {
  const double pi_hi = 3.141592653589793116;     /* the double nearest pi */
  const double pi_lo = 1.2246467991473532e-16;   /* pi - pi_hi */
  const double r = x > 1.5707963267948966 ? (pi_hi - x) + pi_lo : x;
  const double r2 = r * r;
  /* (-1)^n / (2n + 1)!, n = 11 .. 1 */
  double s = -1.0 / 25852016738884976640000.0;
  s = s * r2 + 1.0 / 51090942171709440000.0;
  s = s * r2 - 1.0 / 121645100408832000.0;
  s = s * r2 + 1.0 / 355687428096000.0;
  s = s * r2 - 1.0 / 1307674368000.0;
  s = s * r2 + 1.0 / 6227020800.0;
  s = s * r2 - 1.0 / 39916800.0;
  s = s * r2 + 1.0 / 362880.0;
  s = s * r2 - 1.0 / 5040.0;
  s = s * r2 + 1.0 / 120.0;
  s = s * r2 - 1.0 / 6.0;
  return r + r * (r2 * s);
}

/* sin and cos for |x| < 2^20 pi / 2, shared in the same way by the device's GYRE
 * analytic forcing (usrdef_sbc.F90) and the oracle. Method: Cody and Waite's
 * additive reduction x = k pi/2 + r, k the nearest integer to x 2/pi, with pi/2
 * split into three parts of 32, 32 and 53 bits (k times each of the first two is
 * exact for |k| < 2^21), so |r| <= pi/4 to about 2^-100 x; then the Taylor series
 * of sin (to r^19 / 19!) or cos (to r^18 / 18!) on r by Horner's rule in r^2, and the
 * quadrant k mod 4. Separate IEEE operations, as above. */
#define NEMO_PIO2_1 1.5707963267341256      /* pi/2 truncated to 32 bits */
#define NEMO_PIO2_2 6.077100506303966e-11   /* the next 32 bits */
#define NEMO_PIO2_3 2.0222662487959506e-21  /* the rest, rounded */
#define NEMO_2_PI 0.6366197723675814        /* 2/pi */

NEMO_SIN_FN double nemo_sin_kernel(double r) {
  const double r2 = r * r;
  double s = -1.0 / 121645100408832000.0;
  s = s * r2 + 1.0 / 355687428096000.0;
  s = s * r2 - 1.0 / 1307674368000.0;
  s = s * r2 + 1.0 / 6227020800.0;
  s = s * r2 - 1.0 / 39916800.0;
  s = s * r2 + 1.0 / 362880.0;
  s = s * r2 - 1.0 / 5040.0;
  s = s * r2 + 1.0 / 120.0;
  s = s * r2 - 1.0 / 6.0;
  return r + r * (r2 * s);
}
NEMO_SIN_FN double nemo_cos_kernel(double r) {
  const double r2 = r * r;
  double c = 1.0 / 6402373705728000.0;
  c = c * r2 - 1.0 / 20922789888000.0;
  c = c * r2 + 1.0 / 87178291200.0;
  c = c * r2 - 1.0 / 479001600.0;
  c = c * r2 + 1.0 / 3628800.0;
  c = c * r2 - 1.0 / 40320.0;
  c = c * r2 + 1.0 / 720.0;
  c = c * r2 - 1.0 / 24.0;
  c = c * r2 + 0.5;
  return 1.0 - r2 * c;
}
/* the reduced argument of x and its quadrant k mod 4 */
NEMO_SIN_FN double nemo_reduce(double x, int *q) {
  const double k = rint(x * NEMO_2_PI);
  *q = (int)((long long)k & 3);
  return ((x - k * NEMO_PIO2_1) - k * NEMO_PIO2_2) - k * NEMO_PIO2_3;
}
NEMO_SIN_FN double nemo_sin(double x) {
  int q;
  const double r = nemo_reduce(x, &q);
  return q == 0 ? nemo_sin_kernel(r) : q == 1 ? nemo_cos_kernel(r) : q == 2 ? -nemo_sin_kernel(r) : -nemo_cos_kernel(r);
}
NEMO_SIN_FN double nemo_cos(double x) {
  int q;
  const double r = nemo_reduce(x, &q);
  return q == 0 ? nemo_cos_kernel(r) : q == 1 ? -nemo_sin_kernel(r) : q == 2 ? -nemo_cos_kernel(r) : nemo_sin_kernel(r);
}

#undef NEMO_SIN_FN
#endif
