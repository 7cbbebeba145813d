/* nemo_sin.h -- sin(x) on [0, pi] in FP64, one evaluation shared by the CUDA kernels
 * and the test oracle (C), so that both give the same value for the Langmuir-cell
 * source of the TKE closure (zdftke.F90:300, SIN( rpi * pdepw / zhlc ) with
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

#undef NEMO_SIN_FN
#endif
