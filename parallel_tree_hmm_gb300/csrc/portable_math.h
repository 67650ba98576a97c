/* Reproducible natural exp and log for float and double.
 *
 * MAP reconstruction and posterior sampling take logarithms of the model
 * factors and exponentials inside log-sum-exp; their results are discrete, so
 * a one-ulp difference in exp or log can change a state. These functions give
 * identical results on the GPU and on the host (x86-64 and aarch64) because
 * every rounding step is spelled out: fused multiply-adds are explicit, all
 * other operations use the round-to-nearest intrinsics on the device and are
 * compiled with -ffp-contract=off on the host.
 *
 * Methods (written from the mathematics, not from any vendor library):
 *   log: x = 2^e * m with m in [sqrt(1/2), sqrt(2)), f = m - 1 (exact),
 *        s = f / (2 + f), log(1 + f) = 2 atanh(s) = f - f^2/2 + s (f^2/2 + R),
 *        R = sum_k 2 s^(2k) / (2k + 1) (the odd Taylor series of atanh), and
 *        e ln 2 added with a Cody-Waite two-part ln 2.
 *   exp: n = round(x / ln 2), r = x - n ln 2 (Cody-Waite, |r| <= ln2/2),
 *        e^r by its Taylor series in Horner form, then scaled by 2^n built
 *        from exponent bits (two steps when 2^n is subnormal).
 * Truncation error is below 2^-30 (float) and 2^-56 (double) relative, so the
 * results are within about one ulp of the exact values.
 */
#ifndef THMM_PORTABLE_MATH_H_
#define THMM_PORTABLE_MATH_H_

#include <stdint.h>
#include <string.h>
#if !defined(__CUDACC__)
#include <math.h>
#endif

#if defined(__CUDACC__)
#define THMM_MATH_FN static __host__ __device__ __forceinline__
#else
#define THMM_MATH_FN static inline
#endif

#if defined(__CUDA_ARCH__)
#define THMM_FMAF(a, b, c) __fmaf_rn((a), (b), (c))
#define THMM_MULF(a, b) __fmul_rn((a), (b))
#define THMM_ADDF(a, b) __fadd_rn((a), (b))
#define THMM_SUBF(a, b) __fsub_rn((a), (b))
#define THMM_DIVF(a, b) __fdiv_rn((a), (b))
#define THMM_FMA(a, b, c) __fma_rn((a), (b), (c))
#define THMM_MUL(a, b) __dmul_rn((a), (b))
#define THMM_ADD(a, b) __dadd_rn((a), (b))
#define THMM_SUB(a, b) __dsub_rn((a), (b))
#define THMM_DIV(a, b) __ddiv_rn((a), (b))
#else
#define THMM_FMAF(a, b, c) fmaf((a), (b), (c))
#define THMM_MULF(a, b) ((a) * (b))
#define THMM_ADDF(a, b) ((a) + (b))
#define THMM_SUBF(a, b) ((a) - (b))
#define THMM_DIVF(a, b) ((a) / (b))
#define THMM_FMA(a, b, c) fma((a), (b), (c))
#define THMM_MUL(a, b) ((a) * (b))
#define THMM_ADD(a, b) ((a) + (b))
#define THMM_SUB(a, b) ((a) - (b))
#define THMM_DIV(a, b) ((a) / (b))
#endif

THMM_MATH_FN uint32_t thmm_f2u(float value) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(value);
#else
  uint32_t bits;
  memcpy(&bits, &value, sizeof bits);
  return bits;
#endif
}

THMM_MATH_FN float thmm_u2f(uint32_t bits) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(bits);
#else
  float value;
  memcpy(&value, &bits, sizeof value);
  return value;
#endif
}

THMM_MATH_FN uint64_t thmm_d2u(double value) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(value);
#else
  uint64_t bits;
  memcpy(&bits, &value, sizeof bits);
  return bits;
#endif
}

THMM_MATH_FN double thmm_u2d(uint64_t bits) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)bits);
#else
  double value;
  memcpy(&value, &bits, sizeof value);
  return value;
#endif
}

/* ln 2 split so that n * kLn2HiF is exact for |n| < 2^9. */
#define THMM_LN2_HI_F 0.693145751953125f
#define THMM_LN2_LO_F 1.42860677e-06f
#define THMM_LOG2E_F 1.44269504f
/* ln 2 split so that n * kLn2Hi is exact for |n| < 2^11. */
#define THMM_LN2_HI 0.6931471803691238164901733398437500
#define THMM_LN2_LO 1.9082149292705877000220372080672226e-10
#define THMM_LOG2E 1.4426950408889634073599246810018921

THMM_MATH_FN float thmm_logf(float x) {
  const uint32_t bits = thmm_f2u(x);
  if (x != x)
    return x;
  if (x < 0.0f)
    return thmm_u2f(0x7fc00000u);
  if (x == 0.0f)
    return thmm_u2f(0xff800000u);
  if (bits == 0x7f800000u)
    return x;
  int exponent_bias = 0;
  uint32_t b = bits;
  if (b < 0x00800000u) { /* subnormal: scale by 2^25 exactly */
    b = thmm_f2u(THMM_MULF(x, 33554432.0f));
    exponent_bias = -25;
  }
  int e = (int)((b >> 23) & 0xffu) - 127 + exponent_bias;
  uint32_t mantissa = b & 0x007fffffu;
  /* m in [1, 2); fold m > sqrt(2) into [sqrt(1/2), 1). */
  if (mantissa > 0x003504f3u) {
    mantissa |= 0x3f000000u; /* m / 2 */
    e += 1;
  } else {
    mantissa |= 0x3f800000u;
  }
  const float m = thmm_u2f(mantissa);
  const float f = THMM_SUBF(m, 1.0f);
  const float s = THMM_DIVF(f, THMM_ADDF(2.0f, f));
  const float z = THMM_MULF(s, s);
  /* R = z (2/3 + z (2/5 + z (2/7 + z 2/9))) */
  float r = THMM_FMAF(z, 0.222222222f, 0.285714286f);
  r = THMM_FMAF(z, r, 0.4f);
  r = THMM_FMAF(z, r, 0.666666667f);
  r = THMM_MULF(z, r);
  const float half_f2 = THMM_MULF(THMM_MULF(0.5f, f), f);
  const float ef = (float)e;
  /* log = e ln2_hi + (f - (half_f2 - (s (half_f2 + R) + e ln2_lo))) */
  const float tail = THMM_FMAF(s, THMM_ADDF(half_f2, r), THMM_MULF(ef, THMM_LN2_LO_F));
  const float body = THMM_SUBF(f, THMM_SUBF(half_f2, tail));
  return THMM_FMAF(ef, THMM_LN2_HI_F, body);
}

THMM_MATH_FN float thmm_expf(float x) {
  if (x != x)
    return x;
  if (x > 88.7228394f)
    return thmm_u2f(0x7f800000u);
  if (x < -103.972084f)
    return 0.0f;
  /* n = nearest integer to x / ln 2 (ties away from zero). */
  const float t = THMM_MULF(x, THMM_LOG2E_F);
  const int n = (int)(t < 0.0f ? THMM_SUBF(t, 0.5f) : THMM_ADDF(t, 0.5f));
  const float nf = (float)n;
  float r = THMM_FMAF(-nf, THMM_LN2_HI_F, x);
  r = THMM_FMAF(-nf, THMM_LN2_LO_F, r);
  /* e^r = 1 + r + r^2/2! + ... + r^7/7! */
  float p = THMM_FMAF(r, 1.98412698e-04f, 1.38888889e-03f);
  p = THMM_FMAF(r, p, 8.33333333e-03f);
  p = THMM_FMAF(r, p, 4.16666667e-02f);
  p = THMM_FMAF(r, p, 1.66666667e-01f);
  p = THMM_FMAF(r, p, 0.5f);
  p = THMM_MULF(THMM_MULF(r, r), p);
  p = THMM_ADDF(1.0f, THMM_ADDF(r, p));
  if (n >= -126 && n <= 127)
    return THMM_MULF(p, thmm_u2f((uint32_t)(n + 127) << 23));
  if (n > 127) /* p < 2^0.5, so 2^127 * p * 2^(n-127) */
    return THMM_MULF(THMM_MULF(p, thmm_u2f(0x7f000000u)),
                     thmm_u2f((uint32_t)(n - 127 + 127) << 23));
  /* n < -126: scale by 2^(n + 64) then by 2^-64. */
  return THMM_MULF(THMM_MULF(p, thmm_u2f((uint32_t)(n + 64 + 127) << 23)),
                   thmm_u2f((uint32_t)(-64 + 127) << 23));
}

THMM_MATH_FN double thmm_log(double x) {
  const uint64_t bits = thmm_d2u(x);
  if (x != x)
    return x;
  if (x < 0.0)
    return thmm_u2d(0x7ff8000000000000ull);
  if (x == 0.0)
    return thmm_u2d(0xfff0000000000000ull);
  if (bits == 0x7ff0000000000000ull)
    return x;
  int exponent_bias = 0;
  uint64_t b = bits;
  if (b < 0x0010000000000000ull) { /* subnormal: scale by 2^54 exactly */
    b = thmm_d2u(THMM_MUL(x, 18014398509481984.0));
    exponent_bias = -54;
  }
  int e = (int)((b >> 52) & 0x7ffu) - 1023 + exponent_bias;
  uint64_t mantissa = b & 0x000fffffffffffffull;
  if (mantissa > 0x0006a09e667f3bcdull) {
    mantissa |= 0x3fe0000000000000ull;
    e += 1;
  } else {
    mantissa |= 0x3ff0000000000000ull;
  }
  const double m = thmm_u2d(mantissa);
  const double f = THMM_SUB(m, 1.0);
  const double s = THMM_DIV(f, THMM_ADD(2.0, f));
  const double z = THMM_MUL(s, s);
  /* R = sum_{k=1..10} 2 z^k / (2k + 1) */
  double r = THMM_FMA(z, 2.0 / 21.0, 2.0 / 19.0);
  r = THMM_FMA(z, r, 2.0 / 17.0);
  r = THMM_FMA(z, r, 2.0 / 15.0);
  r = THMM_FMA(z, r, 2.0 / 13.0);
  r = THMM_FMA(z, r, 2.0 / 11.0);
  r = THMM_FMA(z, r, 2.0 / 9.0);
  r = THMM_FMA(z, r, 2.0 / 7.0);
  r = THMM_FMA(z, r, 2.0 / 5.0);
  r = THMM_FMA(z, r, 2.0 / 3.0);
  r = THMM_MUL(z, r);
  const double half_f2 = THMM_MUL(THMM_MUL(0.5, f), f);
  const double ed = (double)e;
  const double tail = THMM_FMA(s, THMM_ADD(half_f2, r), THMM_MUL(ed, THMM_LN2_LO));
  const double body = THMM_SUB(f, THMM_SUB(half_f2, tail));
  return THMM_FMA(ed, THMM_LN2_HI, body);
}

THMM_MATH_FN double thmm_exp(double x) {
  if (x != x)
    return x;
  if (x > 709.782712893383973)
    return thmm_u2d(0x7ff0000000000000ull);
  if (x < -745.133219101941108)
    return 0.0;
  const double t = THMM_MUL(x, THMM_LOG2E);
  const int n = (int)(t < 0.0 ? THMM_SUB(t, 0.5) : THMM_ADD(t, 0.5));
  const double nd = (double)n;
  double r = THMM_FMA(-nd, THMM_LN2_HI, x);
  r = THMM_FMA(-nd, THMM_LN2_LO, r);
  /* e^r = 1 + r + sum_{k=2..13} r^k / k! */
  double p = THMM_FMA(r, 1.0 / 6227020800.0, 1.0 / 479001600.0);
  p = THMM_FMA(r, p, 1.0 / 39916800.0);
  p = THMM_FMA(r, p, 1.0 / 3628800.0);
  p = THMM_FMA(r, p, 1.0 / 362880.0);
  p = THMM_FMA(r, p, 1.0 / 40320.0);
  p = THMM_FMA(r, p, 1.0 / 5040.0);
  p = THMM_FMA(r, p, 1.0 / 720.0);
  p = THMM_FMA(r, p, 1.0 / 120.0);
  p = THMM_FMA(r, p, 1.0 / 24.0);
  p = THMM_FMA(r, p, 1.0 / 6.0);
  p = THMM_FMA(r, p, 0.5);
  p = THMM_MUL(THMM_MUL(r, r), p);
  p = THMM_ADD(1.0, THMM_ADD(r, p));
  if (n >= -1022 && n <= 1023)
    return THMM_MUL(p, thmm_u2d((uint64_t)(n + 1023) << 52));
  if (n > 1023)
    return THMM_MUL(THMM_MUL(p, thmm_u2d(0x7fe0000000000000ull)),
                    thmm_u2d((uint64_t)(n - 1023 + 1023) << 52));
  return THMM_MUL(THMM_MUL(p, thmm_u2d((uint64_t)(n + 256 + 1023) << 52)),
                  thmm_u2d((uint64_t)(-256 + 1023) << 52));
}

#endif /* THMM_PORTABLE_MATH_H_ */
