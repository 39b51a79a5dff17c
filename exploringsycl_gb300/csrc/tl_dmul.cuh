/*
 * tl_dmul.cuh -- IEEE-754 binary64 multiplication, rounded to nearest even,
 * computed on 32-bit integer operations.
 *
 * GB300 issues FP64 instructions at 2 per clock per SM, 1/64 of its 32-bit
 * integer and FP32 rate, and the exact FP64 CG step spends 19 FP64
 * instructions per cell. Moving multiplications to the integer pipes lets
 * both kinds of pipe work at once while every result stays the correctly
 * rounded IEEE product, bit for bit (the exact contract's parity with the
 * CPU oracle is unchanged).
 *
 * Method (schoolbook multiplication of the 53-bit significands in 32-bit
 * limbs). With a = (sa, ea, ma), b = (sb, eb, mb), ma and mb in [2^52, 2^53)
 * including the hidden bit, split ma = a1 2^32 + a0 (a1 < 2^21):
 *   t = a0 b0,  v = a0 b1 + a1 b0 + hi32(t),  w = a1 b1 + hi32(v)
 *   P = ma mb = w 2^64 + lo32(v) 2^32 + lo32(t),  P in [2^104, 2^106).
 * With n = 1 if P >= 2^105 (bit 41 of w), the significand is
 * m = floor(P / 2^(52+n)), the round bit is bit 51+n of P and the sticky bit
 * the OR of the bits below it; round to nearest, ties to even. The result is
 * packed as sign | ((E - 1) << 52) + m with E = ea + eb - 1023 + n, so that a
 * rounding carry out of the significand (m = 2^53) moves into the exponent,
 * and E - 1 = 2046 with a carry gives the infinity that IEEE rounding gives.
 * Operands that are zero, subnormal, infinite or NaN, and products whose
 * exponent would leave the normal range, take the hardware multiplication
 * instead: the fast path covers exactly the cases it computes correctly.
 *
 * The same source compiles for the host (tests/test_dmul.py checks it against
 * the host's multiplication on random and tie-producing operands).
 */
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define TL_HD __host__ __device__ __forceinline__
#else
#define TL_HD static inline
#endif

TL_HD uint64_t tl_dbits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

TL_HD double tl_bitsd(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

/* (hi:lo) << s, high word (0 <= s < 32): the funnel shift of the GPU. */
TL_HD uint32_t tl_shf_l(uint32_t lo, uint32_t hi, uint32_t s) {
#if defined(__CUDA_ARCH__)
  return __funnelshift_l(lo, hi, s);
#else
  return (uint32_t)(((((uint64_t)hi << 32) | lo) << s) >> 32);
#endif
}

/* The integer-pipe product of a and b. Operands or results outside the
 * fast path take the hardware multiplication of the same operands. */
TL_HD double tl_dmul_int_or(double a, double b, double hw_product_fallback_a,
                            double hw_product_fallback_b) {
  const uint64_t ua = tl_dbits(a), ub = tl_dbits(b);
  const uint32_t ha = (uint32_t)(ua >> 32), hb = (uint32_t)(ub >> 32);
  const uint32_t a0 = (uint32_t)ua, b0 = (uint32_t)ub;
  const uint32_t ea = (ha >> 20) & 0x7FFu, eb = (hb >> 20) & 0x7FFu;
  const uint32_t e = ea + eb - 1023u;  /* biased exponent before normalisation */
  if (ea - 1u >= 2046u || eb - 1u >= 2046u || e - 1u >= 2045u) {
    return hw_product_fallback_a * hw_product_fallback_b;
  }
  const uint32_t a1 = (ha & 0xFFFFFu) | 0x100000u;
  const uint32_t b1 = (hb & 0xFFFFFu) | 0x100000u;
  /* P = w 2^64 + vlo 2^32 + tlo */
  const uint64_t t = (uint64_t)a0 * b0;
  uint64_t v = (uint64_t)a0 * b1 + (t >> 32);
  v += (uint64_t)a1 * b0;
  const uint64_t w = (uint64_t)a1 * b1 + (v >> 32);
  const uint32_t wh = (uint32_t)(w >> 32), wl = (uint32_t)w;
  const uint32_t vlo = (uint32_t)v, tlo = (uint32_t)t;
  /* n = 1 if P >= 2^105; the significand is P >> (52 + n) = (w:vlo) >> (20 + n),
   * i.e. the two words of (wh:wl:vlo) << s taken above vlo, s = 12 - n */
  const uint32_t n = (wh >> 9) & 1u;
  const uint32_t sh = 12u - n;
  const uint32_t mh = tl_shf_l(wl, wh, sh);
  const uint32_t ml = tl_shf_l(vlo, wl, sh);
  const uint32_t below = vlo << sh;                 /* the bits under the significand */
  const uint32_t round = below >> 31;
  const uint32_t sticky = ((below << 1) | tlo) != 0u;
  const uint32_t inc = round & (sticky | (ml & 1u));
  /* add the rounding increment and the exponent field (E - 1) << 20 to the
   * significand's high word (its hidden bit adds the last 1) */
  const uint64_t lo_sum = (uint64_t)ml + inc;
  const uint32_t hi = mh + (uint32_t)(lo_sum >> 32) + ((e + n - 1u) << 20);
  return tl_bitsd(((uint64_t)(hi | ((ha ^ hb) & 0x80000000u)) << 32) | (uint32_t)lo_sum);
}

/* a * b, correctly rounded, on the integer pipes where possible. */
TL_HD double tl_dmul(double a, double b) { return tl_dmul_int_or(a, b, a, b); }
