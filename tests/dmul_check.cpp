// Host check of tl_dmul (exploringsycl_gb300/csrc/tl_dmul.cuh) against the
// host's IEEE multiplication: random operands over the exponent range, short
// significands whose products land exactly on rounding ties, and operands at
// the edges of the normal range. Prints the number of cases and mismatches.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "tl_dmul.cuh"

static uint64_t state;
static uint64_t next64() {
  state += 0x9E3779B97F4A7C15ull;
  uint64_t z = state;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static long cases = 0, bad = 0, fast = 0;

static void check(double a, double b) {
  const double want = a * b;
  const double got = tl_dmul(a, b);
  ++cases;
  const uint64_t ea = (tl_dbits(a) >> 52) & 0x7FF, eb = (tl_dbits(b) >> 52) & 0x7FF;
  const int e = (int)ea + (int)eb - 1023;
  if (ea >= 1 && ea <= 2046 && eb >= 1 && eb <= 2046 && e >= 1 && e <= 2045) ++fast;
  if (tl_dbits(want) != tl_dbits(got) && !(isnan(want) && isnan(got))) {
    if (++bad <= 10)
      fprintf(stderr, "mismatch: %a * %a = %a, got %a\n", a, b, want, got);
  }
}

static double make(uint64_t sign, uint64_t exp, uint64_t mant) {
  return tl_bitsd((sign << 63) | ((exp & 0x7FF) << 52) | (mant & 0xFFFFFFFFFFFFFull));
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  state = argc > 2 ? strtoull(argv[2], 0, 10) : 1;
  for (long i = 0; i < n; ++i) {
    const uint64_t r1 = next64(), r2 = next64(), r3 = next64();
    /* 1: uniformly random bit patterns (all classes) */
    check(tl_bitsd(r1), tl_bitsd(r2));
    /* 2: normal operands with exponents near 1023 and random significands */
    check(make(r1 & 1, 900 + (r1 >> 1) % 250, r2), make(r3 & 1, 900 + (r3 >> 1) % 250, r3 >> 7));
    /* 3: short significands (few low bits above the leading ones): frequent ties */
    const int k1 = (int)(r1 % 53), k2 = (int)(r2 % 53);
    const uint64_t m1 = (r2 >> 11) & ((1ull << (r1 % 12)) - 1), m2 = (r3 >> 11) & ((1ull << (r2 % 12)) - 1);
    check(make(0, 1023, m1 << (52 - (k1 < 12 ? 12 : k1))), make(r3 & 1, 1023 + (int)(r3 % 7) - 3,
                                                                  m2 << (52 - (k2 < 12 ? 12 : k2))));
    check(make(0, 1000, (r1 & 0xFFF) << 40 | 1), make(0, 1040, (r2 & 0xFFF) << 40 | 1ull << 39));
    /* 4: exponents at the edges of the normal range (fast path and fall-back) */
    check(make(r1 & 1, 1 + r2 % 40, r3), make(0, 1000 + r1 % 60, r2));
    check(make(0, 2046 - r2 % 40, r3), make(r1 & 1, 1000 + r3 % 60, r1));
    check(make(0, 2046, ~0ull), make(0, 1023, r3));
  }
  printf("cases %ld fast %ld mismatches %ld\n", cases, fast, bad);
  return bad == 0 ? 0 : 1;
}
