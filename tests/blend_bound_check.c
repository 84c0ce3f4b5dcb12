/* Exhaustive check of the integer colour average of k_integrate for weights
 * w = w_old + 1 in [2, 2048]: floor(n / w) = umulhi(n, m) for every
 * numerator n = c_old * w_old + c_new in [0, 255 w], where
 * m = trunc(r * (2^32 + 2^11)) + 1 and r is a reciprocal of w within 2^-22
 * relative (2 ulp; the kernel's is correctly rounded, within 2^-24) and the
 * float product is rounded to
 * nearest (2^-24 relative).  floor(n * m / 2^32) is monotone in m, so the
 * smallest and the largest m those roundings allow cover every case.
 * Prints the number of checks and failures; exits 1 on a failure. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>

int main(void) {
  long long checks = 0, bad = 0;
  const long double bias = 1.0L + ldexpl(1.0L, -21);
  for (uint32_t w = 2; w <= 2048; ++w) {
    const long double exact = ldexpl(1.0L, 32) / w;
    const long double lo = exact * (1.0L - ldexpl(1.0L, -22)) * bias * (1.0L - ldexpl(1.0L, -24));
    const long double hi = exact * (1.0L + ldexpl(1.0L, -22)) * bias * (1.0L + ldexpl(1.0L, -24));
    const uint64_t ms[2] = {(uint64_t)floorl(lo) + 1, (uint64_t)floorl(hi) + 1};
    for (int k = 0; k < 2; ++k) {
      if (ms[k] > 0xFFFFFFFFull) {
        printf("m does not fit 32 bits at w=%u\n", w);
        return 1;
      }
      for (uint32_t n = 0; n <= 255u * w; ++n) {
        ++checks;
        if ((uint32_t)(((uint64_t)n * ms[k]) >> 32) != n / w) ++bad;
      }
    }
  }
  printf("checks %lld failures %lld\n", checks, bad);
  return bad != 0;
}
