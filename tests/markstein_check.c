/* Check of the integration update's divisions: a / b computed as
 *   q = RN(a y),  q' = RN(q + RN_exact(a - b q) y),  y = RN(1 / b)
 * (Markstein's correction with fused multiply-adds) equals the IEEE
 * quotient RN(a / b).
 *   mode 0 (truncation T): for 12 divisors b in [0.007, 3], every float a
 *           with |a| in [2^-30, 64] (both signs), every `step`-th one;
 *   mode 1 (weights): every whole b in [1, 4096], `samples` seeded random
 *           floats a with |a| in [2^-40, 8192] per b;
 *   mode 2 (camera depth): `samples` seeded random pairs, b in [2^-10, 2^8]
 *           and |a| in [2^-30, 2^8] (the projection's x / z and y / z).
 * y is formed as the engine's host code forms RN(1/T): the double quotient
 * rounded once, then checked against its float neighbours.
 * Usage: markstein_check <mode> <step|samples>.  Prints the number of checks
 * and mismatches; exits 1 on a mismatch. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static float f_of(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t u_of(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static float rn_reciprocal(float b) {
  const double ex = 1.0 / (double)b;
  float y = (float)ex;
  const float up = nextafterf(y, INFINITY), down = nextafterf(y, -INFINITY);
  if (fabs((double)up - ex) < fabs((double)y - ex)) y = up;
  if (fabs((double)down - ex) < fabs((double)y - ex)) y = down;
  return y;
}

static long long checks = 0, bad = 0;

static void check(float a, float b, float y) {
  volatile float q0 = a * y;
  const float q = fmaf(fmaf(-b, q0, a), y, q0);
  volatile float ref = a / b;
  ++checks;
  if (u_of(q) != u_of(ref)) {
    if (bad < 5) printf("b=%a a=%a q=%a ref=%a\n", b, a, q, ref);
    ++bad;
  }
}

int main(int argc, char **argv) {
  const int mode = argc > 1 ? atoi(argv[1]) : 0;
  const long long arg = argc > 2 ? atoll(argv[2]) : 1;
  if (mode == 0) {
    const float bs[] = {0.02f, 0.016f, 0.04f, 0.08f, 0.1f, 0.03f,
                        0.0123456f, 0.18f, 0.05f, 0.0667f, 3.0f, 0.007f};
    const uint32_t lo = u_of(9.3132257e-10f), hi = u_of(64.0f);
    for (int k = 0; k < 12; ++k) {
      const float b = bs[k], y = rn_reciprocal(b);
      for (uint32_t u = lo; u <= hi; u += (uint32_t)arg) {
        check(f_of(u), b, y);
        check(f_of(u | 0x80000000u), b, y);
      }
    }
  } else if (mode == 2) {
    uint64_t s = 0x9E3779B97F4A7C15ull;
    const uint32_t blo = u_of(0x1p-10f), bhi = u_of(0x1p8f);
    const uint32_t alo = u_of(0x1p-30f), ahi = u_of(0x1p8f);
    for (long long i = 0; i < arg; ++i) {
      s ^= s << 13; s ^= s >> 7; s ^= s << 17;
      const float b = f_of(blo + (uint32_t)(s % (bhi - blo)));
      const float y = rn_reciprocal(b);
      const uint64_t t = s * 0x2545F4914F6CDD1Dull;
      const float a = f_of((alo + (uint32_t)((t >> 8) % (ahi - alo))) | ((t & 1) ? 0x80000000u : 0));
      check(a, b, y);
    }
  } else {
    uint64_t s = 88172645463325252ull;
    const uint32_t lo = u_of(9.094947e-13f), hi = u_of(8192.0f);
    for (int w = 1; w <= 4096; ++w) {
      const float b = (float)w, y = rn_reciprocal(b);
      for (long long i = 0; i < arg; ++i) {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        const float a = f_of((uint32_t)(lo + s % (hi - lo)) | (((s >> 40) & 1) ? 0x80000000u : 0));
        check(a, b, y);
      }
    }
  }
  printf("checks %lld mismatches %lld\n", checks, bad);
  return bad != 0;
}
