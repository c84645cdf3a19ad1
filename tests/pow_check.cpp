// Host check of the fixed-point gfm_pow (phd-2d-gfm_gb300/csrc/gfm_math.cuh)
// against the oracle's independent restatement (oracle/oracle_math.hpp), bit
// for bit, over bases across the whole positive range, near 1 and at the
// pressure ratios of the Riemann solver, with exponents of either sign.
// Usage: pow_check N [dump]; with "dump" every case is printed as
// "x y pow(x, y)" in hexadecimal for an accuracy check against mpmath.
// Prints "ok <count>" (to stderr when dumping) or the first mismatches.
// Built and run by tests/test_xfp64.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cstdint>
#include "../phd-2d-gfm_gb300/csrc/gfm_math.cuh"
#include "../oracle/oracle_math.hpp"

static uint64_t st = 88172645463325252ULL;
static uint64_t rnd() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static double u01() { return (double)(rnd() >> 11) / 9007199254740992.0; }
static double with_exp(uint64_t frac, int e) {
  const uint64_t b = (frac & 0x000fffffffffffffULL) | ((uint64_t)e << 52);
  double x; std::memcpy(&x, &b, 8); return x;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  const bool dump = argc > 2;
  long bad = 0;
  for (long i = 0; i < n; i++) {
    double x, y;
    switch (i % 6) {
      case 0: x = with_exp(rnd(), 1023 - 15 + (int)(rnd() % 31)); y = (u01() - 0.5) * 16; break;
      case 1: x = 1.0 + (u01() - 0.5) * 1e-3; y = (u01() - 0.5) * 20; break;
      case 2: { const uint64_t r = rnd() & 0x7fffffffffffffffULL; std::memcpy(&x, &r, 8); y = (u01() - 0.5) * 4; break; }
      case 3: x = with_exp(rnd(), 1 + (int)(rnd() % 2046)); y = u01() * 2 - 1; break;
      case 4: x = u01() * 100; y = 1.0 / (1.09 + u01() * 5); break;
      default: x = 0.5 + u01(); y = (u01() - 0.5) * 1e-10; break;
    }
    const double a = gfm::gfm_pow(x, y), b = omath::pow(x, y);
    if (std::memcmp(&a, &b, 8) != 0 && !(a != a && b != b)) {
      if (bad < 5) printf("pow(%a, %a): library %a oracle %a\n", x, y, a, b);
      bad++;
    }
    if (dump) printf("%a %a %a\n", x, y, a);
  }
  const double inf = HUGE_VAL, nan = std::nan("");
  const double xs[] = {0.0, -0.0, 1.0, inf, nan, -2.0, 5e-324}, ys[] = {0.0, -0.0, 2.5, -2.5, inf, -inf, nan};
  for (double x : xs)
    for (double y : ys) {
      const double a = gfm::gfm_pow(x, y), b = omath::pow(x, y);
      if (std::memcmp(&a, &b, 8) != 0 && !(a != a && b != b)) {
        printf("pow(%a, %a): library %a oracle %a\n", x, y, a, b);
        bad++;
      }
    }
  if (bad) { printf("mismatches %ld\n", bad); return 1; }
  fprintf(dump ? stderr : stdout, "ok %ld\n", n);
  return 0;
}
