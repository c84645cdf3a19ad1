// Host check of the integer-arithmetic multiply, add, divide and square root
// of gfm_xfp64.cuh against the host's own IEEE double operations (round to
// nearest even), bit for bit, over: special values; random bit patterns;
// random normal operands over the whole exponent range and near its ends;
// products of short integer significands (exact products and exact ties);
// sums of operands 0..60 binades apart, near-cancellations, ties built from
// half-ulp offsets; every leading 24-bit pattern of a divisor and of a root's
// argument; near squares and near-exact quotients.  Prints "ok <count>" or
// the first mismatch.
// Built and run by tests/test_xfp64.py: xfp64_check [cases per category].
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>
#include "../phd-2d-gfm_gb300/csrc/gfm_xfp64.cuh"

using namespace gfm;

static double dbl(uint64_t b) { double x; std::memcpy(&x, &b, 8); return x; }
static uint64_t bits(double x) { uint64_t b; std::memcpy(&b, &x, 8); return b; }

static uint64_t st = 0x9e3779b97f4a7c15ULL;
static uint64_t rnd() {   // xorshift64*
  st ^= st >> 12; st ^= st << 25; st ^= st >> 27;
  return st * 0x2545f4914f6cdd1dULL;
}
// a normal double with a random significand, a random sign and the biased exponent e
static double normal_with_exp(uint32_t e) {
  return dbl((rnd() & 0x800fffffffffffffULL) | ((uint64_t)e << 52));
}

static long n_checked = 0;
static bool same(double r, double want) {
  if (std::isnan(want)) return std::isnan(r);
  return bits(r) == bits(want);
}
static int check(double a, double b) {
  n_checked++;
  volatile double va = a, vb = b;
  const double pm = va * vb, ps = va + vb, pd = va - vb;
  const double xm = xmul(a, b), xs = xadd(a, b), xd = xadd(a, -b);
  if (!same(xm, pm)) { printf("mul %a * %a = %a, integer path %a\n", a, b, pm, xm); return 1; }
  if (!same(xs, ps)) { printf("add %a + %a = %a, integer path %a\n", a, b, ps, xs); return 1; }
  if (!same(xd, pd)) { printf("sub %a - %a = %a, integer path %a\n", a, b, pd, xd); return 1; }
  const double pq = va / vb, xq = xdiv(a, b);
  if (!same(xq, pq)) { printf("div %a / %a = %a, integer path %a\n", a, b, pq, xq); return 1; }
  volatile double aa = std::fabs(a);
  const double pr = std::sqrt(aa), xr = xsqrt(aa), pn = std::sqrt(va), xn = xsqrt(a);
  if (!same(xr, pr)) { printf("sqrt %a = %a, integer path %a\n", (double)aa, pr, xr); return 1; }
  if (!same(xn, pn)) { printf("sqrt %a = %a, integer path %a\n", a, pn, xn); return 1; }
  return 0;
}

int main(int argc, char** argv) {
  const long N = argc > 1 ? atol(argv[1]) : 2000000;
  std::vector<double> sp = {0.0, -0.0, 1.0, -1.0, 0.5, 3.0, 1e-310, -1e-310, 5e-324, -5e-324,
                            2.2250738585072014e-308, -2.2250738585072014e-308, 1.7976931348623157e308,
                            -1.7976931348623157e308, INFINITY, -INFINITY, NAN, dbl(0x7ff0000000000001ULL),
                            dbl(0x3ff0000000000001ULL), dbl(0x3fefffffffffffffULL), 1e-300, 1e300, 1e154, 1e-154,
                            dbl(0x0010000000000001ULL), dbl(0x7fefffffffffffffULL), dbl(0x7fe0000000000000ULL)};
  for (double a : sp)
    for (double b : sp)
      if (check(a, b)) return 1;
  for (long k = 0; k < N; k++) {
    // random bit patterns (every class)
    if (check(dbl(rnd()), dbl(rnd()))) return 1;
    // random normals over the whole range, and with exponents near the ends
    const uint32_t e1 = 1 + (uint32_t)(rnd() % 2046), e2 = 1 + (uint32_t)(rnd() % 2046);
    if (check(normal_with_exp(e1), normal_with_exp(e2))) return 1;
    const uint32_t lo = 1 + (uint32_t)(rnd() % 60), hi = 2046 - (uint32_t)(rnd() % 60);
    if (check(normal_with_exp(lo), normal_with_exp(hi))) return 1;
    if (check(normal_with_exp(hi), normal_with_exp(1023 + (uint32_t)(rnd() % 8)))) return 1;
    if (check(normal_with_exp(lo), normal_with_exp(1023 - (uint32_t)(rnd() % 8)))) return 1;
    if (check(normal_with_exp(lo + 1000), normal_with_exp(1046 - (uint32_t)(rnd() % 60)))) return 1;
    // short integer significands: exact products and ties of the product
    const double p = (double)(rnd() >> (37 + rnd() % 10)) , q = (double)(rnd() >> (37 + rnd() % 10));
    const int s1 = (int)(rnd() % 200) - 100, s2 = (int)(rnd() % 200) - 100;
    if (check(std::ldexp(p, s1), std::ldexp(q, s2))) return 1;
    // sums of operands d binades apart, d = 0..60
    const uint32_t e3 = 70 + (uint32_t)(rnd() % 1900);
    const uint32_t d = (uint32_t)(rnd() % 61);
    if (check(normal_with_exp(e3), normal_with_exp(e3 - d))) return 1;
    // near-cancellation: b = -a perturbed in its last bits
    const double a = normal_with_exp(e3);
    const double b = dbl(bits(a) ^ (rnd() & 0xffULL));
    if (check(a, -b)) return 1;
    if (check(a, -dbl(bits(a) + 1 + (rnd() & 1)))) return 1;
    // ties of the sum: a plus half an ulp of a (times an odd multiple of a
    // power of two below it)
    const double ulp_half = std::ldexp(1.0, (int)((bits(a) >> 52) & 0x7ff) - 1023 - 53);
    if (check(a, ulp_half)) return 1;
    if (check(a, -ulp_half)) return 1;
    if (check(a, ulp_half * (double)(1 + 2 * (rnd() % 7)))) return 1;
    if (check(a, std::ldexp(ulp_half, -(int)(rnd() % 4)))) return 1;
  }
  // every leading 24-bit pattern of the divisor's and the root's significand
  // (the seeds depend on these bits only), with random low bits, random
  // exponents' parity and a random dividend
  for (uint64_t top = 0; top < (1ull << 24); top += (N >= 2000000 ? 1 : 61)) {
    const uint64_t frac = ((top & 0xffffffull) << 28) | (rnd() & 0xfffffffull);
    const double b = dbl(((uint64_t)(1023 + (rnd() & 1)) << 52) | (frac & 0xfffffffffffffull));
    const double a = normal_with_exp(1000 + (uint32_t)(rnd() % 40));
    if (check(a, b)) return 1;
    if (check(b, b)) return 1;
    if (check(dbl(bits(b) & ~0xfffffffull), dbl((bits(b) & ~0xfffffffull) | 1))) return 1;
  }
  // near squares and near-exact quotients: squares of random 26-bit
  // integers, their neighbours, products of short significands
  for (long k = 0; k < N / 4; k++) {
    const double r = (double)(rnd() >> 38) + 1.0;
    const double sq = r * r;
    if (check(std::ldexp(sq, (int)(rnd() % 100) - 50), 3.0)) return 1;
    if (check(dbl(bits(sq) + 1), dbl(bits(sq) - 1))) return 1;
    const double p = (double)(rnd() >> 40) + 1.0, q = (double)(rnd() >> 40) + 1.0;
    if (check(p * q, q)) return 1;
    if (check(dbl(bits(p * q) + 1), q)) return 1;
    if (check(dbl(bits(p * q) - 1), p)) return 1;
  }
  printf("ok %ld\n", n_checked);
  return 0;
}
