// Host check of the integer-pipe IEEE comparisons of gfm_math.cuh against the
// C comparisons, over special values (signed zeros, infinities, NaNs,
// subnormals, extremes) and random bit patterns.  Prints "ok <count>" or the
// first mismatch.  Built and run by tests/test_compare_bits.py.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include "../phd-2d-gfm_gb300/csrc/gfm_math.cuh"

using namespace gfm;

static double dbl(uint64_t b) { double x; std::memcpy(&x, &b, 8); return x; }

int main() {
  std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 1e-310, -1e-310, 5e-324, -5e-324,
                           2.2250738585072014e-308, -2.2250738585072014e-308, 1.7976931348623157e308,
                           -1.7976931348623157e308, INFINITY, -INFINITY, NAN, -NAN, dbl(0x7ff0000000000001ULL),
                           dbl(0xfff0000000000001ULL), dbl(0x7fffffffffffffffULL), 1e-300, 1e300, -1e300, 3.0,
                           dbl(0x3ff0000000000001ULL), dbl(0x3fefffffffffffffULL), 1e-6, -1e-6};
  uint64_t s = 0x9e3779b97f4a7c15ULL;
  for (int k = 0; k < 4000; k++) {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    v.push_back(dbl(s));
    if (k % 4 == 0) v.push_back(dbl(s & 0x800fffffffffffffULL));   // subnormals
    if (k % 4 == 1) v.push_back(std::ldexp((double)(s >> 11) / 9007199254740992.0, (int)(s % 60) - 30));
  }
  long n = 0;
  for (double a : v) {
    if (i_gt0(a) != (a > 0.0) || i_ge0(a) != (a >= 0.0) || i_lt0(a) != (a < 0.0) || i_le0(a) != (a <= 0.0)) {
      std::printf("mismatch zero-compare %a\n", a); return 1;
    }
    for (size_t q = 0; q < v.size(); q += 7) {
      double b = v[q];
      if (i_lt(a, b) != (a < b) || i_le(a, b) != (a <= b) || i_eq(a, b) != (a == b)) {
        std::printf("mismatch compare %a %a\n", a, b); return 1;
      }
      if (i_quotient_ge0(a, b) != (a / b >= 0.0)) { std::printf("mismatch quotient %a %a\n", a, b); return 1; }
      n++;
    }
  }
  // quotients that underflow to -0 and their neighbours
  const double tiny[] = {5e-324, 1e-320, 1e-310, 2.2250738585072014e-308, 1e-300};
  const double huge[] = {1e10, 1e100, 1e290, 1.7976931348623157e308};
  for (double t : tiny)
    for (double h : huge)
      for (int sg = 0; sg < 4; sg++) {
        double a = (sg & 1) ? -t : t, b = (sg & 2) ? -h : h;
        if (i_quotient_ge0(a, b) != (a / b >= 0.0)) { std::printf("mismatch underflow %a %a\n", a, b); return 1; }
        n++;
      }
  // the division-free physicality tests against the reference forms
  for (int k = 0; k < 200000; k++) {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    double r1 = (double)(s >> 11) / 9007199254740992.0;
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    double r2 = (double)(s >> 11) / 9007199254740992.0;
    const double rho = (k % 7 == 0) ? -r1 : std::ldexp(r1 + 1e-3, (int)(s % 40) - 20);
    const double u = (r2 - 0.5) * 1e3, v = (r1 - 0.5) * 10.0;
    // E chosen so that e sits on either side of zero, down to a few ulps
    const double ke = 0.5 * rho * (u * u + v * v);
    const double E = ke * (1.0 + (r2 - 0.5) * std::ldexp(1.0, -(int)(s % 60)));
    V4 U{rho, rho * u, rho * v, E};
    if (is_physical_state_fast(U) != is_physical_state(U)) { std::printf("mismatch state %a %a %a %a\n", U.a, U.b, U.c, U.d); return 1; }
    V4 W{rho, u, v, (r2 - 0.3) * std::ldexp(1.0, (int)(s % 30) - 10)};
    const double g = 1.4 + r1, pinf = (k & 1) ? 0.0 : 3e8 * r2;
    if (is_physical_primitives_fast(g, pinf, W) != is_physical_primitives(g, pinf, W)) {
      std::printf("mismatch prims %a %a\n", W.a, W.d); return 1;
    }
    const double num = W.d + g * pinf, den = (g - 1.0) * W.a;
    if (i_quotient_ge0(num, den) != quotient_ge0(num, den)) { std::printf("mismatch iq %a %a\n", num, den); return 1; }
    n += 3;
  }
  // shared-reciprocal quotients against the division: random operands over
  // the whole exponent range and mantissas with long runs of ones or zeros
  auto mant = [&](int kind) -> uint64_t {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    switch (kind) {
      case 0: return s & 0xfffffffffffffULL;
      case 1: return 0xfffffffffffffULL ^ (s & 0xffULL);            // near all ones
      case 2: return s & 0xffULL;                                    // near a power of two
      default: return (s & 1) ? 0xfffffffffffffULL : (1ULL << (s % 52));
    }
  };
  long nd = 0;
  for (int k = 0; k < 20000000; k++) {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    const uint64_t ea = 1 + (s % 2046), eb = 1 + ((s >> 12) % 2046);
    const uint64_t sa = (s >> 30) & 1, sb = (s >> 31) & 1;
    const double a = dbl((sa << 63) | (ea << 52) | mant(k & 3));
    const double b = dbl((sb << 63) | (eb << 52) | mant((k >> 2) & 3));
    const Recip R = recip(b);
    const double q = i_rdiv(a, R), ref = a / b;
    uint64_t qb, rb; std::memcpy(&qb, &q, 8); std::memcpy(&rb, &ref, 8);
    if (qb != rb && !(std::isnan(q) && std::isnan(ref))) {
      std::printf("mismatch rdiv %a / %a: %a vs %a\n", a, b, q, ref); return 1;
    }
    nd++;
  }
  for (double a : v)
    for (size_t q = 0; q < v.size(); q += 13) {
      const Recip R = recip(v[q]);
      const double x = i_rdiv(a, R), ref = a / v[q];
      uint64_t xb, rb; std::memcpy(&xb, &x, 8); std::memcpy(&rb, &ref, 8);
      if (xb != rb && !(std::isnan(x) && std::isnan(ref))) { std::printf("mismatch rdiv %a / %a\n", a, v[q]); return 1; }
      nd++;
    }
  std::printf("ok %ld rdiv %ld\n", n, nd);
  return 0;
}
