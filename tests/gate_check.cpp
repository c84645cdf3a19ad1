// Host check that the learned proposal's gate written as two comparisons,
// mlp_gated(ratio) (phd-2d-gfm_gb300/csrc/gfm_mlp.cuh), decides exactly as
// |gfm_log(ratio)| > MLP_GATE with ratio > 0: every double within 2^22 ulps
// of either threshold, then random ratios over the positive range, the
// pressure-ratio range, NaN, infinities and signed zeros.  Prints "ok
// <count>" or the first mismatches.  Built and run by tests/test_xfp64.py.
#include <cstdio>
#include <cstring>
#include <cmath>
#include <cstdint>
#include "../phd-2d-gfm_gb300/csrc/gfm_mlp.cuh"

using namespace gfm;

static double step(double x, int64_t d) { int64_t b; std::memcpy(&b, &x, 8); b += d; std::memcpy(&x, &b, 8); return x; }
static bool by_log(double r) { return r > 0.0 && std::fabs(gfm_log(r)) > MLP_GATE; }

int main() {
  long n = 0, bad = 0;
  auto check = [&](double r) {
    n++;
    if (mlp_gated(r) != by_log(r)) {
      if (bad < 4) std::printf("ratio %a: comparisons %d log %d\n", r, (int)mlp_gated(r), (int)by_log(r));
      bad++;
    }
  };
  for (int64_t d = -(1 << 22); d <= (1 << 22); d++) {
    check(step(MLP_GATE_HI, d));
    check(step(MLP_GATE_LO, d));
  }
  uint64_t st = 88172645463325252ULL;
  for (int i = 0; i < 4000000; i++) {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    double r;
    if (i & 1) {
      const uint64_t b = st & 0x7fffffffffffffffULL;   // any non-negative bit pattern, NaN included
      std::memcpy(&r, &b, 8);
    } else {
      r = 0.9 + 0.2 * ((double)(st >> 11) * 0x1p-53);
    }
    check(r);
  }
  const double special[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -1.0, 1.0, 0x1p-1074};
  for (double r : special) check(r);
  if (bad) { std::printf("mismatches %ld of %ld\n", bad, n); return 1; }
  std::printf("ok %ld\n", n);
  return 0;
}
