// Device check of the integer-arithmetic divide and square root of
// gfm_xfp64.cuh against the GPU's own IEEE double division and square root,
// bit for bit: every leading 24-bit pattern of the divisor's (and the root
// argument's) significand with random low bits, exponent parity and
// dividend, then random bit patterns and near squares.  The device seeds are
// the hardware's approximate reciprocal and reciprocal square root, which
// the host check (xfp64_check.cpp) does not exercise.  Then the fixed-point
// gfm_pow (gfm_math.cuh) on the device against the same function compiled
// for the host, bit for bit, on the argument ranges of the Riemann solver and
// beyond.  Prints "ok <count>" or the first mismatches.  Built and run by
// tests/test_xfp64.py.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>
#include "../phd-2d-gfm_gb300/csrc/gfm_math.cuh"

using namespace gfm;

__device__ __forceinline__ uint64_t mix(uint64_t x) {   // splitmix64
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// case k: mode 0 the seed sweep (k = leading 24 bits), mode 1 random bits,
// mode 2 near squares and near-exact quotients
__global__ void check(int mode, uint64_t n, unsigned long long* bad, double* first) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint64_t r1 = mix(k * 3 + (uint64_t)mode * 0x1000000000ull), r2 = mix(r1), r3 = mix(r2);
  double a, b;
  if (mode == 0) {
    const uint64_t frac = ((k & 0xffffffull) << 28) | (r1 & 0xfffffffull);
    b = __longlong_as_double((long long)((((uint64_t)(1023 + (r2 & 1))) << 52) | frac));
    a = __longlong_as_double((long long)((r3 & 0x800fffffffffffffull) | ((uint64_t)(1000 + r3 % 40) << 52)));
  } else if (mode == 1) {
    a = __longlong_as_double((long long)r1);
    b = __longlong_as_double((long long)r2);
  } else {
    const double r = (double)(r1 >> 38) + 1.0, p = (double)(r2 >> 40) + 1.0, q = (double)(r3 >> 40) + 1.0;
    const double sq = r * r;
    a = (k & 1) ? __longlong_as_double(__double_as_longlong(sq) + (long long)(r3 & 3) - 1) : p * q;
    b = (k & 1) ? sq : q;
  }
  const double ops[6] = {a / b, xdiv(a, b), sqrt(fabs(a)), xsqrt(fabs(a)), sqrt(b), xsqrt(b)};
  for (int t = 0; t < 3; t++) {
    const double want = ops[2 * t], got = ops[2 * t + 1];
    const bool same = (want != want) ? (got != got) : (__double_as_longlong(want) == __double_as_longlong(got));
    if (!same) {
      const unsigned long long s = atomicAdd(bad, 1ull);
      if (s < 4) { first[4 * s] = a; first[4 * s + 1] = b; first[4 * s + 2] = want; first[4 * s + 3] = got; }
    }
  }
}

// pow case k: (x, y) from the same generator on both sides
__host__ __device__ void pow_case(uint64_t k, double& x, double& y) {
  uint64_t a = k * 0x9e3779b97f4a7c15ull + 12345u;
  a ^= a >> 31; a *= 0xbf58476d1ce4e5b9ull; a ^= a >> 29;
  uint64_t b = a * 0x94d049bb133111ebull; b ^= b >> 32;
  // only exact integer work and correctly rounded IEEE operations, so the
  // host and the device build the same arguments
  const double u = (double)(a >> 11) * 0x1p-53, v = (double)(b >> 11) * 0x1p-53;
  const uint64_t frac = a & 0x000fffffffffffffull;
  uint64_t xb;
  switch (k % 5) {
    case 0: xb = frac | ((uint64_t)(1023 - 15 + (b % 31)) << 52); memcpy(&x, &xb, 8);   // pressure ratios
            y = (v - 0.5) * 16.0; break;
    case 1: x = 1.0 + (u - 0.5) * 1e-3; y = (v - 0.5) * 20.0; break;                    // near 1
    case 2: xb = a & 0x7fffffffffffffffull; memcpy(&x, &xb, 8); y = (v - 0.5) * 4.0; break;   // any positive double
    case 3: x = u * 100.0; y = 1.0 / (1.09 + v * 5.0); break;                           // 1/gamma
    default: xb = frac | ((uint64_t)(23 + (b % 2001)) << 52); memcpy(&x, &xb, 8);       // extreme bases
             y = v * 2.0 - 1.0; break;
  }
}
__global__ void pow_dev(uint64_t n, double* out) {
  const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double x, y;
  pow_case(k, x, y);
  out[k] = gfm::gfm_pow(x, y);
}

int main() {
  unsigned long long* bad;
  double* first;
  if (cudaMalloc(&bad, 8) != cudaSuccess || cudaMalloc(&first, 16 * 8) != cudaSuccess) return 2;
  cudaMemset(bad, 0, 8);
  const uint64_t sizes[3] = {1ull << 24, 1ull << 26, 1ull << 24};
  uint64_t total = 0;
  for (int mode = 0; mode < 3; mode++) {
    const uint64_t n = sizes[mode];
    check<<<(unsigned)((n + 255) / 256), 256>>>(mode, n, bad, first);
    total += 3 * n;
  }
  // fixed-point pow: device against host
  const uint64_t np = 1ull << 22;
  double* d_pow;
  if (cudaMalloc(&d_pow, np * 8) != cudaSuccess) return 2;
  pow_dev<<<(unsigned)(np / 256), 256>>>(np, d_pow);
  std::vector<double> hp(np);
  if (cudaMemcpy(hp.data(), d_pow, np * 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  uint64_t pow_bad = 0;
  for (uint64_t k = 0; k < np; k++) {
    double x, y;
    pow_case(k, x, y);
    const double want = gfm::gfm_pow(x, y);
    if (memcmp(&want, &hp[k], 8) != 0 && !(want != want && hp[k] != hp[k])) {
      if (pow_bad < 4) printf("pow(%a, %a): host %a device %a\n", x, y, want, hp[k]);
      pow_bad++;
    }
  }
  if (pow_bad) {
    printf("pow mismatches %llu\n", (unsigned long long)pow_bad);
    return 1;
  }
  total += np;
  unsigned long long h_bad = 0;
  double h_first[16];
  if (cudaMemcpy(&h_bad, bad, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  if (cudaMemcpy(h_first, first, sizeof(h_first), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  if (h_bad) {
    printf("mismatches %llu\n", h_bad);
    for (unsigned s = 0; s < h_bad && s < 4; s++)
      printf("a %a b %a want %a got %a\n", h_first[4 * s], h_first[4 * s + 1], h_first[4 * s + 2], h_first[4 * s + 3]);
    return 1;
  }
  printf("ok %llu\n", (unsigned long long)total);
  return 0;
}
