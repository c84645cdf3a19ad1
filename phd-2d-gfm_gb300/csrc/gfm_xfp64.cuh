// IEEE-754 binary64 multiply and add, correctly rounded to nearest-even,
// computed with 32-bit integer instructions.
//
// On this GPU a warp's FP64 instruction holds its sub-partition's FP64 pipe
// for 64 cycles, while the integer pipes that issue beside it stay idle in
// FP64-bound kernels.  xmul and xadd return exactly the double that a * b and
// a + b return (round to nearest, ties to even: the result is unique), so a
// kernel may move part of its multiplies and adds onto the integer pipes
// without changing a bit of its output.  Operands or results outside the
// range where the integer path is simple (zeros, subnormals, infinities,
// NaNs, products and sums near the ends of the exponent range, exact
// cancellation) take the native instruction instead.
//
// The same source compiles for the host, where tests compare it with the
// host's own double arithmetic on random and boundary operands.
//
// The rounding is the textbook one (Goldberg, "What every computer scientist
// should know about floating-point arithmetic", 1991, section 1.3; IEEE
// 754-2008 section 4.3.1): the exact result is formed with guard bits and a
// sticky bit and rounded once.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define XFP_HD __host__ __device__ __forceinline__
#else
#define XFP_HD inline
#endif

namespace gfm {

XFP_HD void xfp_split(double x, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  hi = (uint32_t)__double2hiint(x);
  lo = (uint32_t)__double2loint(x);
#else
  uint64_t b; memcpy(&b, &x, 8);
  hi = (uint32_t)(b >> 32); lo = (uint32_t)b;
#endif
}

XFP_HD double xfp_join(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x; memcpy(&x, &b, 8); return x;
#endif
}

XFP_HD uint32_t xfp_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__clzll((long long)x);
#else
  return x ? (uint32_t)__builtin_clzll(x) : 64u;
#endif
}

// high 64 bits of the 128-bit product
XFP_HD uint64_t xfp_mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
// high 64 bits of the signed 128-bit product (floor of the product / 2^64)
XFP_HD int64_t xfp_smulhi(int64_t a, int64_t b) {
#if defined(__CUDA_ARCH__)
  return __mul64hi(a, b);
#else
  return (int64_t)(((__int128)a * b) >> 64);
#endif
}

// Seeds of the Newton-Raphson iterations below: 1/f and 1/sqrt(f) for a
// float f in [2^22, 2^24), to about 2^-22 relative (the hardware's
// approximate reciprocal and reciprocal square root on the device, the
// correctly rounded float operations on the host; the iterations and the
// final remainder test make the result independent of which).
XFP_HD float xfp_rcp_seed(float f) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
  return r;
#else
  return 1.0f / f;
#endif
}
XFP_HD float xfp_rsqrt_seed(float f) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
  return r;
#else
  return 1.0f / sqrtf(f);
#endif
}
XFP_HD uint32_t xfp_float_bits(float f) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__float_as_uint(f);
#else
  uint32_t b; memcpy(&b, &f, 4); return b;
#endif
}
// f * 2^k as an unsigned integer, f > 0 a float and the result below 2^64
// (the significand shifted by the exponent; no rounding)
XFP_HD uint64_t xfp_float_fixed(float f, int k) {
  const uint32_t b = xfp_float_bits(f);
  const uint64_t m = (uint64_t)((b & 0x7fffffu) | 0x800000u);
  const int s = (int)(b >> 23) - 150 + k;
  return s >= 0 ? (m << s) : (m >> -s);
}

// Correct rounding of a positive significand: the integer q (with sh + 53
// significant bits below the exact value's rounding point, sh = 2 or 3) and
// the sticky flag (exact value above q) give the rounded 53-bit significand
// plus the exponent carry, packed over the sign and biased exponent E - 1.
XFP_HD double xfp_round_pack(uint32_t sign_bit, int E, uint64_t q, uint32_t sh, uint32_t sticky) {
  const uint64_t mant = q >> sh;
  const uint32_t rem = (uint32_t)q & ((1u << sh) - 1u);
  const uint32_t up = (((rem << 1) | sticky) + ((uint32_t)mant & 1u)) > (1u << sh);
  const uint32_t top = sign_bit | ((uint32_t)(E - 1) << 20);
  return xfp_join(((uint64_t)top << 32) + mant + up);
}

// a * b.  Integer path when both operands are normal and the biased
// exponent sum E0 = ea + eb - 1023 lies in [1, 2045]: the product of the two
// 53-bit significands (each shifted to the top of 64 bits) has its leading
// one at bit 127 or 126 of the 128-bit product; the top 53 bits below it are
// the significand, the next bit the guard bit, the rest (and the low 64
// bits) the sticky bit.  A carry out of the rounded significand moves into
// the exponent field, and an exponent field of 2047 with a zero fraction is
// the correctly rounded overflow to infinity.
XFP_HD double xmul(double a, double b) {
  uint32_t ha, la, hb, lb;
  xfp_split(a, ha, la);
  xfp_split(b, hb, lb);
  const uint32_t ea = (ha >> 20) & 0x7ffu, eb = (hb >> 20) & 0x7ffu;
  const int E0 = (int)(ea + eb) - 1023;
  if (!((ea - 1u < 2046u) & (eb - 1u < 2046u) & ((uint32_t)(E0 - 1) < 2045u))) return a * b;
  const uint32_t A1 = (ha << 11) | (la >> 21) | 0x80000000u, A0 = la << 11;
  const uint32_t B1 = (hb << 11) | (lb >> 21) | 0x80000000u, B0 = lb << 11;
  const uint64_t p00 = (uint64_t)A0 * B0, p01 = (uint64_t)A0 * B1;
  const uint64_t p10 = (uint64_t)A1 * B0, p11 = (uint64_t)A1 * B1;
  const uint64_t mid = (p00 >> 32) + (uint32_t)p01 + (uint32_t)p10;
  const uint64_t hi = p11 + (p01 >> 32) + (p10 >> 32) + (mid >> 32);
  const uint32_t lo_nz = ((uint32_t)p00 | (uint32_t)mid) != 0u;
  const uint32_t s = (uint32_t)(hi >> 63);
  const uint32_t sh = 10u + s;
  const uint64_t mant = hi >> sh;
  const uint32_t rem = (uint32_t)hi & ((1u << sh) - 1u);
  const uint32_t up = (((rem << 1) | lo_nz) + ((uint32_t)mant & 1u)) > (1u << sh);
  const uint32_t top = ((ha ^ hb) & 0x80000000u) | ((uint32_t)(E0 + (int)s - 1) << 20);
  return xfp_join(((uint64_t)top << 32) + mant + up);
}

// a + b.  Integer path when both operands are normal with exponents below
// 2045 (no overflow) and the sum is normal and nonzero: the larger-magnitude
// operand's significand is placed with its leading one at bit 62, the
// other's aligned to it with the bits shifted out jammed into bit 0 (ten
// guard bits lie below the significand), added or subtracted, normalised so
// that the leading one is again at bit 62, and rounded at bit 10.  An
// operand 55 or more binades below the other is below a quarter of the
// larger one's unit in the last place and leaves it unchanged.
XFP_HD double xadd(double a, double b) {
  uint32_t ha, la, hb, lb;
  xfp_split(a, ha, la);
  xfp_split(b, hb, lb);
  const uint32_t ea = (ha >> 20) & 0x7ffu, eb = (hb >> 20) & 0x7ffu;
  if (!((ea - 1u < 2044u) & (eb - 1u < 2044u))) return a + b;
  const uint64_t ma = ((uint64_t)(ha & 0x7fffffffu) << 32) | la;
  const uint64_t mb = ((uint64_t)(hb & 0x7fffffffu) << 32) | lb;
  const bool swap = mb > ma;
  const uint64_t mx = swap ? mb : ma, my = swap ? ma : mb;
  const uint32_t ex = swap ? eb : ea, ey = swap ? ea : eb;
  const uint32_t sx = (swap ? hb : ha) & 0x80000000u;
  const uint32_t d = ex - ey;
  if (d >= 55u) return swap ? b : a;
  const uint64_t X = ((mx & 0x000fffffffffffffull) | 0x0010000000000000ull) << 10;
  const uint64_t Y0 = ((my & 0x000fffffffffffffull) | 0x0010000000000000ull) << 10;
  const uint64_t Y = (Y0 >> d) | (uint64_t)((Y0 << ((64u - d) & 63u)) != 0u && d != 0u);
  const uint64_t m = ((ha ^ hb) & 0x80000000u) ? X - Y : X + Y;
  if (m == 0u) return a + b;
  const uint32_t L = 63u - xfp_clz64(m);          // 63 after a carry, <= 62 otherwise
  const int er = (int)ex + (int)L - 62;
  if (er < 1) return a + b;
  const uint64_t n = (L == 63u) ? ((m >> 1) | (m & 1u)) : (m << (62u - L));
  const uint64_t mant = n >> 10;
  const uint32_t rem = (uint32_t)n & 0x3ffu;
  const uint32_t up = (rem + ((uint32_t)mant & 1u)) > 0x200u;
  const uint32_t top = sx | ((uint32_t)(er - 1) << 20);
  return xfp_join(((uint64_t)top << 32) + mant + up);
}

// a / b.  Division by Newton-Raphson reciprocal iteration with a final
// remainder correction (Muller et al., "Handbook of Floating-Point
// Arithmetic", 2nd ed. 2018, sections 4.7 and 5.3; the integer form follows
// Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): with A, B the significands shifted to the top
// of 64 bits, a 24-bit float seed of 2^127/B is refined by one step in 32-bit
// precision and one in 64-bit, the truncated quotient Q = floor(Ma 2^55 / Mb)
// (55 or 56 bits) is formed from it to within one unit and made exact by the
// sign and size of the remainder Ma 2^55 - Q Mb, which also gives the sticky
// bit.  Integer path when both operands are normal and the biased exponent
// difference E = ea - eb + 1023 lies in [2, 2045].  About 200 cycles of
// dependent integer work against some 560 for the FP64 division, and no
// FP64 instruction.
XFP_HD double xdiv(double a, double b) {
  uint32_t ha, la, hb, lb;
  xfp_split(a, ha, la);
  xfp_split(b, hb, lb);
  const uint32_t ea = (ha >> 20) & 0x7ffu, eb = (hb >> 20) & 0x7ffu;
  const int E = (int)ea - (int)eb + 1023;
  if (!((ea - 1u < 2046u) & (eb - 1u < 2046u) & ((uint32_t)(E - 2) < 2044u))) return a / b;
  const uint64_t Ma = ((uint64_t)((ha & 0xfffffu) | 0x100000u) << 32) | la;
  const uint64_t Mb = ((uint64_t)((hb & 0xfffffu) | 0x100000u) << 32) | lb;
  const uint64_t A = Ma << 11, B = Mb << 11;
  // seed X0 ~ 2^63 / B32 in (2^31, 2^32], B32 = B / 2^32
  const uint32_t B32 = (uint32_t)(B >> 32);
  const uint64_t X0 = xfp_float_fixed(xfp_rcp_seed((float)(B32 >> 8)), 55);
  // step 1: X1 = X0 (1 + e), e = 1 - B32 X0 / 2^63 (|e| ~ 2^-22)
  const uint64_t P = (uint64_t)B32 * X0;
  const int64_t D = (int64_t)((1ull << 63) - P);
  const uint64_t Dm = (uint64_t)(D < 0 ? -D : D) >> 12;
  const uint64_t c1 = (X0 * Dm) >> 51;
  uint64_t X1 = D < 0 ? X0 - c1 : X0 + c1;
  if (X1 > 0xffffffffull) X1 = 0xffffffffull;
  // step 2 in 64 bits: X2 ~ 2^127 / B to about 2^-60
  const uint64_t X = X1 << 32;
  const uint64_t Ph = xfp_mulhi(B, X);
  const int64_t D2 = (int64_t)((1ull << 63) - Ph);
  const uint64_t c2 = xfp_mulhi(X, (uint64_t)(D2 < 0 ? -D2 : D2) << 1);
  uint64_t X2 = D2 < 0 ? X - c2 : X + c2;
  if (D2 >= 0 && X2 < X) X2 = ~0ull;
  // quotient to within one unit, then exact
  uint64_t Q = xfp_mulhi(A, X2) >> 8;
  int64_t R = (int64_t)((Ma << 55) - Q * Mb);
  if (R < 0) { Q -= 1; R += (int64_t)Mb; }
  else if (R >= (int64_t)Mb) { Q += 1; R -= (int64_t)Mb; }
  const uint32_t hi = (uint32_t)(Q >> 55);
  return xfp_round_pack((ha ^ hb) & 0x80000000u, E - 1 + (int)hi, Q, 2u + hi, R != 0);
}

// sqrt(x).  Newton-Raphson on the reciprocal square root (Muller et al.,
// section 5.4) with a final remainder correction: the significand, shifted
// by the exponent's parity and to the top of 64 bits (C), gets a 24-bit float
// seed of 2^95/sqrt(C) refined once in 32-bit and once in 64-bit precision;
// S = floor(sqrt(C 2^46)) (55 bits) follows to within one unit and is made
// exact by the remainder C 2^46 - S^2.  Integer path for positive normal x.
// About 200 cycles of dependent integer work against some 680 for the FP64
// square root.
XFP_HD double xsqrt(double x) {
  uint32_t h, l;
  xfp_split(x, h, l);
  const uint32_t ex = h >> 20;   // the sign bit too: positive numbers only
  if (ex - 1u >= 2046u) return sqrt(x);
  const uint64_t Mx = ((uint64_t)((h & 0xfffffu) | 0x100000u) << 32) | l;
  const int e = (int)ex - 1075;
  const int odd = e & 1;
  const uint64_t C = Mx << (10 + odd);   // [2^62, 2^64); value sqrt(C 2^46) 2^(-28 + (e - odd)/2)
  // seed Y0 ~ 2^30 / sqrt(c), c = C / 2^64 (Y0 in (2^30, 2^31])
  const uint64_t Y0 = xfp_float_fixed(xfp_rsqrt_seed((float)(C >> 40)), 42);
  // step 1: y1 = y0 (1 + (1 - c y0^2) / 2), 62 fraction bits
  const uint32_t c32 = (uint32_t)(C >> 32);
  const uint64_t t = ((Y0 * Y0) >> 30) * c32;
  const int64_t E1 = (int64_t)((1ull << 62) - t);
  const uint64_t c1 = (Y0 * ((uint64_t)(E1 < 0 ? -E1 : E1) >> 11)) >> 20;
  const uint64_t Y1 = E1 < 0 ? (Y0 << 32) - c1 : (Y0 << 32) + c1;
  // step 2 in 64 bits
  const uint64_t t2 = xfp_mulhi(xfp_mulhi(Y1, Y1), C);
  const int64_t E2 = (int64_t)((1ull << 60) - t2);
  const uint64_t c2 = xfp_mulhi(Y1, (uint64_t)(E2 < 0 ? -E2 : E2) << 3);
  const uint64_t Y2 = E2 < 0 ? Y1 - c2 : Y1 + c2;
  // root to within one unit, then exact
  uint64_t S = xfp_mulhi(C, Y2) >> 7;
  int64_t R = (int64_t)((C << 46) - S * S);
  if (R < 0) { R += (int64_t)(2 * S - 1); S -= 1; }
  else if (R > (int64_t)(2 * S)) { S += 1; R -= (int64_t)(2 * S - 1); }
  return xfp_round_pack(0u, 1049 + ((e - odd) >> 1), S, 2u, R != 0);
}

}  // namespace gfm
