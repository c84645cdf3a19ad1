// Scalar FP64 arithmetic of the two-fluid ghost-fluid Euler step, shared by
// every kernel (and compiled for the host by the unit tests).
//
// Every function here fixes its operation order so that a CPU restatement
// compiled with -ffp-contract=off and these kernels compiled with
// --fmad=false produce bit-identical doubles.  The elementary functions
// (exp, log, pow, acos) are this project's own, so neither libm nor CUDA's
// math library decides a single bit of the result.
//
// Contents, with the reference code each part follows:
//   * stiffened-gas EOS (pressure, specific_ie, soundspeed,
//     isentropic_extrapolation).  The reference calls these from its absent
//     PhD-Common dependency (headers/euler_misc.hpp:46,59,77,96,156,173,
//     sourcecode/GFM_original.cpp:76); the standard stiffened-gas forms are used.
//   * misc:: state algebra, headers/euler_misc.hpp:23-180.
//   * exact stiffened-gas Riemann solver: Toro, "Riemann Solvers and Numerical
//     Methods for Fluid Dynamics", ch. 4 (pressure functions, Newton-Raphson
//     from the PVRS guess, refined by the two-shock guess for two materials,
//     sampling), with p -> p + p_inf.  It replaces the
//     absent exact_rs_stiffenedgas used at sourcecode/pure_RS_exact.cpp:29-45
//     and sourcecode/mixed_RS_exact.cpp:33-47.
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>
#include "gfm_tables.h"
#include "gfm_xfp64.cuh"

#if defined(__CUDACC__)
#define GFM_HD __host__ __device__ __forceinline__
#else
#define GFM_HD inline
#endif

namespace gfm {

// The products of the functions below.  In the device code of a translation
// unit compiled with GFM_INT_MUL defined (the flux update built with
// GFM_FLUX_INT_MUL) they are formed on the integer pipes (xmul,
// gfm_xfp64.cuh: the same bits as the FP64 multiply); everywhere else, the
// host included, they are the FP64 multiply itself.
#if defined(__CUDA_ARCH__) && defined(GFM_INT_MUL)
GFM_HD double mulx(double a, double b) { return xmul(a, b); }
#else
GFM_HD double mulx(double a, double b) { return a * b; }
#endif

// The quotients and square roots of the functions below.  In device code
// they are formed in integer arithmetic (xdiv, xsqrt: the correctly rounded
// result, so the same bits as the FP64 division and square root), which
// takes none of the FP64 pipe's time: 2.4 (division) and 3.1 (square root)
// times the FP64 operations' throughput on GB300, where the FP64 pipe bounds
// every full-grid kernel here.  GFM_FP64_DIV selects the FP64 operations
// everywhere; the host always uses them.
// The functions that divide or take roots carry the choice as their template
// argument ID (true: integer arithmetic); the latency-bound interface loop,
// where a dependent integer quotient (about 510 cycles) saves little over the
// FP64 one (560) and its longer code costs more, instantiates them with false.
template <bool ID = true>
GFM_HD double divx(double a, double b) {
#if defined(__CUDA_ARCH__) && !defined(GFM_FP64_DIV)
  if (ID) return xdiv(a, b);
#endif
  return a / b;
}
template <bool ID = true>
GFM_HD double sqrtx(double x) {
#if defined(__CUDA_ARCH__) && !defined(GFM_FP64_DIV)
  if (ID) return xsqrt(x);
#endif
  return sqrt(x);
}

// ---------------------------------------------------------------------------
// Status bits written by kernels (never __trap or assert on the device).
// ---------------------------------------------------------------------------
enum : uint32_t {
  ST_OK = 0,
  ST_UNPHYSICAL = 1u << 0,       // rho < 0 or e < 0 where the reference asserts
  ST_NEWTON_NO_CONVERGE = 1u << 1,
  ST_VACUUM = 1u << 2,           // Riemann data generate vacuum
  ST_NAN = 1u << 3,              // NaN p* from the mixed solver (GFM_real.cpp:173)
  ST_DT_NONPOSITIVE = 1u << 4,   // sim_twofluid.cpp:155
  ST_SCHEDULE_LIMIT = 1u << 5,   // interface schedule exceeded its round limit
  ST_BAD_ARGUMENT = 1u << 6,
};

// ---------------------------------------------------------------------------
// Bit casts and constant tables
// ---------------------------------------------------------------------------
GFM_HD int64_t as_bits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t b; memcpy(&b, &x, 8); return b;
#endif
}
GFM_HD double from_bits(int64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x; memcpy(&x, &b, 8); return x;
#endif
}

#if defined(__CUDACC__)
__device__ static const double d_exp2_tab[64] = GFM_EXP2_TABLE;
__device__ static const double d_logf_tab[97] = GFM_LOGF_TABLE;
__device__ static const double d_invf_tab[97] = GFM_INVF_TABLE;
#endif
static const double h_exp2_tab[64] = GFM_EXP2_TABLE;
static const double h_logf_tab[97] = GFM_LOGF_TABLE;
static const double h_invf_tab[97] = GFM_INVF_TABLE;
static const double h_asin_c[28] = GFM_ASIN_COEFFS;
#if defined(__CUDACC__)
__device__ static const double d_asin_c[28] = GFM_ASIN_COEFFS;
#endif

GFM_HD double tab_exp2(int j) {
#if defined(__CUDA_ARCH__)
  return __ldg(&d_exp2_tab[j]);
#else
  return h_exp2_tab[j];
#endif
}
GFM_HD double tab_logf(int j) {
#if defined(__CUDA_ARCH__)
  return __ldg(&d_logf_tab[j]);
#else
  return h_logf_tab[j];
#endif
}
GFM_HD double tab_invf(int j) {
#if defined(__CUDA_ARCH__)
  return __ldg(&d_invf_tab[j]);
#else
  return h_invf_tab[j];
#endif
}
GFM_HD double tab_asin(int j) {
#if defined(__CUDA_ARCH__)
  return __ldg(&d_asin_c[j]);
#else
  return h_asin_c[j];
#endif
}

// tables of the fixed-point pow (gen_tables.py)
#if defined(__CUDACC__)
__device__ static const uint32_t d_xlog1_ri[49] = GFM_XLOG1_RI;
__device__ static const int64_t d_xlog1_t[49] = GFM_XLOG1_T;
__device__ static const uint32_t d_xlog2_ri[97] = GFM_XLOG2_RI;
__device__ static const int64_t d_xlog2_t[97] = GFM_XLOG2_T;
__device__ static const uint64_t d_xexp1_e[64] = GFM_XEXP1_E;
__device__ static const uint64_t d_xexp2_e[64] = GFM_XEXP2_E;
#endif
static const uint32_t h_xlog1_ri[49] = GFM_XLOG1_RI;
static const int64_t h_xlog1_t[49] = GFM_XLOG1_T;
static const uint32_t h_xlog2_ri[97] = GFM_XLOG2_RI;
static const int64_t h_xlog2_t[97] = GFM_XLOG2_T;
static const uint64_t h_xexp1_e[64] = GFM_XEXP1_E;
static const uint64_t h_xexp2_e[64] = GFM_XEXP2_E;
#if defined(__CUDA_ARCH__)
#define GFM_XTAB(name, j) __ldg(&d_##name[j])
#define GFM_XTAB64(type, name, j) ((type)__ldg((const unsigned long long*)&d_##name[j]))
#else
#define GFM_XTAB(name, j) (h_##name[j])
#define GFM_XTAB64(type, name, j) (h_##name[j])
#endif

GFM_HD double gfm_inf() { return from_bits(0x7ff0000000000000LL); }
GFM_HD double gfm_nan() { return from_bits(0x7ff8000000000000LL); }

// ---------------------------------------------------------------------------
// IEEE comparisons on the integer pipe.  On GB300 an FP64 compare holds the
// FP64 pipe about as long as a multiply-add, and that pipe bounds every kernel
// here, while integer instructions issue beside it.  Each function returns
// exactly what the C comparison returns for all doubles, NaN and signed zeros
// included; host builds use the C comparison itself.
//   key: |x| bits for x >= +0, -(|x| bits) for x <= -0, so -0 and +0 share 0
// ---------------------------------------------------------------------------
#define GFM_MAG_BITS 0x7fffffffffffffffLL
#define GFM_INF_BITS 0x7ff0000000000000LL

GFM_HD bool nan_bits(int64_t b) { return (b & GFM_MAG_BITS) > GFM_INF_BITS; }
GFM_HD int64_t order_key(int64_t b) { return b < 0 ? -(b & GFM_MAG_BITS) : b; }
GFM_HD bool i_lt(double a, double b) {
  const int64_t x = as_bits(a), y = as_bits(b);
  return !nan_bits(x) && !nan_bits(y) && order_key(x) < order_key(y);
}
GFM_HD bool i_le(double a, double b) {
  const int64_t x = as_bits(a), y = as_bits(b);
  return !nan_bits(x) && !nan_bits(y) && order_key(x) <= order_key(y);
}
GFM_HD bool i_eq(double a, double b) {
  const int64_t x = as_bits(a), y = as_bits(b);
  return !nan_bits(x) && order_key(x) == order_key(y);
}
GFM_HD bool i_gt0(double a) { const int64_t x = as_bits(a); return x > 0 && x <= GFM_INF_BITS; }
GFM_HD bool i_ge0(double a) {
  const int64_t x = as_bits(a);
  return (x >= 0 && x <= GFM_INF_BITS) || x == (int64_t)0x8000000000000000ULL;
}
GFM_HD bool i_lt0(double a) {
  const int64_t x = as_bits(a), m = x & GFM_MAG_BITS;
  return x < 0 && m != 0 && m <= GFM_INF_BITS;
}
GFM_HD bool i_le0(double a) {
  const int64_t x = as_bits(a), m = x & GFM_MAG_BITS;
  return m == 0 || (x < 0 && m <= GFM_INF_BITS);
}
// (n / d) >= 0.0 without the division where the operands decide it: the
// quotient's sign is the XOR of the signs, NaN comes from a NaN operand, 0/0
// or inf/inf, and a negative quotient reads as -0 (>= 0) only when it
// underflows, which needs exponents about 1000 apart; then the division
// itself decides.
GFM_HD bool i_quotient_ge0(double n, double d) {
  const int64_t x = as_bits(n), y = as_bits(d);
  const int64_t mx = x & GFM_MAG_BITS, my = y & GFM_MAG_BITS;
  if (mx > GFM_INF_BITS || my > GFM_INF_BITS) return false;
  if (mx == 0) return my != 0;
  if (mx == GFM_INF_BITS && my == GFM_INF_BITS) return false;
  if ((x ^ y) >= 0) return true;
  if (my == GFM_INF_BITS) return true;
  if ((int)(mx >> 52) - (int)(my >> 52) > -900) return false;
  return n / d >= 0.0;
}
#if defined(__CUDA_ARCH__)
GFM_HD bool c_lt(double a, double b) { return i_lt(a, b); }
GFM_HD bool c_le(double a, double b) { return i_le(a, b); }
GFM_HD bool c_eq(double a, double b) { return i_eq(a, b); }
GFM_HD bool c_gt0(double a) { return i_gt0(a); }
GFM_HD bool c_ge0(double a) { return i_ge0(a); }
GFM_HD bool c_lt0(double a) { return i_lt0(a); }
GFM_HD bool c_le0(double a) { return i_le0(a); }
GFM_HD bool c_isnan(double a) { return nan_bits(as_bits(a)); }
GFM_HD bool quotient_ge0(double n, double d) { return i_quotient_ge0(n, d); }
#else
GFM_HD bool c_lt(double a, double b) { return a < b; }
GFM_HD bool c_le(double a, double b) { return a <= b; }
GFM_HD bool c_eq(double a, double b) { return a == b; }
GFM_HD bool c_gt0(double a) { return a > 0.0; }
GFM_HD bool c_ge0(double a) { return a >= 0.0; }
GFM_HD bool c_lt0(double a) { return a < 0.0; }
GFM_HD bool c_le0(double a) { return a <= 0.0; }
GFM_HD bool c_isnan(double a) { return a != a; }
GFM_HD bool quotient_ge0(double n, double d) { return n / d >= 0.0; }
#endif
GFM_HD bool c_gt(double a, double b) { return c_lt(b, a); }
GFM_HD bool c_ge(double a, double b) { return c_le(b, a); }


// ---------------------------------------------------------------------------
// Several quotients with one divisor b: a / b correctly rounded from one
// reciprocal (Markstein, IBM J. Res. Dev. 34(1), 1990): with y = RN(1/b),
// q = RN(a y) lies within an ulp of a/b, the remainder r = a - b q is exact
// (one fma), and RN(q + r y) = RN(a/b) while every value stays in the normal
// range -- here |a| and |b| within 2^-500 .. 2^500 (a = +-0 gives q);
// outside it the division itself is used.  Three multiply-adds per quotient
// instead of a division; the same bits as the division
// (tests/compare_bits_check.cpp).
// ---------------------------------------------------------------------------
struct Recip { double b, y; bool fast; };

GFM_HD bool mid_range(double x) {   // 2^-500 <= |x| < 2^500 (exponent field 523 .. 1522)
  const int e = (int)((as_bits(x) >> 52) & 0x7ff);
  return e >= 523 && e < 1523;
}
template <bool ID = true>
GFM_HD Recip recip(double b) {
  Recip r;
  r.b = b;
  r.y = divx<ID>(1.0, b);
  r.fast = mid_range(b);
  return r;
}
GFM_HD double i_rdiv(double a, const Recip& R) {
  if (R.fast && mid_range(a)) {
    const double q = mulx(a, R.y);
    const double rem = fma(-R.b, q, a);
    return fma(rem, R.y, q);
  }
  if (R.fast && (as_bits(a) & GFM_MAG_BITS) == 0) return a * R.y;   // signed zero
  return divx(a, R.b);
}
#if defined(__CUDA_ARCH__)
GFM_HD double rdiv(double a, const Recip& R) { return i_rdiv(a, R); }
#else
GFM_HD double rdiv(double a, const Recip& R) { return a / R.b; }
#endif

// ---------------------------------------------------------------------------
// The elementary functions are arranged for GB300's FP64 pipe, which is the
// bottleneck of every kernel here: explicit fused multiply-adds (fma is
// correctly rounded on the GPU and in C, so host and device agree), and the
// range reduction's rounding, exponent and table index done with integer
// operations on the bit pattern instead of FP64 instructions.
// ---------------------------------------------------------------------------
#define GFM_ROUND_MAGIC 0x1.8p52   // 1.5 * 2^52: x + MAGIC rounds x to an integer

// exp: Tang (ACM TOMS 15(2), 1989) with a 64-entry table.
//   n = round(x 64/ln2) (fma into 1.5*2^52), x = n ln2/64 + r, |r| <= ln2/128
//   exp(x) = 2^(n>>6) * 2^((n&63)/64) * (1 + q(r)),
//   q = r + r^2 (1/2 + r (1/6 + r (1/24 + r (1/120 + r/720))))   (Horner, fma)
// exp(0) == 1 exactly.  11 FP64 instructions for |x| < 704.
GFM_HD double gfm_exp(double x) {
  const int64_t bx = as_bits(x);
  const bool big = ((bx >> 32) & 0x7fffffff) >= 0x40860000;   // |x| >= 704, inf or NaN
  if (big) {
    if (x != x) return x;
    if (x > 709.78) return gfm_inf();
    if (x < -745.2) return 0.0;
  }
  const double t = fma(x, GFM_INV_LN2_64, GFM_ROUND_MAGIC);
  const int k = (int)(uint32_t)as_bits(t);   // n, from the low mantissa bits
  const double kd = t - GFM_ROUND_MAGIC;
  double r = fma(kd, -GFM_LN2_64_HI, x);     // exact: kd * HI is exact
  r = fma(kd, -GFM_LN2_64_LO, r);
  double p = fma(r, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7);
  p = fma(p, r, 0x1.5555555555555p-5);
  p = fma(p, r, 0x1.5555555555555p-3);
  p = fma(p, r, 0.5);
  const double q = fma(mulx(r, r), p, r);
  const double tj = tab_exp2(k & 63);
  const double y = fma(tj, q, tj);
  const int m = k >> 6;   // floor(n / 64)
  if (big && m < -1020) {  // result near or below the normal range: scale in two steps
    const double z = y * from_bits((int64_t)(m + 1023 + 200) << 52);
    return z * from_bits((int64_t)(1023 - 200) << 52);
  }
  return from_bits(as_bits(y) + ((int64_t)m << 52));   // y * 2^m (normal result)
}

// log: Tang (ACM TOMS 16(4), 1990) with a 97-entry table.
//   x = 2^e * m, m in [0.75, 1.5) (so x near 1 has e = 0 and no cancellation)
//   F = 1 + j/128 nearest to m (j = -32..64, ties away from zero, from the
//   mantissa bits);  f = m - F (exact)
//   log(x) = e ln2 + log(F) + log1p(r),  r = f * (1/F),  |r| <= 2^-8 / 0.75
//   log1p(r) - r = r^2 (-1/2 + r (1/3 + r (-1/4 + r (1/5 + r (-1/6 + r/7)))))
// log(1) == 0 exactly.  14 FP64 instructions for normal positive x.
GFM_HD double gfm_log(double x) {
  int64_t b = as_bits(x);
  int e = 0;
  if ((uint64_t)(b - 0x0010000000000000LL) >= (uint64_t)(0x7ff0000000000000LL - 0x0010000000000000LL)) {
    // zero, subnormal, negative, inf or NaN
    if (!(x > 0.0)) return (x == 0.0) ? -gfm_inf() : gfm_nan();
    if (x == gfm_inf()) return x;
    b = as_bits(x * 0x1p54);   // subnormal
    e = -54;
  }
  e += (int)(b >> 52) - 1023;
  const int64_t mant = b & 0x000fffffffffffffLL;
  int j;
  int64_t mbits, fbits;
  if (mant >= (1LL << 51)) {   // 1.mant >= 1.5: m = 1.mant / 2 in [0.75, 1)
    e += 1;
    mbits = mant | 0x3fe0000000000000LL;
    j = (int)((mant + (1LL << 45)) >> 46) - 64;      // round(128 (m - 1))
    fbits = 0x3fe0000000000000LL + ((int64_t)(64 + j) << 46);
  } else {                     // m = 1.mant in [1, 1.5)
    mbits = mant | 0x3ff0000000000000LL;
    j = (int)((mant + (1LL << 44)) >> 45);
    fbits = 0x3ff0000000000000LL + ((int64_t)j << 45);
  }
  const double f = from_bits(mbits) - from_bits(fbits);
  const double r = mulx(f, tab_invf(j + 32));
  double a = fma(r, 0x1.2492492492492p-3, -0x1.5555555555555p-3);
  a = fma(a, r, 0x1.999999999999ap-3);
  a = fma(a, r, -0.25);
  a = fma(a, r, 0x1.5555555555555p-2);
  a = fma(a, r, -0.5);
  const double p = mulx(mulx(r, r), a);
  const double ed = (double)e;
  const double hi = fma(ed, GFM_LN2_HI, tab_logf(j + 32));   // exact product
  const double lo = fma(ed, GFM_LN2_LO, p);
  return hi + (r + lo);
}

// ---------------------------------------------------------------------------
// pow in fixed point on the integer pipes.  A dependent chain of FP64
// instructions costs 64 cycles each on GB300, and exp(y log x) in FP64 is
// about 25 of them; here x^y = 2^(y log2 x) is formed in 32-, 64- and
// 128-bit integer arithmetic with few dependent 64-bit products, and rounded
// once:
//   log2 x = e + log2 m, m in [0.75, 1.5).  Two table reductions:
//   j = round(64 (m - 1)) picks R1 = RI1_j / 2^16 ~ 1/(1 + j/64), then
//   k = round(4096 (m R1 - 1)) picks R2 = RI2_k / 2^24, so that
//   m R1 R2 = 1 + r exactly (|r| < 2^-12.97, formed in integers as r 2^75);
//   ln(1 + r) = r - r^2/2 + r^3/3 - r^4/4 (r^2 from a 64-bit product, the
//   two small terms in 32-bit), times 1/ln2, plus log2(1/R1) + log2(1/R2)
//   (tables), all in Q62.
//   T = y log2 x exactly as a 128-bit product of y's significand and
//   (e 2^62 + log2 m 2^62), scaled to T 2^64 = n 2^64 + f.
//   2^T = 2^n 2^(j/64) 2^(k/4096) 2^g, g < 2^-12: the first two factors
//   from tables (Q63, and 2^(k/4096) - 1 in Q64), 2^g - 1 = u + u^2/2 +
//   u^3/6 + u^4/24 with u = g ln2 (u and u^2 from 64-bit products, the
//   small terms in 32-bit), rounded to nearest even.
// The result is within about 2^-57 of x^y (relative; 0.51 ulp for the
// exponents of the Riemann solver); the same integer operations on the host
// and the device give the same bits.  Tables: gen_tables.py (mpmath).
// ---------------------------------------------------------------------------
struct XLog2 { int e; int64_t f; };   // log2 x = e + f 2^-62

// high 32 bits of 32 x 32-bit products (signed: floor of the product / 2^32)
GFM_HD int32_t xfp_smulhi32(int32_t a, int32_t b) {
#if defined(__CUDA_ARCH__)
  return __mulhi(a, b);
#else
  return (int32_t)(((int64_t)a * b) >> 32);
#endif
}
GFM_HD uint32_t xfp_umulhi32(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}

// log2 of a positive finite x
GFM_HD XLog2 xlog2_fixed(double x) {
  const uint64_t b = (uint64_t)as_bits(x);
  int ex = (int)(b >> 52);
  uint64_t M = b & 0x000fffffffffffffull;
  if (ex == 0) {   // subnormal: normalise the significand
    const int sh = (int)xfp_clz64(M) - 11;
    M <<= sh;
    ex = 1 - sh;
  } else {
    M |= 1ull << 52;
  }
  const int h = (int)((M >> 51) & 1u);            // m >= 1.5: halve it
  const uint64_t mq = h ? M : (M << 1);           // m 2^53, m in [0.75, 1.5)
  const int j = (int)(((int64_t)mq - (1ll << 53) + (1ll << 46)) >> 47);   // -16..32
  const uint64_t R1 = (uint64_t)GFM_XTAB(xlog1_ri, j + 16);
  const uint64_t p1l = mq * R1, p1h = xfp_mulhi(mq, R1);                   // m R1 2^69
  const uint64_t t = p1l + (1ull << 56);
  const int k = (int)((int64_t)(((p1h + (t < p1l ? 1u : 0u)) << 7) | (t >> 57)) - 4096);   // -48..48
  const uint64_t R2 = (uint64_t)GFM_XTAB(xlog2_ri, k + 48);
  const uint64_t p2l = p1l * R2, p2h = xfp_mulhi(p1l, R2) + p1h * R2;     // m R1 R2 2^93
  const int64_t rho = (int64_t)((p2h << 46) | (p2l >> 18));               // r 2^75
  const int64_t s2 = xfp_smulhi(rho, rho);                                 // r^2 2^86
  const int32_t a2 = (int32_t)(s2 >> 30);                                  // r^2 2^56
  const int32_t a1 = (int32_t)(rho >> 32);                                 // r 2^43
  const int32_t a1d3 = xfp_smulhi32(a1, 0x55555556);                       // r/3 2^43
  const int64_t ln1p = rho - (s2 >> 12) + (((int64_t)a2 * a1d3) >> 24) - (((int64_t)a2 * a2) >> 39);   // Q75
  XLog2 L;
  L.e = ex - 1023 + h;
  L.f = GFM_XTAB64(int64_t, xlog1_t, j + 16) + GFM_XTAB64(int64_t, xlog2_t, k + 48) +
        (xfp_smulhi(ln1p, GFM_XLOG_INVLN2) >> 11);
  return L;
}

// 2^(n + f 2^-64), n an integer and f in Q64
GFM_HD double xexp2_fixed(int64_t n, uint64_t f) {
  const int j = (int)(f >> 58), k = (int)((f >> 52) & 63u);
  const uint64_t g76 = (f & 0x000fffffffffffffull) << 12;                 // g 2^76
  const uint64_t u = xfp_mulhi(g76, GFM_XEXP_LN2);                         // g ln2, Q76
  const uint64_t u2 = xfp_mulhi(u, u);                                     // Q88
  const uint32_t b1 = (uint32_t)(u >> 32), b2 = (uint32_t)(u2 >> 32);      // Q44, Q56
  const uint32_t b1d6 = xfp_umulhi32(b1, 0x2aaaaaabu);                     // u/6
  const uint32_t b2d24 = xfp_umulhi32(b2, 0x0aaaaaabu);                    // u^2/24
  const uint64_t q = (u + (u2 >> 13) + (((uint64_t)b1d6 * b2) >> 24) + (((uint64_t)b2d24 * b2) >> 36)) >> 12;   // 2^g - 1, Q64
  const uint64_t E1 = GFM_XTAB64(uint64_t, xexp1_e, j);
  const uint64_t E = E1 + xfp_mulhi(E1, GFM_XTAB64(uint64_t, xexp2_e, k));  // 2^(j/64 + k/4096), Q63
  const uint64_t R = E + xfp_mulhi(E, q);                                   // 2^(f 2^-64), Q63
  uint64_t mant = R >> 11;
  const uint32_t rem = (uint32_t)R & 0x7ffu;
  mant += (rem > 0x400u || (rem == 0x400u && (mant & 1u) != 0u)) ? 1u : 0u;   // [2^52, 2^53]
  const int64_t be = n + 1023;
  if (be >= 1 && be <= 2046) return from_bits((int64_t)(((uint64_t)(be - 1) << 52) + mant));
  if (be > 2046) return gfm_inf();
  if (be < -60) return 0.0;
  // below the normal range: the rounded significand scaled by 2^(n + 600),
  // exactly, then by 2^-600 with one more rounding
  const double s = from_bits((int64_t)(((uint64_t)(be + 599) << 52) + mant));
  return s * from_bits((int64_t)((uint64_t)(1023 - 600) << 52));
}

// 2^(y log2 x) for log2 x = L of a positive finite x and a finite y
GFM_HD double xpow_fixed(const XLog2& L, double y) {
  const uint64_t yb = (uint64_t)as_bits(y);
  int ey = (int)((yb >> 52) & 0x7ffu);
  uint64_t My = yb & 0x000fffffffffffffull;
  if (ey == 0) ey = 1;   // subnormal y (or zero: a zero product below)
  else My |= 1ull << 52;
  // Lambda = e 2^62 + f, signed 128-bit (lh, ll), then its magnitude
  uint64_t ll = (uint64_t)(int64_t)L.e << 62;
  int64_t lh = (int64_t)L.e >> 2;
  const uint64_t s1 = ll + (uint64_t)L.f;
  lh += (L.f < 0 ? -1 : 0) + (s1 < ll ? 1 : 0);
  ll = s1;
  const bool lneg = lh < 0;
  if (lneg) {
    ll = ~ll + 1u;
    lh = (int64_t)(~(uint64_t)lh + (ll == 0u ? 1u : 0u));
  }
  // Pi = My |Lambda| < 2^126; |T| 2^64 = Pi 2^(ey - 1073)
  uint64_t pl = My * ll;
  uint64_t ph = xfp_mulhi(My, ll) + My * (uint64_t)lh;
  if ((pl | ph) == 0u) return 1.0;
  const int bits = ph ? 128 - (int)xfp_clz64(ph) : 64 - (int)xfp_clz64(pl);
  const int sh = ey - 1073;
  const bool neg = lneg != ((yb >> 63) != 0u);
  if (bits + sh > 75) return neg ? 0.0 : gfm_inf();   // |T| >= 2^11
  if (sh > 0) {
    if (sh >= 64) { ph = pl << (sh - 64); pl = 0u; }
    else { ph = (ph << sh) | (pl >> (64 - sh)); pl <<= sh; }
  } else if (sh < 0) {
    const int k = -sh;
    if (k >= 128) { pl = 0u; ph = 0u; }
    else if (k >= 64) { pl = ph >> (k - 64); ph = 0u; }
    else { pl = (pl >> k) | (ph << (64 - k)); ph >>= k; }
  }
  if (neg) {
    pl = ~pl + 1u;
    ph = ~ph + (pl == 0u ? 1u : 0u);
  }
  return xexp2_fixed((int64_t)ph, pl);   // n = floor(T), f = T - n in Q64
}

// x^y for x >= 0 (every use has a positive base; a negative or NaN base
// gives NaN): 1 for y = 0; 0 or inf for x = 0 and x = inf by y's sign; x = 1
// gives 1 exactly.
GFM_HD bool xpow_plain(double x) {   // positive and finite: the fixed-point path
  const int64_t b = as_bits(x);
  return b > 0 && b < GFM_INF_BITS;
}
GFM_HD double gfm_pow(double x, double y) {
  const int64_t xb = as_bits(x), yb = as_bits(y);
  const int64_t xm = xb & GFM_MAG_BITS, ym = yb & GFM_MAG_BITS;
  if (ym == 0) return 1.0;
  if (xm > GFM_INF_BITS || ym > GFM_INF_BITS || (xb < 0 && xm != 0)) return gfm_nan();
  if (xm == 0) return yb > 0 ? 0.0 : gfm_inf();
  if (xm == GFM_INF_BITS) return yb > 0 ? gfm_inf() : 0.0;
  if (ym == GFM_INF_BITS) {
    if (xb == 0x3ff0000000000000LL) return 1.0;
    return ((xb > 0x3ff0000000000000LL) == (yb > 0)) ? gfm_inf() : 0.0;
  }
  return xpow_fixed(xlog2_fixed(x), y);
}

// asin on [-0.5, 0.5] by its Taylor series (28 terms), in Horner form in x^2.
GFM_HD double gfm_asin_small(double x) {
  double s = x * x;
  double acc = tab_asin(27);
  for (int n = 26; n >= 1; n--) acc = fma(s, acc, tab_asin(n));
  return fma(x, s * acc, x);
}

// acos on [-1, 1]: series for |x| <= 0.5, half-angle reduction otherwise.
template <bool ID = true>
GFM_HD double gfm_acos(double x) {
  if (x > 0.5) return 2.0 * gfm_asin_small(sqrtx<ID>((1.0 - x) * 0.5));
  if (x < -0.5) return GFM_PI - 2.0 * gfm_asin_small(sqrtx<ID>((1.0 + x) * 0.5));
  return GFM_PI_2 - gfm_asin_small(x);
}

// ---------------------------------------------------------------------------
// Stiffened-gas EOS: p = (g-1) rho e - g pinf
// ---------------------------------------------------------------------------
GFM_HD double eos_pressure(double g, double pinf, double e, double rho) {
  return mulx(mulx(g - 1.0, rho), e) - mulx(g, pinf);
}
template <bool ID = true>
GFM_HD double eos_specific_ie(double g, double pinf, double p, double rho) {
  return divx<ID>(p + mulx(g, pinf), mulx(g - 1.0, rho));
}
template <bool ID = true>
GFM_HD double eos_soundspeed(double g, double pinf, double p, double rho) {
  return sqrtx<ID>(divx<ID>(g * (p + pinf), rho));
}
// the same with a reciprocal of rho at hand
template <bool ID = true>
GFM_HD double eos_soundspeed_r(double g, double pinf, double p, const Recip& R) {
  return sqrtx<ID>(rdiv(mulx(g, p + pinf), R));
}
template <bool ID = true>
GFM_HD double eos_isentropic_extrapolation(double g, double pinf, double rho1, double p1, double p2) {
  return rho1 * gfm_pow(divx<ID>(p2 + pinf, p1 + pinf), divx<ID>(1.0, g));
}

// ---------------------------------------------------------------------------
// misc:: state algebra (headers/euler_misc.hpp:23-180).  States are 4 doubles:
// conserved U = (rho, rho u, rho v, E), primitive W = (rho, u, v, p).
// ---------------------------------------------------------------------------
struct V4 { double a, b, c, d; };

// euler_misc.hpp:23-29
template <bool ID = true>
GFM_HD double misc_specific_ie(const V4& U) {
  double rho = U.a;
  const Recip R = recip<ID>(rho);
  double u = rdiv(U.b, R);
  double v = rdiv(U.c, R);
  return rdiv(U.d, R) - mulx(0.5, mulx(u, u) + mulx(v, v));
}
// euler_misc.hpp:32-41
template <bool ID = true>
GFM_HD bool is_physical_state(const V4& U) {
  double rho = U.a;
  const Recip R = recip<ID>(rho);
  double u = rdiv(U.b, R);
  double v = rdiv(U.c, R);
  double e = rdiv(U.d, R) - mulx(0.5, mulx(u, u) + mulx(v, v));
  return c_ge0(rho) && c_ge0(e);
}
// is_physical_state without its three divisions when the state is plainly
// physical: rho > 0, E > 0 and 2 E rho >= (1 + 2^-40) ((rho u)^2 + (rho v)^2)
// with 2 E rho a normal number well inside the range put e = E/rho -
// (u^2 + v^2)/2 above zero by far more than the rounding of either form.
template <bool ID = true>
GFM_HD bool is_physical_state_fast(const V4& U) {
  if (c_gt0(U.a) && c_gt0(U.d)) {
    const double lhs = mulx(2.0, mulx(U.d, U.a));
    const double rhs = mulx(mulx(U.b, U.b) + mulx(U.c, U.c), 1.0 + 0x1p-40);
    const int el = (int)(as_bits(lhs) >> 52);
    if (el > 200 && el < 2047 && c_le(rhs, lhs)) return true;
  }
  return is_physical_state<ID>(U);
}
// euler_misc.hpp:44-49
template <bool ID = true>
GFM_HD bool is_physical_primitives(double g, double pinf, const V4& W) {
  double e = eos_specific_ie<ID>(g, pinf, W.d, W.a);
  return c_ge0(e) && c_ge0(W.a);
}
// the same test with e's sign taken from its numerator and denominator
GFM_HD bool is_physical_primitives_fast(double g, double pinf, const V4& W) {
  return quotient_ge0(W.d + mulx(g, pinf), mulx(g - 1.0, W.a)) && c_ge0(W.a);
}
// euler_misc.hpp:52-67
template <bool ID = true>
GFM_HD V4 cons_to_prims(double g, double pinf, const V4& U) {
  double rho = U.a;
  const Recip R = recip<ID>(rho);
  double u = rdiv(U.b, R);
  double v = rdiv(U.c, R);
  double e = rdiv(U.d, R) - mulx(0.5, mulx(u, u) + mulx(v, v));
  double p = eos_pressure(g, pinf, e, rho);
  return V4{rho, u, v, p};
}
// conserved_to_primitives together with is_physical_state of the same state:
// both compute u, v and e with the same operations, done here once.
template <bool ID = true>
GFM_HD V4 cons_to_prims_phys(double g, double pinf, const V4& U, bool* phys, Recip* Rout = nullptr) {
  double rho = U.a;
  const Recip R = recip<ID>(rho);
  if (Rout) *Rout = R;
  double u = rdiv(U.b, R);
  double v = rdiv(U.c, R);
  double e = rdiv(U.d, R) - mulx(0.5, mulx(u, u) + mulx(v, v));
  *phys = c_ge0(rho) && c_ge0(e);
  double p = eos_pressure(g, pinf, e, rho);
  return V4{rho, u, v, p};
}
// primitives_to_conserved given e = specific_ie(p, rho) already computed
// (by is_physical_primitives of the same state)
GFM_HD V4 prims_to_cons_e(const V4& W, double e) {
  double rho = W.a, u = W.b, v = W.c;
  return V4{rho, mulx(rho, u), mulx(rho, v), mulx(rho, e) + mulx(mulx(0.5, rho), mulx(u, u) + mulx(v, v))};
}

// euler_misc.hpp:70-86
template <bool ID = true>
GFM_HD V4 flux_primitive_var(double g, double pinf, const V4& W) {
  double rho = W.a, u = W.b, v = W.c, p = W.d;
  double e = eos_specific_ie<ID>(g, pinf, p, rho);
  double E = mulx(rho, e) + mulx(mulx(0.5, rho), mulx(u, u) + mulx(v, v));
  const double ru = mulx(rho, u);
  return V4{ru, mulx(ru, u) + p, mulx(ru, v), mulx(u, E + p)};
}
// euler_misc.hpp:89-108 (the asserts become a returned flag)
template <bool ID = true>
GFM_HD V4 prims_to_cons(double g, double pinf, const V4& W, bool* ok) {
  double rho = W.a, u = W.b, v = W.c, p = W.d;
  double e = eos_specific_ie<ID>(g, pinf, p, rho);
  if (ok) *ok = c_ge0(rho) && c_ge0(e);
  return V4{rho, mulx(rho, u), mulx(rho, v), mulx(rho, e) + mulx(mulx(0.5, rho), mulx(u, u) + mulx(v, v))};
}

// ---------------------------------------------------------------------------
// Exact Riemann solver for the stiffened gas (Toro ch. 4, p -> p + pinf).
//
// Arithmetic is arranged for GB300, where an FP64 division or square root
// costs about ten multiplies: every gamma-derived constant is computed once
// per material (Gas), every per-side reciprocal once per solve (RSSide), and
// Newton's stopping test is 2|p - p_old| <= TOL (p + p_old + 2 pinf_min) with
// TOL = 1e-7: the pressure function f is increasing and concave with
// |f''/f'| <= 3.5/(p + pinf), so a step that small leaves the new iterate
// within about 2e-14 (relative) of the root.
// ---------------------------------------------------------------------------
#define GFM_RS_TOL 1e-7
#define GFM_RS_MAXIT 60

struct Gas {
  double g, pinf;
  double G1, G2, G3, G4, G5, G6, G7, IG;
  int maxit;   // Newton iteration limit of the exact solves with this material
};

GFM_HD Gas make_gas(double g, double pinf) {
  Gas k;
  k.g = g; k.pinf = pinf;
  k.G1 = (g - 1.0) / (2.0 * g);
  k.G2 = (g + 1.0) / (2.0 * g);
  k.G3 = 2.0 * g / (g - 1.0);
  k.G4 = 2.0 / (g - 1.0);
  k.G5 = 2.0 / (g + 1.0);
  k.G6 = (g - 1.0) / (g + 1.0);
  k.G7 = (g - 1.0) / 2.0;
  k.IG = 1.0 / g;
  k.maxit = GFM_RS_MAXIT;
  return k;
}

struct RSSide {
  double rho, u, p;   // primitive 1D state
  double pb;          // p + pinf
  double c;           // sound speed sqrt(g pb / rho)
  double AK, BK;      // shock constants G5/rho, G6 pb
  double ipb;         // 1 / pb
  double G4c;         // G4 c
  double irc;         // 1 / (rho c)
  double irho;        // 1 / rho when the caller has it (has_irho), else filled in by rs_side_consts
  bool has_irho;
};

// The state itself; the constants that only iteration and wave sampling use
// are filled in by rs_side_consts (skipped when the data hold no waves).
GFM_HD RSSide rs_side(double rho, double u, double p, const Gas& k) {
  RSSide s;
  s.rho = rho; s.u = u; s.p = p;
  s.pb = p + k.pinf;
  s.c = 0.0; s.AK = 0.0; s.BK = 0.0; s.ipb = 0.0; s.G4c = 0.0; s.irc = 0.0;
  s.irho = 0.0; s.has_irho = false;
  return s;
}
// the same with 1/rho already formed (the correctly rounded quotient, as
// rs_side_consts would form it)
GFM_HD RSSide rs_side_r(double rho, double irho, double u, double p, const Gas& k) {
  RSSide s = rs_side(rho, u, p, k);
  s.irho = irho;
  s.has_irho = true;
  return s;
}
// Two divisions and one square root per side (1/rho, 1/pb, c); A = G5/rho and
// 1/(rho c) = c / (g pb) follow by multiplication.
template <bool ID = true>
GFM_HD void rs_side_consts(RSSide& s, const Gas& k) {
  double irho = s.has_irho ? s.irho : divx<ID>(1.0, s.rho);
  s.ipb = divx<ID>(1.0, s.pb);
  s.c = sqrtx<ID>(mulx(mulx(k.g, s.pb), irho));
  s.AK = mulx(k.G5, irho);
  s.BK = mulx(k.G6, s.pb);
  s.G4c = mulx(k.G4, s.c);
  s.irc = mulx(mulx(s.c, s.ipb), k.IG);
}

// Toro's PREFUN: pressure function f_K and its derivative at pressure p.
template <bool ID = true>
GFM_HD void rs_prefun(const RSSide& K, const Gas& k, double p, double* f, double* fd) {
  double pb = p + k.pinf;
  if (c_gt(p, K.p)) {  // shock
    double r = divx<ID>(1.0, pb + K.BK);
    double qrt = sqrtx<ID>(mulx(K.AK, r));
    *f = mulx(p - K.p, qrt);
    *fd = mulx(1.0 - mulx(0.5, mulx(p - K.p, r)), qrt);
  } else {        // rarefaction
    double prat = mulx(pb, K.ipb);
    double pw = gfm_pow(prat, k.G1);
    *f = mulx(K.G4c, pw - 1.0);
    *fd = mulx(K.irc, divx<ID>(pw, prat));
  }
}

// rs_prefun with the two branches' divisions (1/(pb + B) of the shock,
// pw/prat of the rarefaction) issued as one: when lanes of a warp take
// different branches the division runs once for all of them.  Every value
// comes from the same operations as in rs_prefun.
template <bool ID = true>
GFM_HD void rs_prefun_merged(const RSSide& K, const Gas& k, double p, double* f, double* fd) {
  const double pb = p + k.pinf;
  const bool shock = c_gt(p, K.p);
  double pw = 0.0, prat = 1.0;
  if (!shock) {
    prat = mulx(pb, K.ipb);
    pw = gfm_pow(prat, k.G1);
  }
  const double q = divx<ID>(shock ? 1.0 : pw, shock ? pb + K.BK : prat);
  if (shock) {
    const double qrt = sqrtx<ID>(mulx(K.AK, q));
    *f = mulx(p - K.p, qrt);
    *fd = mulx(1.0 - mulx(0.5, mulx(p - K.p, q)), qrt);
  } else {
    *f = mulx(K.G4c, pw - 1.0);
    *fd = mulx(K.irc, q);
  }
}

struct RSStar {
  double p, u;        // P_STAR, S_STAR
  int iters;
  uint32_t status;
  bool trivial;       // equal u and p: no waves, W_L | W_R across the contact
};


// Newton-Raphson on p* (Toro's STARPU) from the initial guess p0, then u*
// from the last pressure-function evaluation taken to p* along its tangent.
template <bool ID = true>
GFM_HD RSStar rs_star(const RSSide& L, const Gas& kL, const RSSide& R, const Gas& kR, double p0) {
  RSStar s;
  s.status = ST_OK;
  double udiff = R.u - L.u;
  if (c_le(L.G4c + R.G4c, udiff)) s.status |= ST_VACUUM;
  double pinf_min = c_lt(kL.pinf, kR.pinf) ? kL.pinf : kR.pinf;
  double pbmin = c_lt(L.pb, R.pb) ? L.pb : R.pb;
  double pfl = mulx(1e-6, pbmin) - pinf_min;
  double pold = c_gt(p0, pfl) ? p0 : pfl;
  double fL = 0.0, fLd = 0.0, fR = 0.0, fRd = 0.0;
  double p = pold, dp = 0.0;
  int it = 0;
  // The lower-pressure side is evaluated first: with p between the two side
  // pressures it takes the shock branch and the other side the rarefaction
  // branch, so neighbouring solves (the lanes of a warp) tend to take the
  // same branch in each call.  Each call depends only on its own side, so
  // the values are those of evaluating L then R.
  const bool rfirst = c_lt(R.p, L.p);
  const RSSide A = rfirst ? R : L, B = rfirst ? L : R;
  const Gas kA = rfirst ? kR : kL, kB = rfirst ? kL : kR;
  for (;;) {
    double fA, fAd, fB, fBd;
    rs_prefun_merged<ID>(A, kA, pold, &fA, &fAd);   // lanes of a warp may take different branches
    rs_prefun_merged<ID>(B, kB, pold, &fB, &fBd);
    fL = rfirst ? fB : fA; fLd = rfirst ? fBd : fAd;
    fR = rfirst ? fA : fB; fRd = rfirst ? fAd : fBd;
    p = pold - divx<ID>(fL + fR + udiff, fLd + fRd);
    if (c_lt(p, pfl)) p = pfl;
    it++;
    bool conv = c_le(mulx(2.0, fabs(p - pold)), mulx(GFM_RS_TOL, p + pold + mulx(2.0, pinf_min)));
    dp = p - pold;
    pold = p;
    if (conv) break;
    if (it >= kL.maxit) { s.status |= ST_NEWTON_NO_CONVERGE; break; }
  }
  s.p = p;
  // the pressure functions carried from the last evaluation point to p along
  // their tangents, so u* keeps the accuracy of p*
  s.u = mulx(0.5, L.u + R.u + (fR + mulx(fRd, dp)) - (fL + mulx(fLd, dp)));
  s.iters = it;
  return s;
}

// PVRS guess (Toro eq. 4.47)
GFM_HD double rs_guess_pvrs(const RSSide& L, const RSSide& R) {
  return mulx(0.5, L.p + R.p) - mulx(mulx(mulx(0.125, R.u - L.u), L.rho + R.rho), L.c + R.c);
}

// Two-shock guess (TSRS, Toro eq. 9.42) with the shock constants taken at pg;
// used by the mixed (two-material) solve, whose data hold strong waves.
template <bool ID = true>
GFM_HD double rs_guess_tsrs(const RSSide& L, const Gas& kL, const RSSide& R, const Gas& kR, double pg) {
  const double gL = sqrtx<ID>(divx<ID>(L.AK, pg + kL.pinf + L.BK));
  const double gR = sqrtx<ID>(divx<ID>(R.AK, pg + kR.pinf + R.BK));
  return divx<ID>(gL * L.p + gR * R.p - (R.u - L.u), gL + gR);
}

// Whole solve.  When u and p agree on both sides the data hold at most a
// contact and the exact answer p* = p, u* = u is returned without iterating.
template <bool ID = true>
GFM_HD RSStar rs_solve(RSSide& L, const Gas& kL, RSSide& R, const Gas& kR, bool two_shock = false) {
  if (c_eq(L.u, R.u) && c_eq(L.p, R.p)) {
    RSStar s;
    s.p = L.p;
    s.u = L.u;
    s.iters = 0;
    s.status = ST_OK;
    s.trivial = true;
    return s;
  }
  rs_side_consts<ID>(L, kL);
  rs_side_consts<ID>(R, kR);
  double p0 = rs_guess_pvrs(L, R);
  if (two_shock) {   // at max(PVRS, the Newton floor of rs_star)
    const double pinf_min = c_lt(kL.pinf, kR.pinf) ? kL.pinf : kR.pinf;
    const double pbmin = c_lt(L.pb, R.pb) ? L.pb : R.pb;
    const double pfl = 1e-6 * pbmin - pinf_min;
    p0 = rs_guess_tsrs<ID>(L, kL, R, kR, c_gt(p0, pfl) ? p0 : pfl);
  }
  RSStar s = rs_star<ID>(L, kL, R, kR, p0);
  s.trivial = false;
  return s;
}

// Star density behind the K wave (shock or rarefaction).
template <bool ID = true>
GFM_HD double rs_rho_star(const RSSide& K, const Gas& k, double pstar) {
  double pr = mulx(pstar + k.pinf, K.ipb);
  if (c_gt(pstar, K.p)) return mulx(K.rho, divx<ID>(pr + k.G6, mulx(pr, k.G6) + 1.0));
  return mulx(K.rho, gfm_pow(pr, k.IG));
}

// Toro's SAMPLE at speed S; returns (rho, u, p).
//
// The side K that S falls on (left of the contact: L) is selected first and
// one code path serves both sides, with the sign of each wave speed term taken
// from the side: a warp whose lanes sample different sides issues the FP64
// work once, not once per side.  Every value comes from the same operations
// as Toro's four branches (a - b is formed as a + (-b), which is the same
// IEEE operation), and a rarefaction's star density shares the fixed-point
// log2 of (p* + pinf)/(p_K + pinf) with the tail speed (the same values as
// two gfm_pow calls).
struct RS1D { double rho, u, p; };
template <bool ID = true>
GFM_HD RS1D rs_sample(const RSSide& L, const Gas& kL, const RSSide& R, const Gas& kR, const RSStar& st,
                      double S) {
  RS1D w;
  if (st.trivial) {
    if (c_le(S, st.u)) { w.rho = L.rho; w.u = L.u; w.p = L.p; }
    else { w.rho = R.rho; w.u = R.u; w.p = R.p; }
    return w;
  }
  const bool left = c_le(S, st.u);
  const double Krho = left ? L.rho : R.rho, Ku = left ? L.u : R.u, Kp = left ? L.p : R.p;
  const double Kpb = left ? L.pb : R.pb, Kc = left ? L.c : R.c, Kipb = left ? L.ipb : R.ipb;
  const double pinf = left ? kL.pinf : kR.pinf, G1 = left ? kL.G1 : kR.G1, G2 = left ? kL.G2 : kR.G2;
  const double G3 = left ? kL.G3 : kR.G3, G4 = left ? kL.G4 : kR.G4, G5 = left ? kL.G5 : kR.G5;
  const double G6 = left ? kL.G6 : kR.G6, G7 = left ? kL.G7 : kR.G7, IG = left ? kL.IG : kR.IG;
  // left: rarefaction when p* <= p_L; right: shock when p* > p_R
  const bool shock = left ? !c_le(st.p, L.p) : c_gt(st.p, R.p);
  const double pr = mulx(st.p + pinf, Kipb);
  if (shock) {
    const double q = mulx(Kc, sqrtx<ID>(mulx(G2, pr) + G1));
    const double sK = Ku + (left ? -q : q);   // shock speed
    if (left ? c_le(S, sK) : c_ge(S, sK)) { w.rho = Krho; w.u = Ku; w.p = Kp; return w; }
    // rs_rho_star behind the K wave
    w.rho = c_gt(st.p, Kp) ? mulx(Krho, divx<ID>(pr + G6, mulx(pr, G6) + 1.0)) : mulx(Krho, gfm_pow(pr, IG));
    w.u = st.u; w.p = st.p;
    return w;
  }
  const double hK = Ku + (left ? -Kc : Kc);   // rarefaction head
  if (left ? c_le(S, hK) : c_ge(S, hK)) { w.rho = Krho; w.u = Ku; w.p = Kp; return w; }
  const bool plain = xpow_plain(pr);
  XLog2 lpr;
  if (plain) lpr = xlog2_fixed(pr);
  const double cm = mulx(Kc, plain ? xpow_fixed(lpr, G1) : gfm_pow(pr, G1));
  const double tK = st.u + (left ? -cm : cm);   // rarefaction tail
  if (left ? c_gt(S, tK) : c_le(S, tK)) {
    // rs_rho_star of a rarefaction (p* <= p_K here, or NaN on the right)
    w.rho = mulx(Krho, plain ? xpow_fixed(lpr, IG) : gfm_pow(pr, IG));
    w.u = st.u; w.p = st.p;
    return w;
  }
  // inside the fan
  const double t = mulx(G7, Ku - S);
  const double c = mulx(G5, Kc + (left ? t : -t));
  const double cr = divx<ID>(c, Kc);
  w.rho = mulx(Krho, gfm_pow(cr, G4));
  w.u = mulx(G5, (left ? Kc : -Kc) + mulx(G7, Ku) + S);
  w.p = mulx(Kpb, gfm_pow(cr, G3)) - pinf;
  return w;
}

// pure_RS_exact::solve_RP (sourcecode/pure_RS_exact.cpp:9-73): flux of the
// exact solution at x/t = 0 between conserved states UL and UR, one material,
// in two parts so that a kernel can set aside the faces whose data hold waves
// and solve those together:
//   rs_face_front  the conversions, the 1D states (rho, u_n, p) of both sides
//                  and their tangential velocities; returns rs_solve's
//                  no-wave test (equal u_n and p)
//   rs_face_finish the solve, the sample at x/t = 0 and the flux.
// irhoL, irhoR: the conversions' reciprocals 1/rho, which the solve reuses
struct FaceData { double rhoL, uL, pL, rhoR, uR, pR, utL, utR, irhoL, irhoR; };

template <bool ID = true>
GFM_HD bool rs_face_front(bool paralleltox, const Gas& k, const V4& UL, const V4& UR, uint32_t* status,
                          FaceData& d) {
  bool okL, okR;
  Recip RL, RR;
  V4 Lp = cons_to_prims_phys<ID>(k.g, k.pinf, UL, &okL, &RL);
  V4 Rp = cons_to_prims_phys<ID>(k.g, k.pinf, UR, &okR, &RR);
  if (!okL || !okR) *status |= ST_UNPHYSICAL;
  d.rhoL = Lp.a; d.uL = paralleltox ? Lp.b : Lp.c; d.pL = Lp.d;
  d.rhoR = Rp.a; d.uR = paralleltox ? Rp.b : Rp.c; d.pR = Rp.d;
  d.irhoL = RL.y; d.irhoR = RR.y;
  d.utL = paralleltox ? Lp.c : Lp.b;
  d.utR = paralleltox ? Rp.c : Rp.b;
  return c_eq(d.uL, d.uR) && c_eq(d.pL, d.pR);
}

template <bool ID = true>
GFM_HD V4 rs_face_finish(bool paralleltox, const Gas& k, const FaceData& d, uint32_t* status, int* iters) {
  RSSide L = rs_side_r(d.rhoL, d.irhoL, d.uL, d.pL, k);
  RSSide R = rs_side_r(d.rhoR, d.irhoR, d.uR, d.pR, k);
  RSStar st = rs_solve<ID>(L, k, R, k);
  *status |= st.status;
  *iters += st.iters;
  RS1D w = rs_sample<ID>(L, k, R, k, st, 0.0);
  double ut = c_le0(st.u) ? d.utR : d.utL;
  V4 f = flux_primitive_var<ID>(k.g, k.pinf, V4{w.rho, w.u, ut, w.p});
  if (!paralleltox) { double t = f.b; f.b = f.c; f.c = t; }
  return f;
}

template <bool ID = true>
GFM_HD V4 pure_rs_flux(bool paralleltox, const Gas& k, const V4& UL, const V4& UR, uint32_t* status, int* iters) {
  FaceData d;
  rs_face_front<ID>(paralleltox, k, UL, UR, status, d);
  return rs_face_finish<ID>(paralleltox, k, d, status, iters);
}

// mixed_RS_exact::solve_mixed_RP (sourcecode/mixed_RS_exact.cpp:8-48).
struct MixedStar { double p_star, u_star, rho_star_L, rho_star_R; };
template <bool ID = true>
GFM_HD MixedStar mixed_rs(const Gas& kL, const Gas& kR, const V4& UL, const V4& UR, uint32_t* status, int* iters) {
  bool okL, okR;
  V4 Lp = cons_to_prims_phys<ID>(kL.g, kL.pinf, UL, &okL);
  V4 Rp = cons_to_prims_phys<ID>(kR.g, kR.pinf, UR, &okR);
  if (!okL || !okR) *status |= ST_UNPHYSICAL;
  RSSide L = rs_side(Lp.a, Lp.b, Lp.d, kL);
  RSSide R = rs_side(Rp.a, Rp.b, Rp.d, kR);
  RSStar st = rs_solve<ID>(L, kL, R, kR, true);
  *status |= st.status;
  *iters += st.iters;
  MixedStar m;
  m.p_star = st.p;
  m.u_star = st.u;
  m.rho_star_L = st.trivial ? L.rho : rs_rho_star<ID>(L, kL, st.p);
  m.rho_star_R = st.trivial ? R.rho : rs_rho_star<ID>(R, kR, st.p);
  if (c_isnan(m.p_star)) *status |= ST_NAN;
  return m;
}

// minmod slope, one component (sourcecode/FS_MUSCL.cpp:310-327)
GFM_HD double minmod(double dL, double dR) {
  if (c_gt0(dR)) {
    double m = c_lt(dR, dL) ? dR : dL;  // std::min(dL, dR)
    return c_gt0(m) ? m : 0.0;          // std::max(0.0, m)
  }
  double m = c_lt(dL, dR) ? dR : dL;    // std::max(dL, dR)
  return c_lt0(m) ? m : 0.0;            // std::min(0.0, m)
}

}  // namespace gfm
