// TEST INFRASTRUCTURE -- part of the CPU oracle.  Only tests/, the smoke check
// and bench.py's cpu_baseline leg may load it.
//
// Scalar arithmetic of the oracle, written independently of the CUDA kernels
// from the same specification (same operations in the same order, so a
// -ffp-contract=off build agrees bit for bit with --fmad=false kernels):
//   * Tang's table-driven exp and log (ACM TOMS 15(2) 1989, 16(4) 1990) and
//     acos by the asin Taylor series with half-angle reduction, polynomials in
//     Horner form with fused multiply-adds (std::fma is correctly rounded,
//     like the GPU's); pow as 2^(y log2 x) in 32/64/128-bit fixed point (two
//     table reductions of log2 to |r| < 2^-12.97 and the series of ln(1 + r)
//     to r^4 in Q75, the exact 128-bit product y log2 x, exp2 by 2^(j/64)
//     and 2^(k/4096) tables and the series of 2^g - 1 to g^4, one rounding),
//     written here with the compiler's 128-bit integers.  The table data come from the generated
//     gfm_tables.h.
//   * the stiffened-gas EOS that the reference takes from its absent
//     PhD-Common dependency (call sites headers/euler_misc.hpp:46,59,77,96).
//   * exact_rs_stiffenedgas, the absent exact solver called at
//     sourcecode/pure_RS_exact.cpp:29-45 and sourcecode/mixed_RS_exact.cpp:33-47,
//     restated from Toro, "Riemann Solvers and Numerical Methods for Fluid
//     Dynamics", ch. 4 (STARPU, PREFUN, SAMPLE) with p -> p + p_inf.
// Parity with the reference is unpinned for these parts: the reference's own
// implementations are not in its repository.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include "../phd-2d-gfm_gb300/csrc/gfm_tables.h"

namespace omath {

static const double EXP2T[64] = GFM_EXP2_TABLE;
static const double LOGFT[97] = GFM_LOGF_TABLE;
static const double INVFT[97] = GFM_INVF_TABLE;
static const double ASINC[28] = GFM_ASIN_COEFFS;
static const uint32_t XLOG1_RI[49] = GFM_XLOG1_RI;
static const int64_t XLOG1_T[49] = GFM_XLOG1_T;
static const uint32_t XLOG2_RI[97] = GFM_XLOG2_RI;
static const int64_t XLOG2_T[97] = GFM_XLOG2_T;
static const uint64_t XEXP1_E[64] = GFM_XEXP1_E;
static const uint64_t XEXP2_E[64] = GFM_XEXP2_E;

inline int64_t bits_of(double x) { int64_t b; std::memcpy(&b, &x, 8); return b; }
inline double double_of(int64_t b) { double x; std::memcpy(&x, &b, 8); return x; }

// Rounding constant: fma(x, c, 1.5 * 2^52) rounds x c to an integer n that
// sits in the low mantissa bits.
static const double ROUND_MAGIC = 6755399441055744.0;

inline double exp(double x) {
  const uint64_t ax = static_cast<uint64_t>(bits_of(x)) & 0x7fffffffffffffffULL;
  const bool wide = ax >= 0x4086000000000000ULL;  // |x| >= 704 (or inf/NaN)
  if (wide) {
    if (std::isnan(x)) return x;
    if (x > 709.78) return HUGE_VAL;
    if (x < -745.2) return 0.0;
  }
  const double t = std::fma(x, GFM_INV_LN2_64, ROUND_MAGIC);
  const int n = static_cast<int32_t>(static_cast<uint32_t>(bits_of(t) & 0xffffffff));
  const double nd = t - ROUND_MAGIC;
  const double r = std::fma(nd, -GFM_LN2_64_LO, std::fma(nd, -GFM_LN2_64_HI, x));
  // expm1(r) to degree 6, Horner with fma:
  // r + r^2 (1/2 + r (1/6 + r (1/24 + r (1/120 + r/720))))
  const double c6 = 0x1.6c16c16c16c17p-10, c5 = 0x1.1111111111111p-7, c4 = 0x1.5555555555555p-5,
               c3 = 0x1.5555555555555p-3;
  const double h = std::fma(std::fma(std::fma(std::fma(r, c6, c5), r, c4), r, c3), r, 0.5);
  const double q = std::fma(r * r, h, r);
  const double tab = EXP2T[n & 63];
  const double y = std::fma(tab, q, tab);
  const int m = n >> 6;
  if (wide && m < -1020) {
    const double z = y * double_of(static_cast<int64_t>(m + 1023 + 200) << 52);
    return z * double_of(static_cast<int64_t>(1023 - 200) << 52);
  }
  return double_of(bits_of(y) + (static_cast<int64_t>(m) << 52));
}

inline double log(double x) {
  int64_t b = bits_of(x);
  int expo = 0;
  const bool normal_pos = b >= 0x0010000000000000LL && b < 0x7ff0000000000000LL;
  if (!normal_pos) {
    if (!(x > 0.0)) return (x == 0.0) ? -HUGE_VAL : std::nan("");
    if (std::isinf(x)) return x;
    b = bits_of(x * 0x1p54);
    expo = -54;
  }
  expo += static_cast<int>(b >> 52) - 1023;
  const int64_t frac = b & 0x000fffffffffffffLL;
  // mantissa m in [0.75, 1.5) (no cancellation near x = 1); j = round(128 (m - 1)),
  // halves away from zero, and F = 1 + j/128, all from the bits
  int j;
  double m, F;
  if (frac >= (int64_t(1) << 51)) {
    expo += 1;
    m = double_of(frac | 0x3fe0000000000000LL);
    j = static_cast<int>((frac + (int64_t(1) << 45)) >> 46) - 64;
    F = 0.5 + (64 + j) * 0x1p-7;
  } else {
    m = double_of(frac | 0x3ff0000000000000LL);
    j = static_cast<int>((frac + (int64_t(1) << 44)) >> 45);
    F = 1.0 + j * 0x1p-7;
  }
  const double r = (m - F) * INVFT[j + 32];
  // log1p(r) - r to degree 7, Horner with fma
  const double c3 = 0x1.5555555555555p-2, c5 = 0x1.999999999999ap-3, c6 = -0x1.5555555555555p-3,
               c7 = 0x1.2492492492492p-3;
  const double h = std::fma(std::fma(std::fma(std::fma(std::fma(r, c7, c6), r, c5), r, -0.25), r, c3), r, -0.5);
  const double poly = (r * r) * h;
  const double e = static_cast<double>(expo);
  const double hi = std::fma(e, GFM_LN2_HI, LOGFT[j + 32]);
  const double lo = std::fma(e, GFM_LN2_LO, poly);
  return hi + (r + lo);
}

// log2 x * 2^62 for a positive finite x, as a 128-bit integer
inline __int128 log2_q62(double x) {
  const uint64_t b = (uint64_t)bits_of(x);
  int be = (int)(b >> 52);
  uint64_t sig = b & 0x000fffffffffffffULL;
  if (be == 0) {                       // subnormal
    const int s = __builtin_clzll(sig) - 11;
    sig <<= s;
    be = 1 - s;
  } else {
    sig |= 1ULL << 52;
  }
  // m = sig / 2^52 in [1, 2); taken to [0.75, 1.5) with the exponent
  const bool halve = sig >= (3ULL << 51);
  const int64_t m53 = (int64_t)(halve ? sig : sig << 1);   // m 2^53
  const int expo = be - 1023 + (halve ? 1 : 0);
  const int j = (int)((m53 - (1LL << 53) + (1LL << 46)) >> 47);         // round(64 (m - 1))
  const unsigned __int128 P1 = (unsigned __int128)(uint64_t)m53 * XLOG1_RI[j + 16];   // m R1 2^69
  const int k = (int)((P1 + ((unsigned __int128)1 << 56)) >> 57) - 4096;  // round(4096 (m R1 - 1))
  const unsigned __int128 P2 = P1 * XLOG2_RI[k + 48];                     // m R1 R2 2^93
  const int64_t r75 = (int64_t)(uint64_t)(P2 >> 18);                      // (m R1 R2 - 1) 2^75, mod 2^64
  // ln(1 + r) = r - r^2/2 + r^3/3 - r^4/4, Q75; r^3/3 and r^4/4 from the
  // leading 32 bits of r 2^43 and r^2 2^56
  const int64_t r2_86 = (int64_t)(((__int128)r75 * r75) >> 64);
  const int32_t r2_56 = (int32_t)(r2_86 >> 30);
  const int32_t r_43 = (int32_t)(r75 >> 32);
  const int32_t r_43_third = (int32_t)(((int64_t)r_43 * 0x55555556LL) >> 32);
  const int64_t ln1p = r75 - (r2_86 >> 12) + (((int64_t)r2_56 * r_43_third) >> 24) -
                       (((int64_t)r2_56 * r2_56) >> 39);
  const int64_t log2_1p = (int64_t)(((__int128)ln1p * GFM_XLOG_INVLN2) >> 75);   // Q62
  return (__int128)expo * ((__int128)1 << 62) + XLOG1_T[j + 16] + XLOG2_T[k + 48] + log2_1p;
}

// 2^(t 2^-64) for a 128-bit t with |t| < 2^75
inline double exp2_q64(__int128 t) {
  const int64_t n = (int64_t)(t >> 64);
  const uint64_t f = (uint64_t)t;
  const int j = (int)(f >> 58), k = (int)((f >> 52) & 63);
  const uint64_t g76 = (f & 0x000fffffffffffffULL) << 12;                // (f 2^-64 - j/64 - k/4096) 2^76
  const uint64_t u = (uint64_t)(((unsigned __int128)g76 * GFM_XEXP_LN2) >> 64);   // g ln2, Q76
  const uint64_t u2 = (uint64_t)(((unsigned __int128)u * u) >> 64);     // Q88
  const uint32_t u_44 = (uint32_t)(u >> 32), u2_56 = (uint32_t)(u2 >> 32);
  const uint32_t u_sixth = (uint32_t)(((uint64_t)u_44 * 0x2aaaaaabULL) >> 32);
  const uint32_t u2_24th = (uint32_t)(((uint64_t)u2_56 * 0x0aaaaaabULL) >> 32);
  const uint64_t q = (u + (u2 >> 13) + (((uint64_t)u_sixth * u2_56) >> 24) + (((uint64_t)u2_24th * u2_56) >> 36)) >> 12;
  const uint64_t E = XEXP1_E[j] + (uint64_t)(((unsigned __int128)XEXP1_E[j] * XEXP2_E[k]) >> 64);   // Q63
  const uint64_t R = E + (uint64_t)(((unsigned __int128)E * q) >> 64);
  uint64_t mant = R >> 11;
  const uint64_t rem = R & 0x7ff;
  if (rem > 0x400 || (rem == 0x400 && (mant & 1))) mant++;
  const int64_t bexp = n + 1023;
  if (bexp >= 1 && bexp <= 2046) return double_of((int64_t)(((uint64_t)(bexp - 1) << 52) + mant));
  if (bexp > 2046) return HUGE_VAL;
  if (bexp < -60) return 0.0;
  const double s = double_of((int64_t)(((uint64_t)(bexp + 599) << 52) + mant));
  return s * double_of((int64_t)((uint64_t)423 << 52));   // 2^-600
}

// x^y = 2^(y log2 x) for a positive finite x and a finite y
inline double pow_fixed(double x, double y) {
  const __int128 L = log2_q62(x);
  if (y == 0.0 || L == 0) return 1.0;
  const uint64_t yb = (uint64_t)bits_of(y);
  int ey = (int)((yb >> 52) & 0x7ff);
  uint64_t my = yb & 0x000fffffffffffffULL;
  if (ey == 0) ey = 1; else my |= 1ULL << 52;
  const unsigned __int128 mag = (unsigned __int128)(L < 0 ? -L : L) * my;   // |y| |L| 2^(1075 - ey + 62)
  const uint64_t mag_hi = (uint64_t)(mag >> 64), mag_lo = (uint64_t)mag;
  const int nbits = mag_hi ? 128 - __builtin_clzll(mag_hi) : (mag_lo ? 64 - __builtin_clzll(mag_lo) : 0);
  const bool neg = (L < 0) != ((yb >> 63) != 0);
  const int sh = ey - 1073;                                // |T| 2^64 = mag 2^sh
  if (nbits + sh > 75) return neg ? 0.0 : HUGE_VAL;
  unsigned __int128 t = sh >= 0 ? (mag << sh) : (-sh >= 128 ? 0 : (mag >> -sh));
  const __int128 T = neg ? -(__int128)t : (__int128)t;
  return exp2_q64(T);
}

inline double pow(double x, double y) {
  if (y == 0.0) return 1.0;
  if (std::isnan(x) || std::isnan(y) || x < 0.0) return NAN;
  if (x == 0.0) return (y > 0.0) ? 0.0 : HUGE_VAL;
  if (std::isinf(x)) return (y > 0.0) ? HUGE_VAL : 0.0;
  if (std::isinf(y)) {
    if (x == 1.0) return 1.0;
    return ((x > 1.0) == (y > 0.0)) ? HUGE_VAL : 0.0;
  }
  return pow_fixed(x, y);
}

inline double asin_series(double x) {
  const double s = x * x;
  double acc = ASINC[27];
  for (int n = 26; n >= 1; n--) acc = std::fma(s, acc, ASINC[n]);
  return std::fma(x, s * acc, x);
}

inline double acos(double x) {
  if (x > 0.5) return 2.0 * asin_series(std::sqrt((1.0 - x) * 0.5));
  if (x < -0.5) return GFM_PI - 2.0 * asin_series(std::sqrt((1.0 + x) * 0.5));
  return GFM_PI_2 - asin_series(x);
}

}  // namespace omath

// Stiffened-gas equation of state, p = (gamma - 1) rho e - gamma pinf.
namespace eos {
inline double pressure(double gamma, double pinf, double e, double rho) {
  return (gamma - 1.0) * rho * e - gamma * pinf;
}
inline double specific_ie(double gamma, double pinf, double p, double rho) {
  return (p + gamma * pinf) / ((gamma - 1.0) * rho);
}
inline double soundspeed(double gamma, double pinf, double p, double rho) {
  return std::sqrt(gamma * (p + pinf) / rho);
}
inline double isentropic_extrapolation(double gamma, double pinf, double rho1, double p1, double p2) {
  return rho1 * omath::pow((p2 + pinf) / (p1 + pinf), 1.0 / gamma);
}
}  // namespace eos

// The exact stiffened-gas Riemann solver with the interface the reference
// uses: constructor (gammaL, gammaR, pinfL, pinfR), solve_RP(L, R) with
// 1D primitive states (rho, u, p), members P_STAR, S_STAR, rho_star_L,
// rho_star_R, and sample_solution(L, R, S).
//
// Operation order (shared with the kernels): gamma constants
// G1 = (g-1)/(2g), G2 = (g+1)/(2g), G3 = 2g/(g-1), G4 = 2/(g-1), G5 = 2/(g+1),
// G6 = (g-1)/(g+1), G7 = (g-1)/2, IG = 1/g; per side pb = p + pinf,
// 1/rho, 1/pb, c = sqrt(g pb (1/rho)), A = G5 (1/rho), B = G6 pb, G4 c,
// 1/(rho c) = c (1/pb) (1/g);
// Newton stops when 2|p - p_old| <= 1e-7 (p + p_old + 2 min(pinf)): the
// pressure function f is increasing and concave with |f''/f'| <= 3.5/(p+pinf),
// so a step that small leaves the new iterate within about 2e-14 (relative) of
// the root.  Initial guess: PVRS (Toro eq. 4.47); the mixed (two-material)
// solve refines it by the two-shock approximation (TSRS, Toro eq. 9.42) with
// the shock constants taken at max(PVRS, floor).
namespace omath {
class exact_rs_stiffenedgas {
 public:
  struct Gas {
    double g, pinf, G1, G2, G3, G4, G5, G6, G7, IG;
    Gas(double gamma, double pinf_) : g(gamma), pinf(pinf_) {
      G1 = (g - 1.0) / (2.0 * g);
      G2 = (g + 1.0) / (2.0 * g);
      G3 = 2.0 * g / (g - 1.0);
      G4 = 2.0 / (g - 1.0);
      G5 = 2.0 / (g + 1.0);
      G6 = (g - 1.0) / (g + 1.0);
      G7 = (g - 1.0) / 2.0;
      IG = 1.0 / g;
    }
  };
  struct Side {
    double rho, u, p, pb, c, A, B, ipb, G4c, irc;
    Side(const double W[3], const Gas& k) : rho(W[0]), u(W[1]), p(W[2]) {
      pb = p + k.pinf;
      const double irho = 1.0 / rho;
      ipb = 1.0 / pb;
      c = std::sqrt(k.g * pb * irho);
      A = k.G5 * irho;
      B = k.G6 * pb;
      G4c = k.G4 * c;
      irc = c * ipb * k.IG;   // 1/(rho c) = c/(g pb)
    }
  };

  Gas KL, KR;
  double P_STAR = 0.0, S_STAR = 0.0, rho_star_L = 0.0, rho_star_R = 0.0;
  int iterations = 0;
  bool vacuum = false, converged = true, trivial = false;
  bool two_shock_guess = false;   // set for mixed_RS_exact's solves

  exact_rs_stiffenedgas(double gammaL, double gammaR, double pinf_L, double pinf_R)
      : KL(gammaL, pinf_L), KR(gammaR, pinf_R) {}

  static const int MAXIT = 60;

  // Toro's PREFUN for one side.
  static void prefun(double p, const Side& K, const Gas& k, double& f, double& fd) {
    const double pb = p + k.pinf;
    if (p > K.p) {
      const double r = 1.0 / (pb + K.B);
      const double qrt = std::sqrt(K.A * r);
      f = (p - K.p) * qrt;
      fd = (1.0 - 0.5 * ((p - K.p) * r)) * qrt;
    } else {
      const double prat = pb * K.ipb;
      const double pw = omath::pow(prat, k.G1);
      f = K.G4c * (pw - 1.0);
      fd = K.irc * (pw / prat);
    }
  }

  static double star_density(double pstar, const Side& K, const Gas& k) {
    const double pr = (pstar + k.pinf) * K.ipb;
    if (pstar > K.p) return K.rho * ((pr + k.G6) / (pr * k.G6 + 1.0));
    return K.rho * omath::pow(pr, k.IG);
  }

  void solve_RP(const double L[3], const double R[3]) {
    const Side SL(L, KL), SR(R, KR);
    vacuum = false;
    converged = true;
    trivial = SL.u == SR.u && SL.p == SR.p;
    if (trivial) {
      // No pressure or velocity jump: a contact at most; the star states are
      // the data themselves.
      P_STAR = SL.p;
      S_STAR = SL.u;
      iterations = 0;
      rho_star_L = SL.rho;
      rho_star_R = SR.rho;
      return;
    } else {
      const double udiff = SR.u - SL.u;
      if (SL.G4c + SR.G4c <= udiff) vacuum = true;
      const double pinfmin = KL.pinf < KR.pinf ? KL.pinf : KR.pinf;
      const double pbmin = SL.pb < SR.pb ? SL.pb : SR.pb;
      const double pfloor = 1e-6 * pbmin - pinfmin;
      // PVRS initial guess (Toro eq. 4.47)
      const double ppv = 0.5 * (SL.p + SR.p) - 0.125 * (SR.u - SL.u) * (SL.rho + SR.rho) * (SL.c + SR.c);
      double p0 = ppv;
      if (two_shock_guess) {
        const double pg = ppv > pfloor ? ppv : pfloor;
        const double gL = std::sqrt(SL.A / (pg + KL.pinf + SL.B));
        const double gR = std::sqrt(SR.A / (pg + KR.pinf + SR.B));
        p0 = (gL * SL.p + gR * SR.p - (SR.u - SL.u)) / (gL + gR);
      }
      double pold = p0 > pfloor ? p0 : pfloor;
      double fL = 0.0, fLd = 0.0, fR = 0.0, fRd = 0.0, p = pold, dp = 0.0;
      int it = 0;
      while (true) {
        prefun(pold, SL, KL, fL, fLd);
        prefun(pold, SR, KR, fR, fRd);
        p = pold - (fL + fR + udiff) / (fLd + fRd);
        if (p < pfloor) p = pfloor;
        it++;
        const bool conv = 2.0 * std::fabs(p - pold) <= 1e-7 * (p + pold + 2.0 * pinfmin);
        dp = p - pold;
        pold = p;
        if (conv) break;
        if (it >= MAXIT) { converged = false; break; }
      }
      P_STAR = p;
      // pressure functions carried from the last evaluation point to p* along
      // their tangents, so u* keeps the accuracy of p*
      S_STAR = 0.5 * (SL.u + SR.u + (fR + fRd * dp) - (fL + fLd * dp));
      iterations = it;
    }
    rho_star_L = star_density(P_STAR, SL, KL);
    rho_star_R = star_density(P_STAR, SR, KR);
  }

  // Toro's SAMPLE at wave speed S = x/t, after solve_RP.
  void sample_solution(const double L[3], const double R[3], double S, double out[3]) const {
    if (trivial) {
      const double* W = (S <= S_STAR) ? L : R;
      out[0] = W[0]; out[1] = W[1]; out[2] = W[2];
      return;
    }
    const Side SL(L, KL), SR(R, KR);
    if (S <= S_STAR) {
      if (P_STAR <= SL.p) {
        const double shl = SL.u - SL.c;
        if (S <= shl) { out[0] = SL.rho; out[1] = SL.u; out[2] = SL.p; return; }
        const double cml = SL.c * omath::pow((P_STAR + KL.pinf) * SL.ipb, KL.G1);
        const double stl = S_STAR - cml;
        if (S > stl) { out[0] = rho_star_L; out[1] = S_STAR; out[2] = P_STAR; return; }
        const double c = KL.G5 * (SL.c + KL.G7 * (SL.u - S));
        const double cr = c / SL.c;
        out[0] = SL.rho * omath::pow(cr, KL.G4);
        out[1] = KL.G5 * (SL.c + KL.G7 * SL.u + S);
        out[2] = SL.pb * omath::pow(cr, KL.G3) - KL.pinf;
        return;
      }
      const double pml = (P_STAR + KL.pinf) * SL.ipb;
      const double sl = SL.u - SL.c * std::sqrt(KL.G2 * pml + KL.G1);
      if (S <= sl) { out[0] = SL.rho; out[1] = SL.u; out[2] = SL.p; return; }
      out[0] = rho_star_L; out[1] = S_STAR; out[2] = P_STAR;
      return;
    }
    if (P_STAR > SR.p) {
      const double pmr = (P_STAR + KR.pinf) * SR.ipb;
      const double sr = SR.u + SR.c * std::sqrt(KR.G2 * pmr + KR.G1);
      if (S >= sr) { out[0] = SR.rho; out[1] = SR.u; out[2] = SR.p; return; }
      out[0] = rho_star_R; out[1] = S_STAR; out[2] = P_STAR;
      return;
    }
    const double shr = SR.u + SR.c;
    if (S >= shr) { out[0] = SR.rho; out[1] = SR.u; out[2] = SR.p; return; }
    const double cmr = SR.c * omath::pow((P_STAR + KR.pinf) * SR.ipb, KR.G1);
    const double str = S_STAR + cmr;
    if (S <= str) { out[0] = rho_star_R; out[1] = S_STAR; out[2] = P_STAR; return; }
    const double c = KR.G5 * (SR.c - KR.G7 * (SR.u - S));
    const double cr = c / SR.c;
    out[0] = SR.rho * omath::pow(cr, KR.G4);
    out[1] = KR.G5 * (-SR.c + KR.G7 * SR.u + S);
    out[2] = SR.pb * omath::pow(cr, KR.G3) - KR.pinf;
  }
};
}  // namespace omath
