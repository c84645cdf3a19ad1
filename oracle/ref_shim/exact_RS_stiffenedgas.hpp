// TEST INFRASTRUCTURE -- stand-in for exact_riemann_solver_stiffenedgas's
// exact_RS_stiffenedgas.hpp (absent from the reference's repository; linked
// from outside it, Makefile:19,24).  The interface the reference's adapters
// use (sourcecode/pure_RS_exact.cpp:29-45, sourcecode/mixed_RS_exact.cpp:
// 33-47): constructor (gammaL, gammaR, pinfL, pinfR), solve_RP and
// sample_solution on blitz arrays (rho, u, p), members P_STAR, S_STAR,
// rho_star_L and rho_star_R.  The solver is the oracle's
// (omath::exact_rs_stiffenedgas, oracle_math.hpp).
//
// The oracle starts the two-material solves of the ghost-fluid methods from
// the two-shock guess and the flux solves from PVRS; the reference's adapter
// classes do not say which solve is which, so the driver (ref_driver.cpp)
// sets ref_shim_mixed_solves around the ghost fill.
#pragma once

#include <blitz/array.h>

#include "../oracle_math.hpp"

inline bool ref_shim_mixed_solves = false;
inline long long ref_shim_newton_iters = 0;
inline bool ref_shim_not_converged = false;

class exact_rs_stiffenedgas {
 public:
  double P_STAR = 0.0, S_STAR = 0.0, rho_star_L = 0.0, rho_star_R = 0.0;

  exact_rs_stiffenedgas(double gammaL, double gammaR, double pinfL, double pinfR)
      : rs_(gammaL, gammaR, pinfL, pinfR) {}

  void solve_RP(const blitz::Array<double, 1>& L, const blitz::Array<double, 1>& R) {
    const double l[3] = {L(0), L(1), L(2)}, r[3] = {R(0), R(1), R(2)};
    rs_.two_shock_guess = ref_shim_mixed_solves;
    rs_.solve_RP(l, r);
    P_STAR = rs_.P_STAR;
    S_STAR = rs_.S_STAR;
    rho_star_L = rs_.rho_star_L;
    rho_star_R = rs_.rho_star_R;
    ref_shim_newton_iters += rs_.iterations;
    if (!rs_.converged) ref_shim_not_converged = true;
  }

  blitz::Array<double, 1> sample_solution(const blitz::Array<double, 1>& L, const blitz::Array<double, 1>& R,
                                          double S) const {
    const double l[3] = {L(0), L(1), L(2)}, r[3] = {R(0), R(1), R(2)};
    double o[3];
    rs_.sample_solution(l, r, S, o);
    blitz::Array<double, 1> out(3);
    out(0) = o[0]; out(1) = o[1]; out(2) = o[2];
    return out;
  }

 private:
  omath::exact_rs_stiffenedgas rs_;
};
