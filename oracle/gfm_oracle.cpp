// TEST INFRASTRUCTURE: the CPU oracle of the two-fluid ghost-fluid Euler step.
//
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may load
// this library, and only as the test reference / CPU baseline.  It is never on the
// product path.
//
// A single-threaded C++ restatement of murraycutforth/PhD-2D-GFM's hot path,
// following the reference's loops, loop bounds, branch structure and quirks
// one for one (file:line cited per function).  Grids are the reference's
// nested std::vector<std::vector<vec4>> indexed grid[i][j] (row i = y).
//
// PARITY UNPINNED: the reference cannot be compiled here (it needs Eigen,
// blitz++, PhD-Common, PhD-Interface-tracking-methods, the exact stiffened-gas
// solver and NLopt, none of which are available), and it ships no golden
// vectors.  The parts it takes from absent dependencies (EOS, exact Riemann
// solver, level set, bilinear interpolation, cell-centre coordinates) are
// restated from published methods in oracle_math.hpp and below.
//
// Arithmetic order is fixed (Eigen expressions are evaluated coefficient by
// coefficient, left to right; the 4x4 quasilinear matrix products as
// sum_k (s A_ik) d_k), and the build uses -ffp-contract=off.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../include/gfm_gb300.h"
#include "oracle_itm.hpp"
#include "oracle_math.hpp"

static_assert(oitm::BC_TRANSMISSIVE == GFM_BC_TRANSMISSIVE && oitm::BC_REFLECTIVE == GFM_BC_REFLECTIVE &&
                  oitm::BC_PERIODIC == GFM_BC_PERIODIC,
              "boundary-condition codes");
using omath::exact_rs_stiffenedgas;
using oitm::vec4type;
using oitm::vec2;
using oitm::grideuler2type;
using oitm::gridVector2dtype;
using oitm::griddoubletype;

namespace {

using oitm::sim_info;
using oitm::apply_BCs_scalar;
using oitm::Levelset;
using oitm::VOFTracker;
namespace vof = oitm::vof;

uint32_t g_status = 0;     // OR of GFM_ST_* raised where the reference asserts
int g_last_realcells[8] = {0};   // realcells1, realcells2 of the last two-fluid step
int64_t g_newton_iters = 0;
int64_t g_mixed_calls = 0, g_mixed_iters = 0;   // mixed solves only
int64_t g_iter_hist[16] = {0};                    // Newton iterations per solve (15 = 15 or more)
static void count_iters(int it) { g_iter_hist[it < 15 ? it : 15]++; }

inline vec4type add(const vec4type& a, const vec4type& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]}; }
inline vec4type sub(const vec4type& a, const vec4type& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]}; }
inline vec4type scale(double s, const vec4type& a) { return {s * a[0], s * a[1], s * a[2], s * a[3]}; }

struct binarySGparams {
  double gamma1, pinf1, gamma2, pinf2;
};

struct BBrange {
  int imin, imax, jmin, jmax;
};

void keep_realcells(const BBrange& a, const BBrange& b) {
  const BBrange* rcs[2] = {&a, &b};
  for (int f = 0; f < 2; f++) {
    g_last_realcells[4 * f] = rcs[f]->imin;
    g_last_realcells[4 * f + 1] = rcs[f]->imax;
    g_last_realcells[4 * f + 2] = rcs[f]->jmin;
    g_last_realcells[4 * f + 3] = rcs[f]->jmax;
  }
}

sim_info make_params(const gfm_grid_desc* d) {
  sim_info p;
  p.Nx = d->Nx; p.Ny = d->Ny; p.numGC = d->numGC;
  p.x0 = d->x0; p.y0 = d->y0; p.dx = d->dx; p.dy = d->dy;
  p.BC_L = d->BC_L; p.BC_R = d->BC_R; p.BC_B = d->BC_B; p.BC_T = d->BC_T;
  return p;
}

// ----------------------------------------------------------------------------
// misc:: (headers/euler_misc.hpp)
// ----------------------------------------------------------------------------
namespace misc {

// euler_misc.hpp:23-29
inline double specific_ie(const vec4type& U) {
  double rho = U[0];
  double u = U[1] / rho;
  double v = U[2] / rho;
  return (U[3] / rho) - 0.5 * (u * u + v * v);
}
// euler_misc.hpp:32-41
inline bool is_physical_state(double, double, const vec4type& U) {
  double rho = U[0];
  double u = U[1] / rho;
  double v = U[2] / rho;
  double e = (U[3] / rho) - 0.5 * (u * u + v * v);
  return rho >= 0.0 && e >= 0.0;
}
// euler_misc.hpp:44-49
inline bool is_physical_primitives(double gamma, double pinf, const vec4type& W) {
  double e = eos::specific_ie(gamma, pinf, W[3], W[0]);
  return e >= 0.0 && W[0] >= 0.0;
}
// euler_misc.hpp:52-67
inline vec4type conserved_to_primitives(double gamma, double pinf, const vec4type& U) {
  double rho = U[0];
  double u = U[1] / rho;
  double v = U[2] / rho;
  double e = (U[3] / rho) - 0.5 * (u * u + v * v);
  double p = eos::pressure(gamma, pinf, e, rho);
  return {rho, u, v, p};
}
// euler_misc.hpp:70-86
inline vec4type flux_primitive_var(double gamma, double pinf, const vec4type& W) {
  double rho = W[0], u = W[1], v = W[2], p = W[3];
  double e = eos::specific_ie(gamma, pinf, p, rho);
  double E = rho * e + 0.5 * rho * (u * u + v * v);
  return {rho * u, rho * u * u + p, rho * u * v, u * (E + p)};
}
// euler_misc.hpp:89-108 (assert -> status bit)
inline vec4type primitives_to_conserved(double gamma, double pinf, const vec4type& W) {
  double rho = W[0], u = W[1], v = W[2], p = W[3];
  double e = eos::specific_ie(gamma, pinf, p, rho);
  if (!(rho >= 0.0) || !(e >= 0.0)) g_status |= GFM_ST_UNPHYSICAL;
  return {rho, rho * u, rho * v, rho * e + 0.5 * rho * (u * u + v * v)};
}

// (s M) d for the sparse quasilinear matrices: row sums left to right over
// the non-zero entries (adding an exact zero never changes a sum's value).
// quasilinear_form_A, euler_misc.hpp:149-163
inline vec4type A_times(double s, double gamma, double pinf, const vec4type& W, const vec4type& d) {
  double rho = W[0], u = W[1], p = W[3];
  double c = eos::soundspeed(gamma, pinf, p, rho);
  double a01 = rho, a13 = 1.0 / rho, a31 = rho * c * c;
  double su = s * u;
  return {su * d[0] + (s * a01) * d[1], su * d[1] + (s * a13) * d[3], su * d[2], (s * a31) * d[1] + su * d[3]};
}
// quasilinear_form_B, euler_misc.hpp:166-180
inline vec4type B_times(double s, double gamma, double pinf, const vec4type& W, const vec4type& d) {
  double rho = W[0], v = W[2], p = W[3];
  double c = eos::soundspeed(gamma, pinf, p, rho);
  double b02 = rho, b23 = 1.0 / rho, b32 = rho * c * c;
  double sv = s * v;
  return {sv * d[0] + (s * b02) * d[2], sv * d[1], sv * d[2] + (s * b23) * d[3], (s * b32) * d[2] + sv * d[3]};
}

}  // namespace misc

// ----------------------------------------------------------------------------
// pure_RS_exact::solve_RP (sourcecode/pure_RS_exact.cpp:9-73)
// ----------------------------------------------------------------------------
void pure_RS_solve_RP(bool paralleltox, double gamma, double pinf, const vec4type& Lstate, const vec4type& Rstate,
                      vec4type& flux) {
  if (!misc::is_physical_state(gamma, pinf, Lstate) || !misc::is_physical_state(gamma, pinf, Rstate))
    g_status |= GFM_ST_UNPHYSICAL;
  vec4type Lprims = misc::conserved_to_primitives(gamma, pinf, Lstate);
  vec4type Rprims = misc::conserved_to_primitives(gamma, pinf, Rstate);
  vec4type soln;
  double Lb[3], Rb[3], sb[3];
  exact_rs_stiffenedgas RS(gamma, gamma, pinf, pinf);
  if (paralleltox) {
    Lb[0] = Lprims[0]; Lb[1] = Lprims[1]; Lb[2] = Lprims[3];
    Rb[0] = Rprims[0]; Rb[1] = Rprims[1]; Rb[2] = Rprims[3];
    RS.solve_RP(Lb, Rb);
    RS.sample_solution(Lb, Rb, 0.0, sb);
    soln = {sb[0], sb[1], RS.S_STAR <= 0.0 ? Rprims[2] : Lprims[2], sb[2]};
    flux = misc::flux_primitive_var(gamma, pinf, soln);
  } else {
    Lb[0] = Lprims[0]; Lb[1] = Lprims[2]; Lb[2] = Lprims[3];
    Rb[0] = Rprims[0]; Rb[1] = Rprims[2]; Rb[2] = Rprims[3];
    RS.solve_RP(Lb, Rb);
    RS.sample_solution(Lb, Rb, 0.0, sb);
    soln = {sb[0], sb[1], RS.S_STAR <= 0.0 ? Rprims[1] : Lprims[1], sb[2]};
    flux = misc::flux_primitive_var(gamma, pinf, soln);
    std::swap(flux[1], flux[2]);
  }
  if (RS.vacuum) g_status |= GFM_ST_VACUUM;
  if (!RS.converged) g_status |= GFM_ST_NEWTON_NO_CONVERGE;
  g_newton_iters += RS.iterations;
  count_iters(RS.iterations);
}

// mixed_RS_exact::solve_mixed_RP (sourcecode/mixed_RS_exact.cpp:8-48)
void mixed_RS_solve(double gammaL, double pinfL, double gammaR, double pinfR, const vec4type& Lstate,
                    const vec4type& Rstate, double& p_star, double& u_star, double& rho_star_L, double& rho_star_R) {
  if (!misc::is_physical_state(gammaL, pinfL, Lstate) || !misc::is_physical_state(gammaR, pinfR, Rstate))
    g_status |= GFM_ST_UNPHYSICAL;
  vec4type Lprims = misc::conserved_to_primitives(gammaL, pinfL, Lstate);
  vec4type Rprims = misc::conserved_to_primitives(gammaR, pinfR, Rstate);
  double Lb[3] = {Lprims[0], Lprims[1], Lprims[3]};
  double Rb[3] = {Rprims[0], Rprims[1], Rprims[3]};
  exact_rs_stiffenedgas RS(gammaL, gammaR, pinfL, pinfR);
  RS.two_shock_guess = true;
  RS.solve_RP(Lb, Rb);
  p_star = RS.P_STAR;
  u_star = RS.S_STAR;
  rho_star_L = RS.rho_star_L;
  rho_star_R = RS.rho_star_R;
  if (RS.vacuum) g_status |= GFM_ST_VACUUM;
  if (!RS.converged) g_status |= GFM_ST_NEWTON_NO_CONVERGE;
  if (p_star != p_star) g_status |= GFM_ST_NAN;
  g_newton_iters += RS.iterations;
  g_mixed_calls += 1;
  count_iters(RS.iterations);
  g_mixed_iters += RS.iterations;
}

// ----------------------------------------------------------------------------
// apply_BCs_euler (headers/euler_bc.hpp:5-103), including its quirk: the right
// boundary negates u when BC_L (not BC_R) is reflective (:51).  Periodic
// follows :7-20; it is defined for Nx == Ny only (the loop bounds there swap
// Nx and Ny), which the library enforces.
// ----------------------------------------------------------------------------
template <typename G>
void apply_BCs_euler(const sim_info& params, G& grid) {
  const int g = params.numGC, Nx = params.Nx, Ny = params.Ny;
  if (params.BC_T == GFM_BC_PERIODIC && params.BC_L == GFM_BC_PERIODIC && params.BC_B == GFM_BC_PERIODIC &&
      params.BC_R == GFM_BC_PERIODIC) {
    for (int i = 0; i < Nx + 2 * g; i++)
      for (int j = 0; j < Ny + 2 * g; j++)
        grid[i][j] = grid[(i - g + Ny) % Ny + g][(j - g + Nx) % Nx + g];
    return;
  }
  for (int i = g; i < Ny + g; i++)
    for (int j = 0; j < g; j++) {
      grid[i][j] = grid[i][2 * g - j - 1];
      if (params.BC_L == GFM_BC_REFLECTIVE) grid[i][j][1] = -grid[i][j][1];
    }
  for (int i = g; i < Ny + g; i++)
    for (int j = 0; j < g; j++) {
      grid[i][j + Nx + g] = grid[i][Nx + g - 1 - j];
      if (params.BC_L == GFM_BC_REFLECTIVE) grid[i][j + Nx + g][1] = -grid[i][j + Nx + g][1];
    }
  for (int j = 0; j < Nx + 2 * g; j++)
    for (int i = 0; i < g; i++) {
      grid[i][j] = grid[2 * g - i - 1][j];
      if (params.BC_B == GFM_BC_REFLECTIVE) grid[i][j][2] = -grid[i][j][2];
    }
  for (int j = 0; j < Nx + 2 * g; j++)
    for (int i = 0; i < g; i++) {
      grid[i + Ny + g][j] = grid[Ny + g - 1 - i][j];
      if (params.BC_T == GFM_BC_REFLECTIVE) grid[i + Ny + g][j][2] = -grid[i + Ny + g][j][2];
    }
}

// ----------------------------------------------------------------------------
// FS_MUSCL::pure_fluid_update (sourcecode/FS_MUSCL.cpp:148-304) and
// minmod_limited_slope (:310-327)
// ----------------------------------------------------------------------------
vec4type minmod_limited_slope(const vec4type& diff_L, const vec4type& diff_R) {
  vec4type slope;
  for (int k = 0; k < 4; k++) {
    if (diff_R[k] > 0.0)
      slope[k] = std::max(0.0, std::min(diff_L[k], diff_R[k]));
    else
      slope[k] = std::min(0.0, std::max(diff_L[k], diff_R[k]));
  }
  return slope;
}

void FS_MUSCL_update(const sim_info& params, double gamma, double pinf, double dt, const BBrange& realcells,
                     grideuler2type& grid, grideuler2type& future_grid) {
  using namespace misc;
  const double dtodx = dt / params.dx;
  const double dtody = dt / params.dy;
  for (int i = realcells.imin; i < realcells.imax; i++)
    for (int j = realcells.jmin; j < realcells.jmax; j++) {
      future_grid[i][j] = grid[i][j];
      if (!is_physical_state(gamma, pinf, grid[i][j])) g_status |= GFM_ST_UNPHYSICAL;
    }
  const double sx = 0.5 * dtodx, sy = 0.5 * dtody;
  for (int i = realcells.imin; i < realcells.imax + 1; i++) {
    for (int j = realcells.jmin; j < realcells.jmax + 1; j++) {
      vec4type W_i_j = conserved_to_primitives(gamma, pinf, grid[i][j]);
      vec4type W_ip_j = conserved_to_primitives(gamma, pinf, grid[i + 1][j]);
      vec4type W_im_j = conserved_to_primitives(gamma, pinf, grid[i - 1][j]);
      vec4type W_imm_j = conserved_to_primitives(gamma, pinf, grid[i - 2][j]);
      vec4type W_i_jp = conserved_to_primitives(gamma, pinf, grid[i][j + 1]);
      vec4type W_i_jm = conserved_to_primitives(gamma, pinf, grid[i][j - 1]);
      vec4type W_i_jmm = conserved_to_primitives(gamma, pinf, grid[i][j - 2]);
      vec4type W_im_jm = conserved_to_primitives(gamma, pinf, grid[i - 1][j - 1]);

      vec4type slope_C_x = minmod_limited_slope(sub(W_i_j, W_i_jm), sub(W_i_jp, W_i_j));
      vec4type slope_C_y = minmod_limited_slope(sub(W_i_j, W_im_j), sub(W_ip_j, W_i_j));
      vec4type slope_L_x = minmod_limited_slope(sub(W_i_jm, W_i_jmm), sub(W_i_j, W_i_jm));
      vec4type slope_L_y = minmod_limited_slope(
          sub(W_i_jm, W_im_jm), sub(conserved_to_primitives(gamma, pinf, grid[i + 1][j - 1]), W_i_jm));
      vec4type slope_B_x = minmod_limited_slope(
          sub(W_im_j, W_im_jm), sub(conserved_to_primitives(gamma, pinf, grid[i - 1][j + 1]), W_im_j));
      vec4type slope_B_y = minmod_limited_slope(sub(W_im_j, W_imm_j), sub(W_i_j, W_im_j));

      vec4type C_BEV_L = sub(W_i_j, scale(0.5, slope_C_x));
      vec4type C_BEV_R = add(W_i_j, scale(0.5, slope_C_x));
      vec4type C_BEV_B = sub(W_i_j, scale(0.5, slope_C_y));
      vec4type C_BEV_T = add(W_i_j, scale(0.5, slope_C_y));
      vec4type B_BEV_L = sub(W_im_j, scale(0.5, slope_B_x));
      vec4type B_BEV_R = add(W_im_j, scale(0.5, slope_B_x));
      vec4type B_BEV_B = sub(W_im_j, scale(0.5, slope_B_y));
      vec4type B_BEV_T = add(W_im_j, scale(0.5, slope_B_y));
      vec4type L_BEV_L = sub(W_i_jm, scale(0.5, slope_L_x));
      vec4type L_BEV_R = add(W_i_jm, scale(0.5, slope_L_x));
      vec4type L_BEV_B = sub(W_i_jm, scale(0.5, slope_L_y));
      vec4type L_BEV_T = add(W_i_jm, scale(0.5, slope_L_y));

      if (!is_physical_primitives(gamma, pinf, C_BEV_L) || !is_physical_primitives(gamma, pinf, C_BEV_R)) {
        C_BEV_L = W_i_j; C_BEV_R = W_i_j;
      }
      if (!is_physical_primitives(gamma, pinf, C_BEV_B) || !is_physical_primitives(gamma, pinf, C_BEV_T)) {
        C_BEV_B = W_i_j; C_BEV_T = W_i_j;
      }
      if (!is_physical_primitives(gamma, pinf, B_BEV_L) || !is_physical_primitives(gamma, pinf, B_BEV_R)) {
        B_BEV_L = W_im_j; B_BEV_R = W_im_j;
      }
      if (!is_physical_primitives(gamma, pinf, B_BEV_B) || !is_physical_primitives(gamma, pinf, B_BEV_T)) {
        B_BEV_B = W_im_j; B_BEV_T = W_im_j;
      }
      if (!is_physical_primitives(gamma, pinf, L_BEV_L) || !is_physical_primitives(gamma, pinf, L_BEV_R)) {
        L_BEV_L = W_i_jm; L_BEV_R = W_i_jm;
      }
      if (!is_physical_primitives(gamma, pinf, L_BEV_B) || !is_physical_primitives(gamma, pinf, L_BEV_T)) {
        L_BEV_B = W_i_jm; L_BEV_T = W_i_jm;
      }

      // C_BEV + 0.5 dt/dx A (L - R) + 0.5 dt/dy B (B - T)   (:258-272)
      vec4type XC = A_times(sx, gamma, pinf, W_i_j, sub(C_BEV_L, C_BEV_R));
      vec4type YC = B_times(sy, gamma, pinf, W_i_j, sub(C_BEV_B, C_BEV_T));
      vec4type XL = A_times(sx, gamma, pinf, W_i_jm, sub(L_BEV_L, L_BEV_R));
      vec4type YL = B_times(sy, gamma, pinf, W_i_jm, sub(L_BEV_B, L_BEV_T));
      vec4type XB = A_times(sx, gamma, pinf, W_im_j, sub(B_BEV_L, B_BEV_R));
      vec4type YB = B_times(sy, gamma, pinf, W_im_j, sub(B_BEV_B, B_BEV_T));
      vec4type C_BEV_L_evolved = add(add(C_BEV_L, XC), YC);
      vec4type C_BEV_B_evolved = add(add(C_BEV_B, XC), YC);
      vec4type L_BEV_R_evolved = add(add(L_BEV_R, XL), YL);
      vec4type B_BEV_T_evolved = add(add(B_BEV_T, XB), YB);

      if (!is_physical_primitives(gamma, pinf, C_BEV_L_evolved) ||
          !is_physical_primitives(gamma, pinf, L_BEV_R_evolved)) {
        C_BEV_L_evolved = W_i_j;
        L_BEV_R_evolved = W_i_jm;
      }
      if (!is_physical_primitives(gamma, pinf, C_BEV_B_evolved) ||
          !is_physical_primitives(gamma, pinf, B_BEV_T_evolved)) {
        C_BEV_B_evolved = W_i_j;
        B_BEV_T_evolved = W_im_j;
      }

      vec4type flux_x, flux_y;
      pure_RS_solve_RP(true, gamma, pinf, primitives_to_conserved(gamma, pinf, L_BEV_R_evolved),
                       primitives_to_conserved(gamma, pinf, C_BEV_L_evolved), flux_x);
      pure_RS_solve_RP(false, gamma, pinf, primitives_to_conserved(gamma, pinf, B_BEV_T_evolved),
                       primitives_to_conserved(gamma, pinf, C_BEV_B_evolved), flux_y);

      future_grid[i][j] = add(future_grid[i][j], add(scale(dtodx, flux_x), scale(dtody, flux_y)));
      future_grid[i][j - 1] = sub(future_grid[i][j - 1], scale(dtodx, flux_x));
      future_grid[i - 1][j] = sub(future_grid[i - 1][j], scale(dtody, flux_y));
    }
  }
  for (int i = realcells.imin; i < realcells.imax; i++)
    for (int j = realcells.jmin; j < realcells.jmax; j++) grid[i][j] = future_grid[i][j];
}

// FS_godunov::pure_fluid_update (sourcecode/FS_godunov.cpp:5-50)
void FS_godunov_update(const sim_info& params, double gamma, double pinf, double dt, const BBrange& realcells,
                       grideuler2type& grid, grideuler2type& future_grid) {
  const double dtodx = dt / params.dx;
  const double dtody = dt / params.dy;
  vec4type flux_x, flux_y;
  for (int i = realcells.imin; i < realcells.imax; i++)
    for (int j = realcells.jmin; j < realcells.jmax; j++) {
      future_grid[i][j] = grid[i][j];
      if (!misc::is_physical_state(gamma, pinf, grid[i][j])) g_status |= GFM_ST_UNPHYSICAL;
    }
  for (int i = realcells.imin; i < realcells.imax + 1; i++)
    for (int j = realcells.jmin; j < realcells.jmax + 1; j++) {
      pure_RS_solve_RP(true, gamma, pinf, grid[i][j - 1], grid[i][j], flux_x);
      pure_RS_solve_RP(false, gamma, pinf, grid[i - 1][j], grid[i][j], flux_y);
      future_grid[i][j] = add(future_grid[i][j], add(scale(dtodx, flux_x), scale(dtody, flux_y)));
      future_grid[i][j - 1] = sub(future_grid[i][j - 1], scale(dtodx, flux_x));
      future_grid[i - 1][j] = sub(future_grid[i - 1][j], scale(dtody, flux_y));
    }
  for (int i = realcells.imin; i < realcells.imax; i++)
    for (int j = realcells.jmin; j < realcells.jmax; j++) grid[i][j] = future_grid[i][j];
}

void FS_update(int fs, const sim_info& params, double gamma, double pinf, double dt, const BBrange& rc,
               grideuler2type& grid, grideuler2type& future_grid) {
  if (fs == GFM_FS_MUSCL)
    FS_MUSCL_update(params, gamma, pinf, dt, rc, grid, future_grid);
  else
    FS_godunov_update(params, gamma, pinf, dt, rc, grid, future_grid);
}

// unit normal with the reference's fallback (e.g. sourcecode/GFM_riemann.cpp:58-68)
inline vec2 unit_normal(const Levelset& ls, int i, int j) {
  vec2 n = ls.get_normal(i, j);
  double nn = std::sqrt(n[0] * n[0] + n[1] * n[1]);
  if (nn < 1e-12) return {1.0, 0.0};
  return {n[0] / nn, n[1] / nn};
}

// grid_bilinear_interpolate (PhD-Common; absent): bilinear in the four cell
// centres surrounding x.
vec4type grid_bilinear_interpolate(const sim_info& params, const grideuler2type& grid, const vec2& x) {
  int i0, j0;
  double a, b;
  oitm::bilinear_cell(params, x, i0, j0, a, b);
  vec4type out;
  for (int k = 0; k < 4; k++)
    out[k] = ((1.0 - a) * (1.0 - b)) * grid[i0][j0][k] + (a * (1.0 - b)) * grid[i0][j0 + 1][k] +
             ((1.0 - a) * b) * grid[i0 + 1][j0][k] + (a * b) * grid[i0 + 1][j0 + 1][k];
  return out;
}

// GFM_base::get_interpolated_mixedRPstates (sourcecode/GFM_base.cpp:4-33)
void get_interpolated_mixedRPstates(const sim_info& params, const grideuler2type& prims1,
                                    const grideuler2type& prims2, const Levelset& ls, int i, int j, double ds,
                                    vec4type& Lprims, vec4type& Rprims) {
  vec2 CC = params.cellcentre_coord(i, j);
  double lsval = ls.get_sdf(i, j);
  vec2 normal = ls.get_normal(i, j);
  double normmag = std::sqrt(normal[0] * normal[0] + normal[1] * normal[1]);
  if (std::fabs(lsval) > ds) lsval = std::copysign(ds, lsval);
  vec2 nh = {normal[0] / normmag, normal[1] / normmag};
  vec2 interfacelocation = {CC[0] - lsval * nh[0], CC[1] - lsval * nh[1]};
  vec2 sampleposL = {interfacelocation[0] + ds * nh[0], interfacelocation[1] + ds * nh[1]};
  vec2 sampleposR = {interfacelocation[0] - ds * nh[0], interfacelocation[1] - ds * nh[1]};
  Lprims = grid_bilinear_interpolate(params, prims2, sampleposL);
  Rprims = grid_bilinear_interpolate(params, prims1, sampleposR);
}

// ----------------------------------------------------------------------------
// extrapolate_vector / extrapolate_vector_mgfm (sourcecode/extrapolate_vector.cpp:5-141, 150-288)
// ----------------------------------------------------------------------------
void extrapolate_vector_impl(const sim_info& params, const Levelset& ls, int N, grideuler2type& grid1,
                             grideuler2type& grid2, bool skip_interfacial) {
  const int g = params.numGC;
  grideuler2type updated_grid1 = grid1, updated_grid2 = grid2;
  const double dt = 0.5 * std::min(params.dx, params.dy);
  for (int num = 0; num < N; num++) {
    grid1 = updated_grid1;
    grid2 = updated_grid2;
    for (int i = g; i < params.Ny + g; i++)
      for (int j = g; j < params.Nx + g; j++) {
        double lsval = ls.get_sdf(i, j);
        vec2 normal = unit_normal(ls, i, j);
        if (skip_interfacial && ls.is_interfacial_cell(i, j)) continue;
        vec4type del_vec_x, del_vec_y;
        if (lsval <= 0.0) {
          del_vec_x = (normal[0] > 0.0) ? sub(grid2[i][j + 1], grid2[i][j]) : sub(grid2[i][j], grid2[i][j - 1]);
          del_vec_y = (normal[1] > 0.0) ? sub(grid2[i + 1][j], grid2[i][j]) : sub(grid2[i][j], grid2[i - 1][j]);
          updated_grid2[i][j] = add(add(grid2[i][j], scale((dt / params.dx) * normal[0], del_vec_x)),
                                    scale((dt / params.dy) * normal[1], del_vec_y));
        } else {
          del_vec_x = (normal[0] > 0.0) ? sub(grid1[i][j], grid1[i][j - 1]) : sub(grid1[i][j + 1], grid1[i][j]);
          del_vec_y = (normal[1] > 0.0) ? sub(grid1[i][j], grid1[i - 1][j]) : sub(grid1[i + 1][j], grid1[i][j]);
          updated_grid1[i][j] = sub(sub(grid1[i][j], scale((dt / params.dx) * normal[0], del_vec_x)),
                                    scale((dt / params.dy) * normal[1], del_vec_y));
        }
      }
    apply_BCs_euler(params, updated_grid1);
    apply_BCs_euler(params, updated_grid2);
  }
  grid1 = updated_grid1;
  grid2 = updated_grid2;
}

// extrapolate_extension_vfield (sourcecode/extrapolate_extension_vfield.cpp:4-122);
// BCs by the vector analogue of the Euler mirror (velocity components copied).
void extrapolate_extension_vfield(const sim_info& params, const Levelset& ls, int N, gridVector2dtype& vel) {
  const int g = params.numGC;
  gridVector2dtype updated = vel;
  const double dt = 0.5 * std::min(params.dx, params.dy);
  for (int num = 0; num < N; num++) {
    vel = updated;
    for (int i = g; i < params.Ny + g; i++)
      for (int j = g; j < params.Nx + g; j++) {
        if (ls.is_interfacial_cell(i, j)) continue;
        double lsval = ls.get_sdf(i, j);
        vec2 n = ls.get_normal(i, j);
        double nn = std::sqrt(n[0] * n[0] + n[1] * n[1]);
        if (!(nn > 1e-12)) continue;
        vec2 normal = {n[0] / nn, n[1] / nn};
        vec2 dvx, dvy;
        if (lsval <= 0.0) {
          for (int k = 0; k < 2; k++) {
            dvx[k] = (normal[0] > 0.0) ? vel[i][j + 1][k] - vel[i][j][k] : vel[i][j][k] - vel[i][j - 1][k];
            dvy[k] = (normal[1] > 0.0) ? vel[i + 1][j][k] - vel[i][j][k] : vel[i][j][k] - vel[i - 1][j][k];
          }
          for (int k = 0; k < 2; k++)
            updated[i][j][k] = (vel[i][j][k] + ((dt / params.dx) * normal[0]) * dvx[k]) +
                               ((dt / params.dy) * normal[1]) * dvy[k];
        } else {
          for (int k = 0; k < 2; k++) {
            dvx[k] = (normal[0] > 0.0) ? vel[i][j][k] - vel[i][j - 1][k] : vel[i][j + 1][k] - vel[i][j][k];
            dvy[k] = (normal[1] > 0.0) ? vel[i][j][k] - vel[i - 1][j][k] : vel[i + 1][j][k] - vel[i][j][k];
          }
          for (int k = 0; k < 2; k++)
            updated[i][j][k] = (vel[i][j][k] - ((dt / params.dx) * normal[0]) * dvx[k]) -
                               ((dt / params.dy) * normal[1]) * dvy[k];
        }
      }
    // vector mirror BCs
    const int Nx = params.Nx, Ny = params.Ny;
    for (int i = g; i < Ny + g; i++)
      for (int j = 0; j < g; j++) {
        updated[i][j] = updated[i][2 * g - j - 1];
        updated[i][j + Nx + g] = updated[i][Nx + g - 1 - j];
      }
    for (int j = 0; j < Nx + 2 * g; j++)
      for (int i = 0; i < g; i++) {
        updated[i][j] = updated[2 * g - i - 1][j];
        updated[i + Ny + g][j] = updated[Ny + g - 1 - i][j];
      }
  }
  vel = updated;
}

// composite velocity field: the real fluid's velocity in every cell
void real_fluid_velocities(const sim_info& params, const Levelset& ls, const grideuler2type& prims1,
                           const grideuler2type& prims2, gridVector2dtype& vel) {
  for (int i = 0; i < params.Ny + 2 * params.numGC; i++)
    for (int j = 0; j < params.Nx + 2 * params.numGC; j++) {
      if (ls.get_sdf(i, j) <= 0.0)
        vel[i][j] = {prims1[i][j][1], prims1[i][j][2]};
      else
        vel[i][j] = {prims2[i][j][1], prims2[i][j][2]};
    }
}

// ----------------------------------------------------------------------------
// GFM variants: set_ghost_states.  Scratch grids are locals (the reference's
// function-static scratch, e.g. sourcecode/GFM_riemann.cpp:20-30, is only a
// reuse of storage).
// ----------------------------------------------------------------------------
struct GFMState {
  gridVector2dtype newvelocities;  // vfield handed to the level set
  int64_t n_interfacial = 0;
};

void gfm_convert_all(const sim_info& params, const binarySGparams& eos, const grideuler2type& grid1,
                     const grideuler2type& grid2, grideuler2type& prims1, grideuler2type& prims2) {
  for (int i = 0; i < params.Ny + 2 * params.numGC; i++)
    for (int j = 0; j < params.Nx + 2 * params.numGC; j++) {
      prims1[i][j] = misc::conserved_to_primitives(eos.gamma1, eos.pinf1, grid1[i][j]);
      prims2[i][j] = misc::conserved_to_primitives(eos.gamma2, eos.pinf2, grid2[i][j]);
    }
}

void gfm_back_to_conserved(const sim_info& params, const binarySGparams& eos, const grideuler2type& prims1,
                           const grideuler2type& prims2, grideuler2type& grid1, grideuler2type& grid2) {
  for (int i = 0; i < params.Ny + 2 * params.numGC; i++)
    for (int j = 0; j < params.Nx + 2 * params.numGC; j++) {
      grid1[i][j] = misc::primitives_to_conserved(eos.gamma1, eos.pinf1, prims1[i][j]);
      grid2[i][j] = misc::primitives_to_conserved(eos.gamma2, eos.pinf2, prims2[i][j]);
    }
}

// The mixed Riemann problem in the interface-normal frame, shared by the
// Riemann, real and modified GFM (e.g. sourcecode/GFM_riemann.cpp:76-122).
struct MRPResult {
  double p_star, u_star, rho_star_L, rho_star_R;
  vec2 u1_tang, u2_tang;
};
MRPResult solve_interface_RP(const binarySGparams& eos, const vec4type& interfaceprims1,
                             const vec4type& interfaceprims2, const vec2& normal) {
  vec2 u1 = {interfaceprims1[1], interfaceprims1[2]};
  vec2 u2 = {interfaceprims2[1], interfaceprims2[2]};
  double u1n = u1[0] * normal[0] + u1[1] * normal[1];
  double u2n = u2[0] * normal[0] + u2[1] * normal[1];
  vec2 u1_normal = {u1n * normal[0], u1n * normal[1]};
  vec2 u2_normal = {u2n * normal[0], u2n * normal[1]};
  MRPResult r;
  r.u1_tang = {u1[0] - u1_normal[0], u1[1] - u1_normal[1]};
  r.u2_tang = {u2[0] - u2_normal[0], u2[1] - u2_normal[1]};
  vec4type Lprims = {interfaceprims1[0], u1n, 0.0, std::max(1e-6, interfaceprims1[3])};
  vec4type Rprims = {interfaceprims2[0], u2n, 0.0, std::max(1e-6, interfaceprims2[3])};
  vec4type Lstate = misc::primitives_to_conserved(eos.gamma1, eos.pinf1, Lprims);
  vec4type Rstate = misc::primitives_to_conserved(eos.gamma2, eos.pinf2, Rprims);
  mixed_RS_solve(eos.gamma1, eos.pinf1, eos.gamma2, eos.pinf2, Lstate, Rstate, r.p_star, r.u_star, r.rho_star_L,
                 r.rho_star_R);
  return r;
}

// GFM_riemann::set_ghost_states (sourcecode/GFM_riemann.cpp:8-188)
void GFM_riemann_set_ghost_states(const sim_info& params, const Levelset& ls, const binarySGparams& eos,
                                  const gfm_method_desc& m, grideuler2type& grid1, grideuler2type& grid2,
                                  GFMState& st) {
  const int g = params.numGC;
  const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
  grideuler2type prims1(nr, std::vector<vec4type>(nc)), prims2(nr, std::vector<vec4type>(nc));
  st.newvelocities.assign(nr, std::vector<vec2>(nc, vec2{0.0, 0.0}));
  const double ds = 1.0 * std::min(params.dx, params.dy);
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      if (!misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j]) ||
          !misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j]))
        g_status |= GFM_ST_UNPHYSICAL;
    }
  gfm_convert_all(params, eos, grid1, grid2, prims1, prims2);
  extrapolate_vector_impl(params, ls, 2, prims1, prims2, false);
  st.n_interfacial = 0;
  for (int i = g; i < params.Ny + g; i++)
    for (int j = g; j < params.Nx + g; j++) {
      if (!ls.is_interfacial_cell(i, j)) continue;
      st.n_interfacial++;
      double lsval = ls.get_sdf(i, j);
      vec2 normal = unit_normal(ls, i, j);
      vec4type interfaceprims1, interfaceprims2;
      get_interpolated_mixedRPstates(params, prims1, prims2, ls, i, j, ds, interfaceprims2, interfaceprims1);
      MRPResult r = solve_interface_RP(eos, interfaceprims1, interfaceprims2, normal);
      vec2 u1_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
      vec2 u2_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
      if (lsval <= 0.0)
        prims1[i][j] = {r.rho_star_L, u1_star[0], u1_star[1], r.p_star};
      else
        prims2[i][j] = {r.rho_star_R, u2_star[0], u2_star[1], r.p_star};
      st.newvelocities[i][j] = {r.u_star * normal[0], r.u_star * normal[1]};
    }
  extrapolate_vector_impl(params, ls, 6, prims1, prims2, false);
  if (m.use_extension_vfield)
    extrapolate_extension_vfield(params, ls, 20, st.newvelocities);
  else
    real_fluid_velocities(params, ls, prims1, prims2, st.newvelocities);
  gfm_back_to_conserved(params, eos, prims1, prims2, grid1, grid2);
}

// GFM_real::set_ghost_states (sourcecode/GFM_real.cpp:8-248)
void GFM_real_set_ghost_states(const sim_info& params, const Levelset& ls, const binarySGparams& eos,
                               const gfm_method_desc& m, grideuler2type& grid1, grideuler2type& grid2,
                               GFMState& st) {
  const int g = params.numGC;
  const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
  grideuler2type prims1(nr, std::vector<vec4type>(nc)), prims2(nr, std::vector<vec4type>(nc));
  st.newvelocities.assign(nr, std::vector<vec2>(nc, vec2{0.0, 0.0}));
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      double lsval = ls.get_sdf(i, j);
      prims1[i][j] = misc::conserved_to_primitives(eos.gamma1, eos.pinf1, grid1[i][j]);
      prims2[i][j] = misc::conserved_to_primitives(eos.gamma2, eos.pinf2, grid2[i][j]);
      bool ok = (lsval <= 0.0) ? misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j])
                               : misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j]);
      if (!ok) g_status |= GFM_ST_UNPHYSICAL;
    }
  st.n_interfacial = 0;
  for (int i = g; i < params.Ny + g; i++)
    for (int j = g; j < params.Nx + g; j++) {
      if (!ls.is_interfacial_cell(i, j)) continue;
      st.n_interfacial++;
      double lsval = ls.get_sdf(i, j);
      vec2 normal = unit_normal(ls, i, j);
      // :77-117 neighbour with opposite phi sign and the closest normal direction
      double mindiff = 1e100;
      int i_opp = -1000, j_opp = -1000;
      for (int xinc = -1; xinc <= 1; xinc++)
        for (int yinc = -1; yinc <= 1; yinc++) {
          double otherlsval = ls.get_sdf(i + yinc, j + xinc);
          if (lsval * otherlsval <= 0.0) {
            vec2 othernormal = unit_normal(ls, i + yinc, j + xinc);
            double dotprod = normal[0] * othernormal[0] + normal[1] * othernormal[1];
            dotprod = std::max(dotprod, -1.0);
            dotprod = std::min(dotprod, 1.0);
            double anglediff = omath::acos(dotprod);
            if (anglediff < mindiff) {
              i_opp = i + yinc;
              j_opp = j + xinc;
              mindiff = anglediff;
            }
          }
        }
      vec4type interfaceprims1, interfaceprims2;
      if (lsval <= 0.0) {
        interfaceprims1 = prims1[i][j];
        interfaceprims2 = prims2[i_opp][j_opp];
      } else {
        interfaceprims2 = prims2[i][j];
        interfaceprims1 = prims1[i_opp][j_opp];
      }
      MRPResult r = solve_interface_RP(eos, interfaceprims1, interfaceprims2, normal);
      vec2 u1_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
      vec2 u2_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
      if (lsval <= 0.0)
        prims1[i][j] = {r.rho_star_L, u1_star[0], u1_star[1], r.p_star};
      else
        prims2[i][j] = {r.rho_star_R, u2_star[0], u2_star[1], r.p_star};
      st.newvelocities[i][j] = {r.u_star * normal[0], r.u_star * normal[1]};
    }
  extrapolate_vector_impl(params, ls, 6, prims1, prims2, false);
  if (m.use_extension_vfield)
    extrapolate_extension_vfield(params, ls, 20, st.newvelocities);
  else
    real_fluid_velocities(params, ls, prims1, prims2, st.newvelocities);
  gfm_back_to_conserved(params, eos, prims1, prims2, grid1, grid2);
}

// GFM_modified::set_ghost_states (sourcecode/GFM_modified.cpp:8-240), with
// its quirk: the grids are rebuilt from new_prims (:234-235), so the
// extrapolation of prims (:202) only reaches the velocity field.
void GFM_modified_set_ghost_states(const sim_info& params, const Levelset& ls, const binarySGparams& eos,
                                   const gfm_method_desc& m, grideuler2type& grid1, grideuler2type& grid2,
                                   GFMState& st) {
  const int g = params.numGC;
  const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
  grideuler2type prims1(nr, std::vector<vec4type>(nc)), prims2(nr, std::vector<vec4type>(nc));
  st.newvelocities.assign(nr, std::vector<vec2>(nc, vec2{0.0, 0.0}));
  const double ds = 1.0 * std::min(params.dx, params.dy);
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      double lsval = ls.get_sdf(i, j);
      prims1[i][j] = misc::conserved_to_primitives(eos.gamma1, eos.pinf1, grid1[i][j]);
      prims2[i][j] = misc::conserved_to_primitives(eos.gamma2, eos.pinf2, grid2[i][j]);
      bool ok = (lsval <= 0.0) ? misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j])
                               : misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j]);
      if (!ok) g_status |= GFM_ST_UNPHYSICAL;
    }
  grideuler2type new_prims1 = prims1, new_prims2 = prims2;
  extrapolate_vector_impl(params, ls, 2, prims1, prims2, false);
  st.n_interfacial = 0;
  for (int i = g; i < params.Ny + g; i++)
    for (int j = g; j < params.Nx + g; j++) {
      double lsval = ls.get_sdf(i, j);
      if (!ls.is_interfacial_cell(i, j)) continue;
      st.n_interfacial++;
      vec2 normal = unit_normal(ls, i, j);
      vec4type interfaceprims1, interfaceprims2;
      get_interpolated_mixedRPstates(params, prims1, prims2, ls, i, j, ds, interfaceprims2, interfaceprims1);
      MRPResult r = solve_interface_RP(eos, interfaceprims1, interfaceprims2, normal);
      vec2 u1_star, u2_star;
      if (m.use_slip_BCs) {
        u1_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
        u2_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
      } else if (lsval <= 0.0) {
        u1_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
        u2_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
      } else {
        u1_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
        u2_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
      }
      if (lsval <= 0.0) {
        new_prims1[i][j][0] = eos::isentropic_extrapolation(eos.gamma1, eos.pinf1, r.rho_star_L, r.p_star,
                                                            prims1[i][j][3]);
        new_prims2[i][j] = {r.rho_star_R, u2_star[0], u2_star[1], r.p_star};
      } else {
        new_prims2[i][j][0] = eos::isentropic_extrapolation(eos.gamma2, eos.pinf2, r.rho_star_R, r.p_star,
                                                            prims2[i][j][3]);
        new_prims1[i][j] = {r.rho_star_L, u1_star[0], u1_star[1], r.p_star};
      }
      st.newvelocities[i][j] = {r.u_star * normal[0], r.u_star * normal[1]};
    }
  extrapolate_vector_impl(params, ls, 6, prims1, prims2, true);
  if (m.use_extension_vfield)
    extrapolate_extension_vfield(params, ls, 20, st.newvelocities);
  else
    real_fluid_velocities(params, ls, prims1, prims2, st.newvelocities);
  gfm_back_to_conserved(params, eos, new_prims1, new_prims2, grid1, grid2);
}

// GFM_original::set_ghost_states (sourcecode/GFM_original.cpp:8-166)
void GFM_original_set_ghost_states(const sim_info& params, const Levelset& ls, const binarySGparams& eos,
                                   const gfm_method_desc& m, grideuler2type& grid1, grideuler2type& grid2,
                                   BBrange& realcells1, BBrange& realcells2, GFMState& st) {
  const int g = params.numGC;
  const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
  grideuler2type prims1(nr, std::vector<vec4type>(nc)), prims2(nr, std::vector<vec4type>(nc));
  st.newvelocities.assign(nr, std::vector<vec2>(nc, vec2{0.0, 0.0}));
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      if (!misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j]) ||
          !misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j]))
        g_status |= GFM_ST_UNPHYSICAL;
    }
  gfm_convert_all(params, eos, grid1, grid2, prims1, prims2);
  realcells1 = {g + params.Ny, g, g + params.Nx, g};
  realcells2 = {g + params.Ny, g, g + params.Nx, g};
  extrapolate_vector_impl(params, ls, 6, prims1, prims2, false);
  st.n_interfacial = 0;
  for (int i = g; i < params.Ny + g; i++)
    for (int j = g; j < params.Nx + g; j++) {
      double lsval = ls.get_sdf(i, j);
      if (ls.is_interfacial_cell(i, j)) st.n_interfacial++;
      if (lsval <= 0.0) {
        if (ls.is_interfacial_cell(i, j)) st.newvelocities[i][j] = {prims1[i][j][1], prims1[i][j][2]};
        double u_new = prims1[i][j][1], v_new = prims1[i][j][2], p_new = prims1[i][j][3];
        double rho_new = eos::isentropic_extrapolation(eos.gamma2, eos.pinf2, prims2[i][j][0], prims2[i][j][3], p_new);
        if (!(rho_new >= 0.0)) g_status |= GFM_ST_UNPHYSICAL;
        prims2[i][j] = {rho_new, u_new, v_new, p_new};
        realcells1.imin = std::min(realcells1.imin, i - 2);
        realcells1.imax = std::max(realcells1.imax, i + 2);
        realcells1.jmin = std::min(realcells1.jmin, j - 2);
        realcells1.jmax = std::max(realcells1.jmax, j + 2);
      } else {
        if (ls.is_interfacial_cell(i, j)) st.newvelocities[i][j] = {prims2[i][j][1], prims2[i][j][2]};
        double u_new = prims2[i][j][1], v_new = prims2[i][j][2], p_new = prims2[i][j][3];
        double rho_new = eos::isentropic_extrapolation(eos.gamma1, eos.pinf1, prims1[i][j][0], prims1[i][j][3], p_new);
        if (!(rho_new >= 0.0)) g_status |= GFM_ST_UNPHYSICAL;
        prims1[i][j] = {rho_new, u_new, v_new, p_new};
        realcells2.imin = std::min(realcells2.imin, i - 2);
        realcells2.imax = std::max(realcells2.imax, i + 2);
        realcells2.jmin = std::min(realcells2.jmin, j - 2);
        realcells2.jmax = std::max(realcells2.jmax, j + 2);
      }
    }
  realcells1.imin = std::max(realcells1.imin, g);
  realcells1.imax = std::min(realcells1.imax, g + params.Ny);
  realcells1.jmin = std::max(realcells1.jmin, g);
  realcells1.jmax = std::min(realcells1.jmax, g + params.Nx);
  realcells2.imin = std::max(realcells2.imin, g);
  realcells2.imax = std::min(realcells2.imax, g + params.Ny);
  realcells2.jmin = std::max(realcells2.jmin, g);
  realcells2.jmax = std::min(realcells2.jmax, g + params.Nx);
  gfm_back_to_conserved(params, eos, prims1, prims2, grid1, grid2);
  if (m.use_extension_vfield)
    extrapolate_extension_vfield(params, ls, 20, st.newvelocities);
  else
    real_fluid_velocities(params, ls, prims1, prims2, st.newvelocities);
}

// GFM_base::get_interpolated_mixedRPstates_VOF (sourcecode/GFM_base.cpp:36-55)
void get_interpolated_mixedRPstates_VOF(const sim_info& params, const grideuler2type& prims1,
                                        const grideuler2type& prims2, const vec2& normal, const vec2& loc,
                                        double ds, vec4type& Lprims, vec4type& Rprims) {
  vec2 sampleposL = {loc[0] + ds * normal[0], loc[1] + ds * normal[1]};
  vec2 sampleposR = {loc[0] - ds * normal[0], loc[1] - ds * normal[1]};
  Lprims = grid_bilinear_interpolate(params, prims2, sampleposL);
  Rprims = grid_bilinear_interpolate(params, prims1, sampleposR);
}

// The flags of the VOF GFMs' mixed-cell loop: every cell within ghostrad of a
// mixed cell gets 1 (z == 0), 2 (z == 1) or 0 (mixed).
void vof_set_flags(const VOFTracker& vof, int i, int j, int ghostrad, std::vector<std::vector<int>>& flag) {
  for (int xinc = -ghostrad; xinc <= ghostrad; xinc++)
    for (int yinc = -ghostrad; yinc <= ghostrad; yinc++) {
      double zz = vof.get_z(i + yinc, j + xinc);
      flag[i + yinc][j + xinc] = (zz == 0.0) ? 1 : (zz == 1.0) ? 2 : 0;
    }
}

// Inverse-distance average of the mixed cells' states (flag 0) within
// ghostrad of real cell (i,j) (e.g. sourcecode/GFM_VOF.cpp:240-262).
vec4type vof_invdist_average(const sim_info& params, const std::vector<std::vector<int>>& flag,
                             const grideuler2type& MRPsoln, int i, int j, int ghostrad) {
  vec2 CC = params.cellcentre_coord(i, j);
  double suminvdist = 0.0;
  vec4type sumprims = {0.0, 0.0, 0.0, 0.0};
  for (int xinc = -ghostrad; xinc <= ghostrad; xinc++)
    for (int yinc = -ghostrad; yinc <= ghostrad; yinc++) {
      if (flag[i + yinc][j + xinc] != 0) continue;
      vec2 thisCC = params.cellcentre_coord(i + yinc, j + xinc);
      double ddx = thisCC[0] - CC[0], ddy = thisCC[1] - CC[1];
      double thisinvdist = 1.0 / std::sqrt(ddx * ddx + ddy * ddy);
      suminvdist += thisinvdist;
      sumprims = add(sumprims, scale(thisinvdist, MRPsoln[i + yinc][j + xinc]));
    }
  return {sumprims[0] / suminvdist, sumprims[1] / suminvdist, sumprims[2] / suminvdist, sumprims[3] / suminvdist};
}

// GFM_VOF::set_ghost_states (sourcecode/GFM_VOF.cpp:8-325)
void GFM_VOF_set_ghost_states(const sim_info& params, const VOFTracker& vof, const binarySGparams& eos,
                              const gfm_method_desc& m, grideuler2type& grid1, grideuler2type& grid2,
                              GFMState& st) {
  const int g = params.numGC;
  const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
  grideuler2type prims1(nr, std::vector<vec4type>(nc)), prims2(nr, std::vector<vec4type>(nc));
  grideuler2type MRPsoln1(nr, std::vector<vec4type>(nc, vec4type{0.0, 0.0, 0.0, 0.0}));
  grideuler2type MRPsoln2 = MRPsoln1;
  std::vector<std::vector<int>> flag(nr, std::vector<int>(nc, -1));
  st.newvelocities.assign(nr, std::vector<vec2>(nc, vec2{0.0, 0.0}));
  const double ds = 1.0 * std::min(params.dx, params.dy);
  const int ghostrad = 3;
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      double z = vof.get_z(i, j);
      prims1[i][j] = misc::conserved_to_primitives(eos.gamma1, eos.pinf1, grid1[i][j]);
      prims2[i][j] = misc::conserved_to_primitives(eos.gamma2, eos.pinf2, grid2[i][j]);
      bool ok = (z >= 0.5) ? misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j])
                           : misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j]);
      if (!ok) g_status |= GFM_ST_UNPHYSICAL;
    }
  st.n_interfacial = 0;
  for (int i = g - ghostrad; i < params.Ny + g + ghostrad; i++)
    for (int j = g - ghostrad; j < params.Nx + g + ghostrad; j++) {
      double z = vof.get_z(i, j);
      if (!(0.0 < z && z < 1.0)) continue;
      st.n_interfacial++;
      vof_set_flags(vof, i, j, ghostrad, flag);
      vec2 normal = vof.get_mixedcell_normal(i, j);
      vec2 loc = vof.get_interfacelocation(i, j);
      vec4type interfaceprims1, interfaceprims2;
      get_interpolated_mixedRPstates_VOF(params, prims1, prims2, normal, loc, ds, interfaceprims2, interfaceprims1);
      MRPResult r = solve_interface_RP(eos, interfaceprims1, interfaceprims2, normal);
      vec2 u1_star, u2_star;
      if (m.use_slip_BCs) {
        u1_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
        u2_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
      } else if (z > 0.5) {
        u1_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
        u2_star = {r.u_star * normal[0] + r.u1_tang[0], r.u_star * normal[1] + r.u1_tang[1]};
      } else {
        u1_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
        u2_star = {r.u_star * normal[0] + r.u2_tang[0], r.u_star * normal[1] + r.u2_tang[1]};
      }
      MRPsoln1[i][j] = {r.rho_star_L, u1_star[0], u1_star[1], r.p_star};
      MRPsoln2[i][j] = {r.rho_star_R, u2_star[0], u2_star[1], r.p_star};
      if (z > 0.5) {
        prims1[i][j][0] = eos::isentropic_extrapolation(eos.gamma1, eos.pinf1, r.rho_star_L, r.p_star, prims1[i][j][3]);
        prims2[i][j] = {r.rho_star_R, u2_star[0], u2_star[1], r.p_star};
      } else {
        prims2[i][j][0] = eos::isentropic_extrapolation(eos.gamma2, eos.pinf2, r.rho_star_R, r.p_star, prims2[i][j][3]);
        prims1[i][j] = {r.rho_star_L, u1_star[0], u1_star[1], r.p_star};
      }
    }
  for (int i = g; i < params.Ny + g; i++)
    for (int j = g; j < params.Nx + g; j++) {
      if (flag[i][j] == 1) prims1[i][j] = vof_invdist_average(params, flag, MRPsoln1, i, j, ghostrad);
      else if (flag[i][j] == 2) prims2[i][j] = vof_invdist_average(params, flag, MRPsoln2, i, j, ghostrad);
    }
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      grid1[i][j] = misc::primitives_to_conserved(eos.gamma1, eos.pinf1, prims1[i][j]);
      grid2[i][j] = misc::primitives_to_conserved(eos.gamma2, eos.pinf2, prims2[i][j]);
      if (!misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j]) ||
          !misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j]))
        g_status |= GFM_ST_UNPHYSICAL;
    }
  apply_BCs_euler(params, grid1);
  apply_BCs_euler(params, grid2);
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      if (vof.get_z(i, j) >= 0.5) st.newvelocities[i][j] = {prims1[i][j][1], prims1[i][j][2]};
      else st.newvelocities[i][j] = {prims2[i][j][1], prims2[i][j][2]};
    }
}

// OGFM_VOF::set_ghost_states (sourcecode/OGFM_VOF.cpp:8-274)
void OGFM_VOF_set_ghost_states(const sim_info& params, const VOFTracker& vof, const binarySGparams& eos,
                               grideuler2type& grid1, grideuler2type& grid2, BBrange& realcells1,
                               BBrange& realcells2, GFMState& st) {
  const int g = params.numGC;
  const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
  grideuler2type prims1(nr, std::vector<vec4type>(nc)), prims2(nr, std::vector<vec4type>(nc));
  grideuler2type MRPsoln1(nr, std::vector<vec4type>(nc, vec4type{0.0, 0.0, 0.0, 0.0}));
  grideuler2type MRPsoln2 = MRPsoln1;
  std::vector<std::vector<int>> flag(nr, std::vector<int>(nc, -1));
  st.newvelocities.assign(nr, std::vector<vec2>(nc, vec2{0.0, 0.0}));
  const double ds = 1.0 * std::min(params.dx, params.dy);
  const int ghostrad = 3;
  realcells1 = {g + params.Ny, g, g + params.Nx, g};
  realcells2 = {g + params.Ny, g, g + params.Nx, g};
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      double z = vof.get_z(i, j);
      prims1[i][j] = misc::conserved_to_primitives(eos.gamma1, eos.pinf1, grid1[i][j]);
      prims2[i][j] = misc::conserved_to_primitives(eos.gamma2, eos.pinf2, grid2[i][j]);
      if (z >= 0.5) {
        if (!misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j])) g_status |= GFM_ST_UNPHYSICAL;
        realcells1.imin = std::min(realcells1.imin, i - 2);
        realcells1.imax = std::max(realcells1.imax, i + 2);
        realcells1.jmin = std::min(realcells1.jmin, j - 2);
        realcells1.jmax = std::max(realcells1.jmax, j + 2);
      } else {
        if (!misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j])) g_status |= GFM_ST_UNPHYSICAL;
        realcells2.imin = std::min(realcells2.imin, i - 2);
        realcells2.imax = std::max(realcells2.imax, i + 2);
        realcells2.jmin = std::min(realcells2.jmin, j - 2);
        realcells2.jmax = std::max(realcells2.jmax, j + 2);
      }
    }
  realcells1.imin = std::max(realcells1.imin, g);
  realcells1.imax = std::min(realcells1.imax, g + params.Ny);
  realcells1.jmin = std::max(realcells1.jmin, g);
  realcells1.jmax = std::min(realcells1.jmax, g + params.Nx);
  realcells2.imin = std::max(realcells2.imin, g);
  realcells2.imax = std::min(realcells2.imax, g + params.Ny);
  realcells2.jmin = std::max(realcells2.jmin, g);
  realcells2.jmax = std::min(realcells2.jmax, g + params.Nx);
  st.n_interfacial = 0;
  for (int i = g - ghostrad; i < params.Ny + g + ghostrad; i++)
    for (int j = g - ghostrad; j < params.Nx + g + ghostrad; j++) {
      double z = vof.get_z(i, j);
      if (0.0 < z && z < 1.0) {
        st.n_interfacial++;
        vof_set_flags(vof, i, j, ghostrad, flag);
        vec2 normal = vof.get_mixedcell_normal(i, j);
        vec2 loc = vof.get_interfacelocation(i, j);
        vec4type interfaceprims1, interfaceprims2;
        get_interpolated_mixedRPstates_VOF(params, prims1, prims2, normal, loc, ds, interfaceprims2,
                                           interfaceprims1);
        MRPsoln1[i][j] = interfaceprims1;
        MRPsoln2[i][j] = interfaceprims2;
        if (z > 0.5) {
          double rho = eos::isentropic_extrapolation(eos.gamma2, eos.pinf2, MRPsoln2[i][j][0], MRPsoln2[i][j][3],
                                                     prims1[i][j][3]);
          prims2[i][j] = {rho, prims1[i][j][1], prims1[i][j][2], prims1[i][j][3]};
        } else {
          double rho = eos::isentropic_extrapolation(eos.gamma1, eos.pinf1, MRPsoln1[i][j][0], MRPsoln1[i][j][3],
                                                     prims2[i][j][3]);
          prims1[i][j] = {rho, prims2[i][j][1], prims2[i][j][2], prims2[i][j][3]};
        }
      }
      if (z >= 0.5) st.newvelocities[i][j] = {prims1[i][j][1], prims1[i][j][2]};
      else st.newvelocities[i][j] = {prims2[i][j][1], prims2[i][j][2]};
    }
  for (int i = g; i < params.Ny + g; i++)
    for (int j = g; j < params.Nx + g; j++) {
      if (flag[i][j] == 1) {
        vec4type s = vof_invdist_average(params, flag, MRPsoln1, i, j, ghostrad);
        double rho = eos::isentropic_extrapolation(eos.gamma1, eos.pinf1, s[0], s[3], prims2[i][j][3]);
        prims1[i][j] = {rho, prims2[i][j][1], prims2[i][j][2], prims2[i][j][3]};
      } else if (flag[i][j] == 2) {
        vec4type s = vof_invdist_average(params, flag, MRPsoln2, i, j, ghostrad);
        double rho = eos::isentropic_extrapolation(eos.gamma2, eos.pinf2, s[0], s[3], prims1[i][j][3]);
        prims2[i][j] = {rho, prims1[i][j][1], prims1[i][j][2], prims1[i][j][3]};
      }
      grid1[i][j] = misc::primitives_to_conserved(eos.gamma1, eos.pinf1, prims1[i][j]);
      grid2[i][j] = misc::primitives_to_conserved(eos.gamma2, eos.pinf2, prims2[i][j]);
      if (!misc::is_physical_state(eos.gamma1, eos.pinf1, grid1[i][j]) ||
          !misc::is_physical_state(eos.gamma2, eos.pinf2, grid2[i][j]))
        g_status |= GFM_ST_UNPHYSICAL;
    }
  apply_BCs_euler(params, grid1);
  apply_BCs_euler(params, grid2);
}

// ----------------------------------------------------------------------------
// compute_dt (sourcecode/sim_twofluid.cpp:108-157, sim_onefluid.cpp:68-91)
// ----------------------------------------------------------------------------
template <class ITM>
double compute_dt_twofluid(double CFL, const sim_info& params, const grideuler2type& grid1,
                           const grideuler2type& grid2, const ITM& ls, const binarySGparams& eos, double T,
                           double t) {
  double maxu = 0.0, maxv = 0.0;
  for (int i = params.numGC; i < params.Ny + params.numGC; i++)
    for (int j = params.numGC; j < params.Nx + params.numGC; j++) {
      double phi = ls.get_sdf(i, j);
      const vec4type& U = (phi < 0.0) ? grid1[i][j] : grid2[i][j];
      double gamma = (phi < 0.0) ? eos.gamma1 : eos.gamma2;
      double pinf = (phi < 0.0) ? eos.pinf1 : eos.pinf2;
      double rho = U[0];
      double e = misc::specific_ie(U);
      double p = eos::pressure(gamma, pinf, e, rho);
      double c = eos::soundspeed(gamma, pinf, p, rho);
      maxu = std::max(maxu, std::fabs(U[1]) / rho + c);
      maxv = std::max(maxv, std::fabs(U[2]) / rho + c);
    }
  double dt = CFL * std::min(params.dx / maxu, params.dy / maxv);
  if (t + dt > T) dt = T - t;
  if (!(dt > 0.0)) g_status |= GFM_ST_DT_NONPOSITIVE;
  return dt;
}

double compute_dt_onefluid(double CFL, const sim_info& params, const grideuler2type& grid, const binarySGparams& eos,
                           double T, double t) {
  double maxu = 0.0, maxv = 0.0;
  for (int i = params.numGC; i < params.Ny + params.numGC; i++)
    for (int j = params.numGC; j < params.Nx + params.numGC; j++) {
      double rho = grid[i][j][0];
      double e = misc::specific_ie(grid[i][j]);
      double p = eos::pressure(eos.gamma1, eos.pinf1, e, rho);
      double c = eos::soundspeed(eos.gamma1, eos.pinf1, p, rho);
      maxu = std::max(maxu, std::fabs(grid[i][j][1]) / rho + c);
      maxv = std::max(maxv, std::fabs(grid[i][j][2]) / rho + c);
    }
  double dt = CFL * std::min(params.dx / maxu, params.dy / maxv);
  if (t + dt > T) dt = T - t;
  return dt;
}

// SoA planes <-> nested grid
grideuler2type from_soa(const sim_info& p, const double* U) {
  const int nr = p.Ny + 2 * p.numGC, nc = p.Nx + 2 * p.numGC;
  const size_t plane = static_cast<size_t>(nr) * nc;
  grideuler2type g(nr, std::vector<vec4type>(nc));
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++)
      for (int k = 0; k < 4; k++) g[i][j][k] = U[k * plane + static_cast<size_t>(i) * nc + j];
  return g;
}
void to_soa(const sim_info& p, const grideuler2type& g, double* U) {
  const int nr = p.Ny + 2 * p.numGC, nc = p.Nx + 2 * p.numGC;
  const size_t plane = static_cast<size_t>(nr) * nc;
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++)
      for (int k = 0; k < 4; k++) U[k * plane + static_cast<size_t>(i) * nc + j] = g[i][j][k];
}
griddoubletype phi_from(const sim_info& p, const double* f) {
  const int nr = p.Ny + 2 * p.numGC, nc = p.Nx + 2 * p.numGC;
  griddoubletype g(nr, std::vector<double>(nc));
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) g[i][j] = f[static_cast<size_t>(i) * nc + j];
  return g;
}
void phi_to(const sim_info& p, const griddoubletype& g, double* f) {
  const int nr = p.Ny + 2 * p.numGC, nc = p.Nx + 2 * p.numGC;
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) f[static_cast<size_t>(i) * nc + j] = g[i][j];
}

}  // namespace

// ============================================================================
// C ABI of the oracle (loaded with ctypes by the tests)
// ============================================================================
// ----------------------------------------------------------------------------
// Initial conditions of the timed workloads, restated here so that the CPU
// baseline needs nothing of the library: the one-fluid circular explosion
// (sourcecode/sim_onefluid.cpp:359-415: primitives blended by the 10x10
// sub-sampled area fraction of the circle) and the two-fluid shock-bubble and
// underwater explosion, built as the reference's set_sim_ICs builds its
// bubble cases (sourcecode/sim_twofluid.cpp:774-859): every padded cell from
// its centre, fluid 1 uniform, fluid 2 with a planar shock, phi = distance
// to the centre - radius; then apply_BCs_euler on the grids.
// ----------------------------------------------------------------------------
// Rankine-Hugoniot state behind a shock of Mach M running into (rho1, p1) at
// rest towards -x
void post_shock_state(double g, double M, double rho1, double p1, double& rho2, double& u2, double& p2) {
  const double M2 = M * M;
  p2 = p1 * (1.0 + 2.0 * g / (g + 1.0) * (M2 - 1.0));
  rho2 = rho1 * ((g + 1.0) * M2 / ((g - 1.0) * M2 + 2.0));
  const double W = M * std::sqrt(g * p1 / rho1);
  u2 = -W * (1.0 - rho1 / rho2);
}

struct BubbleIC {
  vec4type s1, s2_left, s2_right;   // conserved states; fluid 2 splits at x = xsplit
  double xsplit, cx, cy, r;
};

void fill_bubble(const gfm_grid_desc* d, const BubbleIC& b, double* U1, double* U2, double* phi) {
  sim_info params = make_params(d);
  const int nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
  grideuler2type g1(nr, std::vector<vec4type>(nc)), g2 = g1;
  griddoubletype ls(nr, std::vector<double>(nc));
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) {
      const vec2 cc = params.cellcentre_coord(i, j);
      g1[i][j] = b.s1;
      g2[i][j] = (cc[0] < b.xsplit) ? b.s2_left : b.s2_right;
      ls[i][j] = std::sqrt((cc[0] - b.cx) * (cc[0] - b.cx) + (cc[1] - b.cy) * (cc[1] - b.cy)) - b.r;
    }
  apply_BCs_euler(params, g1);
  apply_BCs_euler(params, g2);
  to_soa(params, g1, U1);
  to_soa(params, g2, U2);
  phi_to(params, ls, phi);
}

void base_grid(gfm_grid_desc* d, int Nx, int Ny, int g) {
  std::memset(d, 0, sizeof(*d));
  d->Nx = Nx; d->Ny = Ny; d->numGC = g;
  d->x0 = 0.0; d->y0 = 0.0;
  d->dx = 1.0 / Nx; d->dy = 1.0 / Ny;
  d->BC_L = d->BC_R = d->BC_B = d->BC_T = GFM_BC_TRANSMISSIVE;
  d->gamma1 = 1.4; d->gamma2 = 1.4; d->pinf1 = 0.0; d->pinf2 = 0.0;
}

vec4type p2c(double g, double pinf, double rho, double u, double v, double p) {
  return misc::primitives_to_conserved(g, pinf, vec4type{rho, u, v, p});
}

extern "C" {

uint32_t oracle_status(void) { return g_status; }
void oracle_clear_status(void) {
  g_status = 0; g_newton_iters = 0; g_mixed_calls = 0; g_mixed_iters = 0;
  for (int k = 0; k < 16; k++) g_iter_hist[k] = 0;
}
void oracle_iter_histogram(int64_t* h) { for (int k = 0; k < 16; k++) h[k] = g_iter_hist[k]; }
void oracle_mixed_stats(int64_t* calls, int64_t* iters) { *calls = g_mixed_calls; *iters = g_mixed_iters; }
int64_t oracle_newton_iters(void) { return g_newton_iters; }

double oracle_exp(double x) { return omath::exp(x); }
double oracle_log(double x) { return omath::log(x); }
double oracle_pow(double x, double y) { return omath::pow(x, y); }
double oracle_acos(double x) { return omath::acos(x); }

void oracle_rs_pure_batch(int n, int paralleltox, double gamma, double pinf, const double* UL, const double* UR,
                          double* flux) {
  for (int k = 0; k < n; k++) {
    vec4type L = {UL[4 * k], UL[4 * k + 1], UL[4 * k + 2], UL[4 * k + 3]};
    vec4type R = {UR[4 * k], UR[4 * k + 1], UR[4 * k + 2], UR[4 * k + 3]};
    vec4type f;
    pure_RS_solve_RP(paralleltox != 0, gamma, pinf, L, R, f);
    for (int c = 0; c < 4; c++) flux[4 * k + c] = f[c];
  }
}

void oracle_rs_mixed_batch(int n, double gL, double pinfL, double gR, double pinfR, const double* UL,
                           const double* UR, double* out) {
  for (int k = 0; k < n; k++) {
    vec4type L = {UL[4 * k], UL[4 * k + 1], UL[4 * k + 2], UL[4 * k + 3]};
    vec4type R = {UR[4 * k], UR[4 * k + 1], UR[4 * k + 2], UR[4 * k + 3]};
    mixed_RS_solve(gL, pinfL, gR, pinfR, L, R, out[4 * k], out[4 * k + 1], out[4 * k + 2], out[4 * k + 3]);
  }
}

// One-fluid run (sim_onefluid::run_sim loop, sourcecode/sim_onefluid.cpp:40-54):
// advances U (SoA planes) by nsteps steps or until t >= T.  t and numsteps are
// in/out.  Returns the number of steps taken.
int oracle_onefluid_run(const gfm_grid_desc* d, const gfm_method_desc* m, double* U, int nsteps, double* t,
                        int* numsteps) {
  sim_info params = make_params(d);
  binarySGparams eos = {d->gamma1, d->pinf1, d->gamma2, d->pinf2};
  grideuler2type grid = from_soa(params, U);
  grideuler2type future_grid = grid;
  BBrange realcells = {params.numGC, params.Ny + params.numGC, params.numGC, params.Nx + params.numGC};
  int taken = 0;
  while (*t < m->T && taken < nsteps) {
    double CFL = (*numsteps < 5) ? std::min(m->CFL, 0.2) : m->CFL;
    double dt = compute_dt_onefluid(CFL, params, grid, eos, m->T, *t);
    FS_update(m->fs, params, eos.gamma1, eos.pinf1, dt, realcells, grid, future_grid);
    apply_BCs_euler(params, grid);
    (*numsteps)++;
    *t += dt;
    taken++;
  }
  to_soa(params, grid, U);
  return taken;
}

// Two-fluid run (sim_twofluid::run_sim loop, sourcecode/sim_twofluid.cpp:64-88).
// U1, U2: SoA planes; phi: one plane; vel (optional, 2 planes): the velocity
// field of the last ghost fill.  Returns the number of steps taken.
int oracle_twofluid_run(const gfm_grid_desc* d, const gfm_method_desc* m, double* U1, double* U2, double* phi,
                        int nsteps, double* t, int* numsteps, double* vel, int64_t* n_interfacial) {
  sim_info params = make_params(d);
  binarySGparams eos = {d->gamma1, d->pinf1, d->gamma2, d->pinf2};
  grideuler2type grid1 = from_soa(params, U1), grid2 = from_soa(params, U2);
  grideuler2type future_grid1 = grid1, future_grid2 = grid2;
  if (m->itm == GFM_ITM_VOF) {
    // phi holds the volume fraction z; GFM_VOF or OGFM_VOF
    VOFTracker vof;
    vof.params = params;
    vof.z = phi_from(params, phi);
    vof.steps = *numsteps;
    const int g = params.numGC;
    GFMState st;
    int taken = 0;
    while (*t < m->T && taken < nsteps) {
      BBrange realcells1 = {g, params.Ny + g, g, params.Nx + g};
      BBrange realcells2 = realcells1;
      double CFL = (*numsteps < 5) ? std::min(m->CFL, 0.2) : m->CFL;
      double dt = compute_dt_twofluid(CFL, params, grid1, grid2, vof, eos, m->T, *t);
      if (m->gfm == GFM_OGFM_VOF) OGFM_VOF_set_ghost_states(params, vof, eos, grid1, grid2, realcells1, realcells2, st);
      else GFM_VOF_set_ghost_states(params, vof, eos, *m, grid1, grid2, st);
      FS_update(m->fs, params, eos.gamma1, eos.pinf1, dt, realcells1, grid1, future_grid1);
      FS_update(m->fs, params, eos.gamma2, eos.pinf2, dt, realcells2, grid2, future_grid2);
      keep_realcells(realcells1, realcells2);
      vof.update_interface_coupled(st.newvelocities, dt);
      apply_BCs_euler(params, grid1);
      apply_BCs_euler(params, grid2);
      (*numsteps)++;
      *t += dt;
      taken++;
    }
    to_soa(params, grid1, U1);
    to_soa(params, grid2, U2);
    phi_to(params, vof.z, phi);
    if (vel && !st.newvelocities.empty()) {
      const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
      const size_t plane = static_cast<size_t>(nr) * nc;
      for (int i = 0; i < nr; i++)
        for (int j = 0; j < nc; j++) {
          vel[static_cast<size_t>(i) * nc + j] = st.newvelocities[i][j][0];
          vel[plane + static_cast<size_t>(i) * nc + j] = st.newvelocities[i][j][1];
        }
    }
    if (n_interfacial) *n_interfacial = st.n_interfacial;
    return taken;
  }
  Levelset ls;
  ls.params = params;
  ls.phi = phi_from(params, phi);
  ls.order = m->ls_order;
  ls.reinit_every = m->reinit_every;
  ls.reinit_iters = m->reinit_iters;
  ls.updates = *numsteps;
  const int g = params.numGC;
  GFMState st;
  int taken = 0;
  while (*t < m->T && taken < nsteps) {
    BBrange realcells1 = {g, params.Ny + g, g, params.Nx + g};
    BBrange realcells2 = realcells1;
    double CFL = (*numsteps < 5) ? std::min(m->CFL, 0.2) : m->CFL;
    double dt = compute_dt_twofluid(CFL, params, grid1, grid2, ls, eos, m->T, *t);
    switch (m->gfm) {
      case GFM_RIEMANN: GFM_riemann_set_ghost_states(params, ls, eos, *m, grid1, grid2, st); break;
      case GFM_REAL: GFM_real_set_ghost_states(params, ls, eos, *m, grid1, grid2, st); break;
      case GFM_MODIFIED: GFM_modified_set_ghost_states(params, ls, eos, *m, grid1, grid2, st); break;
      default:
        GFM_original_set_ghost_states(params, ls, eos, *m, grid1, grid2, realcells1, realcells2, st);
        break;
    }
    FS_update(m->fs, params, eos.gamma1, eos.pinf1, dt, realcells1, grid1, future_grid1);
    FS_update(m->fs, params, eos.gamma2, eos.pinf2, dt, realcells2, grid2, future_grid2);
    keep_realcells(realcells1, realcells2);
    ls.update_interface_coupled(st.newvelocities, dt);
    apply_BCs_euler(params, grid1);
    apply_BCs_euler(params, grid2);
    (*numsteps)++;
    *t += dt;
    taken++;
  }
  to_soa(params, grid1, U1);
  to_soa(params, grid2, U2);
  phi_to(params, ls.phi, phi);
  if (vel && !st.newvelocities.empty()) {
    const int nr = params.Ny + 2 * g, nc = params.Nx + 2 * g;
    const size_t plane = static_cast<size_t>(nr) * nc;
    for (int i = 0; i < nr; i++)
      for (int j = 0; j < nc; j++) {
        vel[static_cast<size_t>(i) * nc + j] = st.newvelocities[i][j][0];
        vel[plane + static_cast<size_t>(i) * nc + j] = st.newvelocities[i][j][1];
      }
  }
  if (n_interfacial) *n_interfacial = st.n_interfacial;
  return taken;
}

// realcells1 and realcells2 of the last two-fluid step (imin, imax, jmin, jmax each)
void oracle_last_realcells(int* boxes) {
  for (int q = 0; q < 8; q++) boxes[q] = g_last_realcells[q];
}

// Interfacial-cell mask of phi (Levelset::is_interfacial_cell over real cells).
void oracle_interfacial_mask(const gfm_grid_desc* d, const double* phi, uint8_t* mask) {
  sim_info params = make_params(d);
  Levelset ls;
  ls.params = params;
  ls.phi = phi_from(params, phi);
  const int g = params.numGC, nc = params.Nx + 2 * g;
  for (int i = 0; i < params.Ny + 2 * g; i++)
    for (int j = 0; j < nc; j++) {
      bool inner = i >= g && i < params.Ny + g && j >= g && j < params.Nx + g;
      mask[static_cast<size_t>(i) * nc + j] = inner && ls.is_interfacial_cell(i, j) ? 1 : 0;
    }
}

double oracle_fluid_mass(const gfm_grid_desc* d, double interiorsign, const double* U, const double* phi) {
  sim_info params = make_params(d);
  const int g = params.numGC, nc = params.Nx + 2 * g;
  double total = 0.0;
  for (int i = g; i < params.Ny + g; i++)
    for (int j = g; j < params.Nx + g; j++) {
      double lsval = phi[static_cast<size_t>(i) * nc + j];
      if (interiorsign * lsval > 0.0) total += U[static_cast<size_t>(i) * nc + j] * params.dx * params.dy;
    }
  return total;
}

// Grid description and end time of a timed workload (onefluid
// circularexplosion; twofluid shock_bubble, underwater_explosion_sg);
// -1 for any other name.
int oracle_case_params(const char* sim_type, const char* test_case, int Nx, int Ny, gfm_grid_desc* d, double* T) {
  const std::string st(sim_type), tc(test_case);
  if (st == "onefluid" && tc == "circularexplosion") {
    base_grid(d, Nx, Ny, 2);   // sourcecode/sim_onefluid.cpp:96-146
    d->gamma2 = 0.0;
    d->dx = 2.0 / Nx; d->dy = 2.0 / Ny;
    *T = 0.25;
    return 0;
  }
  if (st != "twofluid") return -1;
  base_grid(d, Nx, Ny, 8);     // sourcecode/sim_twofluid.cpp:336-360
  if (tc == "shock_bubble") {
    // 0.25 x 0.089, light-gas bubble (gamma 1.648) in air, walls top and bottom
    d->gamma1 = 1.648; d->dx = 0.25 / Nx; d->dy = 0.089 / Ny;
    d->BC_T = d->BC_B = GFM_BC_REFLECTIVE;
    *T = 1.0;
    return 0;
  }
  if (tc == "underwater_explosion_sg") {
    // [-1,1]^2, air bubble in stiffened-gas water (gamma 4.4, pinf 6e8)
    d->gamma2 = 4.4; d->pinf2 = 6e8;
    d->x0 = -1.0; d->y0 = -1.0; d->dx = 2.0 / Nx; d->dy = 2.0 / Ny;
    *T = 1.0;
    return 0;
  }
  return -1;
}

// Initial state of a timed workload into SoA planes (U2, phi unused for one fluid).
int oracle_case_init(const char* sim_type, const char* test_case, const gfm_grid_desc* d, double* U1, double* U2,
                     double* phi) {
  const std::string st(sim_type), tc(test_case);
  if (st == "onefluid" && tc == "circularexplosion") {
    sim_info params = make_params(d);
    const int nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
    grideuler2type grid(nr, std::vector<vec4type>(nc));
    const vec4type L = {1.0, 0.0, 0.0, 1.0}, R = {0.125, 0.0, 0.0, 0.1};
    const double cx = 1.0, cy = 1.0, rad = 0.4;
    const int N = 10;
    for (int i = 0; i < nr; i++)
      for (int j = 0; j < nc; j++) {
        const vec2 cc = params.cellcentre_coord(i, j);
        const double delx = params.dx / N, dely = params.dy / N;
        const double blx = cc[0] - 0.5 * params.dx, bly = cc[1] - 0.5 * params.dy;
        int inside = 0;
        for (int a = 0; a < N; a++)
          for (int b = 0; b < N; b++) {
            const double sx = blx + (a + 0.5) * delx - cx, sy = bly + (b + 0.5) * dely - cy;
            if (std::sqrt(sx * sx + sy * sy) <= rad) inside++;
          }
        const double frac = double(inside) / (N * N);
        vec4type W;
        for (int k = 0; k < 4; k++) W[k] = frac * L[k] + (1.0 - frac) * R[k];
        grid[i][j] = misc::primitives_to_conserved(d->gamma1, d->pinf1, W);
      }
    apply_BCs_euler(params, grid);
    to_soa(params, grid, U1);
    return 0;
  }
  if (st != "twofluid") return -1;
  BubbleIC b;
  if (tc == "shock_bubble") {
    double rho2, u2, p2;
    post_shock_state(d->gamma2, 1.22, 1.0, 1e5, rho2, u2, p2);
    b.s1 = p2c(d->gamma1, d->pinf1, 0.182, 0, 0, 1e5);
    b.s2_left = p2c(d->gamma2, d->pinf2, 1.0, 0, 0, 1e5);
    b.s2_right = p2c(d->gamma2, d->pinf2, rho2, u2, 0, p2);
    b.xsplit = 0.225; b.cx = 0.175; b.cy = 0.0445; b.r = 0.025;
  } else if (tc == "underwater_explosion_sg") {
    b.s1 = p2c(d->gamma1, d->pinf1, 1270.0, 0, 0, 8.29e8);
    b.s2_left = b.s2_right = p2c(d->gamma2, d->pinf2, 1000.0, 0, 0, 1e5);
    b.xsplit = INFINITY; b.cx = 0.0; b.cy = 0.0; b.r = 0.2;
  } else {
    return -1;
  }
  fill_bubble(d, b, U1, U2, phi);
  return 0;
}

// The batched workload's shock-bubble family: the 1000 x 400 geometry on any
// grid (width 0.25, square cells, walls top and bottom), bubble of fluid 1
// (gamma_bubble, rho = rho_ratio, p 1e5) of radius radius_frac x height at
// (0.7 width, height / 2), shock of Mach `mach` in air from x = 0.9 width.
int oracle_bubble_case(double mach, double gamma_bubble, double rho_ratio, double radius_frac, int Nx, int Ny,
                       gfm_grid_desc* d, double* T) {
  base_grid(d, Nx, Ny, 8);
  d->dx = 0.25 / Nx; d->dy = d->dx;
  d->BC_B = d->BC_T = GFM_BC_REFLECTIVE;
  d->gamma1 = gamma_bubble;
  *T = 1.0;
  (void)mach; (void)rho_ratio; (void)radius_frac;
  return 0;
}

int oracle_bubble_init(double mach, double gamma_bubble, double rho_ratio, double radius_frac, const gfm_grid_desc* d,
                       double* U1, double* U2, double* phi) {
  (void)gamma_bubble;
  const double W = d->dx * d->Nx, H = d->dy * d->Ny;
  double rho2, u2, p2;
  post_shock_state(d->gamma2, mach, 1.0, 1e5, rho2, u2, p2);
  BubbleIC b;
  b.s1 = p2c(d->gamma1, d->pinf1, rho_ratio, 0, 0, 1e5);
  b.s2_left = p2c(d->gamma2, d->pinf2, 1.0, 0, 0, 1e5);
  b.s2_right = p2c(d->gamma2, d->pinf2, rho2, u2, 0, p2);
  b.xsplit = 0.9 * W; b.cx = 0.7 * W; b.cy = 0.5 * H; b.r = radius_frac * H;
  fill_bubble(d, b, U1, U2, phi);
  return 0;
}

}  // extern "C"
