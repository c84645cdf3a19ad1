// TEST INFRASTRUCTURE -- part of the CPU oracle.  Only tests/, the smoke check
// and bench.py's cpu_baseline leg may load it.
//
// The pieces of the time step that the reference takes from libraries absent
// from its repository, defined here once for the oracle (gfm_oracle.cpp) and
// for the stand-in headers under ref_shim/ that let the reference's own
// sources be compiled (build_ref.py):
//   * sim_info::cellcentre_coord (PhD-Common): x0 + (j - numGC + 1/2) dx
//   * the interface field's boundary conditions (mirror copy or wrap)
//   * the level set (PhD-Interface-tracking-methods "Levelset")
//   * the VOF tracker (PhD-Interface-tracking-methods "VOF", settings ITM PYVOF)
//   * the cell and weights of grid_bilinear_interpolate (PhD-Common)
// These are this project's own definitions from published methods; the
// reference's implementations are not in its repository, so parity is
// unpinned for them.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <vector>

namespace oitm {

// boundary-condition codes (the values of GFM_BC_* in include/gfm_gb300.h)
enum { BC_TRANSMISSIVE = 0, BC_REFLECTIVE = 1, BC_PERIODIC = 2 };

typedef std::array<double, 4> vec4type;
typedef std::array<double, 2> vec2;
typedef std::vector<std::vector<vec4type>> grideuler2type;
typedef std::vector<std::vector<vec2>> gridVector2dtype;
typedef std::vector<std::vector<double>> griddoubletype;

// sim_info (PhD-Common): grid geometry, boundary conditions.
struct sim_info {
  int Nx, Ny, numGC;
  double x0, y0, dx, dy;
  int BC_L, BC_R, BC_B, BC_T;
  // cell centre of grid[i][j]
  vec2 cellcentre_coord(int i, int j) const {
    return {x0 + (static_cast<double>(j - numGC) + 0.5) * dx, y0 + (static_cast<double>(i - numGC) + 0.5) * dy};
  }
};

// Scalar-field BCs for phi (the level set's own boundary handling, which the
// reference takes from its absent ITM library): mirror copy, or wrap.
inline void apply_BCs_scalar(const sim_info& params, griddoubletype& f) {
  const int g = params.numGC, Nx = params.Nx, Ny = params.Ny;
  if (params.BC_T == BC_PERIODIC && params.BC_L == BC_PERIODIC && params.BC_B == BC_PERIODIC &&
      params.BC_R == BC_PERIODIC) {
    for (int i = 0; i < Ny + 2 * g; i++)
      for (int j = 0; j < Nx + 2 * g; j++)
        f[i][j] = f[(i - g + Ny) % Ny + g][(j - g + Nx) % Nx + g];
    return;
  }
  for (int i = g; i < Ny + g; i++)
    for (int j = 0; j < g; j++) {
      f[i][j] = f[i][2 * g - j - 1];
      f[i][j + Nx + g] = f[i][Nx + g - 1 - j];
    }
  for (int j = 0; j < Nx + 2 * g; j++)
    for (int i = 0; i < g; i++) {
      f[i][j] = f[2 * g - i - 1][j];
      f[i + Ny + g][j] = f[Ny + g - 1 - i][j];
    }
}

// ----------------------------------------------------------------------------
// Level set (the reference's Levelset class lives in the absent
// PhD-Interface-tracking-methods library; this is the project's own
// definition, call sites sourcecode/sim_twofluid.cpp:47,72,555-570).
//   normal at a cell centre: central-difference gradient of phi
//   interfacial cell: phi <= 0 differs from a 4-neighbour's phi <= 0
//   advection: order 1 = first-order upwind, forward Euler;
//              order 5 = HOUC5 with 3-stage TVD Runge-Kutta, frozen velocity
//   reinitialisation: Sussman-Smereka-Osher PDE, Godunov upwinding,
//              dtau = 0.5 min(dx, dy), S(phi0) = phi0 / sqrt(phi0^2 + h^2)
// ----------------------------------------------------------------------------
struct Levelset {
  sim_info params;
  griddoubletype phi;
  int order = 5, reinit_every = 1, reinit_iters = 5;
  int updates = 0;

  double get_sdf(int i, int j) const { return phi[i][j]; }
  vec2 get_normal(int i, int j) const {
    return {(phi[i][j + 1] - phi[i][j - 1]) / (2.0 * params.dx), (phi[i + 1][j] - phi[i - 1][j]) / (2.0 * params.dy)};
  }
  bool is_interfacial_cell(int i, int j) const {
    bool s = phi[i][j] <= 0.0;
    return (phi[i][j - 1] <= 0.0) != s || (phi[i][j + 1] <= 0.0) != s || (phi[i - 1][j] <= 0.0) != s ||
           (phi[i + 1][j] <= 0.0) != s;
  }

  // HOUC5 one-sided derivative for velocity sign a; inv60h = 1 / (60 h)
  static double houc5(double a, double fm3, double fm2, double fm1, double f0, double fp1, double fp2, double fp3,
                      double inv60h) {
    if (a >= 0.0)
      return (-2.0 * fm3 + 15.0 * fm2 - 60.0 * fm1 + 20.0 * f0 + 30.0 * fp1 - 3.0 * fp2) * inv60h;
    return (3.0 * fm2 - 30.0 * fm1 - 20.0 * f0 + 60.0 * fp1 - 15.0 * fp2 + 2.0 * fp3) * inv60h;
  }

  // rate L(f) = -(u f_x + v f_y) on real cells (derivatives multiply by 1/dx)
  void rate(const griddoubletype& f, const gridVector2dtype& vel, griddoubletype& out) const {
    const int g = params.numGC;
    const double idx = 1.0 / params.dx, idy = 1.0 / params.dy;
    const double i60x = 1.0 / (60.0 * params.dx), i60y = 1.0 / (60.0 * params.dy);
    for (int i = g; i < params.Ny + g; i++)
      for (int j = g; j < params.Nx + g; j++) {
        double u = vel[i][j][0], v = vel[i][j][1];
        double fx, fy;
        if (order == 1) {
          fx = (u >= 0.0) ? (f[i][j] - f[i][j - 1]) * idx : (f[i][j + 1] - f[i][j]) * idx;
          fy = (v >= 0.0) ? (f[i][j] - f[i - 1][j]) * idy : (f[i + 1][j] - f[i][j]) * idy;
        } else {
          fx = houc5(u, f[i][j - 3], f[i][j - 2], f[i][j - 1], f[i][j], f[i][j + 1], f[i][j + 2], f[i][j + 3], i60x);
          fy = houc5(v, f[i - 3][j], f[i - 2][j], f[i - 1][j], f[i][j], f[i + 1][j], f[i + 2][j], f[i + 3][j], i60y);
        }
        out[i][j] = -(u * fx + v * fy);
      }
  }

  void advect(const gridVector2dtype& vel, double dt) {
    const int g = params.numGC;
    griddoubletype L(phi.size(), std::vector<double>(phi[0].size(), 0.0));
    if (order == 1) {
      rate(phi, vel, L);
      for (int i = g; i < params.Ny + g; i++)
        for (int j = g; j < params.Nx + g; j++) phi[i][j] = phi[i][j] + dt * L[i][j];
      apply_BCs_scalar(params, phi);
      return;
    }
    griddoubletype p1 = phi, p2 = phi;
    rate(phi, vel, L);
    for (int i = g; i < params.Ny + g; i++)
      for (int j = g; j < params.Nx + g; j++) p1[i][j] = phi[i][j] + dt * L[i][j];
    apply_BCs_scalar(params, p1);
    rate(p1, vel, L);
    for (int i = g; i < params.Ny + g; i++)
      for (int j = g; j < params.Nx + g; j++) p2[i][j] = 0.75 * phi[i][j] + 0.25 * (p1[i][j] + dt * L[i][j]);
    apply_BCs_scalar(params, p2);
    rate(p2, vel, L);
    for (int i = g; i < params.Ny + g; i++)
      for (int j = g; j < params.Nx + g; j++)
        phi[i][j] = (1.0 / 3.0) * phi[i][j] + (2.0 / 3.0) * (p2[i][j] + dt * L[i][j]);
    apply_BCs_scalar(params, phi);
  }

  void reinitialise() {
    const int g = params.numGC;
    const double h = std::min(params.dx, params.dy);
    const double dtau = 0.5 * h;
    const double idx = 1.0 / params.dx, idy = 1.0 / params.dy;
    griddoubletype phi0 = phi, next = phi;
    for (int it = 0; it < reinit_iters; it++) {
      for (int i = g; i < params.Ny + g; i++)
        for (int j = g; j < params.Nx + g; j++) {
          double p0 = phi0[i][j];
          double S = p0 / std::sqrt(p0 * p0 + h * h);
          double a = (phi[i][j] - phi[i][j - 1]) * idx;
          double b = (phi[i][j + 1] - phi[i][j]) * idx;
          double c = (phi[i][j] - phi[i - 1][j]) * idy;
          double d = (phi[i + 1][j] - phi[i][j]) * idy;
          double gx, gy;
          if (p0 > 0.0) {
            double ap = std::max(a, 0.0), bm = std::min(b, 0.0), cp = std::max(c, 0.0), dm = std::min(d, 0.0);
            gx = std::max(ap * ap, bm * bm);
            gy = std::max(cp * cp, dm * dm);
          } else {
            double am = std::min(a, 0.0), bp = std::max(b, 0.0), cm = std::min(c, 0.0), dp = std::max(d, 0.0);
            gx = std::max(am * am, bp * bp);
            gy = std::max(cm * cm, dp * dp);
          }
          double G = std::sqrt(gx + gy) - 1.0;
          next[i][j] = phi[i][j] - dtau * S * G;
        }
      apply_BCs_scalar(params, next);
      phi = next;
    }
  }

  // update_interface_coupled(vfield, t, dt)
  void update_interface_coupled(const gridVector2dtype& vel, double dt) {
    advect(vel, dt);
    updates++;
    if (reinit_every > 0 && updates % reinit_every == 0) reinitialise();
  }
};

// ----------------------------------------------------------------------------
// VOF interface tracker.  The reference's VOF class (settings ITM "PYVOF",
// sourcecode/sim_twofluid.cpp:575-579) lives in the absent
// PhD-Interface-tracking-methods library; GFM_VOF and OGFM_VOF use its
// get_z, get_mixedcell_normal and get_interfacelocation
// (sourcecode/GFM_VOF.cpp:20,59,80-98; sourcecode/OGFM_VOF.cpp:23,60,118-152)
// and compute_dt its get_sdf (sourcecode/sim_twofluid.cpp:129).  This is the
// project's own definition from published methods:
//   z        volume fraction of fluid 1; a cell is mixed when 0 < z < 1
//   normal   Youngs (1982) with the Parker & Youngs (1992) 3x3 weights: minus
//            the weighted central-difference gradient of z, unit length,
//            pointing from fluid 1 into fluid 2; (1, 0) where it vanishes
//   PLIC     the line with that normal cutting the cell at area fraction z
//            (Scardovelli & Zaleski, J. Comput. Phys. 164 (2000), analytic
//            area / line-constant relations); the interface location is the
//            midpoint of the line's segment inside the cell
//   advection  directional splitting (x then y on even steps, y then x on
//            odd ones), each face's flux the PLIC fluid-1 area of the donor
//            strip of width |u_f| dt / h, u_f the mean of the two cells'
//            velocities, with the divergence term of Weymouth & Yue
//            (J. Comput. Phys. 229 (2010)), c = 1 where z > 0.5 at the start
//            of the step, else 0; values within 1e-8 of 0 or 1 become 0 or 1,
//            and the mirror / wrap BCs of phi follow each sweep
//   get_sdf  0.5 - z (negative in fluid 1, as the level set's phi)
// ----------------------------------------------------------------------------
namespace vof {
constexpr double ZEPS = 1e-8;

inline double lo(double a, double b) { return (b < a) ? b : a; }
inline double hi(double a, double b) { return (b < a) ? a : b; }

// area fraction of {c1 t + c2 s <= b} in the unit square (c1, c2 >= 0)
inline double area(double b, double c1, double c2) {
  const double m1 = lo(c1, c2), m2 = hi(c1, c2);
  if (b <= 0.0) return 0.0;
  const double s = m1 + m2;
  if (b >= s) return 1.0;
  if (m1 == 0.0) return b / m2;
  const double d = (2.0 * m1) * m2;
  if (b < m1) return (b * b) / d;
  if (b <= m2) return (b - 0.5 * m1) / m2;
  const double r = s - b;
  return 1.0 - (r * r) / d;
}

// the line constant b with area(b, m1, m2) = z, 0 < z < 1, m1 <= m2, m2 > 0
inline double line_constant(double z, double m1, double m2) {
  if (m1 == 0.0) return z * m2;
  const double v1 = m1 / (2.0 * m2);
  const double d = (2.0 * m1) * m2;
  if (z < v1) return std::sqrt(d * z);
  if (z <= 1.0 - v1) return z * m2 + 0.5 * m1;
  return (m1 + m2) - std::sqrt(d * (1.0 - z));
}

// PLIC reconstruction of a mixed cell.  In the unit cell with the axes
// reflected where the normal component is negative, fluid 1 fills
// {a xi + b eta <= beta}, a = |nx| dx, b = |ny| dy.
struct Plic {
  double nx, ny, a, b, beta;
};

inline Plic reconstruct(const sim_info& p, const griddoubletype& z, int i, int j) {
  const double gx = ((z[i - 1][j + 1] + 2.0 * z[i][j + 1]) + z[i + 1][j + 1]) -
                    ((z[i - 1][j - 1] + 2.0 * z[i][j - 1]) + z[i + 1][j - 1]);
  const double gy = ((z[i + 1][j - 1] + 2.0 * z[i + 1][j]) + z[i + 1][j + 1]) -
                    ((z[i - 1][j - 1] + 2.0 * z[i - 1][j]) + z[i - 1][j + 1]);
  const double mx = -gx / p.dx, my = -gy / p.dy;
  const double nn = std::sqrt(mx * mx + my * my);
  Plic r;
  if (nn > 0.0) { r.nx = mx / nn; r.ny = my / nn; }
  else { r.nx = 1.0; r.ny = 0.0; }
  r.a = std::fabs(r.nx) * p.dx;
  r.b = std::fabs(r.ny) * p.dy;
  r.beta = line_constant(z[i][j], lo(r.a, r.b), hi(r.a, r.b));
  return r;
}

// midpoint of the PLIC segment in physical coordinates
inline vec2 segment_midpoint(const sim_info& p, const Plic& r, int i, int j) {
  const double m1 = lo(r.a, r.b), m2 = hi(r.a, r.b);
  const bool swapped = r.b < r.a;   // the m1 axis is eta
  const double be = r.beta;
  double u1, w1, u2, w2;
  if (be < m1) { u1 = be / m1; w1 = 0.0; u2 = 0.0; w2 = be / m2; }
  else if (be <= m2) { u1 = 0.0; w1 = be / m2; u2 = 1.0; w2 = (be - m1) / m2; }
  else { u1 = 1.0; w1 = (be - m1) / m2; u2 = (be - m2) / m1; w2 = 1.0; }
  const double um = 0.5 * (u1 + u2), wm = 0.5 * (w1 + w2);
  const double xr = swapped ? wm : um, er = swapped ? um : wm;
  const double xi = (r.nx < 0.0) ? 1.0 - xr : xr;
  const double eta = (r.ny < 0.0) ? 1.0 - er : er;
  const vec2 cc = p.cellcentre_coord(i, j);
  return {cc[0] + (xi - 0.5) * p.dx, cc[1] + (eta - 0.5) * p.dy};
}

// fluid-1 volume of cell (i,j), as a fraction of the cell, inside the strip of
// width w (0 < w <= 1) along axis dir (0: x, 1: y) touching the cell's high
// face (high = true) or its low face
inline double strip_fraction(const sim_info& p, const griddoubletype& z, int i, int j, int dir, bool high,
                             double w) {
  const double zc = z[i][j];
  if (zc == 1.0) return w;
  if (zc == 0.0) return 0.0;
  const Plic r = reconstruct(p, z, i, j);
  const double n = dir == 0 ? r.nx : r.ny;
  const double cd = dir == 0 ? r.a : r.b, co = dir == 0 ? r.b : r.a;
  const bool refl = n < 0.0;
  const double start = (high != refl) ? 1.0 - w : 0.0;   // strip start in reflected coordinates
  return w * area(r.beta - cd * start, cd * w, co);
}
}  // namespace vof

struct VOFTracker {
  sim_info params;
  griddoubletype z;
  int steps = 0;   // interface updates so far (sets the sweep order)

  double get_z(int i, int j) const { return z[i][j]; }
  double get_sdf(int i, int j) const { return 0.5 - z[i][j]; }
  vec2 get_mixedcell_normal(int i, int j) const {
    vof::Plic r = vof::reconstruct(params, z, i, j);
    return {r.nx, r.ny};
  }
  vec2 get_interfacelocation(int i, int j) const {
    return vof::segment_midpoint(params, vof::reconstruct(params, z, i, j), i, j);
  }

  // face flux (signed, + towards the high cell) between cell lo and the next
  // cell along dir, for Courant number s
  double face_flux(const griddoubletype& zz, int i, int j, int dir, double s) const {
    const int i2 = dir == 0 ? i : i + 1, j2 = dir == 0 ? j + 1 : j;
    if (s > 0.0) return vof::strip_fraction(params, zz, i, j, dir, true, s);
    if (s < 0.0) return -vof::strip_fraction(params, zz, i2, j2, dir, false, -s);
    return 0.0;
  }

  void sweep(int dir, const gridVector2dtype& vel, double dt, const griddoubletype& z0) {
    const int g = params.numGC;
    const double dtdh = dt / (dir == 0 ? params.dx : params.dy);
    griddoubletype out = z;
    for (int i = g; i < params.Ny + g; i++)
      for (int j = g; j < params.Nx + g; j++) {
        const int il = dir == 0 ? i : i - 1, jl = dir == 0 ? j - 1 : j;
        const int ih = dir == 0 ? i : i + 1, jh = dir == 0 ? j + 1 : j;
        const double uL = 0.5 * (vel[il][jl][dir] + vel[i][j][dir]);
        const double uH = 0.5 * (vel[i][j][dir] + vel[ih][jh][dir]);
        const double sL = uL * dtdh, sH = uH * dtdh;
        const double FL = face_flux(z, il, jl, dir, sL);
        const double FH = face_flux(z, i, j, dir, sH);
        const double c = (z0[i][j] > 0.5) ? 1.0 : 0.0;
        double zn = z[i][j] - ((FH - c * sH) - (FL - c * sL));
        if (zn < vof::ZEPS) zn = 0.0;
        else if (zn > 1.0 - vof::ZEPS) zn = 1.0;
        out[i][j] = zn;
      }
    apply_BCs_scalar(params, out);
    z = out;
  }

  // update_interface_coupled(vfield, t, dt)
  void update_interface_coupled(const gridVector2dtype& vel, double dt) {
    const griddoubletype z0 = z;
    const int first = (steps % 2 == 0) ? 0 : 1;
    sweep(first, vel, dt, z0);
    sweep(1 - first, vel, dt, z0);
    steps++;
  }
};

// grid_bilinear_interpolate (PhD-Common; absent): the lower-left of the four
// cell centres surrounding x, clamped to the padded grid, and the weights
// a (x direction) and b (y direction).
inline void bilinear_cell(const sim_info& params, const vec2& x, int& i0, int& j0, double& a, double& b) {
  const double idx = 1.0 / params.dx, idy = 1.0 / params.dy;
  double s = (x[0] - params.x0) * idx + static_cast<double>(params.numGC) - 0.5;
  double t = (x[1] - params.y0) * idy + static_cast<double>(params.numGC) - 0.5;
  j0 = static_cast<int>(std::floor(s));
  i0 = static_cast<int>(std::floor(t));
  const int nrow = params.Ny + 2 * params.numGC, ncol = params.Nx + 2 * params.numGC;
  j0 = std::min(std::max(j0, 0), ncol - 2);
  i0 = std::min(std::max(i0, 0), nrow - 2);
  a = s - static_cast<double>(j0);
  b = t - static_cast<double>(i0);
}

}  // namespace oitm
