// Host-side set-up of named test cases: the parameters of
// sim_twofluid::set_sim_parameters (sourcecode/sim_twofluid.cpp:336-490) and
// sim_onefluid::set_sim_parameters (sourcecode/sim_onefluid.cpp:96-146), and
// the initial conditions of set_sim_ICs (sourcecode/sim_twofluid.cpp:599-1799,
// sourcecode/sim_onefluid.cpp:196-449), followed by apply_BCs_euler as there.
//
// Also the workloads the GB300 build is measured on:
//   shock_bubble            1000x400 shock-bubble on [0,0.25]x[0,0.089]
//   underwater_explosion_sg 800x800 stiffened-gas underwater explosion on [-1,1]^2
//   circularexplosion       one-fluid 200x200 circular explosion on [0,2]^2
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "gfm_cases.cuh"
#include "../../include/gfm_gb300.h"

using gfm::CaseSpec;
using gfm::V4;

namespace {

struct Geo {
  int Nx, Ny, g;
  double x0, y0, dx, dy;
  int nc, nr;
  double ccx(int j) const { return x0 + ((double)(j - g) + 0.5) * dx; }
  double ccy(int i) const { return y0 + ((double)(i - g) + 0.5) * dy; }
};

Geo geo_of(const gfm_grid_desc* d) {
  Geo G;
  G.Nx = d->Nx; G.Ny = d->Ny; G.g = d->numGC;
  G.x0 = d->x0; G.y0 = d->y0; G.dx = d->dx; G.dy = d->dy;
  G.nc = G.Nx + 2 * G.g; G.nr = G.Ny + 2 * G.g;
  return G;
}

V4 p2c(double g, double pinf, double rho, double u, double v, double p) {
  return gfm::prims_to_cons(g, pinf, V4{rho, u, v, p}, nullptr);
}

void put(const Geo& G, double* U, int i, int j, const V4& s) {
  size_t plane = (size_t)G.nr * G.nc, c = (size_t)i * G.nc + j;
  U[c] = s.a; U[plane + c] = s.b; U[2 * plane + c] = s.c; U[3 * plane + c] = s.d;
}

// apply_BCs_euler on a host SoA grid (headers/euler_bc.hpp:5-103)
void host_bcs(const gfm_grid_desc* d, double* U) {
  Geo G = geo_of(d);
  const int g = G.g, Nx = G.Nx, Ny = G.Ny, nc = G.nc;
  size_t plane = (size_t)G.nr * G.nc;
  auto at = [&](int k, int i, int j) -> double& { return U[k * plane + (size_t)i * nc + j]; };
  auto copy = [&](int i, int j, int si, int sj) { for (int k = 0; k < 4; k++) at(k, i, j) = at(k, si, sj); };
  bool per = d->BC_L == GFM_BC_PERIODIC && d->BC_R == GFM_BC_PERIODIC && d->BC_B == GFM_BC_PERIODIC &&
             d->BC_T == GFM_BC_PERIODIC;
  if (per) {
    for (int i = 0; i < Ny + 2 * g; i++)
      for (int j = 0; j < Nx + 2 * g; j++) copy(i, j, (i - g + Ny) % Ny + g, (j - g + Nx) % Nx + g);
    return;
  }
  for (int i = g; i < Ny + g; i++)
    for (int j = 0; j < g; j++) {
      copy(i, j, i, 2 * g - j - 1);
      if (d->BC_L == GFM_BC_REFLECTIVE) at(1, i, j) = -at(1, i, j);
    }
  for (int i = g; i < Ny + g; i++)
    for (int j = 0; j < g; j++) {
      copy(i, j + Nx + g, i, Nx + g - 1 - j);
      if (d->BC_L == GFM_BC_REFLECTIVE) at(1, i, j + Nx + g) = -at(1, i, j + Nx + g);
    }
  for (int j = 0; j < Nx + 2 * g; j++)
    for (int i = 0; i < g; i++) {
      copy(i, j, 2 * g - i - 1, j);
      if (d->BC_B == GFM_BC_REFLECTIVE) at(2, i, j) = -at(2, i, j);
    }
  for (int j = 0; j < Nx + 2 * g; j++)
    for (int i = 0; i < g; i++) {
      copy(i + Ny + g, j, Ny + g - 1 - i, j);
      if (d->BC_T == GFM_BC_REFLECTIVE) at(2, i + Ny + g, j) = -at(2, i + Ny + g, j);
    }
}

void base_desc(gfm_grid_desc* d, int Nx, int Ny, int g) {
  memset(d, 0, sizeof(*d));
  d->Nx = Nx; d->Ny = Ny; d->numGC = g;
  d->x0 = 0.0; d->y0 = 0.0;
  d->dx = 1.0 / Nx; d->dy = 1.0 / Ny;
  d->BC_L = d->BC_R = d->BC_B = d->BC_T = GFM_BC_TRANSMISSIVE;
  d->gamma1 = 1.4; d->gamma2 = 1.4; d->pinf1 = 0.0; d->pinf2 = 0.0;
}

// Rankine-Hugoniot post-shock state behind a shock of Mach M running into
// (rho1, p1) at rest, the shock moving towards -x.
void post_shock(double g, double M, double rho1, double p1, double& rho2, double& u2, double& p2) {
  double M2 = M * M;
  p2 = p1 * (1.0 + 2.0 * g / (g + 1.0) * (M2 - 1.0));
  rho2 = rho1 * ((g + 1.0) * M2 / ((g - 1.0) * M2 + 2.0));
  double W = M * std::sqrt(g * p1 / rho1);
  u2 = -W * (1.0 - rho1 / rho2);
}

gfm::CaseGeo case_geo(const Geo& G) {
  gfm::CaseGeo C;
  C.Nx = G.Nx; C.Ny = G.Ny; C.g = G.g; C.nr = G.nr; C.nc = G.nc;
  C.x0 = G.x0; C.y0 = G.y0; C.dx = G.dx; C.dy = G.dy;
  return C;
}

// every padded cell from the case's spec, then apply_BCs_euler on the grids
void fill_case(const CaseSpec& cs, const gfm_grid_desc* d, bool two, double* U1, double* U2, double* phi, double* z) {
  Geo G = geo_of(d);
  const gfm::CaseGeo C = case_geo(G);
  for (int i = 0; i < G.nr; i++)
    for (int j = 0; j < G.nc; j++) {
      V4 u1, u2 = V4{0.0, 0.0, 0.0, 0.0};
      double ph = 0.0, zz = 0.0;
      gfm::case_cell(cs, C, i, j, z != nullptr, u1, u2, ph, zz);
      put(G, U1, i, j, u1);
      if (two) {
        put(G, U2, i, j, u2);
        phi[(size_t)i * G.nc + j] = ph;
        if (z) z[(size_t)i * G.nc + j] = zz;
      }
    }
  host_bcs(d, U1);
  if (two) host_bcs(d, U2);
}

}  // namespace

namespace gfm {

// The parameters of a named case (set_sim_ICs, sourcecode/sim_twofluid.cpp:599-1799,
// sourcecode/sim_onefluid.cpp:196-449, and the benchmark workloads).
bool make_case_spec(const char* sim_type, const char* test_case, const gfm_grid_desc* d, CaseSpec* out) {
  std::string st(sim_type), tc(test_case);
  const double g1 = d->gamma1, q1 = d->pinf1, g2 = d->gamma2, q2 = d->pinf2;
  CaseSpec c;
  memset(&c, 0, sizeof(c));
  c.g1 = g1; c.q1 = q1; c.g2 = g2; c.q2 = q2;
  c.xsplit = INFINITY;
  if (st == "onefluid") {
    bool ydir = tc.size() > 2 && tc.substr(tc.size() - 2) == "_y";
    c.kind = gfm::CASE_PLANAR;
    c.pa = ydir ? 0.0 : 1.0; c.pb = ydir ? 1.0 : 0.0; c.pc = 0.5;
    if (tc == "TTC1_x" || tc == "TTC1_y") { c.L = p2c(g1, q1, 1.0, 0, 0, 1.0); c.R = p2c(g1, q1, 0.125, 0, 0, 0.1); }
    else if (tc == "TTC2_x") { c.L = p2c(g1, q1, 1.0, -2.0, 0, 0.4); c.R = p2c(g1, q1, 1.0, 2.0, 0, 0.4); }
    else if (tc == "TTC2_y") { c.L = p2c(g1, q1, 1.0, 0, -2.0, 0.4); c.R = p2c(g1, q1, 1.0, 0, 2.0, 0.4); }
    else if (tc == "TTC3_x" || tc == "TTC3_y") { c.L = p2c(g1, q1, 1.0, 0, 0, 1000.0); c.R = p2c(g1, q1, 1.0, 0, 0, 0.01); }
    else if (tc == "TTC4_x" || tc == "TTC4_y") { c.L = p2c(g1, q1, 1.0, 0, 0, 0.1); c.R = p2c(g1, q1, 1.0, 0, 0, 100.0); }
    else if (tc == "TTC5_x") {
      c.L = p2c(g1, q1, 5.99924, 19.5975, 0, 460.894); c.R = p2c(g1, q1, 5.99242, -6.19633, 0, 46.0950);
    } else if (tc == "TTC5_y") {
      c.L = p2c(g1, q1, 5.99924, 0, 19.5975, 460.894); c.R = p2c(g1, q1, 5.99242, 0, -6.19633, 46.0950);
    } else if (tc == "circularexplosion") {
      // sourcecode/sim_onefluid.cpp:359-415: primitives blended by area fraction
      c.kind = gfm::CASE_BLEND_CIRCLE;
      c.L = V4{1.0, 0.0, 0.0, 1.0}; c.R = V4{0.125, 0.0, 0.0, 0.1};
      c.cx = 1.0; c.cy = 1.0; c.r = 0.4;
    } else {
      return false;
    }
    *out = c;
    return true;
  }
  if (st != "twofluid") return false;
  c.kind = gfm::CASE_CIRCLE;
  if (tc == "circularexplosion") {
    c.s1 = p2c(g1, q1, 1.0, 0, 0, 1.0); c.s2a = c.s2b = p2c(g2, q2, 0.125, 0, 0, 0.1);
    c.cx = 1.0; c.cy = 1.0; c.r = 0.4;
  } else if (tc == "ST1_x") {
    c.kind = gfm::CASE_PLANE_X; c.c = 0.5;
    c.s1 = p2c(g1, q1, 1.0, 0, 0, 100000.0); c.s2a = c.s2b = p2c(g2, q2, 0.125, 0, 0, 10000.0);
  } else if (tc == "ST2_y") {
    c.kind = gfm::CASE_PLANE_Y; c.c = 0.7;
    c.s1 = p2c(g1, q1, 1000.0, 0, 0, 1000000000.0); c.s2a = c.s2b = p2c(g2, q2, 50.0, 0, 0, 100000.0);
  } else if (tc == "GDA") {
    c.kind = gfm::CASE_GDA;
  } else if (tc == "shocked_helium_bubble") {
    c.s1 = p2c(g1, q1, 0.138, 0, 0, 1.0);
    c.s2a = p2c(g2, q2, 1.0, 0, 0, 1.0); c.s2b = p2c(g2, q2, 1.3764, -0.394, 0, 1.5698); c.xsplit = 225.0;
    c.cx = 175.0; c.cy = 44.5; c.r = 25.0;
  } else if (tc == "shocked_R22_bubble") {
    c.s1 = p2c(g1, q1, 3.863, 0, 0, 1.01325e5);
    c.s2a = p2c(g2, q2, 1.225, 0, 0, 1.01325e5); c.s2b = p2c(g2, q2, 1.686, -113.5, 0, 1.59e5); c.xsplit = 0.275;
    c.cx = 0.225; c.cy = 0.0445; c.r = 0.025;
  } else if (tc == "shock_bubble") {
    // light-gas bubble (fluid 1) hit by a Mach 1.22 shock in air (fluid 2)
    double rho2, u2, p2;
    post_shock(g2, 1.22, 1.0, 1e5, rho2, u2, p2);
    c.s1 = p2c(g1, q1, 0.182, 0, 0, 1e5);
    c.s2a = p2c(g2, q2, 1.0, 0, 0, 1e5); c.s2b = p2c(g2, q2, rho2, u2, 0, p2); c.xsplit = 0.225;
    c.cx = 0.175; c.cy = 0.0445; c.r = 0.025;
  } else if (tc == "underwater_explosion_sg") {
    // high-pressure air bubble (fluid 1) in stiffened-gas water (fluid 2)
    c.s1 = p2c(g1, q1, 1270.0, 0, 0, 8.29e8); c.s2a = c.s2b = p2c(g2, q2, 1000.0, 0, 0, 1e5);
    c.cx = 0.0; c.cy = 0.0; c.r = 0.2;
  } else {
    return false;
  }
  *out = c;
  return true;
}

// Shock-bubble family of the batched workload (gfm_case_shock_bubble's grids)
bool make_bubble_spec(const gfm_bubble_params* p, const gfm_grid_desc* d, CaseSpec* out) {
  CaseSpec c;
  memset(&c, 0, sizeof(c));
  const double W = d->dx * d->Nx, H = d->dy * d->Ny;
  double rho2, u2, p2;
  post_shock(d->gamma2, p->mach, 1.0, 1e5, rho2, u2, p2);
  c.kind = gfm::CASE_CIRCLE;
  c.g1 = d->gamma1; c.q1 = d->pinf1; c.g2 = d->gamma2; c.q2 = d->pinf2;
  c.s1 = p2c(d->gamma1, d->pinf1, p->rho_ratio, 0, 0, 1e5);
  c.s2a = p2c(d->gamma2, d->pinf2, 1.0, 0, 0, 1e5);
  c.s2b = p2c(d->gamma2, d->pinf2, rho2, u2, 0, p2);
  c.xsplit = 0.9 * W;
  c.cx = 0.7 * W; c.cy = 0.5 * H; c.r = p->radius_frac * H;
  *out = c;
  return true;
}

}  // namespace gfm

extern "C" {

gfm_status_t gfm_case_params(const char* sim_type, const char* test_case, int Nx, int Ny, gfm_grid_desc* d,
                             double* T) {
  if (!sim_type || !test_case || !d || !T || Nx < 1 || Ny < 1) return GFM_ERR_ARG;
  std::string st(sim_type), tc(test_case);
  if (st == "onefluid") {
    // sourcecode/sim_onefluid.cpp:96-146
    base_desc(d, Nx, Ny, 2);
    d->gamma2 = 0.0;
    if (tc == "TTC1_x" || tc == "TTC1_y") *T = 0.25;
    else if (tc == "TTC2_x" || tc == "TTC2_y") *T = 0.15;
    else if (tc == "TTC3_x" || tc == "TTC3_y") *T = 0.012;
    else if (tc == "TTC4_x" || tc == "TTC4_y") *T = 0.035;
    else if (tc == "TTC5_x" || tc == "TTC5_y") *T = 0.035;
    else if (tc == "circularexplosion") { d->dx = 2.0 / Nx; d->dy = 2.0 / Ny; *T = 0.25; }
    else return GFM_ERR_ARG;
    return GFM_OK;
  }
  if (st != "twofluid") return GFM_ERR_ARG;
  // sourcecode/sim_twofluid.cpp:336-490
  base_desc(d, Nx, Ny, 8);
  if (tc == "circularexplosion") { d->dx = 2.0 / Nx; d->dy = 2.0 / Ny; *T = 0.25; }
  else if (tc == "ST1_x") { d->gamma2 = 1.2; *T = 0.0007; }
  else if (tc == "ST2_y") {
    d->gamma1 = 4.4; d->pinf1 = 600000000.0;
    d->x0 = -2.0; d->y0 = -2.0; d->dx = 4.0 / Nx; d->dy = 4.0 / Ny; *T = 0.0009;
  } else if (tc == "GDA") {
    d->BC_L = d->BC_R = d->BC_B = d->BC_T = GFM_BC_PERIODIC; *T = 10.0;
  } else if (tc == "shocked_helium_bubble") {
    d->gamma1 = 1.667; d->dx = 325.0 / Nx; d->dy = 89.0 / Ny; *T = 280.0;
    d->BC_T = d->BC_B = GFM_BC_REFLECTIVE;
  } else if (tc == "shocked_R22_bubble") {
    d->gamma1 = 1.249; d->dx = 0.445 / Nx; d->dy = 0.089 / Ny; *T = 0.0014;
    d->BC_T = d->BC_B = GFM_BC_REFLECTIVE;
  } else if (tc == "shock_bubble") {
    // light-gas bubble (fluid 1) hit by a Mach 1.22 shock in air (fluid 2)
    d->gamma1 = 1.648; d->dx = 0.25 / Nx; d->dy = 0.089 / Ny; *T = 1.0;
    d->BC_T = d->BC_B = GFM_BC_REFLECTIVE;
  } else if (tc == "underwater_explosion_sg") {
    // high-pressure air bubble (fluid 1) in stiffened-gas water (fluid 2)
    d->gamma2 = 4.4; d->pinf2 = 6e8;
    d->x0 = -1.0; d->y0 = -1.0; d->dx = 2.0 / Nx; d->dy = 2.0 / Ny; *T = 1.0;
  } else {
    return GFM_ERR_ARG;
  }
  return GFM_OK;
}

gfm_status_t gfm_case_init(const char* sim_type, const char* test_case, const gfm_grid_desc* d, double* U1,
                           double* U2, double* phi) {
  if (!sim_type || !test_case || !d || !U1) return GFM_ERR_ARG;
  CaseSpec cs;
  if (!gfm::make_case_spec(sim_type, test_case, d, &cs)) return GFM_ERR_ARG;
  const bool two = std::string(sim_type) == "twofluid";
  if (two && (!U2 || !phi)) return GFM_ERR_ARG;
  fill_case(cs, d, two, U1, U2, phi, nullptr);
  return GFM_OK;
}

// Volume fraction of fluid 1 for the VOF interface tracker: the zval of
// set_sim_ICs (10x10 sub-sampled area fractions for circles,
// sourcecode/sim_twofluid.cpp:646-668,825-856; the clipped linear profiles of
// the planar tubes, :697,731; z = 1 for GDA, :769).
gfm_status_t gfm_case_init_z(const char* test_case, const gfm_grid_desc* d, double* z) {
  if (!test_case || !d || !z) return GFM_ERR_ARG;
  CaseSpec cs;
  if (!gfm::make_case_spec("twofluid", test_case, d, &cs)) return GFM_ERR_ARG;
  Geo G = geo_of(d);
  const gfm::CaseGeo C = case_geo(G);
  for (int i = 0; i < G.nr; i++)
    for (int j = 0; j < G.nc; j++) {
      V4 u1, u2;
      double ph, zz;
      gfm::case_cell(cs, C, i, j, true, u1, u2, ph, zz);
      z[(size_t)i * G.nc + j] = zz;
    }
  return GFM_OK;
}

// Shock-bubble family of the batched workload: the 1000x400 case's geometry
// scaled to any grid (width 0.25, square cells, height 0.25 Ny/Nx), bubble
// of fluid 1 centred at (0.7 W, H/2), left-moving shock in air at x = 0.9 W.
gfm_status_t gfm_case_shock_bubble(const gfm_bubble_params* p, int Nx, int Ny, gfm_grid_desc* d, double* T) {
  if (!p || !d || !T || Nx < 8 || Ny < 8) return GFM_ERR_ARG;
  if (!(p->mach > 1.0) || !(p->gamma_bubble > 1.0) || !(p->rho_ratio > 0.0) || !(p->radius_frac > 0.0) ||
      !(p->radius_frac <= 0.45))
    return GFM_ERR_ARG;
  memset(d, 0, sizeof(*d));
  d->Nx = Nx; d->Ny = Ny; d->numGC = 8;
  d->x0 = 0.0; d->y0 = 0.0;
  d->dx = 0.25 / Nx; d->dy = d->dx;
  d->BC_L = d->BC_R = GFM_BC_TRANSMISSIVE;
  d->BC_B = d->BC_T = GFM_BC_REFLECTIVE;
  d->gamma1 = p->gamma_bubble; d->pinf1 = 0.0;
  d->gamma2 = 1.4; d->pinf2 = 0.0;
  *T = 1.0;
  return GFM_OK;
}

gfm_status_t gfm_case_init_shock_bubble(const gfm_bubble_params* p, const gfm_grid_desc* d, double* U1, double* U2,
                                        double* phi) {
  if (!p || !d || !U1 || !U2 || !phi) return GFM_ERR_ARG;
  CaseSpec cs;
  if (!gfm::make_bubble_spec(p, d, &cs)) return GFM_ERR_ARG;
  fill_case(cs, d, true, U1, U2, phi, nullptr);
  return GFM_OK;
}

gfm_status_t gfm_case_init_shock_bubble_z(const gfm_bubble_params* p, const gfm_grid_desc* d, double* z) {
  if (!p || !d || !z) return GFM_ERR_ARG;
  CaseSpec cs;
  if (!gfm::make_bubble_spec(p, d, &cs)) return GFM_ERR_ARG;
  Geo G = geo_of(d);
  const gfm::CaseGeo C = case_geo(G);
  for (int i = 0; i < G.nr; i++)
    for (int j = 0; j < G.nc; j++) {
      V4 u1, u2;
      double ph, zz;
      gfm::case_cell(cs, C, i, j, true, u1, u2, ph, zz);
      z[(size_t)i * G.nc + j] = zz;
    }
  return GFM_OK;
}

}  // extern "C"
