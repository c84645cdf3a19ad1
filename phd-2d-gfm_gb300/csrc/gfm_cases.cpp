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
#include "gfm_math.cuh"
#include "../../include/gfm_gb300.h"

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

// fraction of 10x10 sub-samples of cell (i,j) within radius R of (cx, cy)
double area_fraction(const Geo& G, int i, int j, double cx, double cy, double R) {
  const int N = 10;
  int inside = 0;
  double delx = G.dx / N, dely = G.dy / N;
  double blx = G.ccx(j) - 0.5 * G.dx, bly = G.ccy(i) - 0.5 * G.dy;
  for (int a = 0; a < N; a++)
    for (int b = 0; b < N; b++) {
      double sx = blx + (a + 0.5) * delx - cx;
      double sy = bly + (b + 0.5) * dely - cy;
      if (std::sqrt(sx * sx + sy * sy) <= R) inside++;
    }
  return double(inside) / (N * N);
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

}  // namespace

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
  std::string st(sim_type), tc(test_case);
  Geo G = geo_of(d);
  const double g1 = d->gamma1, q1 = d->pinf1, g2 = d->gamma2, q2 = d->pinf2;
  if (st == "onefluid") {
    auto planar = [&](V4 Lst, V4 Rst, double a, double b, double c) {
      for (int i = 0; i < G.nr; i++)
        for (int j = 0; j < G.nc; j++) put(G, U1, i, j, (G.ccx(j) * a + G.ccy(i) * b <= c) ? Lst : Rst);
    };
    bool ydir = tc.size() > 2 && tc.substr(tc.size() - 2) == "_y";
    double a = ydir ? 0.0 : 1.0, b = ydir ? 1.0 : 0.0;
    if (tc == "TTC1_x" || tc == "TTC1_y") planar(p2c(g1, q1, 1.0, 0, 0, 1.0), p2c(g1, q1, 0.125, 0, 0, 0.1), a, b, 0.5);
    else if (tc == "TTC2_x") planar(p2c(g1, q1, 1.0, -2.0, 0, 0.4), p2c(g1, q1, 1.0, 2.0, 0, 0.4), 1.0, 0.0, 0.5);
    else if (tc == "TTC2_y") planar(p2c(g1, q1, 1.0, 0, -2.0, 0.4), p2c(g1, q1, 1.0, 0, 2.0, 0.4), 0.0, 1.0, 0.5);
    else if (tc == "TTC3_x" || tc == "TTC3_y")
      planar(p2c(g1, q1, 1.0, 0, 0, 1000.0), p2c(g1, q1, 1.0, 0, 0, 0.01), a, b, 0.5);
    else if (tc == "TTC4_x" || tc == "TTC4_y")
      planar(p2c(g1, q1, 1.0, 0, 0, 0.1), p2c(g1, q1, 1.0, 0, 0, 100.0), a, b, 0.5);
    else if (tc == "TTC5_x")
      planar(p2c(g1, q1, 5.99924, 19.5975, 0, 460.894), p2c(g1, q1, 5.99242, -6.19633, 0, 46.0950), 1.0, 0.0, 0.5);
    else if (tc == "TTC5_y")
      planar(p2c(g1, q1, 5.99924, 0, 19.5975, 460.894), p2c(g1, q1, 5.99242, 0, -6.19633, 46.0950), 0.0, 1.0, 0.5);
    else if (tc == "circularexplosion") {
      // sourcecode/sim_onefluid.cpp:359-415
      const double L[4] = {1.0, 0.0, 0.0, 1.0}, R[4] = {0.125, 0.0, 0.0, 0.1};
      for (int i = 0; i < G.nr; i++)
        for (int j = 0; j < G.nc; j++) {
          double frac = area_fraction(G, i, j, 1.0, 1.0, 0.4);
          double W[4];
          for (int k = 0; k < 4; k++) W[k] = frac * L[k] + (1.0 - frac) * R[k];
          put(G, U1, i, j, p2c(g1, q1, W[0], W[1], W[2], W[3]));
        }
    } else {
      return GFM_ERR_ARG;
    }
    host_bcs(d, U1);
    return GFM_OK;
  }
  if (st != "twofluid" || !U2 || !phi) return GFM_ERR_ARG;
  auto fill = [&](auto&& f) {
    for (int i = 0; i < G.nr; i++)
      for (int j = 0; j < G.nc; j++) {
        V4 s1, s2;
        double ls;
        f(i, j, G.ccx(j), G.ccy(i), s1, s2, ls);
        put(G, U1, i, j, s1);
        put(G, U2, i, j, s2);
        phi[(size_t)i * G.nc + j] = ls;
      }
  };
  if (tc == "circularexplosion") {
    V4 Ls = p2c(g1, q1, 1.0, 0, 0, 1.0), Rs = p2c(g2, q2, 0.125, 0, 0, 0.1);
    fill([&](int, int, double x, double y, V4& a, V4& b, double& ls) {
      ls = std::sqrt((x - 1.0) * (x - 1.0) + (y - 1.0) * (y - 1.0)) - 0.4;
      a = Ls; b = Rs;
    });
  } else if (tc == "ST1_x") {
    V4 Ls = p2c(g1, q1, 1.0, 0, 0, 100000.0), Rs = p2c(g2, q2, 0.125, 0, 0, 10000.0);
    fill([&](int, int, double x, double, V4& a, V4& b, double& ls) { ls = x - 0.5; a = Ls; b = Rs; });
  } else if (tc == "ST2_y") {
    V4 Ls = p2c(g1, q1, 1000.0, 0, 0, 1000000000.0), Rs = p2c(g2, q2, 50.0, 0, 0, 100000.0);
    fill([&](int, int, double, double y, V4& a, V4& b, double& ls) { ls = y - 0.7; a = Ls; b = Rs; });
  } else if (tc == "GDA") {
    fill([&](int, int, double x, double y, V4& a, V4& b, double& ls) {
      double r2 = (x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5);
      V4 s = p2c(g1, q1, 1.0 + 1000.0 * std::exp(-r2 / (2.0 * 0.1 * 0.1)), 1.0, 1.0, 0.0001);
      a = s; b = s; ls = -1.0;
    });
  } else if (tc == "shocked_helium_bubble") {
    V4 he = p2c(g1, q1, 0.138, 0, 0, 1.0);
    V4 Ls = p2c(g2, q2, 1.3764, -0.394, 0, 1.5698), Rs = p2c(g2, q2, 1.0, 0, 0, 1.0);
    fill([&](int, int, double x, double y, V4& a, V4& b, double& ls) {
      b = (x < 225.0) ? Rs : Ls;
      a = he;
      ls = std::sqrt((x - 175.0) * (x - 175.0) + (y - 44.5) * (y - 44.5)) - 25.0;
    });
  } else if (tc == "shocked_R22_bubble") {
    V4 r22 = p2c(g1, q1, 3.863, 0, 0, 1.01325e5);
    V4 Ls = p2c(g2, q2, 1.686, -113.5, 0, 1.59e5), Rs = p2c(g2, q2, 1.225, 0, 0, 1.01325e5);
    fill([&](int, int, double x, double y, V4& a, V4& b, double& ls) {
      b = (x < 0.275) ? Rs : Ls;
      a = r22;
      ls = std::sqrt((x - 0.225) * (x - 0.225) + (y - 0.0445) * (y - 0.0445)) - 0.025;
    });
  } else if (tc == "shock_bubble") {
    double rho2, u2, p2;
    post_shock(g2, 1.22, 1.0, 1e5, rho2, u2, p2);
    V4 bub = p2c(g1, q1, 0.182, 0, 0, 1e5);
    V4 pre = p2c(g2, q2, 1.0, 0, 0, 1e5), post = p2c(g2, q2, rho2, u2, 0, p2);
    fill([&](int, int, double x, double y, V4& a, V4& b, double& ls) {
      b = (x < 0.225) ? pre : post;
      a = bub;
      ls = std::sqrt((x - 0.175) * (x - 0.175) + (y - 0.0445) * (y - 0.0445)) - 0.025;
    });
  } else if (tc == "underwater_explosion_sg") {
    V4 air = p2c(g1, q1, 1270.0, 0, 0, 8.29e8), water = p2c(g2, q2, 1000.0, 0, 0, 1e5);
    fill([&](int, int, double x, double y, V4& a, V4& b, double& ls) {
      a = air; b = water;
      ls = std::sqrt(x * x + y * y) - 0.2;
    });
  } else {
    return GFM_ERR_ARG;
  }
  host_bcs(d, U1);
  host_bcs(d, U2);
  return GFM_OK;
}

// Volume fraction of fluid 1 for the VOF interface tracker: the zval of
// set_sim_ICs (10x10 sub-sampled area fractions for circles,
// sourcecode/sim_twofluid.cpp:646-668,825-856; the clipped linear profiles of
// the planar tubes, :697,731; z = 1 for GDA, :769).
gfm_status_t gfm_case_init_z(const char* test_case, const gfm_grid_desc* d, double* z) {
  if (!test_case || !d || !z) return GFM_ERR_ARG;
  std::string tc(test_case);
  Geo G = geo_of(d);
  auto clip01 = [](double v) { return std::min(1.0, std::max(0.0, v)); };
  for (int i = 0; i < G.nr; i++)
    for (int j = 0; j < G.nc; j++) {
      const double x = G.ccx(j), y = G.ccy(i);
      double v;
      if (tc == "circularexplosion") v = area_fraction(G, i, j, 1.0, 1.0, 0.4);
      else if (tc == "ST1_x") v = clip01((0.5 - x + 0.5 * G.dx) / G.dx);
      else if (tc == "ST2_y") v = clip01((0.7 - y + 0.5 * G.dy) / G.dy);
      else if (tc == "GDA") v = 1.0;
      else if (tc == "shocked_helium_bubble") v = area_fraction(G, i, j, 175.0, 44.5, 25.0);
      else if (tc == "shocked_R22_bubble") v = area_fraction(G, i, j, 0.225, 0.0445, 0.025);
      else if (tc == "shock_bubble") v = area_fraction(G, i, j, 0.175, 0.0445, 0.025);
      else if (tc == "underwater_explosion_sg") v = area_fraction(G, i, j, 0.0, 0.0, 0.2);
      else return GFM_ERR_ARG;
      z[(size_t)i * G.nc + j] = v;
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
  Geo G = geo_of(d);
  const double W = d->dx * d->Nx, H = d->dy * d->Ny;
  const double xc = 0.7 * W, yc = 0.5 * H, r = p->radius_frac * H, xs = 0.9 * W;
  double rho2, u2, p2;
  post_shock(d->gamma2, p->mach, 1.0, 1e5, rho2, u2, p2);
  const V4 bub = p2c(d->gamma1, d->pinf1, p->rho_ratio, 0, 0, 1e5);
  const V4 pre = p2c(d->gamma2, d->pinf2, 1.0, 0, 0, 1e5), post = p2c(d->gamma2, d->pinf2, rho2, u2, 0, p2);
  for (int i = 0; i < G.nr; i++)
    for (int j = 0; j < G.nc; j++) {
      const double x = G.ccx(j), y = G.ccy(i);
      put(G, U1, i, j, bub);
      put(G, U2, i, j, (x < xs) ? pre : post);
      phi[(size_t)i * G.nc + j] = std::sqrt((x - xc) * (x - xc) + (y - yc) * (y - yc)) - r;
    }
  host_bcs(d, U1);
  host_bcs(d, U2);
  return GFM_OK;
}

}  // extern "C"
