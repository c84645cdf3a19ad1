// Per-cell initial conditions of the named test cases, shared by the host
// set-up (gfm_cases.cpp) and the device set-up (gfm_cases_dev.cu): one
// definition of every case's state, level set and volume fraction, evaluated
// with the same operations on either side.
//
// The reference's set_sim_ICs (sourcecode/sim_twofluid.cpp:599-1799,
// sourcecode/sim_onefluid.cpp:196-449) fills every padded cell from the
// cell-centre coordinate; circles take 10x10 sub-sampled area fractions
// (e.g. :825-856), planar tubes a clipped linear profile (:697, :731).
#pragma once

#include <cmath>

#include "gfm_math.cuh"

namespace gfm {

struct CaseGeo {
  int Nx, Ny, g, nr, nc;
  double x0, y0, dx, dy;
  GFM_HD double ccx(int j) const { return x0 + ((double)(j - g) + 0.5) * dx; }
  GFM_HD double ccy(int i) const { return y0 + ((double)(i - g) + 0.5) * dy; }
};

// fraction of 10x10 sub-samples of cell (i,j) within radius R of (cx, cy)
GFM_HD double area_fraction(const CaseGeo& G, int i, int j, double cx, double cy, double R) {
  const int N = 10;
  int inside = 0;
  const double delx = G.dx / N, dely = G.dy / N;
  const double blx = G.ccx(j) - 0.5 * G.dx, bly = G.ccy(i) - 0.5 * G.dy;
  for (int a = 0; a < N; a++)
    for (int b = 0; b < N; b++) {
      const double sx = blx + (a + 0.5) * delx - cx;
      const double sy = bly + (b + 0.5) * dely - cy;
      if (sqrt(sx * sx + sy * sy) <= R) inside++;
    }
  return double(inside) / (N * N);
}

// std::min(1.0, std::max(0.0, v)) with the library's operand order
GFM_HD double clip01(double v) {
  const double m = (0.0 < v) ? v : 0.0;
  return (m < 1.0) ? m : 1.0;
}

// exp of the Gaussian density of GDA: the C library's on the host (the
// reference's call), this library's table-driven gfm_exp on the device
GFM_HD double case_exp(double x) {
#if defined(__CUDA_ARCH__)
  return gfm_exp(x);
#else
  return std::exp(x);
#endif
}

enum {
  CASE_PLANAR = 0,        // one fluid: L where x a + y b <= c, else R
  CASE_BLEND_CIRCLE = 1,  // one fluid: prims frac L + (1 - frac) R, frac = area fraction of the circle
  CASE_CIRCLE = 2,        // two fluids: fluid 1 inside the circle
  CASE_PLANE_X = 3,       // two fluids: fluid 1 where x < c
  CASE_PLANE_Y = 4,       // two fluids: fluid 1 where y < c
  CASE_GDA = 5,           // two fluids: Gaussian density in uniform flow, fluid 1 everywhere
};

struct CaseSpec {
  int kind;
  double g1, q1, g2, q2;   // gamma, pinf of each fluid
  V4 s1;                   // fluid-1 state (conserved)
  V4 s2a, s2b;             // fluid-2 state where x < xsplit / elsewhere
  double xsplit;
  V4 L, R;                 // one fluid: planar states (conserved) or blend primitives
  double pa, pb, pc;       // planar: x pa + y pb <= pc
  double cx, cy, r;        // circle
  double c;                // plane position
};

// the state of cell (i,j): U1 (and U2, phi, z for two fluids)
GFM_HD void case_cell(const CaseSpec& s, const CaseGeo& G, int i, int j, bool want_z, V4& u1, V4& u2, double& phi,
                      double& z) {
  const double x = G.ccx(j), y = G.ccy(i);
  z = 0.0;
  switch (s.kind) {
    case CASE_PLANAR:
      u1 = (x * s.pa + y * s.pb <= s.pc) ? s.L : s.R;
      return;
    case CASE_BLEND_CIRCLE: {
      const double frac = area_fraction(G, i, j, s.cx, s.cy, s.r);
      const V4 W = V4{frac * s.L.a + (1.0 - frac) * s.R.a, frac * s.L.b + (1.0 - frac) * s.R.b,
                      frac * s.L.c + (1.0 - frac) * s.R.c, frac * s.L.d + (1.0 - frac) * s.R.d};
      u1 = prims_to_cons(s.g1, s.q1, W, nullptr);
      return;
    }
    case CASE_GDA: {
      const double r2 = (x - 0.5) * (x - 0.5) + (y - 0.5) * (y - 0.5);
      u1 = prims_to_cons(s.g1, s.q1, V4{1.0 + 1000.0 * case_exp(-r2 / (2.0 * 0.1 * 0.1)), 1.0, 1.0, 0.0001}, nullptr);
      u2 = u1;
      phi = -1.0;
      z = 1.0;
      return;
    }
    default:
      break;
  }
  u1 = s.s1;
  u2 = (x < s.xsplit) ? s.s2a : s.s2b;
  if (s.kind == CASE_CIRCLE) {
    phi = sqrt((x - s.cx) * (x - s.cx) + (y - s.cy) * (y - s.cy)) - s.r;
    if (want_z) z = area_fraction(G, i, j, s.cx, s.cy, s.r);
  } else if (s.kind == CASE_PLANE_X) {
    phi = x - s.c;
    z = clip01((s.c - x + 0.5 * G.dx) / G.dx);
  } else {
    phi = y - s.c;
    z = clip01((s.c - y + 0.5 * G.dy) / G.dy);
  }
}

}  // namespace gfm
