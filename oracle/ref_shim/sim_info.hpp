// TEST INFRASTRUCTURE -- stand-in for PhD-Common's sim_info.hpp (absent from
// the reference's repository): grid geometry, boundary-condition names and
// the end time, with the cell-centre coordinate of grid[i][j] defined as the
// oracle defines it (oracle_itm.hpp).
#pragma once

#include <string>

#include "../oracle_itm.hpp"
#include "Eigen/Dense"

class sim_info {
 public:
  int Nx = 0, Ny = 0, numGC = 0;
  int output_freq = 0;
  double x0 = 0.0, y0 = 0.0, dx = 0.0, dy = 0.0;
  double T = 0.0;
  std::string BC_L, BC_R, BC_B, BC_T;

  // the same geometry with the boundary conditions as GFM_BC_* codes
  oitm::sim_info as_oracle() const {
    oitm::sim_info p;
    p.Nx = Nx; p.Ny = Ny; p.numGC = numGC;
    p.x0 = x0; p.y0 = y0; p.dx = dx; p.dy = dy;
    p.BC_L = bc_code(BC_L); p.BC_R = bc_code(BC_R); p.BC_B = bc_code(BC_B); p.BC_T = bc_code(BC_T);
    return p;
  }

  Eigen::Vector2d cellcentre_coord(int i, int j) const {
    const oitm::vec2 c = as_oracle().cellcentre_coord(i, j);
    return Eigen::Vector2d(c[0], c[1]);
  }

  static int bc_code(const std::string& s) {
    if (s == "reflective") return oitm::BC_REFLECTIVE;
    if (s == "periodic") return oitm::BC_PERIODIC;
    return oitm::BC_TRANSMISSIVE;
  }
};
