// TEST INFRASTRUCTURE -- stand-in for PhD-Common's interpolation.hpp (absent
// from the reference's repository): grid_bilinear_interpolate in the four
// cell centres around x, with the oracle's cell, weights and sum order
// (oracle_itm.hpp, gfm_oracle.cpp).
#pragma once

#include <vector>

#include "../oracle_itm.hpp"
#include "Eigen/Dense"
#include "sim_info.hpp"

template <typename T>
T grid_bilinear_interpolate(const sim_info& params, const std::vector<std::vector<T, Eigen::aligned_allocator<T>>>& grid,
                            const Eigen::Vector2d& x) {
  int i0, j0;
  double a, b;
  oitm::bilinear_cell(params.as_oracle(), oitm::vec2{x(0), x(1)}, i0, j0, a, b);
  T out;
  for (int k = 0; k < out.size(); k++)
    out(k) = ((1.0 - a) * (1.0 - b)) * grid[i0][j0](k) + (a * (1.0 - b)) * grid[i0][j0 + 1](k) +
             ((1.0 - a) * b) * grid[i0 + 1][j0](k) + (a * b) * grid[i0 + 1][j0 + 1](k);
  return out;
}
