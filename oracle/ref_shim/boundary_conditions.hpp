// TEST INFRASTRUCTURE -- stand-in for PhD-Common's boundary_conditions.hpp
// (absent from the reference's repository): apply_gridVector2dtype_BCs, the
// velocity field's ghost layers as the oracle defines them (mirror copy of
// both components, gfm_oracle.cpp extrapolate_extension_vfield).
#pragma once

#include "sim_info.hpp"
#include "typedefs.hpp"

inline void apply_gridVector2dtype_BCs(const sim_info& params, gridVector2dtype& grid) {
  const int g = params.numGC, Nx = params.Nx, Ny = params.Ny;
  for (int i = g; i < Ny + g; i++)
    for (int j = 0; j < g; j++) {
      grid[i][j] = grid[i][2 * g - j - 1];
      grid[i][j + Nx + g] = grid[i][Nx + g - 1 - j];
    }
  for (int j = 0; j < Nx + 2 * g; j++)
    for (int i = 0; i < g; i++) {
      grid[i][j] = grid[2 * g - i - 1][j];
      grid[i + Ny + g][j] = grid[Ny + g - 1 - i][j];
    }
}
