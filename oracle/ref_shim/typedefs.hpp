// TEST INFRASTRUCTURE -- stand-in for PhD-Common's typedefs.hpp, which the
// reference includes from outside its repository (Makefile:17-27): the
// state vector, the quasilinear matrix and the nested-vector grids
// grid[i][j] (row i = y index) that the reference's signatures use.
#pragma once

#include <cassert>
#include <chrono>
#include <vector>
#include "Eigen/Dense"

// The reference times its loop with OpenMP's omp_get_wtime
// (sourcecode/sim_twofluid.cpp:62,90) and reaches it through these shared
// headers; a steady clock stands in for it.
inline double omp_get_wtime() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

typedef Eigen::Vector4d vec4type;
typedef Eigen::Matrix4d matrix4d;
typedef std::vector<vec4type, Eigen::aligned_allocator<vec4type>> roweuler2type;
typedef std::vector<roweuler2type> grideuler2type;
typedef std::vector<std::vector<Eigen::Vector2d, Eigen::aligned_allocator<Eigen::Vector2d>>> gridVector2dtype;
typedef std::vector<std::vector<double>> griddoubletype;
