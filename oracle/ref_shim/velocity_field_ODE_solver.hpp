// TEST INFRASTRUCTURE -- stand-in for PhD-Interface-tracking-methods'
// velocity_field_ODE_solver.hpp.  The reference uses time_step_RK4 only to
// move the tracer points of its RMI perturbation diagnostic
// (sourcecode/sim_twofluid.cpp:1879-1880), which the checker never runs.
#pragma once

#include <cstdio>
#include <cstdlib>

#include "velocity_field.hpp"

inline void time_step_RK4(const velocity_field_base&, double, double, const Eigen::Vector2d&, Eigen::Vector2d&) {
  std::fprintf(stderr, "time_step_RK4: not part of the checked path\n");
  std::abort();
}
