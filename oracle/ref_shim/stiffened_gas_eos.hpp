// TEST INFRASTRUCTURE -- stand-in for PhD-Common's stiffened_gas_eos.hpp
// (absent from the reference's repository): the two materials' parameters
// and the stiffened-gas equation of state eos::pressure, specific_ie,
// soundspeed and isentropic_extrapolation, which are the oracle's own
// (oracle_math.hpp; same argument order as the reference's call sites,
// e.g. headers/euler_misc.hpp:46,59,77,96).
#pragma once

#include "../oracle_math.hpp"

struct binarySGparams {
  double gamma1 = 1.4, gamma2 = 1.4, pinf1 = 0.0, pinf2 = 0.0;
};
