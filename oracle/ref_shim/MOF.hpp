// TEST INFRASTRUCTURE -- stand-ins for the moment-of-fluid and coupled
// level-set/VOF trackers of PhD-Interface-tracking-methods (settings ITM MOF,
// EMOF2, CLSVOF; sourcecode/sim_twofluid.cpp:571-589).  They are outside the
// checked path: constructing one aborts.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <memory>

#include "GFM_ITM_interface.hpp"
#include "sim_info.hpp"

class untracked_interface : public GFM_ITM_interface {
 public:
  explicit untracked_interface(const char* name) {
    std::fprintf(stderr, "%s: this interface tracker is outside the checked path\n", name);
    std::abort();
  }
  double get_sdf(int, int) const override { return 0.0; }
  void set_sdf(int, int, double) override {}
  double get_z(int, int) const override { return 0.0; }
  void set_z(int, int, double) override {}
  Eigen::Vector2d get_normal(const Eigen::Vector2d&) const override { return Eigen::Vector2d(1.0, 0.0); }
  bool is_interfacial_cell(int, int) const override { return false; }
  void initialisation() override {}
  void update_interface_coupled(const velocity_field_base&, double, double) override {}
};

class EMOF2_reconstruction {
 public:
  EMOF2_reconstruction(int, int) {}
};

class MOF : public untracked_interface {
 public:
  explicit MOF(const sim_info&) : untracked_interface("MOF") {}
  MOF(const sim_info&, std::shared_ptr<EMOF2_reconstruction>) : untracked_interface("MOF") {}
};

class CLSVOF : public untracked_interface {
 public:
  explicit CLSVOF(const sim_info&) : untracked_interface("CLSVOF") {}
};
