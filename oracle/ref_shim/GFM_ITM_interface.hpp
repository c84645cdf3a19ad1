// TEST INFRASTRUCTURE -- stand-in for PhD-Interface-tracking-methods'
// GFM_ITM_interface.hpp (absent from the reference's repository): the
// interface-tracker interface that the reference's ghost-fluid methods, flux
// loop and drivers call (get_sdf / set_sdf, get_z / set_z, get_normal at a
// position, is_interfacial_cell, initialisation, update_interface_coupled;
// call sites e.g. sourcecode/GFM_riemann.cpp:55-58, sourcecode/sim_twofluid.cpp:47,72).
#pragma once

#include "Eigen/Dense"
#include "velocity_field.hpp"

class GFM_ITM_interface {
 public:
  virtual ~GFM_ITM_interface() {}
  virtual double get_sdf(int i, int j) const = 0;
  virtual void set_sdf(int i, int j, double v) = 0;
  virtual double get_z(int i, int j) const = 0;
  virtual void set_z(int i, int j, double v) = 0;
  virtual Eigen::Vector2d get_normal(const Eigen::Vector2d& x) const = 0;
  virtual bool is_interfacial_cell(int i, int j) const = 0;
  virtual void initialisation() = 0;
  virtual void update_interface_coupled(const velocity_field_base& vfield, double t, double dt) = 0;
};
