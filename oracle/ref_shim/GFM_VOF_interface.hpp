// TEST INFRASTRUCTURE -- stand-in for PhD-Interface-tracking-methods'
// GFM_VOF_interface.hpp: what GFM_VOF and OGFM_VOF take from a VOF tracker
// (sourcecode/GFM_VOF.cpp:20,54,103-104; sourcecode/OGFM_VOF.cpp:23,140-141).
#pragma once

#include "Eigen/Dense"

class GFM_VOF_interface {
 public:
  virtual ~GFM_VOF_interface() {}
  virtual double get_z(int i, int j) const = 0;
  virtual Eigen::Vector2d get_mixedcell_normal(int i, int j) const = 0;
  virtual Eigen::Vector2d get_interfacelocation(int i, int j) const = 0;
};
