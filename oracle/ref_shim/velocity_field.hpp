// TEST INFRASTRUCTURE -- stand-in for PhD-Interface-tracking-methods'
// velocity_field.hpp (absent from the reference's repository).  The ghost-fluid
// methods store the composite velocity field of each ghost fill
// (vfield->store_velocity_field, e.g. sourcecode/GFM_riemann.cpp:176) and the
// interface tracker advects with it; here the stored field is the grid
// itself, at cell centres, as the oracle hands it to its level set.
#pragma once

#include <cmath>

#include "Eigen/Dense"
#include "sim_info.hpp"
#include "typedefs.hpp"

class velocity_field_base {
 public:
  virtual ~velocity_field_base() {}
  virtual Eigen::Vector2d get_velocity(const Eigen::Vector2d& x, double t) const = 0;
};

class solved_velocity_field_base : public velocity_field_base {
 public:
  virtual void store_velocity_field(const gridVector2dtype& velocities, double t) = 0;
  virtual const gridVector2dtype& stored() const = 0;
};

// the stored grid; get_velocity returns the value of the cell containing x
class solved_velocity_field_firstorder : public solved_velocity_field_base {
 public:
  explicit solved_velocity_field_firstorder(const sim_info& params) : params_(params) {}
  void store_velocity_field(const gridVector2dtype& velocities, double) override { vel_ = velocities; }
  const gridVector2dtype& stored() const override { return vel_; }
  Eigen::Vector2d get_velocity(const Eigen::Vector2d& x, double) const override {
    const int j = static_cast<int>(std::floor((x(0) - params_.x0) / params_.dx)) + params_.numGC;
    const int i = static_cast<int>(std::floor((x(1) - params_.y0) / params_.dy)) + params_.numGC;
    return vel_[i][j];
  }

 private:
  sim_info params_;
  gridVector2dtype vel_;
};
