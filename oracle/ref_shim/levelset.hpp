// TEST INFRASTRUCTURE -- stand-in for PhD-Interface-tracking-methods'
// levelset.hpp (absent from the reference's repository): the reference's
// Levelset(params, order[, k]) (sourcecode/sim_twofluid.cpp:555-570) backed
// by the oracle's level set (oitm::Levelset in oracle_itm.hpp).
//   get_normal(x)   the central-difference gradient of phi at the cell whose
//                   centre is x (the reference calls it at cell centres only;
//                   anything else aborts)
//   get_z           the indicator of fluid 1 (phi <= 0)
//   initialisation  nothing: the initial conditions set phi in every cell
// The reinitialisation schedule (every k steps, n iterations) is set by the
// checker's driver from the run's method description.
#pragma once

#include <cstdio>
#include <cstdlib>

#include "../oracle_itm.hpp"
#include "GFM_ITM_interface.hpp"
#include "sim_info.hpp"

class Levelset : public GFM_ITM_interface {
 public:
  Levelset(const sim_info& params, int order, int /*k*/ = 1) : params_(params) {
    ls_.params = params.as_oracle();
    ls_.order = order;
    const int nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
    ls_.phi.assign(nr, std::vector<double>(nc, 0.0));
  }
  void configure(int reinit_every, int reinit_iters, int updates_so_far) {
    ls_.reinit_every = reinit_every;
    ls_.reinit_iters = reinit_iters;
    ls_.updates = updates_so_far;
  }
  double get_sdf(int i, int j) const override { return ls_.get_sdf(i, j); }
  void set_sdf(int i, int j, double v) override { ls_.phi[i][j] = v; }
  double get_z(int i, int j) const override { return ls_.phi[i][j] <= 0.0 ? 1.0 : 0.0; }
  void set_z(int, int, double) override {}
  Eigen::Vector2d get_normal(const Eigen::Vector2d& x) const override {
    const int j = static_cast<int>(std::floor((x(0) - params_.x0) / params_.dx)) + params_.numGC;
    const int i = static_cast<int>(std::floor((x(1) - params_.y0) / params_.dy)) + params_.numGC;
    const Eigen::Vector2d cc = params_.cellcentre_coord(i, j);
    if (!(cc(0) == x(0) && cc(1) == x(1))) {
      std::fprintf(stderr, "Levelset::get_normal: (%.17g, %.17g) is not a cell centre\n", x(0), x(1));
      std::abort();
    }
    const oitm::vec2 n = ls_.get_normal(i, j);
    return Eigen::Vector2d(n[0], n[1]);
  }
  bool is_interfacial_cell(int i, int j) const override { return ls_.is_interfacial_cell(i, j); }
  void initialisation() override {}
  void update_interface_coupled(const velocity_field_base& vfield, double, double dt) override {
    const auto& sv = dynamic_cast<const solved_velocity_field_base&>(vfield);
    ls_.update_interface_coupled(as_oracle_grid(sv.stored()), dt);
  }
  const oitm::griddoubletype& phi() const { return ls_.phi; }

  static oitm::gridVector2dtype as_oracle_grid(const gridVector2dtype& v) {
    oitm::gridVector2dtype o(v.size());
    for (size_t i = 0; i < v.size(); i++) {
      o[i].resize(v[i].size());
      for (size_t j = 0; j < v[i].size(); j++) o[i][j] = {v[i][j](0), v[i][j](1)};
    }
    return o;
  }

 private:
  sim_info params_;
  oitm::Levelset ls_;
};
