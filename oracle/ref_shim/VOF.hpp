// TEST INFRASTRUCTURE -- stand-in for PhD-Interface-tracking-methods' VOF.hpp
// (settings ITM "PYVOF", sourcecode/sim_twofluid.cpp:575-579), backed by the
// oracle's VOF tracker (oitm::VOFTracker in oracle_itm.hpp): z is the volume
// fraction of fluid 1 and get_sdf = 0.5 - z.
#pragma once

#include "../oracle_itm.hpp"
#include "GFM_ITM_interface.hpp"
#include "GFM_VOF_interface.hpp"
#include "levelset.hpp"
#include "sim_info.hpp"

class VOF : public GFM_ITM_interface, public GFM_VOF_interface {
 public:
  explicit VOF(const sim_info& params) {
    vof_.params = params.as_oracle();
    const int nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
    vof_.z.assign(nr, std::vector<double>(nc, 0.0));
  }
  void set_steps(int steps_so_far) { vof_.steps = steps_so_far; }
  double get_sdf(int i, int j) const override { return vof_.get_sdf(i, j); }
  void set_sdf(int, int, double) override {}
  double get_z(int i, int j) const override { return vof_.get_z(i, j); }
  void set_z(int i, int j, double v) override { vof_.z[i][j] = v; }
  Eigen::Vector2d get_normal(const Eigen::Vector2d&) const override {
    std::fprintf(stderr, "VOF::get_normal: not used by the VOF ghost-fluid methods\n");
    std::abort();
  }
  bool is_interfacial_cell(int i, int j) const override {
    const double z = vof_.z[i][j];
    return z > 0.0 && z < 1.0;
  }
  Eigen::Vector2d get_mixedcell_normal(int i, int j) const override {
    const oitm::vec2 n = vof_.get_mixedcell_normal(i, j);
    return Eigen::Vector2d(n[0], n[1]);
  }
  Eigen::Vector2d get_interfacelocation(int i, int j) const override {
    const oitm::vec2 x = vof_.get_interfacelocation(i, j);
    return Eigen::Vector2d(x[0], x[1]);
  }
  void initialisation() override {}
  void update_interface_coupled(const velocity_field_base& vfield, double, double dt) override {
    const auto& sv = dynamic_cast<const solved_velocity_field_base&>(vfield);
    vof_.update_interface_coupled(Levelset::as_oracle_grid(sv.stored()), dt);
  }
  const oitm::griddoubletype& z() const { return vof_.z; }

 private:
  oitm::VOFTracker vof_;
};
