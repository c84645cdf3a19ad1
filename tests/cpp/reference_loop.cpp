// The reference's time loop written against the C++ class surface
// (include/gfm_gb300.hpp) as a maintainer of the reference would write it:
// the body of sim_twofluid::run_sim (sourcecode/sim_twofluid.cpp:64-88) and
// sim_onefluid::run_sim (sourcecode/sim_onefluid.cpp:40-54) with the
// strategy objects of set_sim_methods, on host grids.
//
//   reference_loop loop     <settingsfile> <result>   two-fluid loop, SF.nsteps steps
//   reference_loop onefluid <settingsfile> <result>   one-fluid loop, SF.nsteps steps
//   reference_loop run_sim  <settingsfile>            sim_*::run_sim (output files)
//   reference_loop basename <settingsfile>            the settings file's basename (host only)
//
// Result file: int32 nr, nc, numsteps, 0; float64 t; int32 realcells1[4],
// realcells2[4]; float64 planes U1[4], U2[4], phi (or z) of nr x nc each.
#include <cstdio>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "gfm_gb300.hpp"

using namespace gfm_gb300;

static void write_result(const std::string& path, const sim_info& params, int numsteps, double t, const BBrange& rc1,
                         const BBrange& rc2, const grideuler2type& grid1, const grideuler2type* grid2,
                         const std::vector<double>* field) {
  std::ofstream out(path, std::ios::binary);
  const int nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
  const int h[4] = {nr, nc, numsteps, 0};
  out.write(reinterpret_cast<const char*>(h), sizeof(h));
  out.write(reinterpret_cast<const char*>(&t), sizeof(t));
  const int rc[8] = {rc1.imin, rc1.imax, rc1.jmin, rc1.jmax, rc2.imin, rc2.imax, rc2.jmin, rc2.jmax};
  out.write(reinterpret_cast<const char*>(rc), sizeof(rc));
  std::vector<double> U;
  grid_to_planes(grid1, U);
  out.write(reinterpret_cast<const char*>(U.data()), 8 * U.size());
  if (grid2) {
    grid_to_planes(*grid2, U);
    out.write(reinterpret_cast<const char*>(U.data()), 8 * U.size());
    out.write(reinterpret_cast<const char*>(field->data()), 8 * field->size());
  }
}

static int twofluid_loop(const GFM_settingsfile& SF, const std::string& result) {
  sim_twofluid sim;
  sim_info params;
  binarySGparams eosparams;
  sim.set_sim_parameters(SF, params, eosparams);
  std::shared_ptr<FS_base> FS;
  std::shared_ptr<GFM_base> GFM;
  std::shared_ptr<GFM_ITM_interface> ls;
  sim.set_sim_methods(SF, params, FS, GFM, ls);
  grideuler2type grid1, grid2;
  sim.set_sim_ICs(SF, params, eosparams, grid1, grid2, *ls);
  ls->initialisation();
  grideuler2type future_grid1 = grid1, future_grid2 = grid2;
  BBrange realcells1(params.numGC, params.Ny + params.numGC, params.numGC, params.Nx + params.numGC);
  BBrange realcells2(params.numGC, params.Ny + params.numGC, params.numGC, params.Nx + params.numGC);

  int numsteps = 0;
  double t = 0.0, CFL, dt;
  while (t < params.T && numsteps < SF.nsteps) {
    CFL = (numsteps < 5) ? std::min(SF.CFL, 0.2) : SF.CFL;
    dt = sim.compute_dt(CFL, params, grid1, grid2, *ls, eosparams, params.T, t);
    GFM->set_ghost_states(params, *ls, eosparams, t, grid1, grid2, realcells1, realcells2);
    FS->pure_fluid_update(params, eosparams.gamma1, eosparams.pinf1, dt, realcells1, grid1, future_grid1);
    FS->pure_fluid_update(params, eosparams.gamma2, eosparams.pinf2, dt, realcells2, grid2, future_grid2);
    ls->update_interface_coupled(*(GFM->vfield), t, dt);
    apply_BCs_euler(params, grid1);
    apply_BCs_euler(params, grid2);
    numsteps++;
    t += dt;
  }
  write_result(result, params, numsteps, t, realcells1, realcells2, grid1, &grid2, &ls->field());
  return 0;
}

static int onefluid_loop(const GFM_settingsfile& SF, const std::string& result) {
  sim_onefluid sim;
  sim_info params;
  binarySGparams eosparams;
  sim.set_sim_parameters(SF, params, eosparams);
  std::shared_ptr<pure_RS_base> RS;
  std::shared_ptr<FS_base> FS;
  sim.set_sim_methods(SF, RS, FS);
  grideuler2type grid;
  sim.set_sim_ICs(SF, params, eosparams, grid);
  grideuler2type future_grid = grid;
  BBrange realcells(params.numGC, params.Ny + params.numGC, params.numGC, params.Nx + params.numGC);
  int numsteps = 0;
  double t = 0.0;
  while (t < params.T && numsteps < SF.nsteps) {
    const double CFL = (numsteps < 5) ? std::min(SF.CFL, 0.2) : SF.CFL;
    const double dt = sim.compute_dt(CFL, params, grid, eosparams, params.T, t);
    FS->pure_fluid_update(params, eosparams.gamma1, eosparams.pinf1, dt, realcells, grid, future_grid);
    apply_BCs_euler(params, grid);
    numsteps++;
    t += dt;
  }
  write_result(result, params, numsteps, t, realcells, realcells, grid, nullptr, nullptr);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: reference_loop loop|onefluid|run_sim <settingsfile> [result]\n");
    return 2;
  }
  const std::string mode = argv[1];
  GFM_settingsfile SF;
  try {
    SF.read_settings_file(argv[2]);
    if (mode == "loop" && argc == 4) return twofluid_loop(SF, argv[3]);
    if (mode == "onefluid" && argc == 4) return onefluid_loop(SF, argv[3]);
    if (mode == "basename") {
      std::printf("%s\n", SF.basename.c_str());
      return 0;
    }
    if (mode == "run_sim") {
      std::unique_ptr<sim_base> sim;
      if (SF.sim_type == "onefluid") sim.reset(new sim_onefluid());
      else sim.reset(new sim_twofluid());
      sim->run_sim(SF);
      return 0;
    }
  } catch (const numeric_error& e) {
    std::fprintf(stderr, "numeric_error: %s (status 0x%x)\n", e.what(), e.status());
    return 3;
  } catch (const error& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 4;
  }
  std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
  return 2;
}
