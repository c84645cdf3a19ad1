// TEST INFRASTRUCTURE -- the driver of the reference checker (oracle/_ref).
// Only tests/ may run it, and only as a checker of the oracle.
//
// Runs the reference's OWN classes and functions, compiled unchanged from
// murraycutforth/PhD-2D-GFM's sourcecode/ and headers/ against the stand-in
// headers in ref_shim/ (build_ref.py): sim_twofluid::set_sim_parameters,
// set_sim_methods, set_sim_ICs and compute_dt, the GFM_* classes, FS_MUSCL /
// FS_godunov, pure_RS_exact / mixed_RS_exact, extrapolate_vector and
// apply_BCs_euler.  The step loop is the body of sim_twofluid::run_sim
// (sourcecode/sim_twofluid.cpp:64-88) and sim_onefluid::run_sim
// (sourcecode/sim_onefluid.cpp:40-54) without the file output.
//
// Usage: gfm_ref <request file> <result file>
// The request is "key value" lines:
//   sim_type twofluid|onefluid   FS, GFM, ITM (settings-file names)
//   CFL, nsteps, reinit_every, reinit_iters
//   test_case <name>             the reference's own parameters and initial
//                                conditions (two-fluid), or
//   state <path>                 a state file (layout below) with the grid
//                                description keys Nx Ny numGC x0 y0 dx dy
//                                BC_L BC_R BC_B BC_T gamma1 pinf1 gamma2
//                                pinf2 T
// State and result files: little-endian int32 nr, nc, numsteps, 0; float64 t;
// int32 realcells1[4], realcells2[4] (imin, imax, jmin, jmax); then the
// planes (nr x nc float64 each) U1[4], U2[4], phi (or z for the VOF
// tracker); the result adds two interfacial-cell masks (nr x nc uint8 each,
// real cells only; level set only): that of the final phi and that of the
// last step's ghost fill (Levelset::is_interfacial_cell as the ghost fill
// saw it), and int64 Newton iterations.  A state file holds the same planes (its header's realcells
// are ignored).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "BBrange.hpp"
#include "FS_MUSCL.hpp"
#include "FS_godunov.hpp"
#include "GFM_settingsfile.hpp"
#include "VOF.hpp"
#include "euler_bc.hpp"
#include "exact_RS_stiffenedgas.hpp"
#include "levelset.hpp"
#include "pure_RS_exact.hpp"
#include "sim_onefluid.hpp"
#include "sim_twofluid.hpp"

namespace {

// sim_twofluid's set-up steps are protected members: a subclass reaches them.
class twofluid_driver : public sim_twofluid {
 public:
  using sim_twofluid::set_sim_ICs;
  using sim_twofluid::set_sim_methods;
  using sim_twofluid::set_sim_parameters;
};

[[noreturn]] void fail(const std::string& msg) {
  std::fprintf(stderr, "gfm_ref: %s\n", msg.c_str());
  std::exit(2);
}

std::map<std::string, std::string> read_request(const char* path) {
  std::ifstream in(path);
  if (!in) fail(std::string("cannot read ") + path);
  std::map<std::string, std::string> kv;
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream is(line);
    std::string k, v;
    if (is >> k >> v) kv[k] = v;
  }
  return kv;
}

std::string get(const std::map<std::string, std::string>& kv, const char* k, const char* dflt = nullptr) {
  auto it = kv.find(k);
  if (it != kv.end()) return it->second;
  if (dflt) return dflt;
  fail(std::string("request lacks ") + k);
}

struct Planes {
  int nr = 0, nc = 0, numsteps = 0;
  double t = 0.0;
  std::vector<double> U1, U2, phi;
};

Planes read_state(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) fail("cannot read " + path);
  Planes s;
  int32_t h[4];
  in.read(reinterpret_cast<char*>(h), sizeof(h));
  in.read(reinterpret_cast<char*>(&s.t), sizeof(double));
  int32_t rc[8];
  in.read(reinterpret_cast<char*>(rc), sizeof(rc));
  s.nr = h[0]; s.nc = h[1]; s.numsteps = h[2];
  const size_t plane = static_cast<size_t>(s.nr) * s.nc;
  s.U1.resize(4 * plane); s.U2.resize(4 * plane); s.phi.resize(plane);
  in.read(reinterpret_cast<char*>(s.U1.data()), 8 * s.U1.size());
  in.read(reinterpret_cast<char*>(s.U2.data()), 8 * s.U2.size());
  in.read(reinterpret_cast<char*>(s.phi.data()), 8 * s.phi.size());
  if (!in) fail("truncated state file " + path);
  return s;
}

void to_grid(const std::vector<double>& U, int nr, int nc, grideuler2type& g) {
  const size_t plane = static_cast<size_t>(nr) * nc;
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++)
      for (int k = 0; k < 4; k++) g[i][j](k) = U[k * plane + static_cast<size_t>(i) * nc + j];
}

void from_grid(const grideuler2type& g, int nr, int nc, std::vector<double>& U) {
  const size_t plane = static_cast<size_t>(nr) * nc;
  U.assign(4 * plane, 0.0);
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++)
      for (int k = 0; k < 4; k++) U[k * plane + static_cast<size_t>(i) * nc + j] = g[i][j](k);
}

void params_from_request(const std::map<std::string, std::string>& kv, sim_info& p, binarySGparams& e) {
  p.Nx = std::stoi(get(kv, "Nx"));
  p.Ny = std::stoi(get(kv, "Ny"));
  p.numGC = std::stoi(get(kv, "numGC"));
  p.x0 = std::stod(get(kv, "x0"));
  p.y0 = std::stod(get(kv, "y0"));
  p.dx = std::stod(get(kv, "dx"));
  p.dy = std::stod(get(kv, "dy"));
  p.BC_L = get(kv, "BC_L");
  p.BC_R = get(kv, "BC_R");
  p.BC_B = get(kv, "BC_B");
  p.BC_T = get(kv, "BC_T");
  p.T = std::stod(get(kv, "T"));
  e.gamma1 = std::stod(get(kv, "gamma1"));
  e.pinf1 = std::stod(get(kv, "pinf1"));
  e.gamma2 = std::stod(get(kv, "gamma2", "1.4"));
  e.pinf2 = std::stod(get(kv, "pinf2", "0"));
}

void write_result(const std::string& path, const sim_info& p, int numsteps, double t, const BBrange& rc1,
                  const BBrange& rc2, const std::vector<double>& U1, const std::vector<double>& U2,
                  const std::vector<double>& phi, const std::vector<uint8_t>& mask,
                  const std::vector<uint8_t>& mask_fill, int64_t newton) {
  std::ofstream out(path, std::ios::binary);
  if (!out) fail("cannot write " + path);
  const int32_t h[4] = {p.Ny + 2 * p.numGC, p.Nx + 2 * p.numGC, numsteps, 0};
  out.write(reinterpret_cast<const char*>(h), sizeof(h));
  out.write(reinterpret_cast<const char*>(&t), sizeof(double));
  const int32_t rc[8] = {rc1.imin, rc1.imax, rc1.jmin, rc1.jmax, rc2.imin, rc2.imax, rc2.jmin, rc2.jmax};
  out.write(reinterpret_cast<const char*>(rc), sizeof(rc));
  out.write(reinterpret_cast<const char*>(U1.data()), 8 * U1.size());
  out.write(reinterpret_cast<const char*>(U2.data()), 8 * U2.size());
  out.write(reinterpret_cast<const char*>(phi.data()), 8 * phi.size());
  out.write(reinterpret_cast<const char*>(mask.data()), mask.size());
  out.write(reinterpret_cast<const char*>(mask_fill.data()), mask_fill.size());
  out.write(reinterpret_cast<const char*>(&newton), sizeof(newton));
  if (!out) fail("cannot write " + path);
}

int run_twofluid(const std::map<std::string, std::string>& kv, const std::string& result) {
  GFM_settingsfile SF;
  SF.sim_type = "twofluid";
  SF.FS = get(kv, "FS");
  SF.GFM = get(kv, "GFM");
  SF.ITM = get(kv, "ITM");
  SF.CFL = std::stod(get(kv, "CFL"));
  const int nsteps = std::stoi(get(kv, "nsteps"));
  const int reinit_every = std::stoi(get(kv, "reinit_every", "1"));
  const int reinit_iters = std::stoi(get(kv, "reinit_iters", "5"));

  twofluid_driver sim;
  sim_info params;
  binarySGparams eosparams;
  const std::string state = get(kv, "state", "");
  Planes st;
  if (state.empty()) {
    SF.test_case = get(kv, "test_case");
    SF.Nx = std::stoi(get(kv, "Nx"));
    SF.Ny = std::stoi(get(kv, "Ny"));
    sim.set_sim_parameters(SF, params, eosparams);
  } else {
    SF.test_case = "state-file";
    params_from_request(kv, params, eosparams);
    SF.Nx = params.Nx;
    SF.Ny = params.Ny;
    st = read_state(state);
    if (st.nr != params.Ny + 2 * params.numGC || st.nc != params.Nx + 2 * params.numGC)
      fail("state file does not match the grid description");
  }
  std::shared_ptr<FS_base> FS;
  std::shared_ptr<GFM_base> GFM;
  std::shared_ptr<GFM_ITM_interface> ls;
  sim.set_sim_methods(SF, params, FS, GFM, ls);
  GFM->use_extension_vfield = std::stoi(get(kv, "use_extension_vfield", "0")) != 0;
  GFM->use_slip_BCs = std::stoi(get(kv, "use_slip_BCs", "0")) != 0;

  const int nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
  grideuler2type grid1(nr, roweuler2type(nc)), future_grid1(nr, roweuler2type(nc));
  grideuler2type grid2(nr, roweuler2type(nc)), future_grid2(nr, roweuler2type(nc));
  BBrange realcells1(params.numGC, params.Ny + params.numGC, params.numGC, params.Nx + params.numGC);
  BBrange realcells2(params.numGC, params.Ny + params.numGC, params.numGC, params.Nx + params.numGC);
  int numsteps = 0;
  double t = 0.0;
  const bool vof = SF.ITM == "PYVOF";
  if (state.empty()) {
    sim.set_sim_ICs(SF, params, eosparams, grid1, grid2, *ls);
    ls->initialisation();
  } else {
    to_grid(st.U1, nr, nc, grid1);
    to_grid(st.U2, nr, nc, grid2);
    for (int i = 0; i < nr; i++)
      for (int j = 0; j < nc; j++) {
        const double v = st.phi[static_cast<size_t>(i) * nc + j];
        if (vof) ls->set_z(i, j, v);
        else ls->set_sdf(i, j, v);
      }
    numsteps = st.numsteps;
    t = st.t;
  }
  if (auto* L = dynamic_cast<Levelset*>(ls.get())) L->configure(reinit_every, reinit_iters, numsteps);
  if (auto* V = dynamic_cast<VOF*>(ls.get())) V->set_steps(numsteps);
  future_grid1 = grid1;
  future_grid2 = grid2;

  std::vector<uint8_t> mask_fill(static_cast<size_t>(nr) * nc, 0);
  auto interfacial_mask = [&](std::vector<uint8_t>& mask) {
    for (int i = 0; i < nr; i++)
      for (int j = 0; j < nc; j++) {
        const bool inner = i >= params.numGC && i < params.Ny + params.numGC && j >= params.numGC &&
                           j < params.Nx + params.numGC;
        mask[static_cast<size_t>(i) * nc + j] = (!vof && inner && ls->is_interfacial_cell(i, j)) ? 1 : 0;
      }
  };

  // the body of sim_twofluid::run_sim's time loop (sourcecode/sim_twofluid.cpp:64-88)
  int taken = 0;
  while (t < params.T && taken < nsteps) {
    const double CFL = (numsteps < 5) ? std::min(SF.CFL, 0.2) : SF.CFL;
    const double dt = sim.compute_dt(CFL, params, grid1, grid2, *ls, eosparams, params.T, t);
    interfacial_mask(mask_fill);
    ref_shim_mixed_solves = true;
    GFM->set_ghost_states(params, *ls, eosparams, t, grid1, grid2, realcells1, realcells2);
    ref_shim_mixed_solves = false;
    FS->pure_fluid_update(params, eosparams.gamma1, eosparams.pinf1, dt, realcells1, grid1, future_grid1);
    FS->pure_fluid_update(params, eosparams.gamma2, eosparams.pinf2, dt, realcells2, grid2, future_grid2);
    ls->update_interface_coupled(*(GFM->vfield), t, dt);
    apply_BCs_euler(params, grid1);
    apply_BCs_euler(params, grid2);
    numsteps++;
    t += dt;
    taken++;
  }

  std::vector<double> U1, U2, phi(static_cast<size_t>(nr) * nc);
  from_grid(grid1, nr, nc, U1);
  from_grid(grid2, nr, nc, U2);
  std::vector<uint8_t> mask(static_cast<size_t>(nr) * nc, 0);
  for (int i = 0; i < nr; i++)
    for (int j = 0; j < nc; j++) phi[static_cast<size_t>(i) * nc + j] = vof ? ls->get_z(i, j) : ls->get_sdf(i, j);
  interfacial_mask(mask);
  write_result(result, params, numsteps, t, realcells1, realcells2, U1, U2, phi, mask, mask_fill,
               ref_shim_newton_iters);
  return 0;
}

int run_onefluid(const std::map<std::string, std::string>& kv, const std::string& result) {
  // sim_onefluid's set-up members are private: the grid description and the
  // initial state come from the request, the time step, flux solver and
  // boundary conditions from the reference (sourcecode/sim_onefluid.cpp:40-54)
  sim_onefluid sim;
  sim_info params;
  binarySGparams eosparams;
  params_from_request(kv, params, eosparams);
  const double CFLset = std::stod(get(kv, "CFL"));
  const int nsteps = std::stoi(get(kv, "nsteps"));
  std::shared_ptr<pure_RS_base> RS = std::make_shared<pure_RS_exact>();
  std::shared_ptr<FS_base> FS;
  if (get(kv, "FS") == "MUSCL") FS = std::make_shared<FS_MUSCL>(RS);
  else FS = std::make_shared<FS_godunov>(RS);
  const int nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
  Planes st = read_state(get(kv, "state"));
  if (st.nr != nr || st.nc != nc) fail("state file does not match the grid description");
  grideuler2type grid(nr, roweuler2type(nc)), future_grid(nr, roweuler2type(nc));
  to_grid(st.U1, nr, nc, grid);
  future_grid = grid;
  BBrange realcells(params.numGC, params.Ny + params.numGC, params.numGC, params.Nx + params.numGC);
  int numsteps = st.numsteps;
  double t = st.t;
  int taken = 0;
  while (t < params.T && taken < nsteps) {
    const double CFL = (numsteps < 5) ? std::min(CFLset, 0.2) : CFLset;
    const double dt = sim.compute_dt(CFL, params, grid, eosparams, params.T, t);
    FS->pure_fluid_update(params, eosparams.gamma1, eosparams.pinf1, dt, realcells, grid, future_grid);
    apply_BCs_euler(params, grid);
    numsteps++;
    t += dt;
    taken++;
  }
  std::vector<double> U1, U2(4 * static_cast<size_t>(nr) * nc, 0.0), phi(static_cast<size_t>(nr) * nc, 0.0);
  from_grid(grid, nr, nc, U1);
  std::vector<uint8_t> mask(static_cast<size_t>(nr) * nc, 0);
  write_result(result, params, numsteps, t, realcells, realcells, U1, U2, phi, mask, mask, ref_shim_newton_iters);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) fail("usage: gfm_ref <request file> <result file>");
  const auto kv = read_request(argv[1]);
  if (get(kv, "sim_type") == "onefluid") return run_onefluid(kv, argv[2]);
  return run_twofluid(kv, argv[2]);
}
