// The reference's C++ class surface (include/gfm_gb300.hpp) over the C ABI:
// settings file, the Riemann-solver classes, the host-grid sub-steps of the
// FS / GFM / tracker classes and the sim_* drivers.  Each host-grid call runs
// on a device context kept per grid geometry and material pair, so repeated
// calls on one simulation reuse its device buffers.
#include "../../include/gfm_gb300.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

namespace gfm_gb300 {

namespace {

void check(gfm_status_t r, const char* what) {
  if (r != GFM_OK) throw error(std::string(what) + " failed (gfm_status_t " + std::to_string(r) + ")", r);
}

int bc_code(const std::string& s) {
  if (s == "transmissive") return GFM_BC_TRANSMISSIVE;
  if (s == "reflective") return GFM_BC_REFLECTIVE;
  if (s == "periodic") return GFM_BC_PERIODIC;
  throw error("unknown boundary condition \"" + s + "\"", GFM_ERR_ARG);
}

const char* bc_name(int c) {
  return c == GFM_BC_REFLECTIVE ? "reflective" : (c == GFM_BC_PERIODIC ? "periodic" : "transmissive");
}

// Device contexts keyed by the grid description and the fluid count.
class ContextCache {
 public:
  gfm_ctx* get(const gfm_grid_desc& d, int two_fluid) {
    std::string key(reinterpret_cast<const char*>(&d), sizeof(d));
    key.push_back(static_cast<char>(two_fluid));
    std::lock_guard<std::mutex> lk(mu_);
    auto it = ctx_.find(key);
    if (it != ctx_.end()) return it->second;
    gfm_ctx* c = nullptr;
    check(gfm_ctx_create(&d, two_fluid, &c), "gfm_ctx_create");
    if (two_fluid) gfm_set_overlap(c, GFM_OVERLAP_OFF);   // single sub-steps: one stream
    ctx_[key] = c;
    return c;
  }
  ~ContextCache() {
    for (auto& kv : ctx_) gfm_ctx_destroy(kv.second);
  }

 private:
  std::mutex mu_;
  std::map<std::string, gfm_ctx*> ctx_;
};

ContextCache& contexts() {
  static ContextCache cache;
  return cache;
}

// throws numeric_error when the sub-step raised device status bits
void check_status(gfm_ctx* c, const char* what) {
  uint32_t st = 0;
  check(gfm_get_device_status(c, &st), "gfm_get_device_status");
  if (st) {
    gfm_clear_device_status(c);
    throw numeric_error(std::string(what) + ": device status 0x" + [&] {
      char b[16];
      std::snprintf(b, sizeof(b), "%x", st);
      return std::string(b);
    }(), st);
  }
}

gfm_method_desc method_of(int fs, int gfm, int itm, int ls_order, int reinit_every, int reinit_iters, int ext,
                          int slip, double CFL, double T) {
  gfm_method_desc m;
  std::memset(&m, 0, sizeof(m));
  m.fs = fs; m.gfm = gfm; m.itm = itm;
  m.ls_order = ls_order; m.reinit_every = reinit_every; m.reinit_iters = reinit_iters;
  m.use_extension_vfield = ext; m.use_slip_BCs = slip;
  m.CFL = CFL; m.T = T;
  return m;
}

// device buffers for the batched Riemann solves
struct DeviceBuffer {
  void* p = nullptr;
  explicit DeviceBuffer(size_t bytes) {
    if (cudaMalloc(&p, bytes) != cudaSuccess) throw error("cudaMalloc failed", GFM_ERR_CUDA);
  }
  ~DeviceBuffer() { cudaFree(p); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
};

void to_device(void* dst, const void* src, size_t bytes) {
  if (cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) throw error("cudaMemcpy", GFM_ERR_CUDA);
}
void to_host(void* dst, const void* src, size_t bytes) {
  if (cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) throw error("cudaMemcpy", GFM_ERR_CUDA);
}

}  // namespace

// ---------------------------------------------------------------------------
// types
// ---------------------------------------------------------------------------
vec2type sim_info::cellcentre_coord(int i, int j) const {
  return vec2type(x0 + (static_cast<double>(j - numGC) + 0.5) * dx, y0 + (static_cast<double>(i - numGC) + 0.5) * dy);
}

gfm_grid_desc grid_desc(const sim_info& p, const binarySGparams& e) {
  gfm_grid_desc d;
  std::memset(&d, 0, sizeof(d));
  d.Nx = p.Nx; d.Ny = p.Ny; d.numGC = p.numGC;
  d.x0 = p.x0; d.y0 = p.y0; d.dx = p.dx; d.dy = p.dy;
  d.BC_L = bc_code(p.BC_L); d.BC_R = bc_code(p.BC_R); d.BC_B = bc_code(p.BC_B); d.BC_T = bc_code(p.BC_T);
  d.gamma1 = e.gamma1; d.pinf1 = e.pinf1; d.gamma2 = e.gamma2; d.pinf2 = e.pinf2;
  return d;
}

// headers/GFM_settingsfile.hpp:24-59: the same keys and the same basename
void GFM_settingsfile::read_settings_file(std::string filename) {
  std::ifstream infile(filename);
  if (!infile) throw error("cannot read settings file " + filename, GFM_ERR_IO);
  std::string line;
  while (std::getline(infile, line)) {
    std::istringstream iss(line);
    std::string name;
    iss >> name;
    if (name == "Nx") iss >> Nx;
    else if (name == "Ny") iss >> Ny;
    else if (name == "CFL") iss >> CFL;
    else if (name == "sim_type") iss >> sim_type;
    else if (name == "FS") iss >> FS;
    else if (name == "test_case") iss >> test_case;
    else if (name == "ITM") iss >> ITM;
    else if (name == "GFM") iss >> GFM;
    else if (name == "outputpath") iss >> outputpath;
    else if (name == "nsteps") iss >> nsteps;
    else if (name == "reinit_every") iss >> reinit_every;
    else if (name == "reinit_iters") iss >> reinit_iters;
  }
  if (sim_type == "onefluid")
    basename = outputpath + sim_type + "-" + test_case + "-" + FS + "-" + std::to_string(Nx) + "-" + std::to_string(Ny);
  else
    basename = outputpath + GFM + "-" + ITM + "-" + test_case + "-" + FS + "-" + std::to_string(Nx) + "-" +
               std::to_string(Ny);
}

// ---------------------------------------------------------------------------
// Riemann solvers: batches on the device
// ---------------------------------------------------------------------------
void pure_RS_exact::solve_RP_batch(bool paralleltox, double gamma, double pinf, int n, const double* L,
                                   const double* R, double* flux) const {
  if (n <= 0) return;
  const size_t b = sizeof(double) * 4 * static_cast<size_t>(n);
  DeviceBuffer dL(b), dR(b), dF(b), dS(sizeof(uint32_t));
  to_device(dL.p, L, b);
  to_device(dR.p, R, b);
  uint32_t st = 0;
  to_device(dS.p, &st, sizeof(st));
  check(gfm_rs_pure_batch(n, paralleltox ? 1 : 0, gamma, pinf, static_cast<const double*>(dL.p),
                          static_cast<const double*>(dR.p), static_cast<double*>(dF.p), static_cast<uint32_t*>(dS.p),
                          nullptr),
        "gfm_rs_pure_batch");
  to_host(flux, dF.p, b);
  to_host(&st, dS.p, sizeof(st));
  if (st) throw numeric_error("pure_RS_exact::solve_RP", st);
}

void pure_RS_exact::solve_RP(const bool paralleltox, const double gamma, const double pinf, const vec4type& Lstate,
                             const vec4type& Rstate, vec4type& flux) const {
  solve_RP_batch(paralleltox, gamma, pinf, 1, Lstate.v, Rstate.v, flux.v);
}

void mixed_RS_exact::solve_mixed_RP_batch(double gammaL, double pinfL, double gammaR, double pinfR, int n,
                                          const double* L, const double* R, double* out) const {
  if (n <= 0) return;
  const size_t b = sizeof(double) * 4 * static_cast<size_t>(n);
  DeviceBuffer dL(b), dR(b), dO(b), dS(sizeof(uint32_t));
  to_device(dL.p, L, b);
  to_device(dR.p, R, b);
  uint32_t st = 0;
  to_device(dS.p, &st, sizeof(st));
  check(gfm_rs_mixed_batch(n, gammaL, pinfL, gammaR, pinfR, static_cast<const double*>(dL.p),
                           static_cast<const double*>(dR.p), static_cast<double*>(dO.p),
                           static_cast<uint32_t*>(dS.p), nullptr),
        "gfm_rs_mixed_batch");
  to_host(out, dO.p, b);
  to_host(&st, dS.p, sizeof(st));
  if (st) throw numeric_error("mixed_RS_exact::solve_mixed_RP", st);
}

void mixed_RS_exact::solve_mixed_RP(const double gammaL, const double pinfL, const double gammaR, const double pinfR,
                                    const vec4type& Lstate, const vec4type& Rstate, double& p_star, double& u_star,
                                    double& rho_star_L, double& rho_star_R) const {
  double o[4];
  solve_mixed_RP_batch(gammaL, pinfL, gammaR, pinfR, 1, Lstate.v, Rstate.v, o);
  p_star = o[0]; u_star = o[1]; rho_star_L = o[2]; rho_star_R = o[3];
}

// ---------------------------------------------------------------------------
// host-grid sub-steps
// ---------------------------------------------------------------------------
namespace detail {

void fs_update(int fs, const sim_info& params, double gamma, double pinf, double dt, const BBrange& rc,
               std::vector<double>& U) {
  binarySGparams e;
  e.gamma1 = e.gamma2 = gamma;
  e.pinf1 = e.pinf2 = pinf;
  gfm_ctx* c = contexts().get(grid_desc(params, e), 0);
  check(gfm_upload(c, 1, U.data()), "gfm_upload");
  const int boxes[8] = {rc.imin, rc.imax, rc.jmin, rc.jmax, rc.imin, rc.imax, rc.jmin, rc.jmax};
  check(gfm_clear_device_status(c), "gfm_clear_device_status");
  check(gfm_set_step(c, dt, boxes), "gfm_set_step");
  check(gfm_fs_update(c, fs, 1), "gfm_fs_update");
  check(gfm_download(c, 1, U.data()), "gfm_download");
  check_status(c, "FS_base::pure_fluid_update");
}

void apply_bcs(const sim_info& params, std::vector<double>& U) {
  gfm_ctx* c = contexts().get(grid_desc(params, binarySGparams()), 0);
  check(gfm_upload(c, 1, U.data()), "gfm_upload");
  check(gfm_set_step(c, 0.0, nullptr), "gfm_set_step");
  check(gfm_apply_bcs(c, 1), "gfm_apply_bcs");
  check(gfm_download(c, 1, U.data()), "gfm_download");
}

void ghost_fill(const GhostFill& f, const sim_info& params, const std::vector<double>& field,
                const binarySGparams& eosparams, std::vector<double>& U1, std::vector<double>& U2,
                std::vector<double>& vel, int rc[8]) {
  gfm_ctx* c = contexts().get(grid_desc(params, eosparams), 1);
  check(gfm_upload_state(c, U1.data(), U2.data(), field.data()), "gfm_upload_state");
  check(gfm_set_interface_tracker(c, f.itm), "gfm_set_interface_tracker");
  check(gfm_clear_device_status(c), "gfm_clear_device_status");
  check(gfm_set_step(c, 0.0, nullptr), "gfm_set_step");
  const gfm_method_desc m = method_of(GFM_FS_MUSCL, f.gfm, f.itm, 5, 0, 0, f.use_extension_vfield, f.use_slip_BCs,
                                      0.5, HUGE_VAL);
  check(gfm_set_ghost_states(c, &m), "gfm_set_ghost_states");
  std::vector<double> scratch(field.size());
  check(gfm_download_state(c, U1.data(), U2.data(), scratch.data()), "gfm_download_state");
  vel.resize(2 * field.size());
  check(gfm_download_velocity(c, vel.data()), "gfm_download_velocity");
  check(gfm_get_realcells(c, rc), "gfm_get_realcells");
  check_status(c, "GFM_base::set_ghost_states");
}

double compute_dt_twofluid(double CFL, const sim_info& params, const std::vector<double>& U1,
                           const std::vector<double>& U2, const std::vector<double>& field, int itm,
                           const binarySGparams& eosparams, double T, double t) {
  gfm_ctx* c = contexts().get(grid_desc(params, eosparams), 1);
  check(gfm_upload_state(c, U1.data(), U2.data(), field.data()), "gfm_upload_state");
  check(gfm_set_interface_tracker(c, itm), "gfm_set_interface_tracker");
  check(gfm_clear_device_status(c), "gfm_clear_device_status");
  check(gfm_set_time(c, t, 5), "gfm_set_time");   // past the ramp: the caller passes the ramped CFL
  check(gfm_compute_dt(c, CFL, T), "gfm_compute_dt");
  double tt = 0.0, dt = 0.0;
  int n = 0;
  check(gfm_get_time(c, &tt, &n, &dt), "gfm_get_time");
  check_status(c, "sim_twofluid::compute_dt");
  return dt;
}

double compute_dt_onefluid(double CFL, const sim_info& params, const std::vector<double>& U,
                           const binarySGparams& eosparams, double T, double t) {
  gfm_ctx* c = contexts().get(grid_desc(params, eosparams), 0);
  check(gfm_upload(c, 1, U.data()), "gfm_upload");
  check(gfm_clear_device_status(c), "gfm_clear_device_status");
  check(gfm_set_time(c, t, 5), "gfm_set_time");
  check(gfm_compute_dt(c, CFL, T), "gfm_compute_dt");
  double tt = 0.0, dt = 0.0;
  int n = 0;
  check(gfm_get_time(c, &tt, &n, &dt), "gfm_get_time");
  check_status(c, "sim_onefluid::compute_dt");
  return dt;
}

}  // namespace detail

// ---------------------------------------------------------------------------
// velocity field and trackers
// ---------------------------------------------------------------------------
void solved_velocity_field_firstorder::store_velocity_field(const gridVector2dtype& v, double) {
  const size_t nr = v.size(), nc = nr ? v[0].size() : 0, plane = nr * nc;
  vel_.assign(2 * plane, 0.0);
  for (size_t i = 0; i < nr; i++)
    for (size_t j = 0; j < nc; j++) {
      vel_[i * nc + j] = v[i][j](0);
      vel_[plane + i * nc + j] = v[i][j](1);
    }
}

vec2type solved_velocity_field_firstorder::get_velocity(const vec2type& x, double) const {
  const int nc = params_.Nx + 2 * params_.numGC;
  const size_t plane = static_cast<size_t>(params_.Ny + 2 * params_.numGC) * nc;
  const int j = static_cast<int>(std::floor((x(0) - params_.x0) / params_.dx)) + params_.numGC;
  const int i = static_cast<int>(std::floor((x(1) - params_.y0) / params_.dy)) + params_.numGC;
  if (vel_.empty() || i < 0 || j < 0 || i >= params_.Ny + 2 * params_.numGC || j >= nc) return vec2type(0.0, 0.0);
  const size_t c = static_cast<size_t>(i) * nc + j;
  return vec2type(vel_[c], vel_[plane + c]);
}

Levelset::Levelset(const sim_info& params, int order, int reinit_every, int reinit_iters)
    : params_(params), order_(order), reinit_every_(reinit_every), reinit_iters_(reinit_iters) {
  if (order != 1 && order != 5) throw error("Levelset: advection order 1 (LS1) or 5 (LS5)", GFM_ERR_UNSUPPORTED);
  phi_.assign(static_cast<size_t>(params.Ny + 2 * params.numGC) * (params.Nx + 2 * params.numGC), 0.0);
}

vec2type Levelset::get_normal(const vec2type& x) const {
  const int j = static_cast<int>(std::floor((x(0) - params_.x0) / params_.dx)) + params_.numGC;
  const int i = static_cast<int>(std::floor((x(1) - params_.y0) / params_.dy)) + params_.numGC;
  return vec2type((get_sdf(i, j + 1) - get_sdf(i, j - 1)) / (2.0 * params_.dx),
                  (get_sdf(i + 1, j) - get_sdf(i - 1, j)) / (2.0 * params_.dy));
}

bool Levelset::is_interfacial_cell(int i, int j) const {
  const bool s = get_sdf(i, j) <= 0.0;
  return (get_sdf(i, j - 1) <= 0.0) != s || (get_sdf(i, j + 1) <= 0.0) != s || (get_sdf(i - 1, j) <= 0.0) != s ||
         (get_sdf(i + 1, j) <= 0.0) != s;
}

namespace {
// the tracker's update on the device: phi (or z) and the velocity field in,
// advection (and the reinitialisation schedule) there, phi out
void tracker_update(const sim_info& params, std::vector<double>& field, const velocity_field_base& vfield,
                    const gfm_method_desc& m, int updates, double t, double dt) {
  const auto* sv = dynamic_cast<const solved_velocity_field_firstorder*>(&vfield);
  if (!sv || sv->planes().size() != 2 * field.size())
    throw error("update_interface_coupled: the velocity field of a ghost fill of this grid is needed", GFM_ERR_ARG);
  gfm_ctx* c = contexts().get(grid_desc(params, binarySGparams()), 1);
  check(gfm_upload_phi(c, field.data()), "gfm_upload_phi");
  check(gfm_upload_velocity(c, sv->planes().data()), "gfm_upload_velocity");
  check(gfm_set_time(c, t, updates), "gfm_set_time");
  check(gfm_set_step(c, dt, nullptr), "gfm_set_step");
  check(gfm_ls_update(c, &m), "gfm_ls_update");
  check(gfm_download_phi(c, field.data()), "gfm_download_phi");
}
}  // namespace

void Levelset::update_interface_coupled(const velocity_field_base& vfield, double t, double dt) {
  const gfm_method_desc m =
      method_of(GFM_FS_MUSCL, GFM_RIEMANN, GFM_ITM_LEVELSET, order_, reinit_every_, reinit_iters_, 0, 0, 0.5, HUGE_VAL);
  tracker_update(params_, phi_, vfield, m, updates, t, dt);
  updates++;
}

VOF::VOF(const sim_info& params) : params_(params) {
  if (params.numGC < 6) throw error("VOF: the VOF ghost fills read 6 cells outside the real cells", GFM_ERR_ARG);
  z_.assign(static_cast<size_t>(params.Ny + 2 * params.numGC) * (params.Nx + 2 * params.numGC), 0.0);
}

vec2type VOF::get_normal(const vec2type&) const {
  throw error("VOF::get_normal: the VOF ghost fills take their normals from the reconstruction", GFM_ERR_UNSUPPORTED);
}

void VOF::update_interface_coupled(const velocity_field_base& vfield, double t, double dt) {
  const gfm_method_desc m = method_of(GFM_FS_MUSCL, ::GFM_VOF_CODE, GFM_ITM_VOF, 0, 0, 0, 0, 0, 0.5, HUGE_VAL);
  tracker_update(params_, z_, vfield, m, updates, t, dt);
  updates++;
}

// ---------------------------------------------------------------------------
// simulations: the named cases' set-up and the whole run on the device
// ---------------------------------------------------------------------------
namespace {
void params_from_desc(const gfm_grid_desc& d, double T, sim_info& p, binarySGparams& e) {
  p.Nx = d.Nx; p.Ny = d.Ny; p.numGC = d.numGC;
  p.x0 = d.x0; p.y0 = d.y0; p.dx = d.dx; p.dy = d.dy;
  p.BC_L = bc_name(d.BC_L); p.BC_R = bc_name(d.BC_R); p.BC_B = bc_name(d.BC_B); p.BC_T = bc_name(d.BC_T);
  p.T = T;
  e.gamma1 = d.gamma1; e.pinf1 = d.pinf1; e.gamma2 = d.gamma2; e.pinf2 = d.pinf2;
}

int fs_code(const std::string& s) {
  if (s == "MUSCL") return GFM_FS_MUSCL;
  if (s == "Godunov") return GFM_FS_GODUNOV;
  throw error("Invalid FS choice \"" + s + "\"", GFM_ERR_ARG);
}

int gfm_code(const std::string& s) {
  if (s == "OGFM") return GFM_OGFM;
  if (s == "riemannGFM") return GFM_RIEMANN;
  if (s == "realGFM") return GFM_REAL;
  if (s == "MGFM") return GFM_MODIFIED;
  if (s == "VOFGFM") return ::GFM_VOF_CODE;
  if (s == "OGFMVOF") return GFM_OGFM_VOF;
  throw error("Invalid GFM choice \"" + s + "\"", GFM_ERR_ARG);
}

// ITM name -> (tracker, advection order); LS3 and LS9 are not built
void itm_code(const std::string& s, int& itm, int& order) {
  if (s == "LS1") { itm = GFM_ITM_LEVELSET; order = 1; return; }
  if (s == "LS5") { itm = GFM_ITM_LEVELSET; order = 5; return; }
  if (s == "PYVOF") { itm = GFM_ITM_VOF; order = 0; return; }
  throw error("ITM \"" + s + "\" is not built (LS1, LS5, PYVOF are)", GFM_ERR_UNSUPPORTED);
}

// the output frequency of set_sim_parameters (sourcecode/sim_twofluid.cpp:347,392,404;
// sourcecode/sim_onefluid.cpp:102): outputs over T for two fluids, every
// output_freq steps for one fluid
int output_freq(const GFM_settingsfile& SF, int two) {
  if (!two) return 1000000000;
  if (SF.test_case == "GDA") return 0;
  if (SF.test_case == "shocked_helium_bubble") return 2;
  return 4;
}

void run(const GFM_settingsfile& SF, int two) {
  gfm_grid_desc d;
  double T = 0.0;
  check(gfm_case_params(two ? "twofluid" : "onefluid", SF.test_case.c_str(), SF.Nx, SF.Ny, &d, &T),
        "gfm_case_params");
  gfm_method_desc m;
  int itm = GFM_ITM_LEVELSET, order = 5;
  if (two) {
    itm_code(SF.ITM, itm, order);
    const int every = SF.reinit_every >= 0 ? SF.reinit_every : (itm == GFM_ITM_LEVELSET ? 1 : 0);
    // sourcecode/sim_twofluid.cpp:551: no extension velocities, no slip
    m = method_of(fs_code(SF.FS), gfm_code(SF.GFM), itm, order, every, SF.reinit_iters, 0, 0, SF.CFL, T);
  } else {
    m = method_of(fs_code(SF.FS), GFM_RIEMANN, GFM_ITM_LEVELSET, 5, 0, 5, 0, 0, SF.CFL, T);
  }
  const size_t cells = static_cast<size_t>(d.Nx + 2 * d.numGC) * (d.Ny + 2 * d.numGC);
  std::vector<double> U1(4 * cells), U2(two ? 4 * cells : 0), phi(two ? cells : 0);
  const char* st = two ? "twofluid" : "onefluid";
  check(gfm_case_init(st, SF.test_case.c_str(), &d, U1.data(), two ? U2.data() : nullptr, two ? phi.data() : nullptr),
        "gfm_case_init");
  if (two && itm == GFM_ITM_VOF) check(gfm_case_init_z(SF.test_case.c_str(), &d, phi.data()), "gfm_case_init_z");
  gfm_ctx* c = nullptr;
  check(gfm_ctx_create(&d, two, &c), "gfm_ctx_create");
  gfm_status_t r = gfm_upload_state(c, U1.data(), two ? U2.data() : nullptr, two ? phi.data() : nullptr);
  if (r == GFM_OK) r = gfm_set_time(c, 0.0, 0);
  double seconds = 0.0;
  if (r == GFM_OK)
    r = gfm_run_sim(c, &m, &d, SF.basename.c_str(), output_freq(SF, two), SF.nsteps > 0 ? SF.nsteps : 0, &seconds);
  uint32_t bits = 0;
  gfm_get_device_status(c, &bits);
  gfm_ctx_destroy(c);
  check(r, "gfm_run_sim");
  if (bits) throw numeric_error("run_sim", bits);
}
}  // namespace

void sim_onefluid::run_sim(GFM_settingsfile SF) { run(SF, 0); }
void sim_twofluid::run_sim(GFM_settingsfile SF) { run(SF, 1); }

void sim_onefluid::set_sim_parameters(const GFM_settingsfile& SF, sim_info& params, binarySGparams& eosparams) {
  gfm_grid_desc d;
  double T = 0.0;
  check(gfm_case_params("onefluid", SF.test_case.c_str(), SF.Nx, SF.Ny, &d, &T), "gfm_case_params");
  params_from_desc(d, T, params, eosparams);
  params.output_freq = output_freq(SF, 0);
}

void sim_onefluid::set_sim_methods(const GFM_settingsfile& SF, std::shared_ptr<pure_RS_base>& RS,
                                   std::shared_ptr<FS_base>& FS) {
  RS = std::make_shared<pure_RS_exact>();
  if (fs_code(SF.FS) == GFM_FS_MUSCL) FS = std::make_shared<FS_MUSCL>(RS);
  else FS = std::make_shared<FS_godunov>(RS);
}

void sim_onefluid::set_sim_ICs(const GFM_settingsfile& SF, const sim_info& params, const binarySGparams& eosparams,
                               grideuler2type& grid) {
  const gfm_grid_desc d = grid_desc(params, eosparams);
  const size_t nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
  std::vector<double> U(4 * nr * nc);
  check(gfm_case_init("onefluid", SF.test_case.c_str(), &d, U.data(), nullptr, nullptr), "gfm_case_init");
  grid.assign(nr, roweuler2type(nc));
  planes_to_grid(U, grid);
}

void sim_twofluid::set_sim_parameters(const GFM_settingsfile& SF, sim_info& params, binarySGparams& eosparams) {
  gfm_grid_desc d;
  double T = 0.0;
  check(gfm_case_params("twofluid", SF.test_case.c_str(), SF.Nx, SF.Ny, &d, &T), "gfm_case_params");
  params_from_desc(d, T, params, eosparams);
  params.output_freq = output_freq(SF, 1);
}

// sourcecode/sim_twofluid.cpp:495-594: the FS, GFM and ITM named by the settings
void sim_twofluid::set_sim_methods(const GFM_settingsfile& SF, const sim_info& params, std::shared_ptr<FS_base>& FS,
                                   std::shared_ptr<GFM_base>& GFM, std::shared_ptr<GFM_ITM_interface>& ls) {
  std::shared_ptr<pure_RS_base> RS = std::make_shared<pure_RS_exact>();
  if (fs_code(SF.FS) == GFM_FS_MUSCL) FS = std::make_shared<FS_MUSCL>(RS);
  else FS = std::make_shared<FS_godunov>(RS);
  switch (gfm_code(SF.GFM)) {
    case GFM_OGFM: GFM = std::make_shared<GFM_original>(params); break;
    case GFM_RIEMANN: GFM = std::make_shared<GFM_riemann>(params); break;
    case GFM_REAL: GFM = std::make_shared<GFM_real>(params); break;
    case GFM_MODIFIED: GFM = std::make_shared<GFM_modified>(params); break;
    case GFM_OGFM_VOF: GFM = std::make_shared<OGFM_VOF>(params); break;
    default: GFM = std::make_shared<GFM_VOF>(params); break;
  }
  GFM->use_extension_vfield = false;
  GFM->use_slip_BCs = false;
  int itm = 0, order = 0;
  itm_code(SF.ITM, itm, order);
  // the settings' reinit_every / reinit_iters where given, else every step
  if (itm == GFM_ITM_VOF) ls = std::make_shared<VOF>(params);
  else ls = std::make_shared<Levelset>(params, order, SF.reinit_every >= 0 ? SF.reinit_every : 1, SF.reinit_iters);
}

void sim_twofluid::set_sim_ICs(const GFM_settingsfile& SF, const sim_info& params, const binarySGparams& eosparams,
                               grideuler2type& grid1, grideuler2type& grid2, GFM_ITM_interface& ls) {
  const gfm_grid_desc d = grid_desc(params, eosparams);
  const size_t nr = params.Ny + 2 * params.numGC, nc = params.Nx + 2 * params.numGC;
  std::vector<double> U1(4 * nr * nc), U2(4 * nr * nc);
  check(gfm_case_init("twofluid", SF.test_case.c_str(), &d, U1.data(), U2.data(), ls.field().data()),
        "gfm_case_init");
  if (ls.itm() == GFM_ITM_VOF) check(gfm_case_init_z(SF.test_case.c_str(), &d, ls.field().data()), "gfm_case_init_z");
  grid1.assign(nr, roweuler2type(nc));
  grid2.assign(nr, roweuler2type(nc));
  planes_to_grid(U1, grid1);
  planes_to_grid(U2, grid2);
}

}  // namespace gfm_gb300
