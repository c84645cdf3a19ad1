/*
 * gfm_gb300.hpp -- the reference's C++ class surface over the GB300 library.
 *
 * murraycutforth/PhD-2D-GFM structures its solver as strategy classes held by
 * std::shared_ptr (sourcecode/sim_twofluid.cpp:34-37,504-594).  This header
 * gives the same classes, with the same names, constructor arguments and
 * member-function signatures, in namespace gfm_gb300; code written against
 * the reference switches with "using namespace gfm_gb300;".  Every compute
 * call runs on the GPU through the C ABI (include/gfm_gb300.h):
 *
 *   reference (file:line)                                   here
 *   sim_base::run_sim (headers/sim_base.hpp:10)             sim_base::run_sim
 *   sim_onefluid / sim_twofluid (headers/sim_onefluid.hpp:16-36,
 *     headers/sim_twofluid.hpp:18-100)                      sim_onefluid / sim_twofluid
 *   FS_base::pure_fluid_update (headers/FS_base.hpp:23-32)  FS_base::pure_fluid_update
 *   FS_MUSCL, FS_godunov (headers/FS_MUSCL.hpp:64,
 *     headers/FS_godunov.hpp:13)                            FS_MUSCL, FS_godunov
 *   GFM_base::set_ghost_states + use_extension_vfield,
 *     use_slip_BCs, vfield, mixed_RS (headers/GFM_base.hpp:20-47)
 *                                                           GFM_base (same members)
 *   GFM_original/riemann/real/modified, GFM_VOF, OGFM_VOF   same names
 *   pure_RS_base::solve_RP (headers/pure_RS_base.hpp:13-20) pure_RS_base / pure_RS_exact
 *   mixed_RS_base::solve_mixed_RP (headers/mixed_RS_base.hpp:12-24)
 *                                                           mixed_RS_base / mixed_RS_exact
 *   apply_BCs_euler (headers/euler_bc.hpp:5)                apply_BCs_euler
 *   GFM_settingsfile (headers/GFM_settingsfile.hpp:9-60)    GFM_settingsfile
 *   BBrange (headers/BBrange.hpp:4-17)                      BBrange
 *   sim_info, binarySGparams, Levelset, VOF (absent libraries the reference
 *     links, Makefile:17-27)                                same names
 *
 * Grids: the member templates take any grid[i][j](k)-indexable container,
 * the reference's std::vector<std::vector<Eigen::Vector4d>> included; the
 * default types below need no Eigen.  A call on host grids copies them to
 * the device, runs the sub-step there and copies them back, so existing code
 * keeps its host-side loop; sim_*::run_sim keeps the whole run on the device
 * (gfm_run_sim) and is the fast path.  The pure_fluid_update call leaves
 * future_grid equal to grid (the reference uses it as scratch).
 *
 * Errors: the reference aborts on a live assert (an unphysical state, dt <=
 * 0, sourcecode/FS_MUSCL.cpp:167, sourcecode/sim_twofluid.cpp:155).  Here a
 * sub-step that raises a device status bit throws gfm_gb300::numeric_error
 * (its bits in status()), and a failed library call throws gfm_gb300::error.
 *
 * Link: -lgfm_gb300 (the classes are compiled into the library).
 */
#ifndef GFM_GB300_HPP
#define GFM_GB300_HPP

#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gfm_gb300.h"

// The C header's method code GFM_VOF has the name of the reference's class
// GFM_VOF; under C++ the code is GFM_VOF_CODE.
#ifdef GFM_VOF
static constexpr int GFM_VOF_CODE = GFM_VOF;
#undef GFM_VOF
#endif

namespace gfm_gb300 {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
class error : public std::runtime_error {
 public:
  error(const std::string& what, gfm_status_t code) : std::runtime_error(what), code_(code) {}
  gfm_status_t code() const { return code_; }

 private:
  gfm_status_t code_;
};

// a sub-step raised GFM_ST_* bits where the reference would have asserted
class numeric_error : public error {
 public:
  numeric_error(const std::string& what, uint32_t bits) : error(what, GFM_ERR_NUMERIC), bits_(bits) {}
  uint32_t status() const { return bits_; }

 private:
  uint32_t bits_;
};

// ---------------------------------------------------------------------------
// types of the reference's signatures
// ---------------------------------------------------------------------------
struct vec2type {
  double v[2] = {0.0, 0.0};
  vec2type() = default;
  vec2type(double x, double y) : v{x, y} {}
  double& operator()(int k) { return v[k]; }
  const double& operator()(int k) const { return v[k]; }
};

// conserved or primitive state (rho, rho u, rho v, E) / (rho, u, v, p)
struct vec4type {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  vec4type() = default;
  explicit vec4type(int /*size, always 4*/) {}
  vec4type(double a, double b, double c, double d) : v{a, b, c, d} {}
  double& operator()(int k) { return v[k]; }
  const double& operator()(int k) const { return v[k]; }
};

typedef std::vector<vec4type> roweuler2type;
typedef std::vector<roweuler2type> grideuler2type;            // grid[i][j], row i = y index
typedef std::vector<std::vector<vec2type>> gridVector2dtype;  // velocity field

class BBrange {
 public:
  int imin, imax, jmin, jmax;
  BBrange(int imin, int imax, int jmin, int jmax) : imin(imin), imax(imax), jmin(jmin), jmax(jmax) {}
};

// grid geometry, boundary conditions ("transmissive", "reflective",
// "periodic"), end time and output frequency
class sim_info {
 public:
  int Nx = 0, Ny = 0, numGC = 0;
  int output_freq = 0;
  double x0 = 0.0, y0 = 0.0, dx = 0.0, dy = 0.0;
  double T = 0.0;
  std::string BC_L = "transmissive", BC_R = "transmissive", BC_B = "transmissive", BC_T = "transmissive";
  // centre of cell (i, j): (x0 + (j - numGC + 1/2) dx, y0 + (i - numGC + 1/2) dy)
  vec2type cellcentre_coord(int i, int j) const;
};

struct binarySGparams {
  double gamma1 = 1.4, gamma2 = 1.4, pinf1 = 0.0, pinf2 = 0.0;
};

// the settings file: whitespace "key value" lines, unknown keys ignored;
// the reference's keys plus nsteps (0: run to the case's end time),
// reinit_every (-1: the tracker's default) and reinit_iters
class GFM_settingsfile {
 public:
  int Nx = 0;
  int Ny = 0;
  double CFL = 0.0;
  std::string sim_type, FS, ITM, GFM, test_case, outputpath, basename;
  int nsteps = 0;
  int reinit_every = -1;
  int reinit_iters = 5;
  void read_settings_file(std::string filename);
};

// the C ABI's grid description of params + eosparams
gfm_grid_desc grid_desc(const sim_info& params, const binarySGparams& eosparams);

// grid[i][j](k) <-> four planes of (Ny + 2 numGC) x (Nx + 2 numGC) doubles
template <class Grid>
void grid_to_planes(const Grid& g, std::vector<double>& out) {
  const size_t nr = g.size(), nc = nr ? g[0].size() : 0, plane = nr * nc;
  out.resize(4 * plane);
  for (size_t i = 0; i < nr; i++)
    for (size_t j = 0; j < nc; j++)
      for (int k = 0; k < 4; k++) out[k * plane + i * nc + j] = g[i][j](k);
}
template <class Grid>
void planes_to_grid(const std::vector<double>& in, Grid& g) {
  const size_t nr = g.size(), nc = nr ? g[0].size() : 0, plane = nr * nc;
  for (size_t i = 0; i < nr; i++)
    for (size_t j = 0; j < nc; j++)
      for (int k = 0; k < 4; k++) g[i][j](k) = in[k * plane + i * nc + j];
}

// ---------------------------------------------------------------------------
// exact Riemann solvers
// ---------------------------------------------------------------------------
class pure_RS_base {
 public:
  virtual ~pure_RS_base() {}
  // flux at x/t = 0 of the exact stiffened-gas Riemann problem between
  // conserved states L and R, normal to x (paralleltox) or y
  virtual void solve_RP(const bool paralleltox, const double gamma, const double pinf, const vec4type& Lstate,
                        const vec4type& Rstate, vec4type& flux) const = 0;
};

class pure_RS_exact : public pure_RS_base {
 public:
  void solve_RP(const bool paralleltox, const double gamma, const double pinf, const vec4type& Lstate,
                const vec4type& Rstate, vec4type& flux) const override;
  // n problems in one launch: L, R, flux are n x 4 doubles (host memory)
  void solve_RP_batch(bool paralleltox, double gamma, double pinf, int n, const double* L, const double* R,
                      double* flux) const;
};

class mixed_RS_base {
 public:
  virtual ~mixed_RS_base() {}
  virtual void solve_mixed_RP(const double gammaL, const double pinfL, const double gammaR, const double pinfR,
                              const vec4type& Lstate, const vec4type& Rstate, double& p_star, double& u_star,
                              double& rho_star_L, double& rho_star_R) const = 0;
};

class mixed_RS_exact : public mixed_RS_base {
 public:
  void solve_mixed_RP(const double gammaL, const double pinfL, const double gammaR, const double pinfR,
                      const vec4type& Lstate, const vec4type& Rstate, double& p_star, double& u_star,
                      double& rho_star_L, double& rho_star_R) const override;
  // n problems in one launch: out[4k..] = (p*, u*, rho*L, rho*R)
  void solve_mixed_RP_batch(double gammaL, double pinfL, double gammaR, double pinfR, int n, const double* L,
                            const double* R, double* out) const;
};

// ---------------------------------------------------------------------------
// host-grid sub-steps (implemented in the library)
// ---------------------------------------------------------------------------
namespace detail {
void fs_update(int fs, const sim_info& params, double gamma, double pinf, double dt, const BBrange& realcells,
               std::vector<double>& U);
void apply_bcs(const sim_info& params, std::vector<double>& U);
struct GhostFill {
  int gfm = 0, itm = GFM_ITM_LEVELSET, use_extension_vfield = 0, use_slip_BCs = 0;
};
void ghost_fill(const GhostFill& f, const sim_info& params, const std::vector<double>& field,
                const binarySGparams& eosparams, std::vector<double>& U1, std::vector<double>& U2,
                std::vector<double>& vel, int realcells[8]);
double compute_dt_twofluid(double CFL, const sim_info& params, const std::vector<double>& U1,
                           const std::vector<double>& U2, const std::vector<double>& field, int itm,
                           const binarySGparams& eosparams, double T, double t);
double compute_dt_onefluid(double CFL, const sim_info& params, const std::vector<double>& U,
                           const binarySGparams& eosparams, double T, double t);
}  // namespace detail

// ---------------------------------------------------------------------------
// flux solvers
// ---------------------------------------------------------------------------
class FS_base {
 public:
  std::shared_ptr<pure_RS_base> RS;
  explicit FS_base(std::shared_ptr<pure_RS_base> RS) : RS(RS) {}
  virtual ~FS_base() {}
  virtual int kind() const = 0;   // GFM_FS_*

  // one fluid's update over realcells (no BCs), as the reference's
  template <class Grid>
  void pure_fluid_update(const sim_info& params, const double gamma, const double pinf, const double dt,
                         const BBrange& realcells, Grid& grid, Grid& future_grid) {
    std::vector<double> U;
    grid_to_planes(grid, U);
    detail::fs_update(kind(), params, gamma, pinf, dt, realcells, U);
    planes_to_grid(U, grid);
    future_grid = grid;
  }
};

class FS_MUSCL : public FS_base {
 public:
  explicit FS_MUSCL(std::shared_ptr<pure_RS_base> RS) : FS_base(RS) {}
  int kind() const override { return GFM_FS_MUSCL; }
};

class FS_godunov : public FS_base {
 public:
  explicit FS_godunov(std::shared_ptr<pure_RS_base> RS) : FS_base(RS) {}
  int kind() const override { return GFM_FS_GODUNOV; }
};

template <class Grid>
void apply_BCs_euler(const sim_info& params, Grid& grid) {
  std::vector<double> U;
  grid_to_planes(grid, U);
  detail::apply_bcs(params, U);
  planes_to_grid(U, grid);
}

// ---------------------------------------------------------------------------
// velocity field and interface trackers
// ---------------------------------------------------------------------------
class velocity_field_base {
 public:
  virtual ~velocity_field_base() {}
  virtual vec2type get_velocity(const vec2type& x, double t) const = 0;
};

// the composite velocity field of the last ghost fill, at cell centres
class solved_velocity_field_firstorder : public velocity_field_base {
 public:
  explicit solved_velocity_field_firstorder(const sim_info& params) : params_(params) {}
  void store_velocity_field(const gridVector2dtype& velocities, double t);
  vec2type get_velocity(const vec2type& x, double t) const override;   // the value of the cell holding x
  // two planes (u, v) in the layout of phi
  const std::vector<double>& planes() const { return vel_; }
  void store_planes(const std::vector<double>& vel) { vel_ = vel; }

 private:
  sim_info params_;
  std::vector<double> vel_;
};
typedef solved_velocity_field_firstorder solved_velocity_field_base;

class GFM_ITM_interface {
 public:
  virtual ~GFM_ITM_interface() {}
  virtual double get_sdf(int i, int j) const = 0;
  virtual void set_sdf(int i, int j, double v) = 0;
  virtual double get_z(int i, int j) const = 0;
  virtual void set_z(int i, int j, double v) = 0;
  virtual vec2type get_normal(const vec2type& x) const = 0;
  virtual bool is_interfacial_cell(int i, int j) const = 0;
  virtual void initialisation() = 0;
  virtual void update_interface_coupled(const velocity_field_base& vfield, double t, double dt) = 0;
  // the plane the library holds for this tracker (phi, or z for VOF) and its kind
  virtual const std::vector<double>& field() const = 0;
  virtual std::vector<double>& field() = 0;
  virtual int itm() const = 0;
};

// The level set: phi negative in fluid 1; LS1 (first-order upwind) or LS5
// (HOUC5 + TVD RK3) advection, Sussman reinitialisation every
// reinit_every updates (reinit_iters pseudo-time iterations).
class Levelset : public GFM_ITM_interface {
 public:
  Levelset(const sim_info& params, int order, int reinit_every = 1, int reinit_iters = 5);
  double get_sdf(int i, int j) const override { return phi_[idx(i, j)]; }
  void set_sdf(int i, int j, double v) override { phi_[idx(i, j)] = v; }
  double get_z(int i, int j) const override { return phi_[idx(i, j)] <= 0.0 ? 1.0 : 0.0; }
  void set_z(int, int, double) override {}
  vec2type get_normal(const vec2type& x) const override;   // central-difference gradient at x's cell
  bool is_interfacial_cell(int i, int j) const override;
  void initialisation() override {}
  void update_interface_coupled(const velocity_field_base& vfield, double t, double dt) override;
  const std::vector<double>& field() const override { return phi_; }
  std::vector<double>& field() override { return phi_; }
  int itm() const override { return GFM_ITM_LEVELSET; }
  int order() const { return order_; }
  int updates = 0;   // updates so far (the reinitialisation schedule counts them)

 private:
  size_t idx(int i, int j) const { return static_cast<size_t>(i) * (params_.Nx + 2 * params_.numGC) + j; }
  sim_info params_;
  int order_, reinit_every_, reinit_iters_;
  std::vector<double> phi_;
};

// The VOF tracker (settings ITM "PYVOF"): z, the volume fraction of fluid 1,
// PLIC reconstruction and split geometric advection; get_sdf = 0.5 - z.
class VOF : public GFM_ITM_interface {
 public:
  explicit VOF(const sim_info& params);
  double get_sdf(int i, int j) const override { return 0.5 - z_[idx(i, j)]; }
  void set_sdf(int, int, double) override {}
  double get_z(int i, int j) const override { return z_[idx(i, j)]; }
  void set_z(int i, int j, double v) override { z_[idx(i, j)] = v; }
  vec2type get_normal(const vec2type& x) const override;
  bool is_interfacial_cell(int i, int j) const override {
    const double z = z_[idx(i, j)];
    return z > 0.0 && z < 1.0;
  }
  void initialisation() override {}
  void update_interface_coupled(const velocity_field_base& vfield, double t, double dt) override;
  const std::vector<double>& field() const override { return z_; }
  std::vector<double>& field() override { return z_; }
  int itm() const override { return GFM_ITM_VOF; }
  int updates = 0;   // updates so far (the sweep order alternates with them)

 private:
  size_t idx(int i, int j) const { return static_cast<size_t>(i) * (params_.Nx + 2 * params_.numGC) + j; }
  sim_info params_;
  std::vector<double> z_;
};

// ---------------------------------------------------------------------------
// ghost-fluid methods
// ---------------------------------------------------------------------------
class GFM_base {
 public:
  bool use_extension_vfield;
  bool use_slip_BCs;
  std::shared_ptr<solved_velocity_field_base> vfield;
  std::shared_ptr<mixed_RS_base> mixed_RS;

  explicit GFM_base(const sim_info& params)
      : use_extension_vfield(true),
        use_slip_BCs(false),
        vfield(std::make_shared<solved_velocity_field_firstorder>(params)),
        mixed_RS(std::make_shared<mixed_RS_exact>()) {}
  virtual ~GFM_base() {}
  virtual int kind() const = 0;   // GFM_OGFM ... GFM_OGFM_VOF

  // ghost states of both grids (and, for OGFM / OGFM_VOF, the realcells
  // boxes of the flux updates) from the tracker's interface; stores the
  // composite velocity field in vfield
  template <class Grid>
  void set_ghost_states(const sim_info& params, const GFM_ITM_interface& ls, const binarySGparams& eosparams,
                        const double t, Grid& grid1, Grid& grid2, BBrange& realcells1, BBrange& realcells2) {
    std::vector<double> U1, U2, vel;
    grid_to_planes(grid1, U1);
    grid_to_planes(grid2, U2);
    detail::GhostFill f;
    f.gfm = kind();
    f.itm = ls.itm();
    f.use_extension_vfield = use_extension_vfield ? 1 : 0;
    f.use_slip_BCs = use_slip_BCs ? 1 : 0;
    int rc[8] = {realcells1.imin, realcells1.imax, realcells1.jmin, realcells1.jmax,
                 realcells2.imin, realcells2.imax, realcells2.jmin, realcells2.jmax};
    detail::ghost_fill(f, params, ls.field(), eosparams, U1, U2, vel, rc);
    planes_to_grid(U1, grid1);
    planes_to_grid(U2, grid2);
    vfield->store_planes(vel);
    (void)t;
    realcells1 = BBrange(rc[0], rc[1], rc[2], rc[3]);
    realcells2 = BBrange(rc[4], rc[5], rc[6], rc[7]);
  }
};

class GFM_original : public GFM_base {
 public:
  explicit GFM_original(const sim_info& params) : GFM_base(params) {}
  int kind() const override { return GFM_OGFM; }
};
class GFM_riemann : public GFM_base {
 public:
  explicit GFM_riemann(const sim_info& params) : GFM_base(params) {}
  int kind() const override { return GFM_RIEMANN; }
};
class GFM_real : public GFM_base {
 public:
  explicit GFM_real(const sim_info& params) : GFM_base(params) {}
  int kind() const override { return GFM_REAL; }
};
class GFM_modified : public GFM_base {
 public:
  explicit GFM_modified(const sim_info& params) : GFM_base(params) {}
  int kind() const override { return GFM_MODIFIED; }
};
class GFM_VOF : public GFM_base {
 public:
  explicit GFM_VOF(const sim_info& params) : GFM_base(params) {}
  int kind() const override { return GFM_VOF_CODE; }
};
class OGFM_VOF : public GFM_base {
 public:
  explicit OGFM_VOF(const sim_info& params) : GFM_base(params) {}
  int kind() const override { return GFM_OGFM_VOF; }
};

// ---------------------------------------------------------------------------
// simulations
// ---------------------------------------------------------------------------
class sim_base {
 public:
  virtual ~sim_base() {}
  virtual void run_sim(GFM_settingsfile SF) = 0;
};

// set_sim_parameters / set_sim_methods / set_sim_ICs are public here (the
// reference keeps them protected): a caller that runs its own loop on host
// grids gets the named case's set-up from them.
class sim_onefluid : public sim_base {
 public:
  void run_sim(GFM_settingsfile SF) override;
  void set_sim_parameters(const GFM_settingsfile& SF, sim_info& params, binarySGparams& eosparams);
  void set_sim_methods(const GFM_settingsfile& SF, std::shared_ptr<pure_RS_base>& RS, std::shared_ptr<FS_base>& FS);
  void set_sim_ICs(const GFM_settingsfile& SF, const sim_info& params, const binarySGparams& eosparams,
                   grideuler2type& grid);
  template <class Grid>
  double compute_dt(double CFL, const sim_info& params, const Grid& grid, const binarySGparams& eosparams, double T,
                    double t) {
    std::vector<double> U;
    grid_to_planes(grid, U);
    return detail::compute_dt_onefluid(CFL, params, U, eosparams, T, t);
  }
};

class sim_twofluid : public sim_base {
 public:
  void run_sim(GFM_settingsfile SF) override;
  void set_sim_parameters(const GFM_settingsfile& SF, sim_info& params, binarySGparams& eosparams);
  void set_sim_methods(const GFM_settingsfile& SF, const sim_info& params, std::shared_ptr<FS_base>& FS,
                       std::shared_ptr<GFM_base>& GFM, std::shared_ptr<GFM_ITM_interface>& ls);
  void set_sim_ICs(const GFM_settingsfile& SF, const sim_info& params, const binarySGparams& eosparams,
                   grideuler2type& grid1, grideuler2type& grid2, GFM_ITM_interface& ls);
  // the CFL step (CFL already ramped by the caller, as in the reference's loop)
  template <class Grid>
  double compute_dt(double CFL, const sim_info& params, const Grid& grid1, const Grid& grid2,
                    const GFM_ITM_interface& ls, const binarySGparams& eosparams, double T, double t) {
    std::vector<double> U1, U2;
    grid_to_planes(grid1, U1);
    grid_to_planes(grid2, U2);
    return detail::compute_dt_twofluid(CFL, params, U1, U2, ls.field(), ls.itm(), eosparams, T, t);
  }
};

}  // namespace gfm_gb300

#endif
