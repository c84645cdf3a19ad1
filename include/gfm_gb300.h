/*
 * gfm_gb300.h -- C ABI of the GB300 two-fluid ghost-fluid Euler step.
 *
 * Every entry point takes plain pointers and sizes; device memory is owned by
 * the context.  All calls are ordered on the context's CUDA stream (settable
 * with gfm_set_stream).  Each returns a gfm_status_t.
 *
 * Host layout of one fluid grid: 4 planes (rho, rho u, rho v, E), each
 * (Ny + 2 numGC) rows x (Nx + 2 numGC) columns, row i = y index, column
 * j = x index, row-major -- the reference's grid[i][j](k) with k the plane.
 *
 * Reference interfaces replaced (paths within murraycutforth/PhD-2D-GFM):
 *   sim_info / binarySGparams        -> gfm_grid_desc
 *   GFM_settingsfile keys FS, GFM, ITM, CFL -> gfm_method_desc
 *                                       (headers/GFM_settingsfile.hpp:24-59)
 *   FS_base::pure_fluid_update       -> gfm_fs_update      (headers/FS_base.hpp:23-32)
 *   GFM_base::set_ghost_states       -> gfm_set_ghost_states (headers/GFM_base.hpp:37-47)
 *   apply_BCs_euler                  -> gfm_apply_bcs      (headers/euler_bc.hpp:5)
 *   sim_twofluid::compute_dt         -> gfm_compute_dt     (sourcecode/sim_twofluid.cpp:108-157)
 *   sim_onefluid::compute_dt         -> gfm_compute_dt     (sourcecode/sim_onefluid.cpp:68-91)
 *   ls->update_interface_coupled     -> gfm_ls_update      (sourcecode/sim_twofluid.cpp:72)
 *   the while (t < T) loop body      -> gfm_step           (sourcecode/sim_twofluid.cpp:64-88,
 *                                                           sourcecode/sim_onefluid.cpp:40-54)
 *   pure_RS_base::solve_RP           -> gfm_rs_pure_batch  (headers/pure_RS_base.hpp:13-20)
 *   mixed_RS_base::solve_mixed_RP    -> gfm_rs_mixed_batch (headers/mixed_RS_base.hpp:12-24)
 *   sim_twofluid::fluid_mass         -> gfm_fluid_mass     (sourcecode/sim_twofluid.cpp:1803-1827)
 */
#ifndef GFM_GB300_H
#define GFM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int gfm_status_t;
/* return codes */
#define GFM_OK 0
#define GFM_ERR_ARG 1        /* invalid argument (null pointer, bad size, bad enum) */
#define GFM_ERR_CUDA 2       /* a CUDA runtime call failed */
#define GFM_ERR_NUMERIC 3    /* the device status word holds a numeric fault */
#define GFM_ERR_UNSUPPORTED 4
#define GFM_ERR_IO 5         /* a file could not be read or written, or is not a valid checkpoint */

/* boundary conditions (sim_info BC_L/R/B/T strings) */
#define GFM_BC_TRANSMISSIVE 0
#define GFM_BC_REFLECTIVE 1
#define GFM_BC_PERIODIC 2

/* flux solvers (settings key FS) */
#define GFM_FS_GODUNOV 0
#define GFM_FS_MUSCL 1

/* ghost-fluid methods (settings key GFM) */
#define GFM_OGFM 0
#define GFM_RIEMANN 1
#define GFM_REAL 2
#define GFM_MODIFIED 3
#define GFM_VOF 4          /* GFM_VOF: needs the VOF interface tracker */
#define GFM_OGFM_VOF 5     /* OGFM_VOF: needs the VOF interface tracker */

/* interface trackers (settings key ITM) */
#define GFM_ITM_LEVELSET 0 /* LS1 / LS5: phi is a signed distance, negative in fluid 1 */
#define GFM_ITM_VOF 1      /* PYVOF: phi holds z, the volume fraction of fluid 1 */

/* device status bits (gfm_get_device_status) */
#define GFM_ST_UNPHYSICAL (1u << 0)
#define GFM_ST_NEWTON_NO_CONVERGE (1u << 1)
#define GFM_ST_VACUUM (1u << 2)
#define GFM_ST_NAN (1u << 3)
#define GFM_ST_DT_NONPOSITIVE (1u << 4)
#define GFM_ST_SCHEDULE_LIMIT (1u << 5)

/* sim_info + binarySGparams */
typedef struct {
  int Nx, Ny, numGC;
  double x0, y0, dx, dy;
  int BC_L, BC_R, BC_B, BC_T;
  double gamma1, pinf1, gamma2, pinf2;
} gfm_grid_desc;

/* the strategy choices of sim_twofluid::set_sim_methods */
typedef struct {
  int fs;                    /* GFM_FS_* */
  int gfm;                   /* GFM_* (two-fluid only) */
  int ls_order;              /* level-set advection order: 1 (upwind) or 5 (HOUC5 + RK3) */
  int reinit_every;          /* reinitialise phi every k steps; 0 = never */
  int reinit_iters;          /* pseudo-time iterations per reinitialisation */
  int use_extension_vfield;  /* GFM_base::use_extension_vfield */
  int use_slip_BCs;          /* GFM_base::use_slip_BCs */
  double CFL;                /* settings key CFL */
  double T;                  /* end time */
  int itm;                   /* GFM_ITM_*: level set (0, the default) or VOF */
} gfm_method_desc;

typedef struct gfm_ctx gfm_ctx;

/* Context: device grids for one (two_fluid = 0) or two fluids plus phi. */
gfm_status_t gfm_ctx_create(const gfm_grid_desc* grid, int two_fluid, gfm_ctx** out);
gfm_status_t gfm_ctx_destroy(gfm_ctx* ctx);
gfm_status_t gfm_set_stream(gfm_ctx* ctx, void* cuda_stream);

/* host <-> device copies of a fluid grid (fluid 1 or 2) and of phi */
gfm_status_t gfm_upload(gfm_ctx* ctx, int fluid, const double* U);
gfm_status_t gfm_download(gfm_ctx* ctx, int fluid, double* U);
gfm_status_t gfm_upload_phi(gfm_ctx* ctx, const double* phi);
gfm_status_t gfm_download_phi(gfm_ctx* ctx, double* phi);
/* all fields at once (U1, and U2 and phi for two fluids), one synchronisation */
gfm_status_t gfm_upload_state(gfm_ctx* ctx, const double* U1, const double* U2, const double* phi);
gfm_status_t gfm_download_state(gfm_ctx* ctx, double* U1, double* U2, double* phi);
/* gfm_upload_state without the synchronisation: the copies are ordered on the
 * context's stream before the calls that follow (a step, a download), and the
 * host buffers must stay unchanged until a later synchronising call on the
 * context (gfm_download_state, gfm_get_time) has returned */
gfm_status_t gfm_upload_state_async(gfm_ctx* ctx, const double* U1, const double* U2, const double* phi);

/* the velocity field of the last ghost fill (GFM_base::vfield, handed to the
 * interface tracker): 2 planes (u, v), layout of phi */
gfm_status_t gfm_download_velocity(gfm_ctx* ctx, double* vel);

/* interfacial-cell mask of the last ghost fill (Levelset::is_interfacial_cell
 * over real cells; 1 byte per padded cell, same layout as phi) */
gfm_status_t gfm_download_mask(gfm_ctx* ctx, uint8_t* mask);

/* time state kept on the device: t, step count, last dt */
gfm_status_t gfm_set_time(gfm_ctx* ctx, double t, int numsteps);
gfm_status_t gfm_get_time(gfm_ctx* ctx, double* t, int* numsteps, double* dt);
/* realcells1 and realcells2 of the last step (BBrange imin, imax, jmin,
 * jmax each; sourcecode/sim_twofluid.cpp:43-44): the cells each flux update
 * covers.  OGFM and OGFM_VOF shrink them to the real cells of their fluid
 * plus a margin (sourcecode/GFM_original.cpp:47-128); the other methods keep
 * the whole grid. */
gfm_status_t gfm_get_realcells(gfm_ctx* ctx, int* boxes);

/* One sub-step each, stream-ordered, dt kept on the device.
 *   gfm_compute_dt       the CFL step (with the ramp min(CFL, 0.2) while the
 *                        step count is below 5, sourcecode/sim_twofluid.cpp:66)
 *   gfm_set_ghost_states the ghost fill of the method (mask, interface solves,
 *                        extrapolation, velocity field; OGFM's realcells)
 *   gfm_fs_update        one fluid's flux update over its realcells box, no BCs
 *   gfm_ls_update        the interface tracker's update_interface_coupled: level
 *                        set advection, then the reinitialisation on the steps
 *                        that take one ((step count + 1) % reinit_every == 0,
 *                        the step count of gfm_set_time); VOF advection
 *   gfm_apply_bcs        apply_BCs_euler on one fluid
 *   gfm_set_step         dt (>= 0) and, if realcells is not NULL, the realcells
 *                        boxes (8 ints: realcells1 then realcells2, each imin,
 *                        imax, jmin, jmax; within the grid less a 2-cell rim) of
 *                        the sub-steps that follow, as the reference passes them
 *                        to pure_fluid_update (headers/FS_base.hpp:23-32)
 *   gfm_upload_velocity  the velocity field the tracker advects with (2 planes
 *                        u, v in the layout of phi), GFM_base::vfield */
gfm_status_t gfm_compute_dt(gfm_ctx* ctx, double CFL, double T);
gfm_status_t gfm_set_ghost_states(gfm_ctx* ctx, const gfm_method_desc* m);
gfm_status_t gfm_fs_update(gfm_ctx* ctx, int fs, int fluid);
gfm_status_t gfm_ls_update(gfm_ctx* ctx, const gfm_method_desc* m);
gfm_status_t gfm_apply_bcs(gfm_ctx* ctx, int fluid);
gfm_status_t gfm_set_step(gfm_ctx* ctx, double dt, const int* realcells);
gfm_status_t gfm_upload_velocity(gfm_ctx* ctx, const double* vel);
/* The interface field's kind for gfm_compute_dt before any call that takes a
 * method (gfm_set_ghost_states, gfm_ls_update and gfm_step record it): with
 * GFM_ITM_VOF, phi holds z and fluid 1 is where 0.5 - z < 0. */
gfm_status_t gfm_set_interface_tracker(gfm_ctx* ctx, int itm);

/* nsteps iterations of the reference's time loop body (CFL ramp, dt, ghost
 * fill, two flux updates, level set, BCs, t += dt).  Steps after t reaches
 * T do nothing, as the reference's loop would have stopped. */
gfm_status_t gfm_step(gfm_ctx* ctx, const gfm_method_desc* m, int nsteps);

/* gfm_step with CUDA events recorded on the context's stream around each
 * phase; adds the milliseconds of each phase to phase_ms[GFM_NPHASES]:
 * 0 CFL/dt, 1 ghost fill, 2 flux update (both fluids, one launch),
 * 3 boundary conditions (the commit of the new values) and the part of the
 * level set not hidden (it runs beside the flux update and the commit),
 * 4 end of step; phases 0-4 add up to the step.  With the overlapped schedule (gfm_set_overlap) phase 1 runs up
 * to the flux update of the tiles near the interface and phase 2 is that
 * update; phases 5-8 then time parts that overlap inside phases 1-2:
 * 5 the interface loop, 6 the far-field partition's work, 7 the exact
 * extrapolation and conversion of near cells after the loop, 8 the flux
 * update of the far tiles (within 6).  Phases 5-8 are 0 without overlap. */
#define GFM_NPHASES 9
gfm_status_t gfm_step_timed(gfm_ctx* ctx, const gfm_method_desc* m, int nsteps, double* phase_ms);

/* Schedule of the ghost fill for the Riemann and real GFM.
 *   GFM_OVERLAP_OFF   every phase on the context's stream in turn
 *   GFM_OVERLAP_ON    the interface loop on a small SM partition while the
 *                     far field is extrapolated and updated on the rest (8 or
 *                     16 SMs for the loop, chosen step by step from the
 *                     measured times of earlier steps' loop and far field;
 *                     GFM_CHAIN_SMS in the environment, a multiple of 8, fixes
 *                     it)
 *   GFM_OVERLAP_AUTO  (default) ON for the Riemann GFM, whose bilinear probes
 *                     chain interfacial cells many deep, OFF for the real GFM,
 *                     whose cells depend on one opposite cell at most
 * Results are identical in every mode.  GFM_ERR_UNSUPPORTED when ON or AUTO
 * is asked of a context without SM partitions (or side streams). */
#define GFM_OVERLAP_OFF 0
#define GFM_OVERLAP_ON 1
#define GFM_OVERLAP_AUTO 2
gfm_status_t gfm_set_overlap(gfm_ctx* ctx, int mode);

/* Newton iteration limit of the context's exact Riemann solves (flux update
 * and interface solves; default 60).  A solve that reaches it stops there
 * and sets GFM_ST_NEWTON_NO_CONVERGE: the reference has no limit of its own
 * (its solver is an absent library), so this is the device-side stand-in for
 * a solve that does not converge. */
gfm_status_t gfm_set_newton_limit(gfm_ctx* ctx, int max_iterations);

/* Bounded waits of the interface loop (Riemann, real and VOF GFMs): each
 * wait for an earlier cell's result polls its completion flag at most
 * spin_limit times (0: the default, about a second) and then gives up,
 * abandons its own cell and sets GFM_ST_SCHEDULE_LIMIT; the kernel returns
 * and the context stays usable.  withheld_entry (>= 0) is a failure-detection
 * hook for tests: that entry of the interface list (row-major order) is
 * neither solved nor published, so its dependants' waits run out (-1: none,
 * the default).  The step's results are not valid after a withheld entry. */
gfm_status_t gfm_set_interface_wait(gfm_ctx* ctx, int64_t spin_limit, int withheld_entry);

/* Tile shape of the context's flux update: 16 x 32 cells (the default, 512
 * threads per CTA), 16 x 16, 32 x 8 or 64 x 4 (256 threads) per CTA.  Results
 * are identical for every shape (each face flux is formed once and each cell
 * sums its faces in the reference's order); the time differs with the grid.
 * The overlapped ghost fill's passes always use 16 x 32.  gfm_batch_autotune
 * chooses it per grid-size class. */
#define GFM_FLUX_TILE_32x8 0
#define GFM_FLUX_TILE_16x16 1
#define GFM_FLUX_TILE_64x4 2
#define GFM_FLUX_TILE_16x32 3
gfm_status_t gfm_set_flux_tile(gfm_ctx* ctx, int shape);

/* number of kernels this library has launched since it was loaded */
int64_t gfm_launch_count(void);

/* Status word OR-ed by kernels since the last clear (GFM_ST_* bits). */
gfm_status_t gfm_get_device_status(gfm_ctx* ctx, uint32_t* status);
gfm_status_t gfm_clear_device_status(gfm_ctx* ctx);

/* Statistics of the last step: interfacial cells, schedule rounds, Newton
 * iterations summed over all exact Riemann solves. */
gfm_status_t gfm_get_stats(gfm_ctx* ctx, int64_t* n_interfacial, int64_t* n_rounds, int64_t* newton_iters);

/* mass of fluid 1 (interiorsign = -1, phi < 0) or 2 (+1, phi > 0) */
gfm_status_t gfm_fluid_mass(gfm_ctx* ctx, double interiorsign, double* mass);

/* Batched exact Riemann solves on DEVICE arrays (n states of 4 doubles, AoS).
 * pure: flux at x/t = 0 (pure_RS_exact::solve_RP).
 * mixed: out[4*k..] = (p_star, u_star, rho_star_L, rho_star_R). */
gfm_status_t gfm_rs_pure_batch(int n, int paralleltox, double gamma, double pinf, const double* UL,
                               const double* UR, double* flux, uint32_t* status, void* cuda_stream);
gfm_status_t gfm_rs_mixed_batch(int n, double gammaL, double pinfL, double gammaR, double pinfR,
                                const double* UL, const double* UR, double* out, uint32_t* status,
                                void* cuda_stream);

/* Named test cases: sim_type "onefluid" or "twofluid"; test_case one of the
 * reference's (circularexplosion, TTC1_x .. TTC5_y, ST1_x, ST2_y, GDA,
 * shocked_helium_bubble, shocked_R22_bubble) or shock_bubble,
 * underwater_explosion_sg.
 * gfm_case_params: sim_*::set_sim_parameters (sourcecode/sim_twofluid.cpp:336-490,
 *                  sourcecode/sim_onefluid.cpp:96-146); T is the end time.
 * gfm_case_init:   sim_*::set_sim_ICs + apply_BCs_euler (sourcecode/sim_twofluid.cpp:599-1799,
 *                  sourcecode/sim_onefluid.cpp:196-449) into HOST arrays in the
 *                  layout above (U2 and phi unused for one fluid). */
gfm_status_t gfm_case_params(const char* sim_type, const char* test_case, int Nx, int Ny, gfm_grid_desc* grid,
                             double* T);
gfm_status_t gfm_case_init(const char* sim_type, const char* test_case, const gfm_grid_desc* grid, double* U1,
                           double* U2, double* phi);

/* Batches: many independent instances (grids of any size, their own EOS
 * parameters, time and dt; one fluid count for all) stepped together.
 * The reference runs one simulation per process; a batch advances many in
 * one call, which fills the GPU with small grids and overlaps the instances'
 * latency-bound interface loops.  Each instance is an ordinary context
 * (gfm_batch_instance): upload, download, time and status calls work on it
 * as on a context of its own, ordered on the instance's stream.
 *   gfm_step_batched_graph       nsteps steps of every instance: 8 steps of
 *                                all instances are recorded once into a CUDA
 *                                graph (per method descriptor) and replayed;
 *                                a remainder is issued directly; instances run
 *                                side by side on their own streams
 *   gfm_step_batched_sequential  the same steps, one instance after another
 *                                on the batch stream (the unbatched way)
 * Both give each instance the results of stepping it alone.  The batch
 * stream (gfm_batch_set_stream, default: the batch's own) orders the call
 * after earlier work on the instance streams and before later work on them.
 * Instances use the one-stream ghost-fill schedule (GFM_OVERLAP_OFF). */
typedef struct gfm_batch gfm_batch;
gfm_status_t gfm_batch_create(const gfm_grid_desc* grids, int n, int two_fluid, gfm_batch** out);
gfm_status_t gfm_batch_destroy(gfm_batch* b);
gfm_status_t gfm_batch_instance(gfm_batch* b, int i, gfm_ctx** ctx);
gfm_status_t gfm_batch_set_stream(gfm_batch* b, void* cuda_stream);
gfm_status_t gfm_step_batched_graph(gfm_batch* b, const gfm_method_desc* m, int nsteps);
gfm_status_t gfm_step_batched_sequential(gfm_batch* b, const gfm_method_desc* m, int nsteps);
gfm_status_t gfm_batch_synchronize(gfm_batch* b);
/* Schedule of a batched step (both give each instance the results of
 * stepping it alone):
 *   GFM_BATCH_STREAMS  (default) each instance's whole step on its own
 *                      stream, the instances side by side
 *   GFM_BATCH_PHASED   every instance up to its flux update, then one
 *                      persistent flux launch per tile shape over the tiles of
 *                      all instances (CTAs pull instance / fluid / tile work
 *                      items, the largest instances first), then every
 *                      instance's commit
 * gfm_batch_autotune times, on the batch's own current state (restored
 * afterwards), the flux tile shapes of each grid-size class (padded cells
 * below 2^17, below 2^19, larger; on the class's largest instance) and then
 * the two schedules over `steps` steps (rounded up to a multiple of 8), keeps
 * the fastest, and writes a JSON report of the times into report (report_len
 * bytes, may be NULL). */
#define GFM_BATCH_STREAMS 0
#define GFM_BATCH_PHASED 1
gfm_status_t gfm_batch_set_schedule(gfm_batch* b, int schedule);
gfm_status_t gfm_batch_autotune(gfm_batch* b, const gfm_method_desc* m, int steps, char* report, int report_len);

/* Learned star-pressure proposal (no counterpart in the reference): a
 * multilayer perceptron 10 -> 64 -> 64 -> 64 -> 1 (SiLU) maps a two-material
 * Riemann problem's normalised states (rho, u, p + pinf, gamma, pinf of both
 * sides) to the log of p* relative to the solver's two-shock guess; it is
 * applied where that guess moved far (|log| > 1e-2) from the PVRS guess, and
 * Newton's method runs from the proposal to the usual tolerance.
 *   gfm_mlp_create            He-initialised parameters (9089 floats,
 *                             layout W1[10][64] b1 W2[64][64] b2 W3 b3 w4[64] b4)
 *   gfm_mlp_get/set_params    host copies (save / load)
 *   gfm_mlp_generate          n training problems on the device (DEVICE X[n][10],
 *                             Y[n]): gammas U[1.09,4.4], pinf in {0,6e8},
 *                             p_L 10^U[3,8], p_R/p_L log-U[1e-3,1e5], rho_L
 *                             10^U[-1,3], rho_R/rho_L log-U[1e-3,1e3], jump in u
 *                             U[-3,3] x mean sound speed; targets from the exact solver
 *   gfm_mlp_gradient          mean-square-error gradient over DEVICE X, Y (host grad)
 *   gfm_mlp_train             Adam over shuffled minibatches, cosine learning
 *                             rate; loss_per_epoch (host, epochs floats) or NULL
 *   gfm_mlp_infer             DEVICE X[n][10] -> out[n]: FP32 on CUDA cores
 *                             (tensor_cores = 0), BF16 tensor cores with
 *                             tcgen05 over tiles of 128 problems (1), or the
 *                             interface loop's warp-level path, one problem per
 *                             warp with mma.sync BF16 tiles (2); FP32 accumulation
 *   gfm_rs_mixed_batch_learned  gfm_rs_mixed_batch with the proposal (use_net =
 *                             1) or the two-shock guess (0); iters[n] receives
 *                             each solve's Newton iteration count */
typedef struct gfm_mlp gfm_mlp;
gfm_status_t gfm_mlp_create(uint64_t seed, gfm_mlp** out);
gfm_status_t gfm_mlp_destroy(gfm_mlp* m);
gfm_status_t gfm_mlp_set_params(gfm_mlp* m, const float* params);
gfm_status_t gfm_mlp_get_params(gfm_mlp* m, float* params);
int gfm_mlp_param_count(void);
gfm_status_t gfm_mlp_generate(uint64_t seed, int n, float* X, float* Y, int* n_out, void* cuda_stream);
gfm_status_t gfm_mlp_gradient(gfm_mlp* m, const float* X, const float* Y, int n, float* grad, float* loss,
                              void* cuda_stream);
gfm_status_t gfm_mlp_train(gfm_mlp* m, const float* X, const float* Y, int n, int epochs, int batch, float lr,
                           uint64_t seed, float* loss_per_epoch, void* cuda_stream);
gfm_status_t gfm_mlp_infer(gfm_mlp* m, const float* X, int n, float* out, int tensor_cores, void* cuda_stream);
gfm_status_t gfm_rs_mixed_batch_learned(gfm_mlp* m, int n, double gammaL, double pinfL, double gammaR, double pinfR,
                                        const double* UL, const double* UR, double* out, int* iters,
                                        uint32_t* status, int use_net, void* cuda_stream);

/* The context's interface solves (Riemann and real GFM) start Newton's
 * method from the learned proposal where it applies (NULL: the two-shock
 * guess everywhere, the default).  Each warp of the interface loop evaluates
 * the network on the tensor cores on its cell's actual states (one problem at
 * a time, on the loop's latency-bound critical path: BF16 mma.sync tiles with
 * FP32 accumulation, the activations kept in the lanes that feed the next
 * layer).  The network is read at each step (training it between steps takes
 * effect).  Results differ from the default
 * only within the Newton tolerance (p* within about 2e-14); they are not
 * bit-identical to the oracle. */
gfm_status_t gfm_set_mlp(gfm_ctx* ctx, gfm_mlp* mlp);
/* Training data from the solver itself: while set, every step of the Riemann
 * or real GFM appends its gated interface problems (features of the states
 * the interface loop solves, and the target from the solved p*) to the
 * DEVICE arrays X[cap][10], Y[cap]; *count (DEVICE int, zeroed by the caller)
 * counts them (and may exceed cap: the rest are dropped).  NULL arrays stop
 * the capture. */
gfm_status_t gfm_capture_interface_problems(gfm_ctx* ctx, float* X, float* Y, int cap, int* count);
/* Interface solves of the last step: count, Newton iterations, and how many
 * started from the learned proposal. */
gfm_status_t gfm_get_interface_stats(gfm_ctx* ctx, int64_t* n_solves, int64_t* newton_iters, int64_t* n_proposed);
/* The same summed over the steps of gfm_step (and of batched steps) since the
 * context's last gfm_set_time or state upload: read once after a run, a
 * recorded graph included. */
gfm_status_t gfm_get_interface_totals(gfm_ctx* ctx, int64_t* n_solves, int64_t* newton_iters, int64_t* n_proposed);

/* Shock-bubble family of the batched workload: the 1000x400 shock-bubble's
 * geometry on any grid (width 0.25, square cells, height 0.25 Ny/Nx,
 * reflective top and bottom, transmissive ends), air (gamma 1.4, rho 1,
 * p 1e5) with a left-moving shock of Mach number `mach` at x = 0.9 width, a
 * bubble of fluid 1 (gamma_bubble, rho = rho_ratio, p 1e5) of radius
 * radius_frac x height at (0.7 width, height/2).  T is 1 (run by steps). */
/* Output files of the reference's drivers (sim_twofluid::output,
 * output_mass_error and the runtime file, sourcecode/sim_twofluid.cpp:163-331,
 * 92-103; sim_onefluid::output, sourcecode/sim_onefluid.cpp:169-192), numbers
 * printed as std::ostream prints them (%g).  Two-fluid: <base>-<n>-prims.dat,
 * -ls.dat, -vfield.dat, -z.dat, -schlieren.dat and <base>-GDAerr.dat;
 * one-fluid: <base>-<n>-prims.dat.
 *   gfm_write_output_files   from HOST arrays (layouts of gfm_download; field =
 *                            phi or z per itm, vel = 2 planes); no GPU involved
 *   gfm_writer_*             the same files from a context's device state:
 *                            gfm_writer_output stages the grids on the device
 *                            in stream order and returns; a copy stream and a
 *                            writer thread finish the files while the GPU
 *                            keeps stepping.  gfm_writer_mass appends one
 *                            masschange line (t, relative mass errors; masses
 *                            reduced on the device, numsteps == 0 starts the
 *                            file and sets the reference masses)
 *   gfm_run_sim              the reference's time loop with these outputs:
 *                            at the start, when t - lastoutput > T/output_freq
 *                            (two-fluid) or numsteps % output_freq == 0
 *                            (one-fluid), at the end; masschange every step */
typedef struct gfm_writer gfm_writer;
gfm_status_t gfm_write_output_files(const gfm_grid_desc* grid, const char* basename, int two_fluid, int itm,
                                    int numsteps, const double* U1, const double* U2, const double* field,
                                    const double* vel);
gfm_status_t gfm_writer_create(gfm_ctx* ctx, const gfm_grid_desc* grid, const char* basename, gfm_writer** out);
gfm_status_t gfm_writer_output(gfm_writer* w, int numsteps);
gfm_status_t gfm_writer_mass(gfm_writer* w, int numsteps, double t);
gfm_status_t gfm_writer_runtime(gfm_writer* w, double seconds);
gfm_status_t gfm_writer_finish(gfm_writer* w);
gfm_status_t gfm_writer_destroy(gfm_writer* w);
gfm_status_t gfm_run_sim(gfm_ctx* ctx, const gfm_method_desc* m, const gfm_grid_desc* grid, const char* basename,
                         int output_freq, int max_steps, double* seconds);

/* Checkpoint / resume (no counterpart in the reference).  A checkpoint holds
 * the grid description, t, the step count and the padded grids U1 (U2 and
 * the interface field for two fluids): everything later steps read, so a run
 * resumed from it continues bit for bit as the uninterrupted run would.
 * Format (little-endian): "GFMCKPT1", u32 version 1, u32 two_fluid, the grid
 * description field by field (i32 Nx, Ny, numGC, BC_L, BC_R, BC_B, BC_T; f64
 * x0, y0, dx, dy, gamma1, pinf1, gamma2, pinf2), f64 t, i32 numsteps, i32 0,
 * u64 plane count, the planes (rows of Nx + 2 numGC doubles), u64 FNV-1a hash
 * of everything before it.
 *   gfm_checkpoint_save / _load  a context's state (load: same grid, same
 *                                fluid count; GFM_ERR_IO for a bad file)
 *   gfm_checkpoint_write / _read host arrays; _read with NULL arrays returns
 *                                the header only */
gfm_status_t gfm_checkpoint_save(gfm_ctx* ctx, const char* path);
gfm_status_t gfm_checkpoint_load(gfm_ctx* ctx, const char* path);
gfm_status_t gfm_checkpoint_write(const char* path, const gfm_grid_desc* grid, int two_fluid, double t, int numsteps,
                                  const double* U1, const double* U2, const double* phi);
gfm_status_t gfm_checkpoint_read(const char* path, gfm_grid_desc* grid, int* two_fluid, double* t, int* numsteps,
                                 double* U1, double* U2, double* phi);

/* volume fraction z of fluid 1 (one padded plane, layout of phi) of a named
 * two-fluid case, the initial field of the VOF interface tracker */
gfm_status_t gfm_case_init_z(const char* test_case, const gfm_grid_desc* grid, double* z);

typedef struct {
  double mach, gamma_bubble, rho_ratio, radius_frac;
} gfm_bubble_params;
gfm_status_t gfm_case_shock_bubble(const gfm_bubble_params* p, int Nx, int Ny, gfm_grid_desc* grid, double* T);
gfm_status_t gfm_case_init_shock_bubble(const gfm_bubble_params* p, const gfm_grid_desc* grid, double* U1,
                                        double* U2, double* phi);
/* its volume fraction of fluid 1 (10x10 sub-sampled area fractions) */
gfm_status_t gfm_case_init_shock_bubble_z(const gfm_bubble_params* p, const gfm_grid_desc* grid, double* z);
/* Initial conditions written on the device into a context's grids (and phi,
 * or z for itm = GFM_ITM_VOF), time and step count reset: no host set-up or
 * upload.  Bit-identical to gfm_case_init / _z / gfm_case_init_shock_bubble,
 * except GDA's Gaussian density (exp from this library on the device, from
 * the C library on the host: within 1 ulp). */
gfm_status_t gfm_case_init_device(gfm_ctx* ctx, const char* sim_type, const char* test_case, int itm);
gfm_status_t gfm_case_init_shock_bubble_device(gfm_ctx* ctx, const gfm_bubble_params* p, int itm);

/* One-fluid time steps for callers that cannot allocate device memory.
 * No counterpart in the reference: it is an addition of this library.
 * Some callers cannot call cudaMalloc (a host runtime whose memory pool owns
 * the device; real-time code that may not block on an allocation after
 * start-up).  This entry point advances the caller's DEVICE grid U (layout as
 * above, unpitched) in place by up to nsteps steps of sim_onefluid's loop
 * (sourcecode/sim_onefluid.cpp:40-54); t and numsteps are in/out, status
 * receives the GFM_ST_* bits.  The grid description is checked as by
 * gfm_ctx_create (GFM_ERR_ARG otherwise).  It calls no cudaMalloc/cudaFree:
 * its scratch is a built-in 16 MiB device array, which limits the grid to
 * GFM_NOALLOC_MAX_CELLS padded cells ((Nx+2 numGC)(Ny+2 numGC)); larger
 * grids are rejected with GFM_ERR_ARG.  It works in the CUDA context current
 * on the calling thread; the first call in each context (once per device
 * with the runtime's primary context) looks up the array's device address.
 * Every call waits for its own work on the stream (it reads t, numsteps and
 * the status back), so no call can be recorded into a graph.  All calls
 * share the array: calls that overlap on the GPU race. */
#define GFM_NOALLOC_MAX_CELLS 524272
gfm_status_t gfm_onefluid_step_noalloc(const gfm_grid_desc* grid, const gfm_method_desc* m, double* U, int nsteps,
                                       double* t, int* numsteps, uint32_t* status, void* cuda_stream);

/* Measured FP64 peak of the current device: a dependent-chain-free FMA loop
 * on every SM for about 20 ms; *gflops = 2 x FMAs per second / 1e9. */
gfm_status_t gfm_fp64_peak(double* gflops, void* cuda_stream);

/* library version string */
const char* gfm_version(void);

#ifdef __cplusplus
}
#endif

#endif
