// Internal declarations shared by the CUDA translation units: the context
// (device-resident grids of one instance), the padded SoA layout, and the
// boundary-condition index mapping used by kernels that fuse apply_BCs_euler.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include "gfm_math.cuh"
#include "../../include/gfm_gb300.h"

namespace gfm {

// kernels launched by this library (reported by gfm_launch_count)
extern std::atomic<long long> g_launches;
inline void counted(int n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Geometry + EOS of one instance, passed by value to kernels.
struct GridP {
  int Nx, Ny, g;        // real cells, ghost width
  int nr, nc;           // padded rows / columns = Ny + 2g, Nx + 2g
  int pitch;            // doubles per row in device planes (>= nc)
  int64_t plane;        // doubles per plane = nr * pitch
  double x0, y0, dx, dy;
  double idx, idy;      // 1/dx, 1/dy
  int bcL, bcR, bcB, bcT;
  double g1, p1, g2, p2;  // gamma1, pinf1, gamma2, pinf2
  Gas gas1, gas2;         // gamma-derived constants of each material
  bool periodic;
};

// Device time/step state, one per instance (written by kernels only).
struct DevTime {
  double t, dt, T, CFL;
  int numsteps;
  int active;              // t < T at the start of the step
  unsigned long long maxu_bits, maxv_bits;   // CFL reduction (positive doubles)
  uint32_t status;
  int n_ifc;               // interfacial cells of the last ghost fill
  int n_rounds;            // schedule rounds of the last interface solve
  unsigned long long newton_iters;
  unsigned long long ifc_iters;   // Newton iterations of the interface solves (Riemann, real GFM)
  int ifc_gated;                  // interface solves started from the learned proposal
  // the same three summed over the steps since the last gfm_set_time
  unsigned long long ifc_solves_total, ifc_iters_total, ifc_gated_total;
  int rc[8];               // realcells1 (imin,imax,jmin,jmax), realcells2
};

}  // namespace gfm

struct gfm_ctx {
  gfm::GridP P;
  int two_fluid;
  cudaStream_t stream;
  // conserved grids: U[f] current, Unew[f] flux-update output (swapped)
  double* U[2];
  double* Unew[2];
  // primitive work planes
  double* W[2];      // conversion / extrapolation ping
  double* Wt[2];     // extrapolation pong
  double* Wc[2];     // copy of the first conversion (modified GFM)
  double* phi;
  double* phi_a;     // level-set stage buffers
  double* phi_b;
  double* phi0;      // reinitialisation reference
  double* nrm;       // 5 planes: gradient of phi (2), unit normal (2), |gradient|
  double* vel;       // 2 planes: velocity field handed to the level set
  double* vel_t;     // 2 planes: extension-velocity pong
  uint8_t* mask;     // interfacial-cell mask (real cells only)
  int* ifc_map;      // cell -> interface list index, -1 elsewhere
  int* ifc_list;     // interfacial cells in row-major order
  int* chunk_count;  // per-CTA counts of the compaction
  int n_chunks;
  int chunk;         // cells per CTA of the chunked kernels (k_prims, k_vof_prims, k_compact)
  int num_sms;       // SMs of the device, and of the far partition of the overlapped ghost fill
  int far_sms;
  int chain_sms;   // SMs of the overlapped ghost fill's chain partition
  int chain_ctas;  // CTAs of the interface loop (8 warps each) on that partition
  // The partitions the overlapped ghost fill can take (n_parts pairs of chain
  // and far streams; part: the one in use) and the timing events of this
  // step's chain and far paths (fork, near sweeps done, far flux done; null
  // when the step is not measured), from which the next steps choose.
  int n_parts, part;
  cudaStream_t part_chain[2], part_far[2];
  int part_sms[2];
  int chain_ctas_per_sm;
  cudaEvent_t part_ev[3];
  double* stage;     // packed (unpitched) copy of the whole state: 4, 4 and 1 planes of nr x nc
                     // (gfm_upload_state / gfm_download_state)
  // per-interface work arrays (capacity = Nx*Ny)
  int* ifc_done;
  int* ifc_pred;     // 8 per interface
  double* ifc_out;   // 8 per interface: star state (4), extension velocity (2), rho* other side, spare
  double* ifc_mrp;   // 8 per mixed cell of the VOF loop: MRPsoln1, MRPsoln2
  int* probe_ij;     // Riemann GFM: per interfacial cell and side, the bilinear probe's cell (i0, j0)
  double* probe_w;   // and its 4 weights
  int* probe_dep;    // and per bilinear corner the list entry whose published value it reads, or -1
  int itm;           // interface tracker of the last method used (GFM_ITM_*)
  int* ifc_opp;      // real GFM: opposite cell
  long long ifc_spin_limit;  // polls before an interface-loop wait gives up (0: the default)
  int flux_shape;    // tile shape of the flux update (FLUX_SHAPE_*; the overlapped passes use 16 x 32)
  int ifc_withhold;  // test hook: 1 + the interface-list entry left unsolved (0: none)
  gfm::DevTime* dtime;
  gfm::DevTime* h_dtime;  // pinned host mirror
  int steps_done_host;
  // overlapped ghost fill (Riemann and real GFM): the interface chain runs on
  // a small SM partition while the far field is extrapolated and updated on
  // the rest (see launch_ghost_fill_overlapped)
  double* SF[5][2];       // the far field's first five extrapolation sweeps [sweep][fluid]
  uint8_t* near_cell;     // real cells within 6 (Chebyshev) of an interfacial cell
  int* band_cls;          // cells within 6: 7 - the distance (ghost cells: their source's), else 0
  int* band_list;         // 7 segments of band_stride entries: the cells (ghost cells included, by
                          // their source) at distance 0, 1, ..., 6
  int64_t band_stride;
  int* list_n;            // the 7 segments' counts
  int* tile_near;         // per flux tile: its region holds a near cell
  cudaStream_t s_chain, s_far;
  cudaEvent_t ev_fork, ev_chain, ev_far;
  cudaEvent_t ev_far_final;   // far cells' conserved grids and velocities written
  cudaEvent_t tev[6];     // timing events of the overlapped schedule (gfm_step_timed)
  int timing;
  int overlap_ok;         // SM partitions (or two side streams) exist
  int overlap;            // GFM_OVERLAP_* mode (gfm_set_overlap)
  cudaStream_t s_ls;      // level-set update beside the flux update (second-highest priority)
  cudaEvent_t ev_ls_fork, ev_ls_done;
  // overlapped schedule: the work after the interface chain (near-field
  // extrapolation and flux update) on a highest-priority stream, so that its
  // CTAs take the SMs that the far field's flux update frees
  cudaStream_t s_near;
  cudaEvent_t ev_near, ev_phi_free;
  cudaEvent_t ev_lists;   // band lists, near cells and flux-tile flags written (far stream)
  struct gfm_mlp* mlp;    // learned proposal for the interface solves (gfm_set_mlp), or null
  float* cap_X;           // capture of gated interface problems (gfm_capture_interface_problems), or null
  float* cap_Y;
  int* cap_count;
  int cap;
  int graph_mode;         // launches are being recorded into a CUDA graph
  // the step's CFL reduction runs inside the ghost fill's conversion (k_prims)
  // with this last-block counter; null when a separate k_cfl computes dt
  unsigned int* cfl_counter;
};

namespace gfm {

// Source of a padded cell under apply_BCs_euler (headers/euler_bc.hpp:5-103):
// every ghost cell equals one real cell, with u negated (flipu) and/or v
// negated (flipv).  Requires Nx >= g and Ny >= g, so sources are real cells.
struct BCSrc { int i, j; bool flipu, flipv; };

__host__ __device__ inline BCSrc bc_source(const GridP& P, int i, int j) {
  BCSrc s;
  s.flipu = false; s.flipv = false;
  if (P.periodic) {
    s.i = (i - P.g + P.Ny) % P.Ny + P.g;
    s.j = (j - P.g + P.Nx) % P.Nx + P.g;
    return s;
  }
  s.i = i; s.j = j;
  if (j < P.g) { s.j = 2 * P.g - j - 1; s.flipu = (P.bcL == GFM_BC_REFLECTIVE); }
  else if (j >= P.Nx + P.g) { s.j = 2 * (P.Nx + P.g) - 1 - j; s.flipu = (P.bcL == GFM_BC_REFLECTIVE); }
  if (i < P.g) { s.i = 2 * P.g - i - 1; s.flipv = (P.bcB == GFM_BC_REFLECTIVE); }
  else if (i >= P.Ny + P.g) { s.i = 2 * (P.Ny + P.g) - 1 - i; s.flipv = (P.bcT == GFM_BC_REFLECTIVE); }
  return s;
}

__host__ __device__ inline bool is_real(const GridP& P, int i, int j) {
  return i >= P.g && i < P.Ny + P.g && j >= P.g && j < P.Nx + P.g;
}

__device__ __forceinline__ int64_t cidx(const GridP& P, int i, int j) { return (int64_t)i * P.pitch + j; }

__device__ __forceinline__ V4 load4(const double* A, const GridP& P, int64_t c) {
  return V4{A[c], A[c + P.plane], A[c + 2 * P.plane], A[c + 3 * P.plane]};
}
__device__ __forceinline__ void store4(double* A, const GridP& P, int64_t c, const V4& v) {
  A[c] = v.a; A[c + P.plane] = v.b; A[c + 2 * P.plane] = v.c; A[c + 3 * P.plane] = v.d;
}

__device__ __forceinline__ void raise_status(DevTime* dt, uint32_t bits) {
  if (bits) atomicOr(&dt->status, bits);
}

// flux-update tiles (k_flux_update): TX x TY real cells per CTA, 2-cell halo.
// 16 x 32 (512 threads, one CTA per SM) is the default shape and the one the
// overlapped schedule's tile marking uses: on the 1000x400 shock-bubble's
// whole run 2.046 ms per step against 2.064 with 16 x 16, 2.106 with 32 x 8
// and 2.400 with 64 x 4 (the far tiles' update 1.212 against 1.244, 1.307 and
// 1.752 ms).
constexpr int FLUX_TX = 16;
constexpr int FLUX_TY = 32;
inline int flux_tiles_x(const GridP& P) { return (P.Nx + FLUX_TX - 1) / FLUX_TX; }
inline int flux_tiles_y(const GridP& P) { return (P.Ny + FLUX_TY - 1) / FLUX_TY; }

// tile selection of the flux update
enum { TILES_ALL = 0, TILES_FAR = 1, TILES_NEAR = 2 };
// tile shapes of the flux update (gfm_ctx::flux_shape)
enum { FLUX_SHAPE_32x8 = 0, FLUX_SHAPE_16x16 = 1, FLUX_SHAPE_64x4 = 2, FLUX_SHAPE_16x32 = 3, FLUX_SHAPES = 4 };
constexpr int FLUX_SHAPE_DEFAULT = FLUX_SHAPE_16x32;   // FLUX_TX x FLUX_TY
int flux_tile_w(int shape);
int flux_tile_h(int shape);
// the persistent flux update of a batch (k_flux_batch): per-instance
// arguments (flux_batch_args_size() bytes each, filled by flux_batch_args),
// work items instance << 24 | fluid slot << 23 | tile, two counters at zero
void flux_batch_args(const gfm_ctx* ctx, void* out);
size_t flux_batch_args_size();
void launch_flux_batch(int fs, int shape, const void* args, const uint32_t* items, int n_items,
                       unsigned int* counters, int ctas, cudaStream_t stream);
int flux_batch_occupancy(int fs, int shape);

// kernel launch helpers (defined in the .cu files)
void launch_fs_update(gfm_ctx* ctx, int fs, int fluid_mask);
void launch_fs_update_sel(gfm_ctx* ctx, int fs, int fluid_mask, int tiles, cudaStream_t stream);
// SM partitions of a device for the overlapped ghost fill: n pairs of
// (chain, far) streams with chain_sms[k] SMs on the chain side
struct GreenParts {
  int n;
  int chain_sms[2];
  cudaStream_t chain[2], far[2];
};
bool green_streams(int device, GreenParts* parts);
void launch_ghost_fill_overlapped(gfm_ctx* ctx, const gfm_method_desc* m);
void launch_bcs(gfm_ctx* ctx, int fluid_mask);
void launch_commit(gfm_ctx* ctx, int fluid_mask, bool bcs);
void launch_cfl(gfm_ctx* ctx, double CFL, double T);
void launch_ghost_fill(gfm_ctx* ctx, const gfm_method_desc* m);
// the step's level set: parts 1 the advection stages, 2 phi := the result
// (or the reinitialisation from it), 3 both
void launch_level_set(gfm_ctx* ctx, const gfm_method_desc* m, cudaStream_t s, int parts,
                      cudaEvent_t phi_free = nullptr);
void launch_ghost_fill_vof(gfm_ctx* ctx, const gfm_method_desc* m);
void launch_vof_update(gfm_ctx* ctx, cudaStream_t s);
void launch_end_step(gfm_ctx* ctx);
void prepare_kernels();
void prepare_step_kernels();   // occupancy of the grid-stride kernels (gfm_step.cu)
const float* mlp_params(const struct gfm_mlp* m);   // the network's FP32 parameters (device)
const uint32_t* mlp_frag(const struct gfm_mlp* m);  // its B fragments for mlp_forward_warp_tc (device)
void launch_mlp_frag_pack(const struct gfm_mlp* m, cudaStream_t s);   // refresh them from the parameters
// nsteps iterations of the time loop on ctx's stream (gfm_step, gfm_step_timed)
gfm_status_t run_steps(gfm_ctx* ctx, const gfm_method_desc* m, int nsteps, double* phase_ms);
// one-stream step split around the flux update (a batch's phased schedule)
gfm_status_t step_front(gfm_ctx* ctx, const gfm_method_desc* m);
gfm_status_t step_back(gfm_ctx* ctx, const gfm_method_desc* m);
gfm_status_t validate_method(gfm_ctx* ctx, const gfm_method_desc* m);
double* mass_scratch(gfm_ctx* ctx);   // 256 + 1 doubles of the mass reduction
gfm_status_t launch_status();   // GFM_ERR_CUDA (and a message) if a launch failed

}  // namespace gfm
