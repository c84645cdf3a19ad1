// Kernels of the two-fluid time step other than the flux update:
//   CFL time step             sim_twofluid::compute_dt   (sourcecode/sim_twofluid.cpp:108-157)
//                             sim_onefluid::compute_dt   (sourcecode/sim_onefluid.cpp:68-91)
//   boundary conditions       apply_BCs_euler            (headers/euler_bc.hpp:5-103)
//   ghost-fluid fill          GFM_{original,riemann,real,modified}::set_ghost_states
//   narrow-band extrapolation extrapolate_vector(_mgfm)  (sourcecode/extrapolate_vector.cpp:5-288)
//   extension velocity        extrapolate_extension_vfield (sourcecode/extrapolate_extension_vfield.cpp:4-122)
//   level set                 advection + reinitialisation (the project's own Levelset)
//
// Every kernel that the reference follows with apply_BCs_euler computes the
// ghost-layer cells itself: a ghost cell is a mirrored real cell, so its
// thread evaluates that real cell's update and applies the reflective signs.
#include "gfm_internal.cuh"
#include <mutex>
#include <unordered_map>
#include "gfm_mlp.cuh"
#include <climits>

namespace gfm {

// Cells per CTA of the chunked full-grid kernels (k_prims, k_vof_prims,
// k_compact): gfm_ctx::chunk, a multiple of 32 of at least 2048, sized so
// that the chunks make one wave of one CTA per SM on large grids.
constexpr int CHUNK_T = 512;

static int grid_blocks(int64_t n, int per) {
  int64_t b = (n + per - 1) / per;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

// Blocks of a grid-stride kernel of `threads` threads for one full wave on
// `sms` SMs: its resident CTAs per SM (queried once per kernel) times the
// SMs, capped by the cells to cover.  Every SM then takes the same share of
// the cells, where a grid of one CTA per 256 cells leaves a partial last wave
// on some SMs while the others idle.
static int wave_blocks(const void* kernel, int threads, int sms, int64_t n) {
  static std::mutex mu;
  static std::unordered_map<const void*, int> occ;
  int per = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = occ.find(kernel);
    if (it != occ.end()) {
      per = it->second;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0) != cudaSuccess || per < 1) {
        cudaGetLastError();
        per = 1;
      }
      occ[kernel] = per;
    }
  }
  if (sms < 1) sms = 152;
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)per * sms;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}
static int64_t padded_cells(const GridP& P) { return (int64_t)P.nr * P.nc; }

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
// std::max and std::min, NaN semantics included, with the comparison on the
// integer pipe (c_lt): the FP64 pipe bounds the kernels that use them
__device__ __forceinline__ double dmax_std(double a, double b) { return c_lt(a, b) ? b : a; }
__device__ __forceinline__ double dmin_std(double a, double b) { return c_lt(b, a) ? b : a; }
// |x| by clearing the sign bit (an integer operation)
__device__ __forceinline__ double fabs_bits(double x) { return from_bits(as_bits(x) & GFM_MAG_BITS); }

// Normal planes (k_prims): 0,1 raw central-difference gradient of phi,
// 2,3 unit normal with the reference's fallback to (1,0) below 1e-12
// (sourcecode/GFM_riemann.cpp:58-68), 4 the gradient's norm.
__device__ __forceinline__ void unit_normal(const double* nrm, const GridP& P, int64_t c, double& nx, double& ny) {
  nx = nrm[c + 2 * P.plane];
  ny = nrm[c + 3 * P.plane];
}

__device__ __forceinline__ V4 v4d(const V4& x, const V4& y) { return V4{x.a - y.a, x.b - y.b, x.c - y.c, x.d - y.d}; }

__device__ __forceinline__ void linear_to_ij(const GridP& P, int64_t lin, int& i, int& j) {
  i = (int)(lin / P.nc);
  j = (int)(lin - (int64_t)i * P.nc);
}

// ---------------------------------------------------------------------------
// CFL reduction + dt (last-block pattern); also the start-of-step flags
// ---------------------------------------------------------------------------
struct CflArgs {
  GridP P;
  const double* U1;
  const double* U2;
  const double* phi;   // null for one fluid
  DevTime* dt;
  unsigned int* counter;
  double CFL, T;
  int ogfm;            // realcells boxes start empty (GFM_original.cpp:47-55)
  int vof;             // phi holds the volume fraction z: get_sdf = 0.5 - z
};

__global__ void __launch_bounds__(256) k_cfl(CflArgs a) {
  const GridP& P = a.P;
  __shared__ double s_u[8], s_v[8];
  __shared__ bool s_last;
  DevTime* D = a.dt;
  const bool active = D->t < a.T;
  if (!active) {
    if (blockIdx.x == 0 && threadIdx.x == 0) D->active = 0;
    return;
  }
  double mu = 0.0, mv = 0.0;
  const int64_t n = (int64_t)P.Nx * P.Ny;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.Nx) + P.g, j = (int)(k % P.Nx) + P.g;
    int64_t c = cidx(P, i, j);
    bool f1 = (a.phi == nullptr) || (a.vof ? (0.5 - a.phi[c] < 0.0) : (a.phi[c] < 0.0));
    const double* U = f1 ? a.U1 : a.U2;
    double gm = f1 ? P.g1 : P.g2, pinf = f1 ? P.p1 : P.p2;
    V4 u = load4(U, P, c);
    double rho = u.a;
    const Recip R = recip(rho);   // the seven divisions by rho share one reciprocal
    double e = rdiv(u.d, R) - 0.5 * (rdiv(u.b, R) * rdiv(u.b, R) + rdiv(u.c, R) * rdiv(u.c, R));
    double p = eos_pressure(gm, pinf, e, rho);
    double cs = eos_soundspeed_r(gm, pinf, p, R);
    double xu = rdiv(fabs(u.b), R) + cs;
    double xv = rdiv(fabs(u.c), R) + cs;
    mu = dmax_std(mu, xu);   // NaN never replaces the running max (std::max semantics)
    mv = dmax_std(mv, xv);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mu = dmax_std(mu, __shfl_xor_sync(0xffffffffu, mu, o));
    mv = dmax_std(mv, __shfl_xor_sync(0xffffffffu, mv, o));
  }
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { s_u[w] = mu; s_v[w] = mv; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x >> 5); q++) { mu = dmax_std(mu, s_u[q]); mv = dmax_std(mv, s_v[q]); }
    // positive doubles order as their bit patterns
    atomicMax(&D->maxu_bits, (unsigned long long)__double_as_longlong(mu));
    atomicMax(&D->maxv_bits, (unsigned long long)__double_as_longlong(mv));
    __threadfence();
    unsigned int prev = atomicAdd(a.counter, 1u);
    s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    double maxu = __longlong_as_double((long long)atomicAdd(&D->maxu_bits, 0ull));
    double maxv = __longlong_as_double((long long)atomicAdd(&D->maxv_bits, 0ull));
    double cfl = (D->numsteps < 5) ? ((0.2 < a.CFL) ? 0.2 : a.CFL) : a.CFL;   // std::min(CFL, 0.2)
    double dx_u = P.dx / maxu, dy_v = P.dy / maxv;
    double dt = cfl * ((dy_v < dx_u) ? dy_v : dx_u);
    if (D->t + dt > a.T) dt = a.T - D->t;
    if (!(dt > 0.0)) D->status |= ST_DT_NONPOSITIVE;
    D->dt = dt;
    D->T = a.T;
    D->CFL = cfl;
    D->active = 1;
    D->maxu_bits = 0ull;
    D->maxv_bits = 0ull;
    int g = P.g;
    for (int f = 0; f < 2; f++) {
      if (a.ogfm) {
        D->rc[4 * f + 0] = g + P.Ny; D->rc[4 * f + 1] = g; D->rc[4 * f + 2] = g + P.Nx; D->rc[4 * f + 3] = g;
      } else {
        D->rc[4 * f + 0] = g; D->rc[4 * f + 1] = g + P.Ny; D->rc[4 * f + 2] = g; D->rc[4 * f + 3] = g + P.Nx;
      }
    }
    D->newton_iters = 0ull;
    D->ifc_iters = 0ull;
    D->ifc_gated = 0;
    *a.counter = 0u;
  }
}

// The start-of-step flags of k_cfl for the two-fluid steps whose CFL
// reduction runs inside the ghost fill's conversion (k_prims): nothing before
// the flux and level-set updates reads dt, so dt may follow the conversion.
__global__ void k_step_begin(GridP P, DevTime* D, double CFL, double T, int ogfm) {
  if (!(D->t < T)) {
    D->active = 0;
    return;
  }
  D->T = T;
  D->CFL = (D->numsteps < 5) ? ((0.2 < CFL) ? 0.2 : CFL) : CFL;   // std::min(CFL, 0.2)
  D->active = 1;
  const int g = P.g;
  for (int f = 0; f < 2; f++) {
    if (ogfm) {
      D->rc[4 * f + 0] = g + P.Ny; D->rc[4 * f + 1] = g; D->rc[4 * f + 2] = g + P.Nx; D->rc[4 * f + 3] = g;
    } else {
      D->rc[4 * f + 0] = g; D->rc[4 * f + 1] = g + P.Ny; D->rc[4 * f + 2] = g; D->rc[4 * f + 3] = g + P.Nx;
    }
  }
  D->newton_iters = 0ull;
  D->ifc_iters = 0ull;
  D->ifc_gated = 0;
}

// dt from the reduced maxima, by the last CTA of a fused reduction (the same
// operations as the last CTA of k_cfl)
__device__ void cfl_dt_from_max(const GridP& P, DevTime* D, unsigned int* counter) {
  __threadfence();
  const double maxu = __longlong_as_double((long long)atomicAdd(&D->maxu_bits, 0ull));
  const double maxv = __longlong_as_double((long long)atomicAdd(&D->maxv_bits, 0ull));
  const double cfl = D->CFL;
  const double dx_u = P.dx / maxu, dy_v = P.dy / maxv;
  double dt = cfl * ((dy_v < dx_u) ? dy_v : dx_u);
  if (D->t + dt > D->T) dt = D->T - D->t;
  if (!(dt > 0.0)) D->status |= ST_DT_NONPOSITIVE;
  D->dt = dt;
  D->maxu_bits = 0ull;
  D->maxv_bits = 0ull;
  *counter = 0u;
}

__global__ void k_end_step(DevTime* D) {
  if (D->active) {
    D->t += D->dt;
    D->numsteps += 1;
    D->ifc_solves_total += (unsigned long long)D->n_ifc;
    D->ifc_iters_total += D->ifc_iters;
    D->ifc_gated_total += (unsigned long long)D->ifc_gated;
  }
}

void launch_cfl_impl(gfm_ctx* ctx, double CFL, double T, bool ogfm, unsigned int* counter) {
  CflArgs a;
  a.P = ctx->P;
  a.U1 = ctx->U[0];
  a.U2 = ctx->two_fluid ? ctx->U[1] : ctx->U[0];
  a.phi = ctx->two_fluid ? ctx->phi : nullptr;
  a.dt = ctx->dtime;
  a.counter = counter;
  a.CFL = CFL;
  a.T = T;
  a.ogfm = ogfm ? 1 : 0;
  a.vof = (ctx->two_fluid && ctx->itm == GFM_ITM_VOF) ? 1 : 0;
  int64_t n = (int64_t)ctx->P.Nx * ctx->P.Ny;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_cfl<<<blocks, 256, 0, ctx->stream>>>(a); counted();
}

void launch_step_begin(gfm_ctx* ctx, double CFL, double T, bool ogfm) {
  k_step_begin<<<1, 1, 0, ctx->stream>>>(ctx->P, ctx->dtime, CFL, T, ogfm ? 1 : 0); counted();
}

// ---------------------------------------------------------------------------
// apply_BCs_euler on conserved grids (ghost cells only)
// ---------------------------------------------------------------------------
__global__ void k_bc_u(GridP P, double* U, const DevTime* D) {
  if (!D->active) return;
  int64_t n = (int64_t)P.nr * P.nc;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.nc), j = (int)(k % P.nc);
    if (is_real(P, i, j) && !P.periodic) continue;
    BCSrc s = bc_source(P, i, j);
    if (s.i == i && s.j == j) continue;
    V4 v = load4(U, P, cidx(P, s.i, s.j));
    if (s.flipu) v.b = -v.b;
    if (s.flipv) v.c = -v.c;
    store4(U, P, cidx(P, i, j), v);
  }
}

// End of the flux update: U := Unew on real cells and, with bcs, the ghost
// layers of apply_BCs_euler computed from the new real cells (one pass).
// Without bcs the ghost layers keep their values, as pure_fluid_update leaves them.
__global__ void k_commit_u(GridP P, const double* Unew, double* U, int bcs, const DevTime* D) {
  if (!D->active) return;
  int64_t n = (int64_t)P.nr * P.nc;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.nc), j = (int)(k % P.nc);
    bool r = is_real(P, i, j);
    if (!r && !bcs) continue;
    BCSrc s;
    if (r) { s.i = i; s.j = j; s.flipu = false; s.flipv = false; }
    else s = bc_source(P, i, j);
    V4 v = load4(Unew, P, cidx(P, s.i, s.j));
    if (s.flipu) v.b = -v.b;
    if (s.flipv) v.c = -v.c;
    store4(U, P, cidx(P, i, j), v);
  }
}

void launch_commit(gfm_ctx* ctx, int fluid_mask, bool bcs) {
  const int blocks = wave_blocks((const void*)k_commit_u, 256, ctx->num_sms, padded_cells(ctx->P));
  for (int f = 0; f < 2; f++)
    if (fluid_mask & (1 << f)) {
      k_commit_u<<<blocks, 256, 0, ctx->stream>>>(ctx->P, ctx->Unew[f], ctx->U[f], bcs ? 1 : 0, ctx->dtime);
      counted();
    }
}

void launch_bcs(gfm_ctx* ctx, int fluid_mask) {
  int64_t n = (int64_t)ctx->P.nr * ctx->P.nc;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  for (int f = 0; f < 2; f++)
    if (fluid_mask & (1 << f)) {
      k_bc_u<<<blocks, 256, 0, ctx->stream>>>(ctx->P, ctx->U[f], ctx->dtime);
      counted();
    }
}

// ---------------------------------------------------------------------------
// Ghost fill stage 1: conversion of both grids, phi gradient, interfacial
// mask, per-chunk interfacial counts.
// ---------------------------------------------------------------------------
struct PrimArgs {
  GridP P;
  const double* U1; const double* U2;
  double* W1; double* W2;
  double* Wc1; double* Wc2;   // optional copies (modified GFM)
  const double* phi;
  double* nrm;
  uint8_t* mask;
  int* ifc_map;
  int* chunk_count;
  int chunk;                  // cells per CTA
  DevTime* D;
  int check_both;             // 1: assert both grids (OGFM, RGFM); 0: the phi-selected one
  unsigned int* cfl_counter;  // non-null: also the step's CFL reduction and dt (k_cfl's)
  double* vel;                // non-null: the real cells' velocity field (overlapped schedule)
};

__global__ void __launch_bounds__(CHUNK_T) k_prims(PrimArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  __shared__ int s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  const int64_t n = (int64_t)P.nr * P.nc;
  const int64_t base = (int64_t)blockIdx.x * a.chunk;
  const Recip r2dx = recip(2.0 * P.dx), r2dy = recip(2.0 * P.dy);   // central-difference divisors
  uint32_t st = 0;
  int cnt = 0;
  double mu = 0.0, mv = 0.0;   // CFL maxima over the real cells (k_cfl's)
  for (int q = threadIdx.x; q < a.chunk; q += CHUNK_T) {
    int64_t lin = base + q;
    if (lin >= n) break;
    int i, j;
    linear_to_ij(P, lin, i, j);
    int64_t c = cidx(P, i, j);
    V4 u1 = load4(a.U1, P, c), u2 = load4(a.U2, P, c);
    double ph = a.phi[c];
    // conversion and is_physical_state of the same state share their operations
    bool ok1, ok2;
    Recip R1, R2;
    V4 w1 = cons_to_prims_phys(P.g1, P.p1, u1, &ok1, &R1);
    V4 w2 = cons_to_prims_phys(P.g2, P.p2, u2, &ok2, &R2);
    if (a.check_both) {
      if (!ok1 || !ok2) st |= ST_UNPHYSICAL;
    } else {
      if (!(c_le0(ph) ? ok1 : ok2)) st |= ST_UNPHYSICAL;
    }
    if (a.cfl_counter && is_real(P, i, j)) {
      // k_cfl's wave speeds from this conversion: the fluid with phi < 0 is
      // fluid 1, u = (rho u)/rho and p are the values just computed, and for
      // rho > 0 the quotient |rho u| / rho is |u| (round-to-nearest is
      // symmetric), otherwise it is formed as k_cfl forms it
      const bool f1 = c_lt0(ph);
      const V4& u = f1 ? u1 : u2;
      const V4& w = f1 ? w1 : w2;
      const Recip& R = f1 ? R1 : R2;
      const double cs = eos_soundspeed_r(f1 ? P.g1 : P.g2, f1 ? P.p1 : P.p2, w.d, R);
      const bool pos = c_gt0(u.a);
      const double xu = (pos ? fabs(w.b) : rdiv(fabs(u.b), R)) + cs;
      const double xv = (pos ? fabs(w.c) : rdiv(fabs(u.c), R)) + cs;
      mu = dmax_std(mu, xu);   // NaN never replaces the running max (std::max semantics)
      mv = dmax_std(mv, xv);
    }
    store4(a.W1, P, c, w1);
    store4(a.W2, P, c, w2);
    if (a.Wc1) { store4(a.Wc1, P, c, w1); store4(a.Wc2, P, c, w2); }
    if (a.vel && is_real(P, i, j)) {
      // the velocity field of a real cell is its real fluid's velocity after
      // the ghost fill, which changes only the real fluid of interfacial cells
      // (k_ifc_vel) and the other fluid of every cell: these are its values
      const V4& w = c_le0(ph) ? w1 : w2;
      a.vel[c] = w.b;
      a.vel[c + P.plane] = w.c;
    }
    double gx = 0.0, gy = 0.0;
    if (i >= 1 && i < P.nr - 1 && j >= 1 && j < P.nc - 1) {
      gx = rdiv(a.phi[c + 1] - a.phi[c - 1], r2dx);
      gy = rdiv(a.phi[c + P.pitch] - a.phi[c - P.pitch], r2dy);
    }
    // raw gradient, its norm, and the unit normal with the reference's
    // fallback (sourcecode/GFM_riemann.cpp:58-68), once per step
    double nn = sqrtx(gx * gx + gy * gy);
    double ux = 1.0, uy = 0.0;
    if (!c_lt(nn, 1e-12)) {
      const Recip rn = recip(nn);
      ux = rdiv(gx, rn);
      uy = rdiv(gy, rn);
    }
    a.nrm[c] = gx;
    a.nrm[c + P.plane] = gy;
    a.nrm[c + 2 * P.plane] = ux;
    a.nrm[c + 3 * P.plane] = uy;
    a.nrm[c + 4 * P.plane] = nn;
    uint8_t m = 0;
    if (is_real(P, i, j)) {
      bool s = c_le0(ph);
      m = (c_le0(a.phi[c - 1]) != s || c_le0(a.phi[c + 1]) != s || c_le0(a.phi[c - P.pitch]) != s ||
           c_le0(a.phi[c + P.pitch]) != s) ? 1 : 0;
    }
    a.mask[c] = m;
    a.ifc_map[c] = -1;
    cnt += m;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&s_cnt, cnt);
  uint32_t wst = __reduce_or_sync(0xffffffffu, st);
  if ((threadIdx.x & 31) == 0 && wst) atomicOr(&a.D->status, wst);
  __syncthreads();
  if (threadIdx.x == 0) a.chunk_count[blockIdx.x] = s_cnt;
  if (a.cfl_counter) {
    __shared__ double s_u[CHUNK_T / 32], s_v[CHUNK_T / 32];
    __shared__ bool s_last;
    for (int o = 16; o > 0; o >>= 1) {
      mu = dmax_std(mu, __shfl_xor_sync(0xffffffffu, mu, o));
      mv = dmax_std(mv, __shfl_xor_sync(0xffffffffu, mv, o));
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { s_u[w] = mu; s_v[w] = mv; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int q = 1; q < CHUNK_T / 32; q++) { mu = dmax_std(mu, s_u[q]); mv = dmax_std(mv, s_v[q]); }
      // positive doubles order as their bit patterns
      atomicMax(&a.D->maxu_bits, (unsigned long long)__double_as_longlong(mu));
      atomicMax(&a.D->maxv_bits, (unsigned long long)__double_as_longlong(mv));
      __threadfence();
      const unsigned int prev = atomicAdd(a.cfl_counter, 1u);
      s_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) cfl_dt_from_max(P, a.D, a.cfl_counter);
  }
}

// Stage 2: ordered compaction of the interfacial cells (row-major order).
__global__ void __launch_bounds__(CHUNK_T) k_compact(GridP P, const uint8_t* mask, const int* chunk_count,
                                                     int n_chunks, int chunk, int* list, int* ifc_map,
                                                     DevTime* D) {
  if (!D->active) return;
  __shared__ int s_off;
  __shared__ int s_warp[CHUNK_T / 32];
  if (threadIdx.x == 0) s_off = 0;
  __syncthreads();
  int part = 0;
  for (int b = threadIdx.x; b < (int)blockIdx.x; b += CHUNK_T) part += chunk_count[b];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0 && part) atomicAdd(&s_off, part);
  __syncthreads();
  int off = s_off;
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) D->n_ifc = off + chunk_count[blockIdx.x];
  const int64_t n = (int64_t)P.nr * P.nc;
  const int64_t base = (int64_t)blockIdx.x * chunk;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // cells base + it*CHUNK_T + tid of the chunk, in order of it then tid
  const int64_t end = base + chunk < n ? base + chunk : n;
  for (int it = 0; it < (chunk + CHUNK_T - 1) / CHUNK_T; it++) {
    int64_t lin = base + (int64_t)it * CHUNK_T + threadIdx.x;
    int m = 0;
    int i = 0, j = 0;
    if (lin < end) {
      linear_to_ij(P, lin, i, j);
      m = mask[cidx(P, i, j)];
    }
    unsigned bal = __ballot_sync(0xffffffffu, m);
    if (lane == 0) s_warp[w] = __popc(bal);
    __syncthreads();
    int wofs = 0, tot = 0;
    for (int q = 0; q < CHUNK_T / 32; q++) { if (q < w) wofs += s_warp[q]; tot += s_warp[q]; }
    if (m) {
      int k = off + wofs + __popc(bal & ((1u << lane) - 1u));
      list[k] = (int)lin;
      ifc_map[cidx(P, i, j)] = k;
    }
    off += tot;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// extrapolate_vector sweep (+ apply_BCs_euler on the updated grids), one
// launch per iteration.  mode 1 = extrapolate_vector_mgfm (interfacial cells
// are left unchanged).
// ---------------------------------------------------------------------------
constexpr int IFC_OUT = 8;   // doubles of interface output per interfacial cell

// Overlapped ghost fill: the interface loop changes only the real fluid of
// interfacial cells, and a sweep of extrapolate_vector reads a cell and its
// four neighbours, so after sweep k its values differ from those of the same
// sweeps without the loop's results (the far field's, computed beside the
// loop) only within k cells (Chebyshev) of an interfacial cell.  The exact
// extrapolation after the loop therefore writes, in sweep k = 1..6, the cells
// within k: it reads the previous exact sweep inside that band and the far
// field's previous sweep outside, and sweep 6 gives the cells within
// NEAR_RADIUS.  The band's cells are listed in BAND_CLASSES segments by
// distance 0..NEAR_RADIUS (k_band_lists).
constexpr int NEAR_RADIUS = 6;
constexpr int BAND_CLASSES = NEAR_RADIUS + 1;
// CTAs of the listed sweeps after the loop: the band holds a few thousand to
// about ten thousand cells, about one per thread of 40 CTAs of 256 threads
// (they share the loop's own SMs with the level set while the far field's
// flux update fills the other SMs; 20, 80 or 152 CTAs measured within 0.5%)
constexpr int NEAR_CTAS = 40;

struct ExtrapArgs {
  GridP P;
  const double* S1; const double* S2;   // grid1/grid2 of this iteration
  double* D1; double* D2;               // updated_grid1/2
  const double* phi;
  const double* nrm;
  const uint8_t* mask;
  const DevTime* D;
  DevTime* Dw;                          // status word of the fused conversion
  int mgfm;
  // overlay: the interface loop's writes (star state into the real fluid of
  // each interfacial cell) applied on the fly to the source reads
  const double* ov_out;
  const int* ov_map;
  int overlay;
  // band: only cells whose boundary-condition source is marked are written
  // (the others keep the buffer's earlier values), or null for every cell
  const uint8_t* band;
  // list: the cells to write (linear indices over the padded rows), or null
  // for every cell; a list replaces the band test.  It is `nclass`
  // consecutive segments of `list_stride` entries, segment q holding
  // list_n[q] cells.
  const int* list;
  const int* list_n;
  int nclass;
  int64_t list_stride;
  // exact sweep k >= 2 after the loop: F1/F2 the far field's sweep k - 1,
  // read where cls[c] < near_min (outside the band of sweep k - 1), or null
  const double* F1; const double* F2;
  const int* cls;
  int near_min;
  // the conversion back to conserved grids fused into the overlapped
  // schedule's last sweeps (k_finalize's work for these cells): fsel 0 none,
  // 1 the cells whose boundary-condition source is not near (fnear), 2 every
  // written cell; fU1/fU2 the conserved grids, fvel the velocity field of the
  // ghost cells; store_w 0 skips the store of the primitives (D1/D2)
  int fsel;
  const uint8_t* fnear;
  double* fU1; double* fU2;
  double* fvel;
  int store_w;
  // (0.5 min(dx, dy)) / dx and / dy, formed once on the host
  double cdx, cdy;
};

__device__ __forceinline__ V4 ex_rd(const ExtrapArgs& a, int f, int64_t c) {
  if (a.overlay && a.mask[c] && ((a.phi[c] <= 0.0) == (f == 0))) {
    const double* o = a.ov_out + (int64_t)a.ov_map[c] * IFC_OUT;
    return V4{o[0], o[1], o[2], o[3]};
  }
  if (a.F1 && a.cls[c] < a.near_min) return load4(f == 0 ? a.F1 : a.F2, a.P, c);
  return load4(f == 0 ? a.S1 : a.S2, a.P, c);
}

template <bool FUSE>
__device__ __forceinline__ uint32_t extrap_cell(const ExtrapArgs& a, int64_t k) {
  const GridP& P = a.P;
  int i = (int)(k / P.nc), j = (int)(k % P.nc);
  BCSrc s = bc_source(P, i, j);
  int64_t c = cidx(P, s.i, s.j);
  if (a.band && !a.band[c]) return 0u;
  V4 v1 = ex_rd(a, 0, c), v2 = ex_rd(a, 1, c);
  bool skip = a.mgfm && a.mask[c];
  if (!skip) {
    double nx, ny;
    unit_normal(a.nrm, P, c, nx, ny);
    double cx = a.cdx * nx, cy = a.cdy * ny;
    if (c_le0(a.phi[c])) {
      // fluid 2 is ghost: information flows along -normal
      V4 dxv = c_gt0(nx) ? v4d(ex_rd(a, 1, c + 1), v2) : v4d(v2, ex_rd(a, 1, c - 1));
      V4 dyv = c_gt0(ny) ? v4d(ex_rd(a, 1, c + P.pitch), v2) : v4d(v2, ex_rd(a, 1, c - P.pitch));
      v2 = V4{(v2.a + cx * dxv.a) + cy * dyv.a, (v2.b + cx * dxv.b) + cy * dyv.b,
              (v2.c + cx * dxv.c) + cy * dyv.c, (v2.d + cx * dxv.d) + cy * dyv.d};
    } else {
      V4 dxv = c_gt0(nx) ? v4d(v1, ex_rd(a, 0, c - 1)) : v4d(ex_rd(a, 0, c + 1), v1);
      V4 dyv = c_gt0(ny) ? v4d(v1, ex_rd(a, 0, c - P.pitch)) : v4d(ex_rd(a, 0, c + P.pitch), v1);
      v1 = V4{(v1.a - cx * dxv.a) - cy * dyv.a, (v1.b - cx * dxv.b) - cy * dyv.b,
              (v1.c - cx * dxv.c) - cy * dyv.c, (v1.d - cx * dxv.d) - cy * dyv.d};
    }
  }
  if (s.flipu) { v1.b = -v1.b; v2.b = -v2.b; }
  if (s.flipv) { v1.c = -v1.c; v2.c = -v2.c; }
  int64_t o = cidx(P, i, j);
  if (!FUSE || a.store_w) {
    store4(a.D1, P, o, v1);
    store4(a.D2, P, o, v2);
  }
  uint32_t st = 0u;
  if (FUSE && (a.fsel == 2 || (a.fsel == 1 && !a.fnear[c]))) {
    // k_finalize's conversion of these cells (Riemann / real GFM), with the
    // velocity field of the ghost cells
    bool ok1 = true, ok2 = true;
    const V4 u1 = prims_to_cons(P.g1, P.p1, v1, &ok1);
    const V4 u2 = prims_to_cons(P.g2, P.p2, v2, &ok2);
    if (!ok1 || !ok2 || !is_physical_state_fast(u1) || !is_physical_state_fast(u2)) st |= ST_UNPHYSICAL;
    store4(a.fU1, P, o, u1);
    store4(a.fU2, P, o, u2);
    if (!is_real(P, i, j)) {   // the real cells' velocities come from k_prims and k_ifc_vel
      const V4& V = c_le0(a.phi[o]) ? v1 : v2;
      a.fvel[o] = V.b;
      a.fvel[o + P.plane] = V.c;
    }
  }
  return st;
}

// FUSE: the sweep may carry the fused conversion (a separate instance, so
// that the plain sweeps keep their lower register count)
template <bool FUSE>
__global__ void __launch_bounds__(256) k_extrap(ExtrapArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  uint32_t st = 0u;
  if (a.list) {
    int cnt[BAND_CLASSES];
    int n = 0;
    for (int q = 0; q < a.nclass; q++) { cnt[q] = a.list_n[q]; n += cnt[q]; }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
      int q = 0, r = e;
      while (r >= cnt[q]) { r -= cnt[q]; q++; }
      st |= extrap_cell<FUSE>(a, a.list[(int64_t)q * a.list_stride + r]);
    }
  } else {
    const int64_t n = (int64_t)P.nr * P.nc;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
      st |= extrap_cell<FUSE>(a, k);
  }
  if (FUSE && a.fsel) {
    const uint32_t wst = __reduce_or_sync(0xffffffffu, st);
    if ((threadIdx.x & 31) == 0 && wst) atomicOr(&a.Dw->status, wst);
  }
}

// The cells (over the padded rows, ghost cells included) whose
// boundary-condition source lies within NEAR_RADIUS (Chebyshev) of an
// interfacial cell, appended to the segment of their source's distance d
// (counts in nseg[0..NEAR_RADIUS], zeroed by the caller).  cls[c] =
// NEAR_RADIUS + 1 - d of a real cell c (k_band_mark), 0 beyond; the ghost
// cells' entries are set here to their source's.  Also the near-cell mask of
// the real cells.  Order within a segment is free: a sweep writes each listed
// cell from reads of the previous buffers only.
__global__ void k_band_lists(GridP P, int* cls, uint8_t* near_cell, int* band_list, int64_t stride, int* nseg,
                             const DevTime* D) {
  if (!D->active) return;
  const int64_t n = (int64_t)P.nr * P.nc;
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = base + lane;
    int q = -1;
    if (k < n) {
      const int i = (int)(k / P.nc), j = (int)(k % P.nc);
      BCSrc s = bc_source(P, i, j);
      const int v = cls[cidx(P, s.i, s.j)];   // a real cell: k_band_mark's value
      if (v > 0) q = NEAR_RADIUS + 1 - v;
      if (is_real(P, i, j)) near_cell[cidx(P, i, j)] = (v > 0) ? 1 : 0;
      else cls[cidx(P, i, j)] = v;
    }
    const unsigned below = (1u << lane) - 1u;
    for (int c = 0; c < BAND_CLASSES; c++) {
      const unsigned m = __ballot_sync(0xffffffffu, q == c);
      if (!m) continue;
      int o = 0;
      if (lane == 0) o = atomicAdd(&nseg[c], __popc(m));
      o = __shfl_sync(0xffffffffu, o, 0);
      if (q == c) band_list[(int64_t)c * stride + o + __popc(m & below)] = (int)k;
    }
  }
}

// ---------------------------------------------------------------------------
// Interface solve: the loop over interfacial cells of GFM_riemann
// (sourcecode/GFM_riemann.cpp:51-148), GFM_real (sourcecode/GFM_real.cpp:52-208)
// and GFM_modified (sourcecode/GFM_modified.cpp:65-200).
//
// The reference visits interfacial cells in row-major order and, for the
// Riemann and real GFM, overwrites prims of the visited cell's real fluid
// while later cells still read prims (bilinear samples, or the opposite
// cell).  A later cell therefore reads the star state of an earlier
// interfacial cell when that cell lies in its read set and has the read
// fluid as its real fluid, and the original value otherwise.  Each cell here
// resolves its reads by exactly that rule and waits only for those earlier
// cells (its predecessors), so the result is the sequential one while
// independent cells run in parallel.
//
// Cells are claimed in list (row-major) order through a ticket counter, so
// every predecessor was claimed before its dependant by a running thread: the
// lowest unfinished cell can always proceed.  Waits are bounded (IfcArgs::
// spin_limit polls, IFC_SPIN_LIMIT by default: about a second); a wait that
// runs out sets ST_SCHEDULE_LIMIT and the thread abandons its cell, which its
// own dependants see at once.
// ---------------------------------------------------------------------------
enum { IFC_RIEMANN = 0, IFC_REAL = 1, IFC_MODIFIED = 2 };
constexpr long long IFC_SPIN_LIMIT = 1ll << 24;

struct IfcArgs {
  GridP P;
  const double* W1; const double* W2;
  const double* phi; const double* nrm; const uint8_t* mask;
  const int* list; const int* ifc_map;
  int* done;            // per cell of the list: 0 pending, 1 finished, 2 abandoned
  double* out;          // IFC_OUT doubles per cell
  unsigned int* ticket;
  DevTime* D;
  int slip;             // GFM_base::use_slip_BCs
  const float* mlp;     // learned-proposal network (gfm_mlp.cuh), or null
  const uint32_t* mlp_frag;   // its B fragments for the warp-level tensor-core path
  float* cap_X;         // gated problems appended here (features, target), or null
  float* cap_Y;
  int* cap_count;
  int cap;
  // probe geometry of the Riemann GFM's cells from k_ifc_probes (or null):
  // per list entry and side, the bilinear cell (i0, j0) and the 4 weights
  const int* probe_ij;
  const double* probe_w;
  // and per list entry, side and bilinear corner the list entry whose
  // published value that corner reads, or -1 (the corner reads the grid)
  const int* probe_dep;
  long long spin_limit;   // polls of a completion flag before a wait gives up
  int withhold;           // test hook: this list entry is never solved or published (-1: none)
};

// Completion flags of the interface loop: the writer publishes a cell's
// outputs with a release store of its flag, readers poll it with acquire
// loads (tightly at first, then with a short sleep), so a dependant sees the
// outputs as soon as the flag does, without a full fence on either side.
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ bool ifc_wait(const IfcArgs& a, int p) {
  long long spins = 0;
  int v;
  while ((v = ld_acquire(a.done + p)) == 0) {
    if (++spins > a.spin_limit) return false;
    if (spins > 512) __nanosleep(64);
  }
  return v == 1;
}

// Published values of k_interface_warp's cells.  Each of a cell's four
// values that dependants read (out[0..3]: its real fluid's star density,
// velocity and pressure) starts the step as IFC_PENDING (k_ifc_reset) and is
// written once, by one 64-bit store, so a dependant polls the value it needs
// itself: any other bit pattern is the final value (aligned 64-bit accesses
// are single-copy atomic).  A cell that gave up publishes IFC_FAILED.  Both
// are signalling NaNs, which no FP64 operation returns; a published value
// with either pattern (only a NaN copied from the input grids could have
// one) is published as the quiet NaN instead.
constexpr unsigned long long IFC_PENDING = 0x7ff00000c0ffee00ull;
constexpr unsigned long long IFC_FAILED = 0x7ff00000badbad00ull;

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const double* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(double* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void ifc_publish(double* p, double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  if (b == IFC_PENDING || b == IFC_FAILED) b = 0x7fffffffffffffffull;
  st_relaxed_u64(p, b);
}
// value kc of list entry p once it is published; false when the entry gave
// up or the polls ran out
__device__ __forceinline__ bool ifc_poll(const IfcArgs& a, int p, int kc, double& v) {
  const double* w = a.out + (int64_t)p * IFC_OUT + kc;
  long long spins = 0;
  unsigned long long x;
  while ((x = ld_relaxed_u64(w)) == IFC_PENDING) {
    if (++spins > a.spin_limit) return false;
    if (spins > 512) __nanosleep(64);
  }
  if (x == IFC_FAILED) return false;
  v = __longlong_as_double((long long)x);
  return true;
}

__device__ __forceinline__ V4 ifc_out4(const IfcArgs& a, int p) {
  const double* o = a.out + (int64_t)p * IFC_OUT;
  return V4{__ldcg(o), __ldcg(o + 1), __ldcg(o + 2), __ldcg(o + 3)};
}

// Value of fluid f's primitives at cell (i,j) as the sequential loop of cell
// `lin` sees it; waits for the writer if it is an earlier interfacial cell.
__device__ V4 ifc_read(const IfcArgs& a, int f, int i, int j, int64_t lin, bool& ok) {
  const GridP& P = a.P;
  int64_t c = cidx(P, i, j);
  int64_t l2 = (int64_t)i * P.nc + j;
  if (a.mask[c] && ((a.phi[c] <= 0.0) == (f == 0)) && l2 < lin) {
    int p = a.ifc_map[c];
    if (!ifc_wait(a, p)) { ok = false; return V4{0.0, 0.0, 0.0, 0.0}; }
    return ifc_out4(a, p);
  }
  return load4(f == 0 ? a.W1 : a.W2, P, c);
}

// grid_bilinear_interpolate at x (the project's definition, shared with the oracle)
__device__ V4 ifc_bilinear(const IfcArgs& a, int f, double x, double y, int64_t lin, bool resolve, bool& ok) {
  const GridP& P = a.P;
  double s = (x - P.x0) * P.idx + (double)P.g - 0.5;
  double t = (y - P.y0) * P.idy + (double)P.g - 0.5;
  int j0 = (int)floor(s), i0 = (int)floor(t);
  j0 = min(max(j0, 0), P.nc - 2);
  i0 = min(max(i0, 0), P.nr - 2);
  double wa = s - (double)j0, wb = t - (double)i0;
  V4 g00, g01, g10, g11;
  if (resolve) {
    g00 = ifc_read(a, f, i0, j0, lin, ok);
    g01 = ifc_read(a, f, i0, j0 + 1, lin, ok);
    g10 = ifc_read(a, f, i0 + 1, j0, lin, ok);
    g11 = ifc_read(a, f, i0 + 1, j0 + 1, lin, ok);
  } else {
    const double* G = f == 0 ? a.W1 : a.W2;
    g00 = load4(G, P, cidx(P, i0, j0));
    g01 = load4(G, P, cidx(P, i0, j0 + 1));
    g10 = load4(G, P, cidx(P, i0 + 1, j0));
    g11 = load4(G, P, cidx(P, i0 + 1, j0 + 1));
  }
  double w00 = (1.0 - wa) * (1.0 - wb), w01 = wa * (1.0 - wb), w10 = (1.0 - wa) * wb, w11 = wa * wb;
  return V4{w00 * g00.a + w01 * g01.a + w10 * g10.a + w11 * g11.a,
            w00 * g00.b + w01 * g01.b + w10 * g10.b + w11 * g11.b,
            w00 * g00.c + w01 * g01.c + w10 * g10.c + w11 * g11.c,
            w00 * g00.d + w01 * g01.d + w10 * g10.d + w11 * g11.d};
}

// The interface loops are latency-bound chains of dependent cells: they form
// their quotients and roots with the FP64 operations (CHAIN_ID false), whose
// dependent latency is about that of the integer forms while their code is
// shorter.
#ifndef GFM_CHAIN_INT_DIV
constexpr bool CHAIN_ID = false;
#else
constexpr bool CHAIN_ID = true;
#endif

template <int MODE>
__global__ void __launch_bounds__(128) k_interface(IfcArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  const int n = a.D->n_ifc;
  uint32_t st = 0;
  int iters = 0;
  // One interfacial cell per warp, solved by lane 0: on GB300 an FP64
  // instruction occupies its sub-partition's FP64 pipe for the same time
  // whether 1 or 32 lanes are active, so lanes of one warp working on
  // dependent cells would only serialise each other.
  const int lane = threadIdx.x & 31;
  for (;;) {
    int k = 0;
    if (lane == 0) k = (int)atomicAdd(a.ticket, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= n) break;
    if (lane != 0 || k == a.withhold) continue;
    int64_t lin = a.list[k];
    int i = (int)(lin / P.nc), j = (int)(lin % P.nc);
    int64_t c = cidx(P, i, j);
    double lsval = a.phi[c];
    double nx, ny;
    unit_normal(a.nrm, P, c, nx, ny);
    bool ok = true;
    V4 ip1, ip2;   // interfaceprims1, interfaceprims2
    if (MODE == IFC_REAL) {
      // neighbour with opposite phi sign and the closest normal (GFM_real.cpp:77-117)
      // acos is decreasing with slope <= -1 and gfm_acos is accurate to a few
      // ulps, so a candidate whose clamped dot product is more than 1e-6 below
      // the largest one has a strictly larger angle than the minimum and can
      // never be the first minimiser: acos is evaluated only for the others,
      // in the reference's loop order with its strict comparison.
      double dpk[9];
      double dbest = -2.0;
      for (int xinc = -1; xinc <= 1; xinc++)
        for (int yinc = -1; yinc <= 1; yinc++) {
          int q = (xinc + 1) * 3 + (yinc + 1);
          int64_t c2 = cidx(P, i + yinc, j + xinc);
          dpk[q] = -3.0;
          if (lsval * a.phi[c2] <= 0.0) {
            double ox, oy;
            unit_normal(a.nrm, P, c2, ox, oy);
            double dp = nx * ox + ny * oy;
            dp = (dp < -1.0) ? -1.0 : dp;
            dp = (1.0 < dp) ? 1.0 : dp;
            dpk[q] = dp;
            if (dp > dbest) dbest = dp;
          }
        }
      double mindiff = 1e100;
      int iopp = -1000, jopp = -1000;
      for (int xinc = -1; xinc <= 1; xinc++)
        for (int yinc = -1; yinc <= 1; yinc++) {
          double dp = dpk[(xinc + 1) * 3 + (yinc + 1)];
          if (dp < -2.0 || dp < dbest - 1e-6) continue;
          double ang = gfm_acos<CHAIN_ID>(dp);
          if (ang < mindiff) { iopp = i + yinc; jopp = j + xinc; mindiff = ang; }
        }
      if (iopp == -1000) { st |= ST_BAD_ARGUMENT; iopp = i; jopp = j; }
      if (lsval <= 0.0) {
        ip1 = load4(a.W1, P, c);
        ip2 = ifc_read(a, 1, iopp, jopp, lin, ok);
      } else {
        ip2 = load4(a.W2, P, c);
        ip1 = ifc_read(a, 0, iopp, jopp, lin, ok);
      }
    } else {
      // get_interpolated_mixedRPstates (sourcecode/GFM_base.cpp:4-33)
      double ds = 1.0 * (P.dy < P.dx ? P.dy : P.dx);
      double ccx = P.x0 + ((double)(j - P.g) + 0.5) * P.dx;
      double ccy = P.y0 + ((double)(i - P.g) + 0.5) * P.dy;
      double gx = a.nrm[c], gy = a.nrm[c + P.plane];
      double nm = a.nrm[c + 4 * P.plane];
      double lv = lsval;
      if (fabs(lv) > ds) lv = copysign(ds, lv);
      // normal / normmag: the unit normal unless the gradient vanishes
      double hx = nx, hy = ny;
      if (nm < 1e-12) { hx = gx / nm; hy = gy / nm; }
      double ilx = ccx - lv * hx, ily = ccy - lv * hy;
      bool resolve = (MODE == IFC_RIEMANN);
      ip2 = ifc_bilinear(a, 1, ilx + ds * hx, ily + ds * hy, lin, resolve, ok);
      ip1 = ifc_bilinear(a, 0, ilx - ds * hx, ily - ds * hy, lin, resolve, ok);
    }
    double* o = a.out + (int64_t)k * IFC_OUT;
    if (!ok) {
      st |= ST_SCHEDULE_LIMIT;
      st_release(a.done + k, 2);
      continue;
    }
    // mixed Riemann problem in the normal frame (e.g. GFM_riemann.cpp:76-122)
    double u1n = ip1.b * nx + ip1.c * ny;
    double u2n = ip2.b * nx + ip2.c * ny;
    double t1x = ip1.b - u1n * nx, t1y = ip1.c - u1n * ny;
    double t2x = ip2.b - u2n * nx, t2y = ip2.c - u2n * ny;
    V4 Lp = V4{ip1.a, u1n, 0.0, (1e-6 < ip1.d) ? ip1.d : 1e-6};
    V4 Rp = V4{ip2.a, u2n, 0.0, (1e-6 < ip2.d) ? ip2.d : 1e-6};
    bool ok1 = true, ok2 = true;
    V4 Ls = prims_to_cons<CHAIN_ID>(P.g1, P.p1, Lp, &ok1);
    V4 Rs = prims_to_cons<CHAIN_ID>(P.g2, P.p2, Rp, &ok2);
    if (!ok1 || !ok2) st |= ST_UNPHYSICAL;
    MixedStar m = mixed_rs<CHAIN_ID>(P.gas1, P.gas2, Ls, Rs, &st, &iters);
    double snx = m.u_star * nx, sny = m.u_star * ny;
    if (MODE == IFC_MODIFIED) {
      double u1x, u1y, u2x, u2y;
      if (a.slip) { u1x = snx + t1x; u1y = sny + t1y; u2x = snx + t2x; u2y = sny + t2y; }
      else if (lsval <= 0.0) { u1x = snx + t1x; u1y = sny + t1y; u2x = snx + t1x; u2y = sny + t1y; }
      else { u1x = snx + t2x; u1y = sny + t2y; u2x = snx + t2x; u2y = sny + t2y; }
      if (lsval <= 0.0) {
        o[0] = eos_isentropic_extrapolation<CHAIN_ID>(P.g1, P.p1, m.rho_star_L, m.p_star, load4(a.W1, P, c).d);
        o[1] = m.rho_star_R; o[2] = u2x; o[3] = u2y; o[4] = m.p_star;
      } else {
        o[0] = eos_isentropic_extrapolation<CHAIN_ID>(P.g2, P.p2, m.rho_star_R, m.p_star, load4(a.W2, P, c).d);
        o[1] = m.rho_star_L; o[2] = u1x; o[3] = u1y; o[4] = m.p_star;
      }
      o[5] = snx; o[6] = sny;
    } else {
      if (lsval <= 0.0) { o[0] = m.rho_star_L; o[1] = snx + t1x; o[2] = sny + t1y; o[3] = m.p_star; }
      else { o[0] = m.rho_star_R; o[1] = snx + t2x; o[2] = sny + t2y; o[3] = m.p_star; }
      o[4] = snx; o[5] = sny;
    }
    st_release(a.done + k, 1);
  }
  uint32_t wst = __reduce_or_sync(0xffffffffu, st);
  unsigned wit = __reduce_add_sync(0xffffffffu, (unsigned)iters);
  if ((threadIdx.x & 31) == 0) {
    if (wst) atomicOr(&a.D->status, wst);
    if (wit) atomicAdd(&a.D->newton_iters, (unsigned long long)wit);
  }
}

// ---------------------------------------------------------------------------
// Warp-wide interface solve of the Riemann and real GFM.
//
// An FP64 warp instruction holds its sub-partition's FP64 pipe for the same
// time whether 1 or 32 lanes are active, and the interface loop is a chain of
// dependent cells, so the loop's speed is set by the number of FP64
// instructions one cell issues.  Here all 32 lanes of a warp share one cell:
//   lane = 16 s + 4 q + kc : probe side s (0: fluid 1, 1: fluid 2), bilinear
//   corner q (bit 0: next column, bit 1: next row), state component kc.
// Each lane reads one corner value, the four products of a bilinear sum are
// formed at once and added in the scalar order, and the Riemann problem is
// solved with side L on lanes 0-15 and side R on lanes 16-31
// (mixed_rs_pair).  Every value comes from the same operations as in
// k_interface, so the results are identical.
// ---------------------------------------------------------------------------
constexpr unsigned FULL_MASK = 0xffffffffu;

__device__ __forceinline__ double xside(double x) { return __shfl_xor_sync(FULL_MASK, x, 16); }

// component kc of ifc_read for k_interface_warp, whose cells publish their
// values for polling (ifc_poll)
__device__ __forceinline__ double ifc_read1(const IfcArgs& a, int f, int i, int j, int kc, int64_t lin, bool& ok) {
  const GridP& P = a.P;
  int64_t c = cidx(P, i, j);
  int64_t l2 = (int64_t)i * P.nc + j;
  if (a.mask[c] && ((a.phi[c] <= 0.0) == (f == 0)) && l2 < lin) {
    double v = 0.0;
    if (!ifc_poll(a, a.ifc_map[c], kc, v)) ok = false;
    return v;
  }
  return (f == 0 ? a.W1 : a.W2)[c + kc * P.plane];
}

struct PairStar { double p, u, rho_own; bool trivial; };

// mixed_rs (gfm_math.cuh) for the conserved state Uown of this lane's side
// (isR: side R, gas k).  Each lane evaluates only its own side's conversion,
// wave constants, pressure function and star density; quantities of both
// sides are exchanged and combined with the scalar solver's operations, so
// p* and u* are the scalar ones on every lane and rho_own is the star
// density of the lane's side.  The Newton loop is warp-uniform: both halves
// compute the same pressure iterates.
//
// star_side >= 0: rho_own is that side's star density on every lane (the
// caller publishes only it), evaluated once for the warp, so the two halves
// do not take the shock's and the rarefaction's branch one after the other.
//
// With a network (a.mlp), problems whose two-shock guess moved far from PVRS
// (the gate of gfm_mlp.cuh) start from the network's proposal, evaluated by
// the warp in FP32 on the actual states; with a capture buffer, such problems
// are recorded (features and the solved p* relative to the two-shock guess).
__device__ __forceinline__ PairStar mixed_rs_pair(bool isR, const Gas& k, const Gas& kL, const Gas& kR, const V4& Uown,
                                                  uint32_t* status, int* iters, const IfcArgs& a,
                                                  int* proposed, int star_side = -1) {
  // cons_to_prims_phys with its three quotients by rho (rho u, rho v, E) in
  // one: lane kc of each group of four divides component kc + 1 (E twice)
  const int lane = threadIdx.x & 31, grp = lane & ~3, kq = lane & 3;
  const Recip Rr = recip<CHAIN_ID>(Uown.a);
  const double qv = rdiv(kq == 0 ? Uown.b : (kq == 1 ? Uown.c : Uown.d), Rr);
  const double uq = __shfl_sync(FULL_MASK, qv, grp), vq = __shfl_sync(FULL_MASK, qv, grp + 1);
  const double eq = __shfl_sync(FULL_MASK, qv, grp + 2) - 0.5 * (uq * uq + vq * vq);
  const bool ok = c_ge0(Uown.a) && c_ge0(eq);
  const V4 Wp = V4{Uown.a, uq, vq, eos_pressure(k.g, k.pinf, eq, Uown.a)};
  if (!ok) *status |= ST_UNPHYSICAL;
  RSSide S = rs_side(Wp.a, Wp.b, Wp.d, k);
  const double ou = xside(S.u), op = xside(S.p);
  const double uL = isR ? ou : S.u, uR = isR ? S.u : ou;
  const double pL = isR ? op : S.p, pR = isR ? S.p : op;
  PairStar r;
  if (c_eq(uL, uR) && c_eq(pL, pR)) {   // rs_solve's no-wave shortcut
    r.p = pL; r.u = uL; r.rho_own = S.rho; r.trivial = true;
    return r;
  }
  r.trivial = false;
  {
    // rs_side_consts with its two reciprocals (1/rho, 1/pb) in one division:
    // even lanes divide by rho, odd lanes by pb, and exchange
    const double y = divx<CHAIN_ID>(1.0, (lane & 1) ? S.pb : S.rho);
    const double irho = __shfl_sync(FULL_MASK, y, lane & ~1), ipb = __shfl_sync(FULL_MASK, y, lane | 1);
    S.ipb = ipb;
    S.c = sqrtx<CHAIN_ID>(k.g * S.pb * irho);
    S.AK = k.G5 * irho;
    S.BK = k.G6 * S.pb;
    S.G4c = k.G4 * S.c;
    S.irc = S.c * S.ipb * k.IG;
  }
  const double orho = xside(S.rho), oc = xside(S.c), oG4c = xside(S.G4c), opb = xside(S.pb);
  const double rhoL = isR ? orho : S.rho, rhoR = isR ? S.rho : orho;
  const double cL = isR ? oc : S.c, cR = isR ? S.c : oc;
  const double G4cL = isR ? oG4c : S.G4c, G4cR = isR ? S.G4c : oG4c;
  const double pbL = isR ? opb : S.pb, pbR = isR ? S.pb : opb;
  // rs_guess_pvrs, then rs_guess_tsrs at max(PVRS, floor): each lane forms
  // its own side's shock constant
  const double ppv = 0.5 * (pL + pR) - 0.125 * (uR - uL) * (rhoL + rhoR) * (cL + cR);
  const double pinf_min = c_lt(kL.pinf, kR.pinf) ? kL.pinf : kR.pinf;
  const double pbmin = c_lt(pbL, pbR) ? pbL : pbR;
  const double pfl = 1e-6 * pbmin - pinf_min;
  const double pg = c_gt(ppv, pfl) ? ppv : pfl;
  const double gown = sqrtx<CHAIN_ID>(divx<CHAIN_ID>(S.AK, pg + k.pinf + S.BK));
  const double goth = xside(gown);
  const double gL = isR ? goth : gown, gR = isR ? gown : goth;
  const double pts = divx<CHAIN_ID>(gL * pL + gR * pR - (uR - uL), gL + gR);
  double p0 = pts;
  bool gated = false;
  float x[MLP_IN];
  if (a.mlp || a.cap_X) {   // warp-uniform: both halves hold the same values
    const double ratio = divx<CHAIN_ID>(pts + pinf_min, pg + pinf_min);
    gated = mlp_gated(ratio);
    if (gated) mlp_features_f(rhoL, uL, pbL, kL.g, kL.pinf, rhoR, uR, pbR, kR.g, kR.pinf, x);
    if (gated && a.mlp) {
      const float y = fminf(fmaxf(mlp_forward_warp_tc(a.mlp_frag, a.mlp, x), -20.0f), 20.0f);
      p0 = (pts + pinf_min) * gfm_exp((double)y) - pinf_min;
      *proposed += 1;
    }
  }
  // rs_star
  const double udiff = uR - uL;
  if (c_le(G4cL + G4cR, udiff)) *status |= ST_VACUUM;
  double pold = c_gt(p0, pfl) ? p0 : pfl;
  double fL = 0.0, fR = 0.0, fLd = 0.0, fRd = 0.0, p = pold, dp = 0.0;
  int it = 0;
  for (;;) {
    double f, fd;
    rs_prefun_merged(S, k, pold, &f, &fd);   // the halves often take different branches
    const double of = xside(f), ofd = xside(fd);
    fL = isR ? of : f;
    fR = isR ? f : of;
    fLd = isR ? ofd : fd;
    fRd = isR ? fd : ofd;
    p = pold - divx<CHAIN_ID>(fL + fR + udiff, fLd + fRd);
    if (c_lt(p, pfl)) p = pfl;
    it++;
    bool conv = c_le(2.0 * fabs(p - pold), GFM_RS_TOL * (p + pold + 2.0 * pinf_min));
    dp = p - pold;
    pold = p;
    if (conv) break;
    if (it >= kL.maxit) { *status |= ST_NEWTON_NO_CONVERGE; break; }
  }
  r.p = p;
  r.u = 0.5 * (uL + uR + (fR + fRd * dp) - (fL + fLd * dp));
  if (star_side < 0) {
    r.rho_own = rs_rho_star<CHAIN_ID>(S, k, p);
  } else {
    // rs_rho_star reads the side's rho, p and 1/pb
    RSSide K = S;
    K.rho = __shfl_sync(FULL_MASK, S.rho, 16 * star_side);
    K.p = __shfl_sync(FULL_MASK, S.p, 16 * star_side);
    K.ipb = __shfl_sync(FULL_MASK, S.ipb, 16 * star_side);
    r.rho_own = rs_rho_star<CHAIN_ID>(K, star_side ? kR : kL, p);
  }
  *iters += it;
  if (gated && a.cap_X && (threadIdx.x & 31) == 0 && it < kL.maxit && !c_le(G4cL + G4cR, udiff)) {
    const double y = gfm_log((p + pinf_min) / (pts + pinf_min));
    if (fabs(y) < 30.0) {
      const int slot = atomicAdd(a.cap_count, 1);
      if (slot < a.cap) {
        for (int q = 0; q < MLP_IN; q++) a.cap_X[(int64_t)slot * MLP_IN + q] = x[q];
        a.cap_Y[slot] = (float)y;
      }
    }
  }
  return r;
}

// One interfacial cell's Riemann data in the lane layout above: on return
// every lane holds its side's conserved normal-frame state Us (and the
// tangential velocity tx, ty).  Returns false, on every lane, when a wait
// ran out.
struct IfcCell {
  int64_t c;
  int sr;             // side of the cell's real fluid
  double nx, ny, tx, ty;
  V4 Us;
};

// The bilinear probe of side R (isR: interface point + ds n, sampling fluid
// 2) or L (- ds n, fluid 1) of interfacial cell c = (i,j): the lower-left
// cell (i0, j0) and the fractional offsets (wa, wb)
// (get_interpolated_mixedRPstates, sourcecode/GFM_base.cpp:4-33, and the
// project's bilinear interpolation).
__device__ __forceinline__ void ifc_probe(const IfcArgs& a, int64_t c, int i, int j, double lsval, double nx,
                                          double ny, bool isR, int& i0, int& j0, double& wa, double& wb) {
  const GridP& P = a.P;
  const double ds = 1.0 * (P.dy < P.dx ? P.dy : P.dx);
  const double ccx = P.x0 + ((double)(j - P.g) + 0.5) * P.dx;
  const double ccy = P.y0 + ((double)(i - P.g) + 0.5) * P.dy;
  const double gx = a.nrm[c], gy = a.nrm[c + P.plane];
  const double nm = a.nrm[c + 4 * P.plane];
  double lv = lsval;
  if (fabs(lv) > ds) lv = copysign(ds, lv);
  double hx = nx, hy = ny;
  if (nm < 1e-12) { hx = gx / nm; hy = gy / nm; }
  const double ilx = ccx - lv * hx, ily = ccy - lv * hy;
  const double dsx = ds * hx, dsy = ds * hy;
  const double px = ilx + (isR ? dsx : -dsx);
  const double py = ily + (isR ? dsy : -dsy);
  const double sx = (px - P.x0) * P.idx + (double)P.g - 0.5;
  const double sy = (py - P.y0) * P.idy + (double)P.g - 0.5;
  j0 = (int)floor(sx);
  i0 = (int)floor(sy);
  j0 = min(max(j0, 0), P.nc - 2);
  i0 = min(max(i0, 0), P.nr - 2);
  wa = sx - (double)j0;
  wb = sy - (double)i0;
}

// The probes of every interfacial cell ahead of the interface loop: they
// depend on phi and its normals only, so computing them here in parallel
// takes their FP64 instructions off the loop's dependency chain.  So does
// the test of each bilinear corner (ifc_read1's: an earlier interfacial cell
// whose real fluid is the probed one), which depends on the mask, phi and
// the list only: probe_dep holds the list entry the corner waits for, or -1.
__global__ void __launch_bounds__(256) k_ifc_probes(IfcArgs a, int* probe_ij, double* probe_w, int* probe_dep) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  const int n = a.D->n_ifc;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 2 * n; q += gridDim.x * blockDim.x) {
    const int t = q >> 1, s = q & 1;
    const int64_t lin = a.list[t];
    const int i = (int)(lin / P.nc), j = (int)(lin % P.nc);
    const int64_t c = cidx(P, i, j);
    double nx, ny;
    unit_normal(a.nrm, P, c, nx, ny);
    int i0, j0;
    double wa, wb;
    ifc_probe(a, c, i, j, a.phi[c], nx, ny, s == 1, i0, j0, wa, wb);
    probe_ij[4 * (int64_t)t + 2 * s] = i0;
    probe_ij[4 * (int64_t)t + 2 * s + 1] = j0;
    double* w = probe_w + 8 * (int64_t)t + 4 * s;
    int* dep = probe_dep + 8 * (int64_t)t + 4 * s;
    for (int e = 0; e < 4; e++) {
      const double fa = (e & 1) ? wa : 1.0 - wa;
      const double fb = (e & 2) ? wb : 1.0 - wb;
      w[e] = fa * fb;
      const int ci = i0 + (e >> 1), cj = j0 + (e & 1);
      const int64_t cc = cidx(P, ci, cj);
      const int64_t l2 = (int64_t)ci * P.nc + cj;
      dep[e] = (a.mask[cc] && ((a.phi[cc] <= 0.0) == (s == 0)) && l2 < lin) ? a.ifc_map[cc] : -1;
    }
  }
}

template <int MODE>
__device__ __forceinline__ bool ifc_front(const IfcArgs& a, int t, const Gas& k, uint32_t& st, IfcCell& cell) {
  const GridP& P = a.P;
  const int lane = threadIdx.x & 31;
  const int s = lane >> 4, q = (lane >> 2) & 3, kc = lane & 3;
  const bool isR = s == 1;
  const int64_t lin = a.list[t];
  const int i = (int)(lin / P.nc), j = (int)(lin % P.nc);
  const int64_t c = cidx(P, i, j);
  const double lsval = a.phi[c];
  const int sr = (lsval <= 0.0) ? 0 : 1;
  double nx, ny;
  unit_normal(a.nrm, P, c, nx, ny);
  bool ok = true;
  double v = 0.0;   // lanes with q == 0: component kc of side s's state
  if (MODE == IFC_REAL) {
    // neighbour with opposite phi sign and the closest normal
    // (GFM_real.cpp:77-117); lane l < 9 is loop position l (xinc-major).
    // Candidates more than 1e-6 below the largest clamped dot product are
    // skipped as in k_interface; acos runs on the others at once and the
    // first minimiser in loop order wins, as with the reference's strict <.
    double dp = -3.0;
    if (lane < 9) {
      const int xinc = lane / 3 - 1, yinc = lane % 3 - 1;
      const int64_t c2 = cidx(P, i + yinc, j + xinc);
      if (lsval * a.phi[c2] <= 0.0) {
        double ox, oy;
        unit_normal(a.nrm, P, c2, ox, oy);
        double d = nx * ox + ny * oy;
        d = (d < -1.0) ? -1.0 : d;
        d = (1.0 < d) ? 1.0 : d;
        dp = d;
      }
    }
    double dbest = dp;
    for (int o = 8; o >= 1; o >>= 1) {
      const double x = __shfl_xor_sync(FULL_MASK, dbest, o);
      dbest = (x > dbest) ? x : dbest;
    }
    const bool elig = lane < 9 && !(dp < -2.0 || dp < dbest - 1e-6);
    long long key = 0x7ff0000000000000LL;   // +inf: not a candidate
    if (elig) {
      const double ang = gfm_acos<CHAIN_ID>(dp);
      if (ang == ang) key = as_bits(ang);   // angles are >= +0: bits order as values
    }
    int bl = (key == 0x7ff0000000000000LL) ? 32 : lane;
    for (int o = 8; o >= 1; o >>= 1) {
      const long long xk = __shfl_xor_sync(FULL_MASK, key, o);
      const int xl = __shfl_xor_sync(FULL_MASK, bl, o);
      if (xk < key || (xk == key && xl < bl)) { key = xk; bl = xl; }
    }
    bl = __shfl_sync(FULL_MASK, bl, 0);
    int iopp = i, jopp = j;
    if (bl == 32) st |= ST_BAD_ARGUMENT;
    else { iopp = i + (bl % 3 - 1); jopp = j + (bl / 3 - 1); }
    if (q == 0) {
      if (s == sr) v = (s == 0 ? a.W1 : a.W2)[c + kc * P.plane];
      else v = ifc_read1(a, s, iopp, jopp, kc, lin, ok);
    }
  } else {
    // get_interpolated_mixedRPstates (sourcecode/GFM_base.cpp:4-33); the
    // probe geometry depends on phi only and comes from k_ifc_probes when set
    int i0, j0;
    double w, g;
    if (a.probe_ij) {
      i0 = __ldg(a.probe_ij + 4 * (int64_t)t + 2 * s);
      j0 = __ldg(a.probe_ij + 4 * (int64_t)t + 2 * s + 1);
      w = __ldg(a.probe_w + 8 * (int64_t)t + 4 * s + q);
      const int dep = __ldg(a.probe_dep + 8 * (int64_t)t + 4 * s + q);
      if (dep >= 0) {
        g = 0.0;
        if (!ifc_poll(a, dep, kc, g)) ok = false;
      } else {
        g = (s == 0 ? a.W1 : a.W2)[cidx(P, i0 + (q >> 1), j0 + (q & 1)) + kc * P.plane];
      }
    } else {
      double wa, wb;
      ifc_probe(a, c, i, j, lsval, nx, ny, isR, i0, j0, wa, wb);
      const double fa = (q & 1) ? wa : 1.0 - wa;
      const double fb = (q & 2) ? wb : 1.0 - wb;
      w = fa * fb;
      g = ifc_read1(a, s, i0 + (q >> 1), j0 + (q & 1), kc, lin, ok);
    }
    const double pr = w * g;
    const double p1 = __shfl_down_sync(FULL_MASK, pr, 4);
    const double p2 = __shfl_down_sync(FULL_MASK, pr, 8);
    const double p3 = __shfl_down_sync(FULL_MASK, pr, 12);
    v = ((pr + p1) + p2) + p3;
  }
  if (!__all_sync(FULL_MASK, ok)) return false;
  const int base = lane & 16;
  const double ia = __shfl_sync(FULL_MASK, v, base), ib = __shfl_sync(FULL_MASK, v, base + 1);
  const double ic = __shfl_sync(FULL_MASK, v, base + 2), id = __shfl_sync(FULL_MASK, v, base + 3);
  // mixed Riemann problem in the normal frame (e.g. GFM_riemann.cpp:76-122)
  const double un = ib * nx + ic * ny;
  cell.c = c;
  cell.sr = sr;
  cell.nx = nx;
  cell.ny = ny;
  cell.tx = ib - un * nx;
  cell.ty = ic - un * ny;
  bool okp = true;
  cell.Us = prims_to_cons<CHAIN_ID>(k.g, k.pinf, V4{ia, un, 0.0, c_lt(1e-6, id) ? id : 1e-6}, &okp);
  if (!okp) st |= ST_UNPHYSICAL;
  return true;
}

// CTAs of k_interface_warp resident per SM that the register allocation
// must allow: the overlapped schedule launches two CTAs of 8 warps per SM of
// its chain partition, and two resident per SM (128 registers, a few
// spilled) ran the shock-bubble's chain 13% faster than one (212 registers,
// no spills) on an 8-SM partition
#ifndef GFM_CHAIN_MIN_CTAS
#define GFM_CHAIN_MIN_CTAS 2
#endif
template <int MODE>
__global__ void __launch_bounds__(256, GFM_CHAIN_MIN_CTAS) k_interface_warp(IfcArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  const int n = a.D->n_ifc;
  const int lane = threadIdx.x & 31;
  const bool isR = (lane >> 4) == 1;
  const Gas k = isR ? P.gas2 : P.gas1;
  uint32_t st = 0;
  int iters = 0, gated = 0;
  for (;;) {
    int t = 0;
    if (lane == 0) t = (int)atomicAdd(a.ticket, 1u);
    t = __shfl_sync(FULL_MASK, t, 0);
    if (t >= n) break;
    if (t == a.withhold) continue;
    IfcCell cell;
    if (!ifc_front<MODE>(a, t, k, st, cell)) {
      st |= ST_SCHEDULE_LIMIT;
      if (lane < 4) st_relaxed_u64(a.out + (int64_t)t * IFC_OUT + lane, IFC_FAILED);
      continue;
    }
    int it = 0, gt = 0;
    const PairStar m = mixed_rs_pair(isR, k, P.gas1, P.gas2, cell.Us, &st, &it, a, &gt, cell.sr);
    if (lane == 0) { iters += it; gated += gt; }
    if (c_isnan(m.p)) st |= ST_NAN;
    if (lane == 16 * cell.sr) {
      double* o = a.out + (int64_t)t * IFC_OUT;
      const double snx = m.u * cell.nx, sny = m.u * cell.ny;
      o[4] = snx; o[5] = sny;   // read after the loop only
      ifc_publish(o + 3, m.p);
      ifc_publish(o, m.rho_own);
      ifc_publish(o + 1, snx + cell.tx);
      ifc_publish(o + 2, sny + cell.ty);
    }
  }
  uint32_t wst = __reduce_or_sync(FULL_MASK, st);
  unsigned wit = __reduce_add_sync(FULL_MASK, (unsigned)iters);
  unsigned wgt = __reduce_add_sync(FULL_MASK, (unsigned)gated);
  if (lane == 0) {
    if (wst) atomicOr(&a.D->status, wst);
    if (wit) {
      atomicAdd(&a.D->newton_iters, (unsigned long long)wit);
      atomicAdd(&a.D->ifc_iters, (unsigned long long)wit);
    }
    if (wgt) atomicAdd(&a.D->ifc_gated, (int)wgt);
  }
}

// ---------------------------------------------------------------------------
// VOF interface tracker and the VOF ghost-fluid methods.
//
// The interface field (the context's phi plane) holds z, the volume fraction
// of fluid 1.  The tracker is the project's own definition from published
// methods, restated in the oracle:
//   mixed cell   0 < z < 1
//   normal       Youngs (1982) / Parker & Youngs (1992): minus the 3x3
//                weighted central-difference gradient of z, unit length,
//                pointing from fluid 1 into fluid 2; (1, 0) where it vanishes
//   PLIC line    cutting the cell at area fraction z (Scardovelli & Zaleski
//                2000); the interface location is its segment's midpoint
//   advection    directional splitting (x then y on even steps, y then x on
//                odd), geometric donor-strip fluxes of the PLIC fluid-1
//                region, face velocity = mean of the two cells', divergence
//                term of Weymouth & Yue (2010) with c = [z > 0.5] at the start
//                of the step; values within 1e-8 of 0 or 1 become 0 or 1
//   sign         get_sdf = 0.5 - z (negative in fluid 1)
// GFM_VOF (sourcecode/GFM_VOF.cpp:8-325) and OGFM_VOF
// (sourcecode/OGFM_VOF.cpp:8-274) visit the mixed cells of the real cells
// plus a 3-cell ring, in row-major order, and overwrite both fluids' prims of
// the visited cell while later cells read prims by bilinear samples: the
// dependency rule of the Riemann GFM's loop (an earlier mixed cell in a
// sample's corner supplies its new prims) with the warp-per-cell schedule.
// ---------------------------------------------------------------------------
enum { VOF_GFM = 0, VOF_OGFM = 1 };
constexpr double VOF_ZEPS = 1e-8;
constexpr int VOF_RING = 3;   // ghostrad of the reference's loops

__device__ __forceinline__ double vlo(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double vhi(double a, double b) { return (b < a) ? a : b; }

// area fraction of {c1 t + c2 s <= b} in the unit square (c1, c2 >= 0)
__device__ double vof_area(double b, double c1, double c2) {
  const double m1 = vlo(c1, c2), m2 = vhi(c1, c2);
  if (b <= 0.0) return 0.0;
  const double s = m1 + m2;
  if (b >= s) return 1.0;
  if (m1 == 0.0) return divx(b, m2);
  const double d = (2.0 * m1) * m2;
  if (b < m1) return divx(b * b, d);
  if (b <= m2) return divx(b - 0.5 * m1, m2);
  const double r = s - b;
  return 1.0 - divx(r * r, d);
}

// the line constant with vof_area(b, m1, m2) = z (0 < z < 1, m1 <= m2, m2 > 0)
__device__ double vof_line_constant(double z, double m1, double m2) {
  if (m1 == 0.0) return z * m2;
  const double v1 = divx(m1, 2.0 * m2);
  const double d = (2.0 * m1) * m2;
  if (z < v1) return sqrtx(d * z);
  if (z <= 1.0 - v1) return z * m2 + 0.5 * m1;
  return (m1 + m2) - sqrtx(d * (1.0 - z));
}

// PLIC reconstruction of the mixed cell c: in the unit cell with the axes
// reflected where the normal component is negative, fluid 1 fills
// {a xi + b eta <= beta}, a = |nx| dx, b = |ny| dy.
struct VofPlic { double nx, ny, a, b, beta; };

__device__ VofPlic vof_reconstruct(const GridP& P, const double* z, int64_t c) {
  const int64_t w = P.pitch;
  const double gx = ((z[c - w + 1] + 2.0 * z[c + 1]) + z[c + w + 1]) - ((z[c - w - 1] + 2.0 * z[c - 1]) + z[c + w - 1]);
  const double gy = ((z[c + w - 1] + 2.0 * z[c + w]) + z[c + w + 1]) - ((z[c - w - 1] + 2.0 * z[c - w]) + z[c - w + 1]);
  const double mx = divx(-gx, P.dx), my = divx(-gy, P.dy);
  const double nn = sqrtx(mx * mx + my * my);
  VofPlic r;
  if (nn > 0.0) { r.nx = divx(mx, nn); r.ny = divx(my, nn); }
  else { r.nx = 1.0; r.ny = 0.0; }
  r.a = fabs(r.nx) * P.dx;
  r.b = fabs(r.ny) * P.dy;
  r.beta = vof_line_constant(z[c], vlo(r.a, r.b), vhi(r.a, r.b));
  return r;
}

// fluid-1 volume of cell c (fraction of the cell) inside the strip of width w
// along axis dir touching the cell's high face (high) or its low face
__device__ double vof_strip_fraction(const GridP& P, const double* z, int64_t c, int dir, bool high, double w) {
  const double zc = z[c];
  if (zc == 1.0) return w;
  if (zc == 0.0) return 0.0;
  const VofPlic r = vof_reconstruct(P, z, c);
  const double n = dir == 0 ? r.nx : r.ny;
  const double cd = dir == 0 ? r.a : r.b, co = dir == 0 ? r.b : r.a;
  const bool refl = n < 0.0;
  const double start = (high != refl) ? 1.0 - w : 0.0;
  return w * vof_area(r.beta - cd * start, cd * w, co);
}

__device__ __forceinline__ bool vof_in_ring(const GridP& P, int i, int j) {
  return i >= P.g - VOF_RING && i < P.Ny + P.g + VOF_RING && j >= P.g - VOF_RING && j < P.Nx + P.g + VOF_RING;
}

// Stage 1 of the VOF ghost fill: prims of both grids, the real fluid's
// assert (z >= 0.5: fluid 1), the OGFM_VOF realcells boxes, the mixed cells
// of the real cells plus the ring (mask, chunk counts) and, for each, its
// reconstruction: nrm planes 0,1 = interface location, 2,3 = unit normal.
struct VofPrimArgs {
  GridP P;
  const double* U1; const double* U2;
  double* W1; double* W2;
  const double* z;
  double* nrm;
  uint8_t* mask;
  int* ifc_map;
  int* chunk_count;
  int chunk;                  // cells per CTA
  DevTime* D;
  int ogfm;
};

__global__ void __launch_bounds__(CHUNK_T) k_vof_prims(VofPrimArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  __shared__ int s_cnt;
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  const int64_t n = (int64_t)P.nr * P.nc;
  const int64_t base = (int64_t)blockIdx.x * a.chunk;
  uint32_t st = 0;
  int cnt = 0;
  int bb[8] = {INT_MAX, INT_MIN, INT_MAX, INT_MIN, INT_MAX, INT_MIN, INT_MAX, INT_MIN};
  for (int q = threadIdx.x; q < a.chunk; q += CHUNK_T) {
    int64_t lin = base + q;
    if (lin >= n) break;
    int i, j;
    linear_to_ij(P, lin, i, j);
    const int64_t c = cidx(P, i, j);
    const double zc = a.z[c];
    bool ok1, ok2;
    const V4 w1 = cons_to_prims_phys(P.g1, P.p1, load4(a.U1, P, c), &ok1);
    const V4 w2 = cons_to_prims_phys(P.g2, P.p2, load4(a.U2, P, c), &ok2);
    store4(a.W1, P, c, w1);
    store4(a.W2, P, c, w2);
    if (zc >= 0.5) {
      if (!ok1) st |= ST_UNPHYSICAL;
      bb[0] = min(bb[0], i - 2); bb[1] = max(bb[1], i + 2); bb[2] = min(bb[2], j - 2); bb[3] = max(bb[3], j + 2);
    } else {
      if (!ok2) st |= ST_UNPHYSICAL;
      bb[4] = min(bb[4], i - 2); bb[5] = max(bb[5], i + 2); bb[6] = min(bb[6], j - 2); bb[7] = max(bb[7], j + 2);
    }
    uint8_t m = 0;
    if (vof_in_ring(P, i, j) && 0.0 < zc && zc < 1.0) {
      m = 1;
      const VofPlic r = vof_reconstruct(P, a.z, c);
      // midpoint of the PLIC segment
      const double m1 = vlo(r.a, r.b), m2 = vhi(r.a, r.b), be = r.beta;
      double u1, w1v, u2, w2v;
      if (be < m1) { u1 = divx(be, m1); w1v = 0.0; u2 = 0.0; w2v = divx(be, m2); }
      else if (be <= m2) { u1 = 0.0; w1v = divx(be, m2); u2 = 1.0; w2v = divx(be - m1, m2); }
      else { u1 = 1.0; w1v = divx(be - m1, m2); u2 = divx(be - m2, m1); w2v = 1.0; }
      const double um = 0.5 * (u1 + u2), wm = 0.5 * (w1v + w2v);
      const bool swapped = r.b < r.a;
      const double xr = swapped ? wm : um, er = swapped ? um : wm;
      const double xi = (r.nx < 0.0) ? 1.0 - xr : xr;
      const double eta = (r.ny < 0.0) ? 1.0 - er : er;
      const double ccx = P.x0 + ((double)(j - P.g) + 0.5) * P.dx;
      const double ccy = P.y0 + ((double)(i - P.g) + 0.5) * P.dy;
      a.nrm[c] = ccx + (xi - 0.5) * P.dx;
      a.nrm[c + P.plane] = ccy + (eta - 0.5) * P.dy;
      a.nrm[c + 2 * P.plane] = r.nx;
      a.nrm[c + 3 * P.plane] = r.ny;
    }
    a.mask[c] = m;
    a.ifc_map[c] = -1;
    cnt += m;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&s_cnt, cnt);
  uint32_t wst = __reduce_or_sync(0xffffffffu, st);
  if ((threadIdx.x & 31) == 0 && wst) atomicOr(&a.D->status, wst);
  if (a.ogfm) {
    for (int q = 0; q < 8; q++) {
      int v = bb[q];
      if (q & 1) { for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o)); }
      else { for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o)); }
      if ((threadIdx.x & 31) == 0) {
        if (q & 1) { if (v != INT_MIN) atomicMax(&a.D->rc[q], v); }
        else { if (v != INT_MAX) atomicMin(&a.D->rc[q], v); }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) a.chunk_count[blockIdx.x] = s_cnt;
}

// component kc of fluid f's prims at (i,j) as the sequential loop of cell
// `lin` sees them: an earlier mixed cell supplies its new prims (out[4f+kc])
__device__ __forceinline__ double vof_read1(const IfcArgs& a, int f, int i, int j, int kc, int64_t lin, bool& ok) {
  const GridP& P = a.P;
  const int64_t c = cidx(P, i, j);
  const int64_t l2 = (int64_t)i * P.nc + j;
  if (a.mask[c] && l2 < lin) {
    const int p = a.ifc_map[c];
    if (!ifc_wait(a, p)) { ok = false; return 0.0; }
    return __ldcg(a.out + (int64_t)p * IFC_OUT + 4 * f + kc);
  }
  return (f == 0 ? a.W1 : a.W2)[c + kc * P.plane];
}

// The mixed-cell loop, one warp per cell in the lane layout of
// k_interface_warp (lane = 16 s + 4 q + kc: probe side s, bilinear corner q,
// component kc).  out (8 doubles): the cell's new prims of fluid 1 and 2;
// mrp (8 doubles): MRPsoln1, MRPsoln2.
template <int MODE>
__global__ void __launch_bounds__(256) k_vof_chain(IfcArgs a, double* mrp) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  const int n = a.D->n_ifc;
  const int lane = threadIdx.x & 31;
  const int s = lane >> 4, q = (lane >> 2) & 3, kc = lane & 3;
  const bool isR = s == 1;
  const Gas k = isR ? P.gas2 : P.gas1;
  uint32_t st = 0;
  int iters = 0;
  for (;;) {
    int t = 0;
    if (lane == 0) t = (int)atomicAdd(a.ticket, 1u);
    t = __shfl_sync(FULL_MASK, t, 0);
    if (t >= n) break;
    if (t == a.withhold) continue;
    const int64_t lin = a.list[t];
    const int i = (int)(lin / P.nc), j = (int)(lin % P.nc);
    const int64_t c = cidx(P, i, j);
    const double zc = a.phi[c];
    const double lx = a.nrm[c], ly = a.nrm[c + P.plane];
    const double nx = a.nrm[c + 2 * P.plane], ny = a.nrm[c + 3 * P.plane];
    // get_interpolated_mixedRPstates_VOF (sourcecode/GFM_base.cpp:36-55):
    // side 1 samples prims2 at loc + ds n, side 0 prims1 at loc - ds n
    const double ds = 1.0 * (P.dy < P.dx ? P.dy : P.dx);
    const double px = isR ? lx + ds * nx : lx - ds * nx;
    const double py = isR ? ly + ds * ny : ly - ds * ny;
    const double sx = (px - P.x0) * P.idx + (double)P.g - 0.5;
    const double sy = (py - P.y0) * P.idy + (double)P.g - 0.5;
    int j0 = (int)floor(sx), i0 = (int)floor(sy);
    j0 = min(max(j0, 0), P.nc - 2);
    i0 = min(max(i0, 0), P.nr - 2);
    const double wa = sx - (double)j0, wb = sy - (double)i0;
    const double fa = (q & 1) ? wa : 1.0 - wa;
    const double fb = (q & 2) ? wb : 1.0 - wb;
    bool ok = true;
    const double gq = vof_read1(a, s, i0 + (q >> 1), j0 + (q & 1), kc, lin, ok);
    const double pr = (fa * fb) * gq;
    const double p1 = __shfl_down_sync(FULL_MASK, pr, 4);
    const double p2 = __shfl_down_sync(FULL_MASK, pr, 8);
    const double p3 = __shfl_down_sync(FULL_MASK, pr, 12);
    const double v = ((pr + p1) + p2) + p3;   // lanes 16 s + kc
    if (!__all_sync(FULL_MASK, ok)) {
      st |= ST_SCHEDULE_LIMIT;
      if (lane == 0) {
        st_release(a.done + t, 2);
      }
      continue;
    }
    double s0[4], s1[4];   // interfaceprims1 (side 0), interfaceprims2 (side 1)
    for (int m = 0; m < 4; m++) {
      s0[m] = __shfl_sync(FULL_MASK, v, m);
      s1[m] = __shfl_sync(FULL_MASK, v, 16 + m);
    }
    const V4 w1 = load4(a.W1, P, c), w2 = load4(a.W2, P, c);
    double o1[4], o2[4], m1v[4], m2v[4];
    if (MODE == VOF_GFM) {
      // the mixed Riemann problem in the normal frame (sourcecode/GFM_VOF.cpp:100-170)
      const double* own = isR ? s1 : s0;
      const double un = own[1] * nx + own[2] * ny;
      const double tx = own[1] - un * nx, ty = own[2] - un * ny;
      bool okp = true;
      const V4 Us = prims_to_cons<CHAIN_ID>(k.g, k.pinf, V4{own[0], un, 0.0, c_lt(1e-6, own[3]) ? own[3] : 1e-6}, &okp);
      if (!okp) st |= ST_UNPHYSICAL;
      int it = 0, gt = 0;
      const PairStar m = mixed_rs_pair(isR, k, P.gas1, P.gas2, Us, &st, &it, a, &gt);
      if (lane == 0) iters += it;
      if (c_isnan(m.p)) st |= ST_NAN;
      const double orho = xside(m.rho_own), otx = xside(tx), oty = xside(ty);
      const double rhoL = isR ? orho : m.rho_own, rhoR = isR ? m.rho_own : orho;
      const double t1x = isR ? otx : tx, t1y = isR ? oty : ty;
      const double t2x = isR ? tx : otx, t2y = isR ? ty : oty;
      const double snx = m.u * nx, sny = m.u * ny;
      double u1x, u1y, u2x, u2y;
      if (a.slip) { u1x = snx + t1x; u1y = sny + t1y; u2x = snx + t2x; u2y = sny + t2y; }
      else if (zc > 0.5) { u1x = snx + t1x; u1y = sny + t1y; u2x = snx + t1x; u2y = sny + t1y; }
      else { u1x = snx + t2x; u1y = sny + t2y; u2x = snx + t2x; u2y = sny + t2y; }
      m1v[0] = rhoL; m1v[1] = u1x; m1v[2] = u1y; m1v[3] = m.p;
      m2v[0] = rhoR; m2v[1] = u2x; m2v[2] = u2y; m2v[3] = m.p;
      if (zc > 0.5) {
        o1[0] = eos_isentropic_extrapolation<CHAIN_ID>(P.g1, P.p1, rhoL, m.p, w1.d); o1[1] = w1.b; o1[2] = w1.c; o1[3] = w1.d;
        for (int e = 0; e < 4; e++) o2[e] = m2v[e];
      } else {
        o2[0] = eos_isentropic_extrapolation<CHAIN_ID>(P.g2, P.p2, rhoR, m.p, w2.d); o2[1] = w2.b; o2[2] = w2.c; o2[3] = w2.d;
        for (int e = 0; e < 4; e++) o1[e] = m1v[e];
      }
    } else {
      // OGFM_VOF (sourcecode/OGFM_VOF.cpp:138-165): the interpolated states,
      // the ghost fluid's density by isentropic extrapolation
      for (int e = 0; e < 4; e++) { m1v[e] = s0[e]; m2v[e] = s1[e]; }
      if (zc > 0.5) {
        o1[0] = w1.a; o1[1] = w1.b; o1[2] = w1.c; o1[3] = w1.d;
        o2[0] = eos_isentropic_extrapolation<CHAIN_ID>(P.g2, P.p2, m2v[0], m2v[3], w1.d); o2[1] = w1.b; o2[2] = w1.c; o2[3] = w1.d;
      } else {
        o2[0] = w2.a; o2[1] = w2.b; o2[2] = w2.c; o2[3] = w2.d;
        o1[0] = eos_isentropic_extrapolation<CHAIN_ID>(P.g1, P.p1, m1v[0], m1v[3], w2.d); o1[1] = w2.b; o1[2] = w2.c; o1[3] = w2.d;
      }
    }
    if (lane == 0) {
      double* o = a.out + (int64_t)t * IFC_OUT;
      double* r = mrp + (int64_t)t * 8;
      for (int e = 0; e < 4; e++) { o[e] = o1[e]; o[4 + e] = o2[e]; r[e] = m1v[e]; r[4 + e] = m2v[e]; }
      st_release(a.done + t, 1);
    }
  }
  uint32_t wst = __reduce_or_sync(FULL_MASK, st);
  unsigned wit = __reduce_add_sync(FULL_MASK, (unsigned)iters);
  if (lane == 0) {
    if (wst) atomicOr(&a.D->status, wst);
    if (wit) {
      atomicAdd(&a.D->newton_iters, (unsigned long long)wit);
      atomicAdd(&a.D->ifc_iters, (unsigned long long)wit);
    }
  }
}

// After the loop: the inverse-distance ghost states of the real cells within
// the ring of a mixed cell (sourcecode/GFM_VOF.cpp:224-292,
// sourcecode/OGFM_VOF.cpp:171-262), conserved grids, and the velocity field.
struct VofGhostArgs {
  GridP P;
  const double* W1; const double* W2;
  const double* z;
  const uint8_t* mask;
  const int* ifc_map;
  const double* out;
  const double* mrp;
  const uint8_t* near_cell;   // real cells within the ring of a mixed cell
  double* U1; double* U2;
  double* vel;
  DevTime* D;
};

// sum over the mixed cells within the ring of (i,j), xinc-major as the reference
__device__ V4 vof_invdist_average(const VofGhostArgs& a, int i, int j, int f) {
  const GridP& P = a.P;
  const double ccx = P.x0 + ((double)(j - P.g) + 0.5) * P.dx;
  const double ccy = P.y0 + ((double)(i - P.g) + 0.5) * P.dy;
  double sw = 0.0;
  V4 sum = V4{0.0, 0.0, 0.0, 0.0};
  for (int xinc = -VOF_RING; xinc <= VOF_RING; xinc++)
    for (int yinc = -VOF_RING; yinc <= VOF_RING; yinc++) {
      const int64_t c2 = cidx(P, i + yinc, j + xinc);
      if (!a.mask[c2]) continue;
      const double tx = P.x0 + ((double)(j + xinc - P.g) + 0.5) * P.dx;
      const double ty = P.y0 + ((double)(i + yinc - P.g) + 0.5) * P.dy;
      const double ddx = tx - ccx, ddy = ty - ccy;
      const double w = divx(1.0, sqrtx(ddx * ddx + ddy * ddy));
      sw += w;
      const double* r = a.mrp + (int64_t)a.ifc_map[c2] * 8 + 4 * f;
      sum = V4{sum.a + w * r[0], sum.b + w * r[1], sum.c + w * r[2], sum.d + w * r[3]};
    }
  return V4{divx(sum.a, sw), divx(sum.b, sw), divx(sum.c, sw), divx(sum.d, sw)};
}

template <int MODE>
__global__ void __launch_bounds__(256) k_vof_ghost(VofGhostArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  const int64_t n = (int64_t)P.nr * P.nc;
  uint32_t st = 0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / P.nc), j = (int)(k % P.nc);
    const int64_t c = cidx(P, i, j);
    const double zc = a.z[c];
    V4 p1 = load4(a.W1, P, c), p2 = load4(a.W2, P, c);
    if (a.mask[c]) {
      const double* o = a.out + (int64_t)a.ifc_map[c] * IFC_OUT;
      p1 = V4{o[0], o[1], o[2], o[3]};
      p2 = V4{o[4], o[5], o[6], o[7]};
    }
    const bool real = is_real(P, i, j);
    const bool in_ring = vof_in_ring(P, i, j);
    // the velocity field: the real fluid's prims after the loop (for OGFM_VOF
    // stored in the loop, zero outside the ring; the ghost states below never
    // change the real fluid's velocity)
    double vx, vy;
    if (MODE == VOF_OGFM && !in_ring) { vx = 0.0; vy = 0.0; }
    else if (zc >= 0.5) { vx = p1.b; vy = p1.c; }
    else { vx = p2.b; vy = p2.c; }
    if (real && !a.mask[c] && (zc == 0.0 || zc == 1.0)) {
      if (a.near_cell[c]) {
        if (zc == 0.0) {   // flag 1: fluid 1 ghost state
          const V4 s = vof_invdist_average(a, i, j, 0);
          if (MODE == VOF_GFM) p1 = s;
          else p1 = V4{eos_isentropic_extrapolation(P.g1, P.p1, s.a, s.d, p2.d), p2.b, p2.c, p2.d};
        } else {           // flag 2: fluid 2 ghost state
          const V4 s = vof_invdist_average(a, i, j, 1);
          if (MODE == VOF_GFM) p2 = s;
          else p2 = V4{eos_isentropic_extrapolation(P.g2, P.p2, s.a, s.d, p1.d), p1.b, p1.c, p1.d};
        }
      }
    }
    bool ok1 = true, ok2 = true;
    const V4 u1 = prims_to_cons(P.g1, P.p1, p1, &ok1);
    const V4 u2 = prims_to_cons(P.g2, P.p2, p2, &ok2);
    if ((MODE == VOF_GFM || real) && (!ok1 || !ok2 || !is_physical_state_fast(u1) || !is_physical_state_fast(u2)))
      st |= ST_UNPHYSICAL;
    store4(a.U1, P, c, u1);
    store4(a.U2, P, c, u2);
    a.vel[c] = vx;
    a.vel[c + P.plane] = vy;
  }
  uint32_t wst = __reduce_or_sync(0xffffffffu, st);
  if ((threadIdx.x & 31) == 0 && wst) atomicOr(&a.D->status, wst);
}

// One directional sweep of the VOF advection over every padded cell: a ghost
// cell takes the update of its mirror / wrap source (the scalar BCs of phi).
// second: 0 for the step's first sweep, 1 for its second; the direction
// follows the step's parity (x first on even steps).
__global__ void __launch_bounds__(256) k_vof_sweep(GridP P, const double* z, const double* z0, const double* vel,
                                                    double* out, int second, const DevTime* D) {
  if (!D->active) return;
  const int first = (D->numsteps % 2 == 0) ? 0 : 1;
  const int dir = second ? 1 - first : first;
  const double dtdh = D->dt / (dir == 0 ? P.dx : P.dy);
  const int64_t e = dir == 0 ? 1 : P.pitch;
  GridP Q = P;
  if (!P.periodic) { Q.bcL = Q.bcR = Q.bcB = Q.bcT = GFM_BC_TRANSMISSIVE; }
  const int64_t n = (int64_t)P.nr * P.nc;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / P.nc), j = (int)(k % P.nc);
    const BCSrc sc = bc_source(Q, i, j);
    const int64_t c = cidx(P, sc.i, sc.j);
    const int64_t cl = c - e, ch = c + e;
    const double uL = 0.5 * (vel[cl + dir * P.plane] + vel[c + dir * P.plane]);
    const double uH = 0.5 * (vel[c + dir * P.plane] + vel[ch + dir * P.plane]);
    const double sL = uL * dtdh, sH = uH * dtdh;
    double FL = 0.0, FH = 0.0;
    if (sL > 0.0) FL = vof_strip_fraction(P, z, cl, dir, true, sL);
    else if (sL < 0.0) FL = -vof_strip_fraction(P, z, c, dir, false, -sL);
    if (sH > 0.0) FH = vof_strip_fraction(P, z, c, dir, true, sH);
    else if (sH < 0.0) FH = -vof_strip_fraction(P, z, ch, dir, false, -sH);
    const double cw = (z0[c] > 0.5) ? 1.0 : 0.0;
    double zn = z[c] - ((FH - cw * sH) - (FL - cw * sL));
    if (zn < VOF_ZEPS) zn = 0.0;
    else if (zn > 1.0 - VOF_ZEPS) zn = 1.0;
    out[cidx(P, i, j)] = zn;
  }
}

// Reset of the per-step interface bookkeeping.
// Completion flags and (out, for k_interface_warp) published values of the
// interface loop set to pending
__global__ void k_ifc_reset(int* done, double* out, int cap, unsigned int* ticket, const DevTime* D) {
  if (!D->active) return;
  int n = D->n_ifc;
  if (n > cap) n = cap;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    done[k] = 0;
    if (out)
      for (int q = 0; q < 4; q++) out[(int64_t)k * IFC_OUT + q] = __longlong_as_double((long long)IFC_PENDING);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *ticket = 0u;
}

// Scatter of the interface results into the primitive grids.
//   Riemann / real GFM: prims of the real fluid := star state
//   modified GFM: new_prims (Wc) real density and ghost state
struct ScatterArgs {
  GridP P;
  double* W1; double* W2;    // written grids
  const double* phi;
  const int* list;
  const double* out;
  double* vel;               // extension velocity seeds (or null)
  DevTime* D;
  int modified;
};

__global__ void k_ifc_scatter(ScatterArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  const int n = a.D->n_ifc;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int64_t lin = a.list[k];
    int i = (int)(lin / P.nc), j = (int)(lin % P.nc);
    int64_t c = cidx(P, i, j);
    const double* o = a.out + (int64_t)k * IFC_OUT;
    bool f1 = a.phi[c] <= 0.0;
    if (a.modified) {
      double* Wr = f1 ? a.W1 : a.W2;
      double* Wg = f1 ? a.W2 : a.W1;
      Wr[c] = o[0];
      store4(Wg, P, c, V4{o[1], o[2], o[3], o[4]});
      if (a.vel) { a.vel[c] = o[5]; a.vel[c + P.plane] = o[6]; }
    } else {
      store4(f1 ? a.W1 : a.W2, P, c, V4{o[0], o[1], o[2], o[3]});
      if (a.vel) { a.vel[c] = o[4]; a.vel[c + P.plane] = o[5]; }
    }
  }
}

// Velocity field of the interfacial cells after the Riemann / real GFM loop:
// the star state it wrote into the cell's real fluid (the rest of the real
// cells' field comes from the conversion, k_prims with a velocity plane).
__global__ void k_ifc_vel(GridP P, const int* list, const double* out, double* vel, const DevTime* D) {
  if (!D->active) return;
  const int n = D->n_ifc;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    int i, j;
    linear_to_ij(P, list[k], i, j);
    const int64_t c = cidx(P, i, j);
    const double* o = out + (int64_t)k * IFC_OUT;
    vel[c] = o[1];
    vel[c + P.plane] = o[2];
  }
}

// ---------------------------------------------------------------------------
// End of the ghost fill: primitives -> conserved on the whole padded grid,
// velocity field (real fluid's velocity per cell), and for the original GFM
// the ghost assignment of sourcecode/GFM_original.cpp:59-118 with the
// realcells boxes.
// ---------------------------------------------------------------------------
struct FinalArgs {
  GridP P;
  double* W1; double* W2;        // final primitives (modified in place by OGFM)
  const double* C1; const double* C2;   // grids converted to conserved (== W unless modified GFM)
  const double* V1; const double* V2;   // source of the velocity field
  const uint8_t* mask;
  const double* phi;
  double* U1; double* U2;
  double* vel;
  DevTime* D;
  int ogfm;
  int vel_mode;   // 0: real-fluid velocity, 1: extension seeds (OGFM interfacial), 2: leave vel alone
};

__global__ void __launch_bounds__(256) k_finalize(FinalArgs a) {
  const GridP& P = a.P;
  if (!a.D->active) return;
  const int64_t n = (int64_t)P.nr * P.nc;
  uint32_t st = 0;
  int bb[8] = {INT_MAX, INT_MIN, INT_MAX, INT_MIN, INT_MAX, INT_MIN, INT_MAX, INT_MIN};
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.nc), j = (int)(k % P.nc);
    int64_t c = cidx(P, i, j);
    bool f1 = c_le0(a.phi[c]);
    if (a.ogfm) {
      V4 w1 = load4(a.W1, P, c), w2 = load4(a.W2, P, c);
      if (is_real(P, i, j)) {
        if (f1) {
          double rho_new = eos_isentropic_extrapolation(P.g2, P.p2, w2.a, w2.d, w1.d);
          if (!(rho_new >= 0.0)) st |= ST_UNPHYSICAL;
          w2 = V4{rho_new, w1.b, w1.c, w1.d};
          store4(a.W2, P, c, w2);
          bb[0] = min(bb[0], i - 2); bb[1] = max(bb[1], i + 2); bb[2] = min(bb[2], j - 2); bb[3] = max(bb[3], j + 2);
        } else {
          double rho_new = eos_isentropic_extrapolation(P.g1, P.p1, w1.a, w1.d, w2.d);
          if (!(rho_new >= 0.0)) st |= ST_UNPHYSICAL;
          w1 = V4{rho_new, w2.b, w2.c, w2.d};
          store4(a.W1, P, c, w1);
          bb[4] = min(bb[4], i - 2); bb[5] = max(bb[5], i + 2); bb[6] = min(bb[6], j - 2); bb[7] = max(bb[7], j + 2);
        }
      }
    }
    bool ok1 = true, ok2 = true;
    V4 u1 = prims_to_cons(P.g1, P.p1, load4(a.C1, P, c), &ok1);
    V4 u2 = prims_to_cons(P.g2, P.p2, load4(a.C2, P, c), &ok2);
    if (!ok1 || !ok2 || !is_physical_state_fast(u1) || !is_physical_state_fast(u2)) st |= ST_UNPHYSICAL;
    store4(a.U1, P, c, u1);
    store4(a.U2, P, c, u2);
    if (a.vel_mode == 0) {
      const double* V = f1 ? a.V1 : a.V2;
      a.vel[c] = V[c + P.plane];
      a.vel[c + P.plane] = V[c + 2 * P.plane];
    } else if (a.vel_mode == 1) {
      double vx = 0.0, vy = 0.0;
      if (a.mask[c]) { const double* V = f1 ? a.V1 : a.V2; vx = V[c + P.plane]; vy = V[c + 2 * P.plane]; }
      a.vel[c] = vx;
      a.vel[c + P.plane] = vy;
    }
  }
  uint32_t wst = __reduce_or_sync(0xffffffffu, st);
  if ((threadIdx.x & 31) == 0 && wst) atomicOr(&a.D->status, wst);
  if (a.ogfm) {
    for (int q = 0; q < 8; q++) {
      int v = bb[q];
      if (q & 1) { for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o)); }
      else { for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o)); }
      if ((threadIdx.x & 31) == 0) {
        if (q & 1) { if (v != INT_MIN) atomicMax(&a.D->rc[q], v); }
        else { if (v != INT_MAX) atomicMin(&a.D->rc[q], v); }
      }
    }
  }
}

// realcells clamp of sourcecode/GFM_original.cpp:120-128
__global__ void k_rc_clamp(GridP P, DevTime* D) {
  if (!D->active) return;
  for (int f = 0; f < 2; f++) {
    int* r = &D->rc[4 * f];
    r[0] = max(r[0], P.g);
    r[1] = min(r[1], P.g + P.Ny);
    r[2] = max(r[2], P.g);
    r[3] = min(r[3], P.g + P.Nx);
  }
}

// ---------------------------------------------------------------------------
// extrapolate_extension_vfield sweep (sourcecode/extrapolate_extension_vfield.cpp:4-122)
// with the mirror BCs of the vector field, one launch per iteration.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ext_vel(GridP P, const double* S, double* Dd, const double* phi,
                                                const double* nrm, const uint8_t* mask, const DevTime* D) {
  if (!D->active) return;
  const int64_t n = (int64_t)P.nr * P.nc;
  const double dt = 0.5 * dmin_std(P.dx, P.dy);
  GridP Q = P;
  Q.bcL = Q.bcR = Q.bcB = Q.bcT = GFM_BC_TRANSMISSIVE;
  Q.periodic = false;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.nc), j = (int)(k % P.nc);
    BCSrc s = bc_source(Q, i, j);
    int64_t c = cidx(P, s.i, s.j);
    double vx = S[c], vy = S[c + P.plane];
    double nn = nrm[c + 4 * P.plane];
    if (!mask[c] && nn > 1e-12) {
      double nx = nrm[c + 2 * P.plane], ny = nrm[c + 3 * P.plane];
      double cx = (dt / P.dx) * nx, cy = (dt / P.dy) * ny;
      double dxx, dxy, dyx, dyy;
      if (phi[c] <= 0.0) {
        if (nx > 0.0) { dxx = S[c + 1] - vx; dxy = S[c + 1 + P.plane] - vy; }
        else { dxx = vx - S[c - 1]; dxy = vy - S[c - 1 + P.plane]; }
        if (ny > 0.0) { dyx = S[c + P.pitch] - vx; dyy = S[c + P.pitch + P.plane] - vy; }
        else { dyx = vx - S[c - P.pitch]; dyy = vy - S[c - P.pitch + P.plane]; }
        vx = (vx + cx * dxx) + cy * dyx;
        vy = (vy + cx * dxy) + cy * dyy;
      } else {
        if (nx > 0.0) { dxx = vx - S[c - 1]; dxy = vy - S[c - 1 + P.plane]; }
        else { dxx = S[c + 1] - vx; dxy = S[c + 1 + P.plane] - vy; }
        if (ny > 0.0) { dyx = vx - S[c - P.pitch]; dyy = vy - S[c - P.pitch + P.plane]; }
        else { dyx = S[c + P.pitch] - vx; dyy = S[c + P.pitch + P.plane] - vy; }
        vx = (vx - cx * dxx) - cy * dyx;
        vy = (vy - cx * dxy) - cy * dyy;
      }
    }
    int64_t o = cidx(P, i, j);
    Dd[o] = vx;
    Dd[o + P.plane] = vy;
  }
}

// ---------------------------------------------------------------------------
// Level set (the project's Levelset; see the oracle for the same definition)
//   order 1: phi + dt L(phi), first-order upwind
//   order 5: HOUC5 in space, 3-stage TVD Runge-Kutta (Shu-Osher) in time
//   L(f) = -(u f_x + v f_y) with the cell-centred velocity field
// Ghost cells: mirror (or periodic) copies, computed by their own threads.
// ---------------------------------------------------------------------------
// HOUC5 derivative: a >= 0 uses (-2, 15, -60, 20, 30, -3) on f[c-3..c+2],
// a < 0 (3, -30, -20, 60, -15, 2) on f[c-2..c+3], each summed left to right
// as written.  Subtracting b*x is adding (-b)*x (the same IEEE operations), so
// both branches are one sum with coefficients and offset chosen per lane: a
// warp whose lanes upwind in different directions issues it once.
__device__ __forceinline__ double houc5(double a, const double* f, int64_t c, int64_t st, double inv60h) {
  const bool up = c_ge0(a);
  const double k0 = up ? -2.0 : 3.0, k1 = up ? 15.0 : -30.0, k2 = up ? -60.0 : -20.0;
  const double k3 = up ? 20.0 : 60.0, k4 = up ? 30.0 : -15.0, k5 = up ? -3.0 : 2.0;
  const double* g = f + c + (up ? -3 : -2) * st;
  return (k0 * g[0] + k1 * g[st] + k2 * g[2 * st] + k3 * g[3 * st] + k4 * g[4 * st] + k5 * g[5 * st]) * inv60h;
}

// every > 1: part of a reinitialisation that runs only on steps whose number
// (counting from 1) is a multiple of `every`, decided on the device so that a
// captured step graph replays correctly on every step
__device__ __forceinline__ bool reinit_skipped(const DevTime* D, int every) {
  return every > 1 && (D->numsteps + 1) % every != 0;
}

// S non-null (the last stage of a step that reinitialises, unless
// reinit_skipped(D, every)): also the reinitialisation's sign function
// S = r / sqrt(r^2 + h^2) of the new value r, k_reinit_iter's S
template <int ORDER, int STAGE>
__global__ void __launch_bounds__(256) k_ls_stage(GridP P, const double* X, const double* phi, double* out,
                                                  const double* vel, const DevTime* D, double* S, int every) {
  if (!D->active) return;
  const double dt = D->dt;
  const bool sign = S != nullptr && !reinit_skipped(D, every);
  const double h = dmin_std(P.dx, P.dy);
  const int64_t n = (int64_t)P.nr * P.nc;
  GridP Q = P;
  if (!P.periodic) { Q.bcL = Q.bcR = Q.bcB = Q.bcT = GFM_BC_TRANSMISSIVE; }
  const double idx = 1.0 / P.dx, idy = 1.0 / P.dy;
  const double i60x = 1.0 / (60.0 * P.dx), i60y = 1.0 / (60.0 * P.dy);
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.nc), j = (int)(k % P.nc);
    BCSrc s = bc_source(Q, i, j);
    int64_t c = cidx(P, s.i, s.j);
    double u = vel[c], v = vel[c + P.plane];
    double fx, fy;
    if (ORDER == 1) {
      fx = c_ge0(u) ? (X[c] - X[c - 1]) * idx : (X[c + 1] - X[c]) * idx;
      fy = c_ge0(v) ? (X[c] - X[c - P.pitch]) * idy : (X[c + P.pitch] - X[c]) * idy;
    } else {
      fx = houc5(u, X, c, 1, i60x);
      fy = houc5(v, X, c, P.pitch, i60y);
    }
    double L = -(u * fx + v * fy);
    double r;
    if (ORDER == 1 || STAGE == 1) r = X[c] + dt * L;
    else if (STAGE == 2) r = 0.75 * phi[c] + 0.25 * (X[c] + dt * L);
    else r = (1.0 / 3.0) * phi[c] + (2.0 / 3.0) * (X[c] + dt * L);
    out[cidx(P, i, j)] = r;
    if (sign) S[cidx(P, i, j)] = divx(r, sqrtx(r * r + h * h));
  }
}

// invert 0: skipped on the steps reinit_skipped(D, every) names; invert 1: on the others
__global__ void k_copy_plane(GridP P, const double* src, double* dst, const DevTime* D, int every, int invert) {
  if (!D->active || reinit_skipped(D, every) != (invert != 0)) return;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < P.plane; k += (int64_t)gridDim.x * blockDim.x)
    dst[k] = src[k];
}

// one Sussman-Smereka-Osher iteration with Godunov upwinding
__global__ void __launch_bounds__(256) k_reinit_iter(GridP P, const double* cur, const double* S, double* out,
                                                     const DevTime* D, int every) {
  if (!D->active || reinit_skipped(D, every)) return;
  const int64_t n = (int64_t)P.nr * P.nc;
  GridP Q = P;
  if (!P.periodic) { Q.bcL = Q.bcR = Q.bcB = Q.bcT = GFM_BC_TRANSMISSIVE; }
  const double h = dmin_std(P.dx, P.dy);
  const double dtau = 0.5 * h;
  const double idx = 1.0 / P.dx, idy = 1.0 / P.dy;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.nc), j = (int)(k % P.nc);
    BCSrc s = bc_source(Q, i, j);
    int64_t c = cidx(P, s.i, s.j);
    double f = cur[c];
    double sg = S[c];
    double a = (f - cur[c - 1]) * idx;
    double b = (cur[c + 1] - f) * idx;
    double cc = (f - cur[c - P.pitch]) * idy;
    double d = (cur[c + P.pitch] - f) * idy;
    // Godunov's upwind gradient: gx = max(x1^2, x2^2) with (x1, x2) = (max(a,0),
    // min(b,0)) where sg > 0, (min(a,0), max(b,0)) elsewhere (gy alike).  The
    // larger square is the square of the larger magnitude (rounding is
    // monotonic; equal squares are the same double, and a NaN operand keeps
    // max()'s choice of its first argument), so the candidates are compared
    // on the integer pipe and one square is formed per direction.
    double x1, x2, y1, y2;
    if (c_gt0(sg)) {
      x1 = dmax_std(a, 0.0); x2 = dmin_std(b, 0.0); y1 = dmax_std(cc, 0.0); y2 = dmin_std(d, 0.0);
    } else {
      x1 = dmin_std(a, 0.0); x2 = dmax_std(b, 0.0); y1 = dmin_std(cc, 0.0); y2 = dmax_std(d, 0.0);
    }
    const double mx = c_lt(fabs_bits(x1), fabs_bits(x2)) ? x2 : x1;
    const double my = c_lt(fabs_bits(y1), fabs_bits(y2)) ? y2 : y1;
    const double gx = mx * mx, gy = my * my;
    double G = sqrtx(gx + gy) - 1.0;
    out[cidx(P, i, j)] = f - dtau * sg * G;
  }
}

// ---------------------------------------------------------------------------
// fluid mass (sim_twofluid::fluid_mass, sourcecode/sim_twofluid.cpp:1803-1827):
// fixed-order two-pass sum
// ---------------------------------------------------------------------------
__global__ void k_mass_partial(GridP P, const double* U, const double* phi, int vof, double sign, double* part) {
  __shared__ double sh[256];
  double acc = 0.0;
  const int64_t n = (int64_t)P.Nx * P.Ny;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(k / P.Nx) + P.g, j = (int)(k % P.Nx) + P.g;
    int64_t c = cidx(P, i, j);
    double ls = phi ? (vof ? 0.5 - phi[c] : phi[c]) : -1.0;   // get_sdf
    if (sign * ls > 0.0) acc += U[c] * P.dx * P.dy;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_mass_final(const double* part, int nb, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += part[b];
    *out = s;
  }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------

// the sweep's coefficients dt/dx, dt/dy with dt = 0.5 min(dx, dy), correctly
// rounded here exactly as a device division would round them
static void extrap_coeffs(const GridP& P, ExtrapArgs& e) {
  const double dt = 0.5 * ((P.dy < P.dx) ? P.dy : P.dx);
  e.cdx = dt / P.dx;
  e.cdy = dt / P.dy;
}

static void run_extrap(gfm_ctx* ctx, int N, bool mgfm) {
  const GridP& P = ctx->P;
  const int blocks = wave_blocks((const void*)k_extrap<false>, 256, ctx->num_sms, padded_cells(P));
  for (int it = 0; it < N; it++) {
    ExtrapArgs e;
    e.P = P;
    e.S1 = ctx->W[0]; e.S2 = ctx->W[1];
    e.D1 = ctx->Wt[0]; e.D2 = ctx->Wt[1];
    e.phi = ctx->phi; e.nrm = ctx->nrm; e.mask = ctx->mask; e.D = ctx->dtime;
    e.mgfm = mgfm ? 1 : 0;
    e.ov_out = nullptr; e.ov_map = nullptr; e.overlay = 0;
    e.band = nullptr;
    e.list = nullptr; e.list_n = nullptr;
    e.nclass = 0; e.list_stride = 0;
    e.F1 = nullptr; e.F2 = nullptr; e.cls = nullptr; e.near_min = 0;
    e.Dw = ctx->dtime; e.fsel = 0; e.fnear = nullptr; e.fU1 = nullptr; e.fU2 = nullptr; e.fvel = nullptr;
    e.store_w = 1;
    extrap_coeffs(P, e);
    k_extrap<false><<<blocks, 256, 0, ctx->stream>>>(e); counted();
    for (int f = 0; f < 2; f++) { double* t = ctx->W[f]; ctx->W[f] = ctx->Wt[f]; ctx->Wt[f] = t; }
  }
}

static void run_ext_vfield(gfm_ctx* ctx, int N) {
  const GridP& P = ctx->P;
  int blocks = grid_blocks((int64_t)P.nr * P.nc, 256);
  for (int it = 0; it < N; it++) {
    k_ext_vel<<<blocks, 256, 0, ctx->stream>>>(P, ctx->vel, ctx->vel_t, ctx->phi, ctx->nrm, ctx->mask, ctx->dtime); counted();
    double* t = ctx->vel; ctx->vel = ctx->vel_t; ctx->vel_t = t;
  }
}

void launch_cfl(gfm_ctx* ctx, double CFL, double T) { (void)ctx; (void)CFL; (void)T; }

void launch_cfl_ogfm(gfm_ctx* ctx, double CFL, double T, bool ogfm, unsigned int* counter) {
  launch_cfl_impl(ctx, CFL, T, ogfm, counter);
}

// the learned proposal and the capture of training problems (both off by default)
// the learned proposal and the capture of the interface loop launched on
// stream s (the network's fragments are packed on s just before it)
static void set_learning(gfm_ctx* ctx, IfcArgs& ia, cudaStream_t s) {
  ia.mlp = ctx->mlp ? mlp_params(ctx->mlp) : nullptr;
  ia.mlp_frag = ctx->mlp ? mlp_frag(ctx->mlp) : nullptr;
  if (ctx->mlp) launch_mlp_frag_pack(ctx->mlp, s);
  ia.cap_X = ctx->cap_X; ia.cap_Y = ctx->cap_Y; ia.cap_count = ctx->cap_count; ia.cap = ctx->cap;
}

void launch_ghost_fill(gfm_ctx* ctx, const gfm_method_desc* m) {
  const GridP& P = ctx->P;
  cudaStream_t s = ctx->stream;
  const int variant = m->gfm;
  const bool modified = variant == GFM_MODIFIED;
  // 1. conversion, gradient of phi, interfacial mask, chunk counts
  PrimArgs pa;
  pa.P = P;
  pa.U1 = ctx->U[0]; pa.U2 = ctx->U[1];
  pa.W1 = ctx->W[0]; pa.W2 = ctx->W[1];
  pa.Wc1 = modified ? ctx->Wc[0] : nullptr;
  pa.Wc2 = modified ? ctx->Wc[1] : nullptr;
  pa.phi = ctx->phi; pa.nrm = ctx->nrm; pa.mask = ctx->mask; pa.ifc_map = ctx->ifc_map;
  pa.chunk_count = ctx->chunk_count; pa.chunk = ctx->chunk; pa.D = ctx->dtime;
  pa.check_both = (variant == GFM_OGFM || variant == GFM_RIEMANN) ? 1 : 0;
  pa.cfl_counter = ctx->cfl_counter;
  pa.vel = nullptr;   // k_finalize writes the velocity field
  k_prims<<<ctx->n_chunks, CHUNK_T, 0, s>>>(pa); counted();
  k_compact<<<ctx->n_chunks, CHUNK_T, 0, s>>>(P, ctx->mask, ctx->chunk_count, ctx->n_chunks, ctx->chunk, ctx->ifc_list,
                                              ctx->ifc_map, ctx->dtime); counted();
  const bool ext = m->use_extension_vfield != 0;
  const int fblocks = wave_blocks((const void*)k_finalize, 256, ctx->num_sms, padded_cells(P));
  if (variant == GFM_OGFM) {
    run_extrap(ctx, 6, false);
    FinalArgs f;
    f.P = P;
    f.W1 = ctx->W[0]; f.W2 = ctx->W[1];
    f.C1 = ctx->W[0]; f.C2 = ctx->W[1];
    f.V1 = ctx->W[0]; f.V2 = ctx->W[1];
    f.mask = ctx->mask; f.phi = ctx->phi;
    f.U1 = ctx->U[0]; f.U2 = ctx->U[1];
    f.vel = ctx->vel; f.D = ctx->dtime;
    f.ogfm = 1;
    f.vel_mode = ext ? 1 : 0;
    k_finalize<<<fblocks, 256, 0, s>>>(f); counted();
    k_rc_clamp<<<1, 1, 0, s>>>(P, ctx->dtime); counted();
    if (ext) run_ext_vfield(ctx, 20);
    return;
  }
  // 2. extrapolate_vector(2) before the interface loop (Riemann, modified)
  if (variant != GFM_REAL) run_extrap(ctx, 2, false);
  // 3. interface loop
  int cap = P.Nx * P.Ny;
  k_ifc_reset<<<grid_blocks(cap, 256), 256, 0, s>>>(ctx->ifc_done, ctx->ifc_out, cap, (unsigned int*)(ctx->ifc_opp),
                                                     ctx->dtime);
  counted();
  IfcArgs ia;
  ia.P = P;
  ia.W1 = ctx->W[0]; ia.W2 = ctx->W[1];
  ia.phi = ctx->phi; ia.nrm = ctx->nrm; ia.mask = ctx->mask;
  ia.list = ctx->ifc_list; ia.ifc_map = ctx->ifc_map;
  ia.done = ctx->ifc_done; ia.out = ctx->ifc_out;
  ia.ticket = (unsigned int*)(ctx->ifc_opp);
  ia.D = ctx->dtime;
  ia.spin_limit = ctx->ifc_spin_limit > 0 ? ctx->ifc_spin_limit : IFC_SPIN_LIMIT;
  ia.withhold = ctx->ifc_withhold - 1;
  ia.slip = m->use_slip_BCs;
  set_learning(ctx, ia, s);
  ia.probe_ij = nullptr; ia.probe_w = nullptr; ia.probe_dep = nullptr;
  if (variant == GFM_RIEMANN) {
    k_ifc_probes<<<152, 256, 0, s>>>(ia, ctx->probe_ij, ctx->probe_w, ctx->probe_dep); counted();
    ia.probe_ij = ctx->probe_ij; ia.probe_w = ctx->probe_w; ia.probe_dep = ctx->probe_dep;
  }
  int iblocks = 152;   // 4 warps per CTA: one chain warp per SM sub-partition
  if (variant == GFM_RIEMANN) k_interface_warp<IFC_RIEMANN><<<iblocks, 128, 0, s>>>(ia);
  else if (variant == GFM_REAL) k_interface_warp<IFC_REAL><<<iblocks, 128, 0, s>>>(ia);
  else k_interface<IFC_MODIFIED><<<iblocks, 128, 0, s>>>(ia);
  counted();
  if (ext) cudaMemsetAsync(ctx->vel, 0, sizeof(double) * 2 * P.plane, s);
  ScatterArgs sa;
  sa.P = P;
  sa.W1 = modified ? ctx->Wc[0] : ctx->W[0];
  sa.W2 = modified ? ctx->Wc[1] : ctx->W[1];
  sa.phi = ctx->phi; sa.list = ctx->ifc_list; sa.out = ctx->ifc_out;
  sa.vel = ext ? ctx->vel : nullptr;
  sa.D = ctx->dtime;
  sa.modified = modified ? 1 : 0;
  k_ifc_scatter<<<grid_blocks(cap, 256), 256, 0, s>>>(sa); counted();
  // 4. extrapolate_vector(6) / extrapolate_vector_mgfm(6)
  run_extrap(ctx, 6, modified);
  // 5. conserved grids and velocity field
  FinalArgs f;
  f.P = P;
  f.W1 = ctx->W[0]; f.W2 = ctx->W[1];
  f.C1 = modified ? ctx->Wc[0] : ctx->W[0];
  f.C2 = modified ? ctx->Wc[1] : ctx->W[1];
  f.V1 = ctx->W[0]; f.V2 = ctx->W[1];
  f.mask = ctx->mask; f.phi = ctx->phi;
  f.U1 = ctx->U[0]; f.U2 = ctx->U[1];
  f.vel = ctx->vel; f.D = ctx->dtime;
  f.ogfm = 0;
  f.vel_mode = ext ? 2 : 0;
  k_finalize<<<fblocks, 256, 0, s>>>(f); counted();
  if (ext) run_ext_vfield(ctx, 20);
}

// ---------------------------------------------------------------------------
// Overlapped ghost fill for the Riemann and real GFM.
//
// The interface loop only writes the real fluid of interfacial cells, and
// the six Jacobi sweeps of extrapolate_vector that follow move information
// one cell per sweep (5-point stencil; ghost cells copy their BC source), so
// the extrapolated primitives of every cell more than 6 cells (Chebyshev)
// from all interfacial cells do not depend on the interface loop.  Those far
// cells, and the flux update of tiles that read only far cells, are computed
// from the pre-loop primitives on a large SM partition while the interface
// loop (a latency-bound dependency chain) runs on a small one; the near cells
// and near tiles are finished after it.  Results are identical to the
// sequential schedule: every value is computed from the same inputs by the
// same kernels.
// ---------------------------------------------------------------------------

// marks the real cells within `radius` (Chebyshev) of an interfacial cell
__global__ void k_near_mark(GridP P, const int* list, const DevTime* D, uint8_t* near_cell, int radius) {
  if (!D->active) return;
  const int n = D->n_ifc;
  const int side = 2 * radius + 1;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < (int64_t)n * side * side;
       q += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(q / (side * side));
    int r = (int)(q % (side * side));
    int64_t lin = list[k];
    int i = (int)(lin / P.nc) + r / side - radius;
    int j = (int)(lin % P.nc) + r % side - radius;
    if (P.periodic) {
      i = ((i - P.g) % P.Ny + P.Ny) % P.Ny + P.g;
      j = ((j - P.g) % P.Nx + P.Nx) % P.Nx + P.g;
    } else if (!is_real(P, i, j)) {
      continue;
    }
    near_cell[cidx(P, i, j)] = 1;
  }
}

// cls[c] = max over interfacial cells of radius + 1 - (Chebyshev distance to
// the real cell c), for the cells within `radius` (cls zeroed by the caller)
__global__ void k_band_mark(GridP P, const int* list, const DevTime* D, int* cls, int radius) {
  if (!D->active) return;
  const int n = D->n_ifc;
  const int side = 2 * radius + 1;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < (int64_t)n * side * side;
       q += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(q / (side * side));
    int r = (int)(q % (side * side));
    int64_t lin = list[k];
    const int di = r / side - radius, dj = r % side - radius;
    int i = (int)(lin / P.nc) + di;
    int j = (int)(lin % P.nc) + dj;
    if (P.periodic) {
      i = ((i - P.g) % P.Ny + P.Ny) % P.Ny + P.g;
      j = ((j - P.g) % P.Nx + P.Nx) % P.Nx + P.g;
    } else if (!is_real(P, i, j)) {
      continue;
    }
    const int d = max(abs(di), abs(dj));
    atomicMax(&cls[cidx(P, i, j)], radius + 1 - d);
  }
}

// one warp per flux tile: does the tile's read region (tile + 2-cell halo,
// clamped as the flux kernel clamps it) hold a near cell?
__global__ void k_tile_flags(GridP P, const uint8_t* near_cell, int* tile_near, int ntx, int nty, const DevTime* D) {
  if (!D->active) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= ntx * nty) return;
  const int tx = warp % ntx, ty = warp / ntx;
  const int i0 = P.g + ty * FLUX_TY, j0 = P.g + tx * FLUX_TX;
  const int WR = FLUX_TY + 4, WC = FLUX_TX + 4;
  int any = 0;
  for (int q = lane; q < WR * WC; q += 32) {
    int i = min(max(i0 - 2 + q / WC, 0), P.nr - 1);
    int j = min(max(j0 - 2 + q % WC, 0), P.nc - 1);
    BCSrc s = bc_source(P, i, j);
    any |= near_cell[cidx(P, s.i, s.j)];
  }
  any = __any_sync(0xffffffffu, any);
  if (lane == 0) tile_near[warp] = any ? 1 : 0;
}

// one sweep of the overlapped schedule; fsel != 0 fuses k_finalize's
// conversion of the sweep's results (1: far cells, 2: the listed near cells),
// which are then not stored as primitives
static void extrap_sweep(gfm_ctx* ctx, const double* S1, const double* S2, double* D1, double* D2, bool overlay,
                         cudaStream_t s, const int* list, const int* list_n, int nclass,
                         const double* const* far = nullptr, int near_min = 0, int fsel = 0) {
  const GridP& P = ctx->P;
  ExtrapArgs e;
  e.P = P;
  e.S1 = S1; e.S2 = S2; e.D1 = D1; e.D2 = D2;
  e.phi = ctx->phi; e.nrm = ctx->nrm; e.mask = ctx->mask; e.D = ctx->dtime;
  e.mgfm = 0;
  e.ov_out = overlay ? ctx->ifc_out : nullptr;
  e.ov_map = overlay ? ctx->ifc_map : nullptr;
  e.overlay = overlay ? 1 : 0;
  e.band = nullptr;
  e.list = list; e.list_n = list_n;
  e.nclass = nclass;
  e.list_stride = ctx->band_stride;
  e.F1 = far ? far[0] : nullptr; e.F2 = far ? far[1] : nullptr;
  e.cls = ctx->band_cls;
  e.near_min = near_min;
  e.Dw = ctx->dtime;
  e.fsel = fsel;
  e.fnear = ctx->near_cell;
  e.fU1 = ctx->U[0]; e.fU2 = ctx->U[1];
  e.fvel = ctx->vel;
  e.store_w = fsel ? 0 : 1;
  extrap_coeffs(P, e);
  // a listed sweep covers the band around the interface: a few percent of the grid
  if (fsel) {
    const int blocks = list ? NEAR_CTAS : wave_blocks((const void*)k_extrap<true>, 256, ctx->far_sms, padded_cells(P));
    k_extrap<true><<<blocks, 256, 0, s>>>(e);
  } else {
    const int blocks = list ? NEAR_CTAS : wave_blocks((const void*)k_extrap<false>, 256, ctx->far_sms, padded_cells(P));
    k_extrap<false><<<blocks, 256, 0, s>>>(e);
  }
  counted();
}


void launch_ghost_fill_overlapped(gfm_ctx* ctx, const gfm_method_desc* m) {
  const GridP& P = ctx->P;
  cudaStream_t s = ctx->stream;
  const int variant = m->gfm;
  // conversion, normals, mask, ordered list of interfacial cells
  PrimArgs pa;
  pa.P = P;
  pa.U1 = ctx->U[0]; pa.U2 = ctx->U[1];
  pa.W1 = ctx->W[0]; pa.W2 = ctx->W[1];
  pa.Wc1 = nullptr; pa.Wc2 = nullptr;
  pa.phi = ctx->phi; pa.nrm = ctx->nrm; pa.mask = ctx->mask; pa.ifc_map = ctx->ifc_map;
  pa.chunk_count = ctx->chunk_count; pa.chunk = ctx->chunk; pa.D = ctx->dtime;
  pa.check_both = (variant == GFM_RIEMANN) ? 1 : 0;
  pa.cfl_counter = ctx->cfl_counter;
  pa.vel = ctx->vel;  // real cells' velocity field, for a level set that starts after the chain
  k_prims<<<ctx->n_chunks, CHUNK_T, 0, s>>>(pa);
  counted();
  k_compact<<<ctx->n_chunks, CHUNK_T, 0, s>>>(P, ctx->mask, ctx->chunk_count, ctx->n_chunks, ctx->chunk, ctx->ifc_list,
                                              ctx->ifc_map, ctx->dtime);
  counted();
  const int cap = P.Nx * P.Ny;
  // extrapolate_vector(2) before the Riemann GFM's interface loop
  if (variant == GFM_RIEMANN) run_extrap(ctx, 2, false);
  cudaEventRecord(ctx->ev_fork, s);
  if (ctx->timing) cudaEventRecord(ctx->tev[0], s);
  if (ctx->part_ev[0]) cudaEventRecord(ctx->part_ev[0], s);

  // far partition, first: the band around the interface (distance classes,
  // lists), the near cells and the flux tiles that read them; the interface
  // loop does not need them, the far field and the near path after the loop do
  cudaStream_t sf = ctx->s_far;
  cudaStreamWaitEvent(sf, ctx->ev_fork, 0);
  cudaMemsetAsync(ctx->band_cls, 0, sizeof(int) * (size_t)P.plane, sf);
  k_band_mark<<<grid_blocks((int64_t)cap, 256), 256, 0, sf>>>(P, ctx->ifc_list, ctx->dtime, ctx->band_cls,
                                                               NEAR_RADIUS);
  counted();
  cudaMemsetAsync(ctx->list_n, 0, BAND_CLASSES * sizeof(int), sf);
  k_band_lists<<<grid_blocks((int64_t)P.nr * P.nc, 256), 256, 0, sf>>>(P, ctx->band_cls, ctx->near_cell,
                                                                       ctx->band_list, ctx->band_stride,
                                                                       ctx->list_n, ctx->dtime);
  counted();
  const int ntx = flux_tiles_x(P), nty = flux_tiles_y(P);
  k_tile_flags<<<(ntx * nty + 7) / 8, 256, 0, sf>>>(P, ctx->near_cell, ctx->tile_near, ntx, nty, ctx->dtime);
  counted();
  cudaEventRecord(ctx->ev_lists, sf);

  // chain partition: the interface loop
  cudaStreamWaitEvent(ctx->s_chain, ctx->ev_fork, 0);
  k_ifc_reset<<<grid_blocks(cap, 256), 256, 0, ctx->s_chain>>>(ctx->ifc_done, ctx->ifc_out, cap,
                                                               (unsigned int*)(ctx->ifc_opp),
                                                               ctx->dtime);
  counted();
  IfcArgs ia;
  ia.P = P;
  ia.W1 = ctx->W[0]; ia.W2 = ctx->W[1];
  ia.phi = ctx->phi; ia.nrm = ctx->nrm; ia.mask = ctx->mask;
  ia.list = ctx->ifc_list; ia.ifc_map = ctx->ifc_map;
  ia.done = ctx->ifc_done; ia.out = ctx->ifc_out;
  ia.ticket = (unsigned int*)(ctx->ifc_opp);
  ia.D = ctx->dtime;
  ia.spin_limit = ctx->ifc_spin_limit > 0 ? ctx->ifc_spin_limit : IFC_SPIN_LIMIT;
  ia.withhold = ctx->ifc_withhold - 1;
  ia.slip = m->use_slip_BCs;
  set_learning(ctx, ia, ctx->s_chain);
  ia.probe_ij = nullptr; ia.probe_w = nullptr; ia.probe_dep = nullptr;
  if (variant == GFM_RIEMANN) {
    k_ifc_probes<<<16, 256, 0, ctx->s_chain>>>(ia, ctx->probe_ij, ctx->probe_w, ctx->probe_dep); counted();
    ia.probe_ij = ctx->probe_ij; ia.probe_w = ctx->probe_w; ia.probe_dep = ctx->probe_dep;
  }
  const int chain_ctas = ctx->chain_ctas;   // 8 warps each
  if (variant == GFM_RIEMANN) k_interface_warp<IFC_RIEMANN><<<chain_ctas, 256, 0, ctx->s_chain>>>(ia);
  else k_interface_warp<IFC_REAL><<<chain_ctas, 256, 0, ctx->s_chain>>>(ia);
  counted();
  k_ifc_vel<<<chain_ctas, 256, 0, ctx->s_chain>>>(P, ctx->ifc_list, ctx->ifc_out, ctx->vel, ctx->dtime);
  counted();
  cudaEventRecord(ctx->ev_chain, ctx->s_chain);
  if (ctx->timing) cudaEventRecord(ctx->tev[1], ctx->s_chain);

  // far partition: extrapolation without the interface loop's writes,
  // conserved grids of far cells, flux update of far tiles
  {
    const double* src1 = ctx->W[0];
    const double* src2 = ctx->W[1];
    // each of the first five sweeps into its own buffer (the exact sweeps
    // read them); the sixth converts the far cells to conserved grids
    for (int it = 0; it < 6; it++) {
      double** dst = ctx->SF[it < 5 ? it : 4];   // not written by the sixth
      extrap_sweep(ctx, src1, src2, dst[0], dst[1], false, ctx->s_far, nullptr, nullptr, 0, nullptr, 0,
                   it == 5 ? 1 : 0);
      src1 = dst[0]; src2 = dst[1];
    }
  }
  cudaEventRecord(ctx->ev_far_final, ctx->s_far);
  if (ctx->timing) cudaEventRecord(ctx->tev[5], ctx->s_far);
  launch_fs_update_sel(ctx, m->fs, 3, TILES_FAR, ctx->s_far);
  cudaEventRecord(ctx->ev_far, ctx->s_far);
  if (ctx->timing) cudaEventRecord(ctx->tev[2], ctx->s_far);
  if (ctx->part_ev[2]) cudaEventRecord(ctx->part_ev[2], ctx->s_far);

  // after the chain, on the highest-priority stream: the true extrapolation
  // (the loop's writes overlaid on the first sweep's reads), conserved grids
  // of near cells, flux update of near tiles
  cudaStream_t sn = ctx->s_near;
  cudaStreamWaitEvent(sn, ctx->ev_chain, 0);
  cudaStreamWaitEvent(sn, ctx->ev_far_final, 0);   // band lists and the far field's sweeps
  {
    double* bufA[2] = {ctx->Wt[0], ctx->Wt[1]};
    double* bufB[2] = {ctx->Wc[0], ctx->Wc[1]};
    const double* src1 = ctx->W[0];
    const double* src2 = ctx->W[1];
    for (int it = 0; it < 6; it++) {
      double** dst = (it & 1) ? bufB : bufA;
      // sweep k = it + 1 writes the cells within k of an interfacial cell
      // (segments 0..k); sweep 1 reads the pre-loop primitives with the loop's
      // writes overlaid, sweep k > 1 the exact sweep k - 1 within k - 1
      // (cls >= NEAR_RADIUS + 2 - k) and the far field's sweep k - 1 beyond
      // the sixth converts the near cells to conserved grids
      const double* far[2] = {it ? ctx->SF[it - 1][0] : nullptr, it ? ctx->SF[it - 1][1] : nullptr};
      extrap_sweep(ctx, src1, src2, dst[0], dst[1], it == 0, sn, ctx->band_list, ctx->list_n, it + 2,
                   it ? far : nullptr, NEAR_RADIUS + 1 - it, it == 5 ? 2 : 0);
      src1 = dst[0]; src2 = dst[1];
    }
  }
  if (ctx->timing) cudaEventRecord(ctx->tev[3], sn);
  if (ctx->part_ev[1]) cudaEventRecord(ctx->part_ev[1], sn);
  // The near tiles read far cells too: the far cells' conversion is done (the
  // far tiles' flux update writes only its own tiles of Unew).  From here on
  // nothing in the ghost fill reads phi.
  cudaEventRecord(ctx->ev_phi_free, sn);
  if (ctx->timing) cudaEventRecord(ctx->tev[4], sn);
  // the caller issues the level set and the flux update of the near tiles
  // (on s_near) and joins s_near and the far stream back into ctx->stream
}

// The level set of one step: the advection stages (part 1) read phi and the
// velocity field and write phi_a / phi_b, the last of them, on a step that
// reinitialises, also the sign function S; then (part 2) phi := phi_a, or on
// a reinitialisation step the Sussman iterations starting from phi_a
// (phi_a -> phi -> phi_a ...; an even count ends with a copy into phi).
// every: -1 no reinitialisation this step, 0 one this step (decided on the
// host), k >= 1 decided on the device (a step recorded into a graph).
static int ls_reinit_every(const gfm_ctx* ctx, const gfm_method_desc* m) {
  if (m->reinit_every <= 0 || m->reinit_iters <= 0) return -1;
  if (ctx->graph_mode) return m->reinit_every;
  return ((ctx->steps_done_host + 1) % m->reinit_every == 0) ? 0 : -1;
}

void launch_level_set(gfm_ctx* ctx, const gfm_method_desc* m, cudaStream_t s, int parts, cudaEvent_t phi_free) {
  const GridP& P = ctx->P;
  const int64_t n = padded_cells(P);
  const int every = ls_reinit_every(ctx, m);
  double* S = every >= 0 ? ctx->phi0 : nullptr;
  const int ev = every > 0 ? every : 0;
  if (parts & 1) {
    // the stage kernels have one occupancy
    const int blocks = wave_blocks((const void*)k_ls_stage<5, 1>, 256, ctx->num_sms, n);
    if (m->ls_order == 1) {
      k_ls_stage<1, 1><<<blocks, 256, 0, s>>>(P, ctx->phi, ctx->phi, ctx->phi_a, ctx->vel, ctx->dtime, S, ev);
      counted();
    } else {
      k_ls_stage<5, 1><<<blocks, 256, 0, s>>>(P, ctx->phi, ctx->phi, ctx->phi_a, ctx->vel, ctx->dtime, nullptr, 0);
      k_ls_stage<5, 2><<<blocks, 256, 0, s>>>(P, ctx->phi_a, ctx->phi, ctx->phi_b, ctx->vel, ctx->dtime, nullptr, 0);
      k_ls_stage<5, 3><<<blocks, 256, 0, s>>>(P, ctx->phi_b, ctx->phi, ctx->phi_a, ctx->vel, ctx->dtime, S, ev);
      counted(3);
    }
  }
  if (parts & 2) {
    // The advected field is in phi_a.  Only the last write lands in phi, after
    // phi_free (the ghost fill's last read of phi) when given: the
    // reinitialisation's earlier iterations alternate between phi_b (free
    // once the stages have run) and phi_a.
    const int cblocks = wave_blocks((const void*)k_copy_plane, 256, ctx->num_sms, n);
    const int iters = every >= 0 ? m->reinit_iters : 0;
    const int blocks = wave_blocks((const void*)k_reinit_iter, 256, ctx->num_sms, n);
    const double* src = ctx->phi_a;
    for (int it = 0; it + 1 < iters; it++) {
      double* dst = (it & 1) ? ctx->phi_a : ctx->phi_b;
      k_reinit_iter<<<blocks, 256, 0, s>>>(P, src, ctx->phi0, dst, ctx->dtime, ev); counted();
      src = dst;
    }
    if (phi_free) cudaStreamWaitEvent(s, phi_free, 0);
    if (every < 0) {              // no reinitialisation: phi := phi_a
      k_copy_plane<<<cblocks, 256, 0, s>>>(P, ctx->phi_a, ctx->phi, ctx->dtime, 0, 0); counted();
    } else {
      // phi := phi_a on the steps that skip the reinitialisation
      if (every > 1) { k_copy_plane<<<cblocks, 256, 0, s>>>(P, ctx->phi_a, ctx->phi, ctx->dtime, every, 1); counted(); }
      if (iters > 0) {
        k_reinit_iter<<<blocks, 256, 0, s>>>(P, src, ctx->phi0, ctx->phi, ctx->dtime, ev); counted();
      } else {
        k_copy_plane<<<cblocks, 256, 0, s>>>(P, ctx->phi_a, ctx->phi, ctx->dtime, ev, 0); counted();
      }
    }
  }
}

// Occupancy queries of the grid-stride kernels, made once before any launch
// (and so before any stream capture records one)
void prepare_step_kernels() {
  static std::once_flag once;
  std::call_once(once, [] {
    const void* ks[] = {(const void*)k_commit_u, (const void*)k_extrap<false>, (const void*)k_extrap<true>,
                        (const void*)k_finalize,
                        (const void*)k_ls_stage<5, 1>, (const void*)k_copy_plane, (const void*)k_reinit_iter};
    for (const void* k : ks) wave_blocks(k, 256, 1, 1);
  });
}

// GFM_VOF / OGFM_VOF set_ghost_states: prims, mixed cells and their
// reconstruction, the mixed-cell loop, ghost states + conserved grids +
// velocity field, apply_BCs_euler on both grids.
void launch_ghost_fill_vof(gfm_ctx* ctx, const gfm_method_desc* m) {
  const GridP& P = ctx->P;
  cudaStream_t s = ctx->stream;
  const bool og = m->gfm == GFM_OGFM_VOF;
  VofPrimArgs pa;
  pa.P = P;
  pa.U1 = ctx->U[0]; pa.U2 = ctx->U[1];
  pa.W1 = ctx->W[0]; pa.W2 = ctx->W[1];
  pa.z = ctx->phi; pa.nrm = ctx->nrm; pa.mask = ctx->mask; pa.ifc_map = ctx->ifc_map;
  pa.chunk_count = ctx->chunk_count; pa.chunk = ctx->chunk; pa.D = ctx->dtime;
  pa.ogfm = og ? 1 : 0;
  k_vof_prims<<<ctx->n_chunks, CHUNK_T, 0, s>>>(pa); counted();
  if (og) { k_rc_clamp<<<1, 1, 0, s>>>(P, ctx->dtime); counted(); }
  k_compact<<<ctx->n_chunks, CHUNK_T, 0, s>>>(P, ctx->mask, ctx->chunk_count, ctx->n_chunks, ctx->chunk, ctx->ifc_list,
                                              ctx->ifc_map, ctx->dtime); counted();
  const int cap = P.nr * P.nc;
  k_ifc_reset<<<grid_blocks(cap, 256), 256, 0, s>>>(ctx->ifc_done, nullptr, cap, (unsigned int*)(ctx->ifc_opp),
                                                     ctx->dtime);
  counted();
  // the real cells flagged 1 or 2 by the loop: within the ring of a mixed cell
  cudaMemsetAsync(ctx->near_cell, 0, (size_t)P.plane, s);
  k_near_mark<<<grid_blocks((int64_t)P.Nx * P.Ny, 256), 256, 0, s>>>(P, ctx->ifc_list, ctx->dtime, ctx->near_cell,
                                                                      VOF_RING);
  counted();
  IfcArgs ia;
  ia.P = P;
  ia.W1 = ctx->W[0]; ia.W2 = ctx->W[1];
  ia.phi = ctx->phi; ia.nrm = ctx->nrm; ia.mask = ctx->mask;
  ia.list = ctx->ifc_list; ia.ifc_map = ctx->ifc_map;
  ia.done = ctx->ifc_done; ia.out = ctx->ifc_out;
  ia.ticket = (unsigned int*)(ctx->ifc_opp);
  ia.D = ctx->dtime;
  ia.spin_limit = ctx->ifc_spin_limit > 0 ? ctx->ifc_spin_limit : IFC_SPIN_LIMIT;
  ia.withhold = ctx->ifc_withhold - 1;
  ia.slip = m->use_slip_BCs;
  ia.mlp = nullptr; ia.mlp_frag = nullptr; ia.cap_X = nullptr; ia.cap_Y = nullptr; ia.cap_count = nullptr; ia.cap = 0;
  ia.probe_ij = nullptr; ia.probe_w = nullptr; ia.probe_dep = nullptr;
  if (og) k_vof_chain<VOF_OGFM><<<152, 128, 0, s>>>(ia, ctx->ifc_mrp);
  else k_vof_chain<VOF_GFM><<<152, 128, 0, s>>>(ia, ctx->ifc_mrp);
  counted();
  VofGhostArgs ga;
  ga.P = P;
  ga.W1 = ctx->W[0]; ga.W2 = ctx->W[1];
  ga.z = ctx->phi; ga.mask = ctx->mask; ga.ifc_map = ctx->ifc_map;
  ga.out = ctx->ifc_out; ga.mrp = ctx->ifc_mrp;
  ga.near_cell = ctx->near_cell;
  ga.U1 = ctx->U[0]; ga.U2 = ctx->U[1];
  ga.vel = ctx->vel; ga.D = ctx->dtime;
  const int gblocks = grid_blocks((int64_t)P.nr * P.nc, 256);
  if (og) k_vof_ghost<VOF_OGFM><<<gblocks, 256, 0, s>>>(ga);
  else k_vof_ghost<VOF_GFM><<<gblocks, 256, 0, s>>>(ga);
  counted();
  launch_bcs(ctx, 3);
}

// VOF update_interface_coupled: z0 := z, then two directional sweeps
// z -> phi_a -> z on stream s
void launch_vof_update(gfm_ctx* ctx, cudaStream_t s) {
  const GridP& P = ctx->P;
  const int blocks = grid_blocks((int64_t)P.nr * P.nc, 256);
  k_copy_plane<<<blocks, 256, 0, s>>>(P, ctx->phi, ctx->phi0, ctx->dtime, 0, 0); counted();
  k_vof_sweep<<<blocks, 256, 0, s>>>(P, ctx->phi, ctx->phi0, ctx->vel, ctx->phi_a, 0, ctx->dtime); counted();
  k_vof_sweep<<<blocks, 256, 0, s>>>(P, ctx->phi_a, ctx->phi0, ctx->vel, ctx->phi, 1, ctx->dtime); counted();
}

void launch_end_step(gfm_ctx* ctx) {
  k_end_step<<<1, 1, 0, ctx->stream>>>(ctx->dtime);
  counted();
}

void launch_mass(gfm_ctx* ctx, double sign, double* part, double* out) {
  const GridP& P = ctx->P;
  int nb = 256;
  k_mass_partial<<<nb, 256, 0, ctx->stream>>>(P, sign < 0.0 ? ctx->U[0] : ctx->U[ctx->two_fluid ? 1 : 0],
                                               ctx->two_fluid ? ctx->phi : nullptr,
                                               (ctx->two_fluid && ctx->itm == GFM_ITM_VOF) ? 1 : 0, sign, part);
  counted();
  k_mass_final<<<1, 32, 0, ctx->stream>>>(part, nb, out); counted();
}

}  // namespace gfm
