// Fused flux update of one fluid over its realcells box:
// FS_MUSCL::pure_fluid_update (sourcecode/FS_MUSCL.cpp:148-304) and
// FS_godunov::pure_fluid_update (sourcecode/FS_godunov.cpp:5-50).
//
// One CTA owns a TX x TY tile of real cells.
//   phase 1  conserved -> primitive once per cell of the tile + 2-cell halo,
//            into shared memory (the reference converts each neighbour again
//            for every face it touches; the values are identical).
//   phase 2  per cell: minmod slopes, boundary-extrapolated values, the
//            physicality fallback and the half-step evolution, giving the
//            four evolved face states of the cell (shared memory).  The
//            reference recomputes these per face (as cell C, L or B); each
//            cell's values do not depend on which face asks for them.
//   phase 3  per face: the second fallback, primitives -> conserved, and the
//            exact Riemann flux (pure_RS_exact::solve_RP).  Up to the
//            no-wave test the faces run one per thread; then the faces with
//            waves and those without are queued apart and finished by
//            consecutive threads, so that the Newton iterations run with few
//            idle lanes and no warp runs both kinds.
//   phase 4  per cell: U + (dt/dx Fw + dt/dy Fs) - dt/dx Fe - dt/dy Fn, the
//            accumulation order of the reference's face loop (:290-292).
//
// Built with GFM_FLUX_INT_MUL defined, the kernel's products (mulx) are
// formed in integer arithmetic (xmul, gfm_xfp64.cuh: the same bits) instead
// of on the FP64 pipe.  Off by default: measured on the 1000 x 400
// shock-bubble, the launch takes 2.19 ms that way against 1.69 ms with FP64
// multiplies -- each integer product costs about 77 issue cycles of the
// integer pipes, which this kernel already loads, against the 64-cycle FP64
// slot it frees, and its 4 warps per sub-partition do not hide the 208-cycle
// latency.
#ifdef GFM_FLUX_INT_MUL
#define GFM_INT_MUL 1
#endif
#include "gfm_internal.cuh"
#include <cstring>
#include <mutex>

namespace gfm {

// Tile shape TX x TY: the shared-memory regions of one tile, and its CTA's
// threads (NT).  The default 16 x 32 (FLUX_TX x FLUX_TY) is the one the
// overlapped schedule's tile marking assumes, with 512 threads and one CTA
// per SM; 16 x 16, 32 x 8 and 64 x 4 (256 threads, two CTAs per SM) are the
// autotuner's alternatives.
template <int TX, int TY>
struct FluxShape {
  static constexpr int NT = TX * TY >= 512 ? 512 : 256;
  static constexpr int MIN_CTAS = NT == 512 ? 1 : 2;   // resident per SM (launch bounds)
  static constexpr int WR = TY + 4;   // primitive region rows   (i0-2 .. i0+TY+1)
  static constexpr int WC = TX + 4;   // primitive region columns (j0-2 .. j0+TX+1)
  static constexpr int SR = TY + 2;   // face-state cells rows    (i0-1 .. i0+TY)
  static constexpr int SC = TX + 2;   // face-state cells columns (j0-1 .. j0+TX)
  static constexpr int NXF = TY * (TX + 1);
  static constexpr int NYF = (TY + 1) * TX;
  struct Smem {
    double w[4][WR][WC];          // primitives (MUSCL) or conserved (Godunov)
    double irho[WR][WC];          // MUSCL: 1/rho of the conversion, reused by the cell's face states
    double fs[4][4][SR][SC];      // [face L,R,B,T][component][r][c]
    double fx[4][TY][TX + 1];
    double fy[4][TY + 1][TX];
    double qd[6][NXF + NYF];      // queued faces: uR, pR, utL, utR, irhoL, irhoR (rhoL, uL, pL, rhoR sit in the flux slot)
    unsigned short qid[NXF + NYF];
  };
};

struct FluxArgs {
  GridP P;
  const double* U[2];
  double* Unew[2];
  const DevTime* dtime;
  DevTime* dtime_w;
  int fluid_base;
  const int* tile_near;   // per tile: region holds a cell near the interface
  int tiles;              // TILES_ALL, TILES_FAR or TILES_NEAR
};

template <class S>
__device__ __forceinline__ V4 sW(const S& s, int r, int c) {
  return V4{s.w[0][r][c], s.w[1][r][c], s.w[2][r][c], s.w[3][r][c]};
}
template <class S>
__device__ __forceinline__ V4 sFS(const S& s, int f, int r, int c) {
  return V4{s.fs[f][0][r][c], s.fs[f][1][r][c], s.fs[f][2][r][c], s.fs[f][3][r][c]};
}
template <class S>
__device__ __forceinline__ void putFS(S& s, int f, int r, int c, const V4& v) {
  s.fs[f][0][r][c] = v.a; s.fs[f][1][r][c] = v.b; s.fs[f][2][r][c] = v.c; s.fs[f][3][r][c] = v.d;
}
__device__ __forceinline__ V4 v4sub(const V4& x, const V4& y) { return V4{x.a - y.a, x.b - y.b, x.c - y.c, x.d - y.d}; }

// (s A(W)) d, quasilinear_form_A (headers/euler_misc.hpp:149-163), non-zero
// terms; irho = 1/rho and rcc = rho c c are the matrix entries A(1,3), A(3,1).
__device__ __forceinline__ V4 A_times(double s, const V4& W, double irho, double rcc, const V4& d) {
  double su = mulx(s, W.b);
  return V4{mulx(su, d.a) + mulx(mulx(s, W.a), d.b), mulx(su, d.b) + mulx(mulx(s, irho), d.d), mulx(su, d.c),
            mulx(mulx(s, rcc), d.b) + mulx(su, d.d)};
}
// (s B(W)) d, quasilinear_form_B (headers/euler_misc.hpp:166-180)
__device__ __forceinline__ V4 B_times(double s, const V4& W, double irho, double rcc, const V4& d) {
  double sv = mulx(s, W.c);
  return V4{mulx(sv, d.a) + mulx(mulx(s, W.a), d.c), mulx(sv, d.b), mulx(sv, d.c) + mulx(mulx(s, irho), d.d),
            mulx(mulx(s, rcc), d.c) + mulx(sv, d.d)};
}

// Phase 2 for one cell: minmod slopes (FS_MUSCL.cpp:189-196), boundary
// extrapolated values (:199-210), first physicality fallback (:213-247) and
// the half-step evolution with both quasilinear matrices (:250-272).
// out = evolved L, R, B, T face states of the cell.
__device__ __forceinline__ void cell_face_states(const V4& W, double irho_W, const V4& Ww, const V4& We,
                                                 const V4& Ws, const V4& Wn, double gam, double pinf, double sx,
                                                 double sy, V4 out[4]) {
  V4 dxL = v4sub(W, Ww), dxR = v4sub(We, W);
  V4 dyL = v4sub(W, Ws), dyR = v4sub(Wn, W);
  V4 sxv = V4{minmod(dxL.a, dxR.a), minmod(dxL.b, dxR.b), minmod(dxL.c, dxR.c), minmod(dxL.d, dxR.d)};
  V4 syv = V4{minmod(dyL.a, dyR.a), minmod(dyL.b, dyR.b), minmod(dyL.c, dyR.c), minmod(dyL.d, dyR.d)};
  const V4 hx = V4{mulx(0.5, sxv.a), mulx(0.5, sxv.b), mulx(0.5, sxv.c), mulx(0.5, sxv.d)};
  const V4 hy = V4{mulx(0.5, syv.a), mulx(0.5, syv.b), mulx(0.5, syv.c), mulx(0.5, syv.d)};
  V4 L = V4{W.a - hx.a, W.b - hx.b, W.c - hx.c, W.d - hx.d};
  V4 R = V4{W.a + hx.a, W.b + hx.b, W.c + hx.c, W.d + hx.d};
  V4 B = V4{W.a - hy.a, W.b - hy.b, W.c - hy.c, W.d - hy.d};
  V4 T = V4{W.a + hy.a, W.b + hy.b, W.c + hy.c, W.d + hy.d};
  if (!is_physical_primitives_fast(gam, pinf, L) || !is_physical_primitives_fast(gam, pinf, R)) { L = W; R = W; }
  if (!is_physical_primitives_fast(gam, pinf, B) || !is_physical_primitives_fast(gam, pinf, T)) { B = W; T = W; }
  // 1/rho from the cell's conversion (the correctly rounded quotient, as
  // recip(W.a) would form it)
  Recip Rr;
  Rr.b = W.a; Rr.y = irho_W; Rr.fast = mid_range(W.a);
  double cs = eos_soundspeed_r(gam, pinf, W.d, Rr);
  double irho = Rr.y, rcc = mulx(mulx(W.a, cs), cs);   // irho = 1.0 / W.a
  V4 X = A_times(sx, W, irho, rcc, v4sub(L, R));
  V4 Y = B_times(sy, W, irho, rcc, v4sub(B, T));
  out[0] = V4{(L.a + X.a) + Y.a, (L.b + X.b) + Y.b, (L.c + X.c) + Y.c, (L.d + X.d) + Y.d};
  out[1] = V4{(R.a + X.a) + Y.a, (R.b + X.b) + Y.b, (R.c + X.c) + Y.c, (R.d + X.d) + Y.d};
  out[2] = V4{(B.a + X.a) + Y.a, (B.b + X.b) + Y.b, (B.c + X.c) + Y.c, (B.d + X.d) + Y.d};
  out[3] = V4{(T.a + X.a) + Y.a, (T.b + X.b) + Y.b, (T.c + X.c) + Y.c, (T.d + X.d) + Y.d};
}

// Phase 3 for one face (MUSCL): second physicality fallback (FS_MUSCL.cpp:276-285)
// to the cells' primitives Wr/Wl and primitives -> conserved sharing e with
// the check; the exact Riemann flux (:287-288) follows.  Sr/Sl: evolved face
// states of the cell on the high / low side of the face.
__device__ __forceinline__ void muscl_face_cons(V4 Sr, V4 Sl, const V4& Wr, const V4& Wl, const Gas& gas,
                                                uint32_t* st, V4& UL, V4& UR) {
  const double gam = gas.g, pinf = gas.pinf;
  double er = eos_specific_ie(gam, pinf, Sr.d, Sr.a);
  double el = eos_specific_ie(gam, pinf, Sl.d, Sl.a);
  if (!(c_ge0(er) && c_ge0(Sr.a)) || !(c_ge0(el) && c_ge0(Sl.a))) {
    Sr = Wr;
    Sl = Wl;
    er = eos_specific_ie(gam, pinf, Sr.d, Sr.a);
    el = eos_specific_ie(gam, pinf, Sl.d, Sl.a);
  }
  if (!(c_ge0(Sl.a) && c_ge0(el)) || !(c_ge0(Sr.a) && c_ge0(er))) *st |= ST_UNPHYSICAL;
  UL = prims_to_cons_e(Sl, el);
  UR = prims_to_cons_e(Sr, er);
}

__device__ __forceinline__ V4 muscl_face_flux(bool xdir, V4 Sr, V4 Sl, const V4& Wr, const V4& Wl, const Gas& gas,
                                              uint32_t* st, int* iters) {
  V4 UL, UR;
  muscl_face_cons(Sr, Sl, Wr, Wl, gas, st, UL, UR);
  return pure_rs_flux(xdir, gas, UL, UR, st, iters);
}

// One tile (bx, by) of fluid slot bz of the grid a, whose tile rows are gx
// tiles wide, by the whole CTA (Sh::NT threads); the CTA's dynamic shared memory
// holds the tile's Smem.
template <bool MUSCL, int TX, int TY>
__device__ __forceinline__ void flux_tile(const FluxArgs& a, int bx, int by, int bz, int gx, unsigned char* smem_raw) {
  using Sh = FluxShape<TX, TY>;
  constexpr int WR = Sh::WR, WC = Sh::WC, SR = Sh::SR, SC = Sh::SC, NXF = Sh::NXF, NYF = Sh::NYF;
  typename Sh::Smem& s = *reinterpret_cast<typename Sh::Smem*>(smem_raw);
  __shared__ V4 s_uniform_flux[2];
  __shared__ int s_nq, s_nt;   // queued faces with waves and without (phase 3)
  const GridP& P = a.P;
  const int fluid = a.fluid_base + bz;
  const double* __restrict__ U = a.U[bz];
  double* __restrict__ Unew = a.Unew[bz];
  const Gas& gas = fluid == 0 ? P.gas1 : P.gas2;
  const double gam = gas.g;
  const double pinf = gas.pinf;
  const int i0 = P.g + by * TY;
  const int j0 = P.g + bx * TX;
  const int tid = threadIdx.x;
  const bool active = a.dtime->active != 0;
  const int* rc = &a.dtime->rc[4 * fluid];
  const int imin = rc[0], imax = rc[1], jmin = rc[2], jmax = rc[3];

  if (!active) return;   // the step after t reaches T changes nothing
  if (a.tiles != TILES_ALL) {
    const bool near = a.tile_near[by * gx + bx] != 0;
    if ((a.tiles == TILES_NEAR) != near) return;   // the other pass owns this tile
  }
  // tile outside the realcells box: its cells keep their values
  const bool tile_live = !(i0 + TY <= imin || i0 >= imax || j0 + TX <= jmin || j0 >= jmax);
  if (!tile_live) {
    for (int k = tid; k < TX * TY; k += Sh::NT) {
      int i = i0 + k / TX, j = j0 + k % TX;
      if (i < P.Ny + P.g && j < P.Nx + P.g) {
        int64_t c = cidx(P, i, j);
        for (int q = 0; q < 4; q++) Unew[c + q * P.plane] = U[c + q * P.plane];
      }
    }
    return;
  }
  const double dt = a.dtime->dt;
  const double dtodx = dt / P.dx;
  const double dtody = dt / P.dy;
  const double sx = 0.5 * dtodx, sy = 0.5 * dtody;
  uint32_t st = 0;
  int iters = 0;

  // phase 1: load (clamped to the padded grid), convert, and test whether the
  // whole region holds one bit pattern
  const int64_t c00 = cidx(P, min(max(i0 - 2, 0), P.nr - 1), min(max(j0 - 2, 0), P.nc - 1));
  const V4 u00 = load4(U, P, c00);
  if (tid == 0) { s_nq = 0; s_nt = 0; }
  bool same = true;
  for (int k = tid; k < WR * WC; k += Sh::NT) {
    int r = k / WC, c = k % WC;
    int i = min(max(i0 - 2 + r, 0), P.nr - 1);
    int j = min(max(j0 - 2 + c, 0), P.nc - 1);
    V4 u = load4(U, P, cidx(P, i, j));
    same = same && as_bits(u.a) == as_bits(u00.a) && as_bits(u.b) == as_bits(u00.b) &&
           as_bits(u.c) == as_bits(u00.c) && as_bits(u.d) == as_bits(u00.d);
    V4 w = u;
    if (MUSCL) {
      bool phys;
      Recip R;
      w = cons_to_prims_phys(gam, pinf, u, &phys, &R);   // cons_to_prims, and its 1/rho
      s.irho[r][c] = R.y;
    }
    s.w[0][r][c] = w.a; s.w[1][r][c] = w.b; s.w[2][r][c] = w.c; s.w[3][r][c] = w.d;
  }
  // Uniform region: every cell of the tile and its halo has the same state,
  // so every cell computes the same face states and every face of a
  // direction the same flux; one of each is evaluated (bit-identical).
  const bool uniform = __syncthreads_and(same) != 0;

  if (uniform) {
    // lane 0 forms the x faces' flux and lane 1 the y faces', side by side
    // in one instruction stream (both form the cell's face states)
    if (tid < 2) {
      const bool xd = tid == 0;
      V4 W = sW(s, 2, 2);
      V4 f;
      int it = 0;
      if (MUSCL) {
        V4 fs[4];
        cell_face_states(W, s.irho[2][2], W, W, W, W, gam, pinf, sx, sy, fs);
        f = muscl_face_flux(xd, xd ? fs[0] : fs[2], xd ? fs[1] : fs[3], W, W, gas, &st, &it);
      } else {
        f = pure_rs_flux(xd, gas, W, W, &st, &it);
      }
      iters = it * (xd ? NXF : NYF);
      s_uniform_flux[tid] = f;
    }
    __syncthreads();
  } else {
    // phase 2: evolved face states of cells (i0-1 .. i0+TY) x (j0-1 .. j0+TX)
    if (MUSCL) {
      for (int k = tid; k < SR * SC; k += Sh::NT) {
        int r = k / SC, c = k % SC;       // cell (i0-1+r, j0-1+c) = w[r+1][c+1]
        V4 fs[4];
        cell_face_states(sW(s, r + 1, c + 1), s.irho[r + 1][c + 1], sW(s, r + 1, c), sW(s, r + 1, c + 2),
                         sW(s, r, c + 1), sW(s, r + 2, c + 1), gam, pinf, sx, sy, fs);
        for (int f = 0; f < 4; f++) putFS(s, f, r, c, fs[f]);
      }
      __syncthreads();
    }
    // phase 3a: x faces (TY rows x TX+1) then y faces (TY+1 rows x TX) up to
    // the no-wave test, then queued by kind
    //   x face (fr, fc): between cells (i0+fr, j0+fc-1) and (i0+fr, j0+fc)
    //   y face (fr, fc): between cells (i0+fr-1, j0+fc) and (i0+fr, j0+fc)
    // Flux slot of face k, component m: fx[m] (flat) + k, or fy[m] + k - NXF.
    for (int k = tid; k < NXF + NYF; k += Sh::NT) {
      bool xdir = k < NXF;
      int fr, fc;
      if (xdir) { fr = k / (TX + 1); fc = k % (TX + 1); }
      else { int q = k - NXF; fr = q / TX; fc = q % TX; }
      V4 UL, UR;
      if (MUSCL) {
        if (xdir)
          muscl_face_cons(sFS(s, 0, fr + 1, fc + 1), sFS(s, 1, fr + 1, fc), sW(s, fr + 2, fc + 2),
                          sW(s, fr + 2, fc + 1), gas, &st, UL, UR);
        else
          muscl_face_cons(sFS(s, 2, fr + 1, fc + 1), sFS(s, 3, fr, fc + 1), sW(s, fr + 2, fc + 2),
                          sW(s, fr + 1, fc + 2), gas, &st, UL, UR);
      } else {
        if (xdir) { UL = sW(s, fr + 2, fc + 1); UR = sW(s, fr + 2, fc + 2); }
        else { UL = sW(s, fr + 1, fc + 2); UR = sW(s, fr + 2, fc + 2); }
      }
      FaceData d;
      const bool nowave = rs_face_front(xdir, gas, UL, UR, &st, d);
      double* slot = xdir ? &s.fx[0][0][0] + k : &s.fy[0][0][0] + (k - NXF);
      const int cs = xdir ? NXF : NYF;
      // every face is queued, those with waves from the front and those
      // without from the back, so that phase 3b runs each kind in whole warps
      const int e = nowave ? NXF + NYF - 1 - atomicAdd(&s_nt, 1) : atomicAdd(&s_nq, 1);
      s.qid[e] = (unsigned short)k;
      slot[0] = d.rhoL; slot[cs] = d.uL; slot[2 * cs] = d.pL; slot[3 * cs] = d.rhoR;
      s.qd[0][k] = d.uR; s.qd[1][k] = d.pR; s.qd[2][k] = d.utL; s.qd[3][k] = d.utR;
      s.qd[4][k] = d.irhoL; s.qd[5][k] = d.irhoR;
    }
    __syncthreads();
    // phase 3b: the queued faces, those with waves first
    const int nq = s_nq, nt = s_nt;
    for (int e = tid; e < nq + nt; e += Sh::NT) {
      const int k = s.qid[e < nq ? e : NXF + NYF - nt + (e - nq)];
      const bool xdir = k < NXF;
      double* slot = xdir ? &s.fx[0][0][0] + k : &s.fy[0][0][0] + (k - NXF);
      const int cs = xdir ? NXF : NYF;
      FaceData d;
      d.rhoL = slot[0]; d.uL = slot[cs]; d.pL = slot[2 * cs]; d.rhoR = slot[3 * cs];
      d.uR = s.qd[0][k]; d.pR = s.qd[1][k]; d.utL = s.qd[2][k]; d.utR = s.qd[3][k];
      d.irhoL = s.qd[4][k]; d.irhoR = s.qd[5][k];
      V4 f = rs_face_finish(xdir, gas, d, &st, &iters);
      slot[0] = f.a; slot[cs] = f.b; slot[2 * cs] = f.c; slot[3 * cs] = f.d;
    }
    __syncthreads();
  }

  // phase 4: U + (dt/dx Fw + dt/dy Fs) - dt/dx Fe - dt/dy Fn
  const V4 ufx = s_uniform_flux[0], ufy = s_uniform_flux[1];
  for (int k = tid; k < TX * TY; k += Sh::NT) {
    int r = k / TX, c = k % TX;
    int i = i0 + r, j = j0 + c;
    if (i >= P.Ny + P.g || j >= P.Nx + P.g) continue;
    int64_t ci = cidx(P, i, j);
    V4 u = load4(U, P, ci);
    if (i >= imin && i < imax && j >= jmin && j < jmax) {
      if (!is_physical_state_fast(u)) st |= ST_UNPHYSICAL;
      double o[4] = {u.a, u.b, u.c, u.d};
      const double ux[4] = {ufx.a, ufx.b, ufx.c, ufx.d}, uy[4] = {ufy.a, ufy.b, ufy.c, ufy.d};
      for (int q = 0; q < 4; q++) {
        double fw = uniform ? ux[q] : s.fx[q][r][c];
        double fe = uniform ? ux[q] : s.fx[q][r][c + 1];
        double fs_ = uniform ? uy[q] : s.fy[q][r][c];
        double fn = uniform ? uy[q] : s.fy[q][r + 1][c];
        double v = o[q] + (mulx(dtodx, fw) + mulx(dtody, fs_));
        v = v - mulx(dtodx, fe);
        v = v - mulx(dtody, fn);
        o[q] = v;
      }
      u = V4{o[0], o[1], o[2], o[3]};
    }
    store4(Unew, P, ci, u);
  }

  // status and Newton statistics, one atomic per warp
  uint32_t wst = __reduce_or_sync(0xffffffffu, st);
  unsigned wit = __reduce_add_sync(0xffffffffu, (unsigned)iters);
  if ((tid & 31) == 0) {
    if (wst) atomicOr(&a.dtime_w->status, wst);
    if (wit) atomicAdd(&a.dtime_w->newton_iters, (unsigned long long)wit);
  }
}

template <bool MUSCL, int TX, int TY>
__global__ void __launch_bounds__(FluxShape<TX, TY>::NT, FluxShape<TX, TY>::MIN_CTAS) k_flux_update(FluxArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  flux_tile<MUSCL, TX, TY>(a, blockIdx.x, blockIdx.y, blockIdx.z, gridDim.x, smem_raw);
}

// The flux update of many grids in one persistent launch (a batch's phased
// schedule): each CTA takes (instance, fluid, tile) work items in list order
// from a counter -- the list holds the costliest instances first, so the
// uneven grids finish together -- copies the instance's arguments into
// shared memory and runs the tile.  The last CTA to finish resets the
// counters for the next launch (stream-ordered, so a replayed graph finds
// them at zero).  Item: instance << 24 | fluid slot << 23 | tile.
template <bool MUSCL, int TX, int TY>
__global__ void __launch_bounds__(FluxShape<TX, TY>::NT, FluxShape<TX, TY>::MIN_CTAS)
    k_flux_batch(const FluxArgs* __restrict__ args,
                                                       const uint32_t* __restrict__ items, int n_items,
                                                       unsigned int* counters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ FluxArgs s_args;
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(&counters[0], 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) break;
    const uint32_t w = items[it];
    const int inst = (int)(w >> 24), bz = (int)((w >> 23) & 1u), tile = (int)(w & 0x7fffffu);
    {
      const int* src = reinterpret_cast<const int*>(args + inst);
      int* dst = reinterpret_cast<int*>(&s_args);
      for (int q = threadIdx.x; q < (int)(sizeof(FluxArgs) / sizeof(int)); q += FluxShape<TX, TY>::NT) dst[q] = src[q];
    }
    __syncthreads();
    const int gx = (s_args.P.Nx + TX - 1) / TX;
    flux_tile<MUSCL, TX, TY>(s_args, tile % gx, tile / gx, bz, gx, smem_raw);
    __syncthreads();   // the next item reuses the shared memory
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&counters[1], 1u) == gridDim.x - 1) {
      counters[0] = 0u;
      counters[1] = 0u;
      __threadfence();
    }
  }
}

template <int TX, int TY>
static size_t flux_smem() { return sizeof(typename FluxShape<TX, TY>::Smem); }

// the tile shapes a flux update can take (FLUX_SHAPE_*)
template <bool MUSCL, int TX, int TY>
static void set_shape_attributes() {
  cudaFuncSetAttribute(k_flux_update<MUSCL, TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)flux_smem<TX, TY>());
  cudaFuncSetAttribute(k_flux_batch<MUSCL, TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)flux_smem<TX, TY>());
}
template <bool MUSCL>
static void set_flux_attributes() {
  set_shape_attributes<MUSCL, 32, 8>();
  set_shape_attributes<MUSCL, 16, 16>();
  set_shape_attributes<MUSCL, 64, 4>();
  set_shape_attributes<MUSCL, 16, 32>();
}

// Kernel attributes, set once per process before any launch (and so before
// any stream capture).
void prepare_kernels() {
  static std::once_flag once;
  std::call_once(once, [] {
    set_flux_attributes<true>();
    set_flux_attributes<false>();
  });
  prepare_step_kernels();
}

int flux_tile_w(int shape) {
  return (shape == FLUX_SHAPE_16x16 || shape == FLUX_SHAPE_16x32) ? 16 : (shape == FLUX_SHAPE_64x4 ? 64 : 32);
}
int flux_tile_h(int shape) {
  return shape == FLUX_SHAPE_16x16 ? 16 : (shape == FLUX_SHAPE_16x32 ? 32 : (shape == FLUX_SHAPE_64x4 ? 4 : 8));
}

template <int TX, int TY>
static void update_shape(bool muscl, dim3 grid, const FluxArgs& a, cudaStream_t stream) {
  constexpr int nt = FluxShape<TX, TY>::NT;
  if (muscl) k_flux_update<true, TX, TY><<<grid, nt, flux_smem<TX, TY>(), stream>>>(a);
  else k_flux_update<false, TX, TY><<<grid, nt, flux_smem<TX, TY>(), stream>>>(a);
}
template <int TX, int TY>
static void batch_shape(bool muscl, int ctas, const FluxArgs* A, const uint32_t* items, int n_items,
                        unsigned int* counters, cudaStream_t stream) {
  constexpr int nt = FluxShape<TX, TY>::NT;
  if (muscl) k_flux_batch<true, TX, TY><<<ctas, nt, flux_smem<TX, TY>(), stream>>>(A, items, n_items, counters);
  else k_flux_batch<false, TX, TY><<<ctas, nt, flux_smem<TX, TY>(), stream>>>(A, items, n_items, counters);
}
template <int TX, int TY>
static int batch_occupancy(bool muscl) {
  int per = 0;
  const void* k = muscl ? (const void*)k_flux_batch<true, TX, TY> : (const void*)k_flux_batch<false, TX, TY>;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, FluxShape<TX, TY>::NT, flux_smem<TX, TY>()) !=
          cudaSuccess ||
      per < 1) {
    cudaGetLastError();
    per = 1;
  }
  return per;
}

void launch_fs_update(gfm_ctx* ctx, int fs, int fluid_mask) {
  launch_fs_update_sel(ctx, fs, fluid_mask, TILES_ALL, ctx->stream);
}

void launch_fs_update_sel(gfm_ctx* ctx, int fs, int fluid_mask, int tiles, cudaStream_t stream) {
  const GridP& P = ctx->P;
  FluxArgs a;
  a.P = P;
  a.dtime = ctx->dtime;
  a.dtime_w = ctx->dtime;
  a.tile_near = ctx->tile_near;
  a.tiles = tiles;
  int nz = 0;
  a.fluid_base = (fluid_mask & 1) ? 0 : 1;
  for (int f = 0; f < 2; f++) {
    if (!(fluid_mask & (1 << f))) continue;
    a.U[nz] = ctx->U[f];
    a.Unew[nz] = ctx->Unew[f];
    nz++;
  }
  prepare_kernels();
  // the overlapped schedule's passes use the tile grid its marking assumes
  const int shape = tiles == TILES_ALL ? ctx->flux_shape : FLUX_SHAPE_DEFAULT;
  const int tw = flux_tile_w(shape), th = flux_tile_h(shape);
  dim3 grid((P.Nx + tw - 1) / tw, (P.Ny + th - 1) / th, nz);
  const bool mu = fs == GFM_FS_MUSCL;
  if (shape == FLUX_SHAPE_16x32) update_shape<16, 32>(mu, grid, a, stream);
  else if (shape == FLUX_SHAPE_16x16) update_shape<16, 16>(mu, grid, a, stream);
  else if (shape == FLUX_SHAPE_64x4) update_shape<64, 4>(mu, grid, a, stream);
  else update_shape<32, 8>(mu, grid, a, stream);
  counted();
  // the new values are in Unew; launch_commit copies them (with the BCs) to U
}

// The arguments of one instance's flux update of both fluids (the work
// items of k_flux_batch carry the fluid slot).
void flux_batch_args(const gfm_ctx* ctx, void* out) {
  FluxArgs a;
  memset(&a, 0, sizeof(a));
  a.P = ctx->P;
  a.dtime = ctx->dtime;
  a.dtime_w = ctx->dtime;
  a.tile_near = nullptr;
  a.tiles = TILES_ALL;
  a.fluid_base = 0;
  const int nf = ctx->two_fluid ? 2 : 1;
  for (int f = 0; f < nf; f++) {
    a.U[f] = ctx->U[f];
    a.Unew[f] = ctx->Unew[f];
  }
  memcpy(out, &a, sizeof(a));
}
size_t flux_batch_args_size() { return sizeof(FluxArgs); }

void launch_flux_batch(int fs, int shape, const void* args, const uint32_t* items, int n_items,
                       unsigned int* counters, int ctas, cudaStream_t stream) {
  prepare_kernels();
  const bool mu = fs == GFM_FS_MUSCL;
  const FluxArgs* A = static_cast<const FluxArgs*>(args);
  if (shape == FLUX_SHAPE_16x32) batch_shape<16, 32>(mu, ctas, A, items, n_items, counters, stream);
  else if (shape == FLUX_SHAPE_16x16) batch_shape<16, 16>(mu, ctas, A, items, n_items, counters, stream);
  else if (shape == FLUX_SHAPE_64x4) batch_shape<64, 4>(mu, ctas, A, items, n_items, counters, stream);
  else batch_shape<32, 8>(mu, ctas, A, items, n_items, counters, stream);
  counted();
}

// resident CTAs per SM of the batched flux kernel of a shape
int flux_batch_occupancy(int fs, int shape) {
  prepare_kernels();
  const bool mu = fs == GFM_FS_MUSCL;
  if (shape == FLUX_SHAPE_16x32) return batch_occupancy<16, 32>(mu);
  if (shape == FLUX_SHAPE_16x16) return batch_occupancy<16, 16>(mu);
  if (shape == FLUX_SHAPE_64x4) return batch_occupancy<64, 4>(mu);
  return batch_occupancy<32, 8>(mu);
}

}  // namespace gfm
