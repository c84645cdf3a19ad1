// Initial conditions generated on the device: the named cases of
// set_sim_ICs (sourcecode/sim_twofluid.cpp:599-1799,
// sourcecode/sim_onefluid.cpp:196-449) and the shock-bubble family of the
// batched workload, written straight into a context's grids with the per-cell
// definitions the host set-up uses (gfm_cases.cuh), so large batched sweeps
// need no host-side set-up or upload.  Results equal the host set-up bit for
// bit, except GDA's Gaussian density, whose exp is the C library's on the
// host and gfm_exp here (within 1 ulp).
#include <cstring>
#include <string>

#include "gfm_cases.cuh"
#include "gfm_internal.cuh"
#include "../../include/gfm_gb300.h"

namespace gfm {

bool make_case_spec(const char* sim_type, const char* test_case, const gfm_grid_desc* d, CaseSpec* out);
bool make_bubble_spec(const gfm_bubble_params* p, const gfm_grid_desc* d, CaseSpec* out);

__global__ void __launch_bounds__(256) k_case_init(CaseSpec s, CaseGeo G, GridP P, double* U1, double* U2,
                                                   double* field, int two, int want_z) {
  const int64_t n = (int64_t)P.nr * P.nc;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / P.nc), j = (int)(k % P.nc);
    V4 u1, u2 = V4{0.0, 0.0, 0.0, 0.0};
    double ph = 0.0, z = 0.0;
    case_cell(s, G, i, j, want_z != 0, u1, u2, ph, z);
    const int64_t c = cidx(P, i, j);
    store4(U1, P, c, u1);
    if (two) {
      store4(U2, P, c, u2);
      field[c] = want_z ? z : ph;
    }
  }
}

// apply_BCs_euler on a grid before the first step (the time record is not
// active yet, so k_bc_u would not run)
__global__ void k_case_bcs(GridP P, double* U) {
  const int64_t n = (int64_t)P.nr * P.nc;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(k / P.nc), j = (int)(k % P.nc);
    if (is_real(P, i, j) && !P.periodic) continue;
    const BCSrc s = bc_source(P, i, j);
    if (s.i == i && s.j == j) continue;
    V4 v = load4(U, P, cidx(P, s.i, s.j));
    if (s.flipu) v.b = -v.b;
    if (s.flipv) v.c = -v.c;
    store4(U, P, cidx(P, i, j), v);
  }
}

static gfm_grid_desc grid_of(const gfm_ctx* ctx) {
  const GridP& P = ctx->P;
  gfm_grid_desc d;
  memset(&d, 0, sizeof(d));
  d.Nx = P.Nx; d.Ny = P.Ny; d.numGC = P.g;
  d.x0 = P.x0; d.y0 = P.y0; d.dx = P.dx; d.dy = P.dy;
  d.BC_L = P.bcL; d.BC_R = P.bcR; d.BC_B = P.bcB; d.BC_T = P.bcT;
  d.gamma1 = P.g1; d.pinf1 = P.p1; d.gamma2 = P.g2; d.pinf2 = P.p2;
  return d;
}

static gfm_status_t init_from_spec(gfm_ctx* ctx, const CaseSpec& cs, int itm) {
  const GridP& P = ctx->P;
  CaseGeo G;
  G.Nx = P.Nx; G.Ny = P.Ny; G.g = P.g; G.nr = P.nr; G.nc = P.nc;
  G.x0 = P.x0; G.y0 = P.y0; G.dx = P.dx; G.dy = P.dy;
  const int64_t n = (int64_t)P.nr * P.nc;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  const int two = ctx->two_fluid;
  k_case_init<<<blocks, 256, 0, ctx->stream>>>(cs, G, P, ctx->U[0], two ? ctx->U[1] : nullptr,
                                               two ? ctx->phi : nullptr, two, itm == GFM_ITM_VOF ? 1 : 0);
  k_case_bcs<<<blocks, 256, 0, ctx->stream>>>(P, ctx->U[0]);
  if (two) k_case_bcs<<<blocks, 256, 0, ctx->stream>>>(P, ctx->U[1]);
  if (cudaGetLastError() != cudaSuccess) return GFM_ERR_CUDA;
  if (two) ctx->itm = itm;
  return gfm_set_time(ctx, 0.0, 0);
}

}  // namespace gfm

extern "C" {

// the initial state of a named case in the context's grids (and phi, or z
// with itm = GFM_ITM_VOF), t = 0, step 0; the context's grid must be the
// case's (gfm_case_params)
gfm_status_t gfm_case_init_device(gfm_ctx* ctx, const char* sim_type, const char* test_case, int itm) {
  if (!ctx || !sim_type || !test_case || (itm != GFM_ITM_LEVELSET && itm != GFM_ITM_VOF)) return GFM_ERR_ARG;
  const bool two = std::string(sim_type) == "twofluid";
  if (two != (ctx->two_fluid != 0)) return GFM_ERR_ARG;
  const gfm_grid_desc d = gfm::grid_of(ctx);
  gfm::CaseSpec cs;
  if (!gfm::make_case_spec(sim_type, test_case, &d, &cs)) return GFM_ERR_ARG;
  return gfm::init_from_spec(ctx, cs, itm);
}

gfm_status_t gfm_case_init_shock_bubble_device(gfm_ctx* ctx, const gfm_bubble_params* p, int itm) {
  if (!ctx || !p || !ctx->two_fluid || (itm != GFM_ITM_LEVELSET && itm != GFM_ITM_VOF)) return GFM_ERR_ARG;
  const gfm_grid_desc d = gfm::grid_of(ctx);
  gfm::CaseSpec cs;
  if (!gfm::make_bubble_spec(p, &d, &cs)) return GFM_ERR_ARG;
  return gfm::init_from_spec(ctx, cs, itm);
}

}  // extern "C"
