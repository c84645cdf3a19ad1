// One-fluid time steps that allocate no device memory.
//
// Some callers cannot call cudaMalloc: host runtimes whose own memory pool
// owns the device and rejects allocations made behind its back, and
// real-time callers that forbid allocation after start-up because cudaMalloc
// can block and synchronise the whole device.  For them,
// gfm_onefluid_step_noalloc advances a caller-owned device grid in place;
// its scratch (the flux-update output grid, the time/step record and the
// CFL reduction words) lives in the file-scope array below, which every GPU
// that loads this library holds until the process exits.
//
// Set-up: host code may not use the array's name as a device address.  The
// first call in each CUDA context (normally once per device: the runtime's
// primary context) looks up the array's device address with
// cudaGetSymbolAddress, with that context current, and keeps it under the
// context's unique id.  A __device__ array has its own address in every
// context that loads the module, so a caller that makes its own contexts with
// the driver API, or that resets the device (a new primary context), gets a
// fresh look-up there.  Make that first call before any stream capture.
// Calls share the array and it keeps the last call's contents, so every call
// re-initialises what must start at zero; calls that overlap on the GPU
// (different streams, or different host threads on the same device) race on
// it.
#include "gfm_internal.cuh"
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cstdio>
#include <mutex>

namespace gfm {
void launch_cfl_impl(gfm_ctx* ctx, double CFL, double T, bool ogfm, unsigned int* counter);

// 16 MiB: a 256-byte header (time record), 256 bytes of counters, then the
// four planes of the flux-update output grid.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(16) << 20;
constexpr size_t NOALLOC_HEADER = 512;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];
static_assert(sizeof(DevTime) <= 256, "time record must fit its slot");

// The array's address per CUDA context, keyed by the context's unique id
// (cuCtxGetId: ids are never reused within a process, unlike context
// handles).  Driver entry points come through the runtime, so the library
// links no driver library.
static std::mutex g_noalloc_mutex;
struct NoallocSlot { unsigned long long ctx_id; void* ptr; };
static NoallocSlot g_noalloc_slots[64];
static int g_noalloc_nslots = 0;

static bool current_context_id(unsigned long long* id) {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
    looked_up = true;
  }
  if (!get_current || !get_id) return false;
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS;
}

// Device address of the scratch array in the current context; nullptr and
// a message on failure.  Called with g_noalloc_mutex held.
static void* scratch_address() {
  unsigned long long id = 0;
  if (current_context_id(&id))
    for (int k = 0; k < g_noalloc_nslots; k++)
      if (g_noalloc_slots[k].ctx_id == id) return g_noalloc_slots[k].ptr;
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    fprintf(stderr, "gfm_onefluid_step_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
    return nullptr;
  }
  // The look-up has made the runtime's context current if none was: its id
  // is read now.  Kept when a slot is free; otherwise looked up again on the
  // next call (the look-up allocates nothing).
  if (current_context_id(&id) && g_noalloc_nslots < 64) g_noalloc_slots[g_noalloc_nslots++] = NoallocSlot{id, p};
  return p;
}

static bool valid_bc_kind(int b) {
  return b == GFM_BC_TRANSMISSIVE || b == GFM_BC_REFLECTIVE || b == GFM_BC_PERIODIC;
}

__global__ void k_noalloc_init(DevTime* D, unsigned int* counters, double t, int numsteps, GridP P) {
  D->t = t;
  D->dt = 0.0;
  D->T = 0.0;
  D->CFL = 0.0;
  D->numsteps = numsteps;
  D->active = 0;
  D->maxu_bits = 0ull;
  D->maxv_bits = 0ull;
  D->status = 0u;
  D->n_ifc = 0;
  D->n_rounds = 0;
  D->newton_iters = 0ull;
  D->ifc_iters = 0ull;
  D->ifc_gated = 0;
  D->ifc_solves_total = D->ifc_iters_total = D->ifc_gated_total = 0ull;
  int full[4] = {P.g, P.g + P.Ny, P.g, P.g + P.Nx};
  for (int q = 0; q < 8; q++) D->rc[q] = full[q & 3];
  for (int q = 0; q < 64; q++) counters[q] = 0u;
}

}  // namespace gfm

using namespace gfm;

extern "C" gfm_status_t gfm_onefluid_step_noalloc(const gfm_grid_desc* d, const gfm_method_desc* m, double* U,
                                                  int nsteps, double* t, int* numsteps, uint32_t* status,
                                                  void* stream) {
  if (!d || !m || !U || !t || !numsteps || nsteps < 0) return GFM_ERR_ARG;
  // the grid checks of gfm_ctx_create
  if (d->Nx < 1 || d->Ny < 1 || d->numGC < 2 || d->numGC > 64) return GFM_ERR_ARG;
  if (d->Nx < d->numGC || d->Ny < d->numGC || !(d->dx > 0.0) || !(d->dy > 0.0)) return GFM_ERR_ARG;
  if (!valid_bc_kind(d->BC_L) || !valid_bc_kind(d->BC_R) || !valid_bc_kind(d->BC_B) || !valid_bc_kind(d->BC_T))
    return GFM_ERR_ARG;
  if (m->fs != GFM_FS_GODUNOV && m->fs != GFM_FS_MUSCL) return GFM_ERR_ARG;
  if (!(m->CFL > 0.0) || !(d->gamma1 > 1.0)) return GFM_ERR_ARG;
  bool per = d->BC_L == GFM_BC_PERIODIC || d->BC_R == GFM_BC_PERIODIC || d->BC_B == GFM_BC_PERIODIC ||
             d->BC_T == GFM_BC_PERIODIC;
  bool allper = d->BC_L == GFM_BC_PERIODIC && d->BC_R == GFM_BC_PERIODIC && d->BC_B == GFM_BC_PERIODIC &&
                d->BC_T == GFM_BC_PERIODIC;
  if (per && (!allper || d->Nx != d->Ny)) return GFM_ERR_UNSUPPORTED;
  const int64_t nr = d->Ny + 2 * d->numGC, nc = d->Nx + 2 * d->numGC;
  const int64_t cells = nr * nc;
  if ((size_t)cells * 4 * sizeof(double) > NOALLOC_SCRATCH_BYTES - NOALLOC_HEADER) {
    fprintf(stderr,
            "gfm_onefluid_step_noalloc: grid of %lld padded cells exceeds the %d-cell maximum of the built-in "
            "scratch\n",
            (long long)cells, (int)GFM_NOALLOC_MAX_CELLS);
    return GFM_ERR_ARG;
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GFM_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    return GFM_ERR_CUDA;
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    base = scratch_address();
  }
  if (!base) return GFM_ERR_CUDA;
  // a context on the host stack pointing at the caller's grid and the scratch
  gfm_ctx ctx;
  memset(&ctx, 0, sizeof(ctx));
  GridP& P = ctx.P;
  P.Nx = d->Nx; P.Ny = d->Ny; P.g = d->numGC;
  P.nr = (int)nr; P.nc = (int)nc;
  P.pitch = (int)nc;
  P.plane = cells;
  P.x0 = d->x0; P.y0 = d->y0; P.dx = d->dx; P.dy = d->dy;
  P.idx = 1.0 / P.dx; P.idy = 1.0 / P.dy;
  P.bcL = d->BC_L; P.bcR = d->BC_R; P.bcB = d->BC_B; P.bcT = d->BC_T;
  P.g1 = d->gamma1; P.p1 = d->pinf1; P.g2 = d->gamma1; P.p2 = d->pinf1;
  P.gas1 = make_gas(P.g1, P.p1);
  P.gas2 = P.gas1;
  P.periodic = allper;
  ctx.two_fluid = 0;
  ctx.num_sms = sms;   // grid sizes of the grid-stride kernels, as in gfm_ctx_create
  ctx.flux_shape = FLUX_SHAPE_DEFAULT;
  ctx.stream = static_cast<cudaStream_t>(stream);
  ctx.U[0] = U;
  unsigned char* b = static_cast<unsigned char*>(base);
  ctx.dtime = reinterpret_cast<DevTime*>(b);
  unsigned int* counters = reinterpret_cast<unsigned int*>(b + 256);
  ctx.Unew[0] = reinterpret_cast<double*>(b + NOALLOC_HEADER);

  k_noalloc_init<<<1, 1, 0, ctx.stream>>>(ctx.dtime, counters, *t, *numsteps, P);
  counted();
  for (int s = 0; s < nsteps; s++) {
    launch_cfl_impl(&ctx, m->CFL, m->T, false, counters);
    launch_fs_update(&ctx, m->fs, 1);
    launch_commit(&ctx, 1, true);
    launch_end_step(&ctx);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "gfm_onefluid_step_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return GFM_ERR_CUDA;
  }
  DevTime h;
  e = cudaMemcpyAsync(&h, ctx.dtime, sizeof(DevTime), cudaMemcpyDeviceToHost, ctx.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx.stream);
  if (e != cudaSuccess) {
    fprintf(stderr, "gfm_onefluid_step_noalloc: %s\n", cudaGetErrorString(e));
    return GFM_ERR_CUDA;
  }
  *t = h.t;
  *numsteps = h.numsteps;
  if (status) *status = h.status;
  return GFM_OK;
}
