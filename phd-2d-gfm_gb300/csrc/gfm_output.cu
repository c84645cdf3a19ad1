// Output files of the reference's drivers and the asynchronous device -> host
// pipeline that feeds them.
//
//   sim_twofluid::output            (sourcecode/sim_twofluid.cpp:163-297)
//       <base>-<n>-prims.dat  x y rho u v e p   (real fluid: phi < 0 -> fluid 1)
//       <base>-<n>-ls.dat     x y phi           (get_sdf)
//       <base>-<n>-vfield.dat x y u v           (the ghost fill's velocity field)
//       <base>-<n>-z.dat      x y z             (get_z)
//       <base>-<n>-schlieren.dat x y |grad rho| / max   (real cells)
//       <base>-GDAerr.dat     Nx L1err          (Gaussian density advection error)
//     rows i, columns j in [2, N + 2g - 2), a blank line after each row
//   sim_twofluid::output_mass_error (:302-331)  <base>-masschange.dat  t err1 err2
//   sim_twofluid::run_sim           (:92-103)   <base>-runtime.dat     seconds
//   sim_onefluid::output            (sourcecode/sim_onefluid.cpp:169-192)
//       <base>-<n>-prims.dat over every padded cell
//
// Numbers are printed as the reference's std::ostream does by default (the
// %g conversion with 6 significant digits).  get_z of a level set is the
// indicator of fluid 1 (phi <= 0); the VOF tracker's is z itself, and its
// get_sdf is 0.5 - z.  The velocity field is printed at cell centres (the
// first-order field stores one velocity per cell).
//
// The pipeline: an output copies the device grids into device staging
// buffers on the context's stream (a few microseconds), a copy stream moves
// them into pinned host memory, and a writer thread formats the files while
// the GPU keeps stepping.  Mass-change lines copy two device-reduced masses
// per step the same way.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gfm_gb300.h"
#include "gfm_internal.cuh"

namespace gfm {
void launch_mass(gfm_ctx* ctx, double sign, double* part, double* out);
double* mass_scratch(gfm_ctx* ctx);
}

namespace {

struct Geo {
  int Nx, Ny, g, nr, nc;
  double x0, y0, dx, dy, g1, p1, g2, p2;
  double ccx(int j) const { return x0 + ((double)(j - g) + 0.5) * dx; }
  double ccy(int i) const { return y0 + ((double)(i - g) + 0.5) * dy; }
  size_t at(int i, int j) const { return (size_t)i * nc + j; }
  size_t plane() const { return (size_t)nr * nc; }
};

Geo geo_of(const gfm_grid_desc* d) {
  Geo G;
  G.Nx = d->Nx; G.Ny = d->Ny; G.g = d->numGC;
  G.nr = d->Ny + 2 * d->numGC; G.nc = d->Nx + 2 * d->numGC;
  G.x0 = d->x0; G.y0 = d->y0; G.dx = d->dx; G.dy = d->dy;
  G.g1 = d->gamma1; G.p1 = d->pinf1; G.g2 = d->gamma2; G.p2 = d->pinf2;
  return G;
}

// a text file assembled in memory and written at once
struct Text {
  std::string s;
  void num(double v) {
    char b[32];
    int n = snprintf(b, sizeof(b), "%g", v);
    s.append(b, (size_t)n);
  }
  void sp() { s.push_back(' '); }
  void nl() { s.push_back('\n'); }
  bool save(const std::string& path, bool append = false) const {
    FILE* f = fopen(path.c_str(), append ? "ab" : "wb");
    if (!f) return false;
    bool ok = fwrite(s.data(), 1, s.size(), f) == s.size();
    return (fclose(f) == 0) && ok;
  }
};

// misc::specific_ie and eos::pressure (headers/euler_misc.hpp:23-29; the EOS
// of the stiffened gas)
struct PrimOut { double rho, u, v, e, p; };
PrimOut prim_out(double g, double pinf, const double* U, size_t plane, size_t c) {
  PrimOut o;
  o.rho = U[c];
  o.u = U[plane + c] / o.rho;
  o.v = U[2 * plane + c] / o.rho;
  o.e = (U[3 * plane + c] / o.rho) - 0.5 * (o.u * o.u + o.v * o.v);
  o.p = (g - 1.0) * o.rho * o.e - g * pinf;
  return o;
}

void prims_line(Text& t, double x, double y, const PrimOut& o) {
  t.num(x); t.sp(); t.num(y); t.sp(); t.num(o.rho); t.sp(); t.num(o.u); t.sp(); t.num(o.v); t.sp();
  t.num(o.e); t.sp(); t.num(o.p); t.nl();
}

bool write_twofluid(const Geo& G, const std::string& base, int itm, int numsteps, const double* U1,
                    const double* U2, const double* field, const double* vel) {
  const size_t P = G.plane();
  const std::string stem = base + "-" + std::to_string(numsteps);
  auto sdf = [&](int i, int j) { return itm == GFM_ITM_VOF ? 0.5 - field[G.at(i, j)] : field[G.at(i, j)]; };
  auto zval = [&](int i, int j) {
    return itm == GFM_ITM_VOF ? field[G.at(i, j)] : (field[G.at(i, j)] <= 0.0 ? 1.0 : 0.0);
  };
  bool ok[4] = {true, true, true, true};
  // prims
  std::thread t0([&]() {
    Text t;
    t.s.reserve((size_t)G.nr * G.nc * 80);
    for (int i = 2; i < G.nr - 2; i++) {
      for (int j = 2; j < G.nc - 2; j++) {
        const bool f1 = sdf(i, j) < 0.0;
        prims_line(t, G.ccx(j), G.ccy(i),
                   f1 ? prim_out(G.g1, G.p1, U1, P, G.at(i, j)) : prim_out(G.g2, G.p2, U2, P, G.at(i, j)));
      }
      t.nl();
    }
    ok[0] = t.save(stem + "-prims.dat");
  });
  // ls, vfield, z
  std::thread t1([&]() {
    Text a, b, c;
    for (int i = 2; i < G.nr - 2; i++) {
      for (int j = 2; j < G.nc - 2; j++) {
        const double x = G.ccx(j), y = G.ccy(i);
        a.num(x); a.sp(); a.num(y); a.sp(); a.num(sdf(i, j)); a.nl();
        b.num(x); b.sp(); b.num(y); b.sp(); b.num(vel[G.at(i, j)]); b.sp(); b.num(vel[P + G.at(i, j)]); b.nl();
        c.num(x); c.sp(); c.num(y); c.sp(); c.num(zval(i, j)); c.nl();
      }
      a.nl(); b.nl(); c.nl();
    }
    ok[1] = a.save(stem + "-ls.dat") && b.save(stem + "-vfield.dat") && c.save(stem + "-z.dat");
  });
  // schlieren (max of |grad rho| of the real fluid over real cells) and the GDA error
  std::thread t2([&]() {
    const int g = G.g;
    std::vector<double> grads;
    grads.reserve((size_t)G.Nx * G.Ny);
    auto rho = [&](int i, int j) { return sdf(i, j) <= 0.0 ? U1[G.at(i, j)] : U2[G.at(i, j)]; };
    for (int i = g; i < G.Ny + g; i++)
      for (int j = g; j < G.Nx + g; j++) {
        const double gx = (rho(i, j + 1) - rho(i, j - 1)) / (2.0 * G.dx);
        const double gy = (rho(i + 1, j) - rho(i - 1, j)) / (2.0 * G.dy);
        grads.push_back(std::sqrt(gx * gx + gy * gy));
      }
    const double mx = *std::max_element(grads.begin(), grads.end());
    Text s;
    size_t k = 0;
    for (int i = g; i < G.Ny + g; i++) {
      for (int j = g; j < G.Nx + g; j++) {
        s.num(G.ccx(j)); s.sp(); s.num(G.ccy(i)); s.sp(); s.num(grads[k++] / mx); s.nl();
      }
      s.nl();
    }
    ok[2] = s.save(stem + "-schlieren.dat");
    double L1 = 0.0;
    for (int i = g; i < G.Ny + g; i++)
      for (int j = g; j < G.Nx + g; j++) {
        const double dxc = G.ccx(j) - 0.5, dyc = G.ccy(i) - 0.5;
        const double exact = 1.0 + 1000.0 * std::exp(-(dxc * dxc + dyc * dyc) / (2.0 * 0.1 * 0.1));
        L1 += std::fabs(U1[G.at(i, j)] - exact) * G.dx * G.dy;
      }
    Text e;
    e.num((double)G.Nx); e.sp(); e.num(L1); e.nl();
    ok[3] = e.save(base + "-GDAerr.dat");
  });
  t0.join(); t1.join(); t2.join();
  return ok[0] && ok[1] && ok[2] && ok[3];
}

bool write_onefluid(const Geo& G, const std::string& base, int numsteps, const double* U) {
  Text t;
  t.s.reserve((size_t)G.nr * G.nc * 80);
  const size_t P = G.plane();
  for (int i = 0; i < G.nr; i++) {
    for (int j = 0; j < G.nc; j++) prims_line(t, G.ccx(j), G.ccy(i), prim_out(G.g1, G.p1, U, P, G.at(i, j)));
    t.nl();
  }
  return t.save(base + "-" + std::to_string(numsteps) + "-prims.dat");
}

}  // namespace

// ---------------------------------------------------------------------------
// the asynchronous writer
// ---------------------------------------------------------------------------
struct gfm_writer {
  gfm_ctx* ctx = nullptr;
  gfm_grid_desc desc;
  Geo G;
  std::string base;
  int two = 0;
  cudaStream_t copy = nullptr;
  static constexpr int NSLOT = 2, PLANES = 11;   // U1 (4), U2 (4), interface field, velocity (2)
  struct Slot {
    double* dev = nullptr;
    double* host = nullptr;
    cudaEvent_t staged = nullptr, copied = nullptr;
    bool busy = false;
  } slot[NSLOT];
  int next_slot = 0;
  static constexpr int NMASS = 256;
  double* mass_dev = nullptr;    // NMASS x 2
  double* mass_host = nullptr;   // pinned
  cudaEvent_t mass_ev[NMASS];
  bool mass_busy[NMASS];
  int next_mass = 0;
  double m0[2] = {0.0, 0.0};
  bool have_m0 = false;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::function<void()>> jobs;
  bool stop = false;
  bool failed = false;
};

namespace {

void worker_loop(gfm_writer* w) {
  for (;;) {
    std::function<void()> job;
    {
      std::unique_lock<std::mutex> lk(w->mu);
      w->cv.wait(lk, [&] { return w->stop || !w->jobs.empty(); });
      if (w->jobs.empty()) return;
      job = std::move(w->jobs.front());
      w->jobs.pop_front();
    }
    job();
    w->cv.notify_all();
  }
}

void push(gfm_writer* w, std::function<void()> job) {
  {
    std::lock_guard<std::mutex> lk(w->mu);
    w->jobs.push_back(std::move(job));
  }
  w->cv.notify_all();
}

// device pointers of the arrays an output copies (null: absent)
void sources(gfm_writer* w, const double* src[4], size_t planes[4]) {
  gfm_ctx* c = w->ctx;
  src[0] = c->U[0]; planes[0] = 4;
  src[1] = w->two ? c->U[1] : nullptr; planes[1] = 4;
  src[2] = w->two ? c->phi : nullptr; planes[2] = 1;
  src[3] = w->two ? c->vel : nullptr; planes[3] = 2;
}

}  // namespace

extern "C" {

gfm_status_t gfm_write_output_files(const gfm_grid_desc* d, const char* basename, int two_fluid, int itm,
                                    int numsteps, const double* U1, const double* U2, const double* field,
                                    const double* vel) {
  if (!d || !basename || !U1 || d->Nx < 1 || d->Ny < 1 || d->numGC < 2) return GFM_ERR_ARG;
  Geo G = geo_of(d);
  if (two_fluid) {
    if (!U2 || !field || !vel || (itm != GFM_ITM_LEVELSET && itm != GFM_ITM_VOF)) return GFM_ERR_ARG;
    return write_twofluid(G, basename, itm, numsteps, U1, U2, field, vel) ? GFM_OK : GFM_ERR_ARG;
  }
  return write_onefluid(G, basename, numsteps, U1) ? GFM_OK : GFM_ERR_ARG;
}

gfm_status_t gfm_writer_create(gfm_ctx* ctx, const gfm_grid_desc* d, const char* basename, gfm_writer** out) {
  if (!ctx || !d || !basename || !out) return GFM_ERR_ARG;
  gfm_writer* w = new gfm_writer();
  w->ctx = ctx;
  w->desc = *d;
  w->G = geo_of(d);
  w->base = basename;
  w->two = ctx->two_fluid;
  const size_t plane_b = sizeof(double) * (size_t)ctx->P.plane;
  const size_t host_b = sizeof(double) * w->G.plane();
  bool ok = cudaStreamCreateWithFlags(&w->copy, cudaStreamNonBlocking) == cudaSuccess;
  for (int s = 0; s < gfm_writer::NSLOT && ok; s++) {
    ok = cudaMalloc(&w->slot[s].dev, gfm_writer::PLANES * plane_b) == cudaSuccess &&
         cudaMallocHost(&w->slot[s].host, gfm_writer::PLANES * host_b) == cudaSuccess &&
         cudaEventCreateWithFlags(&w->slot[s].staged, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&w->slot[s].copied, cudaEventDisableTiming) == cudaSuccess;
  }
  ok = ok && cudaMalloc(&w->mass_dev, sizeof(double) * 2 * gfm_writer::NMASS) == cudaSuccess &&
       cudaMallocHost(&w->mass_host, sizeof(double) * 2 * gfm_writer::NMASS) == cudaSuccess;
  for (int k = 0; k < gfm_writer::NMASS; k++) {
    w->mass_ev[k] = nullptr;
    w->mass_busy[k] = false;
    if (ok) ok = cudaEventCreateWithFlags(&w->mass_ev[k], cudaEventDisableTiming) == cudaSuccess;
  }
  w->worker = std::thread(worker_loop, w);
  *out = w;
  if (!ok) {
    gfm_writer_destroy(w);
    *out = nullptr;
    return GFM_ERR_CUDA;
  }
  return GFM_OK;
}

// the files of sim_*::output for the context's current state, written by the
// writer thread; returns once the grids are staged on the device
gfm_status_t gfm_writer_output(gfm_writer* w, int numsteps) {
  if (!w) return GFM_ERR_ARG;
  gfm_writer::Slot* s = &w->slot[w->next_slot];
  {
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [&] { return !s->busy; });
    s->busy = true;
  }
  w->next_slot = (w->next_slot + 1) % gfm_writer::NSLOT;
  auto fail = [&]() {   // release the slot: nothing was queued for it
    std::lock_guard<std::mutex> lk(w->mu);
    s->busy = false;
    w->failed = true;
    w->cv.notify_all();
    return GFM_ERR_CUDA;
  };
  const gfm::GridP& P = w->ctx->P;
  const double* src[4];
  size_t planes[4];
  sources(w, src, planes);
  // stage on the device in stream order, then copy to pinned memory beside the compute
  size_t off = 0;
  for (int a = 0; a < 4; a++) {
    if (!src[a]) continue;
    if (cudaMemcpyAsync(s->dev + off * P.plane, src[a], sizeof(double) * planes[a] * P.plane,
                        cudaMemcpyDeviceToDevice, w->ctx->stream) != cudaSuccess)
      return fail();
    off += planes[a];
  }
  if (cudaEventRecord(s->staged, w->ctx->stream) != cudaSuccess) return fail();
  if (cudaStreamWaitEvent(w->copy, s->staged, 0) != cudaSuccess) return fail();
  const size_t wb = sizeof(double) * (size_t)P.nc;
  if (cudaMemcpy2DAsync(s->host, wb, s->dev, sizeof(double) * P.pitch, wb, off * P.nr, cudaMemcpyDeviceToHost,
                        w->copy) != cudaSuccess)
    return fail();
  if (cudaEventRecord(s->copied, w->copy) != cudaSuccess) return fail();
  const int itm = w->ctx->itm;
  push(w, [w, s, numsteps, itm]() {
    bool ok = cudaEventSynchronize(s->copied) == cudaSuccess;
    const size_t pl = w->G.plane();
    if (ok) {
      if (w->two)
        ok = write_twofluid(w->G, w->base, itm, numsteps, s->host, s->host + 4 * pl, s->host + 8 * pl,
                            s->host + 9 * pl);
      else
        ok = write_onefluid(w->G, w->base, numsteps, s->host);
    }
    std::lock_guard<std::mutex> lk(w->mu);
    if (!ok) w->failed = true;
    s->busy = false;
  });
  return GFM_OK;
}

// one line of sim_twofluid::output_mass_error: the masses of fluid 1 (where
// the interface field's sdf < 0) and fluid 2 (sdf > 0), reduced on the device
// (a tree sum: not the reference's row-major summation order, so the last
// bits can differ), relative to those of the first call (numsteps == 0
// starts a new file)
gfm_status_t gfm_writer_mass(gfm_writer* w, int numsteps, double t) {
  if (!w || !w->two) return GFM_ERR_ARG;
  const int k = w->next_mass;
  {
    std::unique_lock<std::mutex> lk(w->mu);
    w->cv.wait(lk, [&] { return !w->mass_busy[k]; });
    w->mass_busy[k] = true;
  }
  w->next_mass = (k + 1) % gfm_writer::NMASS;
  auto fail = [&]() {
    std::lock_guard<std::mutex> lk(w->mu);
    w->mass_busy[k] = false;
    w->failed = true;
    w->cv.notify_all();
    return GFM_ERR_CUDA;
  };
  gfm_ctx* c = w->ctx;
  double* part = gfm::mass_scratch(c);
  gfm::launch_mass(c, -1.0, part, w->mass_dev + 2 * k);
  gfm::launch_mass(c, 1.0, part, w->mass_dev + 2 * k + 1);
  if (cudaMemcpyAsync(w->mass_host + 2 * k, w->mass_dev + 2 * k, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                      c->stream) != cudaSuccess)
    return fail();
  if (cudaEventRecord(w->mass_ev[k], c->stream) != cudaSuccess) return fail();
  push(w, [w, k, numsteps, t]() {
    bool ok = cudaEventSynchronize(w->mass_ev[k]) == cudaSuccess;
    const double m1 = w->mass_host[2 * k], m2 = w->mass_host[2 * k + 1];
    if (ok) {
      if (numsteps == 0 || !w->have_m0) {
        w->m0[0] = m1;
        w->m0[1] = m2;
        w->have_m0 = true;
      }
      Text line;
      line.num(t); line.sp(); line.num((m1 - w->m0[0]) / w->m0[0]); line.sp();
      line.num((m2 - w->m0[1]) / w->m0[1]); line.nl();
      ok = line.save(w->base + "-masschange.dat", numsteps != 0);
    }
    std::lock_guard<std::mutex> lk(w->mu);
    if (!ok) w->failed = true;
    w->mass_busy[k] = false;
  });
  return GFM_OK;
}

gfm_status_t gfm_writer_runtime(gfm_writer* w, double seconds) {
  if (!w) return GFM_ERR_ARG;
  push(w, [w, seconds]() {
    Text t;
    t.num(seconds); t.nl();
    bool ok = t.save(w->base + "-runtime.dat");
    std::lock_guard<std::mutex> lk(w->mu);
    if (!ok) w->failed = true;
  });
  return GFM_OK;
}

gfm_status_t gfm_writer_finish(gfm_writer* w) {
  if (!w) return GFM_ERR_ARG;
  std::unique_lock<std::mutex> lk(w->mu);
  w->cv.wait(lk, [&] {
    if (!w->jobs.empty()) return false;
    for (auto& s : w->slot)
      if (s.busy) return false;
    for (int k = 0; k < gfm_writer::NMASS; k++)
      if (w->mass_busy[k]) return false;
    return true;
  });
  return w->failed ? GFM_ERR_ARG : GFM_OK;
}

gfm_status_t gfm_writer_destroy(gfm_writer* w) {
  if (!w) return GFM_ERR_ARG;
  if (w->worker.joinable()) {
    gfm_writer_finish(w);
    {
      std::lock_guard<std::mutex> lk(w->mu);
      w->stop = true;
    }
    w->cv.notify_all();
    w->worker.join();
  }
  for (auto& s : w->slot) {
    cudaFree(s.dev);
    cudaFreeHost(s.host);
    if (s.staged) cudaEventDestroy(s.staged);
    if (s.copied) cudaEventDestroy(s.copied);
  }
  cudaFree(w->mass_dev);
  cudaFreeHost(w->mass_host);
  for (int k = 0; k < gfm_writer::NMASS; k++)
    if (w->mass_ev[k]) cudaEventDestroy(w->mass_ev[k]);
  if (w->copy) cudaStreamDestroy(w->copy);
  delete w;
  return GFM_OK;
}

// The reference's time loop with its outputs (sim_twofluid::run_sim,
// sourcecode/sim_twofluid.cpp:49-103; sim_onefluid::run_sim,
// sourcecode/sim_onefluid.cpp:36-66): an output at the start, after every
// step at which t - lastoutputtime > T / output_freq (two-fluid) or
// numsteps % output_freq == 0 (one-fluid), and at the end; a mass-change line
// per step and the loop's wall time (two-fluid).  At most max_steps steps
// (<= 0: until t reaches T).  *seconds (optional): the loop's wall time.
gfm_status_t gfm_run_sim(gfm_ctx* ctx, const gfm_method_desc* m, const gfm_grid_desc* d, const char* basename,
                         int output_freq, int max_steps, double* seconds) {
  if (!ctx || !m || !d || !basename) return GFM_ERR_ARG;
  gfm_writer* w = nullptr;
  gfm_status_t r = gfm_writer_create(ctx, d, basename, &w);
  if (r != GFM_OK) return r;
  double t = 0.0, dt = 0.0;
  int n = 0;
  auto fetch = [&]() { return gfm_get_time(ctx, &t, &n, &dt); };
  if ((r = fetch()) != GFM_OK) { gfm_writer_destroy(w); return r; }
  const bool two = ctx->two_fluid != 0;
  if (two) ctx->itm = m->itm;
  r = gfm_writer_output(w, n);
  if (r == GFM_OK && two) r = gfm_writer_mass(w, n, t);
  const double interval = m->T / (double)output_freq;
  double last = 0.0;
  const auto t0 = std::chrono::steady_clock::now();
  int taken = 0;
  while (r == GFM_OK && t < m->T && (max_steps <= 0 || taken < max_steps)) {
    r = gfm::run_steps(ctx, m, 1, nullptr);
    if (r == GFM_OK) r = fetch();
    taken++;
    if (r != GFM_OK) break;
    if (two) {
      if (t - last > interval) {
        r = gfm_writer_output(w, n);
        last = t;
      }
      if (r == GFM_OK) r = gfm_writer_mass(w, n, t);
    } else if (output_freq > 0 && n % output_freq == 0) {
      r = gfm_writer_output(w, n);
    }
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (r == GFM_OK) r = gfm_writer_output(w, n);
  if (r == GFM_OK && two) r = gfm_writer_runtime(w, secs);
  gfm_status_t rf = gfm_writer_finish(w);
  gfm_writer_destroy(w);
  if (seconds) *seconds = secs;
  return r != GFM_OK ? r : rf;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// checkpoint / resume
// ---------------------------------------------------------------------------
namespace {

constexpr char CKPT_MAGIC[8] = {'G', 'F', 'M', 'C', 'K', 'P', 'T', '1'};
constexpr uint32_t CKPT_VERSION = 1;

struct Fnv {
  uint64_t h = 0xcbf29ce484222325ull;
  void add(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t k = 0; k < n; k++) { h ^= b[k]; h *= 0x100000001b3ull; }
  }
};

struct Out {
  FILE* f;
  Fnv fnv;
  bool ok = true;
  void put(const void* p, size_t n) {
    if (ok && fwrite(p, 1, n, f) != n) ok = false;
    fnv.add(p, n);
  }
  template <class T> void val(T v) { put(&v, sizeof(T)); }
};

struct In {
  FILE* f;
  Fnv fnv;
  bool ok = true;
  void get(void* p, size_t n) {
    if (ok && fread(p, 1, n, f) != n) ok = false;
    if (ok) fnv.add(p, n);
  }
  template <class T> T val() { T v{}; get(&v, sizeof(T)); return v; }
};

bool same_grid(const gfm_grid_desc& a, const gfm_grid_desc& b) {
  return a.Nx == b.Nx && a.Ny == b.Ny && a.numGC == b.numGC && a.BC_L == b.BC_L && a.BC_R == b.BC_R &&
         a.BC_B == b.BC_B && a.BC_T == b.BC_T && a.x0 == b.x0 && a.y0 == b.y0 && a.dx == b.dx && a.dy == b.dy &&
         a.gamma1 == b.gamma1 && a.pinf1 == b.pinf1 && a.gamma2 == b.gamma2 && a.pinf2 == b.pinf2;
}

gfm_grid_desc desc_of(const gfm_ctx* ctx) {
  const gfm::GridP& P = ctx->P;
  gfm_grid_desc d;
  memset(&d, 0, sizeof(d));
  d.Nx = P.Nx; d.Ny = P.Ny; d.numGC = P.g;
  d.x0 = P.x0; d.y0 = P.y0; d.dx = P.dx; d.dy = P.dy;
  d.BC_L = P.bcL; d.BC_R = P.bcR; d.BC_B = P.bcB; d.BC_T = P.bcT;
  d.gamma1 = P.g1; d.pinf1 = P.p1; d.gamma2 = P.g2; d.pinf2 = P.p2;
  return d;
}

}  // namespace

extern "C" {

gfm_status_t gfm_checkpoint_write(const char* path, const gfm_grid_desc* d, int two_fluid, double t, int numsteps,
                                  const double* U1, const double* U2, const double* phi) {
  if (!path || !d || !U1 || (two_fluid && (!U2 || !phi)) || d->Nx < 1 || d->Ny < 1 || d->numGC < 1)
    return GFM_ERR_ARG;
  FILE* f = fopen(path, "wb");
  if (!f) return GFM_ERR_IO;
  Out o{f};
  o.put(CKPT_MAGIC, 8);
  o.val<uint32_t>(CKPT_VERSION);
  o.val<uint32_t>(two_fluid ? 1u : 0u);
  for (int v : {d->Nx, d->Ny, d->numGC, d->BC_L, d->BC_R, d->BC_B, d->BC_T}) o.val<int32_t>(v);
  for (double v : {d->x0, d->y0, d->dx, d->dy, d->gamma1, d->pinf1, d->gamma2, d->pinf2}) o.val<double>(v);
  o.val<double>(t);
  o.val<int32_t>(numsteps);
  o.val<int32_t>(0);
  const size_t plane = (size_t)(d->Ny + 2 * d->numGC) * (d->Nx + 2 * d->numGC);
  const uint64_t nplanes = two_fluid ? 9 : 4;
  o.val<uint64_t>(nplanes);
  o.put(U1, sizeof(double) * 4 * plane);
  if (two_fluid) {
    o.put(U2, sizeof(double) * 4 * plane);
    o.put(phi, sizeof(double) * plane);
  }
  const uint64_t h = o.fnv.h;
  if (o.ok && fwrite(&h, sizeof(h), 1, f) != 1) o.ok = false;
  if (fclose(f) != 0) o.ok = false;
  return o.ok ? GFM_OK : GFM_ERR_IO;
}

gfm_status_t gfm_checkpoint_read(const char* path, gfm_grid_desc* d, int* two_fluid, double* t, int* numsteps,
                                 double* U1, double* U2, double* phi) {
  if (!path || !d) return GFM_ERR_ARG;
  FILE* f = fopen(path, "rb");
  if (!f) return GFM_ERR_IO;
  In in{f};
  char magic[8];
  in.get(magic, 8);
  const uint32_t version = in.val<uint32_t>(), two = in.val<uint32_t>();
  gfm_grid_desc g;
  memset(&g, 0, sizeof(g));
  g.Nx = in.val<int32_t>(); g.Ny = in.val<int32_t>(); g.numGC = in.val<int32_t>();
  g.BC_L = in.val<int32_t>(); g.BC_R = in.val<int32_t>(); g.BC_B = in.val<int32_t>(); g.BC_T = in.val<int32_t>();
  g.x0 = in.val<double>(); g.y0 = in.val<double>(); g.dx = in.val<double>(); g.dy = in.val<double>();
  g.gamma1 = in.val<double>(); g.pinf1 = in.val<double>(); g.gamma2 = in.val<double>(); g.pinf2 = in.val<double>();
  const double tt = in.val<double>();
  const int32_t ns = in.val<int32_t>();
  in.val<int32_t>();
  const uint64_t nplanes = in.val<uint64_t>();
  bool ok = in.ok && memcmp(magic, CKPT_MAGIC, 8) == 0 && version == CKPT_VERSION && two <= 1 &&
            nplanes == (two ? 9u : 4u) && g.Nx > 0 && g.Ny > 0 && g.numGC > 0 && g.Nx < (1 << 20) &&
            g.Ny < (1 << 20) && g.numGC < 64;
  if (ok && (U1 || U2 || phi)) {
    const size_t plane = (size_t)(g.Ny + 2 * g.numGC) * (g.Nx + 2 * g.numGC);
    std::vector<double> buf(nplanes * plane);
    in.get(buf.data(), sizeof(double) * buf.size());
    uint64_t h = 0;
    ok = in.ok && fread(&h, sizeof(h), 1, f) == 1 && h == in.fnv.h;
    if (ok) {
      if (U1) memcpy(U1, buf.data(), sizeof(double) * 4 * plane);
      if (two && U2) memcpy(U2, buf.data() + 4 * plane, sizeof(double) * 4 * plane);
      if (two && phi) memcpy(phi, buf.data() + 8 * plane, sizeof(double) * plane);
    }
  }
  fclose(f);
  if (!ok) return GFM_ERR_IO;
  *d = g;
  if (two_fluid) *two_fluid = (int)two;
  if (t) *t = tt;
  if (numsteps) *numsteps = ns;
  return GFM_OK;
}

gfm_status_t gfm_checkpoint_save(gfm_ctx* ctx, const char* path) {
  if (!ctx || !path) return GFM_ERR_ARG;
  const gfm_grid_desc d = desc_of(ctx);
  const size_t plane = (size_t)ctx->P.nr * ctx->P.nc;
  std::vector<double> U1(4 * plane), U2, phi;
  gfm_status_t r = gfm_download(ctx, 1, U1.data());
  if (r == GFM_OK && ctx->two_fluid) {
    U2.resize(4 * plane);
    phi.resize(plane);
    r = gfm_download(ctx, 2, U2.data());
    if (r == GFM_OK) r = gfm_download_phi(ctx, phi.data());
  }
  double t = 0.0, dt = 0.0;
  int n = 0;
  if (r == GFM_OK) r = gfm_get_time(ctx, &t, &n, &dt);
  if (r != GFM_OK) return r;
  return gfm_checkpoint_write(path, &d, ctx->two_fluid, t, n, U1.data(), ctx->two_fluid ? U2.data() : nullptr,
                              ctx->two_fluid ? phi.data() : nullptr);
}

gfm_status_t gfm_checkpoint_load(gfm_ctx* ctx, const char* path) {
  if (!ctx || !path) return GFM_ERR_ARG;
  gfm_grid_desc d;
  int two = 0, n = 0;
  double t = 0.0;
  gfm_status_t r = gfm_checkpoint_read(path, &d, &two, &t, &n, nullptr, nullptr, nullptr);
  if (r != GFM_OK) return r;
  if (!same_grid(d, desc_of(ctx)) || two != ctx->two_fluid) return GFM_ERR_ARG;
  const size_t plane = (size_t)ctx->P.nr * ctx->P.nc;
  std::vector<double> U1(4 * plane), U2(two ? 4 * plane : 0), phi(two ? plane : 0);
  r = gfm_checkpoint_read(path, &d, &two, &t, &n, U1.data(), two ? U2.data() : nullptr, two ? phi.data() : nullptr);
  if (r != GFM_OK) return r;
  r = gfm_upload(ctx, 1, U1.data());
  if (r == GFM_OK && two) r = gfm_upload(ctx, 2, U2.data());
  if (r == GFM_OK && two) r = gfm_upload_phi(ctx, phi.data());
  if (r == GFM_OK) r = gfm_set_time(ctx, t, n);
  return r;
}

}  // extern "C"
