// Batched execution of many independent instances (the reference runs one
// simulation per process; a batch advances many together).
//
// Each instance is an ordinary context (its own grid, EOS parameters, time
// and dt) whose steps are issued on its own stream.  gfm_step_batched_graph
// records K steps of every instance into one CUDA graph -- one fork from the
// batch stream, K steps per instance on the instance streams, one join -- and
// replays it, so the instances' kernels run side by side: small grids fill
// the GPU together and the latency-bound interface loops of all instances
// overlap.  Launches inside a step that depend on the step number (the
// level-set reinitialisation every k steps) are decided on the device while
// recording, so a replayed graph is correct on every step.  Each instance's
// results are those of stepping it alone.
//
// Two schedules of a step (gfm_batch_set_schedule):
//   streams  each instance's whole step on its own stream, the instances side
//            by side (the default);
//   phased   every instance's step up to its flux update on its own stream,
//            then ONE persistent flux launch per tile shape over the tiles of
//            all instances (k_flux_batch: CTAs pull (instance, fluid, tile)
//            items, costliest instances first), then every instance's commit.
// gfm_batch_autotune times the tile shapes per grid-size class and the two
// schedules on the batch itself and keeps the fastest, then keeps the chosen
// shapes only if the whole batch steps faster with them than with the
// default shape.
#include "gfm_internal.cuh"
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>


using namespace gfm;

struct gfm_batch {
  int n;
  int two_fluid;
  std::vector<gfm_ctx*> inst;
  std::vector<cudaStream_t> streams;
  cudaStream_t main;            // orders the batch's calls (the caller's stream, or cap)
  cudaStream_t cap;             // the batch's own stream: graphs are recorded from it
  cudaEvent_t fork;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t exec;
  int graph_k;                  // steps per replay of exec
  gfm_method_desc graph_m;      // method exec was recorded with
  long long graph_launches;     // kernels per replay of exec
  int graph_schedule;           // schedule exec was recorded with
  std::vector<int> graph_shapes;   // instances' flux tile shapes exec was recorded with
  int schedule;                 // GFM_BATCH_STREAMS or GFM_BATCH_PHASED
  // the phased schedule's flux plan: per-instance arguments, work items
  // grouped by tile shape, two counters per shape (device), and its host copy
  std::vector<unsigned char> plan_host;
  void* d_plan;
  size_t d_plan_bytes;
  int item_off[FLUX_SHAPES], item_n[FLUX_SHAPES];
  size_t args_bytes;
};

namespace {

constexpr int GRAPH_STEPS = 8;

void destroy_graph(gfm_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->graph_k = 0;
}

gfm_status_t cuda_status(cudaError_t e) { return e == cudaSuccess ? GFM_OK : GFM_ERR_CUDA; }

// The batch stream waits for the work issued so far on every instance stream
// (uploads, single-instance calls) ...
gfm_status_t join_instances(gfm_batch* b) {
  for (int i = 0; i < b->n; i++) {
    if (cudaEventRecord(b->join[i], b->streams[i]) != cudaSuccess) return GFM_ERR_CUDA;
    if (cudaStreamWaitEvent(b->main, b->join[i], 0) != cudaSuccess) return GFM_ERR_CUDA;
  }
  return GFM_OK;
}
// ... and later work on the instance streams waits for the batch stream.
gfm_status_t release_instances(gfm_batch* b) {
  if (cudaEventRecord(b->fork, b->main) != cudaSuccess) return GFM_ERR_CUDA;
  for (int i = 0; i < b->n; i++)
    if (cudaStreamWaitEvent(b->streams[i], b->fork, 0) != cudaSuccess) return GFM_ERR_CUDA;
  return GFM_OK;
}

// k steps of every instance on its own stream between a fork from and a join
// to stream `s` (recorded into a graph when s is capturing)
gfm_status_t issue_steps(gfm_batch* b, cudaStream_t s, const gfm_method_desc* m, int k) {
  if (cudaEventRecord(b->fork, s) != cudaSuccess) return GFM_ERR_CUDA;
  for (int i = 0; i < b->n; i++) {
    if (cudaStreamWaitEvent(b->streams[i], b->fork, 0) != cudaSuccess) return GFM_ERR_CUDA;
    gfm_status_t r = run_steps(b->inst[i], m, k, nullptr);
    if (r != GFM_OK) return r;
    if (cudaEventRecord(b->join[i], b->streams[i]) != cudaSuccess) return GFM_ERR_CUDA;
    if (cudaStreamWaitEvent(s, b->join[i], 0) != cudaSuccess) return GFM_ERR_CUDA;
  }
  return GFM_OK;
}

// The flux plan of the phased schedule, built on the host: the instances'
// flux arguments, then their work items grouped by tile shape (instances in
// decreasing cell count, so that the costliest start first), then the
// counters.  Uploaded only when it changed, after the batch's earlier work
// (which may read the previous plan) has finished.
gfm_status_t prepare_flux_plan(gfm_batch* b) {
  const size_t ab = flux_batch_args_size();
  std::vector<unsigned char> plan(ab * b->n);
  for (int i = 0; i < b->n; i++) flux_batch_args(b->inst[i], plan.data() + ab * i);
  std::vector<int> order(b->n);
  for (int i = 0; i < b->n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (int64_t)b->inst[x]->P.Nx * b->inst[x]->P.Ny > (int64_t)b->inst[y]->P.Nx * b->inst[y]->P.Ny;
  });
  std::vector<uint32_t> items;
  const int nf = b->two_fluid ? 2 : 1;
  for (int sh = 0; sh < FLUX_SHAPES; sh++) {
    b->item_off[sh] = (int)items.size();
    for (int i : order) {
      const gfm_ctx* c = b->inst[i];
      if (c->flux_shape != sh) continue;
      const int tw = flux_tile_w(sh), th = flux_tile_h(sh);
      const int tiles = ((c->P.Nx + tw - 1) / tw) * ((c->P.Ny + th - 1) / th);
      if (tiles >= (1 << 23) || i >= (1 << 8)) return GFM_ERR_UNSUPPORTED;
      for (int f = 0; f < nf; f++)
        for (int t = 0; t < tiles; t++) items.push_back(((uint32_t)i << 24) | ((uint32_t)f << 23) | (uint32_t)t);
    }
    b->item_n[sh] = (int)items.size() - b->item_off[sh];
  }
  b->args_bytes = (ab * b->n + 255) / 256 * 256;
  const size_t items_bytes = (items.size() * sizeof(uint32_t) + 255) / 256 * 256;
  std::vector<unsigned char> host(b->args_bytes + items_bytes + 2 * FLUX_SHAPES * sizeof(unsigned int), 0);
  memcpy(host.data(), plan.data(), plan.size());
  memcpy(host.data() + b->args_bytes, items.data(), items.size() * sizeof(uint32_t));
  if (host == b->plan_host && b->d_plan) return GFM_OK;
  // earlier launches may still read the previous plan
  if (cudaStreamSynchronize(b->main) != cudaSuccess) return GFM_ERR_CUDA;
  for (cudaStream_t st : b->streams)
    if (cudaStreamSynchronize(st) != cudaSuccess) return GFM_ERR_CUDA;
  if (host.size() > b->d_plan_bytes) {
    if (b->d_plan) cudaFree(b->d_plan);
    b->d_plan = nullptr;
    b->d_plan_bytes = 0;
    if (cudaMalloc(&b->d_plan, host.size()) != cudaSuccess) return GFM_ERR_CUDA;
    b->d_plan_bytes = host.size();
  }
  if (cudaMemcpy(b->d_plan, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) return GFM_ERR_CUDA;
  b->plan_host.swap(host);
  return GFM_OK;
}

// k phased steps of every instance between a fork from and a join to stream s
gfm_status_t issue_steps_phased(gfm_batch* b, cudaStream_t s, const gfm_method_desc* m, int k) {
  unsigned char* base = static_cast<unsigned char*>(b->d_plan);
  const uint32_t* items = reinterpret_cast<const uint32_t*>(base + b->args_bytes);
  unsigned int* counters =
      reinterpret_cast<unsigned int*>(base + b->plan_host.size() - 2 * FLUX_SHAPES * sizeof(unsigned int));
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 152;
  for (int step = 0; step < k; step++) {
    for (int half = 0; half < 2; half++) {
      if (cudaEventRecord(b->fork, s) != cudaSuccess) return GFM_ERR_CUDA;
      for (int i = 0; i < b->n; i++) {
        if (cudaStreamWaitEvent(b->streams[i], b->fork, 0) != cudaSuccess) return GFM_ERR_CUDA;
        gfm_status_t r = half == 0 ? step_front(b->inst[i], m) : step_back(b->inst[i], m);
        if (r != GFM_OK) return r;
        if (cudaEventRecord(b->join[i], b->streams[i]) != cudaSuccess) return GFM_ERR_CUDA;
        if (cudaStreamWaitEvent(s, b->join[i], 0) != cudaSuccess) return GFM_ERR_CUDA;
      }
      if (half == 0)
        for (int sh = 0; sh < FLUX_SHAPES; sh++)
          if (b->item_n[sh] > 0)
            launch_flux_batch(m->fs, sh, b->d_plan, items + b->item_off[sh], b->item_n[sh], counters + 2 * sh,
                              sms * flux_batch_occupancy(m->fs, sh), s);
    }
  }
  return GFM_OK;
}

gfm_status_t issue(gfm_batch* b, cudaStream_t s, const gfm_method_desc* m, int k) {
  return b->schedule == GFM_BATCH_PHASED ? issue_steps_phased(b, s, m, k) : issue_steps(b, s, m, k);
}

std::vector<int> shapes_of(const gfm_batch* b) {
  std::vector<int> v(b->n);
  for (int i = 0; i < b->n; i++) v[i] = b->inst[i]->flux_shape;
  return v;
}

gfm_status_t record_graph(gfm_batch* b, const gfm_method_desc* m, int k) {
  destroy_graph(b);
  std::vector<int> saved(b->n);
  for (int i = 0; i < b->n; i++) {
    saved[i] = b->inst[i]->steps_done_host;
    b->inst[i]->graph_mode = 1;
  }
  const long long l0 = g_launches.load();
  cudaGraph_t graph = nullptr;
  gfm_status_t r = cuda_status(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
  if (r == GFM_OK) {
    gfm_status_t ri = issue(b, b->cap, m, k);
    cudaError_t e = cudaStreamEndCapture(b->cap, &graph);
    r = (ri != GFM_OK) ? ri : cuda_status(e);
  }
  b->graph_launches = g_launches.load() - l0;
  g_launches.fetch_sub(b->graph_launches);   // recorded, not run
  for (int i = 0; i < b->n; i++) {
    b->inst[i]->steps_done_host = saved[i];
    b->inst[i]->graph_mode = 0;
  }
  if (r == GFM_OK) r = cuda_status(cudaGraphInstantiate(&b->exec, graph, 0));
  if (graph) cudaGraphDestroy(graph);
  if (r != GFM_OK) {
    cudaGetLastError();
    b->exec = nullptr;
    return r;
  }
  b->graph_k = k;
  b->graph_m = *m;
  b->graph_schedule = b->schedule;
  b->graph_shapes = shapes_of(b);
  return GFM_OK;
}

}  // namespace

extern "C" {

gfm_status_t gfm_batch_create(const gfm_grid_desc* grids, int n, int two_fluid, gfm_batch** out) {
  if (!grids || !out || n < 1) return GFM_ERR_ARG;
  *out = nullptr;
  gfm_batch* b = new gfm_batch();
  b->n = n;
  b->two_fluid = two_fluid ? 1 : 0;
  b->main = nullptr;
  b->cap = nullptr;
  b->exec = nullptr;
  b->graph_k = 0;
  b->graph_launches = 0;
  memset(&b->graph_m, 0, sizeof(b->graph_m));
  b->graph_schedule = GFM_BATCH_STREAMS;
  b->schedule = GFM_BATCH_STREAMS;
  b->d_plan = nullptr;
  b->d_plan_bytes = 0;
  b->args_bytes = 0;
  for (int sh = 0; sh < FLUX_SHAPES; sh++) b->item_off[sh] = b->item_n[sh] = 0;
  gfm_status_t r = GFM_OK;
  if (cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
    r = GFM_ERR_CUDA;
  b->main = b->cap;
  for (int i = 0; i < n && r == GFM_OK; i++) {
    gfm_ctx* c = nullptr;
    r = gfm_ctx_create(&grids[i], two_fluid, &c);
    if (r != GFM_OK) break;
    b->inst.push_back(c);
    cudaStream_t s;
    cudaEvent_t e;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { r = GFM_ERR_CUDA; break; }
    b->streams.push_back(s);
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { r = GFM_ERR_CUDA; break; }
    b->join.push_back(e);
    c->stream = s;
    c->overlap = GFM_OVERLAP_OFF;   // the SM partitions are per device; instances overlap each other instead
  }
  if (r != GFM_OK) {
    gfm_batch_destroy(b);
    return r;
  }
  prepare_kernels();
  *out = b;
  return GFM_OK;
}

gfm_status_t gfm_batch_destroy(gfm_batch* b) {
  if (!b) return GFM_OK;
  if (b->main) cudaStreamSynchronize(b->main);
  if (b->cap) cudaStreamSynchronize(b->cap);
  destroy_graph(b);
  for (gfm_ctx* c : b->inst) gfm_ctx_destroy(c);
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->d_plan) cudaFree(b->d_plan);
  delete b;
  return GFM_OK;
}

gfm_status_t gfm_batch_instance(gfm_batch* b, int i, gfm_ctx** ctx) {
  if (!b || !ctx || i < 0 || i >= b->n) return GFM_ERR_ARG;
  *ctx = b->inst[i];
  return GFM_OK;
}

gfm_status_t gfm_batch_set_stream(gfm_batch* b, void* cuda_stream) {
  if (!b) return GFM_ERR_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  if (s == b->main) return GFM_OK;
  if (cudaStreamSynchronize(b->main) != cudaSuccess) return GFM_ERR_CUDA;
  b->main = s;   // any stream, the legacy default stream included: graphs are recorded from cap
  return GFM_OK;
}

gfm_status_t gfm_step_batched_graph(gfm_batch* b, const gfm_method_desc* m, int nsteps) {
  if (!b || !m || nsteps < 0) return GFM_ERR_ARG;
  for (int i = 0; i < b->n; i++) {
    gfm_status_t r = validate_method(b->inst[i], m);
    if (r != GFM_OK) return r;
  }
  const int k = GRAPH_STEPS;
  if (b->schedule == GFM_BATCH_PHASED) {
    gfm_status_t r = prepare_flux_plan(b);
    if (r != GFM_OK) return r;
  }
  if (nsteps >= k && (!b->exec || b->graph_k != k || memcmp(&b->graph_m, m, sizeof(*m)) != 0 ||
                      b->graph_schedule != b->schedule || b->graph_shapes != shapes_of(b))) {
    gfm_status_t r = record_graph(b, m, k);
    if (r != GFM_OK) return r;
  }
  int done = 0;
  if (nsteps >= k) {
    gfm_status_t r = join_instances(b);
    if (r != GFM_OK) return r;
  }
  while (nsteps - done >= k) {
    if (cudaGraphLaunch(b->exec, b->main) != cudaSuccess) return GFM_ERR_CUDA;
    g_launches.fetch_add(b->graph_launches);
    for (gfm_ctx* c : b->inst) c->steps_done_host += k;
    done += k;
  }
  if (done > 0) {
    gfm_status_t r = release_instances(b);
    if (r != GFM_OK) return r;
  }
  if (nsteps > done) {   // the remainder, issued directly (fork, instance streams, join)
    gfm_status_t r = issue(b, b->main, m, nsteps - done);
    if (r != GFM_OK) return r;
  }
  return launch_status();
}

gfm_status_t gfm_step_batched_sequential(gfm_batch* b, const gfm_method_desc* m, int nsteps) {
  if (!b || !m || nsteps < 0) return GFM_ERR_ARG;
  for (int i = 0; i < b->n; i++) {
    gfm_ctx* c = b->inst[i];
    // the instance's earlier work on its own stream comes first
    if (cudaEventRecord(b->join[i], c->stream) != cudaSuccess) return GFM_ERR_CUDA;
    if (cudaStreamWaitEvent(b->main, b->join[i], 0) != cudaSuccess) return GFM_ERR_CUDA;
    cudaStream_t own = c->stream;
    c->stream = b->main;
    gfm_status_t r = run_steps(c, m, nsteps, nullptr);
    c->stream = own;
    if (r != GFM_OK) return r;
    if (cudaEventRecord(b->fork, b->main) != cudaSuccess) return GFM_ERR_CUDA;
    if (cudaStreamWaitEvent(own, b->fork, 0) != cudaSuccess) return GFM_ERR_CUDA;
  }
  return launch_status();
}

gfm_status_t gfm_batch_set_schedule(gfm_batch* b, int schedule) {
  if (!b || (schedule != GFM_BATCH_STREAMS && schedule != GFM_BATCH_PHASED)) return GFM_ERR_ARG;
  b->schedule = schedule;
  return GFM_OK;
}

gfm_status_t gfm_batch_autotune(gfm_batch* b, const gfm_method_desc* m, int steps, char* report, int report_len) {
  if (!b || !m || steps < 1) return GFM_ERR_ARG;
  for (int i = 0; i < b->n; i++) {
    gfm_status_t r = validate_method(b->inst[i], m);
    if (r != GFM_OK) return r;
  }
  steps = (steps + GRAPH_STEPS - 1) / GRAPH_STEPS * GRAPH_STEPS;
  if (cudaStreamSynchronize(b->main) != cudaSuccess) return GFM_ERR_CUDA;
  for (cudaStream_t st : b->streams)
    if (cudaStreamSynchronize(st) != cudaSuccess) return GFM_ERR_CUDA;
  // every instance's state, restored after each trial and at the end
  struct Saved { std::vector<double> U1, U2, phi; double t; int n; };
  std::vector<Saved> saved(b->n);
  for (int i = 0; i < b->n; i++) {
    gfm_ctx* c = b->inst[i];
    const size_t cells = (size_t)c->P.nr * c->P.nc;
    Saved& v = saved[i];
    v.U1.resize(4 * cells);
    if (b->two_fluid) { v.U2.resize(4 * cells); v.phi.resize(cells); }
    gfm_status_t r = gfm_download_state(c, v.U1.data(), b->two_fluid ? v.U2.data() : nullptr,
                                        b->two_fluid ? v.phi.data() : nullptr);
    if (r == GFM_OK) r = gfm_get_time(c, &v.t, &v.n, nullptr);
    if (r != GFM_OK) return r;
  }
  auto restore = [&](int i) -> gfm_status_t {
    gfm_ctx* c = b->inst[i];
    Saved& v = saved[i];
    gfm_status_t r = gfm_upload_state(c, v.U1.data(), b->two_fluid ? v.U2.data() : nullptr,
                                      b->two_fluid ? v.phi.data() : nullptr);
    if (r == GFM_OK) r = gfm_set_time(c, v.t, v.n);
    return r;
  };
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return GFM_ERR_CUDA;
  gfm_status_t r = GFM_OK;
  std::string rep = "{\"classes\": [";
  // 1. the tile shape per grid-size class (padded cells < 2^17, < 2^19,
  //    larger), timed on the class's largest instance stepped alone
  const int64_t bounds[3] = {1ll << 17, 1ll << 19, INT64_MAX};
  bool first_class = true;
  for (int cl = 0; cl < 3 && r == GFM_OK; cl++) {
    int rep_i = -1;
    int64_t lo = cl == 0 ? 0 : bounds[cl - 1], best_cells = -1;
    for (int i = 0; i < b->n; i++) {
      const int64_t cells = (int64_t)b->inst[i]->P.nr * b->inst[i]->P.nc;
      if (cells >= lo && cells < bounds[cl] && cells > best_cells) { best_cells = cells; rep_i = i; }
    }
    if (rep_i < 0) continue;
    gfm_ctx* c = b->inst[rep_i];
    float ms[FLUX_SHAPES];
    int best = 0;
    for (int sh = 0; sh < FLUX_SHAPES && r == GFM_OK; sh++) {
      c->flux_shape = sh;
      r = restore(rep_i);
      if (r == GFM_OK) r = run_steps(c, m, 2, nullptr);   // warm-up (occupancy queries, caches)
      if (r == GFM_OK) r = restore(rep_i);
      if (r != GFM_OK) break;
      cudaEventRecord(e0, c->stream);
      r = run_steps(c, m, steps, nullptr);
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) r = GFM_ERR_CUDA;
      cudaEventElapsedTime(&ms[sh], e0, e1);
      if (ms[sh] < ms[best]) best = sh;
    }
    if (r != GFM_OK) break;
    for (int i = 0; i < b->n; i++) {
      const int64_t cells = (int64_t)b->inst[i]->P.nr * b->inst[i]->P.nc;
      if (cells >= lo && cells < bounds[cl]) b->inst[i]->flux_shape = best;
    }
    r = restore(rep_i);
    char buf[320];
    snprintf(buf, sizeof(buf),
             "%s{\"max_padded_cells\": %lld, \"probe_instance\": %d, \"probe_cells\": %lld, "
             "\"ms_per_step\": {\"32x8\": %.4f, \"16x16\": %.4f, \"64x4\": %.4f, \"16x32\": %.4f}, "
             "\"tile\": \"%s\"}",
             first_class ? "" : ", ", cl == 2 ? -1ll : (long long)bounds[cl], rep_i,
             (long long)(c->P.Nx) * c->P.Ny, ms[0] / steps, ms[1] / steps, ms[2] / steps, ms[3] / steps,
             best == 0 ? "32x8" : (best == 1 ? "16x16" : (best == 2 ? "64x4" : "16x32")));
    rep += buf;
    first_class = false;
  }
  // 2. the schedule, timed on the whole batch with the chosen shapes
  float sms_[2] = {0.0f, 0.0f};
  for (int sc = 0; sc < 2 && r == GFM_OK; sc++) {
    b->schedule = sc == 0 ? GFM_BATCH_STREAMS : GFM_BATCH_PHASED;
    for (int i = 0; i < b->n && r == GFM_OK; i++) r = restore(i);
    if (r == GFM_OK) r = gfm_step_batched_graph(b, m, GRAPH_STEPS);   // records the graph (warm-up)
    if (r == GFM_OK && cudaStreamSynchronize(b->main) != cudaSuccess) r = GFM_ERR_CUDA;
    for (int i = 0; i < b->n && r == GFM_OK; i++) r = restore(i);
    if (r != GFM_OK) break;
    cudaEventRecord(e0, b->main);
    r = gfm_step_batched_graph(b, m, steps);
    cudaEventRecord(e1, b->main);
    if (cudaEventSynchronize(e1) != cudaSuccess) r = GFM_ERR_CUDA;
    cudaEventElapsedTime(&sms_[sc], e0, e1);
  }
  if (r == GFM_OK) b->schedule = sms_[1] < sms_[0] ? GFM_BATCH_PHASED : GFM_BATCH_STREAMS;
  // 3. the chosen tiles against the default tile (16x32) of every instance,
  //    on the whole batch with the chosen schedule: a shape that wins on one
  //    instance stepped alone can lose when the instances share the GPU
  float tms[2] = {0.0f, 0.0f};
  std::vector<int> chosen(b->n);
  bool differs = false;
  for (int i = 0; i < b->n; i++) {
    chosen[i] = b->inst[i]->flux_shape;
    differs = differs || chosen[i] != FLUX_SHAPE_DEFAULT;
  }
  bool keep_chosen = true;
  if (r == GFM_OK && differs) {
    for (int v = 0; v < 2 && r == GFM_OK; v++) {
      for (int i = 0; i < b->n; i++) b->inst[i]->flux_shape = v == 0 ? chosen[i] : FLUX_SHAPE_DEFAULT;
      for (int i = 0; i < b->n && r == GFM_OK; i++) r = restore(i);
      if (r == GFM_OK) r = gfm_step_batched_graph(b, m, GRAPH_STEPS);   // records the graph (warm-up)
      if (r == GFM_OK && cudaStreamSynchronize(b->main) != cudaSuccess) r = GFM_ERR_CUDA;
      for (int i = 0; i < b->n && r == GFM_OK; i++) r = restore(i);
      if (r != GFM_OK) break;
      cudaEventRecord(e0, b->main);
      r = gfm_step_batched_graph(b, m, steps);
      cudaEventRecord(e1, b->main);
      if (cudaEventSynchronize(e1) != cudaSuccess) r = GFM_ERR_CUDA;
      cudaEventElapsedTime(&tms[v], e0, e1);
    }
    keep_chosen = !(tms[1] < tms[0]);
    for (int i = 0; i < b->n; i++) b->inst[i]->flux_shape = keep_chosen ? chosen[i] : FLUX_SHAPE_DEFAULT;
  }
  if (r == GFM_OK) {
    for (int i = 0; i < b->n && r == GFM_OK; i++) r = restore(i);
    if (r == GFM_OK && cudaStreamSynchronize(b->main) != cudaSuccess) r = GFM_ERR_CUDA;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r != GFM_OK) return r;
  char buf[384];
  snprintf(buf, sizeof(buf),
           "], \"steps\": %d, \"schedule_ms_per_step\": {\"streams\": %.4f, \"phased\": %.4f}, "
           "\"schedule\": \"%s\", \"tiles_on_batch_ms_per_step\": {\"chosen\": %.4f, \"default\": %.4f}, "
           "\"tiles\": \"%s\"}",
           steps, sms_[0] / steps, sms_[1] / steps, b->schedule == GFM_BATCH_PHASED ? "phased" : "streams",
           tms[0] / steps, tms[1] / steps, keep_chosen ? "per class" : "default everywhere");
  rep += buf;
  if (report && report_len > 0) {
    strncpy(report, rep.c_str(), (size_t)report_len - 1);
    report[report_len - 1] = 0;
  }
  return GFM_OK;
}

gfm_status_t gfm_batch_synchronize(gfm_batch* b) {
  if (!b) return GFM_ERR_ARG;
  if (cudaStreamSynchronize(b->main) != cudaSuccess) return GFM_ERR_CUDA;
  return GFM_OK;
}

}  // extern "C"
