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
#include "gfm_internal.cuh"
#include <cstring>
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
    gfm_status_t ri = issue_steps(b, b->cap, m, k);
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
  if (nsteps >= k && (!b->exec || b->graph_k != k || memcmp(&b->graph_m, m, sizeof(*m)) != 0)) {
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
    gfm_status_t r = issue_steps(b, b->main, m, nsteps - done);
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

gfm_status_t gfm_batch_synchronize(gfm_batch* b) {
  if (!b) return GFM_ERR_ARG;
  if (cudaStreamSynchronize(b->main) != cudaSuccess) return GFM_ERR_CUDA;
  return GFM_OK;
}

}  // extern "C"
