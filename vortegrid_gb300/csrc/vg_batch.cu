// Batched effects: many independent VortonSim steps per frame (no counterpart
// in the reference, whose VortonSim steps one fluid per call).
//
// Every simulation is a context (Poisson technique, fixed grid) with its
// vortons resident on the device.  A frame steps all of them: the step
// (treecode boundary, splat, optional network guess, multigrid, curl, PSE,
// gather) and the vortons' Euler advection.  Host round trips are removed so
// the frame can be captured once as CUDA graphs and replayed:
//   * fixed grids (no bounding-box readback); a vorton that leaves its grid
//     stops and drops out of the solve instead of failing the frame;
//   * a fixed multigrid schedule per simulation, calibrated by one adaptive
//     solve (its phase-1 cycles, and its refinement cycles + 1);
//   * workspaces grown to their final sizes by the calibration step.
// The simulations are dealt round-robin to K branch streams.  Each branch's
// chain of simulations is captured as graphs of at most about kGraphKernels
// kernels (a frame of 256 simulations is ~10^5 kernels; a graph that size
// would be one very deep chain), launched in order on that branch.  A frame
// forks from the batch's main stream into the K branches, launches their
// graphs and joins back, so the GPU runs independent simulations concurrently
// and the host issues a few graph launches per frame.  The autotuner picks K,
// and whether the network warm start pays off, by timing replays.  A
// sequential mode runs the same work simulation after simulation on the main
// stream without graphs, for comparison.
#include <algorithm>
#include <new>
#include <vector>

#include "vg_internal.cuh"

struct vg_ctx : public vg::Ctx {};
struct vg_net;

using namespace vg;

namespace {

constexpr int kMaxStreams = 32;
constexpr unsigned kGraphKernels = 3072;  // a graph ends after the simulation that reaches this

struct Sim {
  vg_ctx* ctx = nullptr;
  float* pos = nullptr;  // float4 per vorton: position, size
  float* w = nullptr;    // float4: angular velocity (updated by PSE)
  float* vel = nullptr;  // float4: velocity (written)
  size_t n = 0;
  bool net_ok = false;   // a network of this simulation's grid edge is loaded
};

struct Chunk {
  cudaGraphExec_t exec = nullptr;
  int stream = 0;
  size_t nodes = 0;
};

}  // namespace

struct vg_batch {
  int device = 0;
  std::string err;
  cudaStream_t main = nullptr;
  cudaStream_t streams[kMaxStreams] = {};
  cudaEvent_t fork = nullptr, join[kMaxStreams] = {};
  int nstreams = 1;
  std::vector<Sim> sims;
  // networks: per grid edge, one per stream (a network's buffers serve one stream at a time)
  std::vector<unsigned> net_edges;
  std::vector<std::vector<vg_net*>> nets;  // [edge index][stream]
  bool use_network = false;
  bool calibrated = false;
  std::vector<Chunk> chunks;  // the frame's graphs, in launch order within each branch
  float graph_dt = 0.f;
  int graph_streams = 0;
  bool graph_network = false;
};

extern "C" {
vg_status vg_step_device(vg_ctx* ctx, const float* pos_size, float* angvel, float* vel, size_t n,
                         const float* extra_minmax, float dt, unsigned frame);
vg_status vg_evolve_device(vg_ctx* ctx, float* pos4, const float* vel4, size_t m, float dt);
vg_status vg_set_network(vg_ctx* ctx, vg_net* net);
vg_status vg_net_create(int device, void* stream, unsigned edge, vg_net** out);
vg_status vg_net_destroy(vg_net* net);
vg_status vg_net_load(vg_net* net, const char* path);
}

namespace {

vg_status bfail(vg_batch* b, vg_status s, const std::string& msg) {
  b->err = msg;
  return s;
}

vg_status bcuda(vg_batch* b, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return VG_OK;
  cudaGetLastError();
  return bfail(b, e == cudaErrorMemoryAllocation ? VG_OOM : VG_CUDA_ERROR,
               std::string(what) + ": " + cudaGetErrorString(e));
}

void drop_graph(vg_batch* b) {
  for (Chunk& k : b->chunks)
    if (k.exec) cudaGraphExecDestroy(k.exec);
  b->chunks.clear();
}

// Points the simulation at stream s and, if the batch uses the network and one
// fits its grid, at that stream's network.
void bind(vg_batch* b, Sim& sim, int s) {
  sim.ctx->stream = b->streams[s];
  vg_net* net = nullptr;
  if (b->use_network && sim.net_ok) {
    const unsigned edge = sim.ctx->cfg.fixed_grid.num_points[0] - 1;
    for (size_t e = 0; e < b->net_edges.size(); ++e)
      if (b->net_edges[e] == edge) net = b->nets[e][s];
  }
  vg_set_network(sim.ctx, net);
  sim.ctx->cfg.warm_start = net ? VG_WARM_NETWORK : VG_WARM_ZERO;
}

vg_status step_one(vg_batch* b, Sim& sim, float dt) {
  vg_status st = vg_step_device(sim.ctx, sim.pos, sim.w, sim.vel, sim.n, nullptr, dt, 0);
  if (st != VG_OK) return bfail(b, st, std::string("step: ") + sim.ctx->err);
  st = vg_evolve_device(sim.ctx, sim.pos, sim.vel, sim.n, dt);
  if (st != VG_OK) return bfail(b, st, std::string("evolve: ") + sim.ctx->err);
  return VG_OK;
}

// Captures branch s's simulations *i, *i + K, ... until the graph holds
// kGraphKernels kernels or the branch ends; *i moves past them.
vg_status capture_chunk(vg_batch* b, int s, size_t* i, float dt) {
  const size_t K = (size_t)b->nstreams;
  cudaStream_t cs = b->streams[s];
  vg_status st;
  if ((st = bcuda(b, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture")) != VG_OK)
    return st;
  vg_status est = VG_OK;
  unsigned kernels = 0;
  while (*i < b->sims.size() && kernels < kGraphKernels) {
    Sim& sim = b->sims[*i];
    bind(b, sim, s);
    if ((est = step_one(b, sim, dt)) != VG_OK) break;
    kernels += sim.ctx->launches + 1;  // the step's kernels and the advection
    *i += K;
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
  if (est != VG_OK) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return est;
  }
  if ((st = bcuda(b, ce, "end capture")) != VG_OK) return st;
  Chunk k;
  k.stream = s;
  cudaGraphGetNodes(graph, nullptr, &k.nodes);
  const cudaError_t ie = cudaGraphInstantiate(&k.exec, graph, 0);
  cudaGraphDestroy(graph);
  if ((st = bcuda(b, ie, "instantiate")) != VG_OK) return st;
  b->chunks.push_back(k);
  return VG_OK;
}

vg_status capture(vg_batch* b, float dt) {
  drop_graph(b);
  vg_status st;
  for (int s = 0; s < b->nstreams; ++s) {
    size_t i = (size_t)s;
    while (i < b->sims.size())
      if ((st = capture_chunk(b, s, &i, dt)) != VG_OK) {
        drop_graph(b);
        return st;
      }
  }
  b->graph_dt = dt;
  b->graph_streams = b->nstreams;
  b->graph_network = b->use_network;
  return VG_OK;
}

// One frame from the captured graphs: fork from main, each branch's graphs in
// capture order on its stream, join.
vg_status launch_frame(vg_batch* b) {
  vg_status st;
  const int K = b->graph_streams;
  if ((st = bcuda(b, cudaEventRecord(b->fork, b->main), "fork")) != VG_OK) return st;
  for (int s = 0; s < K; ++s)
    if ((st = bcuda(b, cudaStreamWaitEvent(b->streams[s], b->fork, 0), "fork wait")) != VG_OK) return st;
  for (const Chunk& k : b->chunks)
    if ((st = bcuda(b, cudaGraphLaunch(k.exec, b->streams[k.stream]), "graph launch")) != VG_OK) return st;
  for (int s = 0; s < K; ++s) {
    if ((st = bcuda(b, cudaEventRecord(b->join[s], b->streams[s]), "join")) != VG_OK) return st;
    if ((st = bcuda(b, cudaStreamWaitEvent(b->main, b->join[s], 0), "join wait")) != VG_OK) return st;
  }
  return VG_OK;
}

vg_status calibrate(vg_batch* b, float dt) {
  // one adaptive step per simulation: grows its workspaces, records its schedule
  vg_status st;
  drop_graph(b);
  // earlier frames may have run on other streams than the ones used below
  if ((st = bcuda(b, cudaStreamSynchronize(b->main), "synchronize")) != VG_OK) return st;
  for (int s = 0; s < kMaxStreams; ++s)
    if ((st = bcuda(b, cudaStreamSynchronize(b->streams[s]), "synchronize")) != VG_OK) return st;
  for (size_t i = 0; i < b->sims.size(); ++i) {
    Sim& sim = b->sims[i];
    sim.ctx->mg_fixed_k1 = sim.ctx->mg_fixed_k2 = 0;
    bind(b, sim, (int)(i % b->nstreams));
    if ((st = step_one(b, sim, dt)) != VG_OK) return st;
  }
  for (Sim& sim : b->sims) {
    if ((st = sync_and_check(sim.ctx, "calibration")) != VG_OK) return bfail(b, st, sim.ctx->err);
    sim.ctx->mg_fixed_k1 = std::max(1, sim.ctx->mg_last_k1);
    sim.ctx->mg_fixed_k2 = sim.ctx->mg_last_k2 + 1;
  }
  b->calibrated = true;
  return VG_OK;
}

vg_status timed_frames(vg_batch* b, int frames, float* ms) {
  vg_status st;
  cudaEvent_t e0, e1;
  *ms = 0.f;
  if ((st = bcuda(b, cudaEventCreate(&e0), "event")) != VG_OK) return st;
  if ((st = bcuda(b, cudaEventCreate(&e1), "event")) != VG_OK) {
    cudaEventDestroy(e0);
    return st;
  }
  st = launch_frame(b);  // warm-up
  if (st == VG_OK) st = bcuda(b, cudaEventRecord(e0, b->main), "event");
  for (int f = 0; f < frames && st == VG_OK; ++f) st = launch_frame(b);
  if (st == VG_OK) st = bcuda(b, cudaEventRecord(e1, b->main), "event");
  if (st == VG_OK) st = bcuda(b, cudaEventSynchronize(e1), "event sync");
  if (st == VG_OK) cudaEventElapsedTime(ms, e0, e1);
  *ms /= std::max(1, frames);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

}  // namespace

extern "C" {

vg_status vg_batch_create(int device, int streams, vg_batch** out) {
  if (!out) return set_noctx_error(VG_INVALID, "vg_batch_create: null output");
  *out = nullptr;
  if (streams < 1 || streams > kMaxStreams) return set_noctx_error(VG_INVALID, "vg_batch_create: streams in 1..32");
  vg_batch* b = new (std::nothrow) vg_batch();
  if (!b) return set_noctx_error(VG_OOM, "vg_batch_create: out of host memory");
  b->device = device;
  b->nstreams = streams;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking);
  for (int s = 0; s < kMaxStreams && e == cudaSuccess; ++s) {
    e = cudaStreamCreateWithFlags(&b->streams[s], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[s], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_noctx_error(VG_CUDA_ERROR, std::string("vg_batch_create: ") + cudaGetErrorString(e));
    delete b;  // the handles created so far are released with the process
    return VG_CUDA_ERROR;
  }
  *out = b;
  return VG_OK;
}

vg_status vg_batch_destroy(vg_batch* b) {
  if (!b) return VG_OK;
  if (b->main) cudaStreamSynchronize(b->main);
  for (int s = 0; s < kMaxStreams; ++s)
    if (b->streams[s]) cudaStreamSynchronize(b->streams[s]);
  drop_graph(b);
  for (Sim& s : b->sims) vg_destroy(s.ctx);
  for (auto& v : b->nets)
    for (vg_net* n : v) vg_net_destroy(n);
  for (int s = 0; s < kMaxStreams; ++s) {
    if (b->streams[s]) cudaStreamDestroy(b->streams[s]);
    if (b->join[s]) cudaEventDestroy(b->join[s]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->main) cudaStreamDestroy(b->main);
  delete b;
  return VG_OK;
}

const char* vg_batch_last_error(const vg_batch* b) { return b ? b->err.c_str() : ""; }

vg_status vg_batch_add(vg_batch* b, const vg_config* cfg, float* pos_size, float* angvel, float* vel, size_t n,
                       int* index) {
  if (!b || !cfg || !pos_size || !angvel || !vel || n == 0) return VG_INVALID;
  if (!cfg->use_fixed_grid || cfg->velocity_technique != VG_VELOCITY_POISSON ||
      cfg->poisson_solver != VG_POISSON_MULTIGRID)
    return bfail(b, VG_INVALID, "vg_batch_add: a batched simulation needs a fixed grid and the multigrid Poisson step");
  vg_config c = *cfg;
  c.stream = b->streams[0];
  c.device = b->device;
  vg_ctx* ctx = nullptr;
  const vg_status st = vg_create(&c, &ctx);
  if (st != VG_OK) return bfail(b, st, std::string("vg_batch_add: ") + vg_last_error(nullptr));
  ctx->freeze_outside = true;  // a vorton that leaves its fixed grid stops and drops out of the solve
  Sim s;
  s.ctx = ctx;
  s.pos = pos_size;
  s.w = angvel;
  s.vel = vel;
  s.n = n;
  b->sims.push_back(s);
  drop_graph(b);
  b->calibrated = false;
  if (index) *index = (int)b->sims.size() - 1;
  return VG_OK;
}

vg_status vg_batch_load_network(vg_batch* b, const char* path) {
  if (!b || !path) return VG_INVALID;
  std::vector<unsigned> edges;
  for (const Sim& s : b->sims) {
    const unsigned* np = s.ctx->cfg.fixed_grid.num_points;
    const unsigned e = np[0] - 1;
    if (np[1] == np[0] && np[2] == np[0] && std::find(edges.begin(), edges.end(), e) == edges.end()) edges.push_back(e);
  }
  for (unsigned edge : edges) {
    if (std::find(b->net_edges.begin(), b->net_edges.end(), edge) != b->net_edges.end()) continue;
    std::vector<vg_net*> per_stream;
    vg_status st = VG_OK;
    for (int s = 0; s < kMaxStreams && st == VG_OK; ++s) {
      vg_net* net = nullptr;
      st = vg_net_create(b->device, b->streams[s], edge, &net);
      if (st == VG_OK) st = vg_net_load(net, path);
      if (st == VG_OK)
        per_stream.push_back(net);
      else if (net)
        vg_net_destroy(net);
    }
    if (st != VG_OK) {  // this edge does not suit the network: those simulations start from zero
      for (vg_net* n : per_stream) vg_net_destroy(n);
      if (st == VG_INVALID) continue;
      return bfail(b, st, "vg_batch_load_network: " + std::string(vg_last_error(nullptr)));
    }
    b->net_edges.push_back(edge);
    b->nets.push_back(per_stream);
  }
  for (Sim& s : b->sims) {
    const unsigned e = s.ctx->cfg.fixed_grid.num_points[0] - 1;
    s.net_ok = std::find(b->net_edges.begin(), b->net_edges.end(), e) != b->net_edges.end();
  }
  b->use_network = !b->net_edges.empty();
  b->calibrated = false;
  drop_graph(b);
  return VG_OK;
}

vg_status vg_batch_configure(vg_batch* b, int streams, int use_network) {
  if (!b || streams < 1 || streams > kMaxStreams) return VG_INVALID;
  const bool net = use_network != 0 && !b->net_edges.empty();
  if (net != b->use_network) b->calibrated = false;  // the schedules depend on the start
  b->nstreams = streams;
  b->use_network = net;
  drop_graph(b);
  return VG_OK;
}

vg_status vg_batch_calibrate(vg_batch* b, float dt) {
  if (!b) return VG_INVALID;
  if (b->sims.empty()) return bfail(b, VG_EMPTY, "vg_batch_calibrate: no simulations");
  return calibrate(b, dt);
}

// mode 0: the captured graphs (captured on first use or after a change);
// mode 1: the same work simulation after simulation on the main stream.
vg_status vg_batch_step(vg_batch* b, float dt, int mode) {
  if (!b || (mode != 0 && mode != 1)) return VG_INVALID;
  if (b->sims.empty()) return bfail(b, VG_EMPTY, "vg_batch_step: no simulations");
  vg_status st;
  if (!b->calibrated && (st = calibrate(b, dt)) != VG_OK) return st;
  if (mode == 1) {
    for (Sim& sim : b->sims) {
      bind(b, sim, 0);
      sim.ctx->stream = b->main;
      if ((st = step_one(b, sim, dt)) != VG_OK) return st;
    }
    return VG_OK;
  }
  if (b->chunks.empty() || b->graph_dt != dt || b->graph_streams != b->nstreams || b->graph_network != b->use_network)
    if ((st = capture(b, dt)) != VG_OK) return st;
  return launch_frame(b);
}

vg_status vg_batch_synchronize(vg_batch* b) {
  if (!b) return VG_INVALID;
  vg_status st = bcuda(b, cudaStreamSynchronize(b->main), "synchronize");
  if (st != VG_OK) return st;
  for (Sim& s : b->sims)
    if ((st = sync_and_check(s.ctx, "batched step")) != VG_OK) return bfail(b, st, s.ctx->err);
  return VG_OK;
}

// Times `frames` graph replays for every stream count in `candidates` (and,
// when a network is loaded, with and without it), keeps the fastest setting
// and reports it.  Steps the simulations while it measures.
vg_status vg_batch_autotune(vg_batch* b, float dt, int frames, const int* candidates, int ncand, int* best_streams,
                            int* best_network, float* best_ms) {
  if (!b || !candidates || ncand < 1 || frames < 1) return VG_INVALID;
  if (b->sims.empty()) return bfail(b, VG_EMPTY, "vg_batch_autotune: no simulations");
  for (int k = 0; k < ncand; ++k)
    if (candidates[k] < 1 || candidates[k] > kMaxStreams) return VG_INVALID;
  float best = 3.4e38f;
  int bs = b->nstreams, bn = b->use_network ? 1 : 0;
  const int nets = b->net_edges.empty() ? 1 : 2;
  vg_status st;
  for (int net = 0; net < nets; ++net) {
    if ((st = vg_batch_configure(b, candidates[0], net)) != VG_OK) return st;
    if ((st = calibrate(b, dt)) != VG_OK) return st;
    for (int k = 0; k < ncand; ++k) {
      b->nstreams = candidates[k];
      if ((st = capture(b, dt)) != VG_OK) return st;
      float ms = 0.f;
      if ((st = timed_frames(b, frames, &ms)) != VG_OK) return st;
      if (ms < best) {
        best = ms;
        bs = candidates[k];
        bn = net;
      }
    }
  }
  if ((st = vg_batch_configure(b, bs, bn)) != VG_OK) return st;
  if ((st = calibrate(b, dt)) != VG_OK) return st;
  if (best_streams) *best_streams = bs;
  if (best_network) *best_network = bn;
  if (best_ms) *best_ms = best;
  return VG_OK;
}

vg_status vg_batch_outside(vg_batch* b, int index, int* outside) {
  if (!b || !outside || index < 0 || index >= (int)b->sims.size()) return VG_INVALID;
  vg_status st = bcuda(b, cudaStreamSynchronize(b->main), "synchronize");
  if (st != VG_OK) return st;
  Ctx* c = b->sims[index].ctx;
  if ((st = bcuda(b, cudaStreamSynchronize(c->stream), "synchronize")) != VG_OK) return st;
  int h = 0;
  if ((st = bcuda(b, cudaMemcpy(&h, c->dflag + 1, sizeof(int), cudaMemcpyDeviceToHost), "read")) != VG_OK) return st;
  if (h && (st = bcuda(b, cudaMemset(c->dflag + 1, 0, sizeof(int)), "clear")) != VG_OK) return st;
  *outside = h != 0;
  return VG_OK;
}

vg_ctx* vg_batch_context(vg_batch* b, int index) {
  if (!b || index < 0 || index >= (int)b->sims.size()) return nullptr;
  return b->sims[index].ctx;
}

int vg_batch_size(const vg_batch* b) { return b ? (int)b->sims.size() : 0; }

vg_status vg_batch_graph_info(const vg_batch* b, int* graphs, size_t* max_nodes, size_t* total_nodes) {
  if (!b) return VG_INVALID;
  size_t mx = 0, tot = 0;
  for (const Chunk& k : b->chunks) {
    mx = std::max(mx, k.nodes);
    tot += k.nodes;
  }
  if (graphs) *graphs = (int)b->chunks.size();
  if (max_nodes) *max_nodes = mx;
  if (total_nodes) *total_nodes = tot;
  return VG_OK;
}

}  // extern "C"
