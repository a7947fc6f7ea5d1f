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
//   * a fixed multigrid schedule per simulation, calibrated by adaptive
//     solves (its phase-1 cycles and refinement cycles, plus a spare
//     refinement cycle when the calibrating solve ended close to the
//     tolerance), each solve
//     starting from the simulation's previous solution (or the network's
//     guess);
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
//
// With the persistent solve (vg_batch_set_solver), a frame has three parts: each
// simulation's step up to its Poisson solve on the branches; one cooperative
// launch on the main stream that runs every qualifying simulation's
// fixed-schedule multigrid solve, teams of CTAs taking the simulations longest
// first (mg_batch_* in vg_mg.cu); then the rest of each step and the
// advection on the branches.  The solve's results are bit-identical to the
// per-simulation launches.  The autotuner also decides between the two forms
// and picks the team size.
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
  int part = 0;  // 0: before the persistent solve (or whole steps), 1: after it
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
  // persistent solve
  bool persistent = false;
  int team_ctas = 0;                   // CTAs per team (0: automatic)
  size_t max_points = 0;               // largest grid (points) the persistent launch takes (0: any)
  std::vector<char> split;             // per simulation: solved by the persistent launch
  MgBatch* mg = nullptr;               // that launch (null: every step whole in the branches)
  cudaGraphExec_t mg_exec = nullptr;   // ... captured as a graph (null: launched directly)
  bool graph_persistent = false;
  int graph_team = 0;
  size_t graph_max_points = 0;
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
  if (b->mg_exec) cudaGraphExecDestroy(b->mg_exec);
  b->mg_exec = nullptr;
  mg_batch_destroy(b->mg);
  b->mg = nullptr;
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
  // without the network, each solve starts from the simulation's previous solution
  sim.ctx->cfg.warm_start = net ? VG_WARM_NETWORK : VG_WARM_PREVIOUS;
}

// part 0: the whole step and the advection; 1: the step up to its Poisson
// solve; 2: the rest of the step (resuming part 1) and the advection.
vg_status step_one(vg_batch* b, Sim& sim, float dt, int part = 0) {
  sim.ctx->step_split = part;
  vg_status st = vg_step_device(sim.ctx, sim.pos, sim.w, sim.vel, sim.n, nullptr, dt, 0);
  sim.ctx->step_split = 0;
  if (st != VG_OK) return bfail(b, st, std::string("step: ") + sim.ctx->err);
  if (part == 1) return VG_OK;
  st = vg_evolve_device(sim.ctx, sim.pos, sim.vel, sim.n, dt);
  if (st != VG_OK) return bfail(b, st, std::string("evolve: ") + sim.ctx->err);
  return VG_OK;
}

// Captures branch s's simulations list[*i], list[*i + 1], ... (their `parts`)
// until the graph holds kGraphKernels kernels or the list ends; *i moves past
// them.  The chunk runs in frame part `fpart`.
vg_status capture_chunk(vg_batch* b, int s, const std::vector<size_t>& list, const std::vector<int>& parts,
                        size_t* i, float dt, int fpart) {
  cudaStream_t cs = b->streams[s];
  vg_status st;
  if ((st = bcuda(b, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture")) != VG_OK)
    return st;
  vg_status est = VG_OK;
  unsigned kernels = 0;
  while (*i < list.size() && kernels < kGraphKernels) {
    Sim& sim = b->sims[list[*i]];
    bind(b, sim, s);
    const unsigned before = parts[*i] == 2 ? sim.ctx->launches : 0;
    if ((est = step_one(b, sim, dt, parts[*i])) != VG_OK) break;
    kernels += sim.ctx->launches - before + 1;  // the step's kernels and the advection
    ++*i;
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
  k.part = fpart;
  cudaGraphGetNodes(graph, nullptr, &k.nodes);
  const cudaError_t ie = cudaGraphInstantiate(&k.exec, graph, 0);
  cudaGraphDestroy(graph);
  if ((st = bcuda(b, ie, "instantiate")) != VG_OK) return st;
  b->chunks.push_back(k);
  return VG_OK;
}

// Captures branch s's simulations in frame part fpart (list: simulation
// indices, parts: the step part of each).
vg_status capture_branch(vg_batch* b, int s, const std::vector<size_t>& list, const std::vector<int>& parts, float dt,
                         int fpart) {
  size_t i = 0;
  vg_status st;
  while (i < list.size())
    if ((st = capture_chunk(b, s, list, parts, &i, dt, fpart)) != VG_OK) return st;
  return VG_OK;
}

vg_status capture(vg_batch* b, float dt) {
  drop_graph(b);
  vg_status st = VG_OK;
  const size_t N = b->sims.size();
  const int K = b->nstreams;
  // the simulations the persistent launch solves: a calibrated fixed
  // schedule whose hierarchy ends in the global sine-transform solve
  b->split.assign(N, 0);
  size_t nsplit = 0;
  for (size_t i = 0; i < N && b->persistent; ++i) {
    const Ctx* c = b->sims[i].ctx;
    const Geom g = to_geom(c->cfg.fixed_grid);
    if (c->mg_fixed_k1 > 0 && mg_batch_eligible(g) && (b->max_points == 0 || g.points() <= b->max_points)) {
      b->split[i] = 1;
      ++nsplit;
    }
  }
  for (int s = 0; s < K && st == VG_OK; ++s) {
    std::vector<size_t> list;
    std::vector<int> parts;
    for (size_t i = (size_t)s; i < N; i += (size_t)K) {
      list.push_back(i);
      parts.push_back(b->split[i] ? 1 : 0);
    }
    st = capture_branch(b, s, list, parts, dt, 0);
  }
  if (st == VG_OK && nsplit > 0) {
    std::vector<MgBatchItem> items;
    for (size_t i = 0; i < N && st == VG_OK; ++i) {
      MgBatchItem it;
      if (!b->split[i]) continue;
      if (split_problem(b->sims[i].ctx, &it))
        items.push_back(it);
      else
        st = bfail(b, VG_INVALID, "persistent solve: a step did not stop before its solve");
    }
    std::string err;
    if (st != VG_OK) {
    } else if ((st = mg_batch_build(items, b->device, b->team_ctas, &b->mg, &err)) != VG_OK) {
      bfail(b, st, err);
    } else {
      // the launch as a graph of its own where capture takes it; launched directly otherwise
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const vg_status est = mg_batch_enqueue(b->mg, b->main, &err);
        const cudaError_t ce = cudaStreamEndCapture(b->main, &graph);
        if (est != VG_OK || ce != cudaSuccess || !graph || cudaGraphInstantiate(&b->mg_exec, graph, 0) != cudaSuccess)
          b->mg_exec = nullptr;
        if (graph) cudaGraphDestroy(graph);
      }
      cudaGetLastError();
      for (int s = 0; s < K && st == VG_OK; ++s) {
        std::vector<size_t> list;
        for (size_t i = (size_t)s; i < N; i += (size_t)K)
          if (b->split[i]) list.push_back(i);
        st = capture_branch(b, s, list, std::vector<int>(list.size(), 2), dt, 1);
      }
    }
  }
  if (st != VG_OK) {
    drop_graph(b);
    return st;
  }
  b->graph_dt = dt;
  b->graph_streams = b->nstreams;
  b->graph_network = b->use_network;
  b->graph_persistent = b->persistent;
  b->graph_team = b->team_ctas;
  b->graph_max_points = b->max_points;
  return VG_OK;
}

vg_status fork_join_part(vg_batch* b, int part) {
  vg_status st;
  const int K = b->graph_streams;
  if ((st = bcuda(b, cudaEventRecord(b->fork, b->main), "fork")) != VG_OK) return st;
  for (int s = 0; s < K; ++s)
    if ((st = bcuda(b, cudaStreamWaitEvent(b->streams[s], b->fork, 0), "fork wait")) != VG_OK) return st;
  for (const Chunk& k : b->chunks)
    if (k.part == part && (st = bcuda(b, cudaGraphLaunch(k.exec, b->streams[k.stream]), "graph launch")) != VG_OK)
      return st;
  for (int s = 0; s < K; ++s) {
    if ((st = bcuda(b, cudaEventRecord(b->join[s], b->streams[s]), "join")) != VG_OK) return st;
    if ((st = bcuda(b, cudaStreamWaitEvent(b->main, b->join[s], 0), "join wait")) != VG_OK) return st;
  }
  return VG_OK;
}

// One frame from the captured graphs: fork from main, each branch's graphs in
// capture order on its stream, join; with the persistent solve, that for the
// steps up to the solve, then the solve on main, then again for the rest.
vg_status launch_frame(vg_batch* b) {
  vg_status st;
  if ((st = fork_join_part(b, 0)) != VG_OK || !b->mg) return st;
  if (b->mg_exec) {
    if ((st = bcuda(b, cudaGraphLaunch(b->mg_exec, b->main), "graph launch")) != VG_OK) return st;
  } else {
    std::string err;
    if ((st = mg_batch_enqueue(b->mg, b->main, &err)) != VG_OK) return bfail(b, st, err);
  }
  return fork_join_part(b, 1);
}

vg_status calibrate(vg_batch* b, float dt) {
  // two adaptive steps per simulation: they grow its workspaces, and the
  // second, started from the first's solution like every later frame,
  // records its schedule
  vg_status st;
  drop_graph(b);
  // earlier frames may have run on other streams than the ones used below
  if ((st = bcuda(b, cudaStreamSynchronize(b->main), "synchronize")) != VG_OK) return st;
  for (int s = 0; s < kMaxStreams; ++s)
    if ((st = bcuda(b, cudaStreamSynchronize(b->streams[s]), "synchronize")) != VG_OK) return st;
  for (int pass = 0; pass < 2; ++pass)
    for (size_t i = 0; i < b->sims.size(); ++i) {
      Sim& sim = b->sims[i];
      sim.ctx->mg_fixed_k1 = sim.ctx->mg_fixed_k2 = 0;
      bind(b, sim, (int)(i % b->nstreams));
      if ((st = step_one(b, sim, dt)) != VG_OK) return st;
    }
  for (Sim& sim : b->sims) {
    if ((st = sync_and_check(sim.ctx, "calibration")) != VG_OK) return bfail(b, st, sim.ctx->err);
    sim.ctx->mg_fixed_k1 = std::max(1, sim.ctx->mg_last_k1);
    // a spare refinement cycle (about a tenfold reduction) unless the
    // calibrating solve already ended ten times below the tolerance
    const bool close = sim.ctx->stats.poisson_relres > 0.1 * sim.ctx->cfg.poisson_tolerance;
    sim.ctx->mg_fixed_k2 = sim.ctx->mg_last_k2 + (close ? 1 : 0);
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
  if (b->chunks.empty() || b->graph_dt != dt || b->graph_streams != b->nstreams ||
      b->graph_network != b->use_network || b->graph_persistent != b->persistent || b->graph_team != b->team_ctas ||
      b->graph_max_points != b->max_points)
    if ((st = capture(b, dt)) != VG_OK) return st;
  return launch_frame(b);
}

vg_status vg_batch_synchronize(vg_batch* b) {
  if (!b) return VG_INVALID;
  vg_status st = bcuda(b, cudaStreamSynchronize(b->main), "synchronize");
  if (st != VG_OK) return st;
  if (b->mg && mg_batch_failed(b->mg))
    return bfail(b, VG_TIMEOUT, "persistent solve: a team barrier gave up (its fields are incomplete)");
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
  const bool pers0 = b->persistent;
  const int team0 = b->team_ctas;
  bool bp = pers0;
  int bt = team0;
  const int nets = b->net_edges.empty() ? 1 : 2;
  vg_status st;
  auto trial = [&](int net) -> vg_status {
    vg_status s2;
    if ((s2 = capture(b, dt)) != VG_OK) return s2;
    float ms = 0.f;
    if ((s2 = timed_frames(b, frames, &ms)) != VG_OK) return s2;
    if (ms < best) {
      best = ms;
      bs = b->nstreams;
      bn = net;
      bp = b->persistent;
      bt = b->team_ctas;
    }
    return VG_OK;
  };
  for (int net = 0; net < nets; ++net) {
    if ((st = vg_batch_configure(b, candidates[0], net)) != VG_OK) return st;
    if ((st = calibrate(b, dt)) != VG_OK) return st;
    for (int k = 0; k < ncand; ++k) {
      b->nstreams = candidates[k];
      if ((st = trial(net)) != VG_OK) return st;
    }
  }
  // the solver at the best stream count: in the branches, or persistent with teams of 4-32 CTAs
  if ((st = vg_batch_configure(b, bs, bn)) != VG_OK) return st;
  if ((st = calibrate(b, dt)) != VG_OK) return st;
  const int teams[] = {0, 4, 8, 16, 32};
  for (int t : teams) {
    b->persistent = t > 0;
    b->team_ctas = t > 0 ? t : team0;
    if (b->persistent == pers0 && (!pers0 || b->team_ctas == team0)) continue;  // measured above
    if ((st = trial(bn)) != VG_OK) return st;
  }
  b->persistent = bp;
  b->team_ctas = bt;
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

vg_status vg_batch_set_solver(vg_batch* b, int persistent, int team_ctas, size_t max_points) {
  if (!b || team_ctas < 0 || team_ctas > 1024) return VG_INVALID;
  b->persistent = persistent != 0;
  b->team_ctas = team_ctas;
  b->max_points = max_points;
  drop_graph(b);
  return VG_OK;
}

vg_status vg_batch_solver_info(const vg_batch* b, int* persistent_sims, int* teams, int* team_ctas, int* captured) {
  if (!b) return VG_INVALID;
  int n = 0;
  for (char x : b->split) n += b->mg && x ? 1 : 0;
  if (persistent_sims) *persistent_sims = n;
  mg_batch_info(b->mg, teams, team_ctas, nullptr);
  if (captured) *captured = b->mg_exec ? 1 : 0;
  return VG_OK;
}

vg_status vg_batch_graph_info(const vg_batch* b, int* graphs, size_t* max_nodes, size_t* total_nodes) {
  if (!b) return VG_INVALID;
  size_t mx = 0, tot = 0;
  for (const Chunk& k : b->chunks) {
    mx = std::max(mx, k.nodes);
    tot += k.nodes;
  }
  if (b->mg_exec) tot += 2;  // the persistent solve: barrier clear and the launch
  if (graphs) *graphs = (int)b->chunks.size() + (b->mg_exec ? 1 : 0);
  if (max_nodes) *max_nodes = mx;
  if (total_nodes) *total_nodes = tot;
  return VG_OK;
}

}  // extern "C"
