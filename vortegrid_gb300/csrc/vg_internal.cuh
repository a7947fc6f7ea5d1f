// Internal declarations shared by the sm_103a kernels of libvortegrid.
//
// Two arithmetic laws are provided for the vorton kernels:
//  * ref_*  -- the reference's exact FP32 operation order (VortonFluid/vorton.h:118-179,
//              Core/Math/math.h:206-216) written with round-to-nearest intrinsics
//              (__fadd_rn, __fmul_rn, ...), which the compiler never fuses, so the
//              results are bit-identical to the reference's CPU build;
//  * fast   -- hardware rsqrt, fused multiply-add and algebraic reassociation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/vortegrid.h"

namespace vg {

constexpr int kMaxLayers = 24;
// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount,
// queried once per device); grids sized in whole waves use it.
int sm_count();

// Grid geometry on the device: identical fields to vg_grid_geom.
struct Geom {
  float mn[3], ext[3], cell[3], cpe[3];
  unsigned np[3];
  __host__ __device__ unsigned nx() const { return np[0]; }
  __host__ __device__ size_t points() const { return (size_t)np[0] * np[1] * np[2]; }
};

inline Geom to_geom(const vg_grid_geom& g) {
  Geom d;
  for (int a = 0; a < 3; ++a) {
    d.mn[a] = g.min_corner[a];
    d.ext[a] = g.extent[a];
    d.cell[a] = g.cell_spacing[a];
    d.cpe[a] = g.cells_per_extent[a];
    d.np[a] = g.num_points[a];
  }
  return d;
}
inline vg_grid_geom from_geom(const Geom& d) {
  vg_grid_geom g;
  for (int a = 0; a < 3; ++a) {
    g.min_corner[a] = d.mn[a];
    g.extent[a] = d.ext[a];
    g.cell_spacing[a] = d.cell[a];
    g.cells_per_extent[a] = d.cpe[a];
    g.num_points[a] = d.np[a];
  }
  return g;
}

// Host geometry rules (Core/SpatialPartition/uniformGrid.h:259-412).
void precompute_spacing(Geom& g);
Geom define_shape(size_t n, const float vmin[3], const float vmax[3], bool pow2);
Geom decimate(const Geom& src, unsigned dec);
int nested_shape(const Geom& g, Geom* layers, unsigned (*decim)[3]);

// ------------------------------------------------------------ device helpers

// IndicesOfPosition (uniformGrid.h:536-574): FP32 (p - min) * cellsPerExtent
// truncated toward zero, each operation rounded separately.
__device__ __forceinline__ unsigned bin_axis(float p, float mn, float cpe) {
  return (unsigned)__float2int_rz(__fmul_rn(__fsub_rn(p, mn), cpe));
}

// finvsqrtf (Core/Math/math.h:206-216): magic-constant estimate + one Newton step.
__device__ __forceinline__ float ref_finvsqrtf(float v) {
  int i = __float_as_int(v);
  i = 0x5f3759df - (i >> 1);
  float y = __int_as_float(i);
  const float x = __fmul_rn(v, 0.5f);
  return __fmul_rn(y, __fsub_rn(1.5f, __fmul_rn(__fmul_rn(x, y), y)));
}

__device__ __forceinline__ float ref_dot_self(float a, float b, float c) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c));
}

// UniformGrid::Interpolate (uniformGrid.h:1117-1148) of K floats per point.
template <int K>
__device__ __forceinline__ void interp(const Geom& g, const float* __restrict__ f, float px, float py, float pz,
                                       float* out) {
  const float p[3] = {px, py, pz};
  unsigned idx[3];
  float tw[3], om[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    idx[a] = bin_axis(p[a], g.mn[a], g.cpe[a]);
    const float cmin = __fadd_rn(g.mn[a], __fmul_rn((float)idx[a], g.cell[a]));
    tw[a] = __fmul_rn(__fsub_rn(p[a], cmin), g.cpe[a]);
    om[a] = __fsub_rn(1.0f, tw[a]);
  }
  const size_t nx = g.np[0], nxy = (size_t)g.np[0] * g.np[1];
  const size_t o = idx[0] + nx * (idx[1] + (size_t)g.np[1] * idx[2]);
#pragma unroll
  for (int a = 0; a < K; ++a) {
    const float v000 = f[K * o + a], v100 = f[K * (o + 1) + a], v010 = f[K * (o + nx) + a],
                v110 = f[K * (o + nx + 1) + a], v001 = f[K * (o + nxy) + a], v101 = f[K * (o + nxy + 1) + a],
                v011 = f[K * (o + nxy + nx) + a], v111 = f[K * (o + nxy + nx + 1) + a];
    const float y0 = __fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(om[0], v000), __fmul_rn(tw[0], v100)), om[1]),
                               __fmul_rn(__fadd_rn(__fmul_rn(om[0], v010), __fmul_rn(tw[0], v110)), tw[1]));
    const float y1 = __fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(om[0], v001), __fmul_rn(tw[0], v101)), om[1]),
                               __fmul_rn(__fadd_rn(__fmul_rn(om[0], v011), __fmul_rn(tw[0], v111)), tw[1]));
    out[a] = __fadd_rn(__fmul_rn(y0, om[2]), __fmul_rn(y1, tw[2]));
  }
}

__device__ __forceinline__ bool inside_cells(const Geom& g, float px, float py, float pz) {
  // The reference requires samples strictly inside the grid's cells
  // (uniformGrid.h:1122-1124); report rather than read out of bounds.
  // bin_axis maps a position one to two cells below the minimum corner to
  // 0xffffffff (truncation gives -1), so compare against np - 1 rather than
  // testing ix + 1 < np, which wraps to 0 there.
  const unsigned ix = bin_axis(px, g.mn[0], g.cpe[0]);
  const unsigned iy = bin_axis(py, g.mn[1], g.cpe[1]);
  const unsigned iz = bin_axis(pz, g.mn[2], g.cpe[2]);
  return ix < g.np[0] - 1u && iy < g.np[1] - 1u && iz < g.np[2] - 1u && px == px && py == py && pz == pz;
}

// 2/3 as the reference's float constant (VortonFluid/vorton.h:92).
#define VG_TWO_THIRDS (2.0f / 3.0f)

// VORTON_ACCUMULATE_VELOCITY_private (vorton.h:161-179), reference order.
__device__ __forceinline__ void ref_accum_velocity(float3& acc, float qx, float qy, float qz, float4 ps, float4 w,
                                                   float sr, float sc) {
  const float d0 = __fsub_rn(qx, ps.x), d1 = __fsub_rn(qy, ps.y), d2 = __fsub_rn(qz, ps.z);
  const float radius = __fmul_rn(__fmul_rn(ps.w, 0.5f), sr);
  const float r2 = __fmul_rn(radius, radius);
  const float dist2 = ref_dot_self(d0, d1, d2);
  const float law = (dist2 < r2) ? __fdiv_rn(1.0f, __fmul_rn(r2, radius))
                                 : __fdiv_rn(ref_finvsqrtf(dist2), dist2);
  const float s = __fmul_rn(__fmul_rn(VG_TWO_THIRDS, r2), radius);
  const float a0 = __fmul_rn(w.x, s), a1 = __fmul_rn(w.y, s), a2 = __fmul_rn(w.z, s);
  const float b0 = __fmul_rn(d0, law), b1 = __fmul_rn(d1, law), b2 = __fmul_rn(d2, law);
  const float c0 = __fsub_rn(__fmul_rn(a1, b2), __fmul_rn(a2, b1));
  const float c1 = __fsub_rn(__fmul_rn(a2, b0), __fmul_rn(a0, b2));
  const float c2 = __fsub_rn(__fmul_rn(a0, b1), __fmul_rn(a1, b0));
  acc.x = __fadd_rn(acc.x, __fmul_rn(c0, sc));
  acc.y = __fadd_rn(acc.y, __fmul_rn(c1, sc));
  acc.z = __fadd_rn(acc.z, __fmul_rn(c2, sc));
}

// VORTON_ACCUMULATE_VECTOR_POTENTIAL_private (vorton.h:118-136), reference order.
__device__ __forceinline__ void ref_accum_vecpot(float3& acc, float qx, float qy, float qz, float4 ps, float4 w,
                                                 float sr, float sc) {
  const float d0 = __fsub_rn(qx, ps.x), d1 = __fsub_rn(qy, ps.y), d2 = __fsub_rn(qz, ps.z);
  const float radius = __fmul_rn(__fmul_rn(ps.w, 0.5f), sr);
  const float r2 = __fmul_rn(radius, radius);
  const float dist2 = ref_dot_self(d0, d1, d2);
  const float law = (dist2 < r2) ? __fdiv_rn(dist2, __fmul_rn(r2, radius)) : ref_finvsqrtf(dist2);
  const float s = __fmul_rn(__fmul_rn(VG_TWO_THIRDS, r2), radius);
  acc.x = __fadd_rn(acc.x, __fmul_rn(__fmul_rn(__fmul_rn(w.x, s), law), sc));
  acc.y = __fadd_rn(acc.y, __fmul_rn(__fmul_rn(__fmul_rn(w.y, s), law), sc));
  acc.z = __fadd_rn(acc.z, __fmul_rn(__fmul_rn(__fmul_rn(w.z, s), law), sc));
}

template <int KIND>
__device__ __forceinline__ void ref_accum(float3& acc, float qx, float qy, float qz, float4 ps, float4 w, float sr,
                                          float sc) {
  if (KIND == 0)
    ref_accum_velocity(acc, qx, qy, qz, ps, w, sr, sc);
  else
    ref_accum_vecpot(acc, qx, qy, qz, ps, w, sr, sc);
}

// Fast law, same mathematics: law = min(rsqrt(d2), 1/r)^3 reproduces both the
// core branch (1/r^3) and the far branch (|d|^-3); vector potential law =
// |d|^2/r^3 inside, 1/|d| outside.
template <int KIND>
__device__ __forceinline__ void fast_accum(float3& acc, float qx, float qy, float qz, float4 ps, float4 w, float sr,
                                           float sc) {
  const float d0 = qx - ps.x, d1 = qy - ps.y, d2 = qz - ps.z;
  const float radius = ps.w * 0.5f * sr;
  const float invr = 1.0f / radius;
  const float dist2 = fmaf(d0, d0, fmaf(d1, d1, d2 * d2));
  const float s = VG_TWO_THIRDS * radius * radius * radius * sc;
  if (KIND == 0) {
    const float inv = fminf(rsqrtf(dist2), invr);
    const float law = inv * inv * inv * s;
    const float b0 = d0 * law, b1 = d1 * law, b2 = d2 * law;
    acc.x = fmaf(w.y, b2, fmaf(-w.z, b1, acc.x));
    acc.y = fmaf(w.z, b0, fmaf(-w.x, b2, acc.y));
    acc.z = fmaf(w.x, b1, fmaf(-w.y, b0, acc.z));
  } else {
    const float law = (dist2 < radius * radius) ? dist2 * invr * invr * invr : rsqrtf(dist2);
    const float f = law * s;
    acc.x = fmaf(w.x, f, acc.x);
    acc.y = fmaf(w.y, f, acc.y);
    acc.z = fmaf(w.z, f, acc.z);
  }
}

// ---------------------------------------------------------------- context

struct Ctx;

// Grow-only device workspace slot.
struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

enum Slot {
  S_BBOX,
  S_CELL,
  S_COUNT,
  S_START,
  S_FILL,
  S_ITEMS,
  S_SCAN,
  S_TREE,
  S_NEGVORT,
  S_VECPOT,
  S_VEL,
  S_JAC,
  S_WOLD,
  S_MG,
  S_DIRECT,
  S_POS,
  S_ANGVEL,
  S_VVEL,
  S_HOSTSTAGE,
  S_TRACERS,
  S_RED,
  S_PREV,
  S_MGINV,
  S_TREEPREP,
  S_PCL,
  S_DENS,   // density grid (baroclinic)
  S_GRAD,   // density gradient grid (baroclinic)
  S_SDF,    // signed distance: pinned flags, statistics, partial sums
  S_MC,     // marching cubes: per-cell counts and offsets
  S_BODY,   // fluid-body collisions: per-block partial sums
  S_EMIT,   // emitters: jitter draws, records, deviation grid, flags
  S_VELCELL,  // the velocity grid by cell (8 corners x float4) for large tracer groups
  S_NUM
};

// A captured multigrid cycle, replayed while the grid and buffers are unchanged.
struct MgGraphCache {
  cudaGraphExec_t exec = nullptr;
  Geom g;
  const void* key[4] = {nullptr, nullptr, nullptr, nullptr};
  unsigned launches = 0;
};

namespace nn {
struct Net;
}

struct Ctx {
  vg_config cfg;
  nn::Net* net = nullptr;   // attached warm-start network (not owned)
  MgGraphCache mg_graph[2];  // phase-1 and phase-2 cycle graphs
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  Buf buf[S_NUM];
  Geom grid;                // last step's grid
  bool have_grid = false;
  vg_step_stats stats;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  // second stream of vg_step_advect (the tracer records' upload beside the
  // vortons' step) and its two ordering events, created on first use
  cudaStream_t aux = nullptr;
  cudaEvent_t aux_ev0 = nullptr, aux_ev1 = nullptr, aux_ev2 = nullptr, aux_ev3 = nullptr;
  unsigned launches = 0;    // kernel launches since the counter was reset
  Geom prev_grid;           // grid of the stored previous solution
  bool have_prev = false;
  int* dflag = nullptr;     // device error word: bit 0 = a sample left the grid
  int* hflag = nullptr;     // pinned host copy of dflag[0], read back with the stream's work
  // vg_step_evolve_device: the step also moves the vortons by velocity x dt
  // (step_evolved: a kernel of the step has done it)
  bool step_evolve = false, step_evolved = false;
  // generation of the step's velocity grid (counted on the host at each step)
  // and the one the by-cell copy in buf[S_VELCELL] was made from
  unsigned long long vel_gen = 0, velcell_gen = ~0ull;
  bool stats_pending = false;
  // Multigrid schedule.  mg_fixed_k1 > 0 runs a fixed schedule with no host
  // round trip (k1 FP32 cycles, then k2 refinement cycles), so that a step can
  // be captured in a CUDA graph; the adaptive solve records the counts it used.
  int mg_fixed_k1 = 0, mg_fixed_k2 = 0;
  int mg_last_k1 = 0, mg_last_k2 = 0;
  double* mg_relres_dev = nullptr;  // fixed schedule: final and initial relative residuals
  bool step_captured = false;       // the last step was recorded into a CUDA graph (its events carry no times)
  // Vortons that leave a fixed grid: an error (false), or stopped and left out
  // of the solve, with dflag[1] recording that it happened (true).
  bool freeze_outside = false;
  // the multigrid coarsest-level inverse held in buf[S_MGINV]: its level's shape and 1 / spacing^2
  unsigned mginv_np[3] = {0, 0, 0};
  double mginv_r2[3] = {0.0, 0.0, 0.0};
  bool mginv_fp64 = false;  // the tables in buf[S_MGINV] are double
  // The coarsest multigrid level (sine transforms over the whole GPU) solved
  // in FP64 instead of FP32 (vg_set_coarsest_fp64).
  bool mg_coarse_fp64 = false;
  // A step split at the Poisson solve, for batched frames that solve every
  // simulation's problem in one persistent launch between the two halves:
  // 0 the whole step; 1 up to the solve (its state kept in *split); 2 from
  // the solve on, resuming *split.
  int step_split = 0;
  struct StepState* split = nullptr;
  // the host-record step's CUDA graph (vg_api.cu), replayed while the same
  // call repeats
  struct HostStepGraph* host_graph = nullptr;
};

// The word a kernel marks when a sample lies outside the grid's cells.
inline int* outside_flag(Ctx* c) { return c->freeze_outside ? c->dflag + 1 : c->dflag; }

// Device-side error bits, reported at the next synchronising call.
enum DevFlag { DF_OUT_OF_GRID = 1, DF_NONFINITE = 2, DF_TIMEOUT = 4 };
vg_status sync_and_check(Ctx* c, const char* what);

// Workspace: returns a device buffer of at least `bytes` for slot s.
void* ws(Ctx* c, int s, size_t bytes, vg_status* st);

vg_status fail(Ctx* c, vg_status s, const std::string& msg);
// Records an error for calls made without a context (vg_last_error(NULL)).
vg_status set_noctx_error(vg_status s, const std::string& msg);
vg_status cuda_check(Ctx* c, cudaError_t e, const char* what);
#define VG_CUDA(ctx, call)                                 \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_check(ctx, e_, #call); \
  } while (0)
#define VG_LAUNCHED(ctx) ((ctx)->launches++)

inline unsigned blocks_for(size_t n, unsigned threads) { return (unsigned)((n + threads - 1) / threads); }

// Programmatic dependent launch for chains of short kernels: a kernel started
// by pdl_launch may be launched as the previous kernel of its stream drains
// (its CTAs' exits trigger it), overlapping the launch with that kernel's
// completion.  Its first statement is pdl_entry(), which waits until the
// previous kernel has completed and its writes are visible
// (griddepcontrol.wait), so the chain's results are those of ordinary
// launches.  Without a programmatic predecessor the wait returns at once.
// (Triggering the next launch at kernel entry measured slower: its waiting
// CTAs held SM slots during the previous kernel's last wave.)
__device__ __forceinline__ void pdl_entry() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t pdl_launch(cudaStream_t s, dim3 grid, dim3 block, size_t smem, void (*kernel)(KArgs...),
                              Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// ---------------------------------------------------------- stage launchers
// (device pointers, context stream; defined in the .cu files)

// Where the velocity step wants the direct sum's results: targets [0, pts)
// as float[3] into grid3, the rest as float4 records into vel.
// When grid is given, targets [0, pts) are that grid's points (the step's
// gridpoint positions), which the packed kernel evaluates row by row without
// reading them from q; after_grid, when given, holds targets [pts, m) (the
// vortons' records) for it in place of q + pts.
struct DirectSplit {
  float* grid3;
  size_t pts;
  float4* vel;
  const Geom* grid;
  const float4* after_grid;
  float4* evolve_pos = nullptr;  // not NULL: the reduction also moves these vortons by velocity x evolve_dt
  float evolve_dt = 0.f;
};
// With split, *split_done says whether the results went there (the
// multi-chunk packed path writes them from its reduction) or to out.
vg_status launch_direct(Ctx* c, int kind, bool ref, const float4* ps, const float4* w, size_t n, const float4* q,
                        size_t m, float sr, float sc, float4* out, const DirectSplit* split = nullptr,
                        bool* split_done = nullptr);

// Cell lists: stable counting sort of vortons by leaf cell (OffsetOfPosition).
struct CellLists {
  unsigned* cell;   // per vorton: leaf offset
  unsigned* start;  // per cell (+1): first item
  unsigned* items;  // vorton indices grouped by cell, ascending within a cell
};
vg_status build_cell_lists(Ctx* c, const Geom& g, const float4* ps, size_t n, CellLists* out);
// Exclusive scan of n values on the context's stream; out[n] receives the total when write_total.
vg_status exclusive_scan(Ctx* c, const unsigned* in, size_t n, unsigned* out, bool write_total);

struct Tree {
  int depth;
  Geom layer[kMaxLayers];
  unsigned decim[kMaxLayers][3];
  size_t base[kMaxLayers];
  size_t total;
  float4* sv_pos;  // per point: pos xyz, size
  float4* sv_w;    // per point: angvel xyz, 0
};
vg_status build_tree(Ctx* c, const Geom& g, const float4* ps, const float4* w, size_t n, const CellLists& cl,
                     Tree* t);
vg_status launch_tree_eval(Ctx* c, int kind, bool ref, const Tree& t, const float4* ps, const float4* w, size_t n,
                           const float4* q, size_t m, float sr, float sc, float4* out);
vg_status launch_boundary_vecpot(Ctx* c, const Tree& t, const Geom& g, const float4* ps, const float4* w, size_t n,
                                 bool copy_odd_x, bool ref, float* grid3);
vg_status launch_splat(Ctx* c, const Geom& g, const float4* ps, const float4* w, size_t n, const CellLists& cl,
                       float scale, float radius, float* grid3);

vg_status launch_sor(Ctx* c, const Geom& g, float* soln3, const float* lap3, int steps);
vg_status launch_downsample(Ctx* c, const Geom& fine, const float* f3, const Geom& coarse, bool inject, float* c3);
vg_status launch_upsample(Ctx* c, const Geom& coarse, const float* c3, const Geom& fine, bool interior, float* f3);
vg_status run_cascade(Ctx* c, const Geom& g, float* soln3, const float* rhs3, int steps);
vg_status run_multigrid(Ctx* c, const Geom& g, float* soln3, const float* rhs3, double tol, int max_cycles,
                        int* cycles, double* relres0, double* relres);
// The same solve on a schedule fixed in advance (c->mg_fixed_k1, mg_fixed_k2): no host round trip.
vg_status run_multigrid_fixed(Ctx* c, const Geom& g, float* soln3, const float* rhs3);

// Persistent batched solve: every qualifying simulation's fixed-schedule
// solve of one frame in a single cooperative launch, teams of CTAs working
// through the simulations with a barrier between phases.  A simulation
// qualifies when its hierarchy ends in the sine-transform solve over the GPU
// (mg_batch_eligible).  Results are bit-identical to run_multigrid_fixed.
struct MgBatchItem {
  Ctx* c;
  Geom g;
  float* soln;
  const float* rhs;
};
struct MgBatch;
// The Poisson problem of the last step that stopped before its solve (step_split 1).
bool split_problem(Ctx* c, MgBatchItem* out);
bool mg_batch_eligible(const Geom& g);
// team_ctas: CTAs per team (0 = automatic).  Not during stream capture (uploads).
vg_status mg_batch_build(const std::vector<MgBatchItem>& items, int device, int team_ctas, MgBatch** out,
                         std::string* err);
// Enqueues the launch on s (capturable): barrier counters cleared, then the kernel.
vg_status mg_batch_enqueue(MgBatch* mb, cudaStream_t s, std::string* err);
// Whether a team barrier gave up since the last call (reads and clears the device word; synchronous).
bool mg_batch_failed(MgBatch* mb);
void mg_batch_info(const MgBatch* mb, int* teams, int* team_ctas, int* ctas);
void mg_batch_destroy(MgBatch* mb);

vg_status launch_jacobian(Ctx* c, const Geom& g, const float* v3, float* jac9);
vg_status launch_curl(Ctx* c, const Geom& g, const float* v3, float* curl3);
// order: NULL, or the vortons' indices grouped by cell (the cell lists' items)
vg_status launch_stretch(Ctx* c, const Geom& g, const float* jac9, const float4* ps, float4* w, size_t n, float dt,
                         const unsigned* order = nullptr);
// The same stretch from the velocity grid (the Jacobian formed at each vorton's cell corners).
vg_status launch_stretch_vel(Ctx* c, const Geom& g, const float* v3, const float4* ps, float4* w, size_t n, float dt,
                             const unsigned* order = nullptr);
vg_status launch_pse(Ctx* c, const Geom& g, const CellLists& cl, const float4* ps, float4* w, size_t n, float nu,
                     float dt);
vg_status launch_heat_pse(Ctx* c, const Geom& g, const CellLists& cl, const float4* ps, float* density, size_t n,
                          float kappa, float ambient, float dt);
// by_cell: a tracer group of the step's own velocity grid (vel3 = buf[S_VEL]),
// which may be gathered from a copy of the grid arranged by cell.
vg_status launch_gather_advect(Ctx* c, const Geom& g, const float* vel3, float4* pos, float4* vel, size_t m,
                               float dt, bool evolve, const unsigned* order = nullptr, bool by_cell = false);
// Whether m tracers on grid g gather from the grid arranged by cell.
bool gather_by_cell(const Geom& g, size_t m);
// The gather + Euler step in place on m staged particle records (position at
// bytes 0-11, velocity at 12-23, pitch bytes apart).
vg_status launch_gather_advect_records(Ctx* c, const Geom& g, const float* vel3, unsigned char* rec, size_t pitch,
                                       size_t m, float dt);
vg_status launch_bbox(Ctx* c, const float4* pos, size_t n, float* out6_dev);
// Density grid (PopulateDensityAndMassFractionGrids), gradient (ComputeGradient),
// baroclinic generation and the signed distance grid (vg_surface.cu).
vg_status launch_density_grid(Ctx* c, const Geom& g, const float4* ps, const float* density, size_t n,
                              float ambient, float* out);
// Density deviation grid of the emitter's tracer mask (density - ambient, accumulated alone).
vg_status launch_density_deviation(Ctx* c, const Geom& g, const float4* ps, const float* density, size_t n,
                                   float ambient, float* out);
vg_status launch_gradient(Ctx* c, const Geom& g, const float* v, float* grad3);
vg_status launch_baroclinic(Ctx* c, const Geom& g, const float* grad3, const float4* ps, float4* w, size_t n,
                            const float grav[3], float ambient, float dt);
vg_status launch_signed_distance(Ctx* c, const Geom& g, const float* dens, float ambient, bool reference_stats,
                                 float* sdf, unsigned char* pinned, float* stats, double* partials,
                                 int partial_blocks);
// Marching cubes: *triangles receives the count; VG_TOO_LARGE when it exceeds cap (nothing written).  Synchronous.
vg_status launch_marching_cubes(Ctx* c, const Geom& g, const float* v, float iso, float* verts, float* normals,
                                size_t cap, size_t* triangles);

namespace nn {
// True when the network applies to grid g ((edge+1)^3 points).
bool fits(const Net* N, const Geom& g);
// Writes the network's guess into the interior points of vp (boundary already set).
vg_status guess(Ctx* c, Net* N, const Geom& g, const float* rhs, float* vp);
}  // namespace nn

}  // namespace vg
