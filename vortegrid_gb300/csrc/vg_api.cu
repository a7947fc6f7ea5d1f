// C ABI of libvortegrid: context, workspace, host-side geometry rules and the
// VortonSim step (VortonFluid/pclOpVortonSim.cpp:51-71,
// VortonFluid/vortonSim.cpp:4117-4344) composed from the stage kernels.
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <new>

#include "vg_internal.cuh"

namespace vg {

// ------------------------------------------------------------ host geometry
// Compiled with -ffp-contract=off so every float operation rounds like the
// reference's.

void precompute_spacing(Geom& g) {  // uniformGrid.h:794-809
  for (int a = 0; a < 3; ++a) g.cell[a] = g.ext[a] / (float)(g.np[a] - 1);
  g.cpe[0] = (float)(g.np[0] - 1) / g.ext[0];
  g.cpe[1] = (float)(g.np[1] - 1) / g.ext[1];
  g.cpe[2] = (0.0f == g.ext[2]) ? 1.0f / FLT_MIN : (float)(g.np[2] - 1) / g.ext[2];
}

static size_t nearest_pow2(size_t v) {  // Core/Math/math.h:149-175
  if (v == 0) return 1;
  --v;
  unsigned shift = 0;
  while ((v >> shift) != 0) ++shift;
  return (size_t)(1U << shift);
}

Geom define_shape(size_t n, const float vmin[3], const float vmax[3], bool pow2) {  // uniformGrid.h:259-322
  Geom g;
  memset(&g, 0, sizeof(g));
  if (n == 0) return g;
  const float nudge = 1.0f + FLT_EPSILON;
  float eff[3];
  int dims = 3;
  for (int a = 0; a < 3; ++a) {
    g.mn[a] = vmin[a];
    g.ext[a] = (vmax[a] - vmin[a]) * nudge;
    eff[a] = g.ext[a];
  }
  for (int a = 0; a < 3; ++a)
    if (0.0f == eff[a]) {
      eff[a] = 1.0f;
      g.ext[a] = 0.0f;
      --dims;
    }
  const float volume = eff[0] * eff[1] * eff[2];
  const float inv_cell = powf(volume / (float)n, -1.0f / (float)dims);
  size_t nc[3];
  for (int a = 0; a < 3; ++a) {
    const size_t c = (size_t)(g.ext[a] * inv_cell + 0.5f);
    nc[a] = c > 1 ? c : 1;
  }
  if (pow2)
    for (int a = 0; a < 3; ++a) nc[a] = nearest_pow2(nc[a]);
  while (nc[0] * nc[1] * nc[2] >= n * 8)
    for (int a = 0; a < 3; ++a) nc[a] = nc[a] / 2 > 1 ? nc[a] / 2 : 1;
  for (int a = 0; a < 3; ++a) g.np[a] = (unsigned)(nc[a] + 1);
  precompute_spacing(g);
  return g;
}

Geom decimate(const Geom& src, unsigned dec) {  // uniformGrid.h:398-412
  Geom d = src;
  for (int a = 0; a < 3; ++a) {
    d.np[a] = (src.np[a] - 1) / dec + 1;
    if (dec > 1 && d.np[a] < 2) d.np[a] = 2;
  }
  precompute_spacing(d);
  return d;
}

int nested_shape(const Geom& g, Geom* layers, unsigned (*decim)[3]) {  // nestedGrid.h:69-85, 312-391
  int depth = 0;
  layers[depth++] = decimate(g, 1);
  while (layers[depth - 1].points() > 8 && depth < kMaxLayers) {
    layers[depth] = decimate(layers[depth - 1], 2);
    ++depth;
  }
  decim[0][0] = decim[0][1] = decim[0][2] = 0;
  for (int l = 1; l < depth; ++l)
    for (int a = 0; a < 3; ++a) decim[l][a] = (layers[l - 1].np[a] - 1) / (layers[l].np[a] - 1);
  return depth;
}

// ------------------------------------------------------------------ context

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return 1;
  }
  if (!cached[dev]) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
      cudaGetLastError();
      sms = 1;
    }
    cached[dev] = sms;
  }
  return cached[dev];
}

vg_status fail(Ctx* c, vg_status s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}

vg_status cuda_check(Ctx* c, cudaError_t e, const char* what) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return fail(c, e == cudaErrorMemoryAllocation ? VG_OOM : VG_CUDA_ERROR, buf);
}

vg_status sync_and_check(Ctx* c, const char* what) {
  int h = 0;
  if (c->hflag) {
    // the error word comes back behind the stream's work: one wait, no second round trip
    VG_CUDA(c, cudaMemcpyAsync(c->hflag, c->dflag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
    h = *c->hflag;
  } else {
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
    VG_CUDA(c, cudaMemcpy(&h, c->dflag, sizeof(int), cudaMemcpyDeviceToHost));
  }
  if (h) {
    VG_CUDA(c, cudaMemset(c->dflag, 0, sizeof(int)));
    if (h & DF_TIMEOUT) return fail(c, VG_TIMEOUT, std::string(what) + ": a bounded device wait gave up");
    if (h & DF_NONFINITE) return fail(c, VG_NONFINITE, std::string(what) + ": non-finite vorton position");
    return fail(c, VG_OUT_OF_GRID, std::string(what) + ": a particle lies outside the grid's cells");
  }
  return VG_OK;
}

void* ws(Ctx* c, int s, size_t bytes, vg_status* st) {
  Buf& b = c->buf[s];
  if (b.bytes >= bytes && b.p) return b.p;
  if (b.p) {
    cudaStreamSynchronize(c->stream);
    cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
  }
  size_t want = bytes + bytes / 8 + 256;
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    *st = fail(c, VG_OOM, "device allocation of " + std::to_string(want) + " bytes failed");
    return nullptr;
  }
  b.bytes = want;
  return b.p;
}

}  // namespace vg

using namespace vg;

struct vg_ctx : public vg::Ctx {};

namespace {

thread_local std::string g_err_noctx;

}  // namespace

vg_status vg::set_noctx_error(vg_status s, const std::string& msg) {
  g_err_noctx = msg;
  return s;
}

namespace {

__global__ void k_unpack_records(const unsigned char* __restrict__ rec, size_t pitch, int n, float4* __restrict__ ps,
                                 float4* __restrict__ w) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = (const float*)(rec + (size_t)i * pitch);
  ps[i] = make_float4(r[0], r[1], r[2], r[13]);  // position @0, size @52
  w[i] = make_float4(r[9], r[10], r[11], 0.f);   // angular velocity @36
}

// k_pack_records followed by PclOpEvolve's Euler step (pclOpEvolve.cpp:36-58)
// on the same records: record bytes [0, 48) -- position + velocity dt, then
// velocity, (unchanged) orientation, angular velocity.
__global__ void k_pack_records_evolve(unsigned char* __restrict__ rec, size_t pitch, int n,
                                      const float4* __restrict__ ps, const float4* __restrict__ v,
                                      const float4* __restrict__ w, float dt) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* r = (float*)(rec + (size_t)i * pitch);
  const float4 p = ps[i], u = v[i], a = w[i];
  r[0] = __fadd_rn(p.x, __fmul_rn(u.x, dt));
  r[1] = __fadd_rn(p.y, __fmul_rn(u.y, dt));
  r[2] = __fadd_rn(p.z, __fmul_rn(u.z, dt));
  r[3] = u.x;
  r[4] = u.y;
  r[5] = u.z;
  r[9] = a.x;
  r[10] = a.y;
  r[11] = a.z;
}

__global__ void k_pack_records(unsigned char* __restrict__ rec, size_t pitch, int n, const float4* __restrict__ v,
                               const float4* __restrict__ w) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* r = (float*)(rec + (size_t)i * pitch);  // record bytes [12, 48)
  r[0] = v[i].x;
  r[1] = v[i].y;
  r[2] = v[i].z;
  r[6] = w[i].x;
  r[7] = w[i].y;
  r[8] = w[i].z;
}

// Targets of the grid-point evaluation: every gridpoint, then (when ps is
// given) the n vortons' position records after them.
__global__ void k_grid_points(Geom g, float4* __restrict__ q, const float4* __restrict__ ps, size_t n) {
  pdl_entry();
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.points()) {
    if (ps && k - g.points() < n) q[k] = ps[k - g.points()];
    return;
  }
  const unsigned x = (unsigned)(k % g.np[0]), y = (unsigned)((k / g.np[0]) % g.np[1]),
                 z = (unsigned)(k / ((size_t)g.np[0] * g.np[1]));
  // gridpoint positions min + i * spacing * (1 - 2 eps) (vortonSim.cpp:2229-2252)
  const float nudge = 1.0f - 2.0f * FLT_EPSILON;
  q[k] = make_float4(__fadd_rn(g.mn[0], __fmul_rn((float)x, __fmul_rn(g.cell[0], nudge))),
                     __fadd_rn(g.mn[1], __fmul_rn((float)y, __fmul_rn(g.cell[1], nudge))),
                     __fadd_rn(g.mn[2], __fmul_rn((float)z, __fmul_rn(g.cell[2], nudge))), 0.f);
}

// Velocities at the targets: the first n (gridpoints) as float[3] into b,
// the next m (vortons, when vel is given) as float4 records into vel.
__global__ void k_f4_to_f3(const float4* __restrict__ a, float* __restrict__ b, size_t n, float4* __restrict__ vel,
                           size_t m) {
  pdl_entry();
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    if (vel && i - n < m) vel[i - n] = a[i];
    return;
  }
  {
    b[3 * i] = a[i].x;
    b[3 * i + 1] = a[i].y;
    b[3 * i + 2] = a[i].z;
  }
}

__global__ void k_copy_pos3(const unsigned char* __restrict__ rec, size_t pitch, int n, float4* __restrict__ p) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = (const float*)(rec + (size_t)i * pitch);
  p[i] = make_float4(r[0], r[1], r[2], 0.f);
}

__global__ void k_store_posvel(unsigned char* __restrict__ rec, size_t pitch, int n, const float4* __restrict__ p,
                               const float4* __restrict__ v) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* r = (float*)(rec + (size_t)i * pitch);  // bytes [0, 24): position, velocity
  r[0] = p[i].x; r[1] = p[i].y; r[2] = p[i].z;
  r[3] = v[i].x; r[4] = v[i].y; r[5] = v[i].z;
}

vg_status check_cfg(Ctx* c, const vg_config* cfg) {
  if (!cfg) return fail(c, VG_INVALID, "config is NULL");
  if (cfg->abi_version != VG_ABI_VERSION) return fail(c, VG_INVALID, "config abi_version mismatch");
  if (cfg->velocity_technique < 0 || cfg->velocity_technique > 2) return fail(c, VG_INVALID, "bad velocity_technique");
  if (cfg->numerics < 0 || cfg->numerics > 1) return fail(c, VG_INVALID, "bad numerics");
  if (cfg->poisson_solver < 0 || cfg->poisson_solver > 1) return fail(c, VG_INVALID, "bad poisson_solver");
  if (cfg->warm_start < 0 || cfg->warm_start > 2) return fail(c, VG_INVALID, "bad warm_start");
  if (!(cfg->viscosity >= 0.0f)) return fail(c, VG_INVALID, "viscosity must be >= 0");
  if (!(cfg->poisson_tolerance > 0.0)) return fail(c, VG_INVALID, "poisson_tolerance must be > 0");
  if (cfg->use_fixed_grid) {
    for (int a = 0; a < 3; ++a)
      if (cfg->fixed_grid.num_points[a] < 2 || !(cfg->fixed_grid.extent[a] > 0.0f))
        return fail(c, VG_INVALID, "fixed grid needs >= 2 points and positive extent per axis");
  }
  return VG_OK;
}

bool finite3(const float* v) { return v && std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// Geometry of a step: VortonSim::FindBoundingBox + UpdateBoundingBox(final)
// (vortonSim.cpp:1001-1096): the vortons' AABB joined with the extra box (or
// the first vorton), padded by 3 vorton radii, DefineShape(n, ..., pow2).
vg_status step_geometry(Ctx* c, const float4* ps, size_t n, const float* first_pos, float radius,
                        const float* extra_min, const float* extra_max, Geom* out) {
  if (c->cfg.use_fixed_grid) {
    Geom g = to_geom(c->cfg.fixed_grid);
    precompute_spacing(g);
    *out = g;
    return VG_OK;
  }
  vg_status st = VG_OK;
  float* d6 = (float*)ws(c, S_RED, 256, &st);
  if (st != VG_OK) return st;
  float* box = d6 + 16;
  if ((st = launch_bbox(c, ps, n, box)) != VG_OK) return st;
  float h[6];
  VG_CUDA(c, cudaMemcpyAsync(h, box, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  if ((st = sync_and_check(c, "bounding box")) != VG_OK) return st;
  float mn[3] = {h[0], h[1], h[2]}, mx[3] = {h[3], h[4], h[5]};
  const bool extra = extra_min && extra_max;
  const float* emin = extra ? extra_min : first_pos;
  const float* emax = extra ? extra_max : first_pos;
  for (int a = 0; a < 3; ++a) {
    mn[a] = mn[a] < emin[a] ? mn[a] : emin[a];
    mx[a] = mx[a] > emax[a] ? mx[a] : emax[a];
  }
  if (!finite3(mn) || !finite3(mx)) return fail(c, VG_NONFINITE, "non-finite vorton position");
  const float margin = (1.0f + 2.0f) * radius;
  for (int a = 0; a < 3; ++a) {
    mn[a] -= margin * 1.0f;
    mx[a] += margin * 1.0f;
  }
  *out = define_shape(n, mn, mx, true);
  return VG_OK;
}

}  // namespace

// The state a step carries across its split at the Poisson solve.
struct vg::StepState {
  float4 *ps, *w, *vel;
  size_t n;
  float radius, dt;
  Geom g;
  CellLists cl;
  Tree t;
  float* velgrid;
  float* vecpot;   // Poisson technique: the solution (boundary values and warm start set)
  float* negvort;  // ... and the right-hand side
};

bool vg::split_problem(Ctx* c, MgBatchItem* out) {
  if (!c->split || !c->split->vecpot) return false;
  out->c = c;
  out->g = c->split->g;
  out->soln = c->split->vecpot;
  out->rhs = c->split->negvort;
  return true;
}

namespace {

// The step up to the Poisson solve: grid, cell lists, tree; for the Poisson
// technique the splat, the boundary values and the warm start; the other
// techniques evaluate the velocity grid here.
static vg_status step_front(Ctx* c, StepState& s, const float* first_pos, const float* extra_min,
                            const float* extra_max) {
  vg_status st = step_geometry(c, s.ps, s.n, first_pos, s.radius, extra_min, extra_max, &s.g);
  if (st != VG_OK) return st;
  const Geom& g = s.g;
  float4 *ps = s.ps, *w = s.w, *vel = s.vel;
  const size_t n = s.n;
  const float radius = s.radius;
  const size_t pts = g.points();
  const bool ref = c->cfg.numerics == VG_NUMERICS_REFERENCE;
  // Cell lists serve the tree, the splat and PSE; the direct technique
  // without diffusion needs none.
  const int tech = c->cfg.velocity_technique;
  s.cl = {nullptr, nullptr, nullptr};
  if (tech != VG_VELOCITY_DIRECT || c->cfg.enable_diffusion) {
    if ((st = build_cell_lists(c, g, ps, n, &s.cl)) != VG_OK) return st;
  }
  s.velgrid = (float*)ws(c, S_VEL, pts * 3 * sizeof(float), &st);
  if (st != VG_OK) return st;
  s.t.depth = 0;
  s.vecpot = s.negvort = nullptr;
  c->stats.poisson_cycles = 0;
  c->stats.poisson_relres = 0.0;
  c->stats.poisson_relres0 = 0.0;
  c->stats.ms_poisson = 0.f;
  if (tech == VG_VELOCITY_POISSON || tech == VG_VELOCITY_TREE) {
    if ((st = build_tree(c, g, ps, w, n, s.cl, &s.t)) != VG_OK) return st;
  }
  if (tech == VG_VELOCITY_POISSON) {
    float* negvort = (float*)ws(c, S_NEGVORT, pts * 3 * sizeof(float), &st);
    if (st != VG_OK) return st;
    float* vecpot = (float*)ws(c, S_VECPOT, pts * 3 * sizeof(float), &st);
    if (st != VG_OK) return st;
    s.negvort = negvort;
    s.vecpot = vecpot;
    if ((st = launch_splat(c, g, ps, w, n, s.cl, -1.0f, radius, negvort)) != VG_OK) return st;
    const bool warm_prev = c->cfg.warm_start == VG_WARM_PREVIOUS && c->have_prev &&
                           memcmp(&c->prev_grid, &g, sizeof(Geom)) == 0;
    c->stats.warm_start_used = warm_prev ? VG_WARM_PREVIOUS : VG_WARM_ZERO;
    if (warm_prev) {
      float* prev = (float*)c->buf[S_PREV].p;
      VG_CUDA(c, cudaMemcpyAsync(vecpot, prev, pts * 3 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    } else {
      VG_CUDA(c, cudaMemsetAsync(vecpot, 0, pts * 3 * sizeof(float), c->stream));
    }
    if ((st = launch_boundary_vecpot(c, s.t, g, ps, w, n, c->cfg.boundary_copy_odd_x != 0, ref, vecpot)) != VG_OK)
      return st;
    VG_CUDA(c, cudaEventRecord(c->ev2, c->stream));
    // the network's guess counts as part of the solve's time
    if (c->cfg.warm_start == VG_WARM_NETWORK && c->net && nn::fits(c->net, g)) {
      if ((st = nn::guess(c, c->net, g, negvort, vecpot)) != VG_OK) return st;
      c->stats.warm_start_used = VG_WARM_NETWORK;
    }
    return VG_OK;
  }
  // velocity at gridpoints by treecode (auto mollification, vortonSim.cpp:2458-2477) or direct sum;
  // the direct technique also evaluates every vorton, in the same launch
  const size_t nq = pts + (tech == VG_VELOCITY_DIRECT ? n : 0);
  float4* q = (float4*)ws(c, S_JAC, nq * sizeof(float4) * 2, &st);
  if (st != VG_OK) return st;
  float4* out4 = q + nq;
  // the direct technique also evaluates every vorton, whose records follow the gridpoints
  // (the FAST direct kernel forms the gridpoint positions itself and reads the vortons' records)
  if (tech == VG_VELOCITY_TREE || ref) {
    pdl_launch(c->stream, blocks_for(nq, 256), 256, 0, k_grid_points, g, q,
               tech == VG_VELOCITY_DIRECT ? (const float4*)ps : nullptr, nq - pts);
    VG_LAUNCHED(c);
  }
  float sr = 1.0f, sc = 1.0f;
  if (tech == VG_VELOCITY_TREE) {
    volatile float cv = g.cell[0] * g.cell[1];
    cv = cv * g.cell[2];
    const float cgl = 1.0f * powf(cv, 1.0f / 3.0f);
    sr = std::max(cgl / radius, 1.0f);
    volatile float s3 = sr * sr;
    s3 = s3 * sr;
    sc = 1.0f / s3;
    if ((st = launch_tree_eval(c, 0, ref, s.t, ps, w, n, q, pts, sr, sc, out4)) != VG_OK) return st;
  } else {
    // COMPUTE_VELOCITY_AT_VORTONS (vorton.h:63-69): direct velocity at every vorton too;
    // the multi-chunk reduction writes the grid and vortons directly
    DirectSplit split = {s.velgrid, pts, vel, &g, (const float4*)ps};
    // the vortons' Euler step folded into the reduction when no later stage
    // of the step reads their positions (stretch and PSE do)
    if (c->step_evolve && !c->cfg.enable_stretch && !c->cfg.enable_diffusion) {
      split.evolve_pos = ps;
      split.evolve_dt = s.dt;
    }
    bool done = false;
    if ((st = launch_direct(c, 0, ref, ps, w, n, q, nq, 1.0f, 1.0f, out4, &split, &done)) != VG_OK) return st;
    if (done) return VG_OK;
  }
  // gridpoint velocities to the grid, and (direct technique) the vortons' velocities to vel
  pdl_launch(c->stream, blocks_for(nq, 256), 256, 0, k_f4_to_f3, out4, s.velgrid, pts,
             tech == VG_VELOCITY_DIRECT ? vel : (float4*)nullptr, nq - pts);
  VG_LAUNCHED(c);
  return VG_OK;
}

// The Poisson solve: the reference cascade, the fixed multigrid schedule, or
// the adaptive multigrid to the tolerance.
static vg_status step_solve(Ctx* c, StepState& s) {
  vg_status st = VG_OK;
  if (c->cfg.poisson_solver == VG_POISSON_REFERENCE_CASCADE) {
    if ((st = run_cascade(c, s.g, s.vecpot, s.negvort, c->cfg.cascade_steps)) != VG_OK) return st;
  } else if (c->mg_fixed_k1 > 0) {
    // fixed schedule: no host round trip; the residuals are read at vg_get_stats
    if ((st = run_multigrid_fixed(c, s.g, s.vecpot, s.negvort)) != VG_OK) return st;
    c->stats.poisson_cycles = c->mg_fixed_k1 + c->mg_fixed_k2;
  } else {
    int cyc = 0;
    double r0 = 0, r1 = 0;
    st = run_multigrid(c, s.g, s.vecpot, s.negvort, c->cfg.poisson_tolerance, c->cfg.poisson_max_cycles, &cyc, &r0,
                       &r1);
    c->stats.poisson_cycles = cyc;
    c->stats.poisson_relres0 = r0;
    c->stats.poisson_relres = r1;
    if (st != VG_OK && st != VG_NOT_CONVERGED) return st;
  }
  return VG_OK;
}

__global__ void k_evolve(float4* __restrict__ pos, const float4* __restrict__ vel, int m, float dt) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  float4 p = pos[i];
  const float4 v = vel[i];
  p.x = __fadd_rn(p.x, __fmul_rn(v.x, dt));  // pcl.mPosition += pcl.mVelocity * timeStep
  p.y = __fadd_rn(p.y, __fmul_rn(v.y, dt));
  p.z = __fadd_rn(p.z, __fmul_rn(v.z, dt));
  pos[i] = p;
}

// The step after the solve: curl of the vector potential, stretching, PSE,
// and the vortons' velocity from the grid.
static vg_status step_back(Ctx* c, StepState& s) {
  const Geom& g = s.g;
  const size_t pts = g.points(), n = s.n;
  const int tech = c->cfg.velocity_technique;
  vg_status st = VG_OK;
  if (tech == VG_VELOCITY_POISSON) {
    VG_CUDA(c, cudaEventRecord(c->ev3, c->stream));
    if (c->cfg.warm_start == VG_WARM_PREVIOUS) {
      float* prev = (float*)ws(c, S_PREV, pts * 3 * sizeof(float), &st);
      if (st != VG_OK) return st;
      VG_CUDA(c, cudaMemcpyAsync(prev, s.vecpot, pts * 3 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
      c->prev_grid = g;
      c->have_prev = true;
    }
    if ((st = launch_curl(c, g, s.vecpot, s.velgrid)) != VG_OK) return st;
  }
  if (c->cfg.enable_stretch) {
    if ((st = launch_stretch_vel(c, g, s.velgrid, s.ps, s.w, n, s.dt, s.cl.items)) != VG_OK) return st;
  }
  if (c->cfg.enable_diffusion) {
    if ((st = launch_pse(c, g, s.cl, s.ps, s.w, n, c->cfg.viscosity, s.dt)) != VG_OK) return st;
  }
  if (tech != VG_VELOCITY_DIRECT) {
    // AssignVelocityFromField(vortons, mVelGrid, 1) (vortonSim.cpp:4251-4255);
    // for vg_step_evolve_device with the Euler step of the same kernel
    if ((st = launch_gather_advect(c, g, s.velgrid, s.ps, s.vel, n, c->step_evolve ? s.dt : 0.0f, c->step_evolve,
                                   s.cl.items)) != VG_OK)
      return st;
    if (c->step_evolve) c->step_evolved = true;
  }
  if (c->step_evolve && !c->step_evolved) {  // PclOpEvolve on the vortons
    pdl_launch(c->stream, blocks_for(n, 256), 256, 0, k_evolve, s.ps, (const float4*)s.vel, (int)n, s.dt);
    VG_LAUNCHED(c);
    c->step_evolved = true;
  }
  VG_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  c->stats_pending = true;
  c->stats.grid = from_geom(g);
  c->stats.tree_depth = s.t.depth;
  c->stats.kernels_launched = c->launches;
  c->grid = g;
  c->have_grid = true;
  ++c->vel_gen;  // a new velocity grid (any by-cell copy is stale)
  return VG_OK;
}

// The step on device-resident vortons (ps: pos+size, w: angvel in place, vel
// out).  c->step_split 1 stops before the Poisson solve (the caller solves),
// 2 resumes after it with the state kept by 1 (the arguments are not read).
vg_status run_step(Ctx* c, float4* ps, float4* w, float4* vel, size_t n, const float* first_pos, float radius,
                   const float* extra_min, const float* extra_max, float dt) {
  if (!c->split) {
    c->split = new (std::nothrow) StepState();
    if (!c->split) return fail(c, VG_OOM, "out of host memory");
  }
  StepState& s = *c->split;
  vg_status st;
  if (c->step_split != 2) {
    if (n == 0) return fail(c, VG_EMPTY, "no vortons");
    if (n > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 vortons");
    c->launches = 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    VG_CUDA(c, cudaStreamIsCapturing(c->stream, &cap));
    c->step_captured = cap != cudaStreamCaptureStatusNone;
    VG_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    s.ps = ps;
    s.w = w;
    s.vel = vel;
    s.n = n;
    s.radius = radius;
    s.dt = dt;
    if ((st = step_front(c, s, first_pos, extra_min, extra_max)) != VG_OK) return st;
    if (c->step_split == 1) {
      if (s.vecpot) c->stats.poisson_cycles = c->mg_fixed_k1 + c->mg_fixed_k2;
      return VG_OK;
    }
    if (s.vecpot && (st = step_solve(c, s)) != VG_OK) return st;
  }
  return step_back(c, s);
}

}  // namespace

extern "C" {

unsigned vg_abi_version(void) { return VG_ABI_VERSION; }

const char* vg_status_string(vg_status s) {
  switch (s) {
    case VG_OK: return "ok";
    case VG_EMPTY: return "empty";
    case VG_OUT_OF_GRID: return "out of grid";
    case VG_NONFINITE: return "non-finite value";
    case VG_OOM: return "out of device memory";
    case VG_TIMEOUT: return "device wait timed out";
    case VG_INVALID: return "invalid argument";
    case VG_CUDA_ERROR: return "CUDA error";
    case VG_NOT_CONVERGED: return "not converged";
    case VG_TOO_LARGE: return "too large";
  }
  return "unknown status";
}

const char* vg_last_error(const vg_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err_noctx.c_str(); }

vg_status vg_config_default(vg_config* cfg) {
  if (!cfg) return VG_INVALID;
  memset(cfg, 0, sizeof(*cfg));
  cfg->abi_version = VG_ABI_VERSION;
  cfg->device = 0;
  cfg->stream = nullptr;
  cfg->velocity_technique = VG_VELOCITY_POISSON;
  cfg->numerics = VG_NUMERICS_FAST;
  cfg->poisson_solver = VG_POISSON_MULTIGRID;
  cfg->warm_start = VG_WARM_ZERO;
  cfg->viscosity = 0.01f;
  cfg->poisson_tolerance = 1e-6;
  cfg->poisson_max_cycles = 50;
  cfg->cascade_steps = 16;
  cfg->enable_stretch = 1;
  cfg->enable_diffusion = 1;
  cfg->boundary_copy_odd_x = 0;
  cfg->use_fixed_grid = 0;
  return VG_OK;
}

vg_status vg_create(const vg_config* cfg, vg_ctx** out) {
  if (!out) return VG_INVALID;
  *out = nullptr;
  vg_ctx* c = new (std::nothrow) vg_ctx();
  if (!c) return VG_OOM;
  vg_status st = check_cfg(c, cfg);
  if (st != VG_OK) {
    g_err_noctx = c->err;
    delete c;
    return st;
  }
  c->cfg = *cfg;
  cudaError_t e = cudaSetDevice(cfg->device);
  if (e == cudaSuccess && cfg->stream) {
    c->stream = (cudaStream_t)cfg->stream;
  } else if (e == cudaSuccess) {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    c->own_stream = e == cudaSuccess;
  }
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev2);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev3);
  if (e == cudaSuccess) e = cudaMalloc(&c->dflag, 256);
  if (e == cudaSuccess) e = cudaMemset(c->dflag, 0, 256);
  if (e == cudaSuccess) e = cudaHostAlloc(&c->hflag, 64, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaMalloc(&c->mg_relres_dev, 2 * sizeof(double));
  if (e != cudaSuccess) {
    g_err_noctx = std::string("vg_create: ") + cudaGetErrorString(e);
    cudaGetLastError();
    vg_destroy(c);
    return VG_CUDA_ERROR;
  }
  memset(&c->stats, 0, sizeof(c->stats));
  *out = c;
  return VG_OK;
}

static void destroy_host_graph(Ctx* c);

vg_status vg_destroy(vg_ctx* c) {
  if (!c) return VG_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int s = 0; s < S_NUM; ++s)
    if (c->buf[s].p) cudaFree(c->buf[s].p);
  for (MgGraphCache& G : c->mg_graph)
    if (G.exec) cudaGraphExecDestroy(G.exec);
  if (c->dflag) cudaFree(c->dflag);
  if (c->hflag) cudaFreeHost(c->hflag);
  if (c->mg_relres_dev) cudaFree(c->mg_relres_dev);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->ev2) cudaEventDestroy(c->ev2);
  if (c->ev3) cudaEventDestroy(c->ev3);
  if (c->aux) {
    cudaStreamSynchronize(c->aux);
    cudaStreamDestroy(c->aux);
  }
  if (c->aux_ev0) cudaEventDestroy(c->aux_ev0);
  if (c->aux_ev1) cudaEventDestroy(c->aux_ev1);
  if (c->aux_ev2) cudaEventDestroy(c->aux_ev2);
  if (c->aux_ev3) cudaEventDestroy(c->aux_ev3);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  delete c->split;
  destroy_host_graph(c);
  delete c;
  return VG_OK;
}

vg_status vg_set_network(vg_ctx* c, vg_net* net) {
  if (!c) return VG_INVALID;
  c->net = reinterpret_cast<vg::nn::Net*>(net);
  return VG_OK;
}

vg_status vg_set_config(vg_ctx* c, const vg_config* cfg) {
  if (!c) return VG_INVALID;
  vg_status st = check_cfg(c, cfg);
  if (st != VG_OK) return st;
  void* stream = c->cfg.stream;
  int dev = c->cfg.device;
  c->cfg = *cfg;
  c->cfg.stream = stream;  // stream and device are fixed at creation
  c->cfg.device = dev;
  return VG_OK;
}

// Tracer records on their way through the advection (vg_advect,
// vg_step_advect): the records (whole when at most 4x the 24 bytes used, as
// one contiguous copy each way; else their bytes [0, 24): position, velocity)
// staged on the device, then float4 position and velocity.
struct TracerJob {
  void* recs = nullptr;
  size_t m = 0, stride = 0, pitch = 0;
  bool whole = true;
  unsigned char* stage = nullptr;
  float4* p = nullptr;
  float4* v = nullptr;
};

static vg_status tracer_prepare(vg_ctx* c, void* particles, size_t m, size_t stride, TracerJob* t) {
  if (!particles || stride < 24 || stride % 4) return fail(c, VG_INVALID, "particles NULL or stride < 24 / unaligned");
  if (m > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 particles");
  vg_status st = VG_OK;
  t->recs = particles;
  t->m = m;
  t->stride = stride;
  t->whole = stride <= 4 * 24;
  t->pitch = t->whole ? stride : 24;
  const size_t rec_bytes = ((m * t->pitch + 255) / 256) * 256;
  t->stage = (unsigned char*)ws(c, S_TRACERS, rec_bytes + 2 * m * sizeof(float4), &st);
  if (st != VG_OK) return st;
  t->p = (float4*)(t->stage + rec_bytes);
  t->v = t->p + m;
  return VG_OK;
}

static cudaError_t tracer_upload(const TracerJob& t, cudaStream_t s) {
  if (t.whole) return cudaMemcpyAsync(t.stage, t.recs, t.m * t.stride, cudaMemcpyHostToDevice, s);
  return cudaMemcpy2DAsync(t.stage, 24, t.recs, t.stride, 12, t.m, cudaMemcpyHostToDevice, s);
}

// The gather + Euler step on the staged records and their copy back, on the
// context's stream, through the last step's velocity grid.
static vg_status tracer_advect_enqueue(vg_ctx* c, const TracerJob& t, float dt) {
  vg_status st = VG_OK;
  const size_t m = t.m;
  const float* vel3 = (const float*)c->buf[S_VEL].p;
  if (gather_by_cell(c->grid, m)) {
    // float4 positions and velocities out of the records, the by-cell gather, and back
    pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_copy_pos3, t.stage, t.pitch, (int)m, t.p);
    if ((st = launch_gather_advect(c, c->grid, vel3, t.p, t.v, m, dt, true, nullptr, true)) != VG_OK) return st;
    pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_store_posvel, t.stage, t.pitch, (int)m, t.p, t.v);
    VG_CUDA(c, cudaGetLastError());
  } else if ((st = launch_gather_advect_records(c, c->grid, vel3, t.stage, t.pitch, m, dt)) != VG_OK) {
    return st;
  }
  if (t.whole)
    VG_CUDA(c, cudaMemcpyAsync(t.recs, t.stage, m * t.stride, cudaMemcpyDeviceToHost, c->stream));
  else
    VG_CUDA(c, cudaMemcpy2DAsync(t.recs, t.stride, t.stage, 24, 24, m, cudaMemcpyDeviceToHost, c->stream));
  return VG_OK;
}


// The host-record step as one CUDA graph.  A frame's call (vg_step,
// vg_step_evolve, vg_step_advect) enqueues some twenty copies, kernels and
// event operations; while the same call repeats -- same records, sizes, dt,
// configuration and workspace -- its work is captured once and replayed with
// one launch.  Only where the step needs no host round trip (a fixed grid; for
// the Poisson technique, a fixed multigrid schedule) and the records are in
// pinned host memory.  The first call of a new key runs directly (and sizes
// the workspace), the second is captured.
struct vg::HostStepGraph {
  cudaGraphExec_t exec = nullptr;
  bool valid = false, nocapture = false;
  int seen = 0;
  const void* vortons = nullptr;
  const void* tracers = nullptr;
  size_t n = 0, stride = 0, m = 0, tstride = 0;
  float dt = 0.f, extra[6] = {0, 0, 0, 0, 0, 0};
  float size0 = 0.f;  // the first vorton's size, read on the host (its radius sets the mollification)
  bool evolve = false, has_extra = false;
  vg_config cfg;
  const void* net = nullptr;
  int k1 = 0, k2 = 0;
  bool coarse64 = false;
  void* bufs[S_NUM];
  size_t bytes[S_NUM];
};

static void destroy_host_graph(Ctx* c) {
  if (!c->host_graph) return;
  if (c->host_graph->exec) cudaGraphExecDestroy(c->host_graph->exec);
  delete c->host_graph;
  c->host_graph = nullptr;
}

static bool pinned_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

static void fill_key(Ctx* c, HostStepGraph* k, const void* vortons, size_t n, size_t stride, const void* tracers,
                     size_t m, size_t tstride, float dt, bool evolve, const float* emin, const float* emax) {
  k->vortons = vortons;
  k->n = n;
  k->stride = stride;
  k->tracers = tracers;
  k->m = m;
  k->tstride = tstride;
  k->dt = dt;
  k->size0 = ((const float*)vortons)[13];
  k->evolve = evolve;
  k->has_extra = emin && emax;
  for (int a = 0; a < 3; ++a) {
    k->extra[a] = k->has_extra ? emin[a] : 0.f;
    k->extra[3 + a] = k->has_extra ? emax[a] : 0.f;
  }
  memcpy(&k->cfg, &c->cfg, sizeof(vg_config));
  k->net = c->net;
  k->k1 = c->mg_fixed_k1;
  k->k2 = c->mg_fixed_k2;
  k->coarse64 = c->mg_coarse_fp64;
  for (int i = 0; i < S_NUM; ++i) {
    k->bufs[i] = c->buf[i].p;
    k->bytes[i] = c->buf[i].bytes;
  }
}

static bool same_key(const HostStepGraph& a, const HostStepGraph& b) {
  return a.vortons == b.vortons && a.n == b.n && a.stride == b.stride && a.tracers == b.tracers && a.m == b.m &&
         a.tstride == b.tstride && memcmp(&a.dt, &b.dt, sizeof(float)) == 0 &&
         memcmp(&a.size0, &b.size0, sizeof(float)) == 0 && a.evolve == b.evolve &&
         a.has_extra == b.has_extra && memcmp(a.extra, b.extra, sizeof(a.extra)) == 0 &&
         memcmp(&a.cfg, &b.cfg, sizeof(vg_config)) == 0 && a.net == b.net && a.k1 == b.k1 && a.k2 == b.k2 &&
         a.coarse64 == b.coarse64 && memcmp(a.bufs, b.bufs, sizeof(a.bufs)) == 0 &&
         memcmp(a.bytes, b.bytes, sizeof(a.bytes)) == 0;
}

// Whether this context's step can run from a graph (no host round trip inside).
static bool graph_step_possible(Ctx* c) {
  if (!c->cfg.use_fixed_grid) return false;
  if (c->cfg.velocity_technique == VG_VELOCITY_POISSON && c->cfg.poisson_solver != VG_POISSON_REFERENCE_CASCADE &&
      c->mg_fixed_k1 <= 0)
    return false;
  return true;
}

static vg_status step_records_body(vg_ctx* c, void* particles, size_t n, size_t stride, const float* extra_min,
                                   const float* extra_max, float dt, bool evolve, bool whole, size_t pitch,
                                   unsigned char* stage, float4* ps, float4* w, float4* vel, bool pack_on_aux);

// vg_step, vg_step_evolve and vg_step_advect on host records (evolve: the
// vortons move by velocity x dt before the records go back; tj: tracer
// records uploaded on a second stream during the step, then advected through
// its velocity grid).
static vg_status step_records(vg_ctx* c, void* particles, size_t n, size_t stride, const float* extra_min,
                              const float* extra_max, float dt, bool evolve, TracerJob* tj = nullptr) {
  if (!c) return VG_INVALID;
  if (n == 0) return fail(c, VG_EMPTY, "no vortons");
  if (!particles || stride < 56 || stride % 4) return fail(c, VG_INVALID, "particles NULL or stride < 56 / unaligned");
  if (!std::isfinite(dt)) return fail(c, VG_INVALID, "dt is not finite");
  vg_status st = VG_OK;
  // Records of up to 4x the 56 bytes used travel whole, as one contiguous copy
  // each way (a strided copy of short rows runs far below the link's rate;
  // kernels reading pinned records in place over the link measured slower
  // still); wider ones travel as their first 56 bytes.
  const bool whole = stride <= 4 * 56;
  const size_t pitch = whole ? stride : 56;
  unsigned char* stage = (unsigned char*)ws(c, S_HOSTSTAGE, n * pitch, &st);
  if (st != VG_OK) return st;
  float4* ps = (float4*)ws(c, S_POS, n * sizeof(float4), &st);
  if (st != VG_OK) return st;
  float4* w = (float4*)ws(c, S_ANGVEL, n * sizeof(float4), &st);
  if (st != VG_OK) return st;
  float4* vel = (float4*)ws(c, S_VVEL, n * sizeof(float4), &st);
  if (st != VG_OK) return st;
  if (tj) {
    if (!c->aux) VG_CUDA(c, cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    if (!c->aux_ev0) VG_CUDA(c, cudaEventCreateWithFlags(&c->aux_ev0, cudaEventDisableTiming));
    if (!c->aux_ev1) VG_CUDA(c, cudaEventCreateWithFlags(&c->aux_ev1, cudaEventDisableTiming));
    if (!c->aux_ev2) VG_CUDA(c, cudaEventCreateWithFlags(&c->aux_ev2, cudaEventDisableTiming));
    if (!c->aux_ev3) VG_CUDA(c, cudaEventCreateWithFlags(&c->aux_ev3, cudaEventDisableTiming));
  }
  const char* what = tj ? "vg_step_advect" : evolve ? "vg_step_evolve" : "vg_step";
  auto enqueue = [&]() -> vg_status {
    if (tj) {
      // the tracer records go up on the second stream while the vortons step
      // (after whatever the context's stream already holds)
      VG_CUDA(c, cudaEventRecord(c->aux_ev0, c->stream));
      VG_CUDA(c, cudaStreamWaitEvent(c->aux, c->aux_ev0, 0));
      VG_CUDA(c, tracer_upload(*tj, c->aux));
      VG_CUDA(c, cudaEventRecord(c->aux_ev1, c->aux));
    }
    vg_status est = step_records_body(c, particles, n, stride, extra_min, extra_max, dt, evolve, whole, pitch, stage,
                                      ps, w, vel, tj != nullptr);
    if (est == VG_OK && tj) {
      VG_CUDA(c, cudaStreamWaitEvent(c->stream, c->aux_ev1, 0));
      est = tracer_advect_enqueue(c, *tj, dt);
      // the vortons' records are back too before the call returns
      if (est == VG_OK) VG_CUDA(c, cudaStreamWaitEvent(c->stream, c->aux_ev3, 0));
    }
    return est;
  };
  // replay, capture, or run directly (the records' pinned check is made when
  // a key is new: a replayed key passed it)
  if (graph_step_possible(c)) {
    if (!c->host_graph) c->host_graph = new (std::nothrow) HostStepGraph();
    HostStepGraph* G = c->host_graph;
    HostStepGraph key;
    if (G) {
      fill_key(c, &key, particles, n, stride, tj ? tj->recs : nullptr, tj ? tj->m : 0, tj ? tj->stride : 0, dt,
               evolve, extra_min, extra_max);
      if (!(G->valid && same_key(*G, key)) && !(pinned_host(particles) && (!tj || pinned_host(tj->recs))))
        G = nullptr;  // pageable records: run directly
    }
    if (G) {
      const bool same = G->valid && same_key(*G, key);
      if (same && G->exec) {
        VG_CUDA(c, cudaGraphLaunch(G->exec, c->stream));
        ++c->vel_gen;  // the replayed step wrote a new velocity grid
        return sync_and_check(c, what);
      }
      if (same && !G->nocapture && G->seen >= 1) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          const vg_status cst = enqueue();
          const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
          if (cst == VG_OK && ce == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
            cudaGraphDestroy(graph);
            // the same call with the workspace as it stands after the capture
            fill_key(c, G, particles, n, stride, tj ? tj->recs : nullptr, tj ? tj->m : 0, tj ? tj->stride : 0, dt,
                     evolve, extra_min, extra_max);
            G->exec = exec;
            G->valid = true;
            VG_CUDA(c, cudaGraphLaunch(G->exec, c->stream));
            ++c->vel_gen;
            return sync_and_check(c, what);
          }
          if (graph) cudaGraphDestroy(graph);
        }
        cudaGetLastError();  // capture refused: run directly from now on for this call
        if (tj) cudaStreamSynchronize(c->aux);
        G->nocapture = true;
      } else if (!same) {
        if (G->exec) cudaGraphExecDestroy(G->exec);
        *G = key;
        G->exec = nullptr;
        G->valid = true;
        G->nocapture = false;
        G->seen = 0;
      }
      ++G->seen;
    }
  }
  st = enqueue();
  if (st != VG_OK) {
    if (tj) cudaStreamSynchronize(c->aux);  // no copy of the caller's records left in flight
    return st;
  }
  return sync_and_check(c, what);
}

// The vortons' part of step_records, enqueued on the context's stream.
static vg_status step_records_body(vg_ctx* c, void* particles, size_t n, size_t stride, const float* extra_min,
                                   const float* extra_max, float dt, bool evolve, bool whole, size_t pitch,
                                   unsigned char* stage, float4* ps, float4* w, float4* vel, bool pack_on_aux) {
  vg_status st = VG_OK;
  // record bytes [0, 56): position, velocity, orientation, angular velocity, density, size
  if (whole)
    VG_CUDA(c, cudaMemcpyAsync(stage, particles, n * stride, cudaMemcpyHostToDevice, c->stream));
  else
    VG_CUDA(c, cudaMemcpy2DAsync(stage, 56, particles, stride, 56, n, cudaMemcpyHostToDevice, c->stream));
  pdl_launch(c->stream, blocks_for(n, 256), 256, 0, k_unpack_records, stage, pitch, (int)n, ps, w);
  VG_CUDA(c, cudaGetLastError());
  const float* rec0 = (const float*)particles;
  const float radius = rec0[13] * 0.5f;  // Particle::GetRadius of the first vorton
  st = run_step(c, ps, w, vel, n, rec0, radius, extra_min, extra_max, dt);
  if (st != VG_OK) return st;
  // pack_on_aux: the vortons' records go back on the second stream while the
  // tracers are advected on the first (aux_ev3 marks their return)
  cudaStream_t ps_stream = c->stream;
  if (pack_on_aux) {
    VG_CUDA(c, cudaEventRecord(c->aux_ev2, c->stream));
    VG_CUDA(c, cudaStreamWaitEvent(c->aux, c->aux_ev2, 0));
    ps_stream = c->aux;
  }
  // write back record bytes [12, 48): velocity, (unchanged) orientation,
  // angular velocity (whole records carry their other bytes back unchanged);
  // evolving, bytes [0, 48) with the moved position
  if (evolve)
    pdl_launch(ps_stream, blocks_for(n, 256), 256, 0, k_pack_records_evolve, stage, pitch, (int)n, (const float4*)ps,
               (const float4*)vel, (const float4*)w, dt);
  else
    pdl_launch(ps_stream, blocks_for(n, 256), 256, 0, k_pack_records, stage + 12, pitch, (int)n, vel, w);
  VG_CUDA(c, cudaGetLastError());
  const size_t from = evolve ? 0 : 12;
  if (whole)
    VG_CUDA(c, cudaMemcpyAsync(particles, stage, n * stride, cudaMemcpyDeviceToHost, ps_stream));
  else
    VG_CUDA(c, cudaMemcpy2DAsync((unsigned char*)particles + from, stride, stage + from, 56, 48 - from, n,
                                 cudaMemcpyDeviceToHost, ps_stream));
  if (pack_on_aux) VG_CUDA(c, cudaEventRecord(c->aux_ev3, c->aux));
  return VG_OK;
}

vg_status vg_step(vg_ctx* c, void* particles, size_t n, size_t stride, const float* extra_min,
                  const float* extra_max, float dt, unsigned frame) {
  (void)frame;
  return step_records(c, particles, n, stride, extra_min, extra_max, dt, false);
}

vg_status vg_step_evolve(vg_ctx* c, void* particles, size_t n, size_t stride, const float* extra_min,
                         const float* extra_max, float dt, unsigned frame) {
  (void)frame;
  return step_records(c, particles, n, stride, extra_min, extra_max, dt, true);
}

vg_status vg_step_advect(vg_ctx* c, void* vortons, size_t n, size_t stride, const float* extra_min,
                         const float* extra_max, float dt, unsigned frame, int evolve_vortons, void* tracers,
                         size_t m, size_t tracer_stride) {
  (void)frame;
  if (!c) return VG_INVALID;
  if (m == 0) return step_records(c, vortons, n, stride, extra_min, extra_max, dt, evolve_vortons != 0);
  // the tracers' staging first: an allocation may synchronise the stream
  TracerJob tj;
  vg_status st = tracer_prepare(c, tracers, m, tracer_stride, &tj);
  if (st != VG_OK) return st;
  return step_records(c, vortons, n, stride, extra_min, extra_max, dt, evolve_vortons != 0, &tj);
}

vg_status vg_step_evolve_device(vg_ctx* c, float* pos_size, float* angvel, float* vel, size_t n,
                                const float* extra_minmax, float dt, unsigned frame) {
  if (!c) return VG_INVALID;
  c->step_evolve = true;
  c->step_evolved = false;
  const vg_status st = vg_step_device(c, pos_size, angvel, vel, n, extra_minmax, dt, frame);
  c->step_evolve = false;
  return st;
}

vg_status vg_step_device(vg_ctx* c, const float* pos_size, float* angvel, float* vel, size_t n,
                         const float* extra_minmax, float dt, unsigned frame) {
  (void)frame;
  if (!c) return VG_INVALID;
  if (n == 0) return fail(c, VG_EMPTY, "no vortons");
  if (!pos_size || !angvel || !vel) return fail(c, VG_INVALID, "NULL device pointer");
  // The first vorton (position for the box rule, radius for the margin and the
  // treecode's mollification) is only needed on the host when the grid is
  // derived from the bounding box or the treecode technique is used.
  float4 p0 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!c->cfg.use_fixed_grid || c->cfg.velocity_technique == VG_VELOCITY_TREE) {
    VG_CUDA(c, cudaMemcpyAsync(&p0, pos_size, sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  const float first[3] = {p0.x, p0.y, p0.z};
  return run_step(c, (float4*)pos_size, (float4*)angvel, (float4*)vel, n, first, p0.w * 0.5f,
                  extra_minmax, extra_minmax ? extra_minmax + 3 : nullptr, dt);
}

vg_status vg_get_velocity_grid(vg_ctx* c, float* xyz, size_t cap_points, vg_grid_geom* geom) {
  if (!c) return VG_INVALID;
  if (!c->have_grid) return fail(c, VG_EMPTY, "no step has run");
  if (geom) *geom = from_geom(c->grid);
  if (xyz) {
    if (cap_points < c->grid.points()) return fail(c, VG_TOO_LARGE, "velocity grid buffer too small");
    VG_CUDA(c, cudaMemcpyAsync(xyz, c->buf[S_VEL].p, c->grid.points() * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                               c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return VG_OK;
}

vg_status vg_get_velocity_grid_device(vg_ctx* c, const float** dev, vg_grid_geom* geom) {
  if (!c || !dev) return VG_INVALID;
  if (!c->have_grid) return fail(c, VG_EMPTY, "no step has run");
  *dev = (const float*)c->buf[S_VEL].p;
  if (geom) *geom = from_geom(c->grid);
  return VG_OK;
}

vg_status vg_get_vector_potential(vg_ctx* c, float* xyz, size_t cap_points, vg_grid_geom* geom) {
  if (!c) return VG_INVALID;
  if (!c->have_grid || c->cfg.velocity_technique != VG_VELOCITY_POISSON)
    return fail(c, VG_EMPTY, "no Poisson step has run");
  if (geom) *geom = from_geom(c->grid);
  if (xyz) {
    if (cap_points < c->grid.points()) return fail(c, VG_TOO_LARGE, "vector potential buffer too small");
    VG_CUDA(c, cudaMemcpyAsync(xyz, c->buf[S_VECPOT].p, c->grid.points() * 3 * sizeof(float),
                               cudaMemcpyDeviceToHost, c->stream));
    VG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return VG_OK;
}

vg_status vg_get_stats(vg_ctx* c, vg_step_stats* s) {
  if (!c || !s) return VG_INVALID;
  if (c->stats_pending) {
    if (c->step_captured) {
      // a step replayed from a graph: no per-step times; the caller has
      // synchronised the graph's stream before asking
      c->stats.ms_total = c->stats.ms_poisson = 0.f;
    } else {
      VG_CUDA(c, cudaEventSynchronize(c->ev1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->ev0, c->ev1);
      c->stats.ms_total = ms;
      if (c->cfg.velocity_technique == VG_VELOCITY_POISSON && cudaEventElapsedTime(&ms, c->ev2, c->ev3) == cudaSuccess)
        c->stats.ms_poisson = ms;
      cudaGetLastError();
    }
    if (c->cfg.velocity_technique == VG_VELOCITY_POISSON && c->mg_fixed_k1 > 0 &&
        c->cfg.poisson_solver == VG_POISSON_MULTIGRID) {
      double h[2] = {0.0, 0.0};
      VG_CUDA(c, cudaMemcpy(h, c->mg_relres_dev, sizeof(h), cudaMemcpyDeviceToHost));
      c->stats.poisson_relres = h[0];
      c->stats.poisson_relres0 = h[1];
    }
    c->stats_pending = false;
  }
  *s = c->stats;
  return VG_OK;
}

vg_status vg_synchronize(vg_ctx* c) {
  if (!c) return VG_INVALID;
  return sync_and_check(c, "device stage");
}

vg_status vg_advect(vg_ctx* c, void* particles, size_t m, size_t stride, float dt) {
  if (!c) return VG_INVALID;
  if (!c->have_grid) return fail(c, VG_EMPTY, "no velocity grid yet: run a step first");
  if (m == 0) return VG_OK;
  TracerJob t;
  vg_status st = tracer_prepare(c, particles, m, stride, &t);
  if (st != VG_OK) return st;
  VG_CUDA(c, tracer_upload(t, c->stream));
  if ((st = tracer_advect_enqueue(c, t, dt)) != VG_OK) return st;
  return sync_and_check(c, "vg_advect");
}

vg_status vg_advect_device(vg_ctx* c, float* pos, float* vel, size_t m, float dt) {
  if (!c) return VG_INVALID;
  if (!c->have_grid) return fail(c, VG_EMPTY, "no velocity grid yet: run a step first");
  if (!pos) return fail(c, VG_INVALID, "NULL position pointer");
  return launch_gather_advect(c, c->grid, (const float*)c->buf[S_VEL].p, (float4*)pos, (float4*)vel, m, dt, true,
                              nullptr, true);
}

namespace {
}  // namespace

vg_status vg_evolve_device(vg_ctx* c, float* pos4, const float* vel4, size_t m, float dt) {
  if (!c || (m && (!pos4 || !vel4))) return VG_INVALID;
  if (m == 0) return VG_OK;
  if (m > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 particles");
  pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_evolve, (float4*)pos4, (const float4*)vel4, (int)m, dt);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

// ------------------------------------------------------------ stage entry points

vg_status vg_define_shape(size_t n, const float vmin[3], const float vmax[3], int pow2, vg_grid_geom* out) {
  if (!vmin || !vmax || !out) return VG_INVALID;
  *out = from_geom(define_shape(n, vmin, vmax, pow2 != 0));
  return VG_OK;
}

namespace {
__global__ void k_bin_only(Geom g, const float4* __restrict__ pos, int m, unsigned* __restrict__ idx3,
                           unsigned* __restrict__ off) {
  pdl_entry();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float4 p = pos[i];
  const unsigned ix = bin_axis(p.x, g.mn[0], g.cpe[0]);
  const unsigned iy = bin_axis(p.y, g.mn[1], g.cpe[1]);
  const unsigned iz = bin_axis(p.z, g.mn[2], g.cpe[2]);
  if (idx3) {
    idx3[3 * i] = ix;
    idx3[3 * i + 1] = iy;
    idx3[3 * i + 2] = iz;
  }
  if (off) off[i] = ix + g.np[0] * (iy + g.np[1] * iz);
}
}  // namespace

vg_status vg_bin_device(vg_ctx* c, const vg_grid_geom* g, const float* pos4, size_t m, unsigned* idx3,
                        unsigned* offset) {
  if (!c || !g || (!pos4 && m)) return VG_INVALID;
  if (m == 0) return VG_OK;
  pdl_launch(c->stream, blocks_for(m, 256), 256, 0, k_bin_only, to_geom(*g), (const float4*)pos4, (int)m, idx3, offset);
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status vg_set_poisson_schedule(vg_ctx* c, int k1, int k2) {
  if (!c || k1 < 0 || k2 < 0 || (k1 == 0 && k2 != 0)) return VG_INVALID;
  c->mg_fixed_k1 = k1;
  c->mg_fixed_k2 = k2;
  return VG_OK;
}

vg_status vg_set_coarsest_fp64(vg_ctx* c, int on) {
  if (!c) return VG_INVALID;
  const bool v = on != 0;
  if (c->mg_coarse_fp64 != v) {
    c->mg_coarse_fp64 = v;
    for (MgGraphCache& G : c->mg_graph)  // the captured cycles hold the other precision's kernels
      if (G.exec) {
        cudaGraphExecDestroy(G.exec);
        G.exec = nullptr;
      }
  }
  return VG_OK;
}

vg_status vg_get_poisson_schedule(const vg_ctx* c, int* k1, int* k2) {
  if (!c || !k1 || !k2) return VG_INVALID;
  *k1 = c->mg_last_k1;
  *k2 = c->mg_last_k2;
  return VG_OK;
}

vg_status vg_partition_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos4, size_t n, unsigned* start,
                              unsigned* items) {
  if (!c || !gg || !start || (n && (!pos4 || !items))) return VG_INVALID;
  const Geom g = to_geom(*gg);
  CellLists cl;
  vg_status st = build_cell_lists(c, g, (const float4*)pos4, n, &cl);
  if (st != VG_OK) return st;
  VG_CUDA(c, cudaMemcpyAsync(start, cl.start, (g.points() + 2) * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                             c->stream));
  if (n) VG_CUDA(c, cudaMemcpyAsync(items, cl.items, n * sizeof(unsigned), cudaMemcpyDeviceToDevice, c->stream));
  return VG_OK;
}

vg_status vg_direct_device(vg_ctx* c, int kind, const float* pos_size, const float* angvel, size_t n, const float* q4,
                           size_t m, float sr, float sc, float* out4) {
  if (!c || (kind != 0 && kind != 1)) return VG_INVALID;
  return launch_direct(c, kind, c->cfg.numerics == VG_NUMERICS_REFERENCE, (const float4*)pos_size,
                       (const float4*)angvel, n, (const float4*)q4, m, sr, sc, (float4*)out4);
}

vg_status vg_direct_grid_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos_size, const float* angvel,
                                size_t n, float* velgrid3, float* vel4) {
  if (!c || !gg || !velgrid3 || (n && (!pos_size || !angvel))) return VG_INVALID;
  if (n > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 vortons");
  const Geom g = to_geom(*gg);
  const size_t pts = g.points();
  if (pts == 0 || pts > 0x3fffffff) return fail(c, VG_INVALID, "direct grid: empty or oversized grid");
  const size_t nq = pts + (vel4 ? n : 0);
  vg_status st = VG_OK;
  float4* q = (float4*)ws(c, S_JAC, nq * sizeof(float4) * 2, &st);
  if (st != VG_OK) return st;
  float4* out4 = q + nq;
  const bool ref = c->cfg.numerics == VG_NUMERICS_REFERENCE;
  if (ref) {  // the reference-order kernel reads every target's position
    pdl_launch(c->stream, blocks_for(nq, 256), 256, 0, k_grid_points, g, q, vel4 ? (const float4*)pos_size : nullptr,
               nq - pts);
    VG_LAUNCHED(c);
  }
  const DirectSplit split = {velgrid3, pts, (float4*)vel4, &g, (const float4*)pos_size};
  bool done = false;
  if ((st = launch_direct(c, 0, ref, (const float4*)pos_size, (const float4*)angvel, n, q, nq, 1.0f, 1.0f, out4,
                          &split, &done)) != VG_OK)
    return st;
  if (!done) {
    pdl_launch(c->stream, blocks_for(nq, 256), 256, 0, k_f4_to_f3, (const float4*)out4, velgrid3, pts, (float4*)vel4,
               nq - pts);
    VG_LAUNCHED(c);
  }
  VG_CUDA(c, cudaGetLastError());
  return VG_OK;
}

vg_status vg_tree_device(vg_ctx* c, int kind, const vg_grid_geom* gg, const float* pos_size, const float* angvel,
                         size_t n, const float* q4, size_t m, float sr, float sc, float* out4, float* tree_out,
                         size_t tree_cap_points, size_t* tree_points) {
  if (!c || !gg || (kind != 0 && kind != 1)) return VG_INVALID;
  if (n == 0) return fail(c, VG_EMPTY, "no vortons");
  Geom g = to_geom(*gg);
  CellLists cl;
  vg_status st = build_cell_lists(c, g, (const float4*)pos_size, n, &cl);
  if (st != VG_OK) return st;
  Tree t;
  if ((st = build_tree(c, g, (const float4*)pos_size, (const float4*)angvel, n, cl, &t)) != VG_OK) return st;
  if (tree_points) *tree_points = t.total;
  if (tree_out) {
    if (tree_cap_points < t.total) return fail(c, VG_TOO_LARGE, "tree buffer too small");
    VG_CUDA(c, cudaMemcpy2DAsync(tree_out, 32, t.sv_pos, 16, 16, t.total, cudaMemcpyDeviceToDevice, c->stream));
    VG_CUDA(c, cudaMemcpy2DAsync(tree_out + 4, 32, t.sv_w, 16, 16, t.total, cudaMemcpyDeviceToDevice, c->stream));
  }
  if (m && q4 && out4)
    return launch_tree_eval(c, kind, c->cfg.numerics == VG_NUMERICS_REFERENCE, t, (const float4*)pos_size,
                            (const float4*)angvel, n, (const float4*)q4, m, sr, sc, (float4*)out4);
  return VG_OK;
}

vg_status vg_splat_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos_size, const float* angvel, size_t n,
                          float scale, float* grid3) {
  if (!c || !gg || !grid3) return VG_INVALID;
  Geom g = to_geom(*gg);
  CellLists cl;
  vg_status st = build_cell_lists(c, g, (const float4*)pos_size, n, &cl);
  if (st != VG_OK) return st;
  return launch_splat(c, g, (const float4*)pos_size, (const float4*)angvel, n, cl, scale, -1.0f, grid3);
}

vg_status vg_boundary_vecpot_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos_size, const float* angvel,
                                    size_t n, int copy_odd_x, float* grid3) {
  if (!c || !gg || !grid3) return VG_INVALID;
  if (n == 0) return fail(c, VG_EMPTY, "no vortons");
  Geom g = to_geom(*gg);
  CellLists cl;
  vg_status st = build_cell_lists(c, g, (const float4*)pos_size, n, &cl);
  if (st != VG_OK) return st;
  Tree t;
  if ((st = build_tree(c, g, (const float4*)pos_size, (const float4*)angvel, n, cl, &t)) != VG_OK) return st;
  return launch_boundary_vecpot(c, t, g, (const float4*)pos_size, (const float4*)angvel, n, copy_odd_x != 0,
                                c->cfg.numerics == VG_NUMERICS_REFERENCE, grid3);
}

vg_status vg_sor_device(vg_ctx* c, const vg_grid_geom* g, float* soln3, const float* lap3, int steps) {
  if (!c || !g || !soln3 || !lap3) return VG_INVALID;
  return launch_sor(c, to_geom(*g), soln3, lap3, steps);
}

vg_status vg_cascade_device(vg_ctx* c, const vg_grid_geom* g, float* soln3, const float* rhs3, int steps) {
  if (!c || !g || !soln3 || !rhs3) return VG_INVALID;
  return run_cascade(c, to_geom(*g), soln3, rhs3, steps);
}

vg_status vg_multigrid_device(vg_ctx* c, const vg_grid_geom* g, float* soln3, const float* rhs3, double tol,
                              int max_cycles, int* cycles, double* relres0, double* relres) {
  if (!c || !g || !soln3 || !rhs3 || !(tol > 0.0)) return VG_INVALID;
  return run_multigrid(c, to_geom(*g), soln3, rhs3, tol, max_cycles, cycles, relres0, relres);
}

vg_status vg_downsample_device(vg_ctx* c, const vg_grid_geom* fine, const float* fine3, const vg_grid_geom* coarse,
                               int inject, float* coarse3) {
  if (!c || !fine || !coarse || !fine3 || !coarse3) return VG_INVALID;
  return launch_downsample(c, to_geom(*fine), fine3, to_geom(*coarse), inject != 0, coarse3);
}

vg_status vg_upsample_device(vg_ctx* c, const vg_grid_geom* coarse, const float* coarse3, const vg_grid_geom* fine,
                             int interior_only, float* fine3) {
  if (!c || !fine || !coarse || !fine3 || !coarse3) return VG_INVALID;
  return launch_upsample(c, to_geom(*coarse), coarse3, to_geom(*fine), interior_only != 0, fine3);
}

vg_status vg_jacobian_curl_device(vg_ctx* c, const vg_grid_geom* gg, const float* vec3, float* jac9, float* curl3) {
  if (!c || !gg || !vec3) return VG_INVALID;
  const Geom g = to_geom(*gg);
  vg_status st = VG_OK;
  if (jac9 && (st = launch_jacobian(c, g, vec3, jac9)) != VG_OK) return st;
  if (curl3 && (st = launch_curl(c, g, vec3, curl3)) != VG_OK) return st;
  return VG_OK;
}

vg_status vg_stretch_device(vg_ctx* c, const vg_grid_geom* gg, const float* vel3, const float* pos_size,
                            float* angvel, size_t n, float dt) {
  if (!c || !gg || !vel3) return VG_INVALID;
  const Geom g = to_geom(*gg);
  vg_status st = VG_OK;
  float* jac = (float*)ws(c, S_JAC, g.points() * 9 * sizeof(float), &st);
  if (st != VG_OK) return st;
  if ((st = launch_jacobian(c, g, vel3, jac)) != VG_OK) return st;
  return launch_stretch(c, g, jac, (const float4*)pos_size, (float4*)angvel, n, dt);
}

vg_status vg_pse_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos_size, float* angvel, size_t n,
                        float viscosity, float dt) {
  if (!c || !gg) return VG_INVALID;
  const Geom g = to_geom(*gg);
  CellLists cl;
  vg_status st = build_cell_lists(c, g, (const float4*)pos_size, n, &cl);
  if (st != VG_OK) return st;
  return launch_pse(c, g, cl, (const float4*)pos_size, (float4*)angvel, n, viscosity, dt);
}

vg_status vg_heat_pse_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos_size, float* density, size_t n,
                             float diffusivity, float ambient_density, float dt) {
  if (!c || !gg || (n && (!pos_size || !density))) return VG_INVALID;
  if (n == 0) return VG_OK;
  if (n > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 vortons");
  const Geom g = to_geom(*gg);
  CellLists cl;
  vg_status st = build_cell_lists(c, g, (const float4*)pos_size, n, &cl);
  if (st != VG_OK) return st;
  return launch_heat_pse(c, g, cl, (const float4*)pos_size, density, n, diffusivity, ambient_density, dt);
}

vg_status vg_gather_advect_device(vg_ctx* c, const vg_grid_geom* gg, const float* vel3, float* pos4, float* vel4,
                                  size_t m, float dt) {
  if (!c || !gg || !vel3 || (!pos4 && m)) return VG_INVALID;
  return launch_gather_advect(c, to_geom(*gg), vel3, (float4*)pos4, (float4*)vel4, m, dt, true);
}

vg_status vg_density_grid_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos_size, const float* density,
                                 size_t n, float ambient_density, float* density_grid) {
  if (!c || !gg || !density_grid || (n && (!pos_size || !density))) return VG_INVALID;
  if (n > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 vortons");
  return launch_density_grid(c, to_geom(*gg), (const float4*)pos_size, density, n, ambient_density, density_grid);
}

vg_status vg_gradient_device(vg_ctx* c, const vg_grid_geom* gg, const float* scalar, float* grad3) {
  if (!c || !gg || !scalar || !grad3) return VG_INVALID;
  const Geom g = to_geom(*gg);
  if (g.np[0] < 2 || g.np[1] < 2 || g.np[2] < 2) return fail(c, VG_INVALID, "gradient: fewer than 2 points on an axis");
  return launch_gradient(c, g, scalar, grad3);
}

vg_status vg_baroclinic_device(vg_ctx* c, const vg_grid_geom* gg, const float* pos_size, const float* density,
                               float* angvel, size_t n, const float grav[3], float ambient_density, float dt,
                               int* applied) {
  if (!c || !gg || !grav || (n && (!pos_size || !density || !angvel))) return VG_INVALID;
  if (applied) *applied = 0;
  if (n == 0) return VG_OK;
  if (n > 0x7fffffff) return fail(c, VG_TOO_LARGE, "more than 2^31 vortons");
  if (!(ambient_density > 0.0f)) return fail(c, VG_INVALID, "baroclinic: ambient density must be positive");
  const Geom g = to_geom(*gg);
  if (g.np[0] < 2 || g.np[1] < 2 || g.np[2] < 2) return fail(c, VG_INVALID, "baroclinic: fewer than 2 points on an axis");
  // no extent along gravity: nothing to generate (vortonSim.cpp:3417-3421)
  const float gdot = grav[0] * g.ext[0] + grav[1] * g.ext[1] + grav[2] * g.ext[2];
  if (fabsf(gdot) < FLT_EPSILON) return VG_OK;
  vg_status st = VG_OK;
  const size_t pts = g.points();
  float* dens = (float*)ws(c, S_DENS, pts * sizeof(float), &st);
  if (st != VG_OK) return st;
  float* grad = (float*)ws(c, S_GRAD, pts * 3 * sizeof(float), &st);
  if (st != VG_OK) return st;
  if ((st = launch_density_grid(c, g, (const float4*)pos_size, density, n, ambient_density, dens)) != VG_OK) return st;
  if ((st = launch_gradient(c, g, dens, grad)) != VG_OK) return st;
  if ((st = launch_baroclinic(c, g, grad, (const float4*)pos_size, (float4*)angvel, n, grav, ambient_density, dt)) !=
      VG_OK)
    return st;
  if (applied) *applied = 1;
  return VG_OK;
}

vg_status vg_signed_distance_device(vg_ctx* c, const vg_grid_geom* gg, const float* density_grid,
                                    float ambient_density, int reference_stats, float* sdf) {
  if (!c || !gg || !density_grid || !sdf) return VG_INVALID;
  const Geom g = to_geom(*gg);
  if (g.np[0] < 2 || g.np[1] < 2 || g.np[2] < 2) return fail(c, VG_INVALID, "signed distance: fewer than 2 points on an axis");
  const size_t pts = g.points();
  if (pts > 0x7fffffff) return fail(c, VG_TOO_LARGE, "signed distance: more than 2^31 points");
  const int nb = 2 * sm_count();
  vg_status st = VG_OK;
  const size_t pin_bytes = (pts + 255) / 256 * 256;
  char* w = (char*)ws(c, S_SDF, pin_bytes + 64 + (size_t)nb * 4 * sizeof(double), &st);
  if (st != VG_OK) return st;
  return launch_signed_distance(c, g, density_grid, ambient_density, reference_stats != 0, sdf, (unsigned char*)w,
                                (float*)(w + pin_bytes), (double*)(w + pin_bytes + 64), nb);
}

vg_status vg_marching_cubes_device(vg_ctx* c, const vg_grid_geom* gg, const float* values, float iso_level,
                                   float* vertices, float* normals, size_t max_triangles, size_t* triangles) {
  if (!c || !gg || !values || !triangles || (max_triangles && !vertices)) return VG_INVALID;
  const Geom g = to_geom(*gg);
  if (g.np[0] < 2 || g.np[1] < 2 || g.np[2] < 2) return fail(c, VG_INVALID, "marching cubes: fewer than 2 points on an axis");
  if (g.points() > 0x7fffffff) return fail(c, VG_TOO_LARGE, "marching cubes: more than 2^31 points");
  return launch_marching_cubes(c, g, values, iso_level, vertices, normals, max_triangles, triangles);
}

}  // extern "C"
