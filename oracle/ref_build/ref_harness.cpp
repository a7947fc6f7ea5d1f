/* C-ABI harness over the reference's own VortonSim code (built from the staged
 * reference sources by oracle/ref_build/Makefile).
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, smoke() and bench.py's CPU-baseline leg
 * call this library to (a) generate golden vectors that pin the C oracle and
 * (b) time the reference's own CPU path.  The product never links it.
 *
 * Every entry point calls the reference's functions in the order the
 * reference's VortonSim step calls them (VortonFluid/vortonSim.cpp,
 * Core/SpatialPartition/uniformGrid.h, uniformGridMath.cpp,
 * Particles/Operation/pclOpAdvect.cpp, pclOpEvolve.cpp); this file is glue
 * that moves flat float arrays in and out of the reference's containers.
 *
 * Vortons cross this boundary as the reference's own Particle records
 * (sizeof(Particle) bytes each, see vgref_sizeof_particle).
 */
#define private public
#define protected public
#include "VortonFluid/vortonSim.h"
#include "VortonFluid/pclOpVortonSim.h"
#include "Particles/Operation/pclOpFindBoundingBox.h"
#include "Particles/Operation/pclOpKillAge.h"
#include "Particles/Operation/pclOpWind.h"
#include "Particles/Operation/pclOpEmit.h"
#include "Core/SpatialPartition/uniformGridMath.h"
#include "FluidBodySim/fluidBodySim.h"
#include "Impulsion/physicalObject.h"
#include "Impulsion/rigidBody.h"
#include "Collision/sphereShape.h"
#include "Collision/convexPolytope.h"
#undef private
#undef protected
#include <cstring>
#include <vector>
#include "tbb/vg_tbb.h"  /* blocked_range for the serial build too */

#if ! USE_TBB
unsigned gNumberOfProcessors = 1;
#endif

extern void AssignVelocityFromField(VECTOR<Particle>& particles, const UniformGrid<Vec3>* velocityGrid, const float gain);

namespace {

struct Geom {
  float mn[3], ext[3], cell[3], cpe[3];
  unsigned np[3];
};

void load_geom(UniformGridGeometry& g, const float* geom12, const unsigned* np) {
  g.mMinCorner = Vec3(geom12[0], geom12[1], geom12[2]);
  g.mGridExtent = Vec3(geom12[3], geom12[4], geom12[5]);
  g.mNumPoints[0] = np[0];
  g.mNumPoints[1] = np[1];
  g.mNumPoints[2] = np[2];
  g.PrecomputeSpacing();
}

void store_geom(const UniformGridGeometry& g, float* geom12, unsigned* np) {
  const Vec3& a = g.GetMinCorner();
  const Vec3& b = g.GetExtent();
  const Vec3& c = g.GetCellSpacing();
  const Vec3& d = g.GetCellsPerExtent();
  const float v[12] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z, d.x, d.y, d.z};
  std::memcpy(geom12, v, sizeof(v));
  np[0] = g.GetNumPoints(0);
  np[1] = g.GetNumPoints(1);
  np[2] = g.GetNumPoints(2);
}

void load_vortons(VECTOR<Vorton>& v, const float* pos, const float* angvel, const float* size, size_t n) {
  v.Clear();
  v.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Vorton w;
    w.mPosition = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    w.mAngularVelocity = Vec3(angvel[3 * i], angvel[3 * i + 1], angvel[3 * i + 2]);
    w.mSize = size[i];
    v.PushBack(w);
  }
}

void grid_to_floats(const UniformGrid<Vec3>& g, float* out) {
  const size_t n = g.GetGridCapacity();
  for (size_t i = 0; i < n; ++i) {
    out[3 * i] = g[i].x;
    out[3 * i + 1] = g[i].y;
    out[3 * i + 2] = g[i].z;
  }
}

void floats_to_grid(UniformGrid<Vec3>& g, const float* in) {
  const size_t n = g.GetGridCapacity();
  for (size_t i = 0; i < n; ++i) g[i] = Vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
}

/* A VortonSim whose grid template is set directly (geom) instead of derived
 * from the bounding box, so each stage can be exercised on a given grid. */
struct Sim {
  VECTOR<Vorton> vortons;
  VortonSim sim;
  Sim(const float* pos, const float* angvel, const float* size, size_t n, const float* geom12, const unsigned* np,
      float viscosity)
      : sim(viscosity, 1.0f) {
    load_vortons(vortons, pos, angvel, size, n);
    sim.SetVortons(&vortons);
    sim.SetFluidSimulationTechnique(VortonSim::FLUID_SIM_VORTEX_PARTICLE_METHOD);
    load_geom(sim.mGridTemplate, geom12, np);
  }
};

/* Run body over [0, m): TBB-parallel in the USE_TBB build, else serial. */
template <class Body>
void run_range(size_t m, const Body& body) {
#if USE_TBB
  tbb::parallel_for(tbb::blocked_range<size_t>(0, m, Max2(size_t(1), m / gNumberOfProcessors)), body);
#else
  body(tbb::blocked_range<size_t>(0, m));
#endif
}

}  // namespace

extern "C" {

int vgref_uses_tbb(void) { return USE_TBB; }
size_t vgref_sizeof_particle(void) { return sizeof(Particle); }

void vgref_set_threads(unsigned n) { gNumberOfProcessors = n ? n : 1; }

/* UniformGridGeometry::DefineShape (uniformGrid.h:259-322). */
void vgref_define_shape(size_t n, const float vmin[3], const float vmax[3], int pow2, float geom12[12], unsigned np[3]) {
  UniformGridGeometry g;
  g.DefineShape(n, Vec3(vmin[0], vmin[1], vmin[2]), Vec3(vmax[0], vmax[1], vmax[2]), pow2 != 0);
  store_geom(g, geom12, np);
}

/* UniformGridGeometry::IndicesOfPosition / OffsetOfPosition (uniformGrid.h:536-574, 645-651). */
void vgref_indices_of_position(const float geom12[12], const unsigned np[3], const float* pos, size_t n,
                               unsigned* idx3, unsigned* offset) {
  UniformGridGeometry g;
  load_geom(g, geom12, np);
  for (size_t i = 0; i < n; ++i) {
    unsigned ind[4];
    const Vec3 p(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    g.IndicesOfPosition(ind, p);
    idx3[3 * i] = ind[0];
    idx3[3 * i + 1] = ind[1];
    idx3[3 * i + 2] = ind[2];
    offset[i] = g.OffsetOfPosition(p);
  }
}

/* NestedGrid::Initialize shape (nestedGrid.h:69-85, 312-391): returns depth. */
int vgref_nested_grid_shape(const float geom12[12], const unsigned np[3], unsigned* layer_np, unsigned* decim, int max_layers) {
  UniformGridGeometry g;
  load_geom(g, geom12, np);
  NestedGrid<Vec3> ng(g);
  const int depth = (int)ng.GetDepth();
  for (int l = 0; l < depth && l < max_layers; ++l) {
    layer_np[3 * l] = ng[l].GetNumPoints(0);
    layer_np[3 * l + 1] = ng[l].GetNumPoints(1);
    layer_np[3 * l + 2] = ng[l].GetNumPoints(2);
    if (l > 0) {
      const unsigned* d = ng.GetDecimations(l);
      decim[3 * l] = d[0];
      decim[3 * l + 1] = d[1];
      decim[3 * l + 2] = d[2];
    } else {
      decim[0] = decim[1] = decim[2] = 0;
    }
  }
  return depth;
}

/* CreateInfluenceTree (vortonSim.cpp:1605-1624): every layer's supervortons as
 * 7 floats per point (pos xyz, angvel xyz, size), layers concatenated leaf first.
 * Returns the number of points written (or needed, if cap is too small). */
size_t vgref_influence_tree(const float* pos, const float* angvel, const float* size, size_t n, const float geom12[12],
                            const unsigned np[3], float* out7, size_t cap_points) {
  Sim s(pos, angvel, size, n, geom12, np, 0.0f);
  NestedGrid<Vorton> tree;
  s.sim.CreateInfluenceTree(tree);
  size_t total = 0;
  for (size_t l = 0; l < tree.GetDepth(); ++l) total += tree[l].GetGridCapacity();
  if (total > cap_points) return total;
  size_t k = 0;
  for (size_t l = 0; l < tree.GetDepth(); ++l) {
    for (size_t i = 0; i < tree[l].GetGridCapacity(); ++i, ++k) {
      const Vorton& v = tree[l][i];
      float* o = out7 + 7 * k;
      o[0] = v.mPosition.x; o[1] = v.mPosition.y; o[2] = v.mPosition.z;
      o[3] = v.mAngularVelocity.x; o[4] = v.mAngularVelocity.y; o[5] = v.mAngularVelocity.z;
      o[6] = v.mSize;
    }
  }
  return total;
}

/* ComputeVelocity_Direct / ComputeVectorPotential_Direct (vortonSim.cpp:1113-1158)
 * at arbitrary query points; kind 0 = velocity, 1 = vector potential. */
void vgref_direct(int kind, const float* pos, const float* angvel, const float* size, size_t n, const float* q, size_t m,
                  float spread_range, float spread_circ, float* out) {
  VECTOR<Vorton> v;
  load_vortons(v, pos, angvel, size, n);
  VortonSim sim(0.0f, 1.0f);
  sim.SetVortons(&v);
  sim.mSpreadingRangeFactor = spread_range;
  sim.mSpreadingCirculationFactor = spread_circ;
  struct Body {
    VortonSim* sim; int kind; const float* q; float* out;
    void operator()(const tbb::blocked_range<size_t>& r) const {
      for (size_t i = r.begin(); i < r.end(); ++i) {
        const Vec3 p(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
        const Vec3 u = kind == 0 ? sim->ComputeVelocity_Direct(p) : sim->ComputeVectorPotential_Direct(p);
        out[3 * i] = u.x; out[3 * i + 1] = u.y; out[3 * i + 2] = u.z;
      }
    }
  } body = {&sim, kind, q, out};
  run_range(m, body);
}

/* ComputeVelocity_Tree / ComputeVectorPotential_Tree (vortonSim.cpp:1650-1905)
 * from the root, as ComputeVelocityAtGridpoints_Slice calls them
 * (vortonSim.cpp:2264-2267), at arbitrary query points. */
void vgref_tree(int kind, const float* pos, const float* angvel, const float* size, size_t n, const float geom12[12],
                const unsigned np[3], const float* q, size_t m, float spread_range, float spread_circ, float* out) {
  Sim s(pos, angvel, size, n, geom12, np, 0.0f);
  NestedGrid<Vorton> tree;
  s.sim.CreateInfluenceTree(tree);
  s.sim.mSpreadingRangeFactor = spread_range;
  s.sim.mSpreadingCirculationFactor = spread_circ;
  UniformGrid<VECTOR<unsigned> > dummy;
  struct Body {
    VortonSim* sim; NestedGrid<Vorton>* tree; UniformGrid<VECTOR<unsigned> >* idx; int kind; const float* q; float* out;
    void operator()(const tbb::blocked_range<size_t>& r) const {
      static const unsigned zeros[3] = {0, 0, 0};
      const size_t numLayers = tree->GetDepth();
      for (size_t i = r.begin(); i < r.end(); ++i) {
        const Vec3 p(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
        Vec3 u;
        if (numLayers > 1)
          u = kind == 0 ? sim->ComputeVelocity_Tree(p, zeros, numLayers - 1, *idx, *tree)
                        : sim->ComputeVectorPotential_Tree(p, zeros, numLayers - 1, *idx, *tree);
        else
          u = kind == 0 ? sim->ComputeVelocity_Direct(p) : sim->ComputeVectorPotential_Direct(p);
        out[3 * i] = u.x; out[3 * i + 1] = u.y; out[3 * i + 2] = u.z;
      }
    }
  } body = {&s.sim, &tree, &dummy, kind, q, out};
  run_range(m, body);
}

/* PopulateVorticityGridFromVortons(grid, scale) (vortonSim.cpp:2372-2436). */
void vgref_splat(const float* pos, const float* angvel, const float* size, size_t n, const float geom12[12],
                 const unsigned np[3], float scale, float* grid_out) {
  Sim s(pos, angvel, size, n, geom12, np, 0.0f);
  UniformGrid<Vec3> g;
  s.sim.PopulateVorticityGridFromVortons(g, scale);
  grid_to_floats(g, grid_out);
}

/* ComputeVectorPotentialFromVorticity_Integral(boundariesOnly) on a zeroed grid
 * (vortonSim.cpp:2055-2138, 2154-2204). */
void vgref_boundary_vecpot(const float* pos, const float* angvel, const float* size, size_t n, const float geom12[12],
                           const unsigned np[3], int boundaries_only, float* grid_out) {
  Sim s(pos, angvel, size, n, geom12, np, 0.0f);
  NestedGrid<Vorton> tree;
  s.sim.CreateInfluenceTree(tree);
  s.sim.mVelGrid.CopyShape(s.sim.mGridTemplate);
  s.sim.mVelGrid.Init();
  s.sim.mVectorPotentialMultiGrid.Initialize(s.sim.mGridTemplate);
  s.sim.mVectorPotentialMultiGrid[0].Init(Vec3(0.0f, 0.0f, 0.0f));
  UniformGrid<VECTOR<unsigned> > dummy;
  s.sim.ComputeVectorPotentialFromVorticity_Integral(boundaries_only != 0, dummy, tree);
  grid_to_floats(s.sim.mVectorPotentialMultiGrid[0], grid_out);
}

/* SolveVectorPoisson(soln, lap, steps, Dirichlet) (uniformGridMath.cpp:1369-1405). */
void vgref_sor(const float geom12[12], const unsigned np[3], float* soln_inout, const float* lap, int steps) {
  UniformGrid<Vec3> soln, rhs;
  load_geom(soln, geom12, np);
  load_geom(rhs, geom12, np);
  soln.Init();
  rhs.Init();
  floats_to_grid(soln, soln_inout);
  floats_to_grid(rhs, lap);
  Stats_Float stats;
  SolveVectorPoisson(soln, rhs, (size_t)steps, BC_DIRICHLET, stats);
  grid_to_floats(soln, soln_inout);
}

/* DownSampleInto(1, mode) then UpSampleFrom(1, region) on a 2-layer NestedGrid
 * (nestedGrid.h:253-293, uniformGrid.h:1453-1700).  fine_in: the fine layer;
 * coarse_out: the restricted coarse layer; fine_out: fine layer after
 * up-sampling coarse_out back into it (region 0 entire, 1 interior only). */
void vgref_down_up(const float geom12[12], const unsigned np[3], const float* fine_in, int accuracy, int region,
                   float* coarse_out, unsigned coarse_np[3], float* fine_out) {
  UniformGridGeometry g;
  load_geom(g, geom12, np);
  NestedGrid<Vec3> ng(g);
  ng[0].Init();
  floats_to_grid(ng[0], fine_in);
  ng[1].Init();
  ng.DownSampleInto(1, accuracy ? UniformGridGeometry::FASTER_LESS_ACCURATE : UniformGridGeometry::SLOWER_MORE_ACCURATE);
  grid_to_floats(ng[1], coarse_out);
  coarse_np[0] = ng[1].GetNumPoints(0);
  coarse_np[1] = ng[1].GetNumPoints(1);
  coarse_np[2] = ng[1].GetNumPoints(2);
  ng.UpSampleFrom(1, region ? UniformGridGeometry::INTERIOR_ONLY : UniformGridGeometry::ENTIRE_DOMAIN);
  grid_to_floats(ng[0], fine_out);
}

/* The multigrid cascade of VortonSim::ComputeVectorPotential
 * (vortonSim.cpp:2539-2571): soln_inout holds the boundary values (interior
 * zero) on entry and the cascade's result on exit; rhs is -vorticity. */
void vgref_cascade(const float geom12[12], const unsigned np[3], float* soln_inout, const float* rhs, int steps) {
  UniformGridGeometry g;
  load_geom(g, geom12, np);
  NestedGrid<Vec3> a(g), b(g);
  for (size_t l = 0; l < a.GetDepth(); ++l) { a[l].Init(); b[l].Init(); }
  floats_to_grid(a[0], soln_inout);
  floats_to_grid(b[0], rhs);
  Stats_Float stats;
  const size_t numSolverSteps = (size_t)steps;
  SolveVectorPoisson(a[0], b[0], numSolverSteps, BC_DIRICHLET, stats);
  unsigned maxValidDepth = 0;
  for (unsigned iLayer = 1; iLayer < b.GetDepth(); ++iLayer) {
    const unsigned minDim = MIN3(b[iLayer].GetNumPoints(0), b[iLayer].GetNumPoints(1), b[iLayer].GetNumPoints(2));
    if (minDim > 2) {
      b.DownSampleInto(iLayer, UniformGridGeometry::FASTER_LESS_ACCURATE);
      a.DownSampleInto(iLayer, UniformGridGeometry::FASTER_LESS_ACCURATE);
      SolveVectorPoisson(a[iLayer], b[iLayer], numSolverSteps, BC_DIRICHLET, stats);
    } else {
      maxValidDepth = iLayer - 1;
      break;
    }
  }
  for (unsigned iLayer = maxValidDepth; iLayer >= 1; --iLayer) {
    a.UpSampleFrom(iLayer, UniformGridGeometry::INTERIOR_ONLY);
    SolveVectorPoisson(a[iLayer - 1], b[iLayer - 1], numSolverSteps, BC_DIRICHLET, stats);
  }
  grid_to_floats(a[0], soln_inout);
}

/* ComputeJacobian + ComputeCurlFromJacobian (uniformGridMath.cpp:207-451). */
void vgref_jacobian_curl(const float geom12[12], const unsigned np[3], const float* vec, float* jac9_out, float* curl_out) {
  UniformGrid<Vec3> v, c;
  UniformGrid<Mat33> j;
  load_geom(v, geom12, np);
  load_geom(c, geom12, np);
  load_geom(j, geom12, np);
  v.Init(); c.Init(); j.Init();
  floats_to_grid(v, vec);
  ComputeJacobian(j, v);
  ComputeCurlFromJacobian(c, j);
  const size_t n = j.GetGridCapacity();
  for (size_t i = 0; i < n; ++i) {
    const Mat33& m = j[i];
    float* o = jac9_out + 9 * i;
    o[0] = m.x.x; o[1] = m.x.y; o[2] = m.x.z;
    o[3] = m.y.x; o[4] = m.y.y; o[5] = m.y.z;
    o[6] = m.z.x; o[7] = m.z.y; o[8] = m.z.z;
  }
  grid_to_floats(c, curl_out);
}

/* StretchAndTiltVortons (vortonSim.cpp:2748-2820) with mVelGrid = velgrid. */
void vgref_stretch(float* pos, float* angvel_inout, const float* size, size_t n, const float geom12[12], const unsigned np[3],
                   const float* velgrid, float dt) {
  Sim s(pos, angvel_inout, size, n, geom12, np, 0.0f);
  s.sim.mVelGrid.CopyShape(s.sim.mGridTemplate);
  s.sim.mVelGrid.Init();
  floats_to_grid(s.sim.mVelGrid, velgrid);
  s.sim.StretchAndTiltVortons(dt, 0);
  for (size_t i = 0; i < n; ++i) {
    angvel_inout[3 * i] = s.vortons[i].mAngularVelocity.x;
    angvel_inout[3 * i + 1] = s.vortons[i].mAngularVelocity.y;
    angvel_inout[3 * i + 2] = s.vortons[i].mAngularVelocity.z;
  }
}

/* PartitionVortons + DiffuseAndDissipateVorticityPSE (vortonSim.cpp:3578-3879). */
void vgref_pse(const float* pos, float* angvel_inout, const float* size, size_t n, const float geom12[12], const unsigned np[3],
               float viscosity, float dt) {
  Sim s(pos, angvel_inout, size, n, geom12, np, viscosity);
  s.sim.PartitionVortons(dt, 0, s.sim.mVortonIndicesGrid);
  s.sim.DiffuseAndDissipateVorticityPSE(dt, 0, s.sim.mVortonIndicesGrid);
  for (size_t i = 0; i < n; ++i) {
    angvel_inout[3 * i] = s.vortons[i].mAngularVelocity.x;
    angvel_inout[3 * i + 1] = s.vortons[i].mAngularVelocity.y;
    angvel_inout[3 * i + 2] = s.vortons[i].mAngularVelocity.z;
  }
}

/* AssignVelocityFromField(gain 1) then Evolve (pclOpAdvect.cpp:42-152,
 * pclOpEvolve.cpp:36-58) on particles given by position; vel_out receives the
 * gathered velocity, pos_inout the advected position. */
void vgref_advect(float* pos_inout, float* vel_out, size_t n, const float geom12[12], const unsigned np[3],
                  const float* velgrid, float dt) {
  UniformGrid<Vec3> g;
  load_geom(g, geom12, np);
  g.Init();
  floats_to_grid(g, velgrid);
  VECTOR<Particle> p;
  p.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Particle q;
    q.mPosition = Vec3(pos_inout[3 * i], pos_inout[3 * i + 1], pos_inout[3 * i + 2]);
    p.PushBack(q);
  }
  AssignVelocityFromField(p, &g, 1.0f);
  for (size_t i = 0; i < n; ++i) {
    vel_out[3 * i] = p[i].mVelocity.x; vel_out[3 * i + 1] = p[i].mVelocity.y; vel_out[3 * i + 2] = p[i].mVelocity.z;
    Particle& pc = p[i];
    pc.mPosition += pc.mVelocity * dt;  /* EvolveParticlesSlice body (pclOpEvolve.cpp:51) */
    pos_inout[3 * i] = pc.mPosition.x; pos_inout[3 * i + 1] = pc.mPosition.y; pos_inout[3 * i + 2] = pc.mPosition.z;
  }
}

/* Find the AABB the way PclOpFindBoundingBox does (pclOpFindBoundingBox.cpp:102-140). */
void vgref_find_bbox(const float* pos, size_t n, float mn[3], float mx[3]) {
  VECTOR<Particle> p;
  p.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Particle q;
    q.mPosition = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    p.PushBack(q);
  }
  Vec3 a(FLT_MAX, FLT_MAX, FLT_MAX), b(-FLT_MAX, -FLT_MAX, -FLT_MAX);
  PclOpFindBoundingBox::FindBoundingBox(p, a, b);
  mn[0] = a.x; mn[1] = a.y; mn[2] = a.z;
  mx[0] = b.x; mx[1] = b.y; mx[2] = b.z;
}

/* One PclOpVortonSim::Operate (pclOpVortonSim.cpp:51-71) on Particle records
 * (sizeof(Particle) stride), with an optional extra box (the tracers' AABB).
 * The reference's grids outlive the call in a static op so that
 * vgref_last_grids can read them. */
static PclOpVortonSim* g_op = 0;

int vgref_step(void* particles, size_t n, const float* extra_min, const float* extra_max, float dt, unsigned frame,
               float viscosity, float geom12_out[12], unsigned np_out[3]) {
  if (!g_op) g_op = new PclOpVortonSim;
  g_op->mVortonSim.mViscosity = viscosity;
  g_op->mVortonSim.SetFluidSimulationTechnique(VortonSim::FLUID_SIM_VORTEX_PARTICLE_METHOD);
  VECTOR<Particle> v;
  v.Reserve(n);
  const Particle* src = static_cast<const Particle*>(particles);
  for (size_t i = 0; i < n; ++i) v.PushBack(src[i]);
  static Vec3 emin, emax;
  if (extra_min && extra_max) {
    emin = Vec3(extra_min[0], extra_min[1], extra_min[2]);
    emax = Vec3(extra_max[0], extra_max[1], extra_max[2]);
    g_op->mMinCorner = &emin;
    g_op->mMaxCorner = &emax;
  } else {
    g_op->mMinCorner = 0;
    g_op->mMaxCorner = 0;
  }
  g_op->Operate(v, dt, frame);
  Particle* dst = static_cast<Particle*>(particles);
  for (size_t i = 0; i < n; ++i) dst[i] = v[i];
  g_op->mVortonSim.SetVortons(0);
  store_geom(g_op->mVortonSim.mGridTemplate, geom12_out, np_out);
  return 0;
}

/* Velocity grid and finest vector-potential / negative-vorticity layers of the
 * last vgref_step (sizes from its np_out). */
void vgref_last_grids(float* vel_out, float* vecpot_out, float* negvort_out) {
  if (!g_op) return;
  if (vel_out) grid_to_floats(g_op->mVortonSim.mVelGrid, vel_out);
  if (vecpot_out) grid_to_floats(g_op->mVortonSim.mVectorPotentialMultiGrid[0], vecpot_out);
  if (negvort_out) grid_to_floats(g_op->mVortonSim.mNegativeVorticityMultiGrid[0], negvort_out);
}

// DiffuseAndDissipateHeatPSE (VortonFluid/vortonSim.cpp:3954-4093) after
// PartitionVortons, on vortons carrying density_inout in mDensity.
void vgref_heat_pse(const float* pos, float* density_inout, const float* size, size_t n, const float geom12[12],
                    const unsigned np[3], float diffusivity, float ambient, float dt) {
  std::vector<float> zero(3 * n, 0.0f);
  Sim s(pos, zero.data(), size, n, geom12, np, 0.0f);
  for (size_t i = 0; i < n; ++i) s.vortons[i].mDensity = density_inout[i];
  s.sim.mThermalDiffusivity = diffusivity;
  s.sim.mAmbientDensity = ambient;
  s.sim.PartitionVortons(dt, 0, s.sim.mVortonIndicesGrid);
  s.sim.DiffuseAndDissipateHeatPSE(dt, 0, s.sim.mVortonIndicesGrid);
  for (size_t i = 0; i < n; ++i) density_inout[i] = s.vortons[i].mDensity;
}

// PclOpKillAge::Operate (Particles/Operation/pclOpKillAge.cpp:22-47) on n
// particles with the given birth times; order_out[0..*m) receives the
// surviving particles' original indices in the order the operation leaves
// them (each particle carries its index in mDensity, exact below 2^24).
void vgref_kill_age(const int* birth, size_t n, unsigned frame, int age_max, unsigned* order_out, size_t* m) {
  VECTOR<Particle> pcl;
  pcl.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Particle p;
    p.mDensity = (float)i;
    p.mBirthTime = birth[i];
    pcl.PushBack(p);
  }
  PclOpKillAge op;
  op.mAgeMax = age_max;
  op.Operate(pcl, 0.0f, frame);
  *m = pcl.Size();
  for (size_t i = 0; i < pcl.Size(); ++i) order_out[i] = (unsigned)pcl[i].mDensity;
}

// PclOpWind::Operate (Particles/Operation/pclOpWind.cpp:18-42) on n particles'
// velocities (xyz, in place).
void vgref_wind(float* vel_inout, size_t n, const float wind[3], float wind_weight, float src_weight) {
  VECTOR<Particle> pcl;
  pcl.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Particle p;
    p.mVelocity = Vec3(vel_inout[3 * i], vel_inout[3 * i + 1], vel_inout[3 * i + 2]);
    pcl.PushBack(p);
  }
  PclOpWind op;
  op.mWind = Vec3(wind[0], wind[1], wind[2]);
  op.mWindWeight = wind_weight;
  op.mSrcWeight = src_weight;
  op.Operate(pcl, 0.0f, 0);
  for (size_t i = 0; i < n; ++i) {
    vel_inout[3 * i] = pcl[i].mVelocity.x;
    vel_inout[3 * i + 1] = pcl[i].mVelocity.y;
    vel_inout[3 * i + 2] = pcl[i].mVelocity.z;
  }
}

// PopulateDensityAndMassFractionGrids (VortonFluid/vortonSim.cpp:2911-3057):
// the density grid on the grid template from n vortons with per-vorton
// densities (mass fractions are not returned).
void vgref_density_grid(const float* pos, const float* size, const float* density, size_t n, const float geom12[12],
                        const unsigned np[3], float ambient, float* out) {
  std::vector<float> zeros(3 * n, 0.0f);
  Sim s(pos, zeros.data(), size, n, geom12, np, 0.0f);
  for (size_t i = 0; i < n; ++i) s.vortons[i].mDensity = density[i];
  s.sim.mAmbientDensity = ambient;
  UniformGrid<float> dg;
  s.sim.PopulateDensityAndMassFractionGrids(dg, reinterpret_cast<VECTOR<Particle>&>(s.vortons), 0);
  for (size_t i = 0; i < dg.GetGridCapacity(); ++i) out[i] = dg[i];
}

// ComputeGradient (Core/SpatialPartition/uniformGridMath.cpp:650-800) of a scalar grid.
void vgref_gradient(const float geom12[12], const unsigned np[3], const float* scalar, float* out3) {
  UniformGrid<float> v;
  load_geom(v, geom12, np);
  v.Init(0.0f);
  for (size_t i = 0; i < v.GetGridCapacity(); ++i) v[i] = scalar[i];
  UniformGrid<Vec3> g;
  g.CopyShape(v);
  g.Init();
  ComputeGradient(g, v);
  grid_to_floats(g, out3);
}

// Baroclinic generation on the grid-density path of
// VortonSim::GenerateBaroclinicVorticity (vortonSim.cpp:3407-3547, the branch
// without per-vorton SPH gradients): density grid, its gradient
// (ComputeGradient), the gradient interpolated at each vorton
// (UniformGrid::Interpolate), then the reference's own
// GenerateBaroclinicVorticitySlice (vortonSim.cpp:3318-3392) on those
// gradients.  Returns 0 when the grid has no extent along gravity (the
// reference's early return, vortonSim.cpp:3417-3421).
int vgref_baroclinic(const float* pos, float* angvel_inout, const float* size, const float* density, size_t n,
                     const float geom12[12], const unsigned np[3], const float grav[3], float ambient, float dt) {
  Sim s(pos, angvel_inout, size, n, geom12, np, 0.0f);
  for (size_t i = 0; i < n; ++i) s.vortons[i].mDensity = density[i];
  s.sim.mAmbientDensity = ambient;
  s.sim.mGravAccel = Vec3(grav[0], grav[1], grav[2]);
  s.sim.mVelGrid.CopyShape(s.sim.mGridTemplate);
  if (fabsf(s.sim.mGravAccel * s.sim.mVelGrid.GetExtent()) < FLT_EPSILON) return 0;
  s.sim.PopulateDensityAndMassFractionGrids(s.sim.mDensityGrid, reinterpret_cast<VECTOR<Particle>&>(s.vortons), 0);
  s.sim.mDensityGradientGrid.Clear();
  s.sim.mDensityGradientGrid.CopyShape(s.sim.mGridTemplate);
  s.sim.mDensityGradientGrid.Init();
  ComputeGradient(s.sim.mDensityGradientGrid, s.sim.mDensityGrid);
  VECTOR<Vec3> grads;
  grads.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Vec3 g;
    s.sim.mDensityGradientGrid.Interpolate(g, s.vortons[i].mPosition);
    grads.PushBack(g);
  }
  s.sim.GenerateBaroclinicVorticitySlice(dt, &grads, 0, n);
  for (size_t i = 0; i < n; ++i) {
    angvel_inout[3 * i] = s.vortons[i].mAngularVelocity.x;
    angvel_inout[3 * i + 1] = s.vortons[i].mAngularVelocity.y;
    angvel_inout[3 * i + 2] = s.vortons[i].mAngularVelocity.z;
  }
  return 1;
}

// PopulateSignedDistanceGridFromDensityGrid (vortonSim.cpp:3266-3290): the
// signed distance grid of a density grid (negative inside the heavy fluid;
// points no crossing reaches come back as NaN).
void vgref_signed_distance(const float geom12[12], const unsigned np[3], const float* density, float ambient,
                           float* out) {
  std::vector<float> zeros(3, 0.0f);
  float one = 1.0f;
  Sim s(zeros.data(), zeros.data(), &one, 1, geom12, np, 0.0f);
  s.sim.mAmbientDensity = ambient;
  s.sim.mDensityGrid.Clear();
  load_geom(s.sim.mDensityGrid, geom12, np);
  s.sim.mDensityGrid.Init(0.0f);
  for (size_t i = 0; i < s.sim.mDensityGrid.GetGridCapacity(); ++i) s.sim.mDensityGrid[i] = density[i];
  UniformGrid<float> sdf;
  s.sim.PopulateSignedDistanceGridFromDensityGrid(sdf, s.sim.mDensityGrid, 0);
  for (size_t i = 0; i < sdf.GetGridCapacity(); ++i) out[i] = sdf[i];
}

}  // extern "C"

// Rigid bodies for the fluid-body boundary conditions, 32 floats each:
// [0] shape (0 sphere, 1 box), [1] hole (box only), [2..4] position,
// [5..7] velocity, [8..10] angular velocity, [11..19] orientation rows
// (x, y, z), [20..22] sphere radius (x) or box dimensions, [23] temperature,
// [24] thermal conductivity.  The reference's own Impulsion and Collision
// objects are built from them.
namespace {
struct Bodies {
  std::vector<Impulsion::PhysicalObject*> objs;
  std::vector<Impulsion::RigidBody*> bodies;
  std::vector<Collision::ShapeBase*> shapes;
  VECTOR<Impulsion::PhysicalObject*> list;
  Bodies(const float* b, int nb) {
    for (int k = 0; k < nb; ++k) {
      const float* q = b + 32 * k;
      Impulsion::RigidBody* rb = new Impulsion::RigidBody(Vec3(q[2], q[3], q[4]), Vec3(q[5], q[6], q[7]), 1.0f);
      rb->SetOrientation(Mat33(Vec3(q[11], q[12], q[13]), Vec3(q[14], q[15], q[16]), Vec3(q[17], q[18], q[19])));
      rb->SetAngularVelocity(Vec3(q[8], q[9], q[10]));
      Collision::ShapeBase* sh;
      if (q[0] == 0.0f) {
        sh = new Collision::SphereShape(q[20]);
      } else {
        Collision::ConvexPolytope* cp = new Collision::ConvexPolytope(q[1] != 0.0f);
        Collision::ConvexPolytope_MakeBox(*cp, Vec3(q[20], q[21], q[22]));
        sh = cp;
      }
      Impulsion::PhysicalObject* po = new Impulsion::PhysicalObject(
          rb, sh, Impulsion::FrictionProperties(), Impulsion::ThermalProperties(q[23], q[24], 1.0f));
      bodies.push_back(rb);
      shapes.push_back(sh);
      objs.push_back(po);
      list.PushBack(po);
    }
  }
  ~Bodies() {
    for (auto* o : objs) delete o;
    for (auto* s : shapes) delete s;
    for (auto* r : bodies) delete r;
  }
};

void load_particles(VECTOR<Particle>& p, const float* pos, const float* vel, const float* angvel, const float* size,
                    const float* density, size_t n) {
  p.Clear();
  p.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Particle q;
    q.mPosition = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    q.mVelocity = Vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    if (angvel) q.mAngularVelocity = Vec3(angvel[3 * i], angvel[3 * i + 1], angvel[3 * i + 2]);
    q.mSize = size[i];
    q.mDensity = density ? density[i] : 1.0f;
    p.PushBack(q);
  }
}

void store_particles(const VECTOR<Particle>& p, float* pos, float* vel, float* angvel, float* density) {
  for (size_t i = 0; i < p.Size(); ++i) {
    pos[3 * i] = p[i].mPosition.x, pos[3 * i + 1] = p[i].mPosition.y, pos[3 * i + 2] = p[i].mPosition.z;
    vel[3 * i] = p[i].mVelocity.x, vel[3 * i + 1] = p[i].mVelocity.y, vel[3 * i + 2] = p[i].mVelocity.z;
    if (angvel)
      angvel[3 * i] = p[i].mAngularVelocity.x, angvel[3 * i + 1] = p[i].mAngularVelocity.y,
      angvel[3 * i + 2] = p[i].mAngularVelocity.z;
    if (density) density[i] = p[i].mDensity;
  }
}
}  // namespace

extern "C" {

// FluidBodySim::CollideVortonsSlice (FluidBodySim/fluidBodySim.cpp:759-1180)
// for each body in turn over all particles, as SolveBoundaryConditions runs
// it for vortons (fluidBodySim.cpp:1651-1715); per body out9 receives the
// linear impulse, angular impulse, heat to body, sum of particle temperatures
// and the number of particles collided.
void vgref_collide_vortons(float* pos, float* vel, float* angvel, const float* size, float* density, size_t n,
                           const float* bodies, int nb, float ambient, float specific_heat, float* out9) {
  VECTOR<Particle> p;
  load_particles(p, pos, vel, angvel, size, density, n);
  Bodies B(bodies, nb);
  for (int k = 0; k < nb; ++k) {
    Vec3 lin, ang;
    float heat = 0.0f, sumT = 0.0f;
    size_t cnt = 0;
    FluidBodySim::CollideVortonsSlice(p, ambient, specific_heat, *B.objs[k], lin, ang, heat, sumT, cnt, 0, n);
    float* o = out9 + 9 * k;
    o[0] = lin.x, o[1] = lin.y, o[2] = lin.z, o[3] = ang.x, o[4] = ang.y, o[5] = ang.z;
    o[6] = heat, o[7] = sumT, o[8] = (float)cnt;
  }
  store_particles(p, pos, vel, angvel, density);
}

// FluidBodySim::CollideTracersSlice (fluidBodySim.cpp:1300-1455) for each body
// in turn; per body out6 receives the linear and angular impulses.
void vgref_collide_tracers(float* pos, float* vel, const float* size, const float* density, size_t n,
                           const float* bodies, int nb, float* out6) {
  VECTOR<Particle> p;
  load_particles(p, pos, vel, nullptr, size, density, n);
  Bodies B(bodies, nb);
  for (int k = 0; k < nb; ++k) {
    Vec3 lin, ang;
    FluidBodySim::CollideTracersSlice(p, *B.objs[k], lin, ang, 0, n);
    float* o = out6 + 6 * k;
    o[0] = lin.x, o[1] = lin.y, o[2] = lin.z, o[3] = ang.x, o[4] = ang.y, o[5] = ang.z;
  }
  std::vector<float> dummy(n);
  store_particles(p, pos, vel, nullptr, nullptr);
}

// FluidBodySim::RemoveEmbeddedParticles (fluidBodySim.cpp:365-417): order_out
// receives the surviving particles' original indices in the order the
// operation leaves them (each particle carries its index in mDensity).
void vgref_remove_embedded(const float* pos, const float* size, size_t n, const float* bodies, int nb,
                           unsigned* order_out, size_t* m) {
  VECTOR<Particle> p;
  p.Reserve(n);
  for (size_t i = 0; i < n; ++i) {
    Particle q;
    q.mPosition = Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    q.mSize = size[i];
    q.mDensity = (float)i;
    p.PushBack(q);
  }
  Bodies B(bodies, nb);
  FluidBodySim::RemoveEmbeddedParticles(p, B.list);
  *m = p.Size();
  for (size_t i = 0; i < p.Size(); ++i) order_out[i] = (unsigned)p[i].mDensity;
}

}  // extern "C"

extern "C" {

// PclOpEmit::Emit (Particles/Operation/pclOpEmit.cpp:77-186) into an empty
// array after srand(seed), with vortons (positions, sizes, densities) when
// use_vortons is set.  Per emitted particle: position (3), density, size.
void vgref_emit_grid(const float geom12[12], const unsigned np[3], unsigned multiplier, const float* vpos,
                     const float* vsize, const float* vdens, size_t nv, int use_vortons, unsigned seed,
                     float* pos_out, float* density_out, float* size_out, size_t max, size_t* count) {
  UniformGridGeometry g;
  load_geom(g, geom12, np);
  VECTOR<Particle> vortons;
  if (use_vortons) load_particles(vortons, vpos, vpos, nullptr, vsize, vdens, nv);
  VECTOR<Particle> out;
  srand(seed);
  PclOpEmit::Emit(out, g, multiplier, use_vortons ? &vortons : nullptr);
  *count = out.Size();
  for (size_t i = 0; i < out.Size() && i < max; ++i) {
    pos_out[3 * i] = out[i].mPosition.x, pos_out[3 * i + 1] = out[i].mPosition.y,
    pos_out[3 * i + 2] = out[i].mPosition.z;
    density_out[i] = out[i].mDensity;
    size_out[i] = out[i].mSize;
  }
}

// PclOpEmit::Operate (pclOpEmit.cpp:188-210) for each of `frames` calls
// (time step dt[f], frame index frame0 + f) after one srand(seed), appending
// to one array.  Template and spread are 17 floats (position, velocity,
// orientation, angular velocity, density, fuel, flame and smoke fractions,
// size); per particle rec_out receives those 17 values and the birth time (as
// a float); remainder_out the emitter's remainder after each call.
void vgref_emit_operate(const float tmpl[17], const float spread[17], float rate, const float* dt, int frames,
                        unsigned frame0, unsigned seed, float* rec_out, size_t max, size_t* count,
                        float* remainder_out) {
  PclOpEmit op;
  Particle* P[2] = {&op.mTemplate, &op.mSpread};
  const float* V[2] = {tmpl, spread};
  for (int k = 0; k < 2; ++k) {
    const float* v = V[k];
    P[k]->mPosition = Vec3(v[0], v[1], v[2]);
    P[k]->mVelocity = Vec3(v[3], v[4], v[5]);
    P[k]->mOrientation = Vec3(v[6], v[7], v[8]);
    P[k]->mAngularVelocity = Vec3(v[9], v[10], v[11]);
    P[k]->mDensity = v[12];
    P[k]->mFuelFraction = v[13];
    P[k]->mFlameFraction = v[14];
    P[k]->mSmokeFraction = v[15];
    P[k]->mSize = v[16];
  }
  op.mEmitRate = rate;
  VECTOR<Particle> out;
  srand(seed);
  for (int f = 0; f < frames; ++f) {
    op.Operate(out, dt[f], frame0 + (unsigned)f);
    remainder_out[f] = op.mRemainder;
  }
  *count = out.Size();
  for (size_t i = 0; i < out.Size() && i < max; ++i) {
    const Particle& q = out[i];
    const float r[18] = {q.mPosition.x, q.mPosition.y, q.mPosition.z, q.mVelocity.x, q.mVelocity.y, q.mVelocity.z,
                         q.mOrientation.x, q.mOrientation.y, q.mOrientation.z, q.mAngularVelocity.x,
                         q.mAngularVelocity.y, q.mAngularVelocity.z, q.mDensity, q.mFuelFraction,
                         q.mFlameFraction, q.mSmokeFraction, q.mSize, (float)q.mBirthTime};
    std::memcpy(rec_out + 18 * i, r, sizeof(r));
  }
}

}  // extern "C"
