/* CPU oracle for the VortonSim velocity-from-vorticity step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load this library, and only as the checker
 * (or the timed CPU baseline).  The product library never links it.
 *
 * Plain C restatement of the reference's algorithms (mijagourlay/VorteGrid,
 * Samples/MjgIntelFluidDemo_Part20); every function cites the reference
 * file:line it follows.  Float arithmetic follows the reference's operation
 * order with no fused multiply-adds (compiled with -ffp-contract=off), so
 * the float results are bit-identical to the reference built the same way.
 * The *_f64 functions are the strict FP64 oracle (exact 1/sqrt, FP64 sums).
 *
 * Parity is pinned: tests/test_oracle_golden.py checks these functions
 * against golden vectors produced by the reference's own code
 * (tests/golden/make_golden.py).
 */
#ifndef VG_ORACLE_H
#define VG_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* UniformGridGeometry (Core/SpatialPartition/uniformGrid.h:144-860). */
typedef struct {
  float mn[3];    /* minimal corner */
  float ext[3];   /* extent */
  float cell[3];  /* cell spacing */
  float cpe[3];   /* cells per extent */
  unsigned np[3]; /* points per axis (= cells + 1) */
} vgo_geom;

#define VGO_MAX_LAYERS 32

float vgo_finvsqrtf(float v);
void vgo_precompute_spacing(vgo_geom* g);
void vgo_define_shape(size_t n, const float vmin[3], const float vmax[3], int pow2, vgo_geom* g);
void vgo_decimate(const vgo_geom* src, unsigned dec, vgo_geom* dst);
void vgo_indices_of_position(const vgo_geom* g, const float p[3], unsigned idx[3]);
unsigned vgo_offset_of_position(const vgo_geom* g, const float p[3]);
void vgo_indices_batch(const vgo_geom* g, const float* pos, size_t n, unsigned* idx3, unsigned* offset);
/* Pair laws the treecode walk evaluates over m queries (its interaction count). */
size_t vgo_tree_interactions(const vgo_geom* g, const float* q, size_t m);
/* PartitionParticles cell lists: items[start[c]..start[c+1]) per point c; start has points+2 entries. */
void vgo_partition(const vgo_geom* g, const float* pos, size_t n, unsigned* start, unsigned* items);
int vgo_nested_shape(const vgo_geom* g, vgo_geom* layers, unsigned* decim3);
void vgo_bbox(const float* pos, size_t n, float mn[3], float mx[3]);
void vgo_step_geometry(const float* pos, size_t n, float radius, const float* extra_min, const float* extra_max,
                       vgo_geom* g);

/* Direct sums (vortonSim.cpp:1113-1158, vorton.h:118-179).  kind 0 velocity,
 * 1 vector potential.  Vortons: pos[3n], angvel[3n] (= vorticity/2),
 * size[n] (= diameter). */
void vgo_direct(int kind, const float* pos, const float* angvel, const float* size, size_t n, const float* q,
                size_t m, float spread_range, float spread_circ, float* out);
void vgo_direct_f64(int kind, const float* pos, const float* angvel, const float* size, size_t n, const float* q,
                    size_t m, float spread_range, float spread_circ, double* out);

/* Influence tree (vortonSim.cpp:1192-1624): writes 7 floats per point per
 * layer (pos, angvel, size), leaf layer first; returns the number of points
 * (call with out7 = NULL to size the buffer). */
size_t vgo_influence_tree(const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g,
                          float* out7);
/* Treecode at arbitrary points (vortonSim.cpp:1650-1905, 2264-2267). */
void vgo_tree(int kind, const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g,
              const float* q, size_t m, float spread_range, float spread_circ, float* out);

/* Grid fields are float[3 * points], x fastest. */
void vgo_splat(const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g, float scale,
               float* grid);
void vgo_boundary_vecpot(const float* pos, const float* angvel, const float* size, size_t n, const vgo_geom* g,
                         int boundaries_only, int copy_odd_x, float* grid);
void vgo_sor(const vgo_geom* g, float* soln, const float* lap, int steps);
void vgo_downsample(const vgo_geom* fine, const float* fine_v, int inject, const vgo_geom* coarse, float* coarse_v);
void vgo_upsample(const vgo_geom* coarse, const float* coarse_v, const vgo_geom* fine, int interior_only,
                  float* fine_v);
void vgo_cascade(const vgo_geom* g, float* soln, const float* rhs, int steps);
void vgo_jacobian(const vgo_geom* g, const float* vec, float* jac9);
void vgo_curl_from_jacobian(size_t points, const float* jac9, float* curl);
void vgo_interpolate3(const vgo_geom* g, const float* field, const float p[3], float out[3]);
void vgo_stretch(const float* pos, float* angvel, size_t n, const vgo_geom* g, const float* jac9, float dt);
void vgo_pse_sequential(const float* pos, float* angvel, const float* size, size_t n, const vgo_geom* g,
                        float viscosity, float dt);
void vgo_pse_symmetric(const float* pos, float* angvel, const float* size, size_t n, const vgo_geom* g,
                       float viscosity, float dt);
void vgo_gather(const vgo_geom* g, const float* velgrid, const float* pos, size_t n, float* vel);
void vgo_evolve(float* pos, const float* vel, size_t n, float dt);

/* DiffuseAndDissipateHeatPSE (VortonFluid/vortonSim.cpp:3880-4093): density
 * exchange between vortons of one cell and of the +x, +y, +z face-neighbour
 * cells, ratio clamp(2 kappa dt exp(-d^2 / (4 size_here)^2), +-0.5), then each
 * vorton of a "here" cell relaxes toward the ambient density by clamp(kappa dt,
 * +-0.5).  Sequential: the reference's in-place order.  Symmetric: every pair
 * exchanges with the values from before the step (the GPU form). */
void vgo_heat_pse_sequential(const float* pos, float* density, const float* size, size_t n, const vgo_geom* g,
                             float diffusivity, float ambient, float dt);
void vgo_heat_pse_symmetric(const float* pos, float* density, const float* size, size_t n, const vgo_geom* g,
                            float diffusivity, float ambient, float dt);
/* PclOpKillAge::Operate (Particles/Operation/pclOpKillAge.cpp:22-47): a particle
 * is removed when int(frame - birth) > age_max, by moving the last particle into
 * its slot (Particles::Kill, Particles/particle.h:490-495) and re-testing the
 * slot.  order[0..*m) receives the survivors' original indices in final order. */
void vgo_kill_age(const int* birth, size_t n, unsigned frame, int age_max, unsigned* order, size_t* m);
/* PclOpWind::Operate (Particles/Operation/pclOpWind.cpp:18-42): vel = (ww wind)
 * + sw vel per component; nothing when ww == 0 and sw == 1. */
void vgo_wind(float* vel, size_t n, const float wind[3], float wind_weight, float src_weight);

/* FP64 relative residual ||b - L a|| / ||b|| over interior points, Dirichlet. */
double vgo_relres_f64(const vgo_geom* g, const float* a, const float* b);
double vgo_relres_f64d(const vgo_geom* g, const double* a, const float* b);

/* One full VortonSim step in the reference's semantics (treecode boundary,
 * cascade, curl, stretch, PSE, gather) on given geometry; returns velocity
 * grid and updates vorton velocity and angvel.  pse_mode: 0 sequential
 * (reference order), 1 symmetric. */
void vgo_step_fields(const float* pos, float* vel, float* angvel, const float* size, size_t n, const vgo_geom* g,
                     float dt, float viscosity, int pse_mode, float* velgrid, float* vecpot, float* negvort);

/* Density grid, gradient, baroclinic generation and signed distance (grid path). */
void vgo_density_grid(const float* pos, const float* size, const float* density, size_t n, const vgo_geom* g,
                      float ambient, float* out);
void vgo_gradient(const vgo_geom* g, const float* v, float* grad3);
int vgo_baroclinic(const float* pos, float* angvel, const float* size, const float* density, size_t n,
                   const vgo_geom* g, const float grav[3], float ambient, float dt);
void vgo_signed_distance(const vgo_geom* g, const float* density, float ambient, int sumstats, float* sdf);
/* Marching cubes: up to cap triangles (9 floats of positions, 9 of normals each); returns the count. */
size_t vgo_marching_cubes(const vgo_geom* g, const float* v, float iso, float* verts, float* normals, size_t cap);
void vgo_marching_cubes_table(int* count, int* tri15);
/* Fluid-body boundary conditions (bodies: 32 floats each, see vg_oracle.c). */
void vgo_collide_vortons(float* pos, float* vel, float* angvel, const float* size, float* density, size_t n,
                         const float* bodies, int nb, float ambient, float specific_heat, float* out9);
void vgo_collide_tracers(float* pos, float* vel, const float* size, const float* density, size_t n,
                         const float* bodies, int nb, float* out6);
void vgo_remove_embedded(const float* pos, const float* size, size_t n, const float* bodies, int nb, unsigned* order,
                         size_t* m);

/* Emitters (PclOpEmit).  host_rand: draw from the C library's rand() (the
 * reference's source), else from vgo_jitter_hash(seed, draw index). */
int vgo_jitter_hash(unsigned seed, uint64_t d);
int vgo_rand_max(void);
void vgo_emit_grid(const vgo_geom* g, unsigned m, const float* vpos, const float* vdens, size_t nv, int use_vortons,
                   int host_rand, unsigned seed, float* pos_out, float* dens_out, float* size_out, size_t max,
                   size_t* count);
size_t vgo_emit_operate(const float tmpl[17], const float spread[17], float rate, float* remainder, float dt,
                        unsigned frame, int host_rand, unsigned seed, uint64_t* draw, float* rec, size_t max);

#ifdef __cplusplus
}
#endif

#endif
