/* vortegrid.h -- C ABI of the GB300 (sm_103a) VortonSim velocity-from-vorticity step.
 *
 * This library is a drop-in for the reference's VortonSim step behind its
 * particle-operation plugin API (mijagourlay/VorteGrid,
 * Samples/MjgIntelFluidDemo_Part20).  Every entry point below names the
 * reference interface it replaces (file:line, paths relative to that sample).
 *
 * Conventions
 *  - Vortons and tracers cross the host boundary as the reference's own
 *    Particle records (Particles/particle.h:425-431): position float[3] at
 *    byte 0, velocity float[3] at 12, angular velocity (= vorticity / 2)
 *    float[3] at 36, size (= diameter) float at 52.  The record stride is a
 *    parameter (96 bytes for the reference's LP64 build).
 *  - *_device entry points take device pointers (CUDA global memory of the
 *    context's device) and run on the context's stream without
 *    synchronising; all others take host pointers and return after the
 *    results are in host memory.
 *  - Grid fields are float[3] per point, x fastest, num_points[0] *
 *    num_points[1] * num_points[2] points; points = cells + 1 per axis.
 *  - Every call returns a vg_status; nothing traps or asserts on the device.
 *    Errors found by device stages (a sample outside the grid, a non-finite
 *    position) set a device flag that the next synchronising call reports.
 *    vg_last_error() gives a one-line explanation of the last failure.
 *  - A context is used by one host thread at a time (the reference's
 *    VortonSim is not re-entrant either, vortonSim.cpp:2668-2670).
 */
#ifndef VORTEGRID_H
#define VORTEGRID_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VG_ABI_VERSION 2

typedef enum vg_status {
  VG_OK = 0,
  VG_EMPTY = 1,         /* no vortons: nothing computed (vortonSim.cpp:4123) */
  VG_OUT_OF_GRID = 2,   /* a query lies outside the grid it samples */
  VG_NONFINITE = 3,     /* NaN or Inf in inputs or results */
  VG_OOM = 4,           /* device allocation failed */
  VG_TIMEOUT = 5,       /* a bounded device wait gave up */
  VG_INVALID = 6,       /* bad argument */
  VG_CUDA_ERROR = 7,    /* CUDA runtime error (see vg_last_error) */
  VG_NOT_CONVERGED = 8, /* Poisson solve hit its cycle limit above tolerance */
  VG_TOO_LARGE = 9      /* a size exceeds a fixed capacity of this entry point */
} vg_status;

/* Velocity-from-vorticity techniques (VortonFluid/vorton.h:39-47). */
typedef enum vg_velocity_technique {
  VG_VELOCITY_POISSON = 0, /* treecode boundary A + Poisson solve + curl (the shipped default) */
  VG_VELOCITY_TREE = 1,    /* treecode at gridpoints */
  VG_VELOCITY_DIRECT = 2   /* direct O(N^2) sum at gridpoints */
} vg_velocity_technique;

/* Arithmetic of the vorton kernels and grid stages. */
typedef enum vg_numerics {
  VG_NUMERICS_FAST = 0,     /* hardware rsqrt, fused multiply-add, reassociated sums */
  VG_NUMERICS_REFERENCE = 1 /* the reference's operation order and magic-constant rsqrt
                               (Core/Math/math.h:206-216): bit-identical FP32 results */
} vg_numerics;

typedef enum vg_poisson_solver {
  VG_POISSON_MULTIGRID = 0,        /* FP32 V-cycles in iterative refinement (FP64-class residual), to a tolerance */
  VG_POISSON_REFERENCE_CASCADE = 1 /* the reference's fixed-work cascade (vortonSim.cpp:2539-2571) */
} vg_poisson_solver;

typedef enum vg_warm_start {
  VG_WARM_ZERO = 0,     /* interior starts at zero (the reference's choice, vortonSim.cpp:2532) */
  VG_WARM_PREVIOUS = 1, /* previous step's solution, when the grid shape is unchanged */
  VG_WARM_NETWORK = 2   /* the learned 3D U-Net guess (vg_set_network) */
} vg_warm_start;

/* UniformGridGeometry (Core/SpatialPartition/uniformGrid.h:144-860). */
typedef struct vg_grid_geom {
  float min_corner[3];
  float extent[3];
  float cell_spacing[3];
  float cells_per_extent[3];
  unsigned num_points[3];
} vg_grid_geom;

typedef struct vg_config {
  unsigned abi_version;      /* VG_ABI_VERSION */
  int device;                /* CUDA device ordinal */
  void* stream;              /* cudaStream_t to run on; NULL = the context creates one */
  int velocity_technique;    /* vg_velocity_technique */
  int numerics;              /* vg_numerics */
  int poisson_solver;        /* vg_poisson_solver */
  int warm_start;            /* vg_warm_start */
  float viscosity;           /* VortonSim(viscosity) (vortonSim.cpp:373) */
  double poisson_tolerance;  /* relative residual ||b - L a|| / ||b|| target (multigrid) */
  int poisson_max_cycles;    /* cap on V-cycles (multigrid) */
  int cascade_steps;         /* SOR sweeps per level (cascade), reference 16 (vortonSim.cpp:2541) */
  int enable_stretch;        /* StretchAndTiltVortons (vortonSim.cpp:4209-4216) */
  int enable_diffusion;      /* DiffuseAndDissipateVorticityPSE (vortonSim.cpp:4238-4241) */
  int boundary_copy_odd_x;   /* reuse even-x boundary values on odd x (vortonSim.cpp:2110-2129) */
  int use_fixed_grid;        /* 1: use fixed_grid instead of the bounding-box rule */
  vg_grid_geom fixed_grid;
} vg_config;

/* Per-step statistics (the reference's Poisson stats, vortonSim.h:318-319, as
 * true residuals). */
typedef struct vg_step_stats {
  vg_grid_geom grid;
  int tree_depth;
  int poisson_cycles;
  double poisson_relres;     /* relative residual after the solve (FP64-class residual, FP64 norm) */
  double poisson_relres0;    /* before the first cycle (warm start quality) */
  float ms_total;            /* device time of the last step (CUDA events) */
  float ms_poisson;          /* device time of the Poisson solve */
  unsigned kernels_launched; /* this library's kernels in the last step */
  int warm_start_used;       /* vg_warm_start the last Poisson solve started from */
} vg_step_stats;

typedef struct vg_ctx vg_ctx;

const char* vg_status_string(vg_status s);
const char* vg_last_error(const vg_ctx* ctx);
unsigned vg_abi_version(void);

/* Fill a config with the reference's shipped settings: Poisson technique,
 * FAST numerics, multigrid to 1e-6, viscosity 0.01, stretch and diffusion on. */
vg_status vg_config_default(vg_config* cfg);

/* Replaces constructing VortonSim / PclOpVortonSim (vortonSim.cpp:373-420,
 * VortonFluid/pclOpVortonSim.h:46-71). */
vg_status vg_create(const vg_config* cfg, vg_ctx** out);
vg_status vg_destroy(vg_ctx* ctx);
vg_status vg_set_config(vg_ctx* ctx, const vg_config* cfg);

/* Replaces PclOpVortonSim::Operate (VortonFluid/pclOpVortonSim.cpp:51-71):
 * FindBoundingBox, UpdateBoundingBox(extra box or first vorton, final),
 * VortonSim::Update (vortonSim.cpp:4279-4344).  Reads positions, angular
 * velocities and sizes of n Particle records; writes back each record's
 * velocity (vortonSim.cpp:4251-4255) and angular velocity (stretch, PSE).
 * extra_min / extra_max: the tracers' box (PclOpVortonSim::mMinCorner /
 * mMaxCorner) or NULL. */
vg_status vg_step(vg_ctx* ctx, void* particles, size_t n, size_t stride, const float* extra_min,
                  const float* extra_max, float dt, unsigned frame);

/* vg_step followed by PclOpEvolve::Operate (Particles/Operation/
 * pclOpEvolve.cpp:36-58) on the same vorton records, fused: each record also
 * gets position += velocity x dt before the records go back to the host --
 * the plugin pair a scene runs on its vorton group, in one call and one copy
 * each way.  Positions bit-identical to vg_step then the Euler step in FP32. */
vg_status vg_step_evolve(vg_ctx* ctx, void* particles, size_t n, size_t stride, const float* extra_min,
                         const float* extra_max, float dt, unsigned frame);

/* One frame of a scene's two particle groups in one call: vg_step (or, with
 * evolve_vortons, vg_step_evolve) on the n vorton records, then vg_advect on
 * the m tracer records through that step's velocity grid -- the vorton
 * group's PclOpVortonSim (+ PclOpEvolve) and the tracer group's
 * PclOpAssignVelocityFromField (gain 1) + PclOpEvolve
 * (Particles/Operation/pclOpAdvect.cpp:132-152, pclOpEvolve.cpp:36-58).  The
 * tracer records' upload runs on a second stream while the vortons step,
 * and the vortons' records return on it while the tracers are advected.
 * Results bit-identical to the two calls; m = 0 is vg_step / vg_step_evolve
 * alone.
 * vg_step, vg_step_evolve and vg_step_advect on a fixed grid (and, for the
 * Poisson technique, a fixed multigrid schedule) with records in pinned host
 * memory capture their work as a CUDA graph on the second identical call and
 * replay it on later ones (identical: the same record pointers, counts,
 * strides, dt, extra box, first vorton's size, configuration and workspace). */
vg_status vg_step_advect(vg_ctx* ctx, void* vortons, size_t n, size_t stride, const float* extra_min,
                         const float* extra_max, float dt, unsigned frame, int evolve_vortons, void* tracers,
                         size_t m, size_t tracer_stride);

/* Device-resident form of vg_step.  pos_size: float4 per vorton (x, y, z,
 * size); angvel: float4 (x, y, z, unused), updated in place; vel: float4
 * written.  extra_minmax: 6 host floats (min xyz, max xyz) or NULL. */
vg_status vg_step_device(vg_ctx* ctx, const float* pos_size, float* angvel, float* vel, size_t n,
                         const float* extra_minmax, float dt, unsigned frame);
/* vg_step_device followed by PclOpEvolve on the same vortons: pos_size's
 * x, y, z also move by velocity x dt (written in place), folded into the
 * kernel that writes the velocities when no later stage of the step reads the
 * positions.  Bit-identical to vg_step_device then vg_evolve_device. */
vg_status vg_step_evolve_device(vg_ctx* ctx, float* pos_size, float* angvel, float* vel, size_t n,
                                const float* extra_minmax, float dt, unsigned frame);

/* Replaces VortonSim::GetVelocityGrid (vortonSim.h:334-335).  Copies the last
 * step's velocity grid (float[3] per point) into host memory when xyz is not
 * NULL and cap_points is large enough; always fills geom. */
vg_status vg_get_velocity_grid(vg_ctx* ctx, float* xyz, size_t cap_points, vg_grid_geom* geom);
/* Device pointer to the velocity grid (float[3] per point). */
vg_status vg_get_velocity_grid_device(vg_ctx* ctx, const float** dev_xyz, vg_grid_geom* geom);
/* Replaces VortonSim::GetVectorPotentialMultiGrid()[0] (vortonSim.h:342-343). */
vg_status vg_get_vector_potential(vg_ctx* ctx, float* xyz, size_t cap_points, vg_grid_geom* geom);
/* Statistics of the last step (waits for that step to finish). */
vg_status vg_get_stats(vg_ctx* ctx, vg_step_stats* stats);

/* Multigrid schedule of a context's Poisson solves.  The default (0, 0) is
 * adaptive: FP32 cycles until the relative residual is near FP32's reach,
 * then refinement rounds until poisson_tolerance, with a residual read back to
 * the host after each phase.  A fixed schedule (fp32_cycles > 0) runs exactly
 * fp32_cycles FP32 cycles and then refinement_cycles refinement cycles with no
 * host round trip, so a step can be captured in a CUDA graph; its residuals
 * are read at vg_get_stats.  vg_get_poisson_schedule returns the counts the
 * last adaptive solve used (a calibration for the fixed schedule).  No
 * counterpart in the reference, whose cascade runs a fixed sweep count
 * (vortonSim.cpp:2539-2571). */
vg_status vg_set_poisson_schedule(vg_ctx* ctx, int fp32_cycles, int refinement_cycles);
vg_status vg_get_poisson_schedule(const vg_ctx* ctx, int* fp32_cycles, int* refinement_cycles);

/* Precision of the multigrid's coarsest solve (sine transforms over the whole
 * GPU, used when the coarsest level has more than 512 interior points): FP32
 * (on = 0, the default) or FP64 tables and arithmetic (on = 1).  No
 * counterpart in the reference, whose cascade has no coarsest solve.  Cycles
 * captured earlier are recaptured; a step captured by the caller in a CUDA
 * graph must be captured again.  The batched persistent solve needs FP32. */
vg_status vg_set_coarsest_fp64(vg_ctx* ctx, int on);
/* Wait for the context's stream and report any error a device stage flagged
 * since the last synchronising call (VG_OUT_OF_GRID, VG_NONFINITE).  The
 * *_device entry points do not synchronise; host-buffer calls do this
 * themselves. */
vg_status vg_synchronize(vg_ctx* ctx);

/* Replaces PclOpAssignVelocityFromField (gain 1) followed by PclOpEvolve
 * (Particles/Operation/pclOpAdvect.cpp:42-152, pclOpEvolve.cpp:36-58) for
 * tracers: velocity gathered trilinearly from the last step's velocity grid,
 * then position += velocity * dt.  Particles must lie inside the grid. */
vg_status vg_advect(vg_ctx* ctx, void* particles, size_t m, size_t stride, float dt);
/* Device form: pos float4 (xyz, w untouched) updated in place, vel float4
 * written (may be NULL). */
vg_status vg_advect_device(vg_ctx* ctx, float* pos, float* vel, size_t m, float dt);

/* Replaces PclOpEvolve (Particles/Operation/pclOpEvolve.cpp:36-58) on device
 * records: pos4[i].xyz += vel4[i].xyz * dt (w untouched). */
vg_status vg_evolve_device(vg_ctx* ctx, float* pos4, const float* vel4, size_t m, float dt);
/* Particle operations on device-resident particles (float4 arrays), for engines that keep vortons
 * and tracers on the GPU across frames.
 * Replaces PclOpWind::Operate (Particles/Operation/pclOpWind.cpp:18-42): vel4[i].xyz =
 * wind_weight * wind + src_weight * vel4[i].xyz, per component in FP32 (nothing when wind_weight
 * == 0 and src_weight == 1, as there). */
vg_status vg_wind_device(vg_ctx* ctx, float* vel4, size_t m, const float wind[3], float wind_weight, float src_weight);
/* Replaces PclOpKillAge::Operate (Particles/Operation/pclOpKillAge.cpp:22-47): a particle with
 * int(frame - birth[i]) > age_max is removed by moving the last particle into its slot
 * (Particles::Kill, Particles/particle.h:490-495), so the survivors end in the reference's order.
 * Up to three float4 arrays (any may be NULL) and birth are permuted together in place; *m_out =
 * survivors.  Synchronises the context's stream. */
vg_status vg_kill_age_device(vg_ctx* ctx, float* a4, float* b4, float* c4, int* birth, size_t m, unsigned frame,
                             int age_max, size_t* m_out);

/* ---- Stage entry points on device memory (run on the context's stream).
 * Each replaces one reference function and is what the step composes; they
 * exist so that callers holding their own buffers can run one stage, and so
 * that each stage can be checked against the oracle. */

/* UniformGridGeometry::DefineShape (uniformGrid.h:259-322), host-side. */
vg_status vg_define_shape(size_t n, const float vmin[3], const float vmax[3], int pow2, vg_grid_geom* out);

/* IndicesOfPosition / OffsetOfPosition (uniformGrid.h:536-574, 645-651):
 * idx3 uint32[3 m] and offset uint32[m] for m float4 positions. */
vg_status vg_bin_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos4, size_t m, unsigned* idx3,
                        unsigned* offset);

/* Particles::PartitionParticles as called by VortonSim::PartitionVortons
 * (Particles/particle.cpp:398-437, VortonFluid/vortonSim.cpp:3578-3607): the
 * cell lists of n float4 positions on grid g.  For each point offset c
 * (OffsetOfPosition), items[start[c] .. start[c+1]) are the indices binned
 * there in ascending order, as the reference's push_back in index order
 * leaves them.  start has points + 2 entries: list `points` holds vortons
 * outside the grid or not finite (undefined behaviour in the reference), and
 * start[points + 1] = n.  items has n entries.  Device pointers, context
 * stream. */
vg_status vg_partition_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos4, size_t n, unsigned* start,
                              unsigned* items);

/* ComputeVelocity_Direct / ComputeVectorPotential_Direct
 * (VortonFluid/vortonSim.cpp:1113-1158) at m query points (float4) from n
 * vortons; kind 0 velocity, 1 vector potential; out float4 per query. */
vg_status vg_direct_device(vg_ctx* ctx, int kind, const float* pos_size, const float* angvel, size_t n,
                           const float* q4, size_t m, float spread_range, float spread_circ, float* out4);

/* The direct technique's velocity grid: ComputeVelocity_Direct
 * (vortonSim.cpp:1113-1158) at every gridpoint of g, the gridpoint positions
 * of ComputeVelocityGridSlice (min + i x spacing x (1 - 2 FLT_EPSILON),
 * vortonSim.cpp:2229-2252) into velgrid3 (float[3] per point, x fastest), and
 * when vel4 is not NULL at each of the n vortons too (float4 records, as
 * COMPUTE_VELOCITY_AT_VORTONS does, vorton.h:63-69).  This is the velocity
 * evaluation of vg_step_device's direct technique. */
vg_status vg_direct_grid_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos_size, const float* angvel,
                                size_t n, float* velgrid3, float* vel4);

/* CreateInfluenceTree (vortonSim.cpp:1605-1624) on grid g; then
 * ComputeVelocity_Tree / ComputeVectorPotential_Tree from the root
 * (vortonSim.cpp:1650-1905) at m query points.  tree_out (optional): 8 floats
 * per point per layer (pos xyz, size, angvel xyz, unused), leaf first;
 * tree_points receives the total point count. */
vg_status vg_tree_device(vg_ctx* ctx, int kind, const vg_grid_geom* g, const float* pos_size,
                         const float* angvel, size_t n, const float* q4, size_t m, float spread_range,
                         float spread_circ, float* out4, float* tree_out, size_t tree_cap_points,
                         size_t* tree_points);

/* PopulateVorticityGridFromVortons(grid, scale) (vortonSim.cpp:2372-2436). */
vg_status vg_splat_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos_size, const float* angvel, size_t n,
                          float scale, float* grid3);

/* ComputeVectorPotentialFromVorticity_Integral, boundaries only
 * (vortonSim.cpp:2055-2204): treecode vector potential on the 6 faces. */
vg_status vg_boundary_vecpot_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos_size,
                                    const float* angvel, size_t n, int copy_odd_x, float* grid3);

/* SolveVectorPoisson, Dirichlet (Core/SpatialPartition/uniformGridMath.cpp:1116-1405). */
vg_status vg_sor_device(vg_ctx* ctx, const vg_grid_geom* g, float* soln3, const float* lap3, int steps);
/* The cascade of VortonSim::ComputeVectorPotential (vortonSim.cpp:2539-2571). */
vg_status vg_cascade_device(vg_ctx* ctx, const vg_grid_geom* g, float* soln3, const float* rhs3, int steps);
/* FP32 V-cycles in iterative refinement to `tolerance` (new; the reference's
 * cascade cannot reach a residual target).  The refinement residual is
 * evaluated to FP64-class accuracy in float-pair arithmetic and its norm in
 * FP64; the coarsest level (at most 32,768 interior points) is solved exactly
 * by sine transforms.  soln3 holds the boundary values and the initial
 * interior guess on entry. */
vg_status vg_multigrid_device(vg_ctx* ctx, const vg_grid_geom* g, float* soln3, const float* rhs3,
                              double tolerance, int max_cycles, int* cycles, double* relres0, double* relres);
/* DownSampleInto / UpSampleFrom (Core/SpatialPartition/nestedGrid.h:253-293,
 * uniformGrid.h:1453-1700): inject 1 = FASTER_LESS_ACCURATE, 0 = 27-point;
 * interior_only 1 = INTERIOR_ONLY. */
vg_status vg_downsample_device(vg_ctx* ctx, const vg_grid_geom* fine, const float* fine3, const vg_grid_geom* coarse,
                               int inject, float* coarse3);
vg_status vg_upsample_device(vg_ctx* ctx, const vg_grid_geom* coarse, const float* coarse3,
                             const vg_grid_geom* fine, int interior_only, float* fine3);

/* ComputeJacobian + ComputeCurlFromJacobian (uniformGridMath.cpp:207-451):
 * jac9 (optional) float[9] per point (j[3a+b] = d v_b / d a), curl3 float[3]. */
vg_status vg_jacobian_curl_device(vg_ctx* ctx, const vg_grid_geom* g, const float* vec3, float* jac9, float* curl3);

/* StretchAndTiltVortons (vortonSim.cpp:2748-2820) with velocity grid vel3. */
vg_status vg_stretch_device(vg_ctx* ctx, const vg_grid_geom* g, const float* vel3, const float* pos_size,
                            float* angvel, size_t n, float dt);

/* DiffuseAndDissipateVorticityPSE (vortonSim.cpp:3578-3879), order-independent
 * form: every pair the reference visits exchanges from the pre-step values. */
vg_status vg_pse_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos_size, float* angvel, size_t n,
                        float viscosity, float dt);

/* DiffuseAndDissipateHeatPSE (vortonSim.cpp:3880-4093) on per-vorton densities (mDensity),
 * order-independent form: every pair the reference visits (one cell, or face neighbours along +x,
 * +y, +z) exchanges clamp(2 diffusivity dt exp(-d^2 / (4 size)^2), +-0.5) of its density difference
 * from the pre-step values; then each vorton of a "here" cell relaxes toward ambient_density by
 * clamp(diffusivity dt, +-0.5).  Matches the reference's in-place order to O(2 diffusivity dt x
 * neighbours) of the change; run it after vg_step_device (before the vortons move), where the
 * reference's step runs it. */
vg_status vg_heat_pse_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos_size, float* density, size_t n,
                             float diffusivity, float ambient_density, float dt);

/* VortonSim::PopulateDensityAndMassFractionGrids, density part
 * (vortonSim.cpp:2911-3016): n vortons' densities (mDensity) times their
 * volume (pi/6 size^3 of the first vorton, particle.h:225-228) over the cell
 * volume, spread trilinearly onto grid g (UniformGrid::Accumulate,
 * uniformGrid.h:1278-1342, summed at each point in vorton order), plus the
 * ambient density times max(1 - contribution, 0) at every point.  density_grid
 * has one float per point.  Mass fractions (combustion) are not computed. */
vg_status vg_density_grid_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos_size, const float* density,
                                 size_t n, float ambient_density, float* density_grid);

/* ComputeGradient (uniformGridMath.cpp:468-503, 650-800) of a scalar grid:
 * centred differences inside, one-sided on the faces; grad3 float[3] per point. */
vg_status vg_gradient_device(vg_ctx* ctx, const vg_grid_geom* g, const float* scalar, float* grad3);

/* Baroclinic generation of vorticity on the density-grid path of
 * VortonSim::GenerateBaroclinicVorticity (vortonSim.cpp:3407-3547) and
 * GenerateBaroclinicVorticitySlice (vortonSim.cpp:3318-3392): the density grid
 * of the vortons (vg_density_grid_device), its gradient, the gradient at each
 * vorton, then angvel += 0.5 (grad x (grav / ambient_density)) dt.  *applied is
 * 0 when the grid has no extent along gravity (the reference's early return).
 * Combustion (CombustAndSetMassFractions) is not run. */
vg_status vg_baroclinic_device(vg_ctx* ctx, const vg_grid_geom* g, const float* pos_size, const float* density,
                               float* angvel, size_t n, const float grav[3], float ambient_density, float dt,
                               int* applied);

/* PopulateSignedDistanceGridFromDensityGrid (vortonSim.cpp:3266-3290) with
 * ComputeImmediateSDFFromDensity_Nearest and
 * ComputeRemainingSDFFromImmediateSDF_Nearest (pclOpEmit.cpp:696-1060): the
 * signed distance (negative inside the heavy fluid) of a density grid, NaN
 * where no surface is reached.  reference_stats = 1 sums the density
 * statistics in FP32 point order as the reference does (one GPU thread; the
 * result is then the reference's bit for bit); 0 sums them in FP64 in
 * parallel (the surface moves by ~1e-6 of the distances). */
vg_status vg_signed_distance_device(vg_ctx* ctx, const vg_grid_geom* g, const float* density_grid,
                                    float ambient_density, int reference_stats, float* sdf);

/* Fluid-body boundary conditions (FluidBodySim/fluidBodySim.cpp) on
 * device-resident particles.  Bodies are given on the host, nb <= 16, as 32
 * floats each:
 *   [0] shape: 0 sphere, 1 box (a ConvexPolytope_MakeBox, Collision/
 *       convexPolytope.cpp:346-376); [1] 1 for a hollow box (a container the
 *       fluid fills); [2..4] position; [5..7] velocity; [8..10] angular
 *       velocity; [11..19] orientation matrix rows; [20] sphere radius, or
 *       [20..22] box dimensions; [23] temperature; [24] thermal conductivity;
 *       [25] one over heat capacity (0: 1); the rest unused.
 * Particles are float4 pos_size (position, diameter), vel4 and angvel4 (the
 * reference's angular velocity, vorticity / 2), and density per particle. */

/* CollideVortonsSlice (fluidBodySim.cpp:759-1180) for each body in turn over
 * all vortons, as SolveBoundaryConditions runs it (fluidBodySim.cpp:
 * 1651-1715): a vorton within 1.5 radii of a body is placed outside it,
 * bounced, given the Brinkman-penalty vorticity blended with the body's spin,
 * and exchanges heat with the body through its density (temperature =
 * 300 ambient / density).  Per body, body_out receives 9 floats: linear
 * impulse (zero in the reference's smoothed-particle form), angular impulse,
 * heat to the body, the sum of the collided vortons' temperatures and the
 * body's new temperature (fluidBodySim.cpp:1703-1714); collided (may be NULL)
 * the collision counts.  The particle results equal the reference's bit for
 * bit; the body sums are FP64 reductions in a fixed order (the reference adds
 * in vorton order in FP32).  Synchronises the context's stream. */
vg_status vg_collide_vortons_device(vg_ctx* ctx, const float* bodies, int nb, float* pos_size, float* vel4,
                                    float* angvel4, float* density, size_t n, float ambient_density,
                                    float specific_heat, float* body_out, unsigned long long* collided);

/* CollideTracersSlice (fluidBodySim.cpp:1300-1455) for each body in turn: a
 * tracer in contact is placed outside the body and bounced; per body body_out
 * receives 6 floats, the linear and angular impulses on the body (tracer mass
 * = density x pi/6 size^3; density may be NULL for 1).  Synchronises. */
vg_status vg_collide_tracers_device(vg_ctx* ctx, const float* bodies, int nb, float* pos_size, float* vel4,
                                    const float* density, size_t n, float* body_out);

/* RemoveEmbeddedParticles (fluidBodySim.cpp:365-417): particles inside a
 * body (sphere: within its radius; box: contact distance below the
 * particle's radius) are removed, for each body in turn, leaving the
 * survivors in the order of the reference's swap-with-last walk.  The
 * records of pos_size and, when given, b4, c4 (float4) and d1 (float) move
 * together; *m_out receives the survivors' count.  Synchronises. */
vg_status vg_remove_embedded_device(vg_ctx* ctx, const float* bodies, int nb, float* pos_size, float* b4, float* c4,
                                    float* d1, size_t m, size_t* m_out);

/* ---- Emitters: particles appended to device-resident arrays (PclOpEmit,
 * Particles/Operation/pclOpEmit.h:16-34, pclOpEmit.cpp:77-210), for engines
 * that keep vortons and tracers on the GPU across frames.
 *
 * The arrays of one particle group.  pos_size is required; any other pointer
 * may be NULL (that attribute is not kept).  Particles [0, count) are live;
 * an emitter writes [count, count + k) and advances count, and refuses with
 * VG_TOO_LARGE, writing nothing, when count + k would exceed capacity. */
typedef struct vg_particles {
  float* pos_size; /* float4: position (mPosition), size (mSize) */
  float* vel4;     /* float4: velocity, w = 0 */
  float* angvel4;  /* float4: angular velocity, w = 0 */
  float* orient4;  /* float4: orientation (axis-angle), w = 0 */
  float* density;  /* float: mDensity */
  float* fire4;    /* float4: fuel, flame and smoke fractions, w = 0 */
  int* birth;      /* int: mBirthTime (frame) */
  size_t count;
  size_t capacity;
} vg_particles;

/* The values of one particle that PclOpEmit's template and spread hold. */
typedef struct vg_particle_values {
  float position[3];
  float velocity[3];
  float orientation[3];
  float angular_velocity[3];
  float density;
  float fuel_fraction;
  float flame_fraction;
  float smoke_fraction;
  float size;
} vg_particle_values;

/* PclOpEmit's state: mTemplate, mSpread, mEmitRate (60 in the reference's
 * constructor) and mRemainder (0 there). */
typedef struct vg_emitter {
  vg_particle_values tmpl;
  vg_particle_values spread;
  float emit_rate;
  float remainder;
} vg_emitter;

/* Where an emitter's random jitter comes from. */
typedef enum vg_jitter {
  VG_JITTER_HOST_RAND = 0, /* the C library's rand() on the host, drawn in the reference's order */
  VG_JITTER_HASH = 1       /* a counter-based stream on the device (seed, draw index): no host work */
} vg_jitter;

/* Replaces PclOpEmit::Operate (pclOpEmit.cpp:188-210): emits int(time_step x
 * emit_rate + remainder) particles, keeping the fraction in em->remainder;
 * each is the template plus RandomSpread (Core/Math/math.h:183-188) of the
 * spread, drawn from the C library's rand() in the reference's order
 * (position z, y, x, then velocity, orientation, angular velocity likewise,
 * then density, fuel, flame, smoke fractions, size), born at `frame`.  The
 * records are made on the host, as the reference's are, and appended to the
 * device arrays with one copy and one kernel.  On VG_TOO_LARGE nothing is
 * drawn and em is unchanged.  Synchronises. */
vg_status vg_emit_device(vg_ctx* ctx, vg_emitter* em, float time_step, unsigned frame, vg_particles* p);

/* Replaces PclOpEmit::Emit (pclOpEmit.cpp:77-186), the tracer seeding:
 * multiplier^3 particles per cell of grid g (cells in z, y, x order, sub-cells
 * likewise), each at its sub-cell's centre plus a jitter below half a
 * sub-cell, density 1 (the reference's ambient), size 1/2 cbrt(cell volume) /
 * multiplier, smoke fraction 1, born at frame 0.  With vortons
 * (vorton_pos_size not NULL; n_vortons may be 0), their density deviations
 * from 1 are accumulated onto g and a particle is kept only where the
 * interpolated deviation is at least half the largest magnitude, with
 * density deviation + that magnitude; nothing is emitted (or drawn) when the
 * deviation is zero everywhere.  jitter VG_JITTER_HOST_RAND consumes 3 rand()
 * per sub-cell exactly as the reference does (bit-identical positions after
 * the same srand); VG_JITTER_HASH draws on the device from seed.  A particle
 * whose position rounds onto the grid's far face with vortons given is not
 * kept and raises VG_OUT_OF_GRID (the reference reads past the grid there).
 * Synchronises. */
vg_status vg_emit_grid_device(vg_ctx* ctx, const vg_grid_geom* g, unsigned multiplier, const float* vorton_pos_size,
                              const float* vorton_density, size_t n_vortons, int jitter, unsigned seed,
                              vg_particles* p);

/* Isosurface of a scalar grid by marching cubes, as ExtractIsoLevel /
 * PolygoniseCellWithNormal do (Render/Resource/marchingCubes.cpp:580-866),
 * into device buffers instead of a vertex buffer: cells in z, y, x order; per
 * triangle 9 floats of vertex positions (the reference's VertexInterp on each
 * crossing edge, corners at min + index x spacing) and, when normals is not
 * NULL, 9 floats of its unit face normal repeated per vertex.  Corners below
 * iso_level are inside; normals point away from them.  The triangulation of
 * each cell is generated by this library (the reference's lookup tables are
 * not used), so triangle connectivity can differ from the reference's in
 * cells with an ambiguous face; the vertex positions on each crossing edge
 * follow the reference's arithmetic.  *triangles receives the count; if it
 * exceeds max_triangles nothing is written and VG_TOO_LARGE is returned (the
 * reference's RESULT_INSUFFICIENT_CAPACITY).  Synchronises the context's
 * stream. */
vg_status vg_marching_cubes_device(vg_ctx* ctx, const vg_grid_geom* g, const float* values, float iso_level,
                                   float* vertices, float* normals, size_t max_triangles, size_t* triangles);

/* AssignParticleVelocityFromField (gain 1) + EvolveParticlesSlice on float4
 * positions with grid vel3; vel4 (optional) receives the gathered velocity. */
vg_status vg_gather_advect_device(vg_ctx* ctx, const vg_grid_geom* g, const float* vel3, float* pos4, float* vel4,
                                  size_t m, float dt);

/* Allocation-free direct sum.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory when they need a velocity -- an
 * application that gives this library a fixed memory budget up front, a
 * real-time frame that must not stall on the allocator's implicit device
 * synchronisation, or an embedding that forbids the CUDA allocator.  Same
 * arguments as vg_direct_device (FAST numerics), but it takes no context and
 * allocates nothing: its scratch is one fixed 8 MiB device array inside this
 * library, reserved when the library's device code is loaded on a device
 * (with lazy module loading, at the first call there) and held by that device
 * until the process exits.
 *  - Results: the kernels and source split of vg_direct_device, so they are
 *    bit-identical to it unless the 8 MiB cap forces fewer source chunks; then
 *    they are equal within rounding (the partial sums are grouped
 *    differently).
 *  - Limits: n <= 32768 sources and m <= (8 MiB - 32 n) / 12 targets;
 *    larger calls return VG_TOO_LARGE (use vg_direct_device).
 *  - Each call looks up the array's address on the current device (this
 *    allocates nothing).  On a device where the library's device code is not
 *    loaded yet, that lookup loads it: make the first call on each device
 *    before any stream capture.
 *  - Every call uses the same array and leaves its contents behind; nothing
 *    in it needs clearing, since each call writes every byte it reads.  Calls
 *    that can overlap on the GPU (on different streams, or on one stream from
 *    different host threads) race and must be ordered by the caller.
 *  - Runs on `stream` (a cudaStream_t; NULL = the legacy default stream) and
 *    returns without synchronising.  Errors: vg_last_error(NULL); a launch
 *    failure is reported from that launch's own return code, so errors other
 *    code left pending are not consumed. */
vg_status vg_direct_noalloc(void* stream, int kind, const float* pos_size, const float* angvel, size_t n,
                            const float* q4, size_t m, float spread_range, float spread_circ, float* out4);

/* ------------------------------------------------------------------------
 * Learned warm start (no counterpart in the reference).  A 3D U-Net (4 levels,
 * 16/32/64/128 channels, 3x3x3 convolutions, BF16 weights and activations,
 * FP32 accumulation) maps the Poisson right-hand side and the Dirichlet
 * boundary values of an (edge+1)^3 grid to an initial vector potential;
 * multigrid then finishes the solve to its tolerance.  The network is trained
 * on this library's own forward and backward kernels.
 *
 * A network object owns its device buffers and a stream (the caller's, or one
 * it creates).  Attached to a context with vg_set_network, it runs on the
 * context's stream inside vg_step; calls on the network itself must not
 * overlap a step of that context unless both use the same stream.
 * Errors: vg_net_last_error(net), or vg_last_error(NULL) from vg_net_create. */
typedef struct vg_net vg_net;

/* edge: network grid edge = grid points per axis - 1; 32 or a multiple of 64 up to 1024. */
vg_status vg_net_create(int device, void* stream, unsigned edge, vg_net** out);
vg_status vg_net_destroy(vg_net* net);
const char* vg_net_last_error(const vg_net* net);
/* Number of FP32 parameters: per layer W[27][Co][Ci] (tap = 9(dz+1) + 3(dy+1) + dx+1), then bias[Co]. */
size_t vg_net_param_count(void);
vg_status vg_net_set_params(vg_net* net, const float* params, size_t count, float out_scale);
vg_status vg_net_get_params(vg_net* net, float* params, size_t count, float* out_scale);
/* Weight file: BF16 weights, FP32 biases and the output scale. */
vg_status vg_net_save(vg_net* net, const char* path);
vg_status vg_net_load(vg_net* net, const char* path);
/* Writes the network's guess into the interior points of vecpot3 (AoS xyz per
 * point, (edge+1)^3 points), whose boundary points already hold the Dirichlet
 * values; rhs3 is the solver's right-hand side (minus the vorticity). */
vg_status vg_net_guess_device(vg_net* net, const vg_grid_geom* g, const float* rhs3, float* vecpot3);
/* Training: forward + backward on one (right-hand side, converged solution)
 * pair (FP32, or BF16 when pair_bf16 != 0); the parameter gradients replace
 * the previous ones, or are added to them when accumulate != 0 (batches).
 * The loss is the squared error of the interior solution relative to the
 * solution's own squared norm; loss (optional, host) receives it and makes
 * the call synchronise. */
vg_status vg_net_backward_device(vg_net* net, const vg_grid_geom* g, int pair_bf16, const void* rhs3,
                                 const void* vecpot3, int accumulate, float* loss);
vg_status vg_net_adam_step(vg_net* net, float lr, float beta1, float beta2, float eps);
vg_status vg_net_get_grads(vg_net* net, float* grads, size_t count);
/* FP32 output of the last forward pass: [edge^3][16], channels 0..2 used. */
vg_status vg_net_get_output(vg_net* net, float* out, size_t count);
/* BF16 activation `which` of the last forward pass as FP32, channels-last:
 * 0 input, then enc0a, enc0b, pool1, enc1a, enc1b, pool2, enc2a, enc2b, pool3,
 * enc3a, enc3b, dec2a, dec2b, dec1a, dec1b, dec0a, dec0b (17). */
vg_status vg_net_get_activation(vg_net* net, int which, float* out, size_t count);
/* BF16 gradient of the last backward pass as FP32, channels-last: of_input = 0
 * the gradient w.r.t. layer `layer`'s pre-activation output (Co channels),
 * of_input = 1 the gradient w.r.t. its (pooled or concatenated) input
 * (Ci channels; layers 2, 4, 6, 8, 10, 12 only). */
vg_status vg_net_get_gradient(vg_net* net, int layer, int of_input, float* out, size_t count);
vg_status vg_net_synchronize(vg_net* net);
/* count FP32 values -> BF16 (training pairs), on stream; no context. */
vg_status vg_net_to_bf16_device(const float* src, void* dst, size_t count, void* stream);
/* Attach (or detach with NULL) a network; with warm_start = VG_WARM_NETWORK
 * the Poisson solve starts from its guess whenever the grid has edge+1 points
 * per axis, and from zero otherwise (vg_step_stats.warm_start_used says which). */
vg_status vg_set_network(vg_ctx* ctx, vg_net* net);

/* ------------------------------------------------------------------------
 * Batched effects (no counterpart in the reference).  Many independent
 * simulations stepped per frame.  Each simulation is a context with a fixed
 * grid and the multigrid Poisson step, and its vortons (float4 arrays as in
 * vg_step_device) stay on the device.  A frame is vg_step_device + the
 * vortons' Euler advection for every simulation; each solve starts from the
 * simulation's previous solution (or the network's guess).  After calibration
 * (two adaptive steps each, which fix each simulation's multigrid schedule and
 * size its workspaces), a frame has no host round trip, so it is
 * captured once as CUDA graphs and replayed: the simulations are dealt to
 * `streams` parallel branches, each branch's chain is captured as graphs of at
 * most a few thousand kernels, and a frame forks into the branches, launches
 * their graphs and joins.  With the persistent solve (vg_batch_set_solver), every simulation whose
 * multigrid hierarchy ends in the sine-transform solve over the GPU has its Poisson solve taken
 * out of its branch: a frame runs the steps up to the solve on the branches, then one cooperative
 * launch in which teams of CTAs run all those solves (largest first, a team barrier between
 * phases, results bit-identical to the per-simulation launches), then the rest of the steps and
 * the advection on the branches.  A vorton that leaves its simulation's fixed grid
 * stops (zero velocity) and drops out of that simulation's solve instead of
 * failing the frame (vg_batch_outside reports it).  Errors: vg_batch_last_error. */
typedef struct vg_batch vg_batch;

vg_status vg_batch_create(int device, int streams /* 1..32 */, vg_batch** out);
vg_status vg_batch_destroy(vg_batch* batch);
const char* vg_batch_last_error(const vg_batch* batch);
/* cfg: use_fixed_grid = 1, VG_VELOCITY_POISSON, VG_POISSON_MULTIGRID (stream and device are the
 * batch's).  The arrays stay the caller's and must outlive the batch. */
vg_status vg_batch_add(vg_batch* batch, const vg_config* cfg, float* pos_size, float* angvel, float* vel, size_t n,
                       int* index);
/* One network per (grid edge, stream) for the simulations whose grids it fits; others start from zero. */
vg_status vg_batch_load_network(vg_batch* batch, const char* path);
/* Stream count and network use (invalidates the graphs; a network change also the calibration). */
vg_status vg_batch_configure(vg_batch* batch, int streams, int use_network);
/* Two adaptive steps of every simulation (they advance them), fixing their multigrid schedules
 * for solves started from the previous frame's solution (or the network's guess). */
vg_status vg_batch_calibrate(vg_batch* batch, float dt);
/* mode 0: the captured graphs (captured on first use and after any change); mode 1: the same work
 * simulation after simulation on one stream, no graph.  Calibrates first if needed.  Does not
 * synchronise. */
vg_status vg_batch_step(vg_batch* batch, float dt, int mode);
/* Waits for the batch and reports device-side errors of any simulation. */
vg_status vg_batch_synchronize(vg_batch* batch);
/* The autotuner: times `frames` graph replays for each stream count in candidates (with and
 * without the network when one is loaded), then, at the best of those, with the persistent solve
 * off and at team sizes of 4, 8, 16 and 32 CTAs; keeps the fastest setting and reports it
 * (best_ms per frame; vg_batch_solver_info gives the solver setting).  Steps the simulations
 * while measuring. */
vg_status vg_batch_autotune(vg_batch* batch, float dt, int frames, const int* candidates, int ncand,
                            int* best_streams, int* best_network, float* best_ms);
/* persistent: 1 solves qualifying simulations in one persistent launch per frame, 0 inside each
 * simulation's branch graphs (the default); team_ctas: CTAs per team (0: 8); max_points: only
 * grids of at most this many points go to the persistent launch (0: any size), the others solve
 * in their branches.  Invalidates the graphs.  A team barrier that waits more than 2 s gives up;
 * vg_batch_synchronize then reports VG_TIMEOUT. */
vg_status vg_batch_set_solver(vg_batch* batch, int persistent, int team_ctas, size_t max_points);
/* The captured frame's solver: simulations in the persistent launch, its teams and CTAs per team,
 * and whether the launch was captured as a graph (1) or is launched directly (0). */
vg_status vg_batch_solver_info(const vg_batch* batch, int* persistent_sims, int* teams, int* team_ctas,
                               int* captured);
/* Diagnostics (no counterpart in the reference): the persistent solve's team barrier on one team
 * of `ctas` CTAs (at most one per SM) of which the last `missing` never arrive, each wait limited
 * to limit_ms (at most 10 s).  *completed = CTAs that passed two barriers; *gave_up = 1 when a
 * wait ran out (the CTAs then return, and the device stays usable). */
vg_status vg_team_barrier_check(int device, int ctas, int missing, float limit_ms, int* completed, int* gave_up);
/* *outside = 1 when a vorton of simulation `index` has left its grid since the last call, which
 * clears the record.  Synchronises the batch. */
vg_status vg_batch_outside(vg_batch* batch, int index, int* outside);
/* A simulation's context (for vg_get_stats, vg_get_velocity_grid), owned by the batch.  After a
 * graph frame, call vg_batch_synchronize before reading it; per-step times are then 0. */
vg_ctx* vg_batch_context(vg_batch* batch, int index);
int vg_batch_size(const vg_batch* batch);
/* The captured frame: how many graphs it launches (the persistent solve's included), and their
 * largest and total node counts (0 before the first graph frame). */
vg_status vg_batch_graph_info(const vg_batch* batch, int* graphs, size_t* max_nodes, size_t* total_nodes);

#ifdef __cplusplus
}
#endif
#endif /* VORTEGRID_H */
