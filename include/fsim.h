/*
 * fsim.h -- C ABI of the GB300-native FLIP step hot path.
 *
 * One handle (fsim_t) owns the device state of one simulation domain: the
 * particle store (SoA, sorted by cell in OpenVDB leaf iteration order), the
 * sparse 8^3 brick layout (active-leaf list, 27-entry neighbour table, per-leaf
 * per-cell particle ranges) and the grid fields stored per leaf.  A handle is
 * bound to one CUDA stream and is not thread-safe.  Every entry point returns
 * an int status (FSIM_OK on success); fsim_last_error() gives the message.
 * Host buffers passed in are copied; the handle owns all device memory.
 *
 * Index space: voxel length 1, cell (i,j,k) covers [i,i+1)x[j,j+1)x[k,k+1),
 * the domain is [0,N) per axis, solid walls are the cells at -1 and N.  MAC
 * staggering: vel(i,j,k)[0] is the x-face at x=i centred at (j+.5,k+.5), and
 * likewise for y and z.  Dense downloads cover voxels [-1,N] per axis and use
 * the linear index ((i+1)*(N1+2) + (j+1))*(N2+2) + (k+1).
 *
 * Each stage function names the reference member function it replaces
 * (schinmayee/fluid-sim-lb, paths relative to that project).
 */
#ifndef FSIM_H
#define FSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  FSIM_OK = 0,
  FSIM_ERR_INVALID = 1,        /* bad argument or configuration */
  FSIM_ERR_CUDA = 2,           /* a CUDA runtime call failed */
  FSIM_ERR_CAPACITY = 3,       /* particle / leaf capacity exceeded */
  FSIM_ERR_NOT_CONVERGED = 4,  /* PCG hit max iterations (relative mode) */
  FSIM_ERR_BREAKDOWN = 5,      /* PCG alpha or beta > 1e5 or not finite
                                  (replaces CHECK_LE(alpha, LARGE_FLOAT),
                                  common/solver.cc:333,361) */
  FSIM_ERR_STATE = 6,          /* call order violated */
  FSIM_ERR_NO_DEVICE = 7,      /* no CUDA device visible */
  FSIM_ERR_TIMEOUT = 8         /* a bounded device-side wait ran out */
};

/* CellType, common/definitions.h:6 */
enum { FSIM_AIR = 0, FSIM_FLUID = 1, FSIM_SOLID = 2 };

/* Boundary kind, FlipApp config "boundary", common/flip_app_sim.cc:105-112 */
enum { FSIM_BOUNDARY_BOX = 0, FSIM_BOUNDARY_TANK = 1 };

typedef struct fsim_sim fsim_t;

/* Simulation parameters.  Mirrors FlipSimulation::InitializeMetadata
 * (common/flip_simulation.cc:84-101) and SetForces (:249-253).  gravity and
 * force are index-space values the caller has already scaled (the reference
 * scales by N/128, common/flip_app_sim.cc:74,87). */
typedef struct fsim_config {
  int32_t global_dims[3];      /* cells per axis, 8 <= N <= 1024 */
  int32_t boundary;            /* FSIM_BOUNDARY_* */
  float gravity;               /* gravity_ used by CFL(): sqrt(0.5*gravity) */
  float force[3];              /* fx_,fy_,fz_: AddGravity adds dt*(fx,-fy,fz) */
  float flip_factor;           /* FLIP/PIC blend */
  int32_t nparticles_per_cell; /* seeding target */
  int64_t max_particles;       /* particle capacity (0: 9 per domain cell,
                                  capped to fit) */
  int32_t device;              /* CUDA device ordinal */
} fsim_config;

int fsim_create(const fsim_config* cfg, fsim_t** out);
int fsim_destroy(fsim_t* sim);
const char* fsim_last_error(const fsim_t* sim); /* sim may be NULL */
/* Library version string, never NULL. */
const char* fsim_version(void);

/* Raw cudaStream_t the handle launches on. */
int fsim_get_stream(fsim_t* sim, void** stream);
int fsim_synchronize(fsim_t* sim);

/* ---- solids (static) --------------------------------------------------- */
/* FlipSimulation::AddSolidCuboid, common/flip_simulation.cc:316-324: the
 * inclusive integer box [lo,hi] intersected with the domain grown by one
 * cell.  Box/tank walls come from cfg->boundary (SetBoxBoundary :256-308,
 * SetTankBoundary :332-377).  At most 32 cuboids. */
int fsim_add_solid_cuboid(fsim_t* sim, const int32_t lo[3], const int32_t hi[3]);

/* ---- scene seeding (setup, not part of a step) ------------------------- */
/* A seeding pass restates FlipSimulation::InitializePhiAndParticles
 * (common/flip_simulation.cc:139-188) for phi = min over the pass's shapes:
 * each non-solid cell whose centre has phi < 0 gets up to
 * nparticles_per_cell particles drawn uniformly in the cell (at most 32
 * draws, a draw is kept where phi(p) <= 0), unless the cell already holds
 * that many.  glibc random() is replaced by a counter-based SplitMix64
 * stream keyed by (seed, pass, cell, draw).  Shapes (index space):
 *   CUBOID: a = start, b = end, phi = inside(inclusive) ? -1 : 1 (:222-233)
 *   SPHERE: a = centre, r = radius, phi = |p-a| - r                (:236-246)
 *   POOL:   a[1] = height, phi = p.y - height                       (:200-219) */
enum { FSIM_SHAPE_CUBOID = 0, FSIM_SHAPE_SPHERE = 1, FSIM_SHAPE_POOL = 2 };
typedef struct fsim_shape {
  int32_t kind;
  float a[3];
  float b[3];
  float r;
} fsim_shape;
#define FSIM_MAX_SHAPES 8
typedef struct fsim_seed_pass {
  int32_t nshapes;
  fsim_shape shapes[FSIM_MAX_SHAPES];
  float velocity[3];           /* initial velocity and grid_velocity */
} fsim_seed_pass;
int fsim_seed_fluid(fsim_t* sim, const fsim_seed_pass* passes, int32_t npasses,
                    uint64_t seed);
/* Adds N(0, sigma^2) per component to particle velocity and grid_velocity
 * (same draw for both), counter-based stream keyed by (seed, particle rank). */
int fsim_perturb_velocities(fsim_t* sim, float sigma, uint64_t seed);

/* ---- water sources ----------------------------------------------------- */
/* application::Source<T> (common/sources.cc), already scaled to index space
 * (boxes times the global dimensions, velocities times the scaled gravity,
 * as FlipDriver::Initialize does, common/flip_app_sim.cc:96-104).  Restated
 * as the reference computes it:
 *   get_box(t) is box1 with its end lowered by 1 on every axis; the
 *     oscillating branch of the reference writes a shadowed local and has no
 *     effect, so an oscillating box stays box1;
 *   get_velocity(t) is velocity1, or, when velocity_oscillating,
 *     v1 + 0.5 (v2 - v1)(cos(pi t / box_period) + 1) (the reference uses the
 *     box period here);
 *   is_active(t) is start_time <= t <= end_time for timed sources, else true.
 * At most FSIM_MAX_SOURCES sources. */
#define FSIM_MAX_SOURCES 16
typedef struct fsim_source {
  float lo[3], hi[3];        /* box1 start, end */
  float lo2[3], hi2[3];      /* box2 start, end (oscillating box) */
  float box_period;
  float velocity[3];         /* velocity1 */
  float velocity2[3];
  float velocity_period;     /* stored; see get_velocity above */
  int32_t box_oscillating;
  int32_t velocity_oscillating;
  int32_t timed;
  float start_time, end_time;
} fsim_source;
/* FlipSimulation::AddWaterSource, common/flip_simulation.cc:327-329 */
int fsim_add_source(fsim_t* sim, const fsim_source* source);
/* The simulation time sources see (the driver's advanced_time_); fsim_step
 * reads it and then adds dt (FlipDriver::AdvanceTime). */
int fsim_set_time(fsim_t* sim, double t);
int fsim_get_time(fsim_t* sim, double* t);
/* FlipSimulation::AddContributionFromSources(t), :1207-1270: every active
 * source adds up to nparticles_per_cell particles to each cell of its box
 * (at most 32 draws; a draw is kept inside the box), with velocity and grid
 * velocity set to the source velocity.  Draws use the seeding generator
 * keyed by the seed of the last fsim_seed_fluid and a per-call stream.  The
 * grid writes of the reference are cleared by ClearGridData before any
 * stage reads them and are not made. */
int fsim_add_contribution_from_sources(fsim_t* sim, float t);
/* FlipSimulation::DeleteFluidInSources(t), :1273-1281: particles inside the
 * box of any source (active or not) are deleted. */
int fsim_delete_fluid_in_sources(fsim_t* sim, float t);

/* ---- init-file scenes --------------------------------------------------- */
/* FlipApp::ParseSimulationConfiguration (common/flip_app.cc:159-251) and the
 * scaling of FlipDriver::Initialize (common/flip_app_sim.cc:70-183) for a
 * grid of dims cells.  Keys (one per line, tokens split on ", :"): fluid,
 * boundary, gravity, force, fluid-cube, fluid-sphere, source-static,
 * source-timed, source-oscillating, solid; other lines are ignored.
 * Defaults: fluid 1, boundary 0, gravity 9.8, force (0,1,0).  The result is
 * what Initialize applies, in its order: the config (scaled gravity =
 * gravity * N1/128, force * scaled gravity), the sources (boxes * dims,
 * velocities * scaled gravity), the boundary, the solids (cubes * dims as
 * get_coord_bbox gives them), and the seeding passes (the fluid preset, then
 * each additional fluid: cubes * dims with their end lowered by 1, spheres
 * * dims, velocities * scaled gravity). */
#define FSIM_SCENE_MAX_SOLIDS 32
typedef struct fsim_scene {
  int32_t fluid;            /* preset: 0 none, 1 sphere drop, 2 dam break */
  int32_t boundary;         /* FSIM_BOUNDARY_* */
  float gravity;            /* scaled: config gravity * N1 / 128 */
  float force[3];           /* config force * scaled gravity */
  int32_t nsolids;
  int32_t solid_lo[FSIM_SCENE_MAX_SOLIDS][3];
  int32_t solid_hi[FSIM_SCENE_MAX_SOLIDS][3];
  int32_t npasses;
  fsim_seed_pass passes[8];
  int32_t nsources;
  fsim_source sources[FSIM_MAX_SOURCES];
} fsim_scene;
/* text: the init file's contents.  FSIM_ERR_INVALID for a malformed line
 * (message in fsim_last_error(NULL)) or a solid cube not on whole cells;
 * FSIM_ERR_CAPACITY past 32 solids, 16 sources or 8 seeding passes. */
int fsim_scene_parse(const char* text, const int32_t dims[3], fsim_scene* out);

/* ---- particle I/O ------------------------------------------------------ */
/* pos/vel/gvel are n xyz triples (AoS float[3*n]).  Upload rebins (stable
 * sort by cell in OpenVDB leaf order) and rebuilds the brick topology. */
int fsim_upload_particles(fsim_t* sim, const float* pos, const float* vel,
                          const float* gvel, int64_t n);
int fsim_particle_count(fsim_t* sim, int64_t* n);
/* Live particles in cell order (the reference's iteration order).
 * Any of pos/vel/gvel may be NULL.  Fails with FSIM_ERR_CAPACITY when the
 * count exceeds capacity (n is still written). */
int fsim_download_particles(fsim_t* sim, float* pos, float* vel, float* gvel,
                            int64_t capacity, int64_t* n);

/* ---- per-stage entry points (FlipSimulation member functions) ---------- */
/* FlipSimulation::CFL, common/flip_simulation.cc:460-488: returns 1/v with
 * v = max(sqrt(0.5*gravity), max |v_d| over active in-box faces), v>=1e-2. */
int fsim_cfl(fsim_t* sim, float* inv_speed);
/* Particles::StepInGrid<VectorGrid,true,1,1> (common/particles.cc:479-546)
 * followed by Particles::DeleteParticlesInSolids (:202-219). */
int fsim_move_particles(fsim_t* sim, float dt);
/* FlipSimulation::ClearGridData, common/flip_simulation.cc:380-389 */
int fsim_clear_grid(fsim_t* sim);
/* FlipSimulation::TransferParticlesToGrid, :809-923 (marker FLUID, weighted
 * velocity, weight, normalisation with the 1e-5 cut). */
int fsim_transfer_particles_to_grid(fsim_t* sim);
/* FlipSimulation::ApplyBoundaryConditions, :657-713 */
int fsim_apply_boundary_conditions(fsim_t* sim);
/* FlipSimulation::SaveGridVelocities, :491-496 */
int fsim_save_grid_velocities(fsim_t* sim);
/* Particles::DeleteOutsideParticles, common/particles.cc:273-293 */
int fsim_delete_outside_particles(fsim_t* sim);
/* FlipSimulation::ReinitializePhiSimple, :529-539 */
int fsim_reinitialize_phi(fsim_t* sim);
/* FlipSimulation::AddGravity, :506-515 */
int fsim_add_gravity(fsim_t* sim, float dt);
/* FlipSimulation::ComputeDivergence, :716-736 */
int fsim_compute_divergence(fsim_t* sim);
/* FlipSimulation::UpdateVelocityFromPressure, :739-778 */
int fsim_update_velocity_from_pressure(fsim_t* sim);
/* FlipSimulation::GetVelocityUpdate, :781-801 */
int fsim_get_velocity_update(fsim_t* sim);
/* FlipSimulation::UpdateParticlesFromGrid, :1025-1091, including both
 * VectorGrid::ExtrapolateToBoundary calls (common/vector_grid.cc:302-381). */
int fsim_update_particles_from_grid(fsim_t* sim);

/* ---- pressure solve (PCGDriver::Solve, common/solver_driver.cc:14-69) --- */
enum {
  FSIM_PCG_ABSOLUTE = 0, /* reference rule: stop when r.r < threshold or
                            iterations >= max (solver_driver.cc:319-337) */
  FSIM_PCG_RELATIVE = 1, /* stop when ||r||/||b|| <= tolerance */
  FSIM_PCG_FIXED = 2     /* exactly max_iterations (fixed_iterations_) */
};
enum {
  FSIM_PREC_FP32 = 0,  /* reference: fp32 vectors and fp32 dot products */
  FSIM_PREC_MIXED = 1, /* fp32 inner PCG with FP64-accumulated dots and an
                          FP64 outer residual refinement r = b - A x */
  FSIM_PREC_FP64 = 2   /* fp64 vectors and dots */
};
typedef struct fsim_pcg_params {
  int32_t mode;            /* FSIM_PCG_* */
  int32_t precision;       /* FSIM_PREC_* */
  int32_t max_iterations;  /* all inner iterations of one solve (reference default 1500) */
  int32_t max_refinements; /* MIXED: outer refinement sweeps (>=1) */
  double threshold;        /* ABSOLUTE: r.r threshold (reference N^3*0.5e-8) */
  double tolerance;        /* RELATIVE: ||r||/||b|| target (outer, MIXED) */
  double inner_tolerance;  /* MIXED: drop of the fp32 recursive residual between fp64
                              residual replacements; no segment iterates below
                              tolerance*||b||, where the fp64 check decides */
} fsim_pcg_params;
typedef struct fsim_pcg_stats {
  int32_t iterations;      /* total inner iterations */
  int32_t refinements;     /* outer sweeps (MIXED), else 1 */
  int32_t n_rows;          /* fluid cells (PCG unknowns) */
  int32_t status;          /* FSIM_OK / NOT_CONVERGED / BREAKDOWN */
  double rr;               /* final r.r (fp64 residual in MIXED) */
  double bb;               /* b.b */
  double loop_ms;          /* device time of the iteration loops (CUDA events on
                              the handle's stream around them; setup and the
                              MIXED replacement sweeps excluded) */
} fsim_pcg_stats;
/* Fills params with the reference defaults for the handle's domain:
 * ABSOLUTE, FP32, 1500 iterations, threshold N1*N2*N3*0.5e-8
 * (common/flip_app.cc:325-332, common/flip_app.h:52-53). */
int fsim_pcg_default_params(const fsim_t* sim, fsim_pcg_params* params);
/* Builds A from the marker (7-point Laplacian, SOLID neighbours excluded,
 * common/solver.cc:198-233), b from the divergence, x0 = 0, runs Jacobi PCG
 * and writes the pressure grid (CopySolution, solver.cc:94-99). */
int fsim_pcg_solve(fsim_t* sim, const fsim_pcg_params* params,
                   fsim_pcg_stats* stats);

/* ---- one step (FlipDriver::RunOneStep, common/flip_app_sim.cc:211-254) -- */
typedef struct fsim_step_stats {
  int64_t particles;       /* live particles after the step */
  int32_t particle_leaves; /* 8^3 leaves holding particles */
  int32_t grid_leaves;     /* leaves holding grid values (dilated by 1) */
  fsim_pcg_stats pcg;
  float next_inv_speed;    /* CFL() of the velocity left by this step */
} fsim_step_stats;
/* With sources: AddContributionFromSources(time) first and
 * DeleteFluidInSources(time) after the move; time then advances by dt.
 * MoveParticles(dt) + DeleteParticlesInSolids, ClearGridData,
 * TransferParticlesToGrid, ApplyBoundaryConditions, SaveGridVelocities,
 * DeleteOutsideParticles, ReinitializePhiSimple, AddGravity(dt),
 * ApplyBoundaryConditions, ComputeDivergence, PCG solve,
 * UpdateVelocityFromPressure, GetVelocityUpdate, UpdateParticlesFromGrid --
 * run as fused device kernels.  stats may be NULL.  A step that fails after
 * the rebinning leaves the particles' PIC velocities (gvel) undefined: the
 * rebinning moves them only for the per-stage calls, since the step's G2P
 * rewrites them. */
int fsim_step(fsim_t* sim, float dt, const fsim_pcg_params* params,
              fsim_step_stats* stats);
/* One step on a host-resident particle state: the same results as
 * fsim_upload_particles(pos, vel, gvel, n); fsim_step(dt, params, stats);
 * fsim_download_particles(out_pos, out_vel, out_gvel, capacity, n_out) --
 * the way the reference steps particles that live in its runtime's host
 * variables (FlipDriver::RunOneStep, common/flip_app_sim.cc:211-254, with
 * the particle store in host memory).  The copies overlap the step: the
 * velocity upload runs while positions are binned and sorted, and the
 * position download runs during the pressure solve (positions are final
 * after the sort).  Outputs may alias the inputs of the same name.  Host
 * buffers should be pinned for full copy bandwidth.  With sources or the
 * tank boundary the three calls run in sequence. */
int fsim_step_host(fsim_t* sim, float dt, const fsim_pcg_params* params, const float* pos,
                   const float* vel, const float* gvel, int64_t n, float* out_pos,
                   float* out_vel, float* out_gvel, int64_t capacity, int64_t* n_out,
                   fsim_step_stats* stats);

/* Global dt rule of FlipDriver::WhileAndComputeDt (flip_app_sim.cc:357-428)
 * for one partition: dt = min(cfl*inv_speed, 1/frame_step), raised to
 * frame_step/10, clipped to the frame end (also when it would pass 0.9 of
 * the frame).  *time_in_frame is advanced by dt.  Host-only. */
int fsim_compute_dt(float inv_speed, int32_t cfl, float frame_step,
                    float* time_in_frame, float* dt);

/* The frame loop of the reference's driver (SimulationDriver::RunSimulation,
 * projects/flip-current-lb/water_app.cc:68-86, with WhileAndComputeDt and
 * AdvanceTime, common/flip_app_sim.cc:357-462): for each of nframes frames
 * of 1/frame_rate, steps run while time_in_frame + 1e-5 < frame step, each
 * with dt from the rule of fsim_compute_dt on CFL() of the previous step's
 * velocity (fsim_cfl before the first step).  on_frame (nullable) is called
 * after each frame (SaveData's place).  The loop is driven from the host:
 * each step rebuilds the leaf topology, whose counts size the next launches,
 * so a step cannot be one graph. */
typedef void (*fsim_frame_fn)(fsim_t* sim, int32_t frame, void* user);
typedef struct fsim_run_stats {
  int32_t frames;
  int32_t steps;
  int64_t pcg_iterations;
  double time;            /* the handle's time after the loop */
  float last_dt;
} fsim_run_stats;
int fsim_run_frames(fsim_t* sim, int32_t nframes, float frame_rate, int32_t cfl,
                    const fsim_pcg_params* params, fsim_frame_fn on_frame, void* user,
                    fsim_run_stats* stats);

/* ---- dense downloads (parity / output) -------------------------------- */
enum {
  FSIM_FIELD_VELOCITY = 0,        /* grid_velocity_ (Vec3) */
  FSIM_FIELD_VELOCITY_UPDATE = 1, /* grid_velocity_update_ (Vec3) */
  FSIM_FIELD_WEIGHT = 2,          /* grid_weight_ (Vec3) */
  FSIM_FIELD_DIVERGENCE = 3,      /* grid_divergence_ (scalar) */
  FSIM_FIELD_PRESSURE = 4,        /* grid_pressure_ (scalar) */
  FSIM_FIELD_PHI = 5              /* grid_phi_ (scalar, background 5) */
};
/* Vec3 fields: out has 3*(N1+2)(N2+2)(N3+2) floats (xyz per voxel); scalar
 * fields one float per voxel.  active (nullable) gets 1 byte per voxel:
 * the OpenVDB active state.  Inactive voxels read the background. */
int fsim_download_field(fsim_t* sim, int32_t field, float* out, uint8_t* active);
/* grid_marker_ as int32 per voxel (AIR background), active per voxel. */
int fsim_download_marker(fsim_t* sim, int32_t* out, uint8_t* active);
/* Particle-tree leaf topology: origins (xyz triples, cells) of the 8^3
 * leaves holding particles, in OpenVDB leaf iteration order. */
int fsim_download_leaves(fsim_t* sim, int32_t* origins, int64_t capacity,
                         int64_t* n);

/* ---- allocation-free CFL ---------------------------------------------- */
/* No counterpart in the reference: it serves callers that cannot call
 * cudaMalloc while they step -- an engine that hands the solver device
 * buffers from its own pre-reserved pool and forbids allocation in its frame
 * loop, or a real-time loop where an allocation would stall the device.
 * Computes FlipSimulation::CFL() (1/v, v = max(sqrt(0.5*gravity), max |v_d|
 * over active in-box faces, excluding the last index on tangential axes),
 * v >= 1e-2) from a face-velocity field the caller already holds in device
 * memory, in the dense layout of fsim_download_field: vel has
 * 3*(N1+2)(N2+2)(N3+2) floats, active one byte per voxel; the result is
 * written to the device float *inv_speed, ordered on stream (NULL: the
 * legacy default stream).  No handle; nothing is allocated: the reduction's
 * scratch is a fixed file-scope device array (4 KB + a counter) that every
 * GPU loading the library holds until exit.  The first call on a device
 * looks up that array's address (cudaGetSymbolAddress) with the device
 * current, so make the first call before any stream capture.  The address
 * is kept per device for the life of the process: after cudaDeviceReset (a
 * new primary context) it is stale, so do not call this across a reset.
 * All calls on a device share the scratch: calls that overlap on the GPU
 * race.
 * Returns FSIM_ERR_CAPACITY when a dimension exceeds 1024 (the maximum),
 * FSIM_ERR_INVALID for a null pointer or a dimension below 8. */
int fsim_cfl_noalloc(const float* vel, const uint8_t* active, const int32_t dims[3],
                     float gravity, float* inv_speed, void* stream);

/* ---- particles to a level set ------------------------------------------ */
/* The method of the reference's converter (projects/particles-to-levelset/
 * convert.cc:80-156, OpenVDB ParticlesToLevelSet::rasterizeSpheres then
 * LevelSetFilter::mean): each live particle is a sphere of `radius` voxels
 * (the converter uses 3); phi at voxel point (i,j,k) is min over particles
 * of |(i,j,k) - p| - radius, clamped to [-half_width, half_width] (OpenVDB's
 * default band is 3); then mean_iterations passes replace every band voxel
 * by the mean of its 3^3 neighbourhood (outside the box counts as
 * half_width) and re-clamp.  OpenVDB's re-normalisation of the band after a
 * filter pass is not restated.  phi (and active, |phi| < half_width) are
 * dense host arrays in the layout of fsim_download_field; the .vdb files the
 * converter writes are left to the caller.  No counterpart in the library
 * path of the reference (it is a separate tool). */
int fsim_particles_to_level_set(fsim_t* sim, float radius, float half_width,
                                int32_t mean_iterations, float* phi, uint8_t* active);

/* ---- differentiable rollout (adjoint of projection and advection) ------ */
/* No counterpart in the reference (the reference has no gradients).  A
 * rollout of `steps` FLIP steps (the fsim_step sequence, box boundary) at a
 * fixed dt from the particle state the handle holds at fsim_rollout_create,
 * with the loss L = 0.5 * sum (u - u_target)^2 over the grid faces active
 * after the last step's pressure update with their node in [0,N]^3; u_target
 * is a dense face field in the layout of fsim_download_field.
 *
 * Gradients are those of the rollout with the discrete choices frozen at the
 * forward run: particle binning and sort order, wall clamping and deletion,
 * the side of the cell centre each particle's trilinear stencil starts on
 * (ScatterWeight / InterpolateComponent), FLUID markers, active faces and
 * the 1e-5 weight cut.  The pressure solves
 * are taken as exact (A is symmetric, so the adjoint solve is the same PCG).
 * The forward keeps a checkpoint of the particle state every
 * checkpoint_every steps and the frozen topology of every step; the backward
 * pass recomputes each segment from its checkpoint and reverses it.
 * Adjoint values accumulate in fp64.  Particle arrays are SoA (x | y | z),
 * 3*n doubles, in the order of the initial particle state. */
typedef struct fsim_rollout fsim_rollout_t;
/* A rollout borrows sim: destroy it before fsim_destroy(sim). */
int fsim_rollout_create(fsim_t* sim, int32_t steps, int32_t checkpoint_every,
                        fsim_rollout_t** out);
int fsim_rollout_destroy(fsim_rollout_t* r);
/* Number of particles of the initial state. */
int fsim_rollout_particle_count(fsim_rollout_t* r, int64_t* n);
/* Initial particle velocity (vel) and grid velocity (gvel), as doubles. */
int fsim_rollout_get_initial_velocity(fsim_rollout_t* r, double* vel, double* gvel);
/* Replaces the initial vel and gvel (rounded to float) before a forward. */
int fsim_rollout_set_initial_velocity(fsim_rollout_t* r, const double* vel,
                                      const double* gvel);
/* The fp32 forward: fsim_step `steps` times (pcg: the solve parameters),
 * recording checkpoints and topology; loss as above.  The handle is left
 * holding the final state. */
int fsim_rollout_forward(fsim_rollout_t* r, float dt, const fsim_pcg_params* pcg,
                         const float* target, double* loss);
/* Gradient of the loss w.r.t. the initial vel and gvel (either pointer may
 * be null).  tape 0: linearised along the fp32 forward (recomputed from the
 * checkpoints); tape 1: along an fp64 replay of the forward with the frozen
 * topology (the fp64 reference gradient).  adj: parameters of the adjoint
 * pressure solves (FP64 or MIXED precision; relative tolerance). */
int fsim_rollout_backward(fsim_rollout_t* r, int32_t tape, const fsim_pcg_params* adj,
                          double* grad_vel, double* grad_gvel);
/* Loss of an fp64 replay of the forward with the frozen topology from the
 * initial positions and the given initial vel / gvel (null: the stored
 * ones).  Pressure solves in FP64: the first replay after a forward solves
 * each step to relative residual 1e-12 and keeps its iteration count, and
 * every later replay runs exactly those counts, so the replay loss is a
 * smooth function of vel / gvel (what central differences need). */
int fsim_rollout_replay_loss(fsim_rollout_t* r, const double* vel, const double* gvel,
                             double* loss);

/* ---- kernel timing (CUDA events on the handle's stream) --------------- */
int fsim_set_profiling(fsim_t* sim, int32_t enabled);
/* Accumulated per-kernel device time since the last reset.  Writes up to
 * capacity entries; names are static strings owned by the library. */
int fsim_get_kernel_times(fsim_t* sim, const char** names, double* total_ms,
                          int64_t* launches, int32_t capacity, int32_t* count);
int fsim_reset_kernel_times(fsim_t* sim);
/* Number of library kernel launches issued on this handle so far. */
int fsim_launch_count(fsim_t* sim, int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* FSIM_H */
