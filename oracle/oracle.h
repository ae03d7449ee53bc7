/*
 * oracle.h -- CPU restatement of the reference FLIP step (TEST INFRASTRUCTURE).
 *
 * This library is the checker for the GPU implementation and the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py may load it.  It restates, with strict IEEE
 * float arithmetic (no FMA contraction, no fast-math), the single-partition
 * CPU path of schinmayee/fluid-sim-lb:
 *   common/flip_simulation.cc  (P2G, BCs, gravity, divergence, pressure
 *                               update, velocity update, G2P, CFL, seeding)
 *   common/particles.cc        (StepInGrid, DeleteParticlesInSolids,
 *                               DeleteOutsideParticles)
 *   common/vector_grid.cc      (ExtrapolateToBoundary)
 *   common/solver.cc, common/solver_driver.cc (Jacobi PCG, stopping rule)
 *   common/flip_app_sim.cc     (RunOneStep order, dt rule)
 * OpenVDB trees are replaced by dense arrays over voxels [-2, N+1]^3 with an
 * explicit "active" byte per voxel, restating OpenVDB's rules: setValue
 * activates, getValue of an inactive voxel returns the background, and leaf
 * iteration follows root (64^3 blocks, lexicographic) -> internal node
 * (x-major 8^3 leaves) -> leaf (x-major voxels).
 *
 * Parity status: the reference cannot be built in this environment (it needs
 * OpenVDB 4.0.1, TBB, Boost, glog, cereal, libevent and the Canary runtime),
 * and it ships no tests or golden data, so this restatement is pinned by
 * known-answer tests only ("parity unpinned" against the reference binary).
 * OpenVDB's math::pcg internals (dot accumulation order/type, Jacobi apply)
 * are restated from their definitions: pcg::Vector::dot sums 100 contiguous
 * chunks serially in T and adds the chunk totals in order (OpenVDB reduces
 * contiguous ranges in parallel; the split is not pinned), the reference's
 * own p.Ap loop is summed as the -Ofast build's 4-wide vector code would
 * (four interleaved lanes, then the tail), and Jacobi is z = r * T(1.0/diag).
 */
#ifndef FSIM_ORACLE_H
#define FSIM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

typedef struct orc_shape {
  int32_t kind; /* 0 cuboid, 1 sphere, 2 pool (same as fsim_shape) */
  float a[3];
  float b[3];
  float r;
} orc_shape;

typedef struct orc_seed_pass {
  int32_t nshapes;
  orc_shape shapes[8];
  float velocity[3];
} orc_seed_pass;

typedef struct orc_pcg_stats {
  int32_t iterations;
  int32_t n_rows;
  int32_t status; /* 0 ok, 4 not converged (relative mode), 5 breakdown */
  int32_t pad;
  double rr;
  double bb;
} orc_pcg_stats;

orc_sim* orc_create(const int32_t dims[3], int32_t boundary, float gravity,
                    const float force[3], float flip, int32_t nppc);
void orc_destroy(orc_sim* s);
/* Host threads of the loops whose results do not depend on the thread count
 * (per particle, per leaf, per matrix row or vector entry, the PCG dot
 * products' chunk sums, whose totals are added in chunk order, and the four
 * lane sums of p.Ap): every result is bit-identical for any n.
 * Process-wide; 1 (the default) runs inline. */
void orc_set_threads(int32_t n);
int32_t orc_get_threads(void);
void orc_add_solid_cuboid(orc_sim* s, const int32_t lo[3], const int32_t hi[3]);
int32_t orc_is_solid(const orc_sim* s, int32_t i, int32_t j, int32_t k);

/* Seeding (FlipSimulation::InitializePhiAndParticles restated with the
 * counter-based SplitMix64 draw shared with the GPU library). */
int64_t orc_seed(orc_sim* s, const orc_seed_pass* passes, int32_t npasses,
                 uint64_t seed);
void orc_perturb_velocities(orc_sim* s, float sigma, uint64_t seed);

/* Particle I/O: AoS xyz triples.  set_particles rebins into cell order. */
void orc_set_particles(orc_sim* s, const float* pos, const float* vel,
                       const float* gvel, int64_t n);
int64_t orc_particle_count(const orc_sim* s);
void orc_get_particles(const orc_sim* s, float* pos, float* vel, float* gvel);
/* 32-bit OpenVDB-order key of each particle's cell (the sort key). */
void orc_get_particle_keys(const orc_sim* s, uint32_t* keys);
/* Origins of the particle-tree leaves in iteration order; returns count. */
int64_t orc_get_leaves(const orc_sim* s, int32_t* origins, int64_t capacity);

/* Stages (reference member functions). */
float orc_cfl(orc_sim* s);
void orc_move_particles(orc_sim* s, float dt);
void orc_delete_particles_in_solids(orc_sim* s);
void orc_clear_grid(orc_sim* s);
void orc_transfer_particles_to_grid(orc_sim* s);
void orc_apply_boundary_conditions(orc_sim* s);
void orc_save_grid_velocities(orc_sim* s);
void orc_delete_outside_particles(orc_sim* s);
void orc_reinitialize_phi(orc_sim* s);
void orc_add_gravity(orc_sim* s, float dt);
void orc_compute_divergence(orc_sim* s);
/* mode: 0 absolute rr < threshold, 1 relative ||r||/||b|| <= tol, 2 fixed.
 * precision: 0 float, 2 double (FP64 oracle solve). */
int32_t orc_pcg_solve(orc_sim* s, int32_t mode, int32_t precision,
                      int32_t max_iterations, double threshold, double tol,
                      orc_pcg_stats* stats);
void orc_update_velocity_from_pressure(orc_sim* s);
int32_t orc_get_velocity_update(orc_sim* s); /* 0 ok, 1 CHECK failure */
void orc_extrapolate_to_boundary(orc_sim* s, int32_t field);
void orc_update_particles_from_grid(orc_sim* s);

/* Water sources (application::Source<T>, common/sources.cc), same layout
 * and rules as fsim_source in include/fsim.h. */
typedef struct orc_source {
  float lo[3], hi[3];
  float lo2[3], hi2[3];
  float box_period;
  float velocity[3];
  float velocity2[3];
  float velocity_period;
  int32_t box_oscillating;
  int32_t velocity_oscillating;
  int32_t timed;
  float start_time, end_time;
} orc_source;
void orc_add_source(orc_sim* s, const orc_source* src);
void orc_set_time(orc_sim* s, double t);
double orc_get_time(const orc_sim* s);
/* FlipSimulation::AddContributionFromSources(t), :1207-1270 */
void orc_add_contribution_from_sources(orc_sim* s, float t);
/* FlipSimulation::DeleteFluidInSources(t), :1273-1281 */
void orc_delete_fluid_in_sources(orc_sim* s, float t);

/* FlipDriver::RunOneStep for one partition (with AddSources before the move
 * and DeleteSources after it, then time += dt); returns the PCG status. */
int32_t orc_step(orc_sim* s, float dt, int32_t mode, int32_t precision,
                 int32_t max_iterations, double threshold, double tol,
                 orc_pcg_stats* stats);
/* dt rule (WhileAndComputeDt); advances *time_in_frame. */
float orc_compute_dt(float inv_speed, int32_t cfl, float frame_step,
                     float* time_in_frame);

/* Dense downloads over voxels [-1,N]^3, index ((i+1)*(N1+2)+(j+1))*(N2+2)+(k+1).
 * field: 0 velocity, 1 velocity update, 2 weight (Vec3), 3 divergence,
 * 4 pressure, 5 phi (scalar).  active may be NULL. */
void orc_get_field(const orc_sim* s, int32_t field, float* out, uint8_t* active);
void orc_get_marker(const orc_sim* s, int32_t* out, uint8_t* active);
/* Pressure as the solver's double-precision vector (FP64 solve), dense. */
void orc_get_pressure_f64(const orc_sim* s, double* out);
/* Set the divergence/marker directly (PCG-only tests): dense [-1,N]^3. */
void orc_set_divergence(orc_sim* s, const float* div);
void orc_set_marker(orc_sim* s, const int32_t* marker);

/* SplitMix64-based uniform draw in [0,1) used by seeding (exported so the
 * tests can check the GPU kernel's draws bit-exactly). */
float orc_seed_uniform(uint64_t seed, int32_t pass, int64_t cell, int32_t draw,
                       int32_t d);

#ifdef __cplusplus
}
#endif

#endif /* FSIM_ORACLE_H */
