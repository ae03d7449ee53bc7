// flip_demo.cc -- a driver written against the reference's call surface.
//
// Runs the sphere-drop scene the way FlipDriver::Initialize and
// FlipDriver::RunOneStep (schinmayee/fluid-sim-lb, common/flip_app_sim.cc:
// 30-206, 211-254) sequence the FlipSimulation / PCGDriver calls, on one GPU
// through fsim_facade.h, then repeats the same steps with the fused
// fsim_step and reports both.  Usage:
//   fsim_demo <N> <steps> <output_dir> [staged|fused] [debug]
// "debug" also writes SaveDebugDataToFile's dumps after the last step.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <sys/stat.h>

#include "fsim_facade.h"

using application::FlipSimulation;
using common::Coord;
using common::Vec3;

typedef FlipSimulation<3, 3, float> Sim;

static float frame_dt(float inv, float* t_in_frame, float frame_step) {
  float dt = 0.f;
  fsim_compute_dt(inv, 1, frame_step, t_in_frame, &dt);
  if (*t_in_frame + 1e-5f >= frame_step) *t_in_frame = 0.f;
  return dt;
}

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 32;
  const int steps = argc > 2 ? std::atoi(argv[2]) : 4;
  const std::string out = argc > 3 ? argv[3] : "demo_out";
  const bool fused = argc > 4 && std::string(argv[4]) == "fused";
  const bool debug = argc > 5 && std::string(argv[5]) == "debug";
  const float g = float(9.8 * n);  // gravity -9.8 with dx = 1/N, index space
  const float frame_step = 1.0f / 30.0f;

  Sim sim;
  Sim::VectorGridT vel, vold, weight;
  Sim::ScalarGridT phi, div, pres;
  Sim::ScalarGridInt marker;
  Sim::ParticlesT particles;
  // FlipDriver::Initialize: metadata, variables, forces, boundary, fluid
  sim.InitializeMetadata(Coord(n), Coord(1), 0, 1.0f, 8, g, 0.95f, out, false);
  sim.set_grid_velocity(&vel);
  sim.set_grid_velocity_update(&vold);
  sim.set_grid_weight(&weight);
  sim.set_grid_phi(&phi);
  sim.set_grid_divergence(&div);
  sim.set_grid_pressure(&pres);
  sim.set_grid_marker(&marker);
  sim.set_particles(&particles);
  sim.SetForces(Vec3<float>(0.f, g, 0.f));
  sim.SetBoxBoundary();
  sim.InitializeVariables();
  sim.InitializeMultipleWaterDrops(0.2f * n, {Vec3<float>(0.5f * n, 0.7f * n, 0.5f * n)},
                                   {0.15f * n});
  const int volume = n * n * n;
  common::PCGDriver<Sim::ScalarGridT> solver(nullptr, "pcg", 1500,
                                             float(volume) * float(0.5 * 1e-8), false,
                                             common::IC, Coord(1), Coord(n));
  solver.SetVariables(&div, &marker, &pres);
  solver.Bind(sim.handle());
  std::printf("particles %zu\n", sim.ParticleCount());
  mkdir((out + "_0").c_str(), 0755);

  float t_in_frame = 0.f;
  float inv = sim.CFL();
  auto t0 = std::chrono::steady_clock::now();
  for (int s = 0; s < steps; ++s) {
    const float dt = frame_dt(inv, &t_in_frame, frame_step);
    int iters = 0;
    if (!fused) {
      sim.MoveParticles(dt, true);
      sim.DeleteParticlesInSolids();
      sim.ClearGridData();
      sim.TransferParticlesToGrid();
      sim.ApplyBoundaryConditions();
      sim.SaveGridVelocities();
      sim.DeleteOutsideParticles();
      sim.ReinitializePhiSimple();
      sim.AddGravity(dt);
      sim.ApplyBoundaryConditions();
      sim.ComputeDivergence();
      solver.Solve();
      sim.UpdateVelocityFromPressure();
      sim.GetVelocityUpdate();
      sim.UpdateParticlesFromGrid();
      iters = solver.stats().iterations;
      inv = sim.CFL();
    } else {
      fsim_pcg_params prm;
      fsim_pcg_default_params(sim.handle(), &prm);
      fsim_step_stats st = sim.RunOneStepFused(dt, prm);
      iters = st.pcg.iterations;
      inv = st.next_inv_speed;
    }
    std::printf("step %d dt %.6f pcg_iterations %d particles %zu fluid_cells %zu "
                "pressure(%d,%d,%d) %.6g\n",
                s, double(dt), iters, sim.ParticleCount(), sim.FluidCellCount(), n / 2, 2,
                n / 2, double(pres.get(n / 2, 2, n / 2)));
  }
  const double ms = std::chrono::duration<double, std::milli>(
                        std::chrono::steady_clock::now() - t0).count();
  sim.SaveDataToFile();
  if (debug) sim.SaveDebugDataToFile();
  std::printf("done %d steps in %.2f ms (%s)\n", steps, ms, fused ? "fused" : "staged");
  return 0;
}
