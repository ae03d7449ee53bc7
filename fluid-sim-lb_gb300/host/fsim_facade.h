// fsim_facade.h -- C++ call surface with the reference's names over the C ABI.
//
// Mirrors the member functions the reference's simulation driver calls
// (schinmayee/fluid-sim-lb: common/flip_simulation.h:26-346,
// common/solver_driver.h:27-106, common/scalar_grid.h:16-149,
// common/vector_grid.h:16-154, common/particles.h:24-455,
// common/metagrid.h), so a driver written against those classes compiles
// against this header with one domain on one GPU.  All field data lives on
// the device in one fsim_t handle owned by FlipSimulation; ScalarGrid /
// VectorGrid / Particles objects are views bound to it through the same
// set_* calls the reference uses (common/flip_app.cc:607-707).  get() and
// Count() download the field on first use after a stage has run.
//
// Differences from the reference, all deliberate:
//  * one partition (MetaGrid partitions = 1x1x1, rank 0); no Canary;
//  * MoveParticles() also deletes particles in solid cells (the device does
//    it while rebinning; DeleteParticlesInSolids() is then a no-op);
//  * ExtrapolateToBoundary() is applied inside UpdateParticlesFromGrid()
//    on the device, exactly as the reference's UpdateParticlesFromGrid
//    calls it for both grids first;
//  * failures throw common::FsimFailure instead of glog CHECK aborts.
#pragma once

#include <sys/stat.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "fsim.h"

namespace common {

typedef int Index;
enum CellType { AIR, FLUID, SOLID, NUM_CELL_TYPES };
enum PreconditionerType { IC, IC0, JACOBI, NUM_PRECONDITIONER_TYPES };

struct Coord {
  int v[3];
  Coord() : v{0, 0, 0} {}
  explicit Coord(int a) : v{a, a, a} {}
  Coord(int a, int b, int c) : v{a, b, c} {}
  int& operator[](int i) { return v[i]; }
  int operator[](int i) const { return v[i]; }
  int x() const { return v[0]; }
  int y() const { return v[1]; }
  int z() const { return v[2]; }
};

struct CoordBBox {
  Coord lo, hi;
  CoordBBox() {}
  CoordBBox(Coord a, Coord b) : lo(a), hi(b) {}
  Coord min() const { return lo; }
  Coord max() const { return hi; }
};

template <typename T>
struct Vec3 {
  T v[3];
  Vec3() : v{T(0), T(0), T(0)} {}
  explicit Vec3(T a) : v{a, a, a} {}
  Vec3(T a, T b, T c) : v{a, b, c} {}
  T& operator[](int i) { return v[i]; }
  T operator[](int i) const { return v[i]; }
  T x() const { return v[0]; }
  T y() const { return v[1]; }
  T z() const { return v[2]; }
};

template <typename T>
struct Cube {
  Vec3<T> start, end;
  Cube() {}
  Cube(Vec3<T> s, Vec3<T> e) : start(s), end(e) {}
  Vec3<T> get_start() const { return start; }
  Vec3<T> get_end() const { return end; }
};

class FsimFailure : public std::runtime_error {
 public:
  FsimFailure(int code, const std::string& m)
      : std::runtime_error("fsim error " + std::to_string(code) + ": " + m), code(code) {}
  int code;
};

inline void check(fsim_t* h, int rc, const char* what) {
  if (rc != FSIM_OK) throw FsimFailure(rc, std::string(what) + ": " + fsim_last_error(h));
}

// MetaGrid for one partition (common/metagrid.cc:25-35 with partitions 1).
class MetaGrid {
 public:
  MetaGrid() : dims_(64) {}
  MetaGrid(Coord global_dims, Coord partitions = Coord(1), int rank = 0)
      : dims_(global_dims) {
    if (partitions[0] * partitions[1] * partitions[2] != 1 || rank != 0)
      throw std::invalid_argument("one partition per GPU: partitions must be 1x1x1");
  }
  Coord global_dims() const { return dims_; }
  Coord start() const { return Coord(0); }
  Coord end() const { return Coord(dims_[0] - 1, dims_[1] - 1, dims_[2] - 1); }
  CoordBBox bbox() const { return CoordBBox(start(), end()); }
  int dims(size_t i) const { return dims_[int(i)]; }
  int rank() const { return 0; }

 private:
  Coord dims_;
};

// Device-field view shared by the grid classes.
class FieldView {
 public:
  void bind(fsim_t* h, int field, Coord dims) {
    h_ = h;
    field_ = field;
    dims_ = dims;
    stale_ = true;
  }
  bool bound() const { return h_ != nullptr; }
  void invalidate() { stale_ = true; }

 protected:
  size_t lin(int i, int j, int k) const {
    return (size_t(i + 1) * (dims_[1] + 2) + size_t(j + 1)) * (dims_[2] + 2) + size_t(k + 1);
  }
  bool inside(int i, int j, int k) const {
    return i >= -1 && j >= -1 && k >= -1 && i <= dims_[0] && j <= dims_[1] && k <= dims_[2];
  }
  size_t total() const { return size_t(dims_[0] + 2) * (dims_[1] + 2) * (dims_[2] + 2); }
  // Active voxels of the box [0, dims - 1 + grow] in OpenVDB Tree3<T,3,3>
  // iteration order: 64^3 root children in lexicographic order, then x-major
  // 8^3 leaves, then x-major voxels.
  std::vector<Coord> vdb_order(const std::vector<uint8_t>& on, int grow) const {
    std::vector<Coord> out;
    for (int i = 0; i <= dims_[0] - 1 + grow; ++i)
      for (int j = 0; j <= dims_[1] - 1 + grow; ++j)
        for (int k = 0; k <= dims_[2] - 1 + grow; ++k)
          if (on[lin(i, j, k)]) out.push_back(Coord(i, j, k));
    auto key = [](const Coord& c) {
      uint64_t r = 0;
      for (int d = 0; d < 3; ++d) r = (r << 16) | uint64_t(uint32_t(c[d] >> 6) & 0xFFFFu);
      for (int d = 0; d < 3; ++d) r = (r << 3) | uint64_t((c[d] >> 3) & 7);
      for (int d = 0; d < 3; ++d) r = (r << 3) | uint64_t(c[d] & 7);
      return r;
    };
    std::stable_sort(out.begin(), out.end(),
                     [&](const Coord& a, const Coord& b) { return key(a) < key(b); });
    return out;
  }
  fsim_t* h_ = nullptr;
  int field_ = -1;
  Coord dims_;
  mutable bool stale_ = true;
};

template <Index N1, Index N2, typename T>
class ScalarGrid : public FieldView {
 public:
  typedef T ValueType;
  template <typename V>
  struct ValueConverter {
    using Type = ScalarGrid<N1, N2, V>;
  };
  T get(int i, int j, int k) const {
    refresh();
    return inside(i, j, k) ? data_[lin(i, j, k)] : background();
  }
  T get(Coord c) const { return get(c[0], c[1], c[2]); }
  bool isOn(int i, int j, int k) const {
    refresh();
    return inside(i, j, k) && on_[lin(i, j, k)];
  }
  bool isOn(Coord c) const { return isOn(c[0], c[1], c[2]); }
  // ScalarGrid::Count(box, value), common/scalar_grid.cc:87-100
  int Count(CoordBBox box, T value) const {
    refresh();
    int n = 0;
    for (int i = box.lo[0]; i <= box.hi[0]; ++i)
      for (int j = box.lo[1]; j <= box.hi[1]; ++j)
        for (int k = box.lo[2]; k <= box.hi[2]; ++k)
          if (isOn(i, j, k) && get(i, j, k) == value) ++n;
    return n;
  }
  // ScalarGrid::Write, common/scalar_grid.cc:135-160: the box start and end,
  // then "i j k : value" for each active voxel of the box, in OpenVDB
  // iteration order (the text flag only selects the fopen mode there).
  void Write(const std::string& file, bool text = true) const {
    refresh();
    FILE* fp = std::fopen(file.c_str(), text ? "wt" : "wb");
    if (!fp) throw std::runtime_error("cannot open " + file);
    std::fprintf(fp, "0 0 0\n%d %d %d\n", dims_[0] - 1, dims_[1] - 1, dims_[2] - 1);
    for (const Coord& c : vdb_order(on_, 0)) {
      std::fprintf(fp, "%d %d %d : %f\n", c[0], c[1], c[2], float(data_[lin(c[0], c[1], c[2])]));
    }
    std::fclose(fp);
  }

 private:
  T background() const { return field_ == FSIM_FIELD_PHI ? T(5) : T(0); }
  void refresh() const {
    if (!stale_) return;
    if (!h_) throw std::logic_error("grid not bound to a simulation");
    data_.resize(total());
    on_.resize(total());
    if (field_ == -2) {  // marker
      std::vector<int32_t> m(total());
      check(h_, fsim_download_marker(h_, m.data(), on_.data()), "download_marker");
      for (size_t i = 0; i < m.size(); ++i) data_[i] = T(m[i]);
    } else {
      std::vector<float> f(total());
      check(h_, fsim_download_field(h_, field_, f.data(), on_.data()), "download_field");
      for (size_t i = 0; i < f.size(); ++i) data_[i] = T(f[i]);
    }
    stale_ = false;
  }
  mutable std::vector<T> data_;
  mutable std::vector<uint8_t> on_;
};

template <Index N1, Index N2, typename T>
class VectorGrid : public FieldView {
 public:
  typedef T ValueType;
  typedef Vec3<T> Vec3T;
  Vec3T get(int i, int j, int k) const {
    refresh();
    if (!inside(i, j, k)) return Vec3T(0);
    const size_t o = lin(i, j, k);
    return Vec3T(data_[3 * o], data_[3 * o + 1], data_[3 * o + 2]);
  }
  Vec3T get(Coord c) const { return get(c[0], c[1], c[2]); }
  bool isOn(int i, int j, int k) const {
    refresh();
    return inside(i, j, k) && on_[lin(i, j, k)];
  }
  bool isOn(Coord c) const { return isOn(c[0], c[1], c[2]); }
  // Applied on the device inside UpdateParticlesFromGrid (see header note).
  void ExtrapolateToBoundary() {}
  // VectorGrid::Write, common/vector_grid.cc:132-160: the box start and end,
  // then "i j k : vx vy vz" for each active voxel of the box grown by one
  // face (staggered), in OpenVDB iteration order.
  void Write(const std::string& file, bool text = true) const {
    refresh();
    FILE* fp = std::fopen(file.c_str(), text ? "wt" : "wb");
    if (!fp) throw std::runtime_error("cannot open " + file);
    std::fprintf(fp, "0 0 0\n%d %d %d\n", dims_[0] - 1, dims_[1] - 1, dims_[2] - 1);
    for (const Coord& c : vdb_order(on_, 1)) {
      const size_t o = lin(c[0], c[1], c[2]);
      std::fprintf(fp, "%d %d %d : %f %f %f\n", c[0], c[1], c[2], float(data_[3 * o]),
                   float(data_[3 * o + 1]), float(data_[3 * o + 2]));
    }
    std::fclose(fp);
  }

 private:
  void refresh() const {
    if (!stale_) return;
    if (!h_) throw std::logic_error("grid not bound to a simulation");
    data_.resize(3 * total());
    on_.resize(total());
    std::vector<float> f(3 * total());
    check(h_, fsim_download_field(h_, field_, f.data(), on_.data()), "download_field");
    for (size_t i = 0; i < f.size(); ++i) data_[i] = T(f[i]);
    stale_ = false;
  }
  mutable std::vector<T> data_;
  mutable std::vector<uint8_t> on_;
};

template <Index N1, Index N2, typename T = float>
class Particles {
 public:
  typedef struct ParticleData {
    Vec3<T> position;
    Vec3<T> velocity;
    Vec3<T> grid_velocity;
  } ParticleData;
  void bind(fsim_t* h, MetaGrid m) {
    h_ = h;
    meta_ = m;
  }
  int size() const {
    int64_t n = 0;
    check(h_, fsim_particle_count(h_, &n), "particle_count");
    return int(n);
  }
  // Visits every particle in cell iteration order (read-only copy).
  void ForEachConst(std::function<void(const ParticleData&, const Coord, int)> op) const {
    std::vector<float> p, v, g;
    const int64_t n = download(p, v, g);
    for (int64_t i = 0; i < n; ++i) {
      ParticleData d;
      for (int a = 0; a < 3; ++a) {
        d.position[a] = p[3 * i + a];
        d.velocity[a] = v[3 * i + a];
        d.grid_velocity[a] = g[3 * i + a];
      }
      Coord c(int(std::floor(d.position[0])), int(std::floor(d.position[1])),
              int(std::floor(d.position[2])));
      op(d, c, int(i));
    }
  }
  // Particles::Write, common/particles.cc:166-200: header start[3], end[3],
  // n; then per particle id, position[3], velocity[3] (binary) or
  // "%d : %f %f %f, %f %f %f" lines (text).
  void Write(const std::string& file, bool text = true) const {
    std::vector<float> p, v, g;
    const int64_t n = download(p, v, g);
    FILE* fp = std::fopen(file.c_str(), text ? "wt" : "wb");
    if (!fp) throw std::runtime_error("cannot open " + file);
    Coord s = meta_.start(), e = meta_.end();
    if (text) {
      std::fprintf(fp, "%d %d %d\n%d %d %d\n%d\n", s[0], s[1], s[2], e[0], e[1], e[2], int(n));
      for (int64_t i = 0; i < n; ++i)
        std::fprintf(fp, "%d : %f %f %f, %f %f %f\n", int(i), p[3 * i], p[3 * i + 1],
                     p[3 * i + 2], v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    } else {
      int hdr[7] = {s[0], s[1], s[2], e[0], e[1], e[2], int(n)};
      std::fwrite(hdr, sizeof(int), 7, fp);
      for (int64_t i = 0; i < n; ++i) {
        int id = int(i);
        std::fwrite(&id, sizeof(int), 1, fp);
        std::fwrite(&p[3 * i], sizeof(float), 3, fp);
        std::fwrite(&v[3 * i], sizeof(float), 3, fp);
      }
    }
    std::fclose(fp);
  }

 private:
  int64_t download(std::vector<float>& p, std::vector<float>& v, std::vector<float>& g) const {
    int64_t n = 0;
    check(h_, fsim_particle_count(h_, &n), "particle_count");
    p.resize(size_t(3 * n));
    v.resize(size_t(3 * n));
    g.resize(size_t(3 * n));
    int64_t got = 0;
    check(h_, fsim_download_particles(h_, p.data(), v.data(), g.data(), n, &got), "download");
    return got;
  }
  fsim_t* h_ = nullptr;
  MetaGrid meta_;
};

// PCGDriver (common/solver_driver.h:31-47, Solve :14-69) for one partition.
template <class ScalarGridT>
class PCGDriver {
 public:
  typedef typename ScalarGridT::ValueType T;
  PCGDriver(void* /*app: no Canary*/, std::string name, int max_iterations, T threshold,
            bool fixed_iterations, PreconditionerType /*ignored: the reference
            always builds Jacobi, common/solver.h:32,39*/,
            Coord partitions, Coord global_dims)
      : name_(std::move(name)), max_iterations_(max_iterations), threshold_(threshold),
        fixed_(fixed_iterations), meta_(global_dims, partitions, 0) {}
  // b = divergence, marker, x = pressure: the device fields are fixed, the
  // call records that the driver was wired as the reference wires it.
  void SetVariables(ScalarGridT* b, void* marker, ScalarGridT* x) {
    b_ = b;
    marker_ = marker;
    x_ = x;
  }
  void Bind(fsim_t* h) { h_ = h; }
  // Extension: FP32 (reference), MIXED or FP64 inner arithmetic.
  void SetPrecision(int precision, double tolerance = 0.0) {
    precision_ = precision;
    tolerance_ = tolerance;
  }
  void Solve() {
    if (!h_) throw std::logic_error("PCGDriver not bound to a simulation");
    fsim_pcg_params p;
    check(h_, fsim_pcg_default_params(h_, &p), "pcg_default_params");
    p.max_iterations = max_iterations_;
    p.threshold = double(threshold_);
    p.mode = fixed_ ? FSIM_PCG_FIXED : FSIM_PCG_ABSOLUTE;
    p.precision = precision_;
    if (tolerance_ > 0.0) {
      p.mode = FSIM_PCG_RELATIVE;
      p.tolerance = tolerance_;
    }
    check(h_, fsim_pcg_solve(h_, &p, &stats_), "pcg_solve");
    if (x_) x_->invalidate();
  }
  const fsim_pcg_stats& stats() const { return stats_; }

 private:
  std::string name_;
  int max_iterations_;
  T threshold_;
  bool fixed_;
  MetaGrid meta_;
  fsim_t* h_ = nullptr;
  ScalarGridT* b_ = nullptr;
  void* marker_ = nullptr;
  ScalarGridT* x_ = nullptr;
  int precision_ = FSIM_PREC_FP32;
  double tolerance_ = 0.0;
  fsim_pcg_stats stats_{};
};

}  // namespace common

namespace application {

template <common::Index N1, common::Index N2, typename T = float>
class FlipSimulation {
 public:
  typedef common::VectorGrid<N1, N2, T> VectorGridT;
  typedef common::ScalarGrid<N1, N2, T> ScalarGridT;
  typedef common::ScalarGrid<N1, N2, int32_t> ScalarGridInt;
  typedef common::Particles<N1, N2, T> ParticlesT;

  ~FlipSimulation() {
    if (h_) fsim_destroy(h_);
  }

  // FlipSimulation::InitializeMetadata, common/flip_simulation.cc:84-101
  void InitializeMetadata(common::Coord global_dims, common::Coord partitions, int rank,
                          T voxel_len = 1, int num_particles_per_cell = 8, T gravity = 9.8,
                          T flip_factor = 1, std::string output_dir = "output",
                          bool debug_flag = false, int device = 0) {
    if (std::fabs(double(voxel_len) - 1.0) > 1e-2) throw std::invalid_argument("voxel_len 1");
    metagrid_ = common::MetaGrid(global_dims, partitions, rank);
    nppc_ = num_particles_per_cell;
    gravity_ = gravity;
    flip_ = flip_factor;
    output_dir_ = output_dir + "_" + std::to_string(rank);
    debug_ = debug_flag;
    device_ = device;
  }
  void SetForces(const common::Vec3<T>& f) { force_ = f; }
  void SetBoxBoundary() { boundary_ = FSIM_BOUNDARY_BOX; }
  void SetTankBoundary() { boundary_ = FSIM_BOUNDARY_TANK; }

  // FlipSimulation::InitializeVariables: creates the device handle and binds
  // the grid views the driver set with set_*.
  void InitializeVariables() {
    if (h_) return;
    fsim_config c{};
    for (int a = 0; a < 3; ++a) {
      c.global_dims[a] = metagrid_.global_dims()[a];
      c.force[a] = float(force_[a]);
    }
    c.boundary = boundary_;
    c.gravity = float(gravity_);
    c.flip_factor = float(flip_);
    c.nparticles_per_cell = nppc_;
    c.max_particles = 0;
    c.device = device_;
    int rc = fsim_create(&c, &h_);
    if (rc != FSIM_OK) throw common::FsimFailure(rc, "fsim_create");
    for (auto& cu : pending_solids_) check_(fsim_add_solid_cuboid(h_, cu.first.v, cu.second.v));
    pending_solids_.clear();
    bind_all();
  }

  // FlipSimulation::AddSolidCuboid, :316-324
  void AddSolidCuboid(const common::CoordBBox& box) {
    if (h_) check_(fsim_add_solid_cuboid(h_, box.lo.v, box.hi.v));
    else pending_solids_.push_back({box.lo, box.hi});
  }

  // Scene initialisation (:200-246): each call is one seeding pass.
  void InitializeMultipleWaterDrops(T height, const std::vector<common::Vec3<T>>& centers,
                                    const std::vector<T>& radii) {
    fsim_seed_pass p{};
    p.nshapes = 1 + int(centers.size());
    p.shapes[0].kind = FSIM_SHAPE_POOL;
    p.shapes[0].a[1] = float(height);
    for (size_t i = 0; i < centers.size(); ++i) {
      p.shapes[i + 1].kind = FSIM_SHAPE_SPHERE;
      for (int a = 0; a < 3; ++a) p.shapes[i + 1].a[a] = float(centers[i][a]);
      p.shapes[i + 1].r = float(radii[i]);
    }
    seed(p);
  }
  void InitializeWaterCuboid(const common::Cube<T>& box, const common::Vec3<T> velocity) {
    fsim_seed_pass p{};
    p.nshapes = 1;
    p.shapes[0].kind = FSIM_SHAPE_CUBOID;
    for (int a = 0; a < 3; ++a) {
      p.shapes[0].a[a] = float(box.start[a]);
      p.shapes[0].b[a] = float(box.end[a]);
      p.velocity[a] = float(velocity[a]);
    }
    seed(p);
  }
  void InitializeWaterSphere(const common::Vec3<T>& center, const T radius,
                             const common::Vec3<T> velocity) {
    fsim_seed_pass p{};
    p.nshapes = 1;
    p.shapes[0].kind = FSIM_SHAPE_SPHERE;
    for (int a = 0; a < 3; ++a) {
      p.shapes[0].a[a] = float(center[a]);
      p.velocity[a] = float(velocity[a]);
    }
    p.shapes[0].r = float(radius);
    seed(p);
  }
  // Runs all recorded seeding passes at once (per-cell counts carry across
  // passes as in the reference).  Called implicitly by the first stage.
  void FinishInitialization(uint64_t seed_value = 0) {
    if (passes_.empty()) return;
    check_(fsim_seed_fluid(h_, passes_.data(), int32_t(passes_.size()), seed_value));
    passes_.clear();
  }

  // stages
  T CFL() {
    ready();
    float inv = 0.f;
    check_(fsim_cfl(h_, &inv));
    return T(inv);
  }
  void MoveParticles(T dt, bool /*defragment*/) {
    ready();
    check_(fsim_move_particles(h_, float(dt)));
    invalidate();
  }
  void DeleteParticlesInSolids() {}  // done by MoveParticles on the device
  void ClearGridData() {
    ready();
    check_(fsim_clear_grid(h_));
    invalidate();
  }
  void TransferParticlesToGrid() { stage(fsim_transfer_particles_to_grid(h_)); }
  void ApplyBoundaryConditions() { stage(fsim_apply_boundary_conditions(h_)); }
  void SaveGridVelocities() { stage(fsim_save_grid_velocities(h_)); }
  void DeleteOutsideParticles() { stage(fsim_delete_outside_particles(h_)); }
  // water sources (common/flip_simulation.cc:327-329, 1207-1281); the source
  // is already scaled to index space (FlipDriver::Initialize)
  void AddWaterSource(const fsim_source& source) { stage(fsim_add_source(h_, &source)); }
  void AddContributionFromSources(T t) {
    stage(fsim_add_contribution_from_sources(h_, float(t)));
  }
  void DeleteFluidInSources(T t) { stage(fsim_delete_fluid_in_sources(h_, float(t))); }
  void ReinitializePhiSimple() { stage(fsim_reinitialize_phi(h_)); }
  void AddGravity(T dt) { stage(fsim_add_gravity(h_, float(dt))); }
  void ComputeDivergence() { stage(fsim_compute_divergence(h_)); }
  void UpdateVelocityFromPressure() { stage(fsim_update_velocity_from_pressure(h_)); }
  void GetVelocityUpdate() { stage(fsim_get_velocity_update(h_)); }
  void UpdateParticlesFromGrid() { stage(fsim_update_particles_from_grid(h_)); }
  // FlipSimulation::SaveDebugDataToFile, common/flip_simulation.cc:1295-1316:
  // into <output_dir>/debug, grid_velocity_%08d, grid_phi_%08d, particles_%08d
  // (text), then grid_velocity_%08d.txt and the pressure as grid_phi_%08d.txt
  // (the reference writes the pressure under the phi prefix).
  void SaveDebugDataToFile() {
    const std::string dir = output_dir_ + "/debug";
    mkdir(output_dir_.c_str(), 0755);
    mkdir(dir.c_str(), 0755);
    char step[16], step_txt[24];
    std::snprintf(step, sizeof(step), "%08d", debug_step_);
    std::snprintf(step_txt, sizeof(step_txt), "%08d.txt", debug_step_);
    if (grid_velocity_) grid_velocity_->Write(dir + "/grid_velocity_" + step);
    if (grid_phi_) grid_phi_->Write(dir + "/grid_phi_" + step);
    if (particles_) particles_->Write(dir + "/particles_" + step);
    if (grid_velocity_) grid_velocity_->Write(dir + "/grid_velocity_" + step_txt, true);
    if (grid_pressure_) grid_pressure_->Write(dir + "/grid_phi_" + step_txt);
    ++debug_step_;
  }
  // Binary particle frame particles_%08d (SaveDataToFile, :1273-1283).
  void SaveDataToFile() {
    char name[32];
    std::snprintf(name, sizeof(name), "particles_%08d", frame_);
    if (particles_) particles_->Write(output_dir_ + "/" + name, false);
  }
  void NextFrame() { ++frame_; }
  size_t FluidCellCount() {
    ScalarGridInt m;
    m.bind(handle(), -2, metagrid_.global_dims());
    return size_t(m.Count(common::CoordBBox(common::Coord(-1),
                                            common::Coord(metagrid_.global_dims()[0])),
                          common::FLUID));
  }
  size_t ParticleCount() {
    int64_t n = 0;
    check_(fsim_particle_count(handle(), &n));
    return size_t(n);
  }

  // Fused RunOneStep (common/flip_app_sim.cc:211-254) in one call.
  fsim_step_stats RunOneStepFused(T dt, const fsim_pcg_params& prm) {
    ready();
    fsim_step_stats st{};
    check_(fsim_step(h_, float(dt), &prm, &st));
    invalidate();
    return st;
  }

  fsim_t* handle() {
    ready();
    return h_;
  }

  // set_* / getters as in common/flip_simulation.h:264-345
  void set_grid_velocity(VectorGridT* g) { grid_velocity_ = g; bind_all(); }
  void set_grid_velocity_update(VectorGridT* g) { grid_velocity_update_ = g; bind_all(); }
  void set_grid_weight(VectorGridT* g) { grid_weight_ = g; bind_all(); }
  void set_grid_phi(ScalarGridT* g) { grid_phi_ = g; bind_all(); }
  void set_grid_divergence(ScalarGridT* g) { grid_divergence_ = g; bind_all(); }
  void set_grid_pressure(ScalarGridT* g) { grid_pressure_ = g; bind_all(); }
  void set_grid_marker(ScalarGridInt* g) { grid_marker_ = g; bind_all(); }
  void set_particles(ParticlesT* p) { particles_ = p; bind_all(); }
  VectorGridT* grid_velocity() { return grid_velocity_; }
  VectorGridT* grid_velocity_update() { return grid_velocity_update_; }
  VectorGridT* grid_weight() { return grid_weight_; }
  ScalarGridT* grid_phi() { return grid_phi_; }
  ScalarGridT* grid_divergence() { return grid_divergence_; }
  ScalarGridT* grid_pressure() { return grid_pressure_; }
  ScalarGridInt* grid_marker() { return grid_marker_; }
  ParticlesT* particles() { return particles_; }

 private:
  void check_(int rc) { common::check(h_, rc, "fsim"); }
  void seed(const fsim_seed_pass& p) { passes_.push_back(p); }
  void ready() {
    if (!h_) InitializeVariables();
    FinishInitialization();
  }
  void stage(int rc) {
    check_(rc);
    invalidate();
  }
  void invalidate() {
    FieldViewInvalidate(grid_velocity_);
    FieldViewInvalidate(grid_velocity_update_);
    FieldViewInvalidate(grid_weight_);
    FieldViewInvalidate(grid_phi_);
    FieldViewInvalidate(grid_divergence_);
    FieldViewInvalidate(grid_pressure_);
    FieldViewInvalidate(grid_marker_);
  }
  template <typename G>
  static void FieldViewInvalidate(G* g) {
    if (g) g->invalidate();
  }
  void bind_all() {
    if (!h_) return;
    const common::Coord d = metagrid_.global_dims();
    if (grid_velocity_) grid_velocity_->bind(h_, FSIM_FIELD_VELOCITY, d);
    if (grid_velocity_update_) grid_velocity_update_->bind(h_, FSIM_FIELD_VELOCITY_UPDATE, d);
    if (grid_weight_) grid_weight_->bind(h_, FSIM_FIELD_WEIGHT, d);
    if (grid_phi_) grid_phi_->bind(h_, FSIM_FIELD_PHI, d);
    if (grid_divergence_) grid_divergence_->bind(h_, FSIM_FIELD_DIVERGENCE, d);
    if (grid_pressure_) grid_pressure_->bind(h_, FSIM_FIELD_PRESSURE, d);
    if (grid_marker_) grid_marker_->bind(h_, -2, d);
    if (particles_) particles_->bind(h_, metagrid_);
  }

  common::MetaGrid metagrid_;
  int nppc_ = 8;
  T gravity_ = T(9.8);
  T flip_ = T(1);
  common::Vec3<T> force_ = common::Vec3<T>(T(0), T(1), T(0));
  int boundary_ = FSIM_BOUNDARY_BOX;
  int device_ = 0;
  int frame_ = 0;
  int debug_step_ = 0;
  bool debug_ = false;
  std::string output_dir_;
  fsim_t* h_ = nullptr;
  std::vector<fsim_seed_pass> passes_;
  std::vector<std::pair<common::Coord, common::Coord>> pending_solids_;
  VectorGridT* grid_velocity_ = nullptr;
  VectorGridT* grid_velocity_update_ = nullptr;
  VectorGridT* grid_weight_ = nullptr;
  ScalarGridT* grid_phi_ = nullptr;
  ScalarGridT* grid_divergence_ = nullptr;
  ScalarGridT* grid_pressure_ = nullptr;
  ScalarGridInt* grid_marker_ = nullptr;
  ParticlesT* particles_ = nullptr;
};

}  // namespace application
