// fsim_internal.cuh -- device layout and shared helpers of the FLIP step.
//
// HBM layout (one handle = one domain of N0 x N1 x N2 cells):
//  * Particles: 9 SoA float arrays (pos xyz, vel xyz, gvel xyz), double
//    buffered for the rebinning gather, plus a 32-bit cell key per particle.
//    Live particles are kept sorted by key, which is the OpenVDB Tree3<T,3,3>
//    iteration order of their cell (root 64^3 blocks lexicographic, then
//    x-major 8^3 leaves, then x-major voxels), so the array order equals the
//    reference's particle iteration order (common/particles.cc:479-546).
//  * Leaves: a dense table over every 8^3 leaf of the padded domain, indexed
//    by the OpenVDB-order leaf id, maps to a compact slot.  Slots
//    [0, n_pleaf) are the leaves holding particles (in iteration order);
//    slots [n_pleaf, n_gleaf) are the leaves within one leaf of them (they
//    hold P2G halo faces, wall markers and ghost velocities).  Each slot has
//    a 27-entry neighbour table (dx,dy,dz in -1..1, index (dx+1)*9+(dy+1)*3
//    +(dz+1); -1 = absent) and, for particle leaves, 512 per-cell particle
//    ranges and one per-leaf range.
//  * Grid fields are stored per slot as 512 voxels (offset x*64+y*8+z):
//    velocity / saved velocity / weight as three 512-float planes per slot,
//    active bits as 16 words per slot, the marker as one byte per voxel,
//    and the PCG vectors (divergence, pressure, r, p, flags; w and s of
//    the single-reduction iteration) per particle-leaf slot.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/fsim.h"

namespace fsim {

constexpr uint32_t kDeadKey = 0xFFFFFFFFu;
constexpr int kMaxCuboids = 32;
constexpr int kLeafVox = 512;

// Static solid description: box/tank walls plus inclusive integer cuboids
// (intersected with [-1,N]^3 as AddSolidCuboid does).
struct SolidDesc {
  int n[3];
  int boundary;
  int ncub;
  int lo[kMaxCuboids][3];
  int hi[kMaxCuboids][3];
};

// Leaf-id mapping (OpenVDB order) for a domain.
struct LeafMap {
  int n[3];     // cells per axis
  int lmax[3];  // max leaf coord: floor(n/8); min is -1
  int R[3];     // 64^3-block counts: floor(lmax/8)+2
  uint32_t dense;  // R0*R1*R2*512
};

__host__ __device__ inline int fdiv(int a, int b) {
  return (a >= 0) ? a / b : -((-a + b - 1) / b);
}

__host__ __device__ inline uint32_t leaf_id(const LeafMap& m, int lx, int ly, int lz) {
  int bx = fdiv(lx, 8) + 1, by = fdiv(ly, 8) + 1, bz = fdiv(lz, 8) + 1;
  uint32_t blk = (uint32_t(bx) * m.R[1] + uint32_t(by)) * m.R[2] + uint32_t(bz);
  return blk * 512u + uint32_t(((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7));
}

__host__ __device__ inline void leaf_coords(const LeafMap& m, uint32_t id, int& lx, int& ly,
                                            int& lz) {
  uint32_t o = id & 511u, blk = id >> 9;
  int bz = int(blk % m.R[2]);
  int by = int((blk / m.R[2]) % m.R[1]);
  int bx = int(blk / (uint32_t(m.R[1]) * m.R[2]));
  lx = (bx - 1) * 8 + int(o >> 6);
  ly = (by - 1) * 8 + int((o >> 3) & 7);
  lz = (bz - 1) * 8 + int(o & 7);
}

__host__ __device__ inline bool leaf_valid(const LeafMap& m, int lx, int ly, int lz) {
  return lx >= -1 && ly >= -1 && lz >= -1 && lx <= m.lmax[0] && ly <= m.lmax[1] &&
         lz <= m.lmax[2];
}

__host__ __device__ inline uint32_t cell_key(const LeafMap& m, int i, int j, int k) {
  return leaf_id(m, fdiv(i, 8), fdiv(j, 8), fdiv(k, 8)) * 512u +
         uint32_t(((i & 7) << 6) | ((j & 7) << 3) | (k & 7));
}

__host__ __device__ inline int key_bits(const LeafMap& m) {
  // smallest b with 2^b > max key + 1, so the dead key (all ones in the
  // sorted bits) orders after every live key
  uint64_t mx = uint64_t(m.dense) * 512ull;
  int b = 0;
  while ((1ull << b) <= mx) ++b;
  return b;
}

// grid_solid_->get(i,j,k) of the reference: walls of SetBoxBoundary /
// SetTankBoundary plus AddSolidCuboid boxes, all within [-1,N]^3.
__host__ __device__ inline bool is_solid(const SolidDesc& s, int i, int j, int k) {
  const int* n = s.n;
  if (i < -1 || j < -1 || k < -1 || i > n[0] || j > n[1] || k > n[2]) return false;
  if (i == -1 || i == n[0] || k == -1 || k == n[2] || j == -1) return true;
  if (j == n[1] && s.boundary == FSIM_BOUNDARY_BOX) return true;
  for (int c = 0; c < s.ncub; ++c)
    if (i >= s.lo[c][0] && i <= s.hi[c][0] && j >= s.lo[c][1] && j <= s.hi[c][1] &&
        k >= s.lo[c][2] && k <= s.hi[c][2])
      return true;
  return false;
}

// Source node of ExtrapolateToBoundary's six ordered passes
// (common/vector_grid.cc:302-381) for component D at node c: the ghost
// layers -1 and N of the two tangential axes take the tangential components
// of the adjacent inner layer; the pass order (x, y, z) decides the edges.
__host__ __device__ inline void ghost_source(const int n[3], int D, const int c[3], int src[3]) {
  src[0] = c[0]; src[1] = c[1]; src[2] = c[2];
  const int i = c[D];
  if (i < 0 || i > n[D]) return;
  const int a = (D == 0) ? 1 : 0;
  const int b = (D == 2) ? 1 : 2;
  const int ta = c[a], tb = c[b];
  const bool ga = (ta == -1 || ta == n[a]), gb = (tb == -1 || tb == n[b]);
  const bool ra = (ta >= 0 && ta <= n[a]), rb = (tb >= 0 && tb <= n[b]);
  auto sr = [](int t, int nn) { return t == -1 ? 0 : (t == nn ? nn - 1 : t); };
  if (gb && ra) {
    src[a] = sr(ta, n[a]);
    src[b] = sr(tb, n[b]);
  } else if (ga && rb) {
    src[a] = sr(ta, n[a]);
  }
}

// Voxels activated by ExtrapolateToBoundary (any pass).
__host__ __device__ inline bool extrap_activated(const int n[3], int i, int j, int k) {
  const bool ri = i >= 0 && i <= n[0], rj = j >= 0 && j <= n[1], rk = k >= 0 && k <= n[2];
  const bool gi = i == -1 || i == n[0], gj = j == -1 || j == n[1], gk = k == -1 || k == n[2];
  return (gi && rj && rk) || (gj && ri && rk) || (gk && ri && rj);
}

// PCG flags byte per cell: bit0 FLUID, bits1..3 diag (# non-solid neighbours).
__host__ __device__ inline int flag_diag(uint8_t f) { return (f >> 1) & 7; }

// State handed from one hot PCG kernel to the next (see k_pcg.cu): the
// residual dots and beta when they are given (after setup or a residual
// replacement) instead of summed from the previous kernel's partials.  The
// single-reduction loop keeps gamma_{i-1} in rz_prev and alpha_{i-1} in alpha.
struct PcgIterState {
  double rr, rz, beta, rz_prev, alpha;
  int iter, done, status, given;
};

// Device scalar block of one PCG solve (16-byte multiple: the hot kernels
// copy it to shared memory in 16-byte pieces).
struct alignas(16) PcgScalars {
  double rz, rz_old, rr, pAp, bb, alpha, beta, rr0;
  int iter, done, status, max_iter;
  int mode, fp32;  // FSIM_PCG_* ; fp32 != 0: scalars are rounded to float
  double thr;      // ABSOLUTE: r.r threshold; RELATIVE: set to tol2*bb
  double tol2;     // RELATIVE: tolerance squared
  double tol2_outer;  // MIXED: outer tolerance squared; a segment never stops below tol2_outer*bb
  unsigned int cnt_s, cnt_r;
  unsigned long long n_rows;  // FLUID cells (unknowns), counted by setup
  // bulk-copy spmv: FSIM_ERR_TIMEOUT when a bounded stage wait gave up (0: none);
  // resident loop: grid-barrier arrivals and its timeout flag
  unsigned int wait_err, bar_count, bar_err, wait_pad;
  // hot-loop hand-off: [0] spmv -> update, [1] update -> spmv (and setup /
  // residual replacement -> spmv)
  PcgIterState st[2];
};

struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
};

struct KernelStat {
  const char* name;
  double ms;
  int64_t launches;
};

}  // namespace fsim

struct fsim_sim {
  fsim_config cfg;
  fsim::SolidDesc solid;
  fsim::LeafMap lm;
  int dev = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  // P2G pass 1 output (k_grid.cu): per particle leaf the 10^3 node block
  unsigned long long* p2g_nodes = nullptr;
  uint32_t* p2g_touch = nullptr;
  uint32_t* p2g_low = nullptr;  // [0] count, then the low-weight faces of P2G pass 2
  int64_t p2g_low_cap = 0;
  int64_t p2g_cap = 0;
  // fsim_step_host: a second stream for the copies that overlap the step
  cudaStream_t io_stream = nullptr;
  cudaEvent_t ev_main = nullptr, ev_io = nullptr;
  // around the PCG iteration loops (fsim_pcg_stats::loop_ms)
  cudaEvent_t ev_loop[2] = {nullptr, nullptr};
  double pcg_loop_ms = 0.0;
  float* io_stage = nullptr;   // AoS staging of the early position download
  int64_t io_stage_cap = 0;
  bool io_vel_pending = false; // vel upload in flight on io_stream (ev_io)
  // fsim_step: the rebinning gather moves pos and vel only; G2P rewrites
  // gvel for every live particle before anything reads it again
  bool gather_skip_gvel = false;
  // graph-loop pass length: the longest graph-loop segment of the previous
  // solve (a MIXED solve runs several; its last one is often short), and the
  // longest of the solve in progress
  int pcg_last_iters = 0;
  int pcg_seg_max = 0;
  float* io_early_pos = nullptr;  // host destination of the early position download
  int64_t io_early_cap = 0;
  int64_t io_early_n = -1;     // particles the early download copied (-1: none)
  std::string err;
  int64_t launches = 0;

  // particles
  int64_t cap_p = 0;
  int64_t n_total = 0;  // particles in the arrays (live + dead tail)
  int64_t n_live = 0;   // sorted prefix with a live key (may include
                        // particles deleted by DeleteOutsideParticles)
  int cur = 0;          // which particle buffer is current
  float* part[2] = {nullptr, nullptr};  // 9 * cap_p floats each
  uint32_t* keys[2] = {nullptr, nullptr};
  uint32_t* vals[2] = {nullptr, nullptr};
  void* sort_tmp = nullptr;
  size_t sort_tmp_bytes = 0;

  // topology
  uint8_t* d_flag = nullptr;     // dense
  int32_t* d_slot = nullptr;     // dense -> slot
  uint64_t* d_scan = nullptr;    // dense scan buffer
  void* scan_tmp = nullptr;
  size_t scan_tmp_bytes = 0;
  int32_t* d_leaf_id = nullptr;  // slot -> dense id (capacity = dense)
  int32_t* d_nbr = nullptr;      // slot*27
  int64_t cap_leaf = 0;          // field capacity (slots)
  int64_t cap_pleaf = 0;         // particle-leaf capacity
  uint2* d_cell_range = nullptr; // pleaf*512
  uint2* d_leaf_range = nullptr; // pleaf
  int n_pleaf = 0, n_gleaf = 0;
  bool have_topology = false;

  // grid fields (per slot)
  float* vel = nullptr;     // slot*1536
  float* vold = nullptr;    // slot*1536
  float* weight = nullptr;  // slot*1536
  uint32_t* vel_on = nullptr;   // slot*16
  uint32_t* vold_on = nullptr;  // slot*16
  int8_t* marker = nullptr;     // slot*512
  // pcg (per particle-leaf slot)
  float* div = nullptr;   // b
  float* pres = nullptr;  // x
  float* r = nullptr;
  float* p[2] = {nullptr, nullptr};
  // single-reduction CG: w = A M r and s = A p, each double-buffered
  float* cgw[2] = {nullptr, nullptr};
  float* cgs[2] = {nullptr, nullptr};
  uint8_t* flags = nullptr;
  // z-face planes per particle leaf (z=0 and z=7, 64 cells each, x*8+y):
  // [r | p_a | p_b] planes and the flags planes, so that a leaf's -z / +z
  // neighbour cells are read contiguously (in the cell layout x*64+y*8+z a
  // z face is 64 scattered cells)
  float* zface = nullptr;     // pleaf * 384
  double* zface64 = nullptr;  // pleaf * 384 (FP64 mode)
  uint8_t* zflags = nullptr;  // pleaf * 128
  double* x64 = nullptr;  // mixed / fp64 solution
  double* r64 = nullptr;  // fp64 mode vectors
  double* p64[2] = {nullptr, nullptr};
  double* Ap64 = nullptr;
  double* b64 = nullptr;
  fsim::PcgScalars* d_sc = nullptr;
  double* d_part = nullptr;  // block partials (3 * max_blocks)
  float* d_partf = nullptr;  // fp32 / double-float partials of the hot PCG kernels (16 * max_blocks)
  int max_blocks = 0;

  // misc device scalars: [0] n_live [1] n_pleaf [2] n_gleaf [3] invalid
  // [4] vmax bits [5] seed count
  int64_t* d_cnt = nullptr;
  int64_t* h_cnt = nullptr;  // pinned
  fsim::PcgScalars* h_sc = nullptr;  // pinned

  // grid state flags (which reference stages have run since ClearGridData)
  bool grid_valid = false;
  bool bc_applied = false;
  bool saved = false;
  bool div_valid = false;
  bool pres_valid = false;
  bool phi_valid = false;
  bool extrapolated = false;
  bool weight_valid = false;
  bool deleted_outside = false;

  // PCG iterations as a CUDA graph with a conditional WHILE node
  bool use_graphs = true;
  // its kernel nodes joined by programmatic (early-launch) edges
  bool use_pdl = true;
  // z-face neighbours of the pipelined kernels: -1 by system size, 0 planes,
  // 1 direct reads (FSIM_PCG_ZDIRECT)
  int zdirect = -1;
  // bulk-copy staged spmv (FSIM_PCG_TMA=1; measured slower, opt-in); tests
  // only: the next solve withholds one stage's flags copy until the stage's
  // bounded wait has given up (FSIM_PCG_TMA_WITHHOLD=1)
  int tma_spmv = 0;
  int tma_withhold = 0;
  // FSIM_PCG_RES_WITHHOLD=1 (tests): in the first solve CTA 0 of the resident
  // loop skips its first barrier arrival, so that every CTA's bounded wait
  // gives up
  int res_withhold = 0;
  // register-pipelined hot kernels (next half leaf loaded during the
  // current; fp32 vectors only: 2% faster per iteration at 256^3)
  bool use_pipe = true;
  // fp32 solves by the single-reduction (Chronopoulos-Gear) iteration, one
  // kernel per iteration (FSIM_PCG_CG1=1; opt-in)
  int pcg_cg1 = 0;
  // fp32 solves by the resident loop (one persistent CTA per SM holding r, p
  // and the flags on chip): -1 by system size, 0 never, 1 wherever it fits
  // (FSIM_PCG_RES)
  int pcg_res = -1;

  // water sources and the time they see
  std::vector<fsim_source> sources;
  double time = 0.0;
  uint64_t seed = 0;         // of the last seeding (source draws use it)
  int64_t source_calls = 0;  // AddContributionFromSources calls (draw stream)
  // the next sort orders by (new key, old key): particles were appended
  // after the sorted array (source particles)
  bool composite_sort = false;
  // regions whose particles the next advection deletes (DeleteFluidInSources)
  bool delete_in_sources = false;
  float src_time = 0.f;
  uint64_t* keys64[2] = {nullptr, nullptr};
  int64_t cap64 = 0;
  void* src_tmp = nullptr;   // source draw counts and offsets
  size_t src_tmp_bytes = 0;

  // profiling
  bool profiling = false;
  std::vector<fsim::KernelStat> kstats;
  struct Pending {
    int stat;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> ev_pool;

  fsim::DevMem dense_tmp;  // dense download staging
};

// ---- host helpers shared by the translation units ------------------------
namespace fsim {

int fail(fsim_sim* s, int code, const std::string& msg);
extern thread_local std::string g_scene_err;  // last fsim_scene_parse error
int cuda_fail(fsim_sim* s, cudaError_t e, const char* what);

struct ProfScope {
  fsim_sim* s;
  int idx = -1;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(fsim_sim* sim, const char* name);
  ~ProfScope();
};

int ensure_leaf_capacity(fsim_sim* s, int64_t n_gleaf, int64_t n_pleaf);
// particle arrays for at least n particles (the current ones are kept)
int grow_particle_capacity(fsim_sim* s, int64_t n);
int rebuild_topology(fsim_sim* s);  // from keys[cur]/vals, n_total
// the topology part, keys[0]/vals[0] sorted; gather: permute the particles by vals[0]
int rebuild_after_sort(fsim_sim* s, bool gather = true);
// upload: rebin the particles whose keys are in keys[1] (sort skipped when sorted)
int rebin_uploaded(fsim_sim* s, int64_t* invalid);

// kernel entry points implemented in the .cu files
int launch_keys_from_positions(fsim_sim* s, int mode, float dt);
int launch_p2g(fsim_sim* s, bool fused, float dt);
int launch_apply_bc(fsim_sim* s);
int launch_save_velocities(fsim_sim* s);
int launch_add_gravity(fsim_sim* s, float dt);
int launch_delete_outside(fsim_sim* s);
int launch_divergence(fsim_sim* s);
int launch_pressure_update(fsim_sim* s, bool fused);
int launch_velocity_update(fsim_sim* s);
int launch_cfl(fsim_sim* s);
int launch_g2p(fsim_sim* s);
// b64: an fp64 right-hand side on the particle-leaf cells instead of the
// divergence (the solution is then read from x64: FP64 / MIXED precision)
int pcg_solve(fsim_sim* s, const fsim_pcg_params* prm, fsim_pcg_stats* st,
              const double* b64 = nullptr);
int download_dense(fsim_sim* s, int field, float* out, uint8_t* active);
int download_marker(fsim_sim* s, int32_t* out, uint8_t* active);
int seed_fluid(fsim_sim* s, const fsim_seed_pass* passes, int npasses, uint64_t seed);
// AddContributionFromSources(t): appends the active sources' particles
int add_source_particles(fsim_sim* s, float t);
// DeleteFluidInSources(t) on the current (sorted) particles: dead keys
int delete_in_sources(fsim_sim* s, float t);
// get_box(t) / get_velocity(t) / is_active(t) of Source<T> (host)
void source_box(const fsim_source& src, float t, float lo[3], float hi[3]);
void source_velocity(const fsim_source& src, float t, float v[3]);
bool source_active(const fsim_source& src, float t);
int perturb(fsim_sim* s, float sigma, uint64_t seed);

}  // namespace fsim

#define FSIM_CK(s, call)                                   \
  do {                                                     \
    cudaError_t _e = (call);                               \
    if (_e != cudaSuccess) return fsim::cuda_fail(s, _e, #call); \
  } while (0)

#define FSIM_LAUNCH(s, name, kernel, grid, block, smem, ...)              \
  do {                                                                    \
    if ((grid) > 0) {                                                     \
      fsim::ProfScope _ps(s, name);                                       \
      kernel<<<(grid), (block), (smem), (s)->stream>>>(__VA_ARGS__);      \
      (s)->launches++;                                                    \
      cudaError_t _e = cudaGetLastError();                                \
      if (_e != cudaSuccess) return fsim::cuda_fail(s, _e, name);         \
    }                                                                     \
  } while (0)
