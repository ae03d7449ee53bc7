// oracle.cc -- CPU restatement of the reference FLIP step (TEST INFRASTRUCTURE).
//
// Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg.  Built strict: -O2 -ffp-contract=off, no fast-math.  One thread by
// default; orc_set_threads spreads the loops whose results do not depend on
// the thread count over a pool (see Pool below).
// Every function cites the reference code it restates (paths relative to the
// schinmayee/fluid-sim-lb project).  Parity status: unpinned against the
// reference binary (it cannot be built here); pinned by known-answer tests.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace {

enum { AIR = 0, FLUID = 1, SOLID = 2 };

inline int floor_div(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }

// ---- host threads -----------------------------------------------------------
// A pool for loops whose iterations write disjoint elements (per particle,
// per leaf, per matrix row, per vector entry), for the chunk sums of the
// PCG dots, whose chunk totals are then added in chunk order, and for the
// four lane sums of p.Ap.  Every result is therefore bit-identical for any
// thread count; the P2G leaf write-back, whose order spans the whole grid,
// stays serial.  bench.py's reference arm uses it; the tests run one thread.
class Pool {
 public:
  ~Pool() { resize(1); }
  int size() const { return nthreads_; }
  void resize(int n) {
    n = std::max(1, std::min(n, 256));
    if (n == nthreads_) return;
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
    workers_.clear();
    stop_ = false;
    nthreads_ = n;
    const uint64_t g0 = gen_;
    for (int w = 1; w < n; ++w) workers_.emplace_back([this, w, g0] { loop(w, g0); });
  }
  // job(t) for t in [0, size()): thread 0 is the caller
  void run(const std::function<void(int)>& job) {
    if (nthreads_ == 1) { job(0); return; }
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &job;
      pending_ = nthreads_ - 1;
      ++gen_;
    }
    cv_.notify_all();
    job(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [this] { return pending_ == 0; });
    job_ = nullptr;
  }

 private:
  void loop(int w, uint64_t seen) {
    for (;;) {
      const std::function<void(int)>* job;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        job = job_;
      }
      (*job)(w);
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_cv_.notify_one();
    }
  }
  int nthreads_ = 1;
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  uint64_t gen_ = 0;
  int pending_ = 0;
  bool stop_ = false;
};
Pool g_pool;

// f(begin, end) over contiguous ranges of [0, n), one per pool thread.
template <class F>
void par_for(size_t n, F&& f) {
  const int T = g_pool.size();
  if (T == 1 || n < 4096) { f(size_t(0), n); return; }
  g_pool.run([&](int t) {
    const size_t b = n * size_t(t) / size_t(T), e = n * size_t(t + 1) / size_t(T);
    if (b < e) f(b, e);
  });
}

// ---- seeding draw: SplitMix64 finaliser (Steele, Lea, Flood 2014) ----------
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
inline float uniform01(uint64_t seed, int pass, int64_t cell, int draw, int d) {
  uint64_t s = mix64(seed ^ mix64((uint64_t(uint32_t(pass)) << 40) ^ uint64_t(cell)));
  uint64_t z = mix64(s + uint64_t(draw * 3 + d));
  return float(z >> 40) * (1.0f / 16777216.0f);
}

struct Dims {
  int n[3];
  int s[3];  // n + 4: voxels [-2, n+1]
  size_t total;
  void init(const int32_t d[3]) {
    for (int a = 0; a < 3; ++a) { n[a] = d[a]; s[a] = d[a] + 4; }
    total = size_t(s[0]) * s[1] * s[2];
  }
  bool in(int i, int j, int k) const {
    return i >= -2 && j >= -2 && k >= -2 && i <= n[0] + 1 && j <= n[1] + 1 && k <= n[2] + 1;
  }
  size_t idx(int i, int j, int k) const {
    return (size_t(i + 2) * s[1] + size_t(j + 2)) * s[2] + size_t(k + 2);
  }
};

struct Vec3f { float v[3]; };

// OpenVDB Tree3<T,3,3> iteration key of a voxel (root 64^3 blocks sorted
// lexicographically, then x-major 8^3 leaves, then x-major voxels).
struct KeyMap {
  int R[3];
  void init(const int n[3]) {
    for (int a = 0; a < 3; ++a) R[a] = floor_div(floor_div(n[a], 8), 8) + 2;
  }
  uint32_t leaf_id(int lx, int ly, int lz) const {
    int bx = floor_div(lx, 8) + 1, by = floor_div(ly, 8) + 1, bz = floor_div(lz, 8) + 1;
    uint32_t blk = (uint32_t(bx) * R[1] + uint32_t(by)) * R[2] + uint32_t(bz);
    return blk * 512u + uint32_t(((lx & 7) << 6) | ((ly & 7) << 3) | (lz & 7));
  }
  uint32_t key(int i, int j, int k) const {
    uint32_t l = leaf_id(floor_div(i, 8), floor_div(j, 8), floor_div(k, 8));
    return l * 512u + uint32_t(((i & 7) << 6) | ((j & 7) << 3) | (k & 7));
  }
};

struct Cuboid { int lo[3], hi[3]; };

}  // namespace

struct orc_sim {
  Dims D;
  KeyMap K;
  int boundary;
  float gravity;
  float fx, fy, fz;
  float flip;
  int nppc;
  std::vector<Cuboid> cuboids;
  std::vector<uint8_t> solid;  // value 1 active / 0 background

  // grids
  std::vector<float> vel, vold, weight;  // 3 per voxel
  std::vector<uint8_t> vel_on, vold_on, weight_on;
  std::vector<int8_t> marker;
  std::vector<uint8_t> marker_on;
  std::vector<float> div, pres;
  std::vector<uint8_t> div_on, pres_on, phi_on;
  std::vector<double> pres64;

  // particles in iteration order
  std::vector<float> pos, vel_p, gvel;
  std::vector<uint32_t> keys;
  std::vector<int32_t> cell;  // 3 per particle

  // water sources and the driver's advanced time
  std::vector<orc_source> sources;
  double time = 0.0;
  uint64_t seed = 0;          // of the last seeding (source draws use it)
  int64_t source_calls = 0;   // draw stream of AddContributionFromSources
};

namespace {

// ---- helpers emulating ScalarGrid/VectorGrid accessors -------------------
inline Vec3f vget(const orc_sim* s, const std::vector<float>& f,
                  const std::vector<uint8_t>& on, int i, int j, int k) {
  Vec3f r{{0.f, 0.f, 0.f}};
  if (!s->D.in(i, j, k)) return r;
  size_t x = s->D.idx(i, j, k);
  if (!on[x]) return r;
  r.v[0] = f[3 * x]; r.v[1] = f[3 * x + 1]; r.v[2] = f[3 * x + 2];
  return r;
}
inline void vset(orc_sim* s, std::vector<float>& f, std::vector<uint8_t>& on,
                 int i, int j, int k, const Vec3f& v) {
  if (!s->D.in(i, j, k)) return;  // never reached by the restated loops
  size_t x = s->D.idx(i, j, k);
  on[x] = 1;
  f[3 * x] = v.v[0]; f[3 * x + 1] = v.v[1]; f[3 * x + 2] = v.v[2];
}
inline bool von(const orc_sim* s, const std::vector<uint8_t>& on, int i, int j, int k) {
  return s->D.in(i, j, k) && on[s->D.idx(i, j, k)];
}
inline int mget(const orc_sim* s, int i, int j, int k) {
  if (!s->D.in(i, j, k)) return AIR;
  size_t x = s->D.idx(i, j, k);
  return s->marker_on[x] ? s->marker[x] : AIR;
}
inline void mset(orc_sim* s, int i, int j, int k, int v) {
  size_t x = s->D.idx(i, j, k);
  s->marker_on[x] = 1;
  s->marker[x] = int8_t(v);
}
inline int sget(const orc_sim* s, int i, int j, int k) {
  if (!s->D.in(i, j, k)) return 0;
  return s->solid[s->D.idx(i, j, k)];
}
inline float fget(const orc_sim* s, const std::vector<float>& f,
                  const std::vector<uint8_t>& on, int i, int j, int k) {
  if (!s->D.in(i, j, k)) return 0.f;
  size_t x = s->D.idx(i, j, k);
  return on[x] ? f[x] : 0.f;
}

void build_walls(orc_sim* s) {
  // SetBoxBoundary / SetTankBoundary, common/flip_simulation.cc:256-308,332-377
  const int* n = s->D.n;
  auto put = [&](int i, int j, int k) { s->solid[s->D.idx(i, j, k)] = 1; };
  for (int j = -1; j <= n[1]; ++j)
    for (int k = -1; k <= n[2]; ++k) { put(-1, j, k); put(n[0], j, k); }
  for (int i = -1; i <= n[0]; ++i)
    for (int k = -1; k <= n[2]; ++k) {
      put(i, -1, k);
      if (s->boundary == 0) put(i, n[1], k);
    }
  for (int i = -1; i <= n[0]; ++i)
    for (int j = -1; j <= n[1]; ++j) { put(i, j, -1); put(i, j, n[2]); }
}

// ---- particle ordering ---------------------------------------------------
// Stable LSD radix sort by key: the rebuilt per-cell lists of StepInGrid
// (common/particles.cc:512-545) keep particles in the order they were
// visited, i.e. a stable sort by the new cell's iteration key.
void reorder_by_key(orc_sim* s) {
  const size_t n = s->keys.size();
  std::vector<uint32_t> idx(n), tmp(n), kin(s->keys), kout(n);
  for (size_t i = 0; i < n; ++i) idx[i] = uint32_t(i);
  // each pool thread counts and scatters one contiguous block; block t's
  // entries of a bucket go after blocks 0..t-1's, so every pass is stable
  const int T = n < 65536 ? 1 : g_pool.size();
  std::vector<size_t> cnt(size_t(T) * 256);
  for (int shift = 0; shift < 32; shift += 8) {
    std::fill(cnt.begin(), cnt.end(), size_t(0));
    auto block = [&](int t, size_t& b, size_t& e) {
      b = n * size_t(t) / size_t(T);
      e = n * size_t(t + 1) / size_t(T);
    };
    auto count = [&](int t) {
      size_t b, e;
      block(t, b, e);
      size_t* c = &cnt[size_t(t) * 256];
      for (size_t i = b; i < e; ++i) c[(kin[i] >> shift) & 255u]++;
    };
    if (T == 1) count(0); else g_pool.run(count);
    size_t run = 0;
    for (int d = 0; d < 256; ++d)
      for (int t = 0; t < T; ++t) {
        const size_t c = cnt[size_t(t) * 256 + d];
        cnt[size_t(t) * 256 + d] = run;
        run += c;
      }
    auto scatter = [&](int t) {
      size_t b, e;
      block(t, b, e);
      size_t* c = &cnt[size_t(t) * 256];
      for (size_t i = b; i < e; ++i) {
        const size_t d = c[(kin[i] >> shift) & 255u]++;
        kout[d] = kin[i];
        tmp[d] = idx[i];
      }
    };
    if (T == 1) scatter(0); else g_pool.run(scatter);
    kin.swap(kout);
    idx.swap(tmp);
  }
  std::vector<float> p2(3 * n), v2(3 * n), g2(3 * n);
  std::vector<int32_t> c2(3 * n);
  par_for(n, [&](size_t i0, size_t i1) {
    for (size_t i = i0; i < i1; ++i) {
      size_t o = idx[i];
      for (int d = 0; d < 3; ++d) {
        p2[3 * i + d] = s->pos[3 * o + d];
        v2[3 * i + d] = s->vel_p[3 * o + d];
        g2[3 * i + d] = s->gvel[3 * o + d];
        c2[3 * i + d] = s->cell[3 * o + d];
      }
    }
  });
  s->pos.swap(p2); s->vel_p.swap(v2); s->gvel.swap(g2); s->cell.swap(c2);
  s->keys.swap(kin);
}

void erase_where(orc_sim* s, const std::vector<uint8_t>& kill) {
  size_t w = 0, n = s->keys.size();
  for (size_t i = 0; i < n; ++i) {
    if (kill[i]) continue;
    for (int d = 0; d < 3; ++d) {
      s->pos[3 * w + d] = s->pos[3 * i + d];
      s->vel_p[3 * w + d] = s->vel_p[3 * i + d];
      s->gvel[3 * w + d] = s->gvel[3 * i + d];
      s->cell[3 * w + d] = s->cell[3 * i + d];
    }
    s->keys[w] = s->keys[i];
    ++w;
  }
  s->pos.resize(3 * w); s->vel_p.resize(3 * w); s->gvel.resize(3 * w);
  s->cell.resize(3 * w); s->keys.resize(w);
}

// Leaf ranges over the sorted particle array: [begin, end) per leaf.
void leaf_ranges(const orc_sim* s, std::vector<size_t>& starts) {
  starts.clear();
  const size_t n = s->keys.size();
  for (size_t i = 0; i < n; ++i)
    if (i == 0 || (s->keys[i] >> 9) != (s->keys[i - 1] >> 9)) starts.push_back(i);
  starts.push_back(n);
}

// ---- P2G weights (FlipSimulation::ScatterWeight<D>, flip_simulation.cc:927-1009)
// Returns the lower node (relative offsets) and the 8 weights [di][dj][dk].
inline void scatter_weights(const float* p, const int* c, int D, int start[3],
                            float w[2][2][2]) {
  float lo[3] = {float(c[0]), float(c[1]), float(c[2])};
  start[0] = c[0]; start[1] = c[1]; start[2] = c[2];
  for (int a = 0; a < 3; ++a) {
    if (a == D) continue;
    lo[a] = lo[a] + 0.5f;
    if (p[a] < lo[a]) { lo[a] = lo[a] - 1.0f; start[a] -= 1; }
  }
  float x = p[0] - lo[0], y = p[1] - lo[1], z = p[2] - lo[2];
  float xy = x * y, yz = y * z, xz = z * x, xyz = xy * z;
  w[1][1][1] = xyz;
  w[1][1][0] = xy - xyz;
  w[1][0][1] = xz - xyz;
  w[1][0][0] = (x - xz) - w[1][1][0];
  w[0][1][1] = yz - xyz;
  w[0][1][0] = (y - yz) - w[1][1][0];
  w[0][0][1] = (z - yz) - w[1][0][1];
  w[0][0][0] = (((1.0f - x) - y) + xy) - w[0][0][1];
}

// FlipSimulation::InterpolateComponent<D>, flip_simulation.cc:1095-1166
inline float interp_component(const float* p, const int* c, int D,
                              const float* buf /*10^3 for component D*/,
                              const int lc[3]) {
  float lo[3] = {float(c[0]), float(c[1]), float(c[2])};
  int st[3] = {lc[0], lc[1], lc[2]};
  for (int a = 0; a < 3; ++a) {
    if (a == D) continue;
    lo[a] = lo[a] + 0.5f;
    if (p[a] < lo[a]) { lo[a] = lo[a] - 1.0f; st[a] -= 1; }
  }
  const int i = st[0], j = st[1], k = st[2];
  float w[3] = {p[0] - lo[0], p[1] - lo[1], p[2] - lo[2]};
  auto B = [&](int a, int b, int cc) { return buf[(a * 10 + b) * 10 + cc]; };
  const float v000 = B(i, j, k), v001 = B(i, j, k + 1);
  const float v010 = B(i, j + 1, k), v011 = B(i, j + 1, k + 1);
  const float v100 = B(i + 1, j, k), v101 = B(i + 1, j, k + 1);
  const float v110 = B(i + 1, j + 1, k), v111 = B(i + 1, j + 1, k + 1);
  float v00 = v000 + w[2] * (v001 - v000);
  float v01 = v010 + w[2] * (v011 - v010);
  float v10 = v100 + w[2] * (v101 - v100);
  float v11 = v110 + w[2] * (v111 - v110);
  float v0 = v00 + w[1] * (v01 - v00);
  float v1 = v10 + w[1] * (v11 - v10);
  return v0 + w[0] * (v1 - v0);
}

float shape_phi(const orc_shape& sh, const float p[3]) {
  if (sh.kind == 0) {  // Cube::IsInside, common/primitives.cc:56-64
    bool in = true;
    for (int d = 0; d < 3; ++d) { in &= (p[d] >= sh.a[d]); in &= (p[d] <= sh.b[d]); }
    return in ? -1.0f : 1.0f;
  } else if (sh.kind == 1) {  // sphere: |p - c| - r
    float dx = p[0] - sh.a[0], dy = p[1] - sh.a[1], dz = p[2] - sh.a[2];
    float l2 = (dx * dx + dy * dy) + dz * dz;
    return std::sqrt(l2) - sh.r;
  } else {  // reservoir: y - height
    return p[1] - sh.a[1];
  }
}
float pass_phi(const orc_seed_pass& ps, const float p[3]) {
  float phi = shape_phi(ps.shapes[0], p);
  for (int i = 1; i < ps.nshapes; ++i) phi = std::fmin(phi, shape_phi(ps.shapes[i], p));
  return phi;
}

void recompute_keys(orc_sim* s) {
  const size_t n = s->pos.size() / 3;
  s->keys.resize(n);
  s->cell.resize(3 * n);
  for (size_t i = 0; i < n; ++i) {
    for (int d = 0; d < 3; ++d) s->cell[3 * i + d] = int(std::floor(s->pos[3 * i + d]));
    s->keys[i] = s->K.key(s->cell[3 * i], s->cell[3 * i + 1], s->cell[3 * i + 2]);
  }
}

template <typename T>
struct PCG {
  // Solver::CreateIndexAndMaskTree / CreateLaplacianMatrix restated
  // (common/solver.cc:115-151, 198-233) and PCGDriver::Solve
  // (common/solver_driver.cc:14-69) with the PCGSolver stages
  // (common/solver.cc:263-366).
  static int32_t run(orc_sim* s, int32_t mode, int32_t max_it, double threshold,
                     double tol, orc_pcg_stats* st) {
    const int* n = s->D.n;
    std::vector<int32_t> idx(s->D.total, -1);
    std::vector<size_t> cells;
    for (int i = 0; i < n[0]; ++i)
      for (int j = 0; j < n[1]; ++j)
        for (int k = 0; k < n[2]; ++k)
          if (mget(s, i, j, k) == FLUID) {
            idx[s->D.idx(i, j, k)] = int32_t(cells.size());
            cells.push_back(s->D.idx(i, j, k));
          }
    const size_t R = cells.size();
    // rows: up to 7 (col, val) sorted by column
    std::vector<int32_t> cols(7 * R, -1);
    std::vector<T> vals(7 * R, T(0));
    std::vector<T> invd(R);
    std::vector<T> b(R), x(R, T(0)), r(R), z(R), p(R), Ap(R);
    static const int off[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0},
                                  {0, 1, 0},  {0, 0, -1}, {0, 0, 1}};
    par_for(R, [&](size_t r0, size_t r1) {
      for (size_t row = r0; row < r1; ++row) {
        const size_t cx = cells[row];
        const int i = int(cx / (size_t(s->D.s[1]) * s->D.s[2])) - 2;
        const int j = int((cx / size_t(s->D.s[2])) % size_t(s->D.s[1])) - 2;
        const int k = int(cx % size_t(s->D.s[2])) - 2;
        T diag = 0;
        std::pair<int32_t, T> ent[7];
        int ne = 0;
        for (int q = 0; q < 6; ++q) {
          int a = i + off[q][0], bb = j + off[q][1], c = k + off[q][2];
          int m = mget(s, a, bb, c);
          if (m == FLUID || m == AIR) diag += T(1);
          if (m == FLUID) ent[ne++] = {idx[s->D.idx(a, bb, c)], T(-1)};
        }
        ent[ne++] = {int32_t(row), diag};
        std::sort(ent, ent + ne,
                  [](const std::pair<int32_t, T>& u, const std::pair<int32_t, T>& v) {
                    return u.first < v.first;
                  });
        for (int e = 0; e < ne; ++e) {
          cols[7 * row + e] = ent[e].first;
          vals[7 * row + e] = ent[e].second;
        }
        invd[row] = T(1.0 / double(diag));
        b[row] = T(fget(s, s->div, s->div_on, i, j, k));
      }
    });
    auto spmv = [&](const std::vector<T>& in, std::vector<T>& out) {
      par_for(R, [&](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; ++q) {
          T acc = 0;
          for (int e = 0; e < 7 && cols[7 * q + e] >= 0; ++e)
            acc += vals[7 * q + e] * in[cols[7 * q + e]];
          out[q] = acc;
        }
      });
    };
    // pcg::Vector<T>::dot of OpenVDB 4.0.1 (third party, absent here) sums
    // contiguous ranges of the vector in parallel and then adds the range
    // totals; its exact split is not pinned.  Restated as kDotChunks equal
    // contiguous chunks (the last one takes the remainder), each summed
    // serially in T, chunk totals added in chunk order.  The split matters:
    // on the first system of the 256^3 dam break (4.02 M rows) a single
    // serial sum needs 1134 iterations to relative 1e-5, 100 chunks 881.
    constexpr size_t kDotChunks = 100;
    std::vector<T> chunk_sum(kDotChunks);
    auto dot = [&](const std::vector<T>& u, const std::vector<T>& v) {
      const size_t sz = R / kDotChunks;
      par_for(kDotChunks, [&](size_t c0, size_t c1) {
        for (size_t c = c0; c < c1; ++c) {
          const size_t e = (c + 1 == kDotChunks) ? R : (c + 1) * sz;
          T a = 0;
          for (size_t q = c * sz; q < e; ++q) a += u[q] * v[q];
          chunk_sum[c] = a;
        }
      });
      T acc = 0;
      for (size_t c = 0; c < kDotChunks; ++c) acc += chunk_sum[c];
      return acc;
    };
    // PreparePCGSolver: r = b - A x; z = M^-1 r; p = z; rz; rr
    spmv(x, Ap);
    par_for(R, [&](size_t q0, size_t q1) {
      for (size_t q = q0; q < q1; ++q) {
        r[q] = b[q] - Ap[q];
        z[q] = invd[q] * r[q];
        p[q] = z[q];
      }
    });
    T rz = dot(r, z), rr = dot(r, r);
    const T bb = dot(b, b);
    const T thr = T(threshold);
    const double tol2bb = tol * tol * double(bb);
    int it = 0;
    int32_t status = 0;
    auto done = [&]() {
      if (mode == 2) return it >= max_it;
      if (it >= max_it) return true;
      if (mode == 0) return rr < thr;
      return double(rr) <= tol2bb;
    };
    while (!done()) {
      // ComputeLocal1
      spmv(p, Ap);
      // The reference's own loop (common/solver.cc:304-307): one running sum
      // in source, built -Ofast (makeinclude/flags.mk:6), which lets the
      // compiler vectorise the reduction.  Restated as 4-wide vector code
      // sums it: lane l accumulates the terms q = l (mod 4) over the
      // multiple-of-4 prefix, the lanes are added as (l0 + l2) + (l1 + l3),
      // then the tail terms in order.  (A single running sum here, with the
      // chunked dots above, diverges on the second system of the 256^3 dam
      // break: p.Ap then carries far more rounding than r.z.)
      const size_t R4 = R & ~size_t(3);
      T lane[4] = {0, 0, 0, 0};
      auto lane_sum = [&](size_t l) {
        T a = 0;
        for (size_t q = l; q < R4; q += 4) a += p[q] * Ap[q];
        lane[l] = a;
      };
      if (g_pool.size() >= 4 && R4 >= 4096)
        g_pool.run([&](int t) {
          for (size_t l = size_t(t); l < 4; l += size_t(g_pool.size())) lane_sum(l);
        });
      else
        for (size_t l = 0; l < 4; ++l) lane_sum(l);
      T pAp = (lane[0] + lane[2]) + (lane[1] + lane[3]);
      for (size_t q = R4; q < R; ++q) pAp += p[q] * Ap[q];
      // ComputeLocal2
      T alpha = rz / pAp;
      if (!(alpha <= T(1e5))) { status = 5; break; }
      par_for(R, [&](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; ++q) {
          x[q] = alpha * p[q] + x[q];
          r[q] = -alpha * Ap[q] + r[q];
          z[q] = invd[q] * r[q];
        }
      });
      rr = dot(r, r);
      T rz_old = rz;
      rz = dot(r, z);
      // ComputeLocal3
      T beta = rz / rz_old;
      if (!(beta <= T(1e5))) { status = 5; ++it; break; }
      par_for(R, [&](size_t q0, size_t q1) {
        for (size_t q = q0; q < q1; ++q) p[q] = z[q] + beta * p[q];
      });
      ++it;
    }
    if (status == 0 && mode == 1 && double(rr) > tol2bb) status = 4;
    // CopySolution: clear pressure grid, write x at FLUID cells
    std::fill(s->pres_on.begin(), s->pres_on.end(), 0);
    std::fill(s->pres.begin(), s->pres.end(), 0.f);
    s->pres64.assign(s->D.total, 0.0);
    for (size_t q = 0; q < R; ++q) {
      s->pres[cells[q]] = float(x[q]);
      s->pres_on[cells[q]] = 1;
      s->pres64[cells[q]] = double(x[q]);
    }
    if (st) {
      st->iterations = it;
      st->n_rows = int32_t(R);
      st->status = status;
      st->rr = double(rr);
      st->bb = double(bb);
    }
    return status;
  }
};

}  // namespace

extern "C" {

orc_sim* orc_create(const int32_t dims[3], int32_t boundary, float gravity,
                    const float force[3], float flip, int32_t nppc) {
  orc_sim* s = new orc_sim();
  s->D.init(dims);
  s->K.init(s->D.n);
  s->boundary = boundary;
  s->gravity = gravity;
  s->fx = force[0]; s->fy = force[1]; s->fz = force[2];
  s->flip = flip;
  s->nppc = nppc;
  const size_t T = s->D.total;
  s->solid.assign(T, 0);
  s->vel.assign(3 * T, 0.f); s->vold.assign(3 * T, 0.f); s->weight.assign(3 * T, 0.f);
  s->vel_on.assign(T, 0); s->vold_on.assign(T, 0); s->weight_on.assign(T, 0);
  s->marker.assign(T, 0); s->marker_on.assign(T, 0);
  s->div.assign(T, 0.f); s->pres.assign(T, 0.f);
  s->div_on.assign(T, 0); s->pres_on.assign(T, 0); s->phi_on.assign(T, 0);
  build_walls(s);
  return s;
}

void orc_destroy(orc_sim* s) { delete s; }

void orc_set_threads(int32_t n) { g_pool.resize(n); }
int32_t orc_get_threads(void) { return g_pool.size(); }

void orc_add_solid_cuboid(orc_sim* s, const int32_t lo[3], const int32_t hi[3]) {
  // AddSolidCuboid, common/flip_simulation.cc:316-324: domain grown by 1,
  // intersected with the box, filled active with 1.
  int a[3], b[3];
  for (int d = 0; d < 3; ++d) {
    a[d] = std::max(lo[d], -1);
    b[d] = std::min(hi[d], s->D.n[d]);
  }
  for (int i = a[0]; i <= b[0]; ++i)
    for (int j = a[1]; j <= b[1]; ++j)
      for (int k = a[2]; k <= b[2]; ++k) s->solid[s->D.idx(i, j, k)] = 1;
  Cuboid c;
  for (int d = 0; d < 3; ++d) { c.lo[d] = lo[d]; c.hi[d] = hi[d]; }
  s->cuboids.push_back(c);
}

int32_t orc_is_solid(const orc_sim* s, int32_t i, int32_t j, int32_t k) {
  return sget(s, i, j, k);
}

float orc_seed_uniform(uint64_t seed, int32_t pass, int64_t cell, int32_t draw, int32_t d) {
  return uniform01(seed, pass, cell, draw, d);
}

int64_t orc_seed(orc_sim* s, const orc_seed_pass* passes, int32_t npasses, uint64_t seed) {
  // FlipSimulation::InitializePhiAndParticles, flip_simulation.cc:139-188,
  // one call per pass; per-cell counts persist across passes.
  s->seed = seed;
  const int* n = s->D.n;
  const size_t ncell = size_t(n[0]) * n[1] * n[2];
  std::vector<int32_t> count(ncell, 0);
  std::vector<std::vector<float>> cp(ncell);  // per cell: 9 floats per particle
  for (int ps = 0; ps < npasses; ++ps) {
    const orc_seed_pass& P = passes[ps];
    for (int i = 0; i < n[0]; ++i)
      for (int j = 0; j < n[1]; ++j)
        for (int k = 0; k < n[2]; ++k) {
          if (sget(s, i, j, k) == 1) continue;
          const float org[3] = {float(i), float(j), float(k)};
          const float ctr[3] = {org[0] + 0.5f, org[1] + 0.5f, org[2] + 0.5f};
          float phi = pass_phi(P, ctr);
          if (!(phi < 0.5f) || !(phi < 0.f)) continue;
          const size_t c = (size_t(i) * n[1] + j) * n[2] + k;
          if (count[c] >= s->nppc) continue;
          int pi = 0, draw = 0;
          for (int att = 0; att < 32 && pi < s->nppc; ++att, ++draw) {
            float pp[3];
            for (int d = 0; d < 3; ++d)
              pp[d] = org[d] + uniform01(seed, ps, int64_t(c), draw, d) * 1.0f;
            if (pass_phi(P, pp) > 0.f) continue;
            for (int d = 0; d < 3; ++d) cp[c].push_back(pp[d]);
            for (int d = 0; d < 3; ++d) cp[c].push_back(P.velocity[d]);
            for (int d = 0; d < 3; ++d) cp[c].push_back(P.velocity[d]);
            ++pi;
            ++att;  // the reference increments num_attempts again on success
            ++count[c];
          }
        }
  }
  // AddParticleToData(i, j, k, pd) files each particle under the cell that
  // generated it, even when its float position rounds onto the upper face
  // (org + u == org + 1); StepInGrid rebins by floor(pos) later.
  s->pos.clear(); s->vel_p.clear(); s->gvel.clear(); s->cell.clear(); s->keys.clear();
  for (size_t c = 0; c < ncell; ++c) {
    const int ci = int(c / (size_t(n[1]) * n[2])), cj = int((c / n[2]) % n[1]), ck = int(c % n[2]);
    for (size_t q = 0; q < cp[c].size(); q += 9) {
      for (int d = 0; d < 3; ++d) s->pos.push_back(cp[c][q + d]);
      for (int d = 0; d < 3; ++d) s->vel_p.push_back(cp[c][q + 3 + d]);
      for (int d = 0; d < 3; ++d) s->gvel.push_back(cp[c][q + 6 + d]);
      s->cell.push_back(ci); s->cell.push_back(cj); s->cell.push_back(ck);
      s->keys.push_back(s->K.key(ci, cj, ck));
    }
  }
  reorder_by_key(s);
  return int64_t(s->keys.size());
}

void orc_perturb_velocities(orc_sim* s, float sigma, uint64_t seed) {
  const size_t n = s->keys.size();
  for (size_t i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      float u1 = uniform01(seed, 1 << 20, int64_t(i), 0, d);
      float u2 = uniform01(seed, 1 << 20, int64_t(i), 1, d);
      float g = std::sqrt(-2.0f * std::log(1.0f - u1)) * std::cos(6.2831853f * u2);
      s->vel_p[3 * i + d] = s->vel_p[3 * i + d] + sigma * g;
      s->gvel[3 * i + d] = s->vel_p[3 * i + d];
    }
}

void orc_set_particles(orc_sim* s, const float* pos, const float* vel, const float* gvel,
                       int64_t n) {
  s->pos.assign(pos, pos + 3 * n);
  s->vel_p.assign(vel, vel + 3 * n);
  s->gvel.assign(gvel, gvel + 3 * n);
  recompute_keys(s);
  reorder_by_key(s);
}

int64_t orc_particle_count(const orc_sim* s) { return int64_t(s->keys.size()); }

void orc_get_particles(const orc_sim* s, float* pos, float* vel, float* gvel) {
  if (pos) std::memcpy(pos, s->pos.data(), s->pos.size() * sizeof(float));
  if (vel) std::memcpy(vel, s->vel_p.data(), s->vel_p.size() * sizeof(float));
  if (gvel) std::memcpy(gvel, s->gvel.data(), s->gvel.size() * sizeof(float));
}

void orc_get_particle_keys(const orc_sim* s, uint32_t* keys) {
  std::memcpy(keys, s->keys.data(), s->keys.size() * sizeof(uint32_t));
}

int64_t orc_get_leaves(const orc_sim* s, int32_t* origins, int64_t capacity) {
  std::vector<size_t> st;
  leaf_ranges(s, st);
  int64_t nl = int64_t(st.size()) - 1;
  for (int64_t l = 0; l < nl && l < capacity; ++l) {
    const int32_t* c = &s->cell[3 * st[l]];
    for (int d = 0; d < 3; ++d) origins[3 * l + d] = floor_div(c[d], 8) * 8;
  }
  return nl;
}

float orc_cfl(orc_sim* s) {
  // FlipSimulation::CFL, flip_simulation.cc:460-488
  const int* n = s->D.n;
  float v_inf = 0.f;
  for (int i = 0; i < n[0]; ++i)
    for (int j = 0; j < n[1]; ++j)
      for (int k = 0; k < n[2]; ++k) {
        size_t x = s->D.idx(i, j, k);
        if (!s->vel_on[x]) continue;
        const float* v = &s->vel[3 * x];
        if (j != n[1] - 1 && k != n[2] - 1) v_inf = std::fmax(v_inf, std::fabs(v[0]));
        if (i != n[0] - 1 && k != n[2] - 1) v_inf = std::fmax(v_inf, std::fabs(v[1]));
        if (i != n[0] - 1 && j != n[1] - 1) v_inf = std::fmax(v_inf, std::fabs(v[2]));
      }
  float v = float(std::fmax(std::sqrt(0.5 * double(s->gravity)), double(v_inf)));
  if (v < 1e-2) v = float(1e-2);
  return float(1.0 / double(v));
}

void orc_move_particles(orc_sim* s, float dt) {
  // Particles::StepInGrid<VectorGrid,true,1,1>, particles.cc:479-546
  const size_t n = s->keys.size();
  const int* dims = s->D.n;
  par_for(n, [&](size_t i0, size_t i1) {
    for (size_t i = i0; i < i1; ++i) {
      float* p = &s->pos[3 * i];
      const float* g = &s->gvel[3 * i];
      for (int d = 0; d < 3; ++d) p[d] = p[d] + g[d] * dt;
      int id[3];
      for (int d = 0; d < 3; ++d) id[d] = int(std::floor(p[d]));
      for (int d = 0; d < 3; ++d)
        if (id[d] < 0) { id[d] = 0; p[d] = 0.f; }
      for (int d = 0; d < 3; ++d)
        if (id[d] >= dims[d]) { id[d] = dims[d]; p[d] = float(dims[d]); }
      for (int d = 0; d < 3; ++d) s->cell[3 * i + d] = id[d];
      s->keys[i] = s->K.key(id[0], id[1], id[2]);
    }
  });
  reorder_by_key(s);
  orc_delete_particles_in_solids(s);
}

void orc_delete_particles_in_solids(orc_sim* s) {
  // Particles::DeleteParticlesInSolids, particles.cc:202-219
  const size_t n = s->keys.size();
  std::vector<uint8_t> kill(n, 0);
  for (size_t i = 0; i < n; ++i) {
    const int* c = &s->cell[3 * i];
    kill[i] = uint8_t(sget(s, c[0], c[1], c[2]) == 1);
  }
  erase_where(s, kill);
}

void orc_clear_grid(orc_sim* s) {
  // FlipSimulation::ClearGridData, flip_simulation.cc:380-389
  std::fill(s->vel_on.begin(), s->vel_on.end(), 0);
  std::fill(s->vold_on.begin(), s->vold_on.end(), 0);
  std::fill(s->weight_on.begin(), s->weight_on.end(), 0);
  std::fill(s->marker_on.begin(), s->marker_on.end(), 0);
  std::fill(s->div_on.begin(), s->div_on.end(), 0);
  std::fill(s->pres_on.begin(), s->pres_on.end(), 0);
  std::fill(s->phi_on.begin(), s->phi_on.end(), 0);
  std::fill(s->vel.begin(), s->vel.end(), 0.f);
  std::fill(s->vold.begin(), s->vold.end(), 0.f);
  std::fill(s->weight.begin(), s->weight.end(), 0.f);
  std::fill(s->marker.begin(), s->marker.end(), 0);
  std::fill(s->div.begin(), s->div.end(), 0.f);
  std::fill(s->pres.begin(), s->pres.end(), 0.f);
}

void orc_transfer_particles_to_grid(orc_sim* s) {
  // FlipSimulation::TransferParticlesToGrid, flip_simulation.cc:809-923
  const int* n = s->D.n;
  std::vector<size_t> st;
  leaf_ranges(s, st);
  const int S = 1000;
  const size_t nleaf = st.size() - 1;
  // Each leaf's (8+2)^3 halo buffers are summed over its particles in list
  // order, then added into the grid leaf by leaf in iteration order.  The
  // buffers of a batch of leaves are filled by the pool (leaves are
  // independent, and a leaf marks only its own cells FLUID); the write-back
  // stays serial in leaf order, so the grid sums do not depend on the
  // thread count.
  const size_t batch = g_pool.size() == 1 ? 1 : 512;
  std::vector<float> vb(batch * 3 * S), wb(batch * 3 * S);
  std::vector<uint8_t> mb(batch * 3 * S);
  std::vector<int> orgs(batch * 3);
  auto fill = [&](size_t l, size_t slot) {
    float* V = &vb[slot * 3 * S];
    float* W = &wb[slot * 3 * S];
    uint8_t* M = &mb[slot * 3 * S];
    int* org = &orgs[slot * 3];
    const int32_t* c0 = &s->cell[3 * st[l]];
    for (int d = 0; d < 3; ++d) org[d] = floor_div(c0[d], 8) * 8 - 1;
    std::fill(V, V + 3 * S, 0.f);
    std::fill(W, W + 3 * S, 0.f);
    std::fill(M, M + 3 * S, uint8_t(0));
    for (size_t q = st[l]; q < st[l + 1]; ++q) {
      const int* c = &s->cell[3 * q];
      if (c[0] >= 0 && c[0] < n[0] && c[1] >= 0 && c[1] < n[1] && c[2] >= 0 && c[2] < n[2])
        mset(s, c[0], c[1], c[2], FLUID);
      const float* p = &s->pos[3 * q];
      const float* v = &s->vel_p[3 * q];
      for (int D = 0; D < 3; ++D) {
        int start[3];
        float w[2][2][2];
        scatter_weights(p, c, D, start, w);
        for (int a = 0; a < 3; ++a) start[a] -= org[a];
        for (int di = 0; di < 2; ++di)
          for (int dj = 0; dj < 2; ++dj)
            for (int dk = 0; dk < 2; ++dk) {
              int o = ((start[0] + di) * 10 + (start[1] + dj)) * 10 + (start[2] + dk);
              V[D * S + o] += w[di][dj][dk] * v[D];
              W[D * S + o] += w[di][dj][dk];
              M[D * S + o] = 1;
            }
      }
    }
  };
  auto write_back = [&](size_t slot) {
    const float* V = &vb[slot * 3 * S];
    const float* W = &wb[slot * 3 * S];
    const uint8_t* M = &mb[slot * 3 * S];
    const int* org = &orgs[slot * 3];
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j)
        for (int k = 0; k < 10; ++k) {
          int o = (i * 10 + j) * 10 + k;
          if (!M[o] && !M[S + o] && !M[2 * S + o]) continue;
          int x = org[0] + i, y = org[1] + j, z = org[2] + k;
          Vec3f v = vget(s, s->vel, s->vel_on, x, y, z);
          for (int D = 0; D < 3; ++D) v.v[D] = v.v[D] + V[D * S + o];
          vset(s, s->vel, s->vel_on, x, y, z, v);
          Vec3f w = vget(s, s->weight, s->weight_on, x, y, z);
          for (int D = 0; D < 3; ++D) w.v[D] = w.v[D] + W[D * S + o];
          vset(s, s->weight, s->weight_on, x, y, z, w);
        }
  };
  for (size_t l0 = 0; l0 < nleaf; l0 += batch) {
    const size_t nb = std::min(batch, nleaf - l0);
    if (nb == 1) {
      fill(l0, 0);
    } else {
      const int T = g_pool.size();
      g_pool.run([&](int t) {
        for (size_t b = nb * size_t(t) / size_t(T); b < nb * size_t(t + 1) / size_t(T); ++b)
          fill(l0 + b, b);
      });
    }
    for (size_t b = 0; b < nb; ++b) write_back(b);
  }
  // normalise every active face (THRESH 1e-5)
  par_for(s->D.total, [&](size_t x0, size_t x1) {
    for (size_t x = x0; x < x1; ++x) {
      if (!s->vel_on[x]) continue;
      for (int D = 0; D < 3; ++D) {
        float ws = s->weight_on[x] ? s->weight[3 * x + D] : 0.f;
        if (double(ws) < 1e-5) s->vel[3 * x + D] = 0.f;  // THRESH is a double literal
        else s->vel[3 * x + D] = s->vel[3 * x + D] / ws;
      }
    }
  });
}

void orc_apply_boundary_conditions(orc_sim* s) {
  // FlipSimulation::ApplyBoundaryConditions, flip_simulation.cc:657-713
  const int* n = s->D.n;
  for (int i = -1; i <= n[0]; ++i)
    for (int j = -1; j <= n[1]; ++j)
      for (int k = -1; k <= n[2]; ++k) {
        if (!sget(s, i, j, k)) continue;
        mset(s, i, j, k, SOLID);
        const int c[3] = {i, j, k};
        for (int d = 0; d < 3; ++d) {
          int lo[3] = {c[0], c[1], c[2]};
          lo[d] -= 1;
          if (sget(s, lo[0], lo[1], lo[2]) == 0 && von(s, s->vel_on, i, j, k)) {
            Vec3f v = vget(s, s->vel, s->vel_on, i, j, k);
            v.v[d] = 0.f;
            vset(s, s->vel, s->vel_on, i, j, k, v);
          }
        }
        for (int d = 0; d < 3; ++d) {
          int up[3] = {c[0], c[1], c[2]};
          up[d] += 1;
          if (sget(s, up[0], up[1], up[2]) == 0 && von(s, s->vel_on, up[0], up[1], up[2])) {
            Vec3f v = vget(s, s->vel, s->vel_on, up[0], up[1], up[2]);
            v.v[d] = 0.f;
            vset(s, s->vel, s->vel_on, up[0], up[1], up[2], v);
          }
        }
      }
}

void orc_save_grid_velocities(orc_sim* s) {
  // FlipSimulation::SaveGridVelocities, flip_simulation.cc:491-496
  for (size_t x = 0; x < s->D.total; ++x) {
    if (!s->vel_on[x]) continue;
    s->vold_on[x] = 1;
    for (int d = 0; d < 3; ++d) s->vold[3 * x + d] = s->vel[3 * x + d];
  }
}

void orc_delete_outside_particles(orc_sim* s) {
  // Particles::DeleteOutsideParticles, particles.cc:273-293
  const size_t n = s->keys.size();
  std::vector<uint8_t> kill(n, 0);
  for (size_t i = 0; i < n; ++i) {
    const int* c = &s->cell[3 * i];
    bool out = false;
    for (int d = 0; d < 3; ++d) out |= (c[d] < 0 || c[d] > s->D.n[d] - 1);
    kill[i] = out;
  }
  erase_where(s, kill);
}

void orc_reinitialize_phi(orc_sim* s) {
  // ReinitializePhiSimple, flip_simulation.cc:529-539: phi = -0.5 in FLUID
  for (size_t x = 0; x < s->D.total; ++x)
    if (s->marker_on[x] && s->marker[x] == FLUID) s->phi_on[x] = 1;
}

void orc_add_gravity(orc_sim* s, float dt) {
  // FlipSimulation::AddGravity, flip_simulation.cc:506-515
  const float gx = dt * s->fx, gy = dt * s->fy, gz = dt * s->fz;
  for (size_t x = 0; x < s->D.total; ++x) {
    if (!s->vel_on[x]) continue;
    s->vel[3 * x] = s->vel[3 * x] + gx;
    s->vel[3 * x + 1] = s->vel[3 * x + 1] - gy;
    s->vel[3 * x + 2] = s->vel[3 * x + 2] + gz;
  }
}

void orc_compute_divergence(orc_sim* s) {
  // FlipSimulation::ComputeDivergence, flip_simulation.cc:716-736
  const int* n = s->D.n;
  for (int i = 0; i < n[0]; ++i)
    for (int j = 0; j < n[1]; ++j)
      for (int k = 0; k < n[2]; ++k) {
        if (mget(s, i, j, k) != FLUID) continue;
        float dv = 0.f;
        dv += vget(s, s->vel, s->vel_on, i + 1, j, k).v[0] - vget(s, s->vel, s->vel_on, i, j, k).v[0];
        dv += vget(s, s->vel, s->vel_on, i, j + 1, k).v[1] - vget(s, s->vel, s->vel_on, i, j, k).v[1];
        dv += vget(s, s->vel, s->vel_on, i, j, k + 1).v[2] - vget(s, s->vel, s->vel_on, i, j, k).v[2];
        size_t x = s->D.idx(i, j, k);
        s->div[x] = dv;
        s->div_on[x] = 1;
      }
}

int32_t orc_pcg_solve(orc_sim* s, int32_t mode, int32_t precision, int32_t max_iterations,
                      double threshold, double tol, orc_pcg_stats* stats) {
  if (precision == 2) return PCG<double>::run(s, mode, max_iterations, threshold, tol, stats);
  return PCG<float>::run(s, mode, max_iterations, threshold, tol, stats);
}

void orc_update_velocity_from_pressure(orc_sim* s) {
  // FlipSimulation::UpdateVelocityFromPressure, flip_simulation.cc:739-778
  const int* n = s->D.n;
  for (int i = 0; i <= n[0]; ++i)
    for (int j = 0; j <= n[1]; ++j)
      for (int k = 0; k <= n[2]; ++k) {
        Vec3f v = vget(s, s->vel, s->vel_on, i, j, k);
        int mc = mget(s, i, j, k);
        if (mc == SOLID) continue;
        bool upd = false;
        const float pc = fget(s, s->pres, s->pres_on, i, j, k);
        const int nb[3][3] = {{i - 1, j, k}, {i, j - 1, k}, {i, j, k - 1}};
        for (int d = 0; d < 3; ++d) {
          int mn = mget(s, nb[d][0], nb[d][1], nb[d][2]);
          if ((mn == FLUID || mc == FLUID) && mn != SOLID) {
            v.v[d] = v.v[d] + (pc - fget(s, s->pres, s->pres_on, nb[d][0], nb[d][1], nb[d][2]));
            upd = true;
          }
        }
        if (upd) vset(s, s->vel, s->vel_on, i, j, k, v);
      }
}

int32_t orc_get_velocity_update(orc_sim* s) {
  // FlipSimulation::GetVelocityUpdate, flip_simulation.cc:781-801
  const int* n = s->D.n;
  int32_t bad = 0;
  for (int i = 0; i <= n[0]; ++i)
    for (int j = 0; j <= n[1]; ++j)
      for (int k = 0; k <= n[2]; ++k) {
        size_t x = s->D.idx(i, j, k);
        if (s->vel_on[x] && !s->vold_on[x]) bad = 1;
        if (s->vel_on[x] && s->vold_on[x])
          for (int d = 0; d < 3; ++d) s->vold[3 * x + d] = s->vel[3 * x + d] - s->vold[3 * x + d];
      }
  return bad;
}

void orc_extrapolate_to_boundary(orc_sim* s, int32_t field) {
  // VectorGrid::ExtrapolateToBoundary, vector_grid.cc:302-381 (six passes,
  // in order; each copies the two tangential components into the ghost layer)
  std::vector<float>& f = field == 0 ? s->vel : s->vold;
  std::vector<uint8_t>& on = field == 0 ? s->vel_on : s->vold_on;
  const int* n = s->D.n;
  for (int side = 0; side < 6; ++side) {
    const int ax = side / 2;
    const bool upper = side & 1;
    const int ghost = upper ? n[ax] : -1;
    const int inner = upper ? n[ax] - 1 : 0;
    const int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
    const int u = std::min(a1, a2), w = std::max(a1, a2);
    for (int p = 0; p <= n[u]; ++p)
      for (int q = 0; q <= n[w]; ++q) {
        int go[3], gi[3];
        go[ax] = ghost; gi[ax] = inner;
        go[u] = gi[u] = p;
        go[w] = gi[w] = q;
        Vec3f vo = vget(s, f, on, go[0], go[1], go[2]);
        Vec3f vi = vget(s, f, on, gi[0], gi[1], gi[2]);
        vo.v[a1] = vi.v[a1];
        vo.v[a2] = vi.v[a2];
        vset(s, f, on, go[0], go[1], go[2], vo);
      }
  }
}

void orc_update_particles_from_grid(orc_sim* s) {
  // FlipSimulation::UpdateParticlesFromGrid, flip_simulation.cc:1025-1091
  // and UpdateSingleParticleFromGrid, :1179-1189
  orc_extrapolate_to_boundary(s, 0);
  orc_extrapolate_to_boundary(s, 1);
  std::vector<size_t> st;
  leaf_ranges(s, st);
  // leaves are independent: each pool thread takes a contiguous range
  par_for(st.size() - 1, [&](size_t l0, size_t l1) {
    std::vector<float> vb(3000), db(3000);
    for (size_t l = l0; l < l1; ++l) {
      const int32_t* c0 = &s->cell[3 * st[l]];
      int org[3];
      for (int d = 0; d < 3; ++d) org[d] = floor_div(c0[d], 8) * 8 - 1;
      for (int i = 0; i < 10; ++i)
        for (int j = 0; j < 10; ++j)
          for (int k = 0; k < 10; ++k) {
            int o = (i * 10 + j) * 10 + k;
            Vec3f v = vget(s, s->vel, s->vel_on, org[0] + i, org[1] + j, org[2] + k);
            Vec3f dv = vget(s, s->vold, s->vold_on, org[0] + i, org[1] + j, org[2] + k);
            for (int D = 0; D < 3; ++D) { vb[D * 1000 + o] = v.v[D]; db[D * 1000 + o] = dv.v[D]; }
          }
      for (size_t q = st[l]; q < st[l + 1]; ++q) {
        const int* c = &s->cell[3 * q];
        const int lc[3] = {c[0] - org[0], c[1] - org[1], c[2] - org[2]};
        const float* p = &s->pos[3 * q];
        float* pv = &s->vel_p[3 * q];
        float* g = &s->gvel[3 * q];
        for (int D = 0; D < 3; ++D) {
          float v = interp_component(p, c, D, &vb[D * 1000], lc);
          float dv = interp_component(p, c, D, &db[D * 1000], lc);
          pv[D] = v + s->flip * ((dv + pv[D]) - v);
          g[D] = v;
        }
      }
    }
  });
}

namespace {

// Source<T>::get_box / get_velocity / is_active, common/sources.cc:66-109
void src_box(const orc_source& q, float t, float lo[3], float hi[3]) {
  (void)t;  // the oscillating branch assigns a shadowed local: box1 is used
  for (int d = 0; d < 3; ++d) {
    lo[d] = q.lo[d];
    hi[d] = q.hi[d] - 1.0f;  // box.set_end(box.get_end() - Vec3(1))
  }
}
void src_velocity(const orc_source& q, float t, float v[3]) {
  if (!q.velocity_oscillating) {
    for (int d = 0; d < 3; ++d) v[d] = q.velocity[d];
    return;
  }
  const float w = float(M_PI * double(t) / double(q.box_period));  // uses box_period_
  for (int d = 0; d < 3; ++d)
    v[d] = float(double(q.velocity[d]) +
                 0.5 * double(q.velocity2[d] - q.velocity[d]) * (double(std::cos(w)) + 1.0));
}
bool src_active(const orc_source& q, float t) {
  return !q.timed || (t >= q.start_time && t <= q.end_time);
}
bool in_box(const float lo[3], const float hi[3], const float p[3]) {
  bool in = true;
  for (int d = 0; d < 3; ++d) in &= (p[d] >= lo[d]) && (p[d] <= hi[d]);  // Cube::IsInside
  return in;
}

}  // namespace

void orc_add_source(orc_sim* s, const orc_source* src) { s->sources.push_back(*src); }
void orc_set_time(orc_sim* s, double t) { s->time = t; }
double orc_get_time(const orc_sim* s) { return s->time; }

void orc_add_contribution_from_sources(orc_sim* s, float t) {
  // FlipSimulation::AddContributionFromSources, flip_simulation.cc:1207-1270.
  // Particles go to the end of their cell's list (AddParticleToData); the
  // grid writes are cleared by ClearGridData before anything reads them.
  const int* n = s->D.n;
  const int64_t call = s->source_calls++;
  bool added = false;
  for (size_t q = 0; q < s->sources.size(); ++q) {
    const orc_source& src = s->sources[q];
    if (!src_active(src, t)) continue;
    float v[3], lo[3], hi[3];
    src_velocity(src, t, v);
    src_box(src, t, lo, hi);
    int a[3], b[3];
    for (int d = 0; d < 3; ++d) {
      a[d] = std::max(int(lo[d]), 0);            // Coord(float) truncates;
      b[d] = std::min(int(hi[d]), n[d] - 1);     // the domain box is [0, N-1]
    }
    const int pass = (1 << 22) + int((call & 0x1FFFF) * 32) + int(q);
    for (int i = a[0]; i <= b[0]; ++i)
      for (int j = a[1]; j <= b[1]; ++j)
        for (int k = a[2]; k <= b[2]; ++k) {
          const float org[3] = {float(i), float(j), float(k)};
          const int64_t c = (int64_t(i) * n[1] + j) * n[2] + k;
          int pi = 0;
          for (int att = 0; att < 32 && pi < s->nppc; ++att) {
            float pp[3];
            for (int d = 0; d < 3; ++d) pp[d] = org[d] + uniform01(s->seed, pass, c, att, d) * 1.0f;
            if (!in_box(lo, hi, pp)) continue;
            for (int d = 0; d < 3; ++d) {
              s->pos.push_back(pp[d]);
              s->vel_p.push_back(v[d]);
              s->gvel.push_back(v[d]);
            }
            s->cell.push_back(i); s->cell.push_back(j); s->cell.push_back(k);
            s->keys.push_back(s->K.key(i, j, k));
            added = true;
            ++pi;
          }
        }
  }
  if (added) reorder_by_key(s);  // stable: each cell's list keeps its old particles first
}

void orc_delete_fluid_in_sources(orc_sim* s, float t) {
  // FlipSimulation::DeleteFluidInSources, flip_simulation.cc:1273-1281, with
  // Particles::DeleteParticlesFromRegions (particles.cc:222-271): a particle
  // inside any source's box (active or not) is removed.
  if (s->sources.empty()) return;
  const size_t n = s->keys.size();
  std::vector<uint8_t> kill(n, 0);
  for (const orc_source& src : s->sources) {
    float lo[3], hi[3];
    src_box(src, t, lo, hi);
    for (size_t i = 0; i < n; ++i)
      if (in_box(lo, hi, &s->pos[3 * i])) kill[i] = 1;
  }
  erase_where(s, kill);
}

int32_t orc_step(orc_sim* s, float dt, int32_t mode, int32_t precision, int32_t max_iterations,
                 double threshold, double tol, orc_pcg_stats* stats) {
  // FlipDriver::RunOneStep, flip_app_sim.cc:211-254
  const float t = float(s->time);  // advanced_time_ (T = float)
  orc_add_contribution_from_sources(s, t);
  orc_move_particles(s, dt);
  orc_delete_fluid_in_sources(s, t);
  orc_clear_grid(s);
  orc_transfer_particles_to_grid(s);
  orc_apply_boundary_conditions(s);
  orc_save_grid_velocities(s);
  orc_delete_outside_particles(s);
  orc_reinitialize_phi(s);
  orc_add_gravity(s, dt);
  orc_apply_boundary_conditions(s);
  orc_compute_divergence(s);
  int32_t st = orc_pcg_solve(s, mode, precision, max_iterations, threshold, tol, stats);
  orc_update_velocity_from_pressure(s);
  orc_get_velocity_update(s);
  orc_update_particles_from_grid(s);
  s->time = double(t + dt);  // FlipDriver::AdvanceTime
  return st;
}

float orc_compute_dt(float inv_speed, int32_t cfl, float frame_step, float* time_in_frame) {
  // FlipDriver::WhileAndComputeDt, flip_app_sim.cc:357-428, one partition
  float local_dt = float(cfl) * inv_speed;
  float dt = float(1.0 / double(frame_step));
  dt = (local_dt < dt) ? local_dt : dt;
  if (dt < frame_step / 10) dt = frame_step / 10;
  float step = *time_in_frame;
  if (step + dt > frame_step) dt = frame_step - step;
  if (double(step + dt) > 0.9 * double(frame_step)) dt = frame_step - step;
  *time_in_frame = step + dt;
  return dt;
}

void orc_get_field(const orc_sim* s, int32_t field, float* out, uint8_t* active) {
  const int* n = s->D.n;
  const size_t s1 = n[1] + 2, s2 = n[2] + 2;
  for (int i = -1; i <= n[0]; ++i)
    for (int j = -1; j <= n[1]; ++j)
      for (int k = -1; k <= n[2]; ++k) {
        size_t o = (size_t(i + 1) * s1 + size_t(j + 1)) * s2 + size_t(k + 1);
        size_t x = s->D.idx(i, j, k);
        if (field <= 2) {
          const std::vector<float>& f = field == 0 ? s->vel : field == 1 ? s->vold : s->weight;
          const std::vector<uint8_t>& on =
              field == 0 ? s->vel_on : field == 1 ? s->vold_on : s->weight_on;
          for (int d = 0; d < 3; ++d) out[3 * o + d] = on[x] ? f[3 * x + d] : 0.f;
          if (active) active[o] = on[x];
        } else if (field == 3) {
          out[o] = s->div_on[x] ? s->div[x] : 0.f;
          if (active) active[o] = s->div_on[x];
        } else if (field == 4) {
          out[o] = s->pres_on[x] ? s->pres[x] : 0.f;
          if (active) active[o] = s->pres_on[x];
        } else {
          out[o] = s->phi_on[x] ? -0.5f : 5.0f;
          if (active) active[o] = s->phi_on[x];
        }
      }
}

void orc_get_marker(const orc_sim* s, int32_t* out, uint8_t* active) {
  const int* n = s->D.n;
  const size_t s1 = n[1] + 2, s2 = n[2] + 2;
  for (int i = -1; i <= n[0]; ++i)
    for (int j = -1; j <= n[1]; ++j)
      for (int k = -1; k <= n[2]; ++k) {
        size_t o = (size_t(i + 1) * s1 + size_t(j + 1)) * s2 + size_t(k + 1);
        size_t x = s->D.idx(i, j, k);
        out[o] = s->marker_on[x] ? s->marker[x] : 0;
        if (active) active[o] = s->marker_on[x];
      }
}

void orc_get_pressure_f64(const orc_sim* s, double* out) {
  const int* n = s->D.n;
  const size_t s1 = n[1] + 2, s2 = n[2] + 2;
  for (int i = -1; i <= n[0]; ++i)
    for (int j = -1; j <= n[1]; ++j)
      for (int k = -1; k <= n[2]; ++k) {
        size_t o = (size_t(i + 1) * s1 + size_t(j + 1)) * s2 + size_t(k + 1);
        out[o] = s->pres64.empty() ? 0.0 : s->pres64[s->D.idx(i, j, k)];
      }
}

void orc_set_divergence(orc_sim* s, const float* div) {
  const int* n = s->D.n;
  const size_t s1 = n[1] + 2, s2 = n[2] + 2;
  for (int i = -1; i <= n[0]; ++i)
    for (int j = -1; j <= n[1]; ++j)
      for (int k = -1; k <= n[2]; ++k) {
        size_t o = (size_t(i + 1) * s1 + size_t(j + 1)) * s2 + size_t(k + 1);
        size_t x = s->D.idx(i, j, k);
        s->div[x] = div[o];
        s->div_on[x] = div[o] != 0.f;
      }
}

void orc_set_marker(orc_sim* s, const int32_t* marker) {
  const int* n = s->D.n;
  const size_t s1 = n[1] + 2, s2 = n[2] + 2;
  for (int i = -1; i <= n[0]; ++i)
    for (int j = -1; j <= n[1]; ++j)
      for (int k = -1; k <= n[2]; ++k) {
        size_t o = (size_t(i + 1) * s1 + size_t(j + 1)) * s2 + size_t(k + 1);
        size_t x = s->D.idx(i, j, k);
        s->marker[x] = int8_t(marker[o]);
        s->marker_on[x] = marker[o] != 0;
      }
}

}  // extern "C"
