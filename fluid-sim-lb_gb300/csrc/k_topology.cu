// k_topology.cu -- advection + rebinning and the sparse 8^3 brick topology.
//
// Restates Particles::StepInGrid<VectorGrid,true,1,1> (common/particles.cc:
// 479-546) and DeleteParticlesInSolids (:202-219) as: one kernel that
// advects every particle (pos += gvel*dt, IEEE round-to-nearest, no FMA
// contraction), clamps it to [0,N] exactly as the reference does and emits
// its cell key (dead key for particles in solids); a stable device radix sort
// by key (this reproduces the reference's rebuilt cell lists, which keep
// particles in visiting order); a gather of the 9 particle arrays; and the
// leaf topology (particle leaves, one-leaf dilation, slots, 27-neighbour
// table, per-cell particle ranges).
#include <algorithm>
#include <cmath>
#include <cstring>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "fsim_internal.cuh"

namespace fsim {

// ---- Source<T> (common/sources.cc:66-109), evaluated on the host --------
void source_box(const fsim_source& src, float t, float lo[3], float hi[3]) {
  (void)t;  // the oscillating branch of get_box assigns a shadowed local
  for (int d = 0; d < 3; ++d) {
    lo[d] = src.lo[d];
    hi[d] = src.hi[d] - 1.0f;  // box.set_end(box.get_end() - Vec3(1))
  }
}
void source_velocity(const fsim_source& src, float t, float v[3]) {
  if (!src.velocity_oscillating) {
    for (int d = 0; d < 3; ++d) v[d] = src.velocity[d];
    return;
  }
  const float w = float(M_PI * double(t) / double(src.box_period));  // T w = M_PI*t/box_period_
  for (int d = 0; d < 3; ++d)
    v[d] = float(double(src.velocity[d]) +
                 0.5 * double(src.velocity2[d] - src.velocity[d]) * (double(std::cos(w)) + 1.0));
}
bool source_active(const fsim_source& src, float t) {
  return !src.timed || (t >= src.start_time && t <= src.end_time);
}

namespace {

// Boxes of DeleteFluidInSources (get_box(t) of every source), passed by value.
struct SourceRegions {
  int n;
  float lo[FSIM_MAX_SOURCES][3], hi[FSIM_MAX_SOURCES][3];
};
__device__ __forceinline__ bool in_regions(const SourceRegions& r, const float p[3]) {
  for (int q = 0; q < r.n; ++q) {
    bool in = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) in &= (p[d] >= r.lo[q][d]) & (p[d] <= r.hi[q][d]);  // Cube::IsInside
    if (in) return true;
  }
  return false;
}

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// mode 0: key from current position (upload); positions outside [0,N]
//         are counted as invalid.
// mode 1: advect by gvel*dt, clamp, delete in solids (MoveParticles).
// mode 1 extras: particles inside a source region get the dead key
// (DeleteFluidInSources right after MoveParticles); kout64 (optional) gets
// (new key << 32 | old key), so that a stable sort on it orders particles as
// the reference's rebuilt lists do when particles were appended to cell lists
// (the visiting order is by old cell, then list position).
__global__ void k_keys(float* __restrict__ part, int64_t cap, const uint32_t* __restrict__ kcur,
                       uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n,
                       LeafMap lm, SolidDesc sd, int mode, float dt,
                       unsigned long long* __restrict__ invalid, const SourceRegions reg,
                       unsigned long long* __restrict__ kout64) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  vout[i] = uint32_t(i);
  float* px = part;
  float* gx = part + 6 * cap;
  float p[3] = {px[i], px[cap + i], px[2 * cap + i]};
  if (mode == 1) {
    if (kcur[i] == kDeadKey) {
      kout[i] = kDeadKey;
      if (kout64) kout64[i] = ~0ull;
      return;
    }
    const float g[3] = {gx[i], gx[cap + i], gx[2 * cap + i]};
    int id[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      p[d] = fadd(p[d], fmul(g[d], dt));
      id[d] = int(floorf(p[d]));
    }
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (id[d] < 0) { id[d] = 0; p[d] = 0.f; }
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (id[d] >= lm.n[d]) { id[d] = lm.n[d]; p[d] = float(lm.n[d]); }
    px[i] = p[0];
    px[cap + i] = p[1];
    px[2 * cap + i] = p[2];
    uint32_t k = is_solid(sd, id[0], id[1], id[2]) ? kDeadKey : cell_key(lm, id[0], id[1], id[2]);
    if (reg.n > 0 && in_regions(reg, p)) k = kDeadKey;
    kout[i] = k;
    if (kout64)
      kout64[i] = (k == kDeadKey) ? ~0ull : ((static_cast<unsigned long long>(k) << 32) | kcur[i]);
  } else {
    bool ok = true;
    int id[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      ok &= (p[d] >= 0.f) && (p[d] <= float(lm.n[d]));
      id[d] = int(floorf(p[d]));
    }
    if (!ok) {
      atomicAdd(invalid, 1ull);
      kout[i] = kDeadKey;
      return;
    }
    kout[i] = cell_key(lm, id[0], id[1], id[2]);
  }
}

// Live particles = index of the first dead key: the keys are sorted and the
// dead key is the largest value.  One block narrows [lo, hi] (which holds
// that index; hi = n when no key is dead) by probing blockDim.x evenly spaced
// keys per round, about 1000x per round, instead of reading all n keys.
__global__ void k_count_live(const uint32_t* __restrict__ k, int64_t n, int64_t* cnt) {
  __shared__ int64_t s_lo, s_hi;
  __shared__ int s_first;
  if (threadIdx.x == 0) {
    s_lo = 0;
    s_hi = n;
  }
  __syncthreads();
  for (;;) {
    const int64_t lo = s_lo, hi = s_hi;
    if (lo >= hi) break;
    const int64_t nb = blockDim.x;
    const int64_t step = (hi - lo + nb - 1) / nb;
    const int64_t pr = lo + int64_t(threadIdx.x) * step;  // this thread's probe
    if (threadIdx.x == 0) s_first = INT_MAX;
    __syncthreads();
    if (pr < hi && k[pr] == kDeadKey) atomicMin(&s_first, int(threadIdx.x));
    __syncthreads();
    if (threadIdx.x == 0) {
      const int t = s_first;
      if (t == INT_MAX) {  // every probe live: the first dead key lies past the last probe
        const int64_t last = lo + ((hi - 1 - lo) / step) * step;
        s_lo = last + 1;
      } else {  // between the last live probe and probe t (dead)
        s_lo = t == 0 ? lo : lo + int64_t(t - 1) * step + 1;
        s_hi = lo + int64_t(t) * step;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) cnt[0] = s_lo;
}

// Four sorted keys per thread (one 16-byte load; key arrays start 256-byte
// aligned), so a warp streams 512 contiguous bytes per request.
constexpr int kKeysPerThread = 4;
__device__ __forceinline__ void load_keys4(const uint32_t* __restrict__ k, int64_t i0, int64_t n,
                                           uint32_t (&v)[kKeysPerThread]) {
  if (i0 + kKeysPerThread <= n) {
    const uint4 q = *reinterpret_cast<const uint4*>(k + i0);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
  } else {
#pragma unroll
    for (int j = 0; j < kKeysPerThread; ++j) v[j] = i0 + j < n ? k[i0 + j] : kDeadKey;
  }
}

// Permutes the first NF particle arrays (9: pos, vel, gvel; 6: pos, vel).
template <int NF>
__global__ void k_gather(const float* __restrict__ in, float* __restrict__ out, int64_t cap,
                         const uint32_t* __restrict__ perm, const int64_t* __restrict__ cnt) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = cnt[0];
  if (i >= n) return;
  const int64_t src = perm[i];
#pragma unroll
  for (int f = 0; f < NF; ++f) out[f * cap + i] = in[f * cap + src];
}

__global__ void k_mark_pleaf(const uint32_t* __restrict__ k, const int64_t* __restrict__ cnt,
                             uint8_t* __restrict__ flag) {
  const int64_t n = cnt[0];
  const int64_t i0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kKeysPerThread;
  if (i0 >= n) return;
  uint32_t v[kKeysPerThread];
  load_keys4(k, i0, n, v);
  uint32_t prev = i0 == 0 ? kDeadKey : (k[i0 - 1] >> 9);  // kDeadKey is no leaf id
#pragma unroll
  for (int j = 0; j < kKeysPerThread; ++j) {
    if (i0 + j >= n) break;
    const uint32_t l = v[j] >> 9;
    if (l != prev) flag[l] = 1;
    prev = l;
  }
}

__global__ void k_dilate(uint8_t* __restrict__ flag, LeafMap lm) {
  uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= lm.dense) return;
  if (flag[d] & 1) return;
  int lx, ly, lz;
  leaf_coords(lm, d, lx, ly, lz);
  if (!leaf_valid(lm, lx, ly, lz)) return;
  for (int dx = -1; dx <= 1; ++dx)
    for (int dy = -1; dy <= 1; ++dy)
      for (int dz = -1; dz <= 1; ++dz) {
        int ax = lx + dx, ay = ly + dy, az = lz + dz;
        if (!leaf_valid(lm, ax, ay, az)) continue;
        if (flag[leaf_id(lm, ax, ay, az)] & 1) {
          flag[d] = 2;
          return;
        }
      }
}

__global__ void k_scan_in(const uint8_t* __restrict__ flag, uint64_t* __restrict__ v, uint32_t n) {
  uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= n) return;
  uint8_t f = flag[d];
  v[d] = uint64_t(f & 1) | (uint64_t(f == 2) << 32);
}

__global__ void k_assign(const uint8_t* __restrict__ flag, const uint64_t* __restrict__ in,
                         const uint64_t* __restrict__ ex, int32_t* __restrict__ slot,
                         int32_t* __restrict__ leaf_of, uint32_t n, int64_t* cnt) {
  uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= n) return;
  const uint64_t tot = ex[n - 1] + in[n - 1];
  const int np = int(tot & 0xFFFFFFFFull);
  const int ng = int(tot >> 32);
  if (d == 0) {
    cnt[1] = np;
    cnt[2] = np + ng;
  }
  uint8_t f = flag[d];
  int s = -1;
  if (f & 1) s = int(ex[d] & 0xFFFFFFFFull);
  else if (f == 2) s = np + int(ex[d] >> 32);
  slot[d] = s;
  if (s >= 0) leaf_of[s] = int32_t(d);
}

__global__ void k_nbr(const int32_t* __restrict__ leaf_of, const int32_t* __restrict__ slot,
                      int32_t* __restrict__ nbr, int ng, LeafMap lm) {
  int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(ng) * 27) return;
  int s = int(t / 27), q = int(t % 27);
  int lx, ly, lz;
  leaf_coords(lm, uint32_t(leaf_of[s]), lx, ly, lz);
  int ax = lx + q / 9 - 1, ay = ly + (q / 3) % 3 - 1, az = lz + q % 3 - 1;
  int v = -1;
  if (leaf_valid(lm, ax, ay, az)) v = slot[leaf_id(lm, ax, ay, az)];
  nbr[t] = v;
}

__global__ void k_ranges(const uint32_t* __restrict__ k, const int64_t* __restrict__ cnt,
                         const int32_t* __restrict__ slot, uint2* __restrict__ cr,
                         uint2* __restrict__ lr) {
  const int64_t n = cnt[0];
  const int64_t i0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kKeysPerThread;
  if (i0 >= n) return;
  uint32_t v[kKeysPerThread + 2];  // the key before, the four keys, the key after
  {
    uint32_t q[kKeysPerThread];
    load_keys4(k, i0, n, q);
#pragma unroll
    for (int j = 0; j < kKeysPerThread; ++j) v[j + 1] = q[j];
  }
  v[0] = i0 == 0 ? kDeadKey : k[i0 - 1];  // kDeadKey: no live key equals it
  v[kKeysPerThread + 1] = i0 + kKeysPerThread < n ? k[i0 + kKeysPerThread] : kDeadKey;
#pragma unroll
  for (int j = 0; j < kKeysPerThread; ++j) {
    const int64_t i = i0 + j;
    if (i >= n) break;
    const uint32_t key = v[j + 1];
    // past the last live key, v holds kDeadKey, which ends every range
    const uint32_t before = v[j], after = v[j + 2];
    const bool cell_start = before != key, cell_end = after != key;
    if (!(cell_start || cell_end)) continue;
    const int s = slot[key >> 9];
    uint2* c = &cr[int64_t(s) * 512 + (key & 511u)];
    if (cell_start) c->x = uint32_t(i);
    if (cell_end) c->y = uint32_t(i + 1);
    if (cell_start && (before >> 9) != (key >> 9)) lr[s].x = uint32_t(i);
    if (cell_end && (after >> 9) != (key >> 9)) lr[s].y = uint32_t(i + 1);
  }
}

// ---- seeding (FlipSimulation::InitializePhiAndParticles restated) -------
struct SeedArgs {
  int npass;
  fsim_seed_pass pass[8];
  uint64_t seed;
  int nppc;
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float uniform01(uint64_t seed, int pass, int64_t cell, int draw,
                                           int d) {
  uint64_t s = mix64(seed ^ mix64((uint64_t(uint32_t(pass)) << 40) ^ uint64_t(cell)));
  uint64_t z = mix64(s + uint64_t(draw * 3 + d));
  return float(z >> 40) * (1.0f / 16777216.0f);
}
__device__ float shape_phi(const fsim_shape& sh, const float p[3]) {
  if (sh.kind == FSIM_SHAPE_CUBOID) {
    bool in = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) in &= (p[d] >= sh.a[d]) & (p[d] <= sh.b[d]);
    return in ? -1.0f : 1.0f;
  } else if (sh.kind == FSIM_SHAPE_SPHERE) {
    float dx = __fsub_rn(p[0], sh.a[0]), dy = __fsub_rn(p[1], sh.a[1]),
          dz = __fsub_rn(p[2], sh.a[2]);
    float l2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    return __fsub_rn(__fsqrt_rn(l2), sh.r);
  }
  return __fsub_rn(p[1], sh.a[1]);
}
__device__ float pass_phi(const fsim_seed_pass& ps, const float p[3]) {
  float phi = shape_phi(ps.shapes[0], p);
  for (int i = 1; i < ps.nshapes; ++i) phi = fminf(phi, shape_phi(ps.shapes[i], p));
  return phi;
}

// write == 0: count only (warp-aggregated atomic into cnt[5]);
// write == 1: reserve with the same aggregation and emit particles + keys.
__global__ void k_seed(const __grid_constant__ SeedArgs a, LeafMap lm, SolidDesc sd, int write,
                       unsigned long long* __restrict__ counter, float* __restrict__ part,
                       int64_t cap, uint32_t* __restrict__ kout, uint32_t* __restrict__ vout) {
  const int64_t ncell = int64_t(lm.n[0]) * lm.n[1] * lm.n[2];
  int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  int count = 0;
  int i = 0, j = 0, k = 0;
  const bool active = c < ncell;
  if (active) {
    i = int(c / (int64_t(lm.n[1]) * lm.n[2]));
    j = int((c / lm.n[2]) % lm.n[1]);
    k = int(c % lm.n[2]);
  }
  const bool use = active && !is_solid(sd, i, j, k);
  const float org[3] = {float(i), float(j), float(k)};
  const float ctr[3] = {__fadd_rn(org[0], 0.5f), __fadd_rn(org[1], 0.5f), __fadd_rn(org[2], 0.5f)};
  if (use) {
    for (int ps = 0; ps < a.npass; ++ps) {
      if (!(pass_phi(a.pass[ps], ctr) < 0.f)) continue;
      if (count >= a.nppc) continue;
      int pi = 0, draw = 0;
      for (int att = 0; att < 32 && pi < a.nppc; ++att, ++draw) {
        float pp[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
          pp[d] = __fadd_rn(org[d], __fmul_rn(uniform01(a.seed, ps, c, draw, d), 1.0f));
        if (pass_phi(a.pass[ps], pp) > 0.f) continue;
        ++pi;
        ++att;
        ++count;
      }
    }
  }
  // warp-aggregated reservation
  const unsigned lane = threadIdx.x & 31;
  int incl = count;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= unsigned(o)) incl += v;
  }
  const int wtot = __shfl_sync(0xffffffffu, incl, 31);
  unsigned long long base = 0;
  if (lane == 31 && wtot > 0) base = atomicAdd(counter, (unsigned long long)wtot);
  base = __shfl_sync(0xffffffffu, base, 31);
  if (!write || count == 0) return;
  int64_t o = int64_t(base) + incl - count;
  const uint32_t key = cell_key(lm, i, j, k);
  for (int ps = 0; ps < a.npass; ++ps) {
    if (!(pass_phi(a.pass[ps], ctr) < 0.f)) continue;
    // cells already holding nppc particles skip the pass (count is
    // re-derived in the same order as the counting sweep)
    int before = int(o - (int64_t(base) + incl - count));
    if (before >= a.nppc) continue;
    int pi = 0, draw = 0;
    for (int att = 0; att < 32 && pi < a.nppc; ++att, ++draw) {
      float pp[3];
#pragma unroll
      for (int d = 0; d < 3; ++d)
        pp[d] = __fadd_rn(org[d], __fmul_rn(uniform01(a.seed, ps, c, draw, d), 1.0f));
      if (pass_phi(a.pass[ps], pp) > 0.f) continue;
      if (o < cap) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          part[d * cap + o] = pp[d];
          part[(3 + d) * cap + o] = a.pass[ps].velocity[d];
          part[(6 + d) * cap + o] = a.pass[ps].velocity[d];
        }
        kout[o] = key;
        vout[o] = uint32_t(o);
      }
      ++o;
      ++pi;
      ++att;
    }
  }
}

__global__ void k_perturb(float* __restrict__ part, int64_t cap, int64_t n, float sigma,
                          uint64_t seed) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float u1 = uniform01(seed, 1 << 20, i, 0, d);
    float u2 = uniform01(seed, 1 << 20, i, 1, d);
    float g = sqrtf(-2.0f * logf(1.0f - u1)) * cosf(6.2831853f * u2);
    float v = __fadd_rn(part[(3 + d) * cap + i], __fmul_rn(sigma, g));
    part[(3 + d) * cap + i] = v;
    part[(6 + d) * cap + i] = v;
  }
}

// ---- AddContributionFromSources (common/flip_simulation.cc:1207-1270) ----
// Work items are (source, cell) pairs, sources in order and each source's
// cells x-major, so that particles land in the reference's list order after
// an exclusive scan of the per-item counts.
struct SourceGen {
  int nsrc;
  int lo[FSIM_MAX_SOURCES][3], dim[FSIM_MAX_SOURCES][3];  // cell range of each source
  int64_t begin[FSIM_MAX_SOURCES + 1];                    // first work item of each source
  float blo[FSIM_MAX_SOURCES][3], bhi[FSIM_MAX_SOURCES][3];  // get_box(t)
  float vel[FSIM_MAX_SOURCES][3];
  int pass[FSIM_MAX_SOURCES];
  uint64_t seed;
  int nppc;
};

// count == nullptr: write pass (offsets from the scan)
__global__ void k_source(const __grid_constant__ SourceGen g, LeafMap lm, uint32_t* __restrict__ cnt,
                         const uint32_t* __restrict__ off, float* __restrict__ part, int64_t cap,
                         int64_t base, uint32_t* __restrict__ kout) {
  const int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= g.begin[g.nsrc]) return;
  int q = 0;
  while (w >= g.begin[q + 1]) ++q;
  const int64_t c = w - g.begin[q];
  const int dy = g.dim[q][1], dz = g.dim[q][2];
  const int i = g.lo[q][0] + int(c / (int64_t(dy) * dz));
  const int j = g.lo[q][1] + int((c / dz) % dy);
  const int k = g.lo[q][2] + int(c % dz);
  const int64_t cell = (int64_t(i) * lm.n[1] + j) * lm.n[2] + k;
  const float org[3] = {float(i), float(j), float(k)};
  int pi = 0;
  int64_t o = cnt ? 0 : base + off[w];
  const uint32_t key = cell_key(lm, i, j, k);
  for (int att = 0; att < 32 && pi < g.nppc; ++att) {
    float pp[3];
    bool in = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      pp[d] = __fadd_rn(org[d], __fmul_rn(uniform01(g.seed, g.pass[q], cell, att, d), 1.0f));
      in &= (pp[d] >= g.blo[q][d]) & (pp[d] <= g.bhi[q][d]);
    }
    if (!in) continue;
    if (!cnt) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        part[d * cap + o] = pp[d];
        part[(3 + d) * cap + o] = g.vel[q][d];
        part[(6 + d) * cap + o] = g.vel[q][d];
      }
      kout[o] = key;
      ++o;
    }
    ++pi;
  }
  if (cnt) cnt[w] = uint32_t(pi);
}

// DeleteFluidInSources on sorted particles (per-stage entry): dead keys
__global__ void k_delete_in_regions(const float* __restrict__ part, int64_t cap,
                                    uint32_t* __restrict__ keys, int64_t n,
                                    const SourceRegions reg,
                                    unsigned long long* __restrict__ ndead) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n || keys[i] == kDeadKey) return;
  const float p[3] = {part[i], part[cap + i], part[2 * cap + i]};
  if (in_regions(reg, p)) {
    keys[i] = kDeadKey;
    atomicAdd(ndead, 1ull);
  }
}

// adjacent pairs out of order (k[i] > k[i+1])
__global__ void k_count_desc(const uint32_t* __restrict__ k, int64_t n,
                             unsigned long long* __restrict__ cnt) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i + 1 < n && k[i] > k[i + 1]) atomicAdd(cnt, 1ull);
}

__global__ void k_hi_keys(const unsigned long long* __restrict__ k64, uint32_t* __restrict__ k,
                          int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) k[i] = uint32_t(k64[i] >> 32);
}

inline unsigned nblk(int64_t n, int b) { return unsigned((n + b - 1) / b); }

SourceRegions regions_at(const fsim_sim* s, float t) {
  SourceRegions r;
  memset(&r, 0, sizeof(r));
  r.n = int(s->sources.size());
  for (int q = 0; q < r.n; ++q) source_box(s->sources[size_t(q)], t, r.lo[q], r.hi[q]);
  return r;
}

}  // namespace

int launch_keys_from_positions(fsim_sim* s, int mode, float dt) {
  const int64_t n = s->n_total;
  FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 3, 0, sizeof(int64_t), s->stream));
  SourceRegions reg;
  memset(&reg, 0, sizeof(reg));
  if (mode == 1 && s->delete_in_sources) reg = regions_at(s, s->src_time);
  unsigned long long* k64 = nullptr;
  if (mode == 1 && s->composite_sort) {
    if (n > s->cap64) {
      for (int b = 0; b < 2; ++b) {
        if (s->keys64[b]) cudaFree(s->keys64[b]);
        s->keys64[b] = nullptr;
        FSIM_CK(s, cudaMalloc(&s->keys64[b], size_t(std::max<int64_t>(n, 1)) * 8));
      }
      s->cap64 = n;
    }
    k64 = reinterpret_cast<unsigned long long*>(s->keys64[1]);
  }
  FSIM_LAUNCH(s, "advect_keys", k_keys, nblk(n, 256), 256, 0, s->part[s->cur], s->cap_p,
              s->keys[0], s->keys[1], s->vals[1], n, s->lm, s->solid, mode, dt,
              reinterpret_cast<unsigned long long*>(s->d_cnt + 3), reg, k64);
  s->delete_in_sources = false;
  return FSIM_OK;
}

// Sorts keys[1]/vals[1] (n_total entries) into keys[0]/vals[0], gathers the
// particles into the other buffer and rebuilds the leaf topology.
int rebuild_topology(fsim_sim* s) {
  const int64_t n = s->n_total;
  const int bits = key_bits(s->lm);
  if (s->composite_sort) {
    // stable sort on (new key << 32 | old key), then the new keys back
    unsigned long long* k64[2] = {reinterpret_cast<unsigned long long*>(s->keys64[0]),
                                  reinterpret_cast<unsigned long long*>(s->keys64[1])};
    size_t need = 0;
    FSIM_CK(s, cub::DeviceRadixSort::SortPairs(nullptr, need, k64[1], k64[0], s->vals[1],
                                               s->vals[0], n, 0, 32 + bits, s->stream));
    if (need > s->sort_tmp_bytes) {
      if (s->sort_tmp) cudaFree(s->sort_tmp);
      s->sort_tmp = nullptr;
      FSIM_CK(s, cudaMalloc(&s->sort_tmp, need));
      s->sort_tmp_bytes = need;
    }
    if (n > 0) {
      fsim::ProfScope ps(s, "radix_sort64(cub)");
      FSIM_CK(s, cub::DeviceRadixSort::SortPairs(s->sort_tmp, need, k64[1], k64[0], s->vals[1],
                                                 s->vals[0], n, 0, 32 + bits, s->stream));
    }
    FSIM_LAUNCH(s, "new_keys", k_hi_keys, nblk(n, 256), 256, 0, k64[0], s->keys[0], n);
    s->composite_sort = false;
    return rebuild_after_sort(s);
  }
  // radix sort (stable)
  size_t need = 0;
  FSIM_CK(s, cub::DeviceRadixSort::SortPairs(nullptr, need, s->keys[1], s->keys[0], s->vals[1],
                                             s->vals[0], n, 0, bits, s->stream));
  if (need > s->sort_tmp_bytes) {
    if (s->sort_tmp) cudaFree(s->sort_tmp);
    s->sort_tmp = nullptr;
    FSIM_CK(s, cudaMalloc(&s->sort_tmp, need));
    s->sort_tmp_bytes = need;
  }
  if (n > 0) {
    fsim::ProfScope ps(s, "radix_sort(cub)");
    FSIM_CK(s, cub::DeviceRadixSort::SortPairs(s->sort_tmp, need, s->keys[1], s->keys[0],
                                               s->vals[1], s->vals[0], n, 0, bits, s->stream));
  }
  return rebuild_after_sort(s);
}

// keys[0]/vals[0] hold the sorted keys and permutation of n_total particles
int rebuild_after_sort(fsim_sim* s, bool gather) {
  const int64_t n = s->n_total;
  FSIM_CK(s, cudaMemsetAsync(s->d_cnt, 0, 3 * sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "count_live", k_count_live, 1, 1024, 0, s->keys[0], n, s->d_cnt);
  if (gather) {
    // a velocity upload still in flight on the I/O stream (fsim_step_host)
    if (s->io_vel_pending) {
      FSIM_CK(s, cudaStreamWaitEvent(s->stream, s->ev_io, 0));
      s->io_vel_pending = false;
    }
    if (s->gather_skip_gvel) {
      FSIM_LAUNCH(s, "gather_particles", k_gather<6>, nblk(n, 256), 256, 0, s->part[s->cur],
                  s->part[s->cur ^ 1], s->cap_p, s->vals[0], s->d_cnt);
    } else {
      FSIM_LAUNCH(s, "gather_particles", k_gather<9>, nblk(n, 256), 256, 0, s->part[s->cur],
                  s->part[s->cur ^ 1], s->cap_p, s->vals[0], s->d_cnt);
    }
    s->cur ^= 1;
  }
  // leaves
  const uint32_t D = s->lm.dense;
  FSIM_CK(s, cudaMemsetAsync(s->d_flag, 0, D, s->stream));
  FSIM_LAUNCH(s, "mark_leaves", k_mark_pleaf, nblk(n, 256 * kKeysPerThread), 256, 0, s->keys[0], s->d_cnt,
              s->d_flag);
  FSIM_LAUNCH(s, "dilate_leaves", k_dilate, nblk(D, 256), 256, 0, s->d_flag, s->lm);
  FSIM_LAUNCH(s, "scan_input", k_scan_in, nblk(D, 256), 256, 0, s->d_flag, s->d_scan, D);
  uint64_t* scan_out = s->d_scan + D;
  size_t sneed = 0;
  FSIM_CK(s, cub::DeviceScan::ExclusiveSum(nullptr, sneed, s->d_scan, scan_out, int(D), s->stream));
  if (sneed > s->scan_tmp_bytes) {
    if (s->scan_tmp) cudaFree(s->scan_tmp);
    s->scan_tmp = nullptr;
    FSIM_CK(s, cudaMalloc(&s->scan_tmp, sneed));
    s->scan_tmp_bytes = sneed;
  }
  {
    fsim::ProfScope ps(s, "leaf_scan(cub)");
    FSIM_CK(s, cub::DeviceScan::ExclusiveSum(s->scan_tmp, sneed, s->d_scan, scan_out, int(D),
                                             s->stream));
  }
  FSIM_LAUNCH(s, "assign_slots", k_assign, nblk(D, 256), 256, 0, s->d_flag, s->d_scan, scan_out,
              s->d_slot, s->d_leaf_id, D, s->d_cnt);
  FSIM_CK(s, cudaMemcpyAsync(s->h_cnt, s->d_cnt, 3 * sizeof(int64_t), cudaMemcpyDeviceToHost,
                             s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  s->n_live = s->h_cnt[0];
  s->n_total = s->n_live;
  s->n_pleaf = int(s->h_cnt[1]);
  s->n_gleaf = int(s->h_cnt[2]);
  int rc = ensure_leaf_capacity(s, s->n_gleaf, s->n_pleaf);
  if (rc != FSIM_OK) return rc;
  FSIM_LAUNCH(s, "neighbour_table", k_nbr, nblk(int64_t(s->n_gleaf) * 27, 256), 256, 0,
              s->d_leaf_id, s->d_slot, s->d_nbr, s->n_gleaf, s->lm);
  if (s->n_pleaf > 0) {
    FSIM_CK(s, cudaMemsetAsync(s->d_cell_range, 0, size_t(s->n_pleaf) * 512 * sizeof(uint2),
                               s->stream));
    FSIM_CK(s, cudaMemsetAsync(s->d_leaf_range, 0, size_t(s->n_pleaf) * sizeof(uint2), s->stream));
  }
  FSIM_LAUNCH(s, "cell_ranges", k_ranges, nblk(s->n_live, 256 * kKeysPerThread), 256, 0, s->keys[0], s->d_cnt,
              s->d_slot, s->d_cell_range, s->d_leaf_range);
  s->have_topology = true;
  s->deleted_outside = false;
  return FSIM_OK;
}

int seed_fluid(fsim_sim* s, const fsim_seed_pass* passes, int npasses, uint64_t seed) {
  if (npasses < 0 || npasses > 8) return fail(s, FSIM_ERR_INVALID, "npasses must be in [0,8]");
  SeedArgs a;
  memset(&a, 0, sizeof(a));
  a.npass = npasses;
  for (int i = 0; i < npasses; ++i) {
    if (passes[i].nshapes < 1 || passes[i].nshapes > FSIM_MAX_SHAPES)
      return fail(s, FSIM_ERR_INVALID, "each seed pass needs 1..8 shapes");
    a.pass[i] = passes[i];
  }
  a.seed = seed;
  a.nppc = s->cfg.nparticles_per_cell;
  const int64_t ncell = int64_t(s->lm.n[0]) * s->lm.n[1] * s->lm.n[2];
  unsigned long long* ctr = reinterpret_cast<unsigned long long*>(s->d_cnt + 5);
  FSIM_CK(s, cudaMemsetAsync(ctr, 0, sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "seed_count", k_seed, nblk(ncell, 256), 256, 0, a, s->lm, s->solid, 0, ctr,
              s->part[s->cur], s->cap_p, s->keys[1], s->vals[1]);
  FSIM_CK(s, cudaMemcpyAsync(s->h_cnt + 5, s->d_cnt + 5, sizeof(int64_t), cudaMemcpyDeviceToHost,
                             s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  const int64_t total = s->h_cnt[5];
  if (total > s->cap_p)
    return fail(s, FSIM_ERR_CAPACITY, "seeded particle count exceeds max_particles");
  FSIM_CK(s, cudaMemsetAsync(ctr, 0, sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "seed_write", k_seed, nblk(ncell, 256), 256, 0, a, s->lm, s->solid, 1, ctr,
              s->part[s->cur], s->cap_p, s->keys[1], s->vals[1]);
  s->n_total = total;
  return rebuild_topology(s);
}

// Upload helper: keys (mode 0) are in keys[1]; when they are already in cell
// order (particles that came from a download) the sort and the gather are
// skipped.  Returns FSIM_OK and sets *invalid to the number of positions
// outside [0, N].
int rebin_uploaded(fsim_sim* s, int64_t* invalid) {
  const int64_t n = s->n_total;
  FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 7, 0, sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "count_unsorted", k_count_desc, nblk(n, 256), 256, 0, s->keys[1], n,
              reinterpret_cast<unsigned long long*>(s->d_cnt + 7));
  FSIM_CK(s, cudaMemcpyAsync(s->h_cnt + 3, s->d_cnt + 3, 5 * sizeof(int64_t),
                             cudaMemcpyDeviceToHost, s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  *invalid = s->h_cnt[3];
  if (*invalid) return FSIM_OK;
  if (s->h_cnt[7] == 0) {
    std::swap(s->keys[0], s->keys[1]);  // sorted already: keep the order
    return rebuild_after_sort(s, false);
  }
  return rebuild_topology(s);
}

int add_source_particles(fsim_sim* s, float t) {
  SourceGen g;
  memset(&g, 0, sizeof(g));
  g.seed = s->seed;
  g.nppc = s->cfg.nparticles_per_cell;
  const int64_t call = s->source_calls++;
  int64_t items = 0;
  for (size_t q = 0; q < s->sources.size(); ++q) {
    const fsim_source& src = s->sources[q];
    g.begin[g.nsrc] = items;
    if (!source_active(src, t)) continue;
    float lo[3], hi[3];
    source_box(src, t, lo, hi);
    int a[3], b[3];
    bool empty = false;
    for (int d = 0; d < 3; ++d) {
      // Coord(float) truncates; the domain box is [0, N-1]
      a[d] = std::max(int(lo[d]), 0);
      b[d] = std::min(int(hi[d]), s->lm.n[d] - 1);
      empty |= b[d] < a[d];
    }
    if (empty) continue;
    const int r = g.nsrc;
    for (int d = 0; d < 3; ++d) {
      g.lo[r][d] = a[d];
      g.dim[r][d] = b[d] - a[d] + 1;
      g.blo[r][d] = lo[d];
      g.bhi[r][d] = hi[d];
    }
    source_velocity(src, t, g.vel[r]);
    g.pass[r] = (1 << 22) + int((call & 0x1FFFF) * 32) + int(q);
    g.begin[r] = items;
    items += int64_t(g.dim[r][0]) * g.dim[r][1] * g.dim[r][2];
    ++g.nsrc;
  }
  g.begin[g.nsrc] = items;
  if (items == 0) return FSIM_OK;
  // counts, exclusive scan, then the particles after the current ones
  size_t sneed = 0;
  uint32_t* cnt = nullptr;
  FSIM_CK(s, cub::DeviceScan::ExclusiveSum(nullptr, sneed, cnt, cnt, int(items + 1), s->stream));
  const size_t cnt_bytes = ((size_t(items + 1) * 4 + 255) / 256) * 256;
  if (cnt_bytes * 2 + sneed > s->src_tmp_bytes) {
    if (s->src_tmp) cudaFree(s->src_tmp);
    s->src_tmp = nullptr;
    FSIM_CK(s, cudaMalloc(&s->src_tmp, cnt_bytes * 2 + sneed));
    s->src_tmp_bytes = cnt_bytes * 2 + sneed;
  }
  cnt = static_cast<uint32_t*>(s->src_tmp);
  uint32_t* off = reinterpret_cast<uint32_t*>(static_cast<char*>(s->src_tmp) + cnt_bytes);
  void* stmp = static_cast<char*>(s->src_tmp) + 2 * cnt_bytes;
  FSIM_CK(s, cudaMemsetAsync(cnt, 0, size_t(items + 1) * 4, s->stream));
  FSIM_LAUNCH(s, "source_count", k_source, nblk(items, 256), 256, 0, g, s->lm, cnt,
              static_cast<const uint32_t*>(nullptr), s->part[s->cur], s->cap_p, int64_t(0),
              s->keys[0]);
  FSIM_CK(s, cub::DeviceScan::ExclusiveSum(stmp, sneed, cnt, off, int(items + 1), s->stream));
  uint32_t added = 0;
  FSIM_CK(s, cudaMemcpyAsync(&added, off + items, 4, cudaMemcpyDeviceToHost, s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  if (added == 0) return FSIM_OK;
  if (s->n_total + int64_t(added) > s->cap_p) {
    // grow by a quarter more than needed (sources keep adding); the current
    // particles and keys move over
    const int rc = grow_particle_capacity(s, (s->n_total + int64_t(added)) * 5 / 4 + 1024);
    if (rc) return rc;
  }
  FSIM_LAUNCH(s, "source_write", k_source, nblk(items, 256), 256, 0, g, s->lm,
              static_cast<uint32_t*>(nullptr), off, s->part[s->cur], s->cap_p, s->n_total,
              s->keys[0]);
  s->n_total += added;
  s->n_live = s->n_total;
  s->composite_sort = true;
  return FSIM_OK;
}

int delete_in_sources(fsim_sim* s, float t) {
  if (s->sources.empty()) return FSIM_OK;
  // dead keys are counted with DeleteOutsideParticles' (d_cnt[6]) until the next sort
  if (!s->deleted_outside) FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 6, 0, 8, s->stream));
  FSIM_LAUNCH(s, "delete_in_sources", k_delete_in_regions, nblk(s->n_total, 256), 256, 0,
              s->part[s->cur], s->cap_p, s->keys[0], s->n_total, regions_at(s, t),
              reinterpret_cast<unsigned long long*>(s->d_cnt + 6));
  return FSIM_OK;
}

int perturb(fsim_sim* s, float sigma, uint64_t seed) {
  FSIM_LAUNCH(s, "perturb_velocity", k_perturb, nblk(s->n_live, 256), 256, 0, s->part[s->cur],
              s->cap_p, s->n_live, sigma, seed);
  return FSIM_OK;
}

}  // namespace fsim
