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
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "fsim_internal.cuh"

namespace fsim {

namespace {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// mode 0: key from current position (upload); positions outside [0,N]
//         are counted as invalid.
// mode 1: advect by gvel*dt, clamp, delete in solids (MoveParticles).
__global__ void k_keys(float* __restrict__ part, int64_t cap, const uint32_t* __restrict__ kcur,
                       uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int64_t n,
                       LeafMap lm, SolidDesc sd, int mode, float dt,
                       unsigned long long* __restrict__ invalid) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  vout[i] = uint32_t(i);
  float* px = part;
  float* gx = part + 6 * cap;
  float p[3] = {px[i], px[cap + i], px[2 * cap + i]};
  if (mode == 1) {
    if (kcur[i] == kDeadKey) {
      kout[i] = kDeadKey;
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
    kout[i] = is_solid(sd, id[0], id[1], id[2]) ? kDeadKey : cell_key(lm, id[0], id[1], id[2]);
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

__global__ void k_count_live(const uint32_t* __restrict__ k, int64_t n, int64_t* cnt) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (k[i] != kDeadKey && (i + 1 == n || k[i + 1] == kDeadKey)) cnt[0] = i + 1;
}

__global__ void k_gather(const float* __restrict__ in, float* __restrict__ out, int64_t cap,
                         const uint32_t* __restrict__ perm, const int64_t* __restrict__ cnt) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = cnt[0];
  if (i >= n) return;
  const int64_t src = perm[i];
#pragma unroll
  for (int f = 0; f < 9; ++f) out[f * cap + i] = in[f * cap + src];
}

__global__ void k_mark_pleaf(const uint32_t* __restrict__ k, const int64_t* __restrict__ cnt,
                             uint8_t* __restrict__ flag) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= cnt[0]) return;
  uint32_t l = k[i] >> 9;
  if (i == 0 || (k[i - 1] >> 9) != l) flag[l] = 1;
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
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t n = cnt[0];
  if (i >= n) return;
  const uint32_t key = k[i];
  const int s = slot[key >> 9];
  uint2* c = &cr[int64_t(s) * 512 + (key & 511u)];
  if (i == 0 || k[i - 1] != key) c->x = uint32_t(i);
  if (i + 1 == n || k[i + 1] != key) c->y = uint32_t(i + 1);
  if (i == 0 || (k[i - 1] >> 9) != (key >> 9)) lr[s].x = uint32_t(i);
  if (i + 1 == n || (k[i + 1] >> 9) != (key >> 9)) lr[s].y = uint32_t(i + 1);
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

inline unsigned nblk(int64_t n, int b) { return unsigned((n + b - 1) / b); }

}  // namespace

int launch_keys_from_positions(fsim_sim* s, int mode, float dt) {
  const int64_t n = s->n_total;
  FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 3, 0, sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "advect_keys", k_keys, nblk(n, 256), 256, 0, s->part[s->cur], s->cap_p,
              s->keys[0], s->keys[1], s->vals[1], n, s->lm, s->solid, mode, dt,
              reinterpret_cast<unsigned long long*>(s->d_cnt + 3));
  return FSIM_OK;
}

// Sorts keys[1]/vals[1] (n_total entries) into keys[0]/vals[0], gathers the
// particles into the other buffer and rebuilds the leaf topology.
int rebuild_topology(fsim_sim* s) {
  const int64_t n = s->n_total;
  const int bits = key_bits(s->lm);
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
  FSIM_CK(s, cudaMemsetAsync(s->d_cnt, 0, 3 * sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "count_live", k_count_live, nblk(n, 256), 256, 0, s->keys[0], n, s->d_cnt);
  FSIM_LAUNCH(s, "gather_particles", k_gather, nblk(n, 256), 256, 0, s->part[s->cur],
              s->part[s->cur ^ 1], s->cap_p, s->vals[0], s->d_cnt);
  s->cur ^= 1;
  // leaves
  const uint32_t D = s->lm.dense;
  FSIM_CK(s, cudaMemsetAsync(s->d_flag, 0, D, s->stream));
  FSIM_LAUNCH(s, "mark_leaves", k_mark_pleaf, nblk(n, 256), 256, 0, s->keys[0], s->d_cnt,
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
  FSIM_LAUNCH(s, "cell_ranges", k_ranges, nblk(s->n_live, 256), 256, 0, s->keys[0], s->d_cnt,
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

int perturb(fsim_sim* s, float sigma, uint64_t seed) {
  FSIM_LAUNCH(s, "perturb_velocity", k_perturb, nblk(s->n_live, 256), 256, 0, s->part[s->cur],
              s->cap_p, s->n_live, sigma, seed);
  return FSIM_OK;
}

}  // namespace fsim
