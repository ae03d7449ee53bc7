// k_grid.cu -- grid stages of the FLIP step on the sparse 8^3 brick layout.
//
// P2G (FlipSimulation::TransferParticlesToGrid, common/flip_simulation.cc:
// 809-923, with ScatterWeight<D> :927-1009) runs in two passes, each particle
// visited once.  Pass 1 (one CTA per particle leaf) splats the leaf's
// particles into a 10^3 node block (the leaf's nodes and the layer around
// them, the halo the reference buffers per leaf) in shared-memory fixed-point
// accumulators and writes the block out.  Pass 2 (one CTA per grid leaf)
// sums, per node, its own block entry and the neighbour blocks that cover it,
// and writes each node exactly once: no global atomics.  The fused pass 2
// folds the rest of the per-node work of the step into that write:
// normalisation with the 1e-5 cut, ApplyBoundaryConditions,
// SaveGridVelocities, AddGravity and the second ApplyBoundaryConditions.
//
// The remaining kernels restate ComputeDivergence (:716-736),
// UpdateVelocityFromPressure (:739-778) fused with GetVelocityUpdate
// (:781-801) and the CFL max (:460-488), and the per-stage variants.
// All arithmetic that the reference does in float is done with explicit
// round-to-nearest intrinsics so that nvcc cannot contract it into FMAs.
#include <cstring>

#include "fsim_internal.cuh"

namespace fsim {

namespace {

struct GridArgs {
  const float* part;
  int64_t cap;
  const uint32_t* keys;
  const int32_t* leaf_id;
  const int32_t* nbr;
  const uint2* cell_range;
  const uint2* leaf_range;
  int n_pleaf, n_gleaf;
  int check_dead;
  LeafMap lm;
  SolidDesc sd;
  float* vel;
  float* vold;
  float* weight;
  uint32_t* vel_on;
  uint32_t* vold_on;
  int8_t* marker;
  const float* pres;
  float* div;
  float dt, fx, fy, fz;
  int64_t* cnt;
  unsigned long long* p2g_nodes;  // P2G pass 1 output: [particle leaf][6][1000]
  uint32_t* p2g_touch;            // [particle leaf][32] touched bits of the 1000 nodes
  uint32_t* p2g_low;              // [0]: count; then slot * 1536 + D * 512 + voxel of the
                                  // low-weight faces pass 2 leaves to k_p2g_low
};

__device__ __forceinline__ void origin_of(const GridArgs& a, int s, int o[3]) {
  int lx, ly, lz;
  leaf_coords(a.lm, uint32_t(a.leaf_id[s]), lx, ly, lz);
  o[0] = lx * 8; o[1] = ly * 8; o[2] = lz * 8;
}

__device__ __forceinline__ int nb_index(int dx, int dy, int dz) {
  return (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1);
}

// neighbour-leaf direction of local coordinate t in [-1, 8]
__device__ __forceinline__ int side(int t) { return t < 0 ? -1 : (t > 7 ? 1 : 0); }

__device__ __forceinline__ bool in_box(const int n[3], int i, int j, int k) {
  return i >= 0 && j >= 0 && k >= 0 && i < n[0] && j < n[1] && k < n[2];
}

// P2G sums are accumulated in 64-bit fixed point (2^-32 units): integer
// atomics commute, so the sums -- and every step -- are bitwise reproducible
// whatever order the CTA's threads add in.  Each float term w*u (and w) is
// converted exactly up to 2^-33; the result is then the correctly rounded
// float of the exact sum of the terms.  Range: |sum| < 2^31 per face.
constexpr float kFixScale = 4294967296.0f;  // 2^32
__device__ __forceinline__ unsigned long long to_fix(float x) {
  return static_cast<unsigned long long>(__float2ll_rn(__fmul_rn(x, kFixScale)));
}
// The float nearest the fixed-point value (one rounding; the 2^-32 scaling is
// exact for the sums a grid can hold).
__device__ __forceinline__ float from_fix(unsigned long long v) {
  return __fmul_rn(__ll2float_rn(static_cast<long long>(v)), 1.0f / 4294967296.0f);
}

// P2G in two passes, each particle visited once.
//
// Pass 1 (k_p2g_cells, one CTA per particle leaf): each thread takes whole
// cells of the leaf.  Per component D the particles of a cell reach an
// 18-node box (3 node positions on each tangential axis -- the stencil starts
// at the cell or one below it, by the side of the cell centre the particle is
// on -- and 2 on the normal axis); the thread sums the cell's particles into
// that box in registers, in list order, and adds each reached node into the
// CTA's 10^3 node block (the leaf's 8^3 nodes and the one-node layer around
// them) with one fixed-point shared atomic.  The block is written out per
// leaf: nodes[6][1000] (value sums for D = 0..2, then weight sums) and 1000
// touched bits.
//
// Pass 2 (k_p2g_nodes, one CTA per grid leaf): each node adds its own leaf's
// entry and the entries of the neighbour particle leaves whose outer layer
// covers it (a face node 1, an edge node 3, a corner node 7), then
// normalises.  Fixed-point sums are exact, so the result does not depend on
// which pass or CTA added a term: it equals the one-pass sum over all cells.
constexpr int kNodeBlock = 1000;  // 10^3 node positions, local coordinates -1..8

__device__ __forceinline__ int node_index(int li, int lj, int lk) {
  return ((li + 1) * 10 + (lj + 1)) * 10 + (lk + 1);
}

// Bits t = (i * e1 + j) * e2 + k of a component-D box (extent 2 on axis D,
// 3 on the others) whose coordinate on axis ax is in the position set m.
// A particle reaches the box nodes in the AND of its per-axis sets.
__host__ __device__ constexpr unsigned box_axis_mask(int D, int ax, unsigned m) {
  unsigned r = 0u;
  const int e0 = D == 0 ? 2 : 3, e1 = D == 1 ? 2 : 3, e2 = D == 2 ? 2 : 3;
  for (int i = 0; i < e0; ++i)
    for (int j = 0; j < e1; ++j)
      for (int k = 0; k < e2; ++k) {
        const int c = ax == 0 ? i : (ax == 1 ? j : k);
        if ((m >> c) & 1u) r |= 1u << ((i * e1 + j) * e2 + k);
      }
  return r;
}

__global__ void __launch_bounds__(256) k_p2g_cells(const __grid_constant__ GridArgs a) {
  __shared__ unsigned long long sv[3][kNodeBlock];
  __shared__ unsigned long long sw[3][kNodeBlock];
  __shared__ uint8_t touched[1024];
  const int s = blockIdx.x;  // particle leaf
  const int tid = threadIdx.x;
  for (int v = tid; v < kNodeBlock; v += 256) {
    sv[0][v] = 0ull; sv[1][v] = 0ull; sv[2][v] = 0ull;
    sw[0][v] = 0ull; sw[1][v] = 0ull; sw[2][v] = 0ull;
  }
  for (int v = tid; v < 1024; v += 256) touched[v] = 0;
  __syncthreads();
  int org[3];
  origin_of(a, s, org);
  const float* px = a.part;
  const int64_t cap = a.cap;
  for (int c = tid; c < 512; c += 256) {
    const int cl[3] = {c >> 6, (c >> 3) & 7, c & 7};
    const uint2 rg = a.cell_range[int64_t(s) * 512 + c];
    if (rg.x >= rg.y) continue;
    const int g[3] = {org[0] + cl[0], org[1] + cl[1], org[2] + cl[2]};
#pragma unroll
    for (int D = 0; D < 3; ++D) {
      // box extents: 3 on the tangential axes, 2 on the normal axis D
      constexpr int kE = 3;
      const int e0 = D == 0 ? 2 : kE, e1 = D == 1 ? 2 : kE, e2 = D == 2 ? 2 : kE;
      float am[18], aw[18];
#pragma unroll
      for (int t = 0; t < 18; ++t) { am[t] = 0.f; aw[t] = 0.f; }
      unsigned reach = 0u;  // box nodes some particle's 8-node stencil includes
      for (uint32_t q = rg.x; q < rg.y; ++q) {
        if (a.check_dead && a.keys[q] == kDeadKey) continue;
        const float uD = px[(3 + D) * cap + q];
        float w1[3][3];   // per-axis weights over the box positions
        unsigned m1[3];   // per-axis reached positions
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          const float pa = px[ax * cap + q];
          const float ga = float(g[ax]);
          if (ax == D) {
            const float x = __fsub_rn(pa, ga);
            w1[ax][0] = __fsub_rn(1.0f, x); w1[ax][1] = x; w1[ax][2] = 0.f;
            m1[ax] = 3u;
          } else {
            const float lo = __fadd_rn(ga, 0.5f);
            if (pa < lo) {  // stencil starts one below the cell
              const float f = __fsub_rn(pa, __fsub_rn(lo, 1.0f));
              w1[ax][0] = __fsub_rn(1.0f, f); w1[ax][1] = f; w1[ax][2] = 0.f;
              m1[ax] = 3u;
            } else {
              const float f = __fsub_rn(pa, lo);
              w1[ax][0] = 0.f; w1[ax][1] = __fsub_rn(1.0f, f); w1[ax][2] = f;
              m1[ax] = 6u;
            }
          }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          if (i >= e0) continue;
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            if (j >= e1) continue;
            const float wij = __fmul_rn(w1[0][i], w1[1][j]);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
              if (k >= e2) continue;
              const int t = (i * e1 + j) * e2 + k;
              const float ww = __fmul_rn(wij, w1[2][k]);
              am[t] = __fadd_rn(am[t], __fmul_rn(ww, uD));
              aw[t] = __fadd_rn(aw[t], ww);
            }
          }
        }
        unsigned rp = box_axis_mask(D, D, 3u);  // every position on the normal axis
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          if (ax == D) continue;
          rp &= m1[ax] == 3u ? box_axis_mask(D, ax, 3u) : box_axis_mask(D, ax, 6u);
        }
        reach |= rp;
      }
      // flush the reached box nodes (local coordinates -1..8)
      const int b0 = cl[0] - (D == 0 ? 0 : 1), b1 = cl[1] - (D == 1 ? 0 : 1),
                b2 = cl[2] - (D == 2 ? 0 : 1);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        if (i >= e0) continue;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          if (j >= e1) continue;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            if (k >= e2) continue;
            const int t = (i * e1 + j) * e2 + k;
            if (!((reach >> t) & 1u)) continue;
            const int o = node_index(b0 + i, b1 + j, b2 + k);
            atomicAdd(&sv[D][o], to_fix(am[t]));
            atomicAdd(&sw[D][o], to_fix(aw[t]));
            touched[o] = 1;
          }
        }
      }
    }
  }
  __syncthreads();
  unsigned long long* out = a.p2g_nodes + int64_t(s) * 6 * kNodeBlock;
  for (int v = tid; v < kNodeBlock; v += 256) {
#pragma unroll
    for (int D = 0; D < 3; ++D) {
      out[D * kNodeBlock + v] = sv[D][v];
      out[(3 + D) * kNodeBlock + v] = sw[D][v];
    }
  }
  for (int v = tid; v < 1024; v += 256) {
    const unsigned bits = __ballot_sync(0xffffffffu, touched[v] != 0);
    if ((tid & 31) == 0) a.p2g_touch[int64_t(s) * 32 + (v >> 5)] = bits;
  }
}

// Faces whose fixed-point weight sum is below kLowWeight are summed again
// exactly as the reference sums them.  Fixed point has absolute resolution
// (2^-33 per cell term), which is a relative error of up to 1e-4 in the
// weight, and more in v = sum(w u) / sum(w), where the total weight is near
// the 1e-5 normalisation cut; the reference's float sums are relative.  Pass
// 2 lists those faces and k_p2g_low re-sums them, one thread per face, so
// pass 2 keeps its registers and occupancy.
constexpr float kLowWeight = 1e-3f;

// The reference's float sums of component D at node g: ScatterWeight's
// weights (common/flip_simulation.cc:976-990, differences of products) and
// its order -- each particle leaf (in OpenVDB leaf order) sums its particles
// in list order into its halo buffer (:853-868), and the buffers are added
// into the grid leaf by leaf (:870-890).  Leaves of slot s's neighbourhood
// only: a node of slot s is reached from cells within one cell of it.
__device__ __noinline__ void ref_node_sums(const GridArgs& a, const int* nb, int s, int D,
                                           const int g[3], float& tm, float& tw) {
  int sl[3];
  leaf_coords(a.lm, uint32_t(a.leaf_id[s]), sl[0], sl[1], sl[2]);
  // cells that reach node g: c_D in {g_D - 1, g_D}, the others in g +- 1
  int clo[3], chi[3], llo[3], lhi[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    clo[ax] = g[ax] - 1;
    chi[ax] = ax == D ? g[ax] : g[ax] + 1;
    llo[ax] = fdiv(clo[ax], 8);
    lhi[ax] = fdiv(chi[ax], 8);
  }
  // candidate leaves in OpenVDB order (at most 8)
  uint32_t lid[8];
  int lslot[8], lc[8][3], nl = 0;
  for (int lx = llo[0]; lx <= lhi[0]; ++lx)
    for (int ly = llo[1]; ly <= lhi[1]; ++ly)
      for (int lz = llo[2]; lz <= lhi[2]; ++lz) {
        const int dx = lx - sl[0], dy = ly - sl[1], dz = lz - sl[2];
        if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) continue;
        const int ns = nb[nb_index(dx, dy, dz)];
        if (ns < 0 || ns >= a.n_pleaf) continue;  // no particles there
        const uint32_t id = uint32_t(a.leaf_id[ns]);
        int q = nl++;
        while (q > 0 && lid[q - 1] > id) {  // insertion sort by leaf id
          lid[q] = lid[q - 1];
          lslot[q] = lslot[q - 1];
          lc[q][0] = lc[q - 1][0]; lc[q][1] = lc[q - 1][1]; lc[q][2] = lc[q - 1][2];
          --q;
        }
        lid[q] = id;
        lslot[q] = ns;
        lc[q][0] = lx; lc[q][1] = ly; lc[q][2] = lz;
      }
  const float* px = a.part;
  const int64_t cap = a.cap;
  float Tm = 0.f, Tw = 0.f;
  for (int l = 0; l < nl; ++l) {
    float Bm = 0.f, Bw = 0.f;
    bool touched = false;
    const int x0 = max(clo[0], lc[l][0] * 8), x1 = min(chi[0], lc[l][0] * 8 + 7);
    const int y0 = max(clo[1], lc[l][1] * 8), y1 = min(chi[1], lc[l][1] * 8 + 7);
    const int z0 = max(clo[2], lc[l][2] * 8), z1 = min(chi[2], lc[l][2] * 8 + 7);
    for (int cx = x0; cx <= x1; ++cx)
      for (int cy = y0; cy <= y1; ++cy)
        for (int cz = z0; cz <= z1; ++cz) {
          const int v = ((cx & 7) << 6) | ((cy & 7) << 3) | (cz & 7);
          const uint2 rg = a.cell_range[int64_t(lslot[l]) * 512 + v];
          const int c[3] = {cx, cy, cz};
          for (uint32_t q = rg.x; q < rg.y; ++q) {
            if (a.check_dead && a.keys[q] == kDeadKey) continue;
            float f[3];
            int corner[3];
            bool reach = true;
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
              const float pa = px[ax * cap + q];
              float lo = float(c[ax]);
              int st = c[ax];
              if (ax != D) {
                lo = __fadd_rn(lo, 0.5f);
                if (pa < lo) { lo = __fsub_rn(lo, 1.0f); st -= 1; }
              }
              f[ax] = __fsub_rn(pa, lo);
              corner[ax] = g[ax] - st;
              reach = reach && (corner[ax] == 0 || corner[ax] == 1);
            }
            if (!reach) continue;
            touched = true;
            const float x = f[0], y = f[1], z = f[2];
            const float xy = __fmul_rn(x, y), yz = __fmul_rn(y, z), xz = __fmul_rn(z, x);
            const float xyz = __fmul_rn(xy, z);
            const float w110 = __fsub_rn(xy, xyz), w101 = __fsub_rn(xz, xyz);
            const float w001 = __fsub_rn(__fsub_rn(z, yz), w101);
            const int k = (corner[0] << 2) | (corner[1] << 1) | corner[2];
            float w;
            switch (k) {
              case 7: w = xyz; break;
              case 6: w = w110; break;
              case 5: w = w101; break;
              case 4: w = __fsub_rn(__fsub_rn(x, xz), w110); break;
              case 3: w = __fsub_rn(yz, xyz); break;
              case 2: w = __fsub_rn(__fsub_rn(y, yz), w110); break;
              case 1: w = w001; break;
              default: w = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(1.0f, x), y), xy), w001);
            }
            Bm = __fadd_rn(Bm, __fmul_rn(w, px[(3 + D) * cap + q]));
            Bw = __fadd_rn(Bw, w);
          }
        }
    if (touched) {
      Tm = __fadd_rn(Tm, Bm);
      Tw = __fadd_rn(Tw, Bw);
    }
  }
  tm = Tm;
  tw = Tw;
}

template <bool FUSED>
__global__ void __launch_bounds__(256) k_p2g_nodes(const __grid_constant__ GridArgs a) {
  __shared__ int nb[27];
  const int s = blockIdx.x;  // grid leaf
  const int tid = threadIdx.x;
  if (tid < 27) nb[tid] = a.nbr[int64_t(s) * 27 + tid];
  __syncthreads();
  int org[3];
  origin_of(a, s, org);
  float* vel = a.vel + int64_t(s) * 1536;
  // this leaf's own block entries for both of the thread's nodes, loaded
  // before either is used; the node loop then adds the neighbour particle
  // leaves that cover a node with their outer layer (integer sums: the order
  // does not matter)
  unsigned long long own_v[2][3], own_w[2][3];
  bool own_on[2];
  {
    const int ns = nb[nb_index(0, 0, 0)];
    const bool own = ns >= 0 && ns < a.n_pleaf;
    const unsigned long long* blk = a.p2g_nodes + int64_t(own ? ns : 0) * 6 * kNodeBlock;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int v = tid + 256 * j;
      const int o = node_index(v >> 6, (v >> 3) & 7, v & 7);
#pragma unroll
      for (int D = 0; D < 3; ++D) {
        own_v[j][D] = own ? blk[D * kNodeBlock + o] : 0ull;
        own_w[j][D] = own ? blk[(3 + D) * kNodeBlock + o] : 0ull;
      }
      own_on[j] = own && ((a.p2g_touch[int64_t(ns) * 32 + (o >> 5)] >> (o & 31)) & 1u);
    }
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int v = tid + 256 * j;
    const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
    const int g[3] = {org[0] + x, org[1] + y, org[2] + z};
    unsigned long long sv[3] = {own_v[j][0], own_v[j][1], own_v[j][2]};
    unsigned long long sw[3] = {own_w[j][0], own_w[j][1], own_w[j][2]};
    bool on = own_on[j];
    const int dlo[3] = {x == 0 ? -1 : 0, y == 0 ? -1 : 0, z == 0 ? -1 : 0};
    const int dhi[3] = {x == 7 ? 1 : 0, y == 7 ? 1 : 0, z == 7 ? 1 : 0};
    for (int dx = dlo[0]; dx <= dhi[0]; ++dx)
      for (int dy = dlo[1]; dy <= dhi[1]; ++dy)
        for (int dz = dlo[2]; dz <= dhi[2]; ++dz) {
          if (dx == 0 && dy == 0 && dz == 0) continue;  // the own block, loaded above
          const int ns = nb[nb_index(dx, dy, dz)];
          if (ns < 0 || ns >= a.n_pleaf) continue;
          const int o = node_index(x - 8 * dx, y - 8 * dy, z - 8 * dz);
          const unsigned long long* blk = a.p2g_nodes + int64_t(ns) * 6 * kNodeBlock;
#pragma unroll
          for (int D = 0; D < 3; ++D) {
            sv[D] += blk[D * kNodeBlock + o];
            sw[D] += blk[(3 + D) * kNodeBlock + o];
          }
          on |= (a.p2g_touch[int64_t(ns) * 32 + (o >> 5)] >> (o & 31)) & 1u;
        }
    float val[3];
    float wsum[3];
#pragma unroll
    for (int D = 0; D < 3; ++D) {
      const float ws = from_fix(sw[D]);
      const float ms = from_fix(sv[D]);
      if (on && ws < kLowWeight)  // re-summed by k_p2g_low, which rewrites this face
        a.p2g_low[1 + atomicAdd(a.p2g_low, 1u)] = unsigned(s) * 1536u + unsigned(D * 512 + v);
      wsum[D] = ws;
      // THRESH is a double literal in the reference: float ws < 1e-5 (double)
      // is ws <= 1e-5f
      val[D] = on ? ((ws <= 1e-5f) ? 0.f : __fdiv_rn(ms, ws)) : 0.f;
    }
    // marker: FLUID for in-box cells holding particles
    bool has = false;
    if (s < a.n_pleaf) {
      const uint2 rg = a.cell_range[int64_t(s) * 512 + v];
      has = rg.y > rg.x;
    }
    int m = (has && in_box(a.lm.n, g[0], g[1], g[2])) ? FSIM_FLUID : FSIM_AIR;
    const unsigned ball = __ballot_sync(0xffffffffu, on);
    if (FUSED) {
      const bool sc = is_solid(a.sd, g[0], g[1], g[2]);
      if (sc) m = FSIM_SOLID;
      bool zero[3];
      zero[0] = sc != is_solid(a.sd, g[0] - 1, g[1], g[2]);
      zero[1] = sc != is_solid(a.sd, g[0], g[1] - 1, g[2]);
      zero[2] = sc != is_solid(a.sd, g[0], g[1], g[2] - 1);
      float* vold = a.vold + int64_t(s) * 1536;
      const float gf[3] = {__fmul_rn(a.dt, a.fx), __fmul_rn(a.dt, a.fy), __fmul_rn(a.dt, a.fz)};
#pragma unroll
      for (int D = 0; D < 3; ++D) {
        float vv = val[D];
        if (on && zero[D]) vv = 0.f;                 // ApplyBoundaryConditions
        vold[D * 512 + v] = vv;                      // SaveGridVelocities
        if (on) vv = (D == 1) ? __fsub_rn(vv, gf[1]) : __fadd_rn(vv, gf[D]);  // AddGravity
        if (on && zero[D]) vv = 0.f;                 // ApplyBoundaryConditions
        vel[D * 512 + v] = vv;
      }
      if ((threadIdx.x & 31) == 0) {
        a.vold_on[int64_t(s) * 16 + (v >> 5)] = ball;
      }
    } else {
      float* wt = a.weight + int64_t(s) * 1536;
#pragma unroll
      for (int D = 0; D < 3; ++D) {
        vel[D * 512 + v] = val[D];
        wt[D * 512 + v] = on ? wsum[D] : 0.f;
      }
      // ClearGridData left the saved velocity empty
      if ((threadIdx.x & 31) == 0) a.vold_on[int64_t(s) * 16 + (v >> 5)] = 0u;
    }
    if ((threadIdx.x & 31) == 0) a.vel_on[int64_t(s) * 16 + (v >> 5)] = ball;
    a.marker[int64_t(s) * 512 + v] = int8_t(m);
  }
}

// The low-weight faces pass 2 listed: the reference's float sums
// (ref_node_sums), normalisation with the 1e-5 cut, and for the fused step
// the rest of pass 2's per-face work (BC, SaveGridVelocities, AddGravity,
// BC).  The faces are independent, so the list's order does not matter.
template <bool FUSED>
__global__ void __launch_bounds__(128) k_p2g_low(const __grid_constant__ GridArgs a) {
  const unsigned n = *a.p2g_low;
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const unsigned code = a.p2g_low[1 + e];
    const int s = int(code / 1536u), D = int((code % 1536u) >> 9), v = int(code & 511u);
    int org[3];
    origin_of(a, s, org);
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    float ms, ws;
    ref_node_sums(a, a.nbr + int64_t(s) * 27, s, D, g, ms, ws);
    const float val = (ws <= 1e-5f) ? 0.f : __fdiv_rn(ms, ws);
    const int64_t o = int64_t(s) * 1536 + D * 512 + v;
    if (FUSED) {
      const bool sc = is_solid(a.sd, g[0], g[1], g[2]);
      const bool zero = sc != is_solid(a.sd, g[0] - (D == 0), g[1] - (D == 1), g[2] - (D == 2));
      const float gf = __fmul_rn(a.dt, D == 0 ? a.fx : (D == 1 ? a.fy : a.fz));
      float vv = zero ? 0.f : val;                              // ApplyBoundaryConditions
      a.vold[o] = vv;                                           // SaveGridVelocities
      vv = (D == 1) ? __fsub_rn(vv, gf) : __fadd_rn(vv, gf);    // AddGravity
      a.vel[o] = zero ? 0.f : vv;                               // ApplyBoundaryConditions
    } else {
      a.vel[o] = val;
      a.weight[o] = ws;
    }
  }
}

__device__ __forceinline__ bool bit_on(const uint32_t* bits, int s, int v) {
  return (bits[int64_t(s) * 16 + (v >> 5)] >> (v & 31)) & 1u;
}

// ApplyBoundaryConditions (per-stage): marker SOLID on solid cells, normal
// component zeroed on active faces with solid on exactly one side.
__global__ void __launch_bounds__(256) k_apply_bc(const __grid_constant__ GridArgs a) {
  const int s = blockIdx.x;
  int org[3];
  origin_of(a, s, org);
  for (int v = threadIdx.x; v < 512; v += 256) {
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    const bool sc = is_solid(a.sd, g[0], g[1], g[2]);
    if (sc) a.marker[int64_t(s) * 512 + v] = FSIM_SOLID;
    if (!bit_on(a.vel_on, s, v)) continue;
    float* vel = a.vel + int64_t(s) * 1536;
    if (sc != is_solid(a.sd, g[0] - 1, g[1], g[2])) vel[v] = 0.f;
    if (sc != is_solid(a.sd, g[0], g[1] - 1, g[2])) vel[512 + v] = 0.f;
    if (sc != is_solid(a.sd, g[0], g[1], g[2] - 1)) vel[1024 + v] = 0.f;
  }
}

__global__ void __launch_bounds__(256) k_save(const __grid_constant__ GridArgs a) {
  const int s = blockIdx.x;
  for (int v = threadIdx.x; v < 512; v += 256) {
    const bool on = bit_on(a.vel_on, s, v);
#pragma unroll
    for (int D = 0; D < 3; ++D)
      a.vold[int64_t(s) * 1536 + D * 512 + v] = on ? a.vel[int64_t(s) * 1536 + D * 512 + v] : 0.f;
    if (v < 16) a.vold_on[int64_t(s) * 16 + v] = a.vel_on[int64_t(s) * 16 + v];
  }
}

__global__ void __launch_bounds__(256) k_gravity(const __grid_constant__ GridArgs a) {
  const int s = blockIdx.x;
  const float gf[3] = {__fmul_rn(a.dt, a.fx), __fmul_rn(a.dt, a.fy), __fmul_rn(a.dt, a.fz)};
  for (int v = threadIdx.x; v < 512; v += 256) {
    if (!bit_on(a.vel_on, s, v)) continue;
    float* vel = a.vel + int64_t(s) * 1536;
    vel[v] = __fadd_rn(vel[v], gf[0]);
    vel[512 + v] = __fsub_rn(vel[512 + v], gf[1]);
    vel[1024 + v] = __fadd_rn(vel[1024 + v], gf[2]);
  }
}

// Particles::DeleteOutsideParticles: particles whose cell is outside the box
// get the dead key (they stop contributing and are dropped at the next sort).
__global__ void k_delete_outside(uint32_t* __restrict__ keys, int64_t n, LeafMap lm,
                                 int64_t* __restrict__ ndead) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = keys[i];
  if (k == kDeadKey) return;
  int lx, ly, lz;
  leaf_coords(lm, k >> 9, lx, ly, lz);
  const int v = int(k & 511u);
  const int c0 = lx * 8 + (v >> 6), c1 = ly * 8 + ((v >> 3) & 7), c2 = lz * 8 + (v & 7);
  if (!in_box(lm.n, c0, c1, c2)) {
    keys[i] = kDeadKey;
    atomicAdd(reinterpret_cast<unsigned long long*>(ndead), 1ull);
  }
}

// velocity component D at global node g, from leaf slot s's neighbourhood
__device__ __forceinline__ float vel_at(const GridArgs& a, const float* field, const int* nb,
                                        const int org[3], int D, int gx, int gy, int gz) {
  const int lx = gx - org[0], ly = gy - org[1], lz = gz - org[2];
  const int ns = nb[nb_index(side(lx), side(ly), side(lz))];
  if (ns < 0) return 0.f;
  const int v = ((gx & 7) << 6) | ((gy & 7) << 3) | (gz & 7);
  return field[int64_t(ns) * 1536 + D * 512 + v];
}

__device__ __forceinline__ int marker_at(const GridArgs& a, const int* nb, const int org[3],
                                         int gx, int gy, int gz) {
  const int lx = gx - org[0], ly = gy - org[1], lz = gz - org[2];
  const int ns = nb[nb_index(side(lx), side(ly), side(lz))];
  if (ns < 0) return FSIM_AIR;
  const int v = ((gx & 7) << 6) | ((gy & 7) << 3) | (gz & 7);
  return a.marker[int64_t(ns) * 512 + v];
}

__device__ __forceinline__ float pres_at(const GridArgs& a, const int* nb, const int org[3],
                                         int gx, int gy, int gz) {
  const int lx = gx - org[0], ly = gy - org[1], lz = gz - org[2];
  const int ns = nb[nb_index(side(lx), side(ly), side(lz))];
  if (ns < 0 || ns >= a.n_pleaf) return 0.f;
  const int v = ((gx & 7) << 6) | ((gy & 7) << 3) | (gz & 7);
  return a.pres[int64_t(ns) * 512 + v];
}

// ComputeDivergence over particle leaves (FLUID cells only live there).
__global__ void __launch_bounds__(256) k_divergence(const __grid_constant__ GridArgs a) {
  __shared__ int nb[27];
  const int s = blockIdx.x;
  if (threadIdx.x < 27) nb[threadIdx.x] = a.nbr[int64_t(s) * 27 + threadIdx.x];
  int org[3];
  origin_of(a, s, org);
  __syncthreads();
  for (int v = threadIdx.x; v < 512; v += 256) {
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    float d = 0.f;
    if (a.marker[int64_t(s) * 512 + v] == FSIM_FLUID) {
      const float* vel = a.vel + int64_t(s) * 1536;
      d = __fsub_rn(vel_at(a, a.vel, nb, org, 0, g[0] + 1, g[1], g[2]), vel[v]);
      d = __fadd_rn(d, __fsub_rn(vel_at(a, a.vel, nb, org, 1, g[0], g[1] + 1, g[2]), vel[512 + v]));
      d = __fadd_rn(d, __fsub_rn(vel_at(a, a.vel, nb, org, 2, g[0], g[1], g[2] + 1), vel[1024 + v]));
    }
    a.div[int64_t(s) * 512 + v] = d;
  }
}

__device__ __forceinline__ void atomic_max_pos(int64_t* cnt, float v) {
  // non-negative floats order like their bit patterns
  atomicMax(reinterpret_cast<unsigned long long*>(cnt), (unsigned long long)__float_as_uint(v));
}

// UpdateVelocityFromPressure over faces [0,N]^3; FUSED also forms
// GetVelocityUpdate (v_old := v - v_old on active faces) and the CFL max.
template <bool FUSED>
__global__ void __launch_bounds__(256) k_pressure_update(const __grid_constant__ GridArgs a) {
  __shared__ int nb[27];
  __shared__ float red[8];
  const int s = blockIdx.x;
  if (threadIdx.x < 27) nb[threadIdx.x] = a.nbr[int64_t(s) * 27 + threadIdx.x];
  int org[3];
  origin_of(a, s, org);
  __syncthreads();
  const int* n = a.lm.n;
  float vmax = 0.f;
  for (int v = threadIdx.x; v < 512; v += 256) {
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    if (g[0] < 0 || g[1] < 0 || g[2] < 0 || g[0] > n[0] || g[1] > n[1] || g[2] > n[2]) continue;
    float* vel = a.vel + int64_t(s) * 1536;
    const int mc = a.marker[int64_t(s) * 512 + v];
    bool on = bit_on(a.vel_on, s, v);
    float val[3] = {vel[v], vel[512 + v], vel[1024 + v]};
    if (mc != FSIM_SOLID) {
      const float pc = (s < a.n_pleaf) ? a.pres[int64_t(s) * 512 + v] : 0.f;
      bool upd = false;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int h0 = g[0] - (d == 0), h1 = g[1] - (d == 1), h2 = g[2] - (d == 2);
        const int mn = marker_at(a, nb, org, h0, h1, h2);
        if ((mn == FSIM_FLUID || mc == FSIM_FLUID) && mn != FSIM_SOLID) {
          val[d] = __fadd_rn(val[d], __fsub_rn(pc, pres_at(a, nb, org, h0, h1, h2)));
          upd = true;
        }
      }
      if (upd) {
        vel[v] = val[0]; vel[512 + v] = val[1]; vel[1024 + v] = val[2];
        if (!on) {
          atomicOr(&a.vel_on[int64_t(s) * 16 + (v >> 5)], 1u << (v & 31));
          on = true;
        }
      }
    }
    if (FUSED && on) {
      float* vold = a.vold + int64_t(s) * 1536;
#pragma unroll
      for (int D = 0; D < 3; ++D) vold[D * 512 + v] = __fsub_rn(val[D], vold[D * 512 + v]);
      if (g[0] < n[0] && g[1] < n[1] && g[2] < n[2]) {
        if (g[1] != n[1] - 1 && g[2] != n[2] - 1) vmax = fmaxf(vmax, fabsf(val[0]));
        if (g[0] != n[0] - 1 && g[2] != n[2] - 1) vmax = fmaxf(vmax, fabsf(val[1]));
        if (g[0] != n[0] - 1 && g[1] != n[1] - 1) vmax = fmaxf(vmax, fabsf(val[2]));
      }
    }
  }
  if (FUSED) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vmax;
    __syncthreads();
    if (threadIdx.x == 0) {
      float m = 0.f;
      for (int w = 0; w < 8; ++w) m = fmaxf(m, red[w]);
      if (m > 0.f) atomic_max_pos(a.cnt + 4, m);
    }
  }
}

// GetVelocityUpdate (per-stage) over faces [0,N]^3.
__global__ void __launch_bounds__(256) k_velocity_update(const __grid_constant__ GridArgs a) {
  const int s = blockIdx.x;
  int org[3];
  origin_of(a, s, org);
  const int* n = a.lm.n;
  for (int v = threadIdx.x; v < 512; v += 256) {
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    if (g[0] < 0 || g[1] < 0 || g[2] < 0 || g[0] > n[0] || g[1] > n[1] || g[2] > n[2]) continue;
    const bool on = bit_on(a.vel_on, s, v), oo = bit_on(a.vold_on, s, v);
    if (on && !oo) atomicAdd(reinterpret_cast<unsigned long long*>(a.cnt + 3), 1ull);
    if (on && oo) {
      float* vel = a.vel + int64_t(s) * 1536;
      float* vold = a.vold + int64_t(s) * 1536;
#pragma unroll
      for (int D = 0; D < 3; ++D) vold[D * 512 + v] = __fsub_rn(vel[D * 512 + v], vold[D * 512 + v]);
    }
  }
}

// CFL max over active in-box faces (FlipSimulation::CFL).
__global__ void __launch_bounds__(256) k_cfl(const __grid_constant__ GridArgs a) {
  __shared__ float red[8];
  const int s = blockIdx.x;
  int org[3];
  origin_of(a, s, org);
  const int* n = a.lm.n;
  float vmax = 0.f;
  for (int v = threadIdx.x; v < 512; v += 256) {
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    if (!in_box(n, g[0], g[1], g[2]) || !bit_on(a.vel_on, s, v)) continue;
    const float* vel = a.vel + int64_t(s) * 1536;
    if (g[1] != n[1] - 1 && g[2] != n[2] - 1) vmax = fmaxf(vmax, fabsf(vel[v]));
    if (g[0] != n[0] - 1 && g[2] != n[2] - 1) vmax = fmaxf(vmax, fabsf(vel[512 + v]));
    if (g[0] != n[0] - 1 && g[1] != n[1] - 1) vmax = fmaxf(vmax, fabsf(vel[1024 + v]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f;
    for (int w = 0; w < 8; ++w) m = fmaxf(m, red[w]);
    if (m > 0.f) atomic_max_pos(a.cnt + 4, m);
  }
}

// ---- dense downloads ------------------------------------------------------
struct DenseArgs {
  LeafMap lm;
  SolidDesc sd;
  const int32_t* slot;  // dense leaf id -> slot
  int n_pleaf;
  const float* vec;     // slot*1536 (Vec3 fields)
  const uint32_t* on;   // slot*16
  const float* sca;     // pleaf*512 (scalar fields)
  const int8_t* marker;
  int field;            // FSIM_FIELD_* or 100 marker
  int valid, extrap, bc;
  float* out;
  int32_t* iout;
  uint8_t* act;
};

__device__ __forceinline__ int slot_of(const DenseArgs& a, int i, int j, int k) {
  const int lx = fdiv(i, 8), ly = fdiv(j, 8), lz = fdiv(k, 8);
  if (!leaf_valid(a.lm, lx, ly, lz)) return -1;
  return a.slot[leaf_id(a.lm, lx, ly, lz)];
}

__global__ void k_dense(const __grid_constant__ DenseArgs a) {
  const int* n = a.lm.n;
  const int64_t s1 = n[1] + 2, s2 = n[2] + 2;
  const int64_t tot = int64_t(n[0] + 2) * s1 * s2;
  int64_t o = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (o >= tot) return;
  const int i = int(o / (s1 * s2)) - 1, j = int((o / s2) % s1) - 1, k = int(o % s2) - 1;
  const int vox = ((i & 7) << 6) | ((j & 7) << 3) | (k & 7);
  const int sl = slot_of(a, i, j, k);
  if (a.field == 100) {  // marker
    int m = 0;
    if (a.valid && sl >= 0) m = a.marker[int64_t(sl) * 512 + vox];
    if (a.bc && is_solid(a.sd, i, j, k)) m = FSIM_SOLID;
    a.iout[o] = m;
    if (a.act) a.act[o] = m != 0;
    return;
  }
  if (a.field <= FSIM_FIELD_WEIGHT) {
    bool on = a.valid && sl >= 0 && ((a.on[int64_t(sl) * 16 + (vox >> 5)] >> (vox & 31)) & 1u);
    const int c[3] = {i, j, k};
    for (int D = 0; D < 3; ++D) {
      float val = 0.f;
      if (a.valid) {
        int src[3] = {i, j, k};
        if (a.extrap && a.field != FSIM_FIELD_WEIGHT) ghost_source(n, D, c, src);
        const int ss = slot_of(a, src[0], src[1], src[2]);
        if (ss >= 0) {
          const int sv = ((src[0] & 7) << 6) | ((src[1] & 7) << 3) | (src[2] & 7);
          const bool son = (a.on[int64_t(ss) * 16 + (sv >> 5)] >> (sv & 31)) & 1u;
          if (son) val = a.vec[int64_t(ss) * 1536 + D * 512 + sv];
        }
      }
      a.out[3 * o + D] = val;
    }
    if (a.extrap && a.field != FSIM_FIELD_WEIGHT && extrap_activated(n, i, j, k)) on = true;
    if (a.act) a.act[o] = on;
    if (!on) { a.out[3 * o] = 0.f; a.out[3 * o + 1] = 0.f; a.out[3 * o + 2] = 0.f; }
    return;
  }
  // scalar fields on FLUID cells (div, pressure, phi)
  bool fl = false;
  if (a.valid && sl >= 0) fl = a.marker[int64_t(sl) * 512 + vox] == FSIM_FLUID;
  float val = (a.field == FSIM_FIELD_PHI) ? 5.0f : 0.f;
  if (fl) {
    if (a.field == FSIM_FIELD_PHI) val = -0.5f;
    else if (sl < a.n_pleaf) val = a.sca[int64_t(sl) * 512 + vox];
  }
  a.out[o] = val;
  if (a.act) a.act[o] = fl;
}

inline unsigned nblk(int64_t n, int b) { return unsigned((n + b - 1) / b); }

GridArgs make_args(fsim_sim* s) {
  GridArgs a;
  a.part = s->part[s->cur];
  a.cap = s->cap_p;
  a.keys = s->keys[0];
  a.leaf_id = s->d_leaf_id;
  a.nbr = s->d_nbr;
  a.cell_range = s->d_cell_range;
  a.leaf_range = s->d_leaf_range;
  a.n_pleaf = s->n_pleaf;
  a.n_gleaf = s->n_gleaf;
  a.check_dead = s->deleted_outside ? 1 : 0;
  a.lm = s->lm;
  a.sd = s->solid;
  a.vel = s->vel;
  a.vold = s->vold;
  a.weight = s->weight;
  a.vel_on = s->vel_on;
  a.vold_on = s->vold_on;
  a.marker = s->marker;
  a.pres = s->pres;
  a.div = s->div;
  a.dt = 0.f;
  a.fx = s->cfg.force[0];
  a.fy = s->cfg.force[1];
  a.fz = s->cfg.force[2];
  a.cnt = s->d_cnt;
  a.p2g_nodes = s->p2g_nodes;
  a.p2g_touch = s->p2g_touch;
  return a;
}

}  // namespace

int launch_p2g(fsim_sim* s, bool fused, float dt) {
  if (s->p2g_cap < s->cap_pleaf) {
    if (s->p2g_nodes) cudaFree(s->p2g_nodes);
    if (s->p2g_touch) cudaFree(s->p2g_touch);
    s->p2g_nodes = nullptr;
    s->p2g_touch = nullptr;
    s->p2g_cap = 0;
    FSIM_CK(s, cudaMalloc(&s->p2g_nodes, size_t(s->cap_pleaf) * 6 * kNodeBlock * 8));
    FSIM_CK(s, cudaMalloc(&s->p2g_touch, size_t(s->cap_pleaf) * 32 * 4));
    s->p2g_cap = s->cap_pleaf;
  }
  // list of low-weight faces: at most every face of every grid leaf, each
  // coded in 32 bits as slot * 1536 + D * 512 + voxel
  if (int64_t(s->n_gleaf) * 1536 >= (int64_t(1) << 32))
    return fail(s, FSIM_ERR_CAPACITY, "too many grid leaves for the P2G low-weight face list");
  const int64_t low_cap = int64_t(s->cap_leaf) * 1536 + 1;
  if (s->p2g_low_cap < low_cap) {
    if (s->p2g_low) cudaFree(s->p2g_low);
    s->p2g_low = nullptr;
    s->p2g_low_cap = 0;
    FSIM_CK(s, cudaMalloc(&s->p2g_low, size_t(low_cap) * sizeof(uint32_t)));
    s->p2g_low_cap = low_cap;
  }
  GridArgs a = make_args(s);
  a.dt = dt;
  a.p2g_low = s->p2g_low;
  FSIM_CK(s, cudaMemsetAsync(s->p2g_low, 0, sizeof(uint32_t), s->stream));
  FSIM_LAUNCH(s, fused ? "p2g_cells_fused" : "p2g_cells", k_p2g_cells, s->n_pleaf, 256, 0, a);
  const int lgrid = std::max(1, s->num_sms * 4);
  if (fused) {
    FSIM_LAUNCH(s, "p2g_fused", k_p2g_nodes<true>, s->n_gleaf, 256, 0, a);
    FSIM_LAUNCH(s, "p2g_low_fused", k_p2g_low<true>, lgrid, 128, 0, a);
  } else {
    FSIM_LAUNCH(s, "p2g", k_p2g_nodes<false>, s->n_gleaf, 256, 0, a);
    FSIM_LAUNCH(s, "p2g_low", k_p2g_low<false>, lgrid, 128, 0, a);
  }
  return FSIM_OK;
}

int launch_apply_bc(fsim_sim* s) {
  FSIM_LAUNCH(s, "apply_bc", k_apply_bc, s->n_gleaf, 256, 0, make_args(s));
  return FSIM_OK;
}

int launch_save_velocities(fsim_sim* s) {
  FSIM_LAUNCH(s, "save_velocities", k_save, s->n_gleaf, 256, 0, make_args(s));
  return FSIM_OK;
}

int launch_add_gravity(fsim_sim* s, float dt) {
  GridArgs a = make_args(s);
  a.dt = dt;
  FSIM_LAUNCH(s, "add_gravity", k_gravity, s->n_gleaf, 256, 0, a);
  return FSIM_OK;
}

int launch_delete_outside(fsim_sim* s) {
  FSIM_LAUNCH(s, "delete_outside", k_delete_outside, nblk(s->n_live, 256), 256, 0, s->keys[0],
              s->n_live, s->lm, s->d_cnt + 6);
  return FSIM_OK;
}

int launch_divergence(fsim_sim* s) {
  FSIM_LAUNCH(s, "divergence", k_divergence, s->n_pleaf, 256, 0, make_args(s));
  return FSIM_OK;
}

int launch_pressure_update(fsim_sim* s, bool fused) {
  if (fused) {
    FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 4, 0, sizeof(int64_t), s->stream));
    FSIM_LAUNCH(s, "pressure_update_fused", k_pressure_update<true>, s->n_gleaf, 256, 0,
                make_args(s));
  } else {
    FSIM_LAUNCH(s, "pressure_update", k_pressure_update<false>, s->n_gleaf, 256, 0, make_args(s));
  }
  return FSIM_OK;
}

int launch_velocity_update(fsim_sim* s) {
  FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 3, 0, sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "velocity_update", k_velocity_update, s->n_gleaf, 256, 0, make_args(s));
  return FSIM_OK;
}

int launch_cfl(fsim_sim* s) {
  FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 4, 0, sizeof(int64_t), s->stream));
  FSIM_LAUNCH(s, "cfl_max", k_cfl, s->n_gleaf, 256, 0, make_args(s));
  return FSIM_OK;
}

static int ensure_dense(fsim_sim* s, size_t bytes) {
  if (s->dense_tmp.bytes >= bytes) return FSIM_OK;
  if (s->dense_tmp.p) cudaFree(s->dense_tmp.p);
  s->dense_tmp.p = nullptr;
  s->dense_tmp.bytes = 0;
  FSIM_CK(s, cudaMalloc(&s->dense_tmp.p, bytes));
  s->dense_tmp.bytes = bytes;
  return FSIM_OK;
}

static DenseArgs dense_args(fsim_sim* s) {
  DenseArgs a;
  memset(&a, 0, sizeof(a));
  a.lm = s->lm;
  a.sd = s->solid;
  a.slot = s->d_slot;
  a.n_pleaf = s->n_pleaf;
  a.marker = s->marker;
  return a;
}

int download_dense(fsim_sim* s, int field, float* out, uint8_t* active) {
  const int* n = s->lm.n;
  const int64_t tot = int64_t(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  const int comps = (field <= FSIM_FIELD_WEIGHT) ? 3 : 1;
  const size_t fb = size_t(tot) * comps * sizeof(float);
  int rc = ensure_dense(s, fb + size_t(tot));
  if (rc) return rc;
  DenseArgs a = dense_args(s);
  a.field = field;
  a.out = static_cast<float*>(s->dense_tmp.p);
  a.act = static_cast<uint8_t*>(s->dense_tmp.p) + fb;
  bool have = s->have_topology && s->grid_valid;
  switch (field) {
    case FSIM_FIELD_VELOCITY: a.vec = s->vel; a.on = s->vel_on; a.valid = have; a.extrap = s->extrapolated; break;
    case FSIM_FIELD_VELOCITY_UPDATE: a.vec = s->vold; a.on = s->vold_on; a.valid = have && s->saved; a.extrap = s->extrapolated; break;
    case FSIM_FIELD_WEIGHT: a.vec = s->weight; a.on = s->vel_on; a.valid = have && s->weight_valid; break;
    case FSIM_FIELD_DIVERGENCE: a.sca = s->div; a.valid = have && s->div_valid; break;
    case FSIM_FIELD_PRESSURE: a.sca = s->pres; a.valid = have && s->pres_valid; break;
    case FSIM_FIELD_PHI: a.valid = have && s->phi_valid; break;
    default: return fail(s, FSIM_ERR_INVALID, "unknown field");
  }
  FSIM_LAUNCH(s, "dense_download", k_dense, nblk(tot, 256), 256, 0, a);
  FSIM_CK(s, cudaMemcpyAsync(out, a.out, fb, cudaMemcpyDeviceToHost, s->stream));
  if (active)
    FSIM_CK(s, cudaMemcpyAsync(active, a.act, size_t(tot), cudaMemcpyDeviceToHost, s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

int download_marker(fsim_sim* s, int32_t* out, uint8_t* active) {
  const int* n = s->lm.n;
  const int64_t tot = int64_t(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  int rc = ensure_dense(s, size_t(tot) * 5);
  if (rc) return rc;
  DenseArgs a = dense_args(s);
  a.field = 100;
  a.iout = static_cast<int32_t*>(s->dense_tmp.p);
  a.act = static_cast<uint8_t*>(s->dense_tmp.p) + size_t(tot) * 4;
  a.valid = s->have_topology && s->grid_valid;
  a.bc = s->bc_applied;
  FSIM_LAUNCH(s, "dense_download", k_dense, nblk(tot, 256), 256, 0, a);
  FSIM_CK(s, cudaMemcpyAsync(out, a.iout, size_t(tot) * 4, cudaMemcpyDeviceToHost, s->stream));
  if (active)
    FSIM_CK(s, cudaMemcpyAsync(active, a.act, size_t(tot), cudaMemcpyDeviceToHost, s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

}  // namespace fsim
