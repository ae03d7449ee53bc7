// k_adjoint.cu -- differentiable rollout: the adjoint of the FLIP step's
// projection and advection.
//
// The reference has no gradients; this module differentiates the step the
// rest of the library restates (FlipDriver::RunOneStep,
// common/flip_app_sim.cc:211-254) with its discrete choices frozen:
// particle binning and order, wall clamping and deletion
// (common/particles.cc:479-546), FLUID markers, active faces and the 1e-5
// weight cut of TransferParticlesToGrid (common/flip_simulation.cc:900-922).
// With those fixed, one step maps the particle state (x, v, g) to
//   x' = clamp(x + g dt)                              advection
//   m_f = sum_p W_f(x') v_p,  w_f = sum_p W_f(x')      P2G (trilinear, MAC)
//   val = m / w  on normalised faces                   normalisation
//   vsave = B val,  u = B (val + gravity)              BC / save / gravity
//   div = D u,  A p = div                              projection
//   u_new = u + G p,  dv = u_new - vsave (in box)      pressure update, GetVelocityUpdate
//   v' = (1-f) I(u_new) + f I(dv) + f v,  g' = I(u_new)  G2P (ghost-extrapolated)
// and its transpose runs stage by stage in reverse: the interpolation
// adjoint scatters into the faces (and differentiates the weights in x'),
// G^T gathers the face adjoints into cells, A^-1 is the same PCG (A is
// symmetric), D^T spreads the cell adjoints to faces, the normalisation
// adjoint gives m-bar = val-bar / w and w-bar = -val-bar val / w, and the P2G
// adjoint gathers them back into v-bar and x'-bar.
//
// The fp32 forward is the production step itself.  Every step records its
// frozen topology; the particle state is checkpointed every K steps, and the
// backward pass recomputes each segment from its checkpoint, taping the
// values the reverse stages read (x', v, w, vsave, u_new, dv).  An fp64
// replay of the same frozen map (positions, velocities and grid fields in
// double, pressure solves in FP64) gives the reference gradient and the
// loss for finite differences.
#include <algorithm>
#include <cstring>
#include <vector>

#include "fsim_internal.cuh"

namespace fsim {
namespace rb {

inline unsigned nblk(int64_t n, int b) { return unsigned(std::max<int64_t>(1, (n + b - 1) / b)); }

// ---- device buffers ---------------------------------------------------------
template <typename T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  Buf(Buf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  ~Buf() { if (p) cudaFree(p); }
  cudaError_t reserve(size_t count) {
    if (count <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
};

// Frozen topology of one step (after its sort and pressure update).
struct TopoRec {
  int64_t n_old = 0, n_live = 0;  // particles before / after the step
  int n_pleaf = 0, n_gleaf = 0;
  Buf<uint32_t> perm;    // n_live: new index -> old index
  Buf<uint32_t> keys;    // n_live: cell key (the particle's bin)
  Buf<uint8_t> clamp;    // n_old: bit 2a: clamped low on axis a, bit 2a+1 high
  Buf<int32_t> slot;     // dense leaf table
  Buf<int32_t> leaf_id;  // n_gleaf
  Buf<int32_t> nbr;      // n_gleaf*27
  Buf<uint2> cell_range; // n_pleaf*512
  Buf<uint2> leaf_range; // n_pleaf
  Buf<int8_t> marker;    // n_gleaf*512
  Buf<uint32_t> vel_on;  // n_gleaf*16, after the pressure update
  Buf<uint32_t> touched; // n_gleaf*16, faces P2G wrote (vold_on)
  Buf<uint32_t> normed;  // n_gleaf*16 words per component (x3): normalised faces
  Buf<uint8_t> side;     // n_live: bit a set when the position after advection lies
                         // below its cell's centre on axis a (the stencil side)
};

// Values of one step taped for the reverse stages; V = float (the fp32
// forward) or double (the fp64 replay).
template <typename V>
struct Tape {
  Buf<V> x1;     // 3*n_live: positions after advection (new order)
  Buf<V> vp;     // 3*n_live: velocities carried into P2G (new order)
  Buf<double> w; // n_gleaf*1536: P2G weight sums
  Buf<V> vsave;  // n_gleaf*1536: saved velocity (B val)
  Buf<V> unew;   // n_gleaf*1536: velocity after the pressure update
  Buf<V> dv;     // n_gleaf*1536: the velocity-update buffer G2P reads
};

struct Checkpoint {  // fp32 production state
  int64_t n = 0;
  Buf<float> part;  // 9*n SoA
  Buf<uint32_t> keys;
};
struct Checkpoint64 {  // fp64 replay state
  int64_t n = 0;
  Buf<double> st;  // 9*n SoA (x, v, g)
};

// Device view of the handle's current (restored) topology.
struct TopoView {
  LeafMap lm;
  SolidDesc sd;
  const int32_t* slot;
  const int32_t* leaf_id;
  const int8_t* marker;
  const uint32_t* vel_on;
  const uint32_t* touched;
  const uint32_t* normed;
  const uint8_t* side;  // recorded stencil sides (new order), or null: from the position
  int n_pleaf, n_gleaf;
};

__device__ __forceinline__ int node_slot(const TopoView& t, int i, int j, int k) {
  const int lx = fdiv(i, 8), ly = fdiv(j, 8), lz = fdiv(k, 8);
  if (!leaf_valid(t.lm, lx, ly, lz)) return -1;
  return t.slot[leaf_id(t.lm, lx, ly, lz)];
}
__device__ __forceinline__ int vox_of(int i, int j, int k) {
  return ((i & 7) << 6) | ((j & 7) << 3) | (k & 7);
}
__device__ __forceinline__ bool bit_at(const uint32_t* b, int s, int v) {
  return (b[int64_t(s) * 16 + (v >> 5)] >> (v & 31)) & 1u;
}
__device__ __forceinline__ bool normed_at(const TopoView& t, int s, int D, int v) {
  return (t.normed[(int64_t(s) * 3 + D) * 16 + (v >> 5)] >> (v & 31)) & 1u;
}
__device__ __forceinline__ void slot_origin(const TopoView& t, int s, int o[3]) {
  int lx, ly, lz;
  leaf_coords(t.lm, uint32_t(t.leaf_id[s]), lx, ly, lz);
  o[0] = lx * 8; o[1] = ly * 8; o[2] = lz * 8;
}
__device__ __forceinline__ void key_cell(const LeafMap& lm, uint32_t key, int c[3]) {
  int lx, ly, lz;
  leaf_coords(lm, key >> 9, lx, ly, lz);
  const int v = int(key & 511u);
  c[0] = lx * 8 + (v >> 6); c[1] = ly * 8 + ((v >> 3) & 7); c[2] = lz * 8 + (v & 7);
}
__device__ __forceinline__ int marker_at(const TopoView& t, int i, int j, int k) {
  const int s = node_slot(t, i, j, k);
  return s < 0 ? FSIM_AIR : int(t.marker[int64_t(s) * 512 + vox_of(i, j, k)]);
}
__device__ __forceinline__ bool in_nodes(const int n[3], const int g[3]) {
  return g[0] >= 0 && g[1] >= 0 && g[2] >= 0 && g[0] <= n[0] && g[1] <= n[1] && g[2] <= n[2];
}

// Lower MAC node of component D for a particle binned in cell c (the rule of
// ScatterWeight / InterpolateComponent, common/flip_simulation.cc:941-973)
// and the offsets of the position from it.  The side of the cell centre on
// each tangential axis is the recorded one (bit a of sb) when sb >= 0, so
// the frozen map stays one polynomial piece around the recorded positions;
// sb < 0 takes it from p.
__device__ __forceinline__ void mac_stencil(int D, const int c[3], const double p[3], int st[3],
                                            double fr[3], int sb) {
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    double lo = double(c[ax]);
    st[ax] = c[ax];
    if (ax != D) {
      lo += 0.5;
      const bool below = sb >= 0 ? ((sb >> ax) & 1) != 0 : p[ax] < lo;
      if (below) { lo -= 1.0; st[ax] -= 1; }
    }
    fr[ax] = p[ax] - lo;
  }
}
__device__ __forceinline__ int side_of(const TopoView& t, int64_t i) {
  return t.side ? int(t.side[i]) : -1;
}
// trilinear weight of corner (di,dj,dk) and its gradient in the position
__device__ __forceinline__ double tri_w(const double f[3], int di, int dj, int dk, double g[3]) {
  const double wx = di ? f[0] : 1.0 - f[0], wy = dj ? f[1] : 1.0 - f[1],
               wz = dk ? f[2] : 1.0 - f[2];
  const double sx = di ? 1.0 : -1.0, sy = dj ? 1.0 : -1.0, sz = dk ? 1.0 : -1.0;
  g[0] = sx * wy * wz;
  g[1] = wx * sy * wz;
  g[2] = wx * wy * sz;
  return wx * wy * wz;
}

// ---- recording ----------------------------------------------------------------
// Wall clamping of MoveParticles (common/particles.cc:519-542) per particle
// of the state before the step, with the production advection arithmetic.
__global__ void k_clamp_bits(const float* __restrict__ part, int64_t cap, int64_t n,
                             const uint32_t* __restrict__ keys, LeafMap lm, float dt,
                             uint8_t* __restrict__ out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint8_t b = 0;
  if (keys[i] != kDeadKey) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float p = __fadd_rn(part[d * cap + i], __fmul_rn(part[(6 + d) * cap + i], dt));
      const int id = int(floorf(p));
      if (id < 0) b |= uint8_t(1u << (2 * d));
      else if (id >= lm.n[d]) b |= uint8_t(2u << (2 * d));
    }
  }
  out[i] = b;
}

// entries where two u32 arrays differ
__global__ void k_count_diff(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                             int64_t n, unsigned long long* __restrict__ cnt) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n && a[i] != b[i]) atomicAdd(cnt, 1ull);
}

// Stencil sides of the production step's positions after advection (new
// order): float(c) + 0.5 is exact, so the fp32 comparison of ScatterWeight
// and this one agree.
__global__ void k_side_bits(const LeafMap lm, int64_t n, const uint32_t* __restrict__ keys,
                            const float* __restrict__ x1, uint8_t* __restrict__ side) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  key_cell(lm, keys[i], c);
  int b = 0;
#pragma unroll
  for (int ax = 0; ax < 3; ++ax)
    if (x1[ax * n + i] < float(c[ax]) + 0.5f) b |= 1 << ax;
  side[i] = uint8_t(b);
}

// Normalised-face bits: P2G wrote the face and its weight sum passed the cut.
__global__ void k_normed_bits(const TopoView t, const double* __restrict__ w,
                              uint32_t* __restrict__ out) {
  const int s = blockIdx.x;
  for (int q = threadIdx.x; q < 1536; q += blockDim.x) {
    const int D = q >> 9, v = q & 511;
    const bool on = bit_at(t.touched, s, v) && w[int64_t(s) * 1536 + q] > 1e-5;
    const unsigned ball = __ballot_sync(0xffffffffu, on);
    if ((threadIdx.x & 31) == 0) out[(int64_t(s) * 3 + D) * 16 + (v >> 5)] = ball;
  }
}

// P2G sums of the frozen map: w (and m when given) per face, fp64 atomics.
template <typename V>
__global__ void k_scatter(const TopoView t, int64_t n, const uint32_t* __restrict__ keys,
                          const V* __restrict__ x1, const V* __restrict__ vp,
                          double* __restrict__ m, double* __restrict__ w) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  key_cell(t.lm, keys[i], c);
  const double p[3] = {double(x1[i]), double(x1[n + i]), double(x1[2 * n + i])};
#pragma unroll
  for (int D = 0; D < 3; ++D) {
    int st[3];
    double fr[3];
    mac_stencil(D, c, p, st, fr, side_of(t, i));
    const double u = vp ? double(vp[D * n + i]) : 0.0;
    for (int q = 0; q < 8; ++q) {
      const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
      const int g[3] = {st[0] + di, st[1] + dj, st[2] + dk};
      const int s = node_slot(t, g[0], g[1], g[2]);
      if (s < 0) continue;
      double gw[3];
      const double ww = tri_w(fr, di, dj, dk, gw);
      const int64_t o = int64_t(s) * 1536 + D * 512 + vox_of(g[0], g[1], g[2]);
      atomicAdd(&w[o], ww);
      if (m) atomicAdd(&m[o], ww * u);
    }
  }
}

// float particle arrays of the handle (stride cap) -> packed tape (stride n)
template <typename V>
__global__ void k_pack3(const float* __restrict__ src, int64_t cap, int64_t n,
                        V* __restrict__ dst) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int d = 0; d < 3; ++d) dst[d * n + i] = V(src[d * cap + i]);
}
template <typename V>
__global__ void k_copy_field(const float* __restrict__ src, V* __restrict__ dst, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = V(src[i]);
}

// ---- fp64 replay of the frozen step ----------------------------------------------
// advection with the recorded clamps, then the recorded sort (gather by perm)
__global__ void k_rp_advect(const double* __restrict__ st, int64_t n_old, int64_t n_live,
                            const uint32_t* __restrict__ perm, const uint8_t* __restrict__ clamp,
                            LeafMap lm, double dt, double* __restrict__ x1,
                            double* __restrict__ vp) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n_live) return;
  const int64_t o = perm[i];
  const uint8_t cb = clamp[o];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double x = st[d * n_old + o] + st[(6 + d) * n_old + o] * dt;
    if (cb & (1u << (2 * d))) x = 0.0;
    if (cb & (2u << (2 * d))) x = double(lm.n[d]);
    x1[d * n_live + i] = x;
    vp[d * n_live + i] = st[(3 + d) * n_old + o];
  }
}

// normalisation, ApplyBoundaryConditions, SaveGridVelocities, AddGravity, BC
__global__ void k_rp_grid(const TopoView t, const double* __restrict__ m,
                          const double* __restrict__ w, double g0, double g1, double g2,
                          double* __restrict__ u, double* __restrict__ vsave) {
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  for (int q = threadIdx.x; q < 1536; q += blockDim.x) {
    const int D = q >> 9, v = q & 511;
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    const int64_t o = int64_t(s) * 1536 + q;
    const bool on = bit_at(t.touched, s, v);
    double val = (on && normed_at(t, s, D, v)) ? m[o] / w[o] : 0.0;
    const bool sc = is_solid(t.sd, g[0], g[1], g[2]);
    const bool zero = on && (sc != is_solid(t.sd, g[0] - (D == 0), g[1] - (D == 1), g[2] - (D == 2)));
    if (zero) val = 0.0;
    vsave[o] = val;
    const double gr = D == 0 ? g0 : (D == 1 ? -g1 : g2);
    u[o] = zero ? 0.0 : (on ? val + gr : val);
  }
}

// ComputeDivergence on the FLUID cells (particle leaves)
__global__ void k_rp_div(const TopoView t, const double* __restrict__ u, double* __restrict__ b) {
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  for (int v = threadIdx.x; v < 512; v += blockDim.x) {
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    double d = 0.0;
    if (t.marker[int64_t(s) * 512 + v] == FSIM_FLUID) {
#pragma unroll
      for (int D = 0; D < 3; ++D) {
        const int h[3] = {g[0] + (D == 0), g[1] + (D == 1), g[2] + (D == 2)};
        const int sh = node_slot(t, h[0], h[1], h[2]);
        const double up = sh < 0 ? 0.0 : u[int64_t(sh) * 1536 + D * 512 + vox_of(h[0], h[1], h[2])];
        d += up - u[int64_t(s) * 1536 + D * 512 + v];
      }
    }
    b[int64_t(s) * 512 + v] = d;
  }
}

// pressure-gradient face condition of UpdateVelocityFromPressure
// (common/flip_simulation.cc:739-778) for component d at node g
__device__ __forceinline__ bool grad_face(const TopoView& t, const int g[3], int d) {
  if (!in_nodes(t.lm.n, g)) return false;
  const int mc = marker_at(t, g[0], g[1], g[2]);
  if (mc == FSIM_SOLID) return false;
  const int mn = marker_at(t, g[0] - (d == 0), g[1] - (d == 1), g[2] - (d == 2));
  return (mn == FSIM_FLUID || mc == FSIM_FLUID) && mn != FSIM_SOLID;
}
__device__ __forceinline__ double cell_val(const TopoView& t, const double* x, int i, int j, int k) {
  const int s = node_slot(t, i, j, k);
  return (s < 0 || s >= t.n_pleaf) ? 0.0 : x[int64_t(s) * 512 + vox_of(i, j, k)];
}

// u_new = u + G p; dv = u_new - vsave on active in-box faces, else vsave
__global__ void k_rp_pupdate(const TopoView t, const double* __restrict__ u,
                             const double* __restrict__ vsave, const double* __restrict__ p,
                             double* __restrict__ unew, double* __restrict__ dv) {
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  for (int q = threadIdx.x; q < 1536; q += blockDim.x) {
    const int D = q >> 9, v = q & 511;
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    const int64_t o = int64_t(s) * 1536 + q;
    double val = u[o];
    if (grad_face(t, g, D))
      val += cell_val(t, p, g[0], g[1], g[2]) -
             cell_val(t, p, g[0] - (D == 0), g[1] - (D == 1), g[2] - (D == 2));
    unew[o] = val;
    dv[o] = (in_nodes(t.lm.n, g) && bit_at(t.vel_on, s, v)) ? val - vsave[o] : vsave[o];
  }
}

// interpolation of one component at the particle (ghost-extrapolated field,
// inactive faces read as 0), with the gradient in the position
template <typename V>
__device__ __forceinline__ double interp(const TopoView& t, const V* __restrict__ f,
                                         const uint32_t* __restrict__ on, int D, const int st[3],
                                         const double fr[3], double grad[3]) {
  double r = 0.0;
  grad[0] = grad[1] = grad[2] = 0.0;
  for (int q = 0; q < 8; ++q) {
    const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
    const int g[3] = {st[0] + di, st[1] + dj, st[2] + dk};
    int src[3];
    ghost_source(t.lm.n, D, g, src);
    const int s = node_slot(t, src[0], src[1], src[2]);
    if (s < 0) continue;
    const int v = vox_of(src[0], src[1], src[2]);
    if (!bit_at(on, s, v)) continue;
    const double val = double(f[int64_t(s) * 1536 + D * 512 + v]);
    double gw[3];
    r += tri_w(fr, di, dj, dk, gw) * val;
    grad[0] += gw[0] * val; grad[1] += gw[1] * val; grad[2] += gw[2] * val;
  }
  return r;
}

__global__ void k_rp_g2p(const TopoView t, int64_t n, const uint32_t* __restrict__ keys,
                         const double* __restrict__ x1, const double* __restrict__ vp,
                         const double* __restrict__ unew, const double* __restrict__ dv,
                         double flip, double* __restrict__ st) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  key_cell(t.lm, keys[i], c);
  const double p[3] = {x1[i], x1[n + i], x1[2 * n + i]};
#pragma unroll
  for (int D = 0; D < 3; ++D) {
    int s3[3];
    double fr[3], gd[3];
    mac_stencil(D, c, p, s3, fr, side_of(t, i));
    const double vi = interp(t, unew, t.vel_on, D, s3, fr, gd);
    const double di = interp(t, dv, t.touched, D, s3, fr, gd);
    st[D * n + i] = p[D];
    st[(3 + D) * n + i] = vi + flip * ((di + vp[D * n + i]) - vi);
    st[(6 + D) * n + i] = vi;
  }
}

// loss 0.5 sum (u - target)^2 over active in-box faces; seeds u-bar
template <typename V>
__global__ void k_loss(const TopoView t, const V* __restrict__ unew,
                       const float* __restrict__ target, double* __restrict__ loss,
                       double* __restrict__ ubar) {
  __shared__ double red[8];
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  const int* n = t.lm.n;
  const int64_t s1 = n[1] + 2, s2 = n[2] + 2;
  double acc = 0.0;
  for (int q = threadIdx.x; q < 1536; q += blockDim.x) {
    const int D = q >> 9, v = q & 511;
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    const int64_t o = int64_t(s) * 1536 + q;
    double d = 0.0;
    if (in_nodes(n, g) && bit_at(t.vel_on, s, v)) {
      const int64_t to = (int64_t(g[0] + 1) * s1 + (g[1] + 1)) * s2 + (g[2] + 1);
      d = double(unew[o]) - double(target[3 * to + D]);
      acc += 0.5 * d * d;
    }
    if (ubar) ubar[o] = d;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) a += red[w];
    atomicAdd(loss, a);
  }
}

// ---- reverse stages -------------------------------------------------------------
// G2P: v' = vi + f((di + v) - vi), g' = vi.  Scatters u-bar / dv-bar into the
// faces the interpolation read (through the ghost mapping), and adds the
// position derivative to x-bar; vp-bar = f v'-bar.
template <typename V>
__global__ void k_ad_g2p(const TopoView t, int64_t n, const uint32_t* __restrict__ keys,
                         const V* __restrict__ x1, const V* __restrict__ unew,
                         const V* __restrict__ dv, double flip, const double* __restrict__ vb,
                         const double* __restrict__ gb, double* __restrict__ ub,
                         double* __restrict__ dvb, double* __restrict__ xb,
                         double* __restrict__ vpb) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  key_cell(t.lm, keys[i], c);
  const double p[3] = {double(x1[i]), double(x1[n + i]), double(x1[2 * n + i])};
  double gx[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int D = 0; D < 3; ++D) {
    const double cv = (1.0 - flip) * vb[D * n + i] + gb[D * n + i];  // d L / d vi
    const double cd = flip * vb[D * n + i];                          // d L / d di
    vpb[D * n + i] = flip * vb[D * n + i];
    int st[3];
    double fr[3];
    mac_stencil(D, c, p, st, fr, side_of(t, i));
    for (int q = 0; q < 8; ++q) {
      const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
      const int g[3] = {st[0] + di, st[1] + dj, st[2] + dk};
      int src[3];
      ghost_source(t.lm.n, D, g, src);
      const int s = node_slot(t, src[0], src[1], src[2]);
      if (s < 0) continue;
      const int v = vox_of(src[0], src[1], src[2]);
      const int64_t o = int64_t(s) * 1536 + D * 512 + v;
      double gw[3];
      const double ww = tri_w(fr, di, dj, dk, gw);
      double k = 0.0;
      if (bit_at(t.vel_on, s, v)) {
        atomicAdd(&ub[o], ww * cv);
        k += double(unew[o]) * cv;
      }
      if (bit_at(t.touched, s, v)) {
        atomicAdd(&dvb[o], ww * cd);
        k += double(dv[o]) * cd;
      }
      gx[0] += gw[0] * k; gx[1] += gw[1] * k; gx[2] += gw[2] * k;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) xb[a * n + i] += gx[a];
}

// dv = u_new - vsave on active in-box faces (else the buffer keeps vsave):
// u-bar += dv-bar, vsave-bar = -dv-bar (or +dv-bar)
__global__ void k_ad_dv(const TopoView t, const double* __restrict__ dvb, double* __restrict__ ub,
                        double* __restrict__ vsb) {
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  for (int q = threadIdx.x; q < 1536; q += blockDim.x) {
    const int v = q & 511;
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    const int64_t o = int64_t(s) * 1536 + q;
    const double d = dvb[o];
    if (in_nodes(t.lm.n, g) && bit_at(t.vel_on, s, v)) {
      ub[o] += d;
      vsb[o] = -d;
    } else {
      vsb[o] = d;
    }
  }
}

// p-bar = G^T u-bar on the FLUID cells
__global__ void k_ad_pgrad(const TopoView t, const double* __restrict__ ub, double* __restrict__ pb) {
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  for (int v = threadIdx.x; v < 512; v += blockDim.x) {
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    double acc = 0.0;
    if (t.marker[int64_t(s) * 512 + v] == FSIM_FLUID) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (grad_face(t, g, d)) acc += ub[int64_t(s) * 1536 + d * 512 + v];
        const int h[3] = {g[0] + (d == 0), g[1] + (d == 1), g[2] + (d == 2)};
        if (grad_face(t, h, d)) {
          const int sh = node_slot(t, h[0], h[1], h[2]);
          if (sh >= 0) acc -= ub[int64_t(sh) * 1536 + d * 512 + vox_of(h[0], h[1], h[2])];
        }
      }
    }
    pb[int64_t(s) * 512 + v] = acc;
  }
}

// u-bar += D^T lambda
__global__ void k_ad_div(const TopoView t, const double* __restrict__ lam, double* __restrict__ ub) {
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  for (int q = threadIdx.x; q < 1536; q += blockDim.x) {
    const int D = q >> 9, v = q & 511;
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    const int h[3] = {g[0] - (D == 0), g[1] - (D == 1), g[2] - (D == 2)};
    double acc = 0.0;
    if (marker_at(t, h[0], h[1], h[2]) == FSIM_FLUID) acc += cell_val(t, lam, h[0], h[1], h[2]);
    if (s < t.n_pleaf && t.marker[int64_t(s) * 512 + v] == FSIM_FLUID)
      acc -= lam[int64_t(s) * 512 + v];
    ub[int64_t(s) * 1536 + q] += acc;
  }
}

// BC / save / gravity and normalisation: val-bar = B (u-bar + vsave-bar);
// m-bar = val-bar / w, w-bar = -val-bar val / w on normalised faces
template <typename V>
__global__ void k_ad_grid(const TopoView t, const double* __restrict__ ub,
                          const double* __restrict__ vsb, const V* __restrict__ vsave,
                          const double* __restrict__ w, double* __restrict__ mb,
                          double* __restrict__ wb) {
  const int s = blockIdx.x;
  int org[3];
  slot_origin(t, s, org);
  for (int q = threadIdx.x; q < 1536; q += blockDim.x) {
    const int D = q >> 9, v = q & 511;
    const int g[3] = {org[0] + (v >> 6), org[1] + ((v >> 3) & 7), org[2] + (v & 7)};
    const int64_t o = int64_t(s) * 1536 + q;
    double m_ = 0.0, w_ = 0.0;
    if (bit_at(t.touched, s, v) && normed_at(t, s, D, v)) {
      const bool sc = is_solid(t.sd, g[0], g[1], g[2]);
      const bool zero = sc != is_solid(t.sd, g[0] - (D == 0), g[1] - (D == 1), g[2] - (D == 2));
      if (!zero) {
        const double vb = ub[o] + vsb[o];
        m_ = vb / w[o];
        w_ = -vb * double(vsave[o]) / w[o];
      }
    }
    mb[o] = m_;
    wb[o] = w_;
  }
}

// P2G: vp-bar += sum W m-bar; x-bar += sum grad W (m-bar v + w-bar)
template <typename V>
__global__ void k_ad_p2g(const TopoView t, int64_t n, const uint32_t* __restrict__ keys,
                         const V* __restrict__ x1, const V* __restrict__ vp,
                         const double* __restrict__ mb, const double* __restrict__ wb,
                         double* __restrict__ xb, double* __restrict__ vpb) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  key_cell(t.lm, keys[i], c);
  const double p[3] = {double(x1[i]), double(x1[n + i]), double(x1[2 * n + i])};
  double gx[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int D = 0; D < 3; ++D) {
    int st[3];
    double fr[3];
    mac_stencil(D, c, p, st, fr, side_of(t, i));
    const double u = double(vp[D * n + i]);
    double acc = 0.0;
    for (int q = 0; q < 8; ++q) {
      const int di = q >> 2, dj = (q >> 1) & 1, dk = q & 1;
      const int g[3] = {st[0] + di, st[1] + dj, st[2] + dk};
      const int s = node_slot(t, g[0], g[1], g[2]);
      if (s < 0) continue;
      const int64_t o = int64_t(s) * 1536 + D * 512 + vox_of(g[0], g[1], g[2]);
      double gw[3];
      const double ww = tri_w(fr, di, dj, dk, gw);
      const double k = mb[o] * u + wb[o];
      acc += ww * mb[o];
      gx[0] += gw[0] * k; gx[1] += gw[1] * k; gx[2] += gw[2] * k;
    }
    vpb[D * n + i] += acc;
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) xb[a * n + i] += gx[a];
}

// advection and sort: x-bar, g-bar, v-bar of the state before the step
__global__ void k_ad_advect(int64_t n_live, int64_t n_old, const uint32_t* __restrict__ perm,
                            const uint8_t* __restrict__ clamp, double dt,
                            const double* __restrict__ xb, const double* __restrict__ vpb,
                            double* __restrict__ xb0, double* __restrict__ vb0,
                            double* __restrict__ gb0) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n_live) return;
  const int64_t o = perm[i];
  const uint8_t cb = clamp[o];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const bool cl = (cb >> (2 * d)) & 3u;
    const double x = cl ? 0.0 : xb[d * n_live + i];
    xb0[d * n_old + o] = x;
    gb0[d * n_old + o] = x * dt;
    vb0[d * n_old + o] = vpb[d * n_live + i];
  }
}

}  // namespace rb
}  // namespace fsim

using namespace fsim;
using namespace fsim::rb;

struct fsim_rollout {
  fsim_sim* s = nullptr;
  int steps = 0, every = 1;
  float dt = 0.f;
  fsim_pcg_params prm{};
  bool have_forward = false;
  Checkpoint init;
  std::vector<Checkpoint> ck;
  std::vector<TopoRec> topo;
  std::vector<Tape<float>> tape32;
  std::vector<Tape<double>> tape64;
  std::vector<Checkpoint64> ck64;
  Buf<float> target;
  // adjoint and replay work buffers
  Buf<double> xb, vpb, vb1, gb1, xb0, vb0, gb0;  // particles
  Buf<double> ub, dvb, vsb, mb, wb;             // faces
  Buf<double> cell;                             // p-bar / divergence (cells)
  Buf<double> st64, st64b, m64, u64;            // replay state and grid scratch
  Buf<double> loss;
  // PCG iterations of each step's replay solve, fixed by the first replay
  // after a forward (0: not yet)
  std::vector<int> replay_iters;
};

namespace {

int ck_err(fsim_sim* s, cudaError_t e, const char* what) {
  return e == cudaSuccess ? FSIM_OK : cuda_fail(s, e, what);
}
#define RB_CK(call)                                     \
  do {                                                  \
    int _rc = ck_err(r->s, (call), #call);              \
    if (_rc) return _rc;                                \
  } while (0)

template <typename T>
cudaError_t d2d(T* dst, const T* src, size_t count, cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  return cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToDevice, st);
}

TopoView view_of(fsim_rollout* r, const TopoRec* rec) {
  fsim_sim* s = r->s;
  TopoView t;
  t.lm = s->lm;
  t.sd = s->solid;
  t.slot = s->d_slot;
  t.leaf_id = s->d_leaf_id;
  t.marker = s->marker;
  t.vel_on = s->vel_on;
  t.touched = s->vold_on;
  t.normed = rec ? rec->normed.p : nullptr;
  t.side = rec ? rec->side.p : nullptr;
  t.n_pleaf = s->n_pleaf;
  t.n_gleaf = s->n_gleaf;
  return t;
}

// handle particle state <-> checkpoint
int save_state(fsim_rollout* r, Checkpoint& c) {
  fsim_sim* s = r->s;
  const int64_t n = s->n_total;
  c.n = n;
  RB_CK(c.part.reserve(size_t(9) * std::max<int64_t>(n, 1)));
  RB_CK(c.keys.reserve(size_t(std::max<int64_t>(n, 1))));
  for (int f = 0; f < 9; ++f)
    RB_CK(d2d(c.part.p + f * n, s->part[s->cur] + f * s->cap_p, size_t(n), s->stream));
  RB_CK(d2d(c.keys.p, s->keys[0], size_t(n), s->stream));
  return FSIM_OK;
}
int load_state(fsim_rollout* r, const Checkpoint& c) {
  fsim_sim* s = r->s;
  const int64_t n = c.n;
  for (int f = 0; f < 9; ++f)
    RB_CK(d2d(s->part[s->cur] + f * s->cap_p, c.part.p + f * n, size_t(n), s->stream));
  RB_CK(d2d(s->keys[0], c.keys.p, size_t(n), s->stream));
  s->n_total = s->n_live = n;
  s->have_topology = true;
  return FSIM_OK;
}

// the handle's topology buffers take the recorded topology of a step
int restore_topo(fsim_rollout* r, const TopoRec& t) {
  fsim_sim* s = r->s;
  int rc = ensure_leaf_capacity(s, t.n_gleaf, t.n_pleaf);
  if (rc) return rc;
  s->n_pleaf = t.n_pleaf;
  s->n_gleaf = t.n_gleaf;
  RB_CK(d2d(s->d_slot, t.slot.p, size_t(s->lm.dense), s->stream));
  RB_CK(d2d(s->d_leaf_id, t.leaf_id.p, size_t(t.n_gleaf), s->stream));
  RB_CK(d2d(s->d_nbr, t.nbr.p, size_t(t.n_gleaf) * 27, s->stream));
  RB_CK(d2d(s->d_cell_range, t.cell_range.p, size_t(t.n_pleaf) * 512, s->stream));
  RB_CK(d2d(s->d_leaf_range, t.leaf_range.p, size_t(t.n_pleaf), s->stream));
  RB_CK(d2d(s->marker, t.marker.p, size_t(t.n_gleaf) * 512, s->stream));
  RB_CK(d2d(s->vel_on, t.vel_on.p, size_t(t.n_gleaf) * 16, s->stream));
  RB_CK(d2d(s->vold_on, t.touched.p, size_t(t.n_gleaf) * 16, s->stream));
  return FSIM_OK;
}

void set_stage_flags(fsim_sim* s) {
  s->grid_valid = s->bc_applied = s->saved = s->phi_valid = true;
  s->div_valid = s->pres_valid = s->extrapolated = true;
  s->weight_valid = false;
  s->deleted_outside = false;
}

// One production step (the fsim_step sequence), recording the step's
// topology (rec) and/or its taped values (tp).
int prod_step(fsim_rollout* r, int k, bool rec, Tape<float>* tp) {
  fsim_sim* s = r->s;
  TopoRec& T = r->topo[size_t(k)];
  const int64_t n_old = s->n_total;
  if (rec) {
    T.n_old = n_old;
    RB_CK(T.clamp.reserve(size_t(std::max<int64_t>(n_old, 1))));
    FSIM_LAUNCH(s, "adj_clamp_bits", k_clamp_bits, nblk(n_old, 256), 256, 0, s->part[s->cur],
                s->cap_p, n_old, s->keys[0], s->lm, r->dt, T.clamp.p);
  }
  int rc = launch_keys_from_positions(s, 1, r->dt);
  if (rc) return rc;
  if ((rc = rebuild_topology(s))) return rc;
  const int64_t nl = s->n_live;
  if (!rec) {
    // a recomputed step must reproduce the recorded binning and order (the
    // step is bitwise deterministic; this guards the tape's indexing)
    if (nl != T.n_live || s->n_pleaf != T.n_pleaf || s->n_gleaf != T.n_gleaf)
      return fail(s, FSIM_ERR_STATE, "recomputed step differs from the recorded topology");
    unsigned long long* cnt = reinterpret_cast<unsigned long long*>(s->d_cnt + 7);
    RB_CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s->stream));
    FSIM_LAUNCH(s, "adj_check_keys", k_count_diff, nblk(nl, 256), 256, 0, s->keys[0], T.keys.p,
                nl, cnt);
    FSIM_LAUNCH(s, "adj_check_perm", k_count_diff, nblk(nl, 256), 256, 0, s->vals[0], T.perm.p,
                nl, cnt);
    RB_CK(cudaMemcpyAsync(s->h_cnt + 7, s->d_cnt + 7, sizeof(int64_t), cudaMemcpyDeviceToHost,
                          s->stream));
    RB_CK(cudaStreamSynchronize(s->stream));
    if (s->h_cnt[7] != 0)
      return fail(s, FSIM_ERR_STATE, "recomputed step differs from the recorded binning");
  }
  if (rec) {
    T.n_live = nl;
    T.n_pleaf = s->n_pleaf;
    T.n_gleaf = s->n_gleaf;
    const size_t np = size_t(std::max(s->n_pleaf, 1)), ng = size_t(std::max(s->n_gleaf, 1));
    RB_CK(T.perm.reserve(size_t(std::max<int64_t>(nl, 1))));
    RB_CK(T.keys.reserve(size_t(std::max<int64_t>(nl, 1))));
    RB_CK(T.slot.reserve(s->lm.dense));
    RB_CK(T.leaf_id.reserve(ng));
    RB_CK(T.nbr.reserve(ng * 27));
    RB_CK(T.cell_range.reserve(np * 512));
    RB_CK(T.leaf_range.reserve(np));
    RB_CK(T.marker.reserve(ng * 512));
    RB_CK(T.vel_on.reserve(ng * 16));
    RB_CK(T.touched.reserve(ng * 16));
    RB_CK(T.normed.reserve(ng * 48));
    RB_CK(d2d(T.perm.p, s->vals[0], size_t(nl), s->stream));
    RB_CK(d2d(T.keys.p, s->keys[0], size_t(nl), s->stream));
    RB_CK(d2d(T.slot.p, s->d_slot, size_t(s->lm.dense), s->stream));
    RB_CK(d2d(T.leaf_id.p, s->d_leaf_id, size_t(s->n_gleaf), s->stream));
    RB_CK(d2d(T.nbr.p, s->d_nbr, size_t(s->n_gleaf) * 27, s->stream));
    RB_CK(d2d(T.cell_range.p, s->d_cell_range, size_t(s->n_pleaf) * 512, s->stream));
    RB_CK(d2d(T.leaf_range.p, s->d_leaf_range, size_t(s->n_pleaf), s->stream));
  }
  set_stage_flags(s);
  if ((rc = launch_p2g(s, true, r->dt))) return rc;
  const size_t nf = size_t(s->n_gleaf) * 1536;
  if (rec || tp) {
    // P2G weight sums of the step (fp64), for the 1e-5 cut and the reverse
    Buf<double> wtmp;
    double* w = nullptr;
    if (tp) {
      RB_CK(tp->w.reserve(std::max<size_t>(nf, 1)));
      w = tp->w.p;
    } else {
      RB_CK(wtmp.reserve(std::max<size_t>(nf, 1)));
      w = wtmp.p;
    }
    RB_CK(cudaMemsetAsync(w, 0, nf * sizeof(double), s->stream));
    TopoView tv = view_of(r, nullptr);
    Buf<float> xs;
    RB_CK(xs.reserve(size_t(3) * std::max<int64_t>(nl, 1)));
    FSIM_LAUNCH(s, "adj_pack_pos", k_pack3<float>, nblk(nl, 256), 256, 0, s->part[s->cur],
                s->cap_p, nl, xs.p);
    if (rec) {
      RB_CK(T.side.reserve(size_t(std::max<int64_t>(nl, 1))));
      FSIM_LAUNCH(s, "adj_side_bits", k_side_bits, nblk(nl, 256), 256, 0, s->lm, nl,
                  s->keys[0], xs.p, T.side.p);
    }
    tv.side = T.side.p;  // recorded above, or by the recording pass of this step
    FSIM_LAUNCH(s, "adj_weights", k_scatter<float>, nblk(nl, 256), 256, 0, tv, nl, s->keys[0],
                xs.p, static_cast<const float*>(nullptr), static_cast<double*>(nullptr), w);
    if (rec) {
      RB_CK(d2d(T.marker.p, s->marker, size_t(s->n_gleaf) * 512, s->stream));
      RB_CK(d2d(T.touched.p, s->vold_on, size_t(s->n_gleaf) * 16, s->stream));
      FSIM_LAUNCH(s, "adj_normed_bits", k_normed_bits, s->n_gleaf, 256, 0, tv, w, T.normed.p);
    }
    if (tp) {
      RB_CK(tp->x1.reserve(size_t(3) * std::max<int64_t>(nl, 1)));
      RB_CK(tp->vp.reserve(size_t(3) * std::max<int64_t>(nl, 1)));
      RB_CK(tp->vsave.reserve(std::max<size_t>(nf, 1)));
      RB_CK(d2d(tp->x1.p, xs.p, size_t(3 * nl), s->stream));
      FSIM_LAUNCH(s, "adj_pack_vel", k_pack3<float>, nblk(nl, 256), 256, 0,
                  s->part[s->cur] + 3 * s->cap_p, s->cap_p, nl, tp->vp.p);
      RB_CK(d2d(tp->vsave.p, s->vold, nf, s->stream));
    }
    RB_CK(cudaStreamSynchronize(s->stream));  // the scratch buffers die here
  }
  if ((rc = launch_divergence(s))) return rc;
  fsim_pcg_stats ps;
  std::memset(&ps, 0, sizeof(ps));
  if ((rc = pcg_solve(s, &r->prm, &ps))) return rc;
  if (ps.status == FSIM_ERR_BREAKDOWN) return fail(s, FSIM_ERR_BREAKDOWN, "PCG breakdown");
  if ((rc = launch_pressure_update(s, true))) return rc;
  if (rec) RB_CK(d2d(T.vel_on.p, s->vel_on, size_t(s->n_gleaf) * 16, s->stream));
  if (tp) {
    RB_CK(tp->unew.reserve(std::max<size_t>(nf, 1)));
    RB_CK(tp->dv.reserve(std::max<size_t>(nf, 1)));
    RB_CK(d2d(tp->unew.p, s->vel, nf, s->stream));
    RB_CK(d2d(tp->dv.p, s->vold, nf, s->stream));
  }
  if ((rc = launch_g2p(s))) return rc;
  return FSIM_OK;
}

// loss of the face field u (tape layout) against the target; seeds u-bar
template <typename V>
int eval_loss(fsim_rollout* r, const TopoRec& t, const V* u, double* ubar, double* out) {
  fsim_sim* s = r->s;
  RB_CK(r->loss.reserve(1));
  RB_CK(cudaMemsetAsync(r->loss.p, 0, sizeof(double), s->stream));
  FSIM_LAUNCH(s, "adj_loss", k_loss<V>, t.n_gleaf, 256, 0, view_of(r, &t), u, r->target.p,
              r->loss.p, ubar);
  RB_CK(cudaMemcpyAsync(out, r->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  RB_CK(cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

fsim_pcg_params solve64_params() {
  fsim_pcg_params p;
  std::memset(&p, 0, sizeof(p));
  p.mode = FSIM_PCG_RELATIVE;
  p.precision = FSIM_PREC_FP64;
  p.max_iterations = 20000;
  p.max_refinements = 20;
  p.tolerance = 1e-12;
  p.inner_tolerance = 1e-3;
  return p;
}

// one fp64 replay step of the frozen map from st64 (old order) into st64b
// (new order); tp (optional) tapes the values
int replay_step(fsim_rollout* r, int k, Tape<double>* tp, bool last_loss, double* loss) {
  fsim_sim* s = r->s;
  const TopoRec& T = r->topo[size_t(k)];
  int rc = restore_topo(r, T);
  if (rc) return rc;
  const int64_t nl = T.n_live, no = T.n_old;
  const size_t nf = size_t(T.n_gleaf) * 1536;
  Tape<double> scratch;
  Tape<double>& V = tp ? *tp : scratch;
  RB_CK(V.x1.reserve(size_t(3) * std::max<int64_t>(nl, 1)));
  RB_CK(V.vp.reserve(size_t(3) * std::max<int64_t>(nl, 1)));
  RB_CK(V.w.reserve(std::max<size_t>(nf, 1)));
  RB_CK(V.vsave.reserve(std::max<size_t>(nf, 1)));
  RB_CK(V.unew.reserve(std::max<size_t>(nf, 1)));
  RB_CK(V.dv.reserve(std::max<size_t>(nf, 1)));
  RB_CK(r->m64.reserve(std::max<size_t>(nf, 1)));
  RB_CK(r->u64.reserve(std::max<size_t>(nf, 1)));
  RB_CK(r->cell.reserve(size_t(std::max(T.n_pleaf, 1)) * 512));
  RB_CK(r->st64b.reserve(size_t(9) * std::max<int64_t>(nl, 1)));
  const TopoView tv = view_of(r, &T);
  FSIM_LAUNCH(s, "rp_advect", k_rp_advect, nblk(nl, 256), 256, 0, r->st64.p, no, nl, T.perm.p,
              T.clamp.p, s->lm, double(r->dt), V.x1.p, V.vp.p);
  RB_CK(cudaMemsetAsync(r->m64.p, 0, nf * sizeof(double), s->stream));
  RB_CK(cudaMemsetAsync(V.w.p, 0, nf * sizeof(double), s->stream));
  FSIM_LAUNCH(s, "rp_p2g", k_scatter<double>, nblk(nl, 256), 256, 0, tv, nl, T.keys.p, V.x1.p,
              V.vp.p, r->m64.p, V.w.p);
  const double dt = double(r->dt);
  FSIM_LAUNCH(s, "rp_grid", k_rp_grid, T.n_gleaf, 256, 0, tv, r->m64.p, V.w.p,
              dt * double(s->cfg.force[0]), dt * double(s->cfg.force[1]),
              dt * double(s->cfg.force[2]), r->u64.p, V.vsave.p);
  FSIM_LAUNCH(s, "rp_divergence", k_rp_div, T.n_pleaf, 256, 0, tv, r->u64.p, r->cell.p);
  // The first replay after a forward solves each step to relative residual
  // 1e-12 and keeps the iteration count; later replays (the perturbed ones of
  // finite differences) run exactly that many iterations.  CG with a fixed
  // iteration count is a smooth function of its right-hand side, whereas a
  // stopping test switches the count, and with it the result at the level of
  // the solver's own error, between nearby right-hand sides.
  fsim_pcg_params p64 = solve64_params();
  int& fixed_iters = r->replay_iters[size_t(k)];
  if (fixed_iters > 0) {
    p64.mode = FSIM_PCG_FIXED;
    p64.max_iterations = fixed_iters;
  }
  fsim_pcg_stats ps;
  std::memset(&ps, 0, sizeof(ps));
  if ((rc = pcg_solve(s, &p64, &ps, r->cell.p))) return rc;
  if (ps.status == FSIM_ERR_BREAKDOWN) return fail(s, FSIM_ERR_BREAKDOWN, "replay PCG breakdown");
  if (fixed_iters <= 0) {
    if (ps.status != FSIM_OK) return fail(s, ps.status, "replay PCG did not converge");
    fixed_iters = std::max(ps.iterations, 1);
  }
  FSIM_LAUNCH(s, "rp_pressure_update", k_rp_pupdate, T.n_gleaf, 256, 0, tv, r->u64.p,
              V.vsave.p, s->x64, V.unew.p, V.dv.p);
  FSIM_LAUNCH(s, "rp_g2p", k_rp_g2p, nblk(nl, 256), 256, 0, tv, nl, T.keys.p, V.x1.p, V.vp.p,
              V.unew.p, V.dv.p, double(s->cfg.flip_factor), r->st64b.p);
  if (last_loss && (rc = eval_loss<double>(r, T, V.unew.p, nullptr, loss))) return rc;
  std::swap(r->st64.p, r->st64b.p);
  std::swap(r->st64.n, r->st64b.n);
  if (!tp) RB_CK(cudaStreamSynchronize(s->stream));  // scratch tape dies here
  return FSIM_OK;
}

// fp64 replay initial state: positions of the initial checkpoint, vel / gvel
// from the host (or the checkpoint)
int replay_init(fsim_rollout* r, const double* vel, const double* gvel) {
  fsim_sim* s = r->s;
  const int64_t n = r->init.n;
  RB_CK(r->st64.reserve(size_t(9) * std::max<int64_t>(n, 1)));
  FSIM_LAUNCH(s, "rp_init", k_copy_field<double>, nblk(9 * n, 256), 256, 0, r->init.part.p,
              r->st64.p, 9 * n);
  if (vel)
    RB_CK(cudaMemcpyAsync(r->st64.p + 3 * n, vel, size_t(3 * n) * sizeof(double),
                          cudaMemcpyHostToDevice, s->stream));
  if (gvel)
    RB_CK(cudaMemcpyAsync(r->st64.p + 6 * n, gvel, size_t(3 * n) * sizeof(double),
                          cudaMemcpyHostToDevice, s->stream));
  RB_CK(cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

// Reverse of one step along a tape (values V).  On entry vb1/gb1/xb hold the
// adjoints of the step's output particle state (new order) and ub the
// adjoint of the step's u_new (loss seed, or 0); on exit xb0/vb0/gb0 hold
// the adjoints of the state before the step (old order).
template <typename V>
int reverse_step(fsim_rollout* r, int k, const Tape<V>& tp, const fsim_pcg_params* adj) {
  fsim_sim* s = r->s;
  const TopoRec& T = r->topo[size_t(k)];
  int rc = restore_topo(r, T);
  if (rc) return rc;
  const TopoView tv = view_of(r, &T);
  const int64_t nl = T.n_live, no = T.n_old;
  const size_t nf = size_t(T.n_gleaf) * 1536;
  RB_CK(r->dvb.reserve(std::max<size_t>(nf, 1)));
  RB_CK(r->vsb.reserve(std::max<size_t>(nf, 1)));
  RB_CK(r->mb.reserve(std::max<size_t>(nf, 1)));
  RB_CK(r->wb.reserve(std::max<size_t>(nf, 1)));
  RB_CK(r->vpb.reserve(size_t(3) * std::max<int64_t>(nl, 1)));
  RB_CK(r->cell.reserve(size_t(std::max(T.n_pleaf, 1)) * 512));
  RB_CK(cudaMemsetAsync(r->dvb.p, 0, nf * sizeof(double), s->stream));
  const double flip = double(s->cfg.flip_factor);
  FSIM_LAUNCH(s, "adj_g2p", k_ad_g2p<V>, nblk(nl, 256), 256, 0, tv, nl, T.keys.p, tp.x1.p,
              tp.unew.p, tp.dv.p, flip, r->vb1.p, r->gb1.p, r->ub.p, r->dvb.p, r->xb.p, r->vpb.p);
  FSIM_LAUNCH(s, "adj_velocity_update", k_ad_dv, T.n_gleaf, 256, 0, tv, r->dvb.p, r->ub.p,
              r->vsb.p);
  FSIM_LAUNCH(s, "adj_pressure_gradient", k_ad_pgrad, T.n_pleaf, 256, 0, tv, r->ub.p, r->cell.p);
  fsim_pcg_stats ps;
  std::memset(&ps, 0, sizeof(ps));
  if ((rc = pcg_solve(s, adj, &ps, r->cell.p))) return rc;
  if (ps.status == FSIM_ERR_BREAKDOWN) return fail(s, FSIM_ERR_BREAKDOWN, "adjoint PCG breakdown");
  FSIM_LAUNCH(s, "adj_divergence", k_ad_div, T.n_gleaf, 256, 0, tv, s->x64, r->ub.p);
  FSIM_LAUNCH(s, "adj_grid", k_ad_grid<V>, T.n_gleaf, 256, 0, tv, r->ub.p, r->vsb.p,
              tp.vsave.p, tp.w.p, r->mb.p, r->wb.p);
  FSIM_LAUNCH(s, "adj_p2g", k_ad_p2g<V>, nblk(nl, 256), 256, 0, tv, nl, T.keys.p, tp.x1.p,
              tp.vp.p, r->mb.p, r->wb.p, r->xb.p, r->vpb.p);
  RB_CK(cudaMemsetAsync(r->xb0.p, 0, size_t(3 * no) * sizeof(double), s->stream));
  RB_CK(cudaMemsetAsync(r->vb0.p, 0, size_t(3 * no) * sizeof(double), s->stream));
  RB_CK(cudaMemsetAsync(r->gb0.p, 0, size_t(3 * no) * sizeof(double), s->stream));
  FSIM_LAUNCH(s, "adj_advect", k_ad_advect, nblk(nl, 256), 256, 0, nl, no, T.perm.p, T.clamp.p,
              double(r->dt), r->xb.p, r->vpb.p, r->xb0.p, r->vb0.p, r->gb0.p);
  // the state before this step is the output of the previous one
  std::swap(r->xb.p, r->xb0.p); std::swap(r->xb.n, r->xb0.n);
  std::swap(r->vb1.p, r->vb0.p); std::swap(r->vb1.n, r->vb0.n);
  std::swap(r->gb1.p, r->gb0.p); std::swap(r->gb1.n, r->gb0.n);
  return FSIM_OK;
}

int reserve_adjoint(fsim_rollout* r) {
  const size_t np = size_t(3) * std::max<int64_t>(r->init.n, 1);
  size_t nf = 1;
  for (const TopoRec& t : r->topo) nf = std::max(nf, size_t(t.n_gleaf) * 1536);
  for (Buf<double>* b : {&r->xb, &r->vb1, &r->gb1, &r->xb0, &r->vb0, &r->gb0})
    RB_CK(b->reserve(np));
  RB_CK(r->ub.reserve(nf));
  return FSIM_OK;
}

template <typename V>
int backward_impl(fsim_rollout* r, int tape, const fsim_pcg_params* adj) {
  fsim_sim* s = r->s;
  int rc = reserve_adjoint(r);
  if (rc) return rc;
  const int K = r->steps, C = r->every;
  const int nseg = (K + C - 1) / C;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int k0 = seg * C, k1 = std::min(K, k0 + C);
    // recompute the segment from its checkpoint, taping its values
    if (tape == 0) {
      if ((rc = load_state(r, r->ck[size_t(seg)]))) return rc;
      for (int k = k0; k < k1; ++k)
        if ((rc = prod_step(r, k, false, &r->tape32[size_t(k - k0)]))) return rc;
    } else {
      const Checkpoint64& c = r->ck64[size_t(seg)];
      RB_CK(r->st64.reserve(size_t(9) * std::max<int64_t>(c.n, 1)));
      RB_CK(d2d(r->st64.p, c.st.p, size_t(9 * c.n), s->stream));
      for (int k = k0; k < k1; ++k)
        if ((rc = replay_step(r, k, &r->tape64[size_t(k - k0)], false, nullptr))) return rc;
    }
    for (int k = k1 - 1; k >= k0; --k) {
      const TopoRec& T = r->topo[size_t(k)];
      const size_t nf = size_t(T.n_gleaf) * 1536;
      const Tape<V>* tp;
      if constexpr (sizeof(V) == 4) tp = &r->tape32[size_t(k - k0)];
      else tp = &r->tape64[size_t(k - k0)];
      if (k == K - 1) {
        // seeds: u-bar = u - target on the loss faces; no particle adjoint
        if ((rc = restore_topo(r, T))) return rc;
        double l = 0.0;
        if ((rc = eval_loss<V>(r, T, tp->unew.p, r->ub.p, &l))) return rc;
        for (Buf<double>* b : {&r->xb, &r->vb1, &r->gb1})
          RB_CK(cudaMemsetAsync(b->p, 0, size_t(3 * T.n_live) * sizeof(double), s->stream));
      } else {
        RB_CK(cudaMemsetAsync(r->ub.p, 0, nf * sizeof(double), s->stream));
      }
      if ((rc = reverse_step<V>(r, k, *tp, adj))) return rc;
    }
  }
  RB_CK(cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

}  // namespace

extern "C" {

int fsim_rollout_create(fsim_t* s, int32_t steps, int32_t every, fsim_rollout_t** out) {
  if (!s || !out || steps < 1 || every < 1) return FSIM_ERR_INVALID;
  *out = nullptr;
  cudaSetDevice(s->dev);
  if (!s->have_topology) return fail(s, FSIM_ERR_STATE, "no particles uploaded or seeded");
  if (s->cfg.boundary != FSIM_BOUNDARY_BOX)
    return fail(s, FSIM_ERR_INVALID, "the rollout supports the box boundary");
  fsim_rollout* r = new (std::nothrow) fsim_rollout();
  if (!r) return FSIM_ERR_CAPACITY;
  r->s = s;
  r->steps = steps;
  r->every = every;
  r->topo.resize(size_t(steps));
  r->ck.resize(size_t((steps + every - 1) / every));
  r->ck64.resize(r->ck.size());
  r->tape32.resize(size_t(std::min(steps, every)));
  r->tape64.resize(size_t(std::min(steps, every)));
  int rc = save_state(r, r->init);
  if (rc == FSIM_OK) rc = ck_err(s, cudaStreamSynchronize(s->stream), "rollout create");
  if (rc) {
    delete r;
    return rc;
  }
  *out = r;
  return FSIM_OK;
}

int fsim_rollout_destroy(fsim_rollout_t* r) {
  if (!r) return FSIM_ERR_INVALID;
  cudaSetDevice(r->s->dev);
  cudaStreamSynchronize(r->s->stream);
  delete r;
  return FSIM_OK;
}

int fsim_rollout_particle_count(fsim_rollout_t* r, int64_t* n) {
  if (!r || !n) return FSIM_ERR_INVALID;
  *n = r->init.n;
  return FSIM_OK;
}

int fsim_rollout_get_initial_velocity(fsim_rollout_t* r, double* vel, double* gvel) {
  if (!r) return FSIM_ERR_INVALID;
  fsim_sim* s = r->s;
  cudaSetDevice(s->dev);
  const int64_t n = r->init.n;
  std::vector<float> tmp(size_t(6 * n));
  RB_CK(cudaMemcpyAsync(tmp.data(), r->init.part.p + 3 * n, size_t(6 * n) * sizeof(float),
                        cudaMemcpyDeviceToHost, s->stream));
  RB_CK(cudaStreamSynchronize(s->stream));
  for (int64_t i = 0; i < 3 * n; ++i) {
    if (vel) vel[i] = double(tmp[size_t(i)]);
    if (gvel) gvel[i] = double(tmp[size_t(3 * n + i)]);
  }
  return FSIM_OK;
}

int fsim_rollout_set_initial_velocity(fsim_rollout_t* r, const double* vel, const double* gvel) {
  if (!r) return FSIM_ERR_INVALID;
  fsim_sim* s = r->s;
  cudaSetDevice(s->dev);
  const int64_t n = r->init.n;
  std::vector<float> tmp(size_t(3 * n));
  for (int f = 0; f < 2; ++f) {
    const double* src = f == 0 ? vel : gvel;
    if (!src) continue;
    for (int64_t i = 0; i < 3 * n; ++i) tmp[size_t(i)] = float(src[i]);
    RB_CK(cudaMemcpyAsync(r->init.part.p + (3 + 3 * f) * n, tmp.data(),
                          size_t(3 * n) * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    RB_CK(cudaStreamSynchronize(s->stream));
  }
  r->have_forward = false;
  return FSIM_OK;
}

int fsim_rollout_forward(fsim_rollout_t* r, float dt, const fsim_pcg_params* pcg,
                         const float* target, double* loss) {
  if (!r || !pcg || !target || !loss || !(dt > 0.f)) return FSIM_ERR_INVALID;
  fsim_sim* s = r->s;
  cudaSetDevice(s->dev);
  r->dt = dt;
  r->prm = *pcg;
  r->have_forward = false;
  r->replay_iters.assign(size_t(r->steps), 0);
  const int64_t nt = int64_t(s->lm.n[0] + 2) * (s->lm.n[1] + 2) * (s->lm.n[2] + 2) * 3;
  RB_CK(r->target.reserve(size_t(nt)));
  RB_CK(cudaMemcpyAsync(r->target.p, target, size_t(nt) * sizeof(float), cudaMemcpyHostToDevice,
                        s->stream));
  int rc = load_state(r, r->init);
  if (rc) return rc;
  for (int k = 0; k < r->steps; ++k) {
    if (k % r->every == 0 && (rc = save_state(r, r->ck[size_t(k / r->every)]))) return rc;
    if ((rc = prod_step(r, k, true, nullptr))) return rc;
  }
  const TopoRec& T = r->topo[size_t(r->steps - 1)];
  if ((rc = eval_loss<float>(r, T, s->vel, nullptr, loss))) return rc;
  r->have_forward = true;
  return FSIM_OK;
}

int fsim_rollout_replay_loss(fsim_rollout_t* r, const double* vel, const double* gvel,
                             double* loss) {
  if (!r || !loss) return FSIM_ERR_INVALID;
  if (!r->have_forward) return fail(r->s, FSIM_ERR_STATE, "run fsim_rollout_forward first");
  cudaSetDevice(r->s->dev);
  int rc = replay_init(r, vel, gvel);
  if (rc) return rc;
  for (int k = 0; k < r->steps; ++k)
    if ((rc = replay_step(r, k, nullptr, k == r->steps - 1, loss))) return rc;
  return FSIM_OK;
}

int fsim_rollout_backward(fsim_rollout_t* r, int32_t tape, const fsim_pcg_params* adj,
                          double* grad_vel, double* grad_gvel) {
  if (!r || !adj || (tape != 0 && tape != 1)) return FSIM_ERR_INVALID;
  fsim_sim* s = r->s;
  if (!r->have_forward) return fail(s, FSIM_ERR_STATE, "run fsim_rollout_forward first");
  if (adj->precision == FSIM_PREC_FP32)
    return fail(s, FSIM_ERR_INVALID, "adjoint solves need FP64 or MIXED precision");
  cudaSetDevice(s->dev);
  int rc;
  if (tape == 1) {
    // fp64 replay forward, checkpointing its state at the segment starts
    if ((rc = replay_init(r, nullptr, nullptr))) return rc;
    for (int k = 0; k < r->steps; ++k) {
      if (k % r->every == 0) {
        Checkpoint64& c = r->ck64[size_t(k / r->every)];
        c.n = r->topo[size_t(k)].n_old;
        RB_CK(c.st.reserve(size_t(9) * std::max<int64_t>(c.n, 1)));
        RB_CK(d2d(c.st.p, r->st64.p, size_t(9 * c.n), s->stream));
      }
      if ((rc = replay_step(r, k, nullptr, false, nullptr))) return rc;
    }
    rc = backward_impl<double>(r, 1, adj);
  } else {
    rc = backward_impl<float>(r, 0, adj);
  }
  if (rc) return rc;
  const int64_t n = r->init.n;
  if (grad_vel)
    RB_CK(cudaMemcpyAsync(grad_vel, r->vb1.p, size_t(3 * n) * sizeof(double),
                          cudaMemcpyDeviceToHost, s->stream));
  if (grad_gvel)
    RB_CK(cudaMemcpyAsync(grad_gvel, r->gb1.p, size_t(3 * n) * sizeof(double),
                          cudaMemcpyDeviceToHost, s->stream));
  RB_CK(cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

}  // extern "C"
