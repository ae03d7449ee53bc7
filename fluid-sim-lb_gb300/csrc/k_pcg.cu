// k_pcg.cu -- Jacobi-preconditioned CG pressure solve on the brick layout.
//
// Restates PCGDriver::Solve (common/solver_driver.cc:14-69) with the
// PCGSolver stages of common/solver.cc: PreparePCGSolver (:263-286),
// ComputeLocal1 (:297-309), ComputeLocal2 (:324-346), ComputeLocal3
// (:356-366), the loop test at the head of each iteration (:319-337) and
// CopySolution (:94-99).  The matrix is never stored: row (i,j,k) of the
// Laplacian of Solver::CreateLaplacianMatrix (:198-233) is diag = number of
// non-SOLID neighbours and -1 at each FLUID neighbour, so A*p only needs a
// per-cell flags byte (bit0 FLUID, bits1-3 diag).  The product is summed in
// the column order of the reference's sorted sparse rows (-x,-y,-z, diag,
// +z,+y,+x), which makes it bit-identical to the oracle for identical p.
//
// Per iteration two kernels run back to back on device-resident scalars
// (FSIM_PCG_CG1=1 runs fp32 solves by the single-reduction form below
// instead, one kernel per iteration):
//   spmv:   head: beta_{j-1} from the previous update's r.r, r.z partials
//           and the loop test; then p_j = z_j + beta_{j-1} p_{j-1} (z =
//           r/diag recomputed, never stored) and p_j.(A p_j) partials.
//   update: head: alpha from the spmv's p.Ap partials; then A p_j
//           recomputed from p_j (Ap is never stored), x += alpha p,
//           r -= alpha Ap, and r.r, r.z partials.
// Every CTA of a kernel sums its predecessor's partials itself (in one fixed
// order), so no last-CTA reduction separates two launches.
// HBM bytes per unknown per iteration: spmv reads r, p_{j-1}, flags and
// writes p_j (13 B); update reads p_j, x, r, flags and writes x, r (21 B).
// Each warp owns half a leaf: a lane holds one z-column of 8 cells in
// registers (loaded and stored as one 256-bit access), the x/y neighbour
// columns come from a per-warp shared tile, and only the faces of the half
// leaf are read from memory besides.  The iterations run as a CUDA graph
// whose conditional WHILE node stops on the device-side loop test; kernels
// launched after the stop flag is set return at once.
//
// Precision modes: FP32 (reference: fp32 vectors, fp32 dots), MIXED (fp32
// vectors, dots accumulated exactly: FMA error-free products and
// double-float sums per thread, fp64 above; plus an fp64 outer refinement
// r = b - A x with x kept in fp64) and FP64 (fp64 vectors and dots).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "fsim_internal.cuh"

namespace fsim {

namespace {

constexpr int kThreads = 256;     // setup / refinement kernels: one CTA per leaf pass
constexpr int kHotThreads = 128;  // spmv / update: 4 warps, one half leaf per warp
// Min resident CTAs per SM requested from ptxas for the hot kernels: 6
// (80 registers, no spills) for fp32 vectors, 2 for fp64.
#ifndef FSIM_PCG_MINB
#define FSIM_PCG_MINB 6
#endif
template <typename T>
constexpr int hot_minb() { return sizeof(T) == 4 ? FSIM_PCG_MINB : 2; }

// Jacobi: T(1.0/diag) (diag 0 gives inf, as 1.0/0 does in the reference)
__constant__ float c_invf[8] = {__builtin_inff(), 1.0f, 0.5f, float(1.0 / 3.0),
                                0.25f, float(1.0 / 5.0), float(1.0 / 6.0), float(1.0 / 7.0)};
__constant__ double c_invd[8] = {__builtin_inf(), 1.0, 0.5, 1.0 / 3.0,
                                 0.25, 1.0 / 5.0, 1.0 / 6.0, 1.0 / 7.0};

template <typename T>
__device__ __forceinline__ T inv_diag(uint8_t f);
template <>
__device__ __forceinline__ float inv_diag<float>(uint8_t f) {
  return (f & 1) ? c_invf[flag_diag(f)] : 0.f;
}
template <>
__device__ __forceinline__ double inv_diag<double>(uint8_t f) {
  return (f & 1) ? c_invd[flag_diag(f)] : 0.0;
}

__device__ __forceinline__ float tmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float tadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float tsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double tmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double tadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double tsub(double a, double b) { return __dsub_rn(a, b); }

// ---- dot accumulators ----------------------------------------------------
// DM 0: plain fp32; DM 1: exact products + double-float sum; DM 2: fp64.
template <int DM>
struct Dot;
template <>
struct Dot<0> {
  float s = 0.f;
  __device__ void add(float a, float b) { s = __fadd_rn(s, __fmul_rn(a, b)); }
  __device__ double value() const { return double(s); }
  __device__ float pvalue() const { return s; }  // block partial, in the partial type
};
template <>
struct Dot<1> {
  float hi = 0.f, lo = 0.f;
  __device__ void add(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);  // exact: a*b = p + e
    const float s = __fadd_rn(hi, p);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
  }
  __device__ double value() const { return double(hi) + double(lo); }
  __device__ float2 pvalue() const { return make_float2(hi, lo); }
};
template <>
struct Dot<2> {
  double s = 0.0;
  __device__ void add(double a, double b) { s = __fma_rn(a, b, s); }
  __device__ double value() const { return s; }
  __device__ double pvalue() const { return s; }
};

// Type of the hot kernels' block partials: fp32 for FP32 dots, a double-float
// pair (hi + lo, about 44 significant bits after the two-sum additions) for
// MIXED, fp64 for FP64.  The FP32 and MIXED sums across threads and CTAs so
// never touch GB300's narrow FP64 pipe.
template <int DM>
using PartT = typename std::conditional<DM == 0, float,
                                        typename std::conditional<DM == 1, float2, double>::type>::type;

// Addition of block partials (double-float: Knuth's two-sum of the high
// parts, the low parts added to its error, then a fast two-sum to
// renormalise; strict fp32 operations).
__device__ __forceinline__ float padd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double padd(double a, double b) { return a + b; }
__device__ __forceinline__ float2 padd(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bp = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bp)), __fsub_rn(b.x, bp));
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  const float hi = __fadd_rn(s, e);
  return make_float2(hi, __fsub_rn(e, __fsub_rn(hi, s)));
}
template <typename P>
__device__ __forceinline__ P pzero() { return P(0); }
template <>
__device__ __forceinline__ float2 pzero<float2>() { return make_float2(0.f, 0.f); }
__device__ __forceinline__ double ptod(float v) { return double(v); }
__device__ __forceinline__ double ptod(double v) { return v; }
__device__ __forceinline__ double ptod(float2 v) { return double(v.x) + double(v.y); }
__device__ __forceinline__ float pshfl_down(float v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double pshfl_down(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ float2 pshfl_down(float2 v, int o) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}

// Block-level sum of NV values.  DM 0 sums in fp32, otherwise fp64.
// Result valid in thread 0.
template <int DM, int NV, int NT = kThreads>
__device__ void block_sum(double (&v)[NV]) {
  __shared__ double sh[NV][NT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    if (DM == 0) {
      float x = float(v[k]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x = __fadd_rn(x, __shfl_down_sync(0xffffffffu, x, o));
      v[k] = double(x);
    } else {
      double x = v[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      v[k] = x;
    }
    if (lane == 0) sh[k][w] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      if (DM == 0) {
        float x = 0.f;
        for (int i = 0; i < NT / 32; ++i) x = __fadd_rn(x, float(sh[k][i]));
        v[k] = double(x);
      } else {
        double x = 0.0;
        for (int i = 0; i < NT / 32; ++i) x += sh[k][i];
        v[k] = x;
      }
    }
  }
  __syncthreads();
}

// Block sum of partial-typed values: warp tree, then thread 0 adds the warp
// results in order (for float, the order and so the totals of block_sum<0>).
// Result valid in thread 0.
template <typename P, int NV, int NT>
__device__ void block_sum_p(P (&v)[NV]) {
  __shared__ P sh[NV][NT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    P x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = padd(x, pshfl_down(x, o));
    v[k] = x;
    if (lane == 0) sh[k][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      P x = pzero<P>();
      for (int i = 0; i < NT / 32; ++i) x = padd(x, sh[k][i]);
      v[k] = x;
    }
  }
}

// Sum of nparts block partials per value (part[k * maxb + b]), in a fixed
// order: thread t adds partials t, t + NT, ... in batches of 8 independent
// loads, then the block tree of block_sum.  Every CTA that calls it on the
// same partials gets the same totals.  Result valid in thread 0.
template <int DM, int NV, int NT>
__device__ __forceinline__ void sum_parts(const double* part, int maxb, int nparts,
                                          double (&acc)[NV]) {
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double* pk = part + k * maxb;
    if (DM == 0) {
      float x = 0.f;
      for (int i0 = threadIdx.x; i0 < nparts; i0 += NT * 8) {
        float t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i0 + u * NT;
          t[u] = i < nparts ? float(__ldcg(pk + i)) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) x = __fadd_rn(x, t[u]);
      }
      acc[k] = double(x);
    } else {
      double x = 0.0;
      for (int i0 = threadIdx.x; i0 < nparts; i0 += NT * 8) {
        double t[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i0 + u * NT;
          t[u] = i < nparts ? __ldcg(pk + i) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) x += t[u];
      }
      acc[k] = x;
    }
  }
  block_sum<DM, NV, NT>(acc);
}

// Single-pass grid reduction: every block deposits its NV partials; the last
// block to arrive sums them in a fixed order (deterministic) and returns
// true in all of its threads with the totals in tot (thread 0).
template <int DM, int NV, int NT = kThreads>
__device__ bool grid_sum(double (&v)[NV], double* part, int maxb, unsigned int* counter,
                         double (&tot)[NV]) {
  __shared__ bool last;
  block_sum<DM, NV, NT>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) part[k * maxb + blockIdx.x] = v[k];
    __threadfence();
    unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[NV];
  sum_parts<DM, NV, NT>(part, maxb, int(gridDim.x), acc);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = acc[k];
    *counter = 0u;
  }
  return true;
}

struct PcgArgs {
  int n_pleaf;
  int maxb;
  const int32_t* nbr;
  const int8_t* marker;
  const float* b;   // divergence (fp32)
  const double* b64;  // fp64 right-hand side instead of b (adjoint / replay solves), or null
  uint8_t* flags;
  void* x;
  void* r;
  void* p0;
  void* p1;
  void* zf;         // z-face planes [leaf][r | p_a | p_b][plane][x*8+y]
  uint8_t* zff;     // flags z-face planes [leaf][plane][x*8+y]
  double* x64;      // MIXED outer solution
  float* dinner;    // MIXED inner solution (the fp32 x of the inner solve)
  PcgScalars* sc;
  double* part;
  float* partf;     // fp32 / double-float block partials of the hot kernels (FP32, MIXED)
  int init_r;       // setup: 1 -> r = b (x0 = 0); 0 -> r already holds the rhs
  int par;          // spmv / update: parity of the iteration this launch serves
  int withhold;     // bulk-copy spmv, test only: CTA 0's first stage withholds its flags copy
  int res_withhold; // resident loop, test only: CTA 0 skips its first barrier arrival
  cudaGraphConditionalHandle cond;  // WHILE-node handle when run as a graph, else 0
  void* w[2];       // single-reduction CG: w = A M r (by parity), or null
  void* sv[2];      // single-reduction CG: s = A p (by parity)
};

// The loop test and the rounding of a total to the vectors' type, from the
// solve's settings (mode, fp32, threshold).
struct PcgRule {
  int mode;
  bool fp32;
  double thr;
};
__device__ __forceinline__ PcgRule pcg_rule(const PcgScalars* sc) {
  return PcgRule{sc->mode, sc->fp32 != 0, sc->thr};
}
__device__ __forceinline__ bool converged(const PcgRule& q, double rr) {
  if (q.mode == FSIM_PCG_FIXED) return false;
  if (q.mode == FSIM_PCG_ABSOLUTE) {
    if (q.fp32) return float(rr) < float(q.thr);
    return rr < q.thr;
  }
  return rr <= q.thr;
}
__device__ __forceinline__ double round_t(const PcgRule& q, double v) {
  return q.fp32 ? double(float(v)) : v;
}
__device__ __forceinline__ bool converged(const PcgScalars* sc, double rr) {
  return converged(pcg_rule(sc), rr);
}
__device__ __forceinline__ double round_t(const PcgScalars* sc, double v) {
  return round_t(pcg_rule(sc), v);
}

// Flags from the marker, r = b (or keep), x = 0, and r.r, r.z, b.b.
template <typename T, int DM>
__global__ void __launch_bounds__(kThreads) k_pcg_setup(const __grid_constant__ PcgArgs a) {
  T* x = static_cast<T*>(a.x);
  T* r = static_cast<T*>(a.r);
  if (std::is_same<T, float>::value && blockIdx.x == gridDim.x - 1) {
    // the null slot n_pleaf read by the pipelined kernels' halo loads
    const int64_t o = int64_t(a.n_pleaf) * 512;
    for (int v = threadIdx.x; v < 512; v += kThreads) {
      a.flags[o + v] = 0;
      r[o + v] = T(0);
      static_cast<T*>(a.p0)[o + v] = T(0);
      static_cast<T*>(a.p1)[o + v] = T(0);
    }
    for (int v = threadIdx.x; v < 384; v += kThreads)
      static_cast<T*>(a.zf)[int64_t(a.n_pleaf) * 384 + v] = T(0);
    for (int v = threadIdx.x; v < 128; v += kThreads) a.zff[int64_t(a.n_pleaf) * 128 + v] = 0;
    if (a.w[0]) {  // the single-reduction loop's halo reads of w and s
      for (int v = threadIdx.x; v < 512; v += kThreads)
        for (int b = 0; b < 2; ++b) {
          static_cast<T*>(a.w[b])[o + v] = T(0);
          static_cast<T*>(a.sv[b])[o + v] = T(0);
        }
    }
  }
  Dot<DM> drr, drz, dbb;
  int nfluid = 0;
  for (int s = blockIdx.x; s < a.n_pleaf; s += gridDim.x) {
    const int32_t* nb = a.nbr + int64_t(s) * 27;
    for (int v = threadIdx.x; v < 512; v += kThreads) {
      const int64_t o = int64_t(s) * 512 + v;
      const int cx = v >> 6, cy = (v >> 3) & 7, cz = v & 7;
      uint8_t f = 0;
      if (a.marker[o] == FSIM_FLUID) {
        int diag = 0;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          int ax = cx, ay = cy, az = cz;
          const int d = (q & 1) ? 1 : -1;
          if (q < 2) ax += d; else if (q < 4) ay += d; else az += d;
          const int sx = ax < 0 ? -1 : (ax > 7 ? 1 : 0), sy = ay < 0 ? -1 : (ay > 7 ? 1 : 0),
                    sz = az < 0 ? -1 : (az > 7 ? 1 : 0);
          const int ns = nb[(sx + 1) * 9 + (sy + 1) * 3 + (sz + 1)];
          int m = FSIM_AIR;
          if (ns >= 0) m = a.marker[int64_t(ns) * 512 + (((ax & 7) << 6) | ((ay & 7) << 3) | (az & 7))];
          diag += (m != FSIM_SOLID);
        }
        f = uint8_t(1 | (diag << 1));
        ++nfluid;
      }
      a.flags[o] = f;
      x[o] = T(0);
      static_cast<T*>(a.p1)[o] = T(0);  // p_old of the first iteration
      T rv;
      if (a.init_r) {
        rv = (f & 1) ? (a.b64 ? T(a.b64[o]) : T(a.b[o])) : T(0);
        r[o] = rv;
      } else {
        rv = r[o];
      }
      if (cz == 0 || cz == 7) {
        const int fi = (cz == 7 ? 64 : 0) + cx * 8 + cy;
        a.zff[int64_t(s) * 128 + fi] = f;
        static_cast<T*>(a.zf)[int64_t(s) * 384 + fi] = rv;
        static_cast<T*>(a.zf)[int64_t(s) * 384 + 256 + fi] = T(0);
      }
      const T z = tmul(inv_diag<T>(f), rv);
      drr.add(rv, rv);
      drz.add(rv, z);
      dbb.add(rv, rv);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nfluid += __shfl_xor_sync(0xffffffffu, nfluid, o);
  if ((threadIdx.x & 31) == 0 && nfluid)
    atomicAdd(&a.sc->n_rows, (unsigned long long)nfluid);
  double v[3] = {drr.value(), drz.value(), dbb.value()};
  double tot[3];
  if (grid_sum<DM, 3>(v, a.part, a.maxb, &a.sc->cnt_s, tot) && threadIdx.x == 0) {
    PcgScalars* sc = a.sc;
    sc->rr = round_t(sc, tot[0]);
    sc->rz = round_t(sc, tot[1]);
    sc->bb = round_t(sc, tot[2]);
    sc->rr0 = sc->rr;
    sc->iter = 0;
    sc->status = FSIM_OK;
    sc->beta = 0.0;
    if (sc->mode == FSIM_PCG_RELATIVE) sc->thr = sc->tol2 * sc->bb;
    sc->done = (sc->max_iter <= 0) || converged(sc, sc->rr);
    // the first spmv takes r.r, r.z and beta = 0 from here
    PcgIterState o = {};
    o.rr = sc->rr;
    o.rz = sc->rz;
    o.beta = 0.0;
    o.rz_prev = 0.0;
    o.iter = 0;
    o.done = sc->done;
    o.status = FSIM_OK;
    o.given = 1;
    sc->st[1] = o;
  }
}

// ---- column-blocked leaf access -------------------------------------------
// One warp owns half of an 8^3 leaf (x in [0,4) or [4,8)).  Lane L owns the
// z-column (xb + (L>>3), L&7); a column is 8 contiguous cells (offset
// x*64 + y*8, 32 B of floats), so the z-neighbours are registers.  The x/y
// neighbour columns go through a per-warp shared tile (below); the columns
// just outside the half leaf (the other half's boundary plane like a
// neighbour face) are each loaded by one lane.  No CTA barrier in the hot
// loop: a warp synchronises only itself around the tile.
template <typename T>
struct Col {
  T v[8];
};

template <typename V>
__device__ __forceinline__ V ldv(const V* p) {
  return *p;
}

// Column offsets are multiples of 8 cells, so a float column starts 32-byte
// aligned: it moves as one 256-bit access per lane (sm_100 and later).  Two
// 128-bit accesses would each touch every 128-byte line of the half leaf, so
// the L1 pipeline would see each line twice.
__device__ __forceinline__ void unpack2(unsigned long long u, float& lo, float& hi) {
  lo = __uint_as_float(unsigned(u));
  hi = __uint_as_float(unsigned(u >> 32));
}
__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
  return (static_cast<unsigned long long>(__float_as_uint(hi)) << 32) | __float_as_uint(lo);
}
__device__ __forceinline__ void ldcol(const float* __restrict__ p, int64_t o, Col<float>& c) {
  const ulonglong4_32a a = *reinterpret_cast<const ulonglong4_32a*>(p + o);
  unpack2(a.x, c.v[0], c.v[1]);
  unpack2(a.y, c.v[2], c.v[3]);
  unpack2(a.z, c.v[4], c.v[5]);
  unpack2(a.w, c.v[6], c.v[7]);
}
__device__ __forceinline__ void ldcol(const double* __restrict__ p, int64_t o, Col<double>& c) {
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const double4_32a a = *reinterpret_cast<const double4_32a*>(p + o + 4 * k);
    c.v[4 * k] = a.x;
    c.v[4 * k + 1] = a.y;
    c.v[4 * k + 2] = a.z;
    c.v[4 * k + 3] = a.w;
  }
}
__device__ __forceinline__ void stcol(float* __restrict__ p, int64_t o, const Col<float>& c) {
  ulonglong4_32a a;
  a.x = pack2(c.v[0], c.v[1]);
  a.y = pack2(c.v[2], c.v[3]);
  a.z = pack2(c.v[4], c.v[5]);
  a.w = pack2(c.v[6], c.v[7]);
  *reinterpret_cast<ulonglong4_32a*>(p + o) = a;
}
__device__ __forceinline__ void stcol(double* __restrict__ p, int64_t o, const Col<double>& c) {
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    double4_32a a;
    a.x = c.v[4 * k];
    a.y = c.v[4 * k + 1];
    a.z = c.v[4 * k + 2];
    a.w = c.v[4 * k + 3];
    *reinterpret_cast<double4_32a*>(p + o + 4 * k) = a;
  }
}
__device__ __forceinline__ uint2 ldflags(const uint8_t* __restrict__ f, int64_t o) {
  return ldv(reinterpret_cast<const uint2*>(f + o));
}
__device__ __forceinline__ uint8_t fbyte(uint2 f, int z) {
  return uint8_t((z < 4 ? f.x : f.y) >> (8 * (z & 3)));
}

// The six face-neighbour slots of a leaf, gathered by lanes 0..5 and
// broadcast: 0 -x, 1 +x, 2 -y, 3 +y, 4 -z, 5 +z.  face_slot_lane loads the
// lane's entry (issued one half leaf ahead); face_slots broadcasts them.
__device__ __forceinline__ int face_slot_lane(const int32_t* nbr, int s, int lane) {
  int q = 13;
  if (lane == 0) q = 4; else if (lane == 1) q = 22; else if (lane == 2) q = 10;
  else if (lane == 3) q = 16; else if (lane == 4) q = 12; else if (lane == 5) q = 14;
  return (lane < 6) ? __ldg(nbr + (unsigned(s) * 27u + unsigned(q))) : -1;
}
__device__ __forceinline__ void face_slots(int mine, int out[6]) {
#pragma unroll
  for (int f = 0; f < 6; ++f) out[f] = __shfl_sync(0xffffffffu, mine, f);
}

// Work split of the hot kernels: one warp per half leaf (x in [xb, xb+4),
// xb = 0 or 4).  Lane (lx = lane>>3, cy = lane&7) owns the interior column
// (xb+lx, cy) and loads one face column of the half leaf's halo:
//   lx == 0: plane x = xb-1, column cy  (-x leaf, or this leaf's x=3 plane)
//   lx == 3: plane x = xb+4, column cy  (this leaf's x=4 plane, or +x leaf)
//   lx == 1: cy < 4: -y leaf column (xb+cy, 7); cy >= 4: +y leaf (xb+cy-4, 0)
//   lx == 2: none
// plus its own column's -z / +z face cells.  Columns are staged in a
// per-warp shared tile [x: xb-1..xb+4][y: -1..8][z: 0..7]; each lane then
// reads its four x/y neighbour columns with 16 B shared loads.
struct HalfLeaf {
  int s, xb, lx, cy, c, fidx;
  int tx, ty;  // halo column position in the tile
};
__device__ __forceinline__ HalfLeaf half_pos(int hw, int lane) {
  HalfLeaf h;
  h.s = hw >> 1;
  h.xb = (hw & 1) * 4;
  h.lx = lane >> 3;
  h.cy = lane & 7;
  h.c = ((h.xb + h.lx) << 6) | (h.cy << 3);
  h.fidx = (h.xb + h.lx) * 8 + h.cy;  // index of the column in a z-face plane
  h.tx = h.lx == 0 ? 0 : (h.lx == 3 ? 5 : (h.cy & 3) + 1);
  h.ty = h.lx == 1 ? (h.cy < 4 ? 0 : 9) : h.cy + 1;
  return h;
}
// The lane's halo column: leaf slot (-1: none) and first voxel.
__device__ __forceinline__ void halo_col(const HalfLeaf& h, const int fs[6], int& hslot,
                                         int& hvox) {
  hslot = -1;
  hvox = 0;
  if (h.lx == 0) {
    hslot = h.xb == 0 ? fs[0] : h.s;
    hvox = ((h.xb == 0 ? 7 : 3) << 6) | (h.cy << 3);
  } else if (h.lx == 3) {
    hslot = h.xb == 0 ? h.s : fs[1];
    hvox = ((h.xb == 0 ? 4 : 0) << 6) | (h.cy << 3);
  } else if (h.lx == 1) {
    const bool lo = h.cy < 4;
    hslot = lo ? fs[2] : fs[3];
    hvox = ((h.xb + (h.cy & 3)) << 6) | ((lo ? 7 : 0) << 3);
  }
}

// Jacobi inverse diagonal T(1.0/diag) by an exact select chain (pure ALU);
// diag 0 gives inf as 1.0/0 does; 0 for cells that are not FLUID.
template <typename T>
__device__ __forceinline__ T inv_sel(uint8_t f) {
  const int d = flag_diag(f);
  T v = T(1.0 / 7.0);
  v = d == 6 ? T(1.0 / 6.0) : v;
  v = d == 5 ? T(1.0 / 5.0) : v;
  v = d == 4 ? T(0.25) : v;
  v = d == 3 ? T(1.0 / 3.0) : v;
  v = d == 2 ? T(0.5) : v;
  v = d == 1 ? T(1.0) : v;
  v = d == 0 ? T(__builtin_inf()) : v;
  return (f & 1) ? v : T(0);
}

// {T(diag), T(1.0/diag)} by flags & 15 (bit 0 FLUID, bits 1-3 diag): the
// values of flag_diag and inv_sel, read from shared memory in one load
// instead of a compare/select chain per cell.
template <typename T>
struct __align__(2 * sizeof(T)) DiagInv {
  T d, inv;
};
template <typename T>
__device__ __forceinline__ void fill_diag_table(DiagInv<T>* tab) {
  if (threadIdx.x < 16) {
    const uint8_t f = uint8_t(threadIdx.x);
    tab[threadIdx.x].d = T(flag_diag(f));
    tab[threadIdx.x].inv = inv_sel<T>(f);
  }
}

// Per-warp tile of p_j columns, stored as 16 B chunk planes
// [chunk][x - xb + 1][y + 1]: the lanes of a quarter warp (consecutive y)
// touch consecutive 16 B words, so tile loads and stores are conflict-free.
template <typename T>
struct __align__(16) Tile {
  static constexpr int kV = int(sizeof(T)) / 2;  // 16 B chunks per 8-cell column
  uint4 c[kV][6][10];
};

template <typename T>
__device__ __forceinline__ void st_col_sh(Tile<T>& t, int x, int y, const Col<T>& c) {
#pragma unroll
  for (int k = 0; k < Tile<T>::kV; ++k) {
    uint4 u;
    memcpy(&u, &c.v[k * (16 / sizeof(T))], 16);
    t.c[k][x][y] = u;
  }
}
template <typename T>
__device__ __forceinline__ void ld_col_sh(const Tile<T>& t, int x, int y, Col<T>& c) {
#pragma unroll
  for (int k = 0; k < Tile<T>::kV; ++k) {
    const uint4 u = t.c[k][x][y];
    memcpy(&c.v[k * (16 / sizeof(T))], &u, 16);
  }
}

// A p on the lane's column, summed in the reference's column order
// (-x,-y,-z, diag, +z,+y,+x); 0 off-fluid.  The four x/y neighbour columns
// come from the tile; zm / zp are the -z / +z face cells.
template <typename T>
__device__ __forceinline__ void stencil_col(const Tile<T>& t, const DiagInv<T>* tab, int lx,
                                            int cy, const Col<T>& P, uint2 f, T zm, T zp,
                                            Col<T>& out) {
  Col<T> xm, xp, ym, yp;
  ld_col_sh(t, lx, cy + 1, xm);
  ld_col_sh(t, lx + 2, cy + 1, xp);
  ld_col_sh(t, lx + 1, cy, ym);
  ld_col_sh(t, lx + 1, cy + 2, yp);
#pragma unroll
  for (int z = 0; z < 8; ++z) {
    const uint8_t g = fbyte(f, z);
    const T vzm = z == 0 ? zm : P.v[(z + 7) & 7], vzp = z == 7 ? zp : P.v[(z + 1) & 7];
    T acc = T(0);
    acc = tsub(acc, xm.v[z]);
    acc = tsub(acc, ym.v[z]);
    acc = tsub(acc, vzm);
    acc = tadd(acc, tmul(tab[g & 15].d, P.v[z]));
    acc = tsub(acc, vzp);
    acc = tsub(acc, yp.v[z]);
    acc = tsub(acc, xp.v[z]);
    out.v[z] = (g & 1) ? acc : T(0);
  }
}

// p = z + beta p_old with z = r/diag.  Off-fluid both terms are 0 (the
// table's inverse is 0 there and r, p are stored 0), and at the first
// iteration beta = 0 and p_old was zeroed by the setup, so no select is needed.
template <typename T>
__device__ __forceinline__ T pnew_of(const DiagInv<T>* tab, uint8_t f, T r, T po, T beta) {
  return tadd(tmul(tab[f & 15].inv, r), tmul(beta, po));
}

// Programmatic dependent launch (the graph's edges are of programmatic type
// unless FSIM_PCG_PDL=0): a hot kernel may start while its predecessor's last CTAs
// finish.  Before pdl_wait() it reads only data written two or more launches
// back (flags, the neighbour table, and the one vector its predecessor does
// not write); pdl_wait() returns once the predecessor grid has completed and
// its writes are visible (at once without a programmatic edge).  Each kernel
// lets its successor launch only after its own wait, so a kernel never runs
// beside the one two launches back.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

// ---- deferred reductions ------------------------------------------------------
// The hot kernels do not finish their own dot products.  Each CTA writes its
// block partial and exits; every CTA of the NEXT kernel sums all of them in
// the same fixed order, so every CTA forms the same alpha or beta,
// deterministically, and no grid-wide atomic or last-CTA step sits between
// two launches: kernel order alone makes the partials visible.
// Partials: update -> spmv (r.r, r.z) at part[0], part[maxb]; spmv -> update
// (p.Ap) at part[3 * maxb].  The rest of the iteration state goes through
// PcgScalars::st: each kernel reads its predecessor's slot and CTA 0 writes
// the other (st[0] spmv -> update, st[1] update -> spmv); the public fields
// (rr, iter, done, status, ...) are written by CTA 0 for the host.
//
// A kernel's head first copies the partial rows and the scalar block into
// shared memory with cp.async (no registers held), then issues its first half
// leaf's loads, and only then waits for the copies and sums: the L2 round
// trip of the head hides under the first loads from HBM.
constexpr int kPartPAp = 3;       // part[] row of the spmv's p.Ap partials
constexpr int kMaxHotGrid = 1022; // hot grids stay below this (even) size
constexpr int kZDirectLeaves = 16384;  // above this many particle leaves: direct z-face reads

struct HotHead {
  int done;
  double s;  // beta (spmv) or alpha (update)
};

template <int NV, typename P>
struct HeadStage {
  P part[NV][kMaxHotGrid + 2];
  PcgScalars sc;
  HotHead out;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

template <int DM>
__device__ __forceinline__ PartT<DM>* part_rows(const PcgArgs& a) {
  if constexpr (DM == 2) return a.part;
  else return reinterpret_cast<PartT<DM>*>(a.partf);
}

// Copies partial rows row0 .. row0+NV-1 of the previous launch (same grid)
// and the scalar block into hs.  Rows start 16-byte aligned (maxb is a
// multiple of 4) and a row copy may take up to 3 values past gridDim.x,
// which lie inside the row and inside hs.part.
template <int DM, int NV>
__device__ __forceinline__ void head_issue(HeadStage<NV, PartT<DM>>& hs, const PcgArgs& a,
                                           int row0) {
  constexpr int per = 16 / int(sizeof(PartT<DM>));
  const int nch = (int(gridDim.x) + per - 1) / per;  // 16-byte chunks per row
  const PartT<DM>* rows = part_rows<DM>(a);
#pragma unroll
  for (int k = 0; k < NV; ++k)
    for (int c = threadIdx.x; c < nch; c += kHotThreads)
      cp_async16(&hs.part[k][per * c], rows + int64_t(row0 + k) * a.maxb + per * c);
  constexpr int nsc = int(sizeof(PcgScalars)) / 16;
  for (int c = threadIdx.x; c < nsc; c += kHotThreads)
    cp_async16(reinterpret_cast<char*>(&hs.sc) + 16 * c,
               reinterpret_cast<const char*>(a.sc) + 16 * c);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Waits for the copies and sums each row in the order of sum_parts (thread t
// adds partials t, t + 128, ...; then the block tree).  Result valid in
// thread 0.
template <int DM, int NV>
__device__ __forceinline__ void head_sum(HeadStage<NV, PartT<DM>>& hs, double (&acc)[NV]) {
  using P = PartT<DM>;
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  const int nparts = int(gridDim.x);
  P x[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    x[k] = pzero<P>();
    for (int i = threadIdx.x; i < nparts; i += kHotThreads) x[k] = padd(x[k], hs.part[k][i]);
  }
  block_sum_p<P, NV, kHotThreads>(x);
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = ptod(x[k]);  // thread 0 uses them
}

// Head of the spmv of iteration j: r.r, r.z of the previous update (summed
// from its partials, or given by setup / residual replacement), beta =
// r.z / r.z_old with ComputeLocal3's CHECK_LE(beta, LARGE_FLOAT), then the
// loop test of PCGDriver::Solve (iterations >= max, or converged).
template <int DM>
__device__ __forceinline__ HotHead spmv_head(HeadStage<2, PartT<DM>>& hs, const PcgArgs& a) {
  double acc[2];
  head_sum<DM, 2>(hs, acc);
  if (threadIdx.x == 0) {
    const PcgScalars* cs = &hs.sc;  // the scalar block as the previous launch left it
    const PcgIterState in = cs->st[1];
    double rr, rz, beta;
    if (in.given) {
      rr = in.rr;
      rz = in.rz;
      beta = in.beta;
    } else {
      rr = round_t(cs, acc[0]);
      rz = round_t(cs, acc[1]);
      beta = cs->fp32 ? double(__fdiv_rn(float(rz), float(in.rz_prev))) : rz / in.rz_prev;
    }
    int done = in.done, status = in.status;
    if (!done) {
      if (!in.given && !(beta <= 1e5)) {  // CHECK_LE(beta, LARGE_FLOAT)
        status = FSIM_ERR_BREAKDOWN;
        done = 1;
      } else {
        done = (in.iter >= cs->max_iter) || converged(cs, rr);
      }
    }
    if (blockIdx.x == 0) {
      PcgScalars* sc = a.sc;
      if (in.done) {
        sc->st[0].done = 1;  // nothing new: pass the stop flag on
      } else {
        PcgIterState o = in;
        o.rr = rr;
        o.rz = rz;
        o.beta = beta;
        o.done = done;
        o.status = status;
        o.given = 0;
        sc->st[0] = o;
        sc->rr = rr;
        sc->rz = rz;
        sc->rz_old = in.rz_prev;
        sc->beta = beta;
        sc->iter = in.iter;
        sc->status = status;
        sc->done = done;
      }
      if (done && a.cond) cudaGraphSetConditional(a.cond, 0u);  // ends the WHILE loop
    }
    hs.out.done = done;
    hs.out.s = beta;
  }
  __syncthreads();
  return hs.out;
}

// Head of the update of iteration j: p.Ap summed from the spmv's partials,
// alpha = r.z / p.Ap with ComputeLocal2's CHECK_LE(alpha, LARGE_FLOAT).
template <int DM>
__device__ __forceinline__ HotHead update_head(HeadStage<1, PartT<DM>>& hs, const PcgArgs& a) {
  double acc[1];
  head_sum<DM, 1>(hs, acc);
  if (threadIdx.x == 0) {
    const PcgScalars* cs = &hs.sc;
    const PcgIterState in = cs->st[0];
    int done = in.done, status = in.status;
    double alpha = 0.0, pAp = 0.0;
    if (!done) {
      pAp = round_t(cs, acc[0]);
      alpha = cs->fp32 ? double(__fdiv_rn(float(in.rz), float(pAp))) : in.rz / pAp;
      if (!(alpha <= 1e5)) {  // CHECK_LE(alpha, LARGE_FLOAT)
        status = FSIM_ERR_BREAKDOWN;
        done = 1;
      }
    }
    if (blockIdx.x == 0) {
      PcgScalars* sc = a.sc;
      if (in.done) {
        sc->st[1].done = 1;
      } else {
        sc->pAp = pAp;
        sc->alpha = alpha;
        if (done) {
          sc->st[1].done = 1;
          sc->st[1].status = status;
          sc->status = status;
          sc->done = 1;
        } else {
          PcgIterState o = {};
          o.rr = 0.0;
          o.rz = 0.0;
          o.beta = 0.0;
          o.rz_prev = in.rz;
          o.iter = in.iter + 1;
          o.done = 0;
          o.status = status;
          o.given = 0;
          sc->st[1] = o;
          sc->iter = in.iter + 1;
        }
      }
      if (done && a.cond) cudaGraphSetConditional(a.cond, 0u);
    }
    hs.out.done = done;
    hs.out.s = alpha;
  }
  __syncthreads();
  return hs.out;
}

// This CTA's share of a dot product, for the next kernel's head.
template <int DM, int NV>
__device__ __forceinline__ void put_partials(const PcgArgs& a, int row0, PartT<DM> (&v)[NV]) {
  block_sum_p<PartT<DM>, NV, kHotThreads>(v);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) part_rows<DM>(a)[(row0 + k) * a.maxb + blockIdx.x] = v[k];
  }
}

// Each launch of the hot kernels serves one iteration of known parity
// (PcgArgs::par), so its buffers are fixed before the scalars are known: the
// first half leaf's own-column loads are issued before the head sums the
// previous kernel's partials.
//
// p_j = z_j + beta_{j-1} p_{j-1} on the half leaf and its halo (z = r/diag
// recomputed, never stored), then this CTA's part of p_j.(A p_j).  Only p_j
// is written: the update kernel recomputes A p_j from it.
template <typename T, int DM>
__global__ void __launch_bounds__(kHotThreads, hot_minb<T>())
    k_pcg_spmv(const __grid_constant__ PcgArgs a) {
  pdl_wait();  // reads its predecessor's outputs from the start
  pdl_trigger();
  __shared__ Tile<T> tiles[kHotThreads / 32];
  __shared__ DiagInv<T> tab[16];
  __shared__ HeadStage<2, PartT<DM>> hs;
  const int par = a.par;
  const T* r = static_cast<const T*>(a.r);
  const T* pold = static_cast<const T*>(par ? a.p0 : a.p1);
  T* pnew = static_cast<T*>(par ? a.p1 : a.p0);
  const int qold = 1 + (par ^ 1), qnew = 1 + par;
  const int lane = threadIdx.x & 31;
  const int wpb = kHotThreads / 32;
  const int nhw = 2 * a.n_pleaf, hstride = gridDim.x * wpb;
  int hw = blockIdx.x * wpb + (threadIdx.x >> 5);
  head_issue<DM, 2>(hs, a, 0);
  // first half leaf: flags, p_{j-1}, r and the face slots
  Col<T> rc, pc;
  uint2 f = make_uint2(0u, 0u);
  const int64_t o0 = hw < nhw ? int64_t(hw >> 1) * 512 + half_pos(hw, lane).c : 0;
  if (hw < nhw) {
    f = ldflags(a.flags, o0);
    ldcol(pold, o0, pc);
    ldcol(r, o0, rc);
  }
  int nbl = hw < nhw ? face_slot_lane(a.nbr, hw >> 1, lane) : -1;
  fill_diag_table<T>(tab);
  const HotHead head = spmv_head<DM>(hs, a);
  if (head.done) return;
  const T beta = T(head.s);
  Tile<T>& tile = tiles[threadIdx.x >> 5];
  Dot<DM> dp;
  for (; hw < nhw; hw += hstride) {
    const int nbl_next = hw + hstride < nhw ? face_slot_lane(a.nbr, (hw + hstride) >> 1, lane) : -1;
    int fs[6];
    face_slots(nbl, fs);
    nbl = nbl_next;
    const HalfLeaf h = half_pos(hw, lane);
    int hslot, hvox;
    halo_col(h, fs, hslot, hvox);
    // halo column
    const bool hv = hslot >= 0 && hslot < a.n_pleaf;
    const int64_t hb = int64_t(hv ? hslot : 0) * 512 + hvox;
    uint2 hf = make_uint2(0u, 0u);
    Col<T> hr, hp;
    if (hv) {
      hf = ldflags(a.flags, hb);
      ldcol(r, hb, hr);
      ldcol(pold, hb, hp);
    } else {
#pragma unroll
      for (int z = 0; z < 8; ++z) hr.v[z] = hp.v[z] = T(0);
    }
    // z faces of the own column, from the neighbours' published planes:
    // the -z leaf's z=7 plane and the +z leaf's z=0 plane
    const int zs0 = fs[4], zs1 = fs[5];
    const bool zv0 = zs0 >= 0 && zs0 < a.n_pleaf, zv1 = zs1 >= 0 && zs1 < a.n_pleaf;
    const T* zf = static_cast<const T*>(a.zf);
    const int64_t zo0 = int64_t(zv0 ? zs0 : 0) * 384 + 64 + h.fidx;
    const int64_t zo1 = int64_t(zv1 ? zs1 : 0) * 384 + h.fidx;
    const uint8_t zf0 = zv0 ? ldv(a.zff + int64_t(zs0) * 128 + 64 + h.fidx) : uint8_t(0);
    const uint8_t zf1 = zv1 ? ldv(a.zff + int64_t(zs1) * 128 + h.fidx) : uint8_t(0);
    const T zr0 = zv0 ? ldv(zf + zo0) : T(0), zr1 = zv1 ? ldv(zf + zo1) : T(0);
    const T zq0 = zv0 ? ldv(zf + zo0 + 128 * qold) : T(0);
    const T zq1 = zv1 ? ldv(zf + zo1 + 128 * qold) : T(0);
    Col<T> P, H;
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      P.v[z] = pnew_of<T>(tab, fbyte(f, z), rc.v[z], pc.v[z], beta);
      H.v[z] = pnew_of<T>(tab, fbyte(hf, z), hr.v[z], hp.v[z], beta);
    }
    const T zm = pnew_of<T>(tab, zf0, zr0, zq0, beta);
    const T zp = pnew_of<T>(tab, zf1, zr1, zq1, beta);
    const int64_t o = int64_t(h.s) * 512 + h.c;
    stcol(pnew, o, P);
    {
      T* zw = static_cast<T*>(a.zf) + int64_t(h.s) * 384 + 128 * qnew + h.fidx;
      zw[0] = P.v[0];
      zw[64] = P.v[7];
    }
    __syncwarp();  // previous half leaf's tile reads are done
    st_col_sh(tile, h.lx + 1, h.cy + 1, P);
    if (h.lx != 2) st_col_sh(tile, h.tx, h.ty, H);
    __syncwarp();
    const uint2 fc = f;
    // next half leaf's own column (registers of this one are free now)
    if (hw + hstride < nhw) {
      const HalfLeaf hn = half_pos(hw + hstride, lane);
      const int64_t on = int64_t(hn.s) * 512 + hn.c;
      f = ldflags(a.flags, on);
      ldcol(r, on, rc);
      ldcol(pold, on, pc);
    }
    Col<T> ap;
    stencil_col<T>(tile, tab, h.lx, h.cy, P, fc, zm, zp, ap);
    // off-fluid P and Ap are 0: their terms add exact zeros
#pragma unroll
    for (int z = 0; z < 8; ++z) dp.add(P.v[z], ap.v[z]);
  }
  PartT<DM> v[1] = {dp.pvalue()};
  put_partials<DM, 1>(a, kPartPAp, v);
}

// A p_j recomputed from p_j (half leaf + halo); x += alpha p;
// r -= alpha Ap; this CTA's parts of r.r and r.z.
template <typename T, int DM>
__global__ void __launch_bounds__(kHotThreads, hot_minb<T>())
    k_pcg_update(const __grid_constant__ PcgArgs a) {
  pdl_wait();  // reads its predecessor's outputs from the start
  pdl_trigger();
  __shared__ Tile<T> tiles[kHotThreads / 32];
  __shared__ DiagInv<T> tab[16];
  __shared__ HeadStage<1, PartT<DM>> hs;
  const int par = a.par;
  const T* p = static_cast<const T*>(par ? a.p1 : a.p0);
  T* x = static_cast<T*>(a.x);
  T* r = static_cast<T*>(a.r);
  const int qcur = 1 + par;
  const int lane = threadIdx.x & 31;
  const int wpb = kHotThreads / 32;
  const int nhw = 2 * a.n_pleaf, hstride = gridDim.x * wpb;
  int hw = blockIdx.x * wpb + (threadIdx.x >> 5);
  head_issue<DM, 1>(hs, a, kPartPAp);
  // first half leaf: flags, x, r, p_j and the face slots
  Col<T> P, xc, rc;
  uint2 f = make_uint2(0u, 0u);
  const int64_t o0 = hw < nhw ? int64_t(hw >> 1) * 512 + half_pos(hw, lane).c : 0;
  if (hw < nhw) {
    f = ldflags(a.flags, o0);
    ldcol(x, o0, xc);
    ldcol(r, o0, rc);
    ldcol(p, o0, P);
  }
  int nbl = hw < nhw ? face_slot_lane(a.nbr, hw >> 1, lane) : -1;
  fill_diag_table<T>(tab);
  const HotHead head = update_head<DM>(hs, a);
  if (head.done) return;
  const T alpha = T(head.s);
  const T nalpha = -alpha;
  Tile<T>& tile = tiles[threadIdx.x >> 5];
  Dot<DM> drr, drz;
  for (; hw < nhw; hw += hstride) {
    const int nbl_next = hw + hstride < nhw ? face_slot_lane(a.nbr, (hw + hstride) >> 1, lane) : -1;
    int fs[6];
    face_slots(nbl, fs);
    nbl = nbl_next;
    const HalfLeaf h = half_pos(hw, lane);
    int hslot, hvox;
    halo_col(h, fs, hslot, hvox);
    Col<T> H;
    const bool hv = hslot >= 0 && hslot < a.n_pleaf;
    if (hv) {
      ldcol(p, int64_t(hslot) * 512 + hvox, H);
    } else {
#pragma unroll
      for (int z = 0; z < 8; ++z) H.v[z] = T(0);
    }
    const int zs0 = fs[4], zs1 = fs[5];
    const T* zfp = static_cast<const T*>(a.zf) + 128 * qcur + h.fidx;
    const T zm = (zs0 >= 0 && zs0 < a.n_pleaf) ? ldv(zfp + int64_t(zs0) * 384 + 64) : T(0);
    const T zp = (zs1 >= 0 && zs1 < a.n_pleaf) ? ldv(zfp + int64_t(zs1) * 384) : T(0);
    __syncwarp();  // previous half leaf's tile reads are done
    st_col_sh(tile, h.lx + 1, h.cy + 1, P);
    if (h.lx != 2) st_col_sh(tile, h.tx, h.ty, H);
    __syncwarp();
    Col<T> ap;
    stencil_col<T>(tile, tab, h.lx, h.cy, P, f, zm, zp, ap);
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      const uint8_t g = fbyte(f, z);
      xc.v[z] = tadd(tmul(alpha, P.v[z]), xc.v[z]);
      rc.v[z] = tadd(tmul(nalpha, ap.v[z]), rc.v[z]);
      // off-fluid r is 0 (Ap is 0 there): the terms add exact zeros
      drr.add(rc.v[z], rc.v[z]);
      drz.add(rc.v[z], tmul(tab[g & 15].inv, rc.v[z]));
    }
    const int64_t o = int64_t(h.s) * 512 + h.c;
    stcol(x, o, xc);
    stcol(r, o, rc);
    {
      T* zw = static_cast<T*>(a.zf) + int64_t(h.s) * 384 + h.fidx;
      zw[0] = rc.v[0];
      zw[64] = rc.v[7];
    }
    // next half leaf's own column
    if (hw + hstride < nhw) {
      const HalfLeaf hn = half_pos(hw + hstride, lane);
      const int64_t on = int64_t(hn.s) * 512 + hn.c;
      f = ldflags(a.flags, on);
      ldcol(p, on, P);
      ldcol(x, on, xc);
      ldcol(r, on, rc);
    }
  }
  PartT<DM> v[2] = {drr.pvalue(), drz.pvalue()};
  put_partials<DM, 2>(a, 0, v);
}

// ---- register-pipelined variants --------------------------------------------
// The same two kernels with every input of the next half leaf (own column,
// halo column, z faces) loaded into registers while the current half leaf
// computes: each warp keeps one half leaf of loads in flight, at the price of
// about 40 more registers (4 CTAs per SM instead of 6).
template <typename T>
struct SpmvIn {
  uint2 f, hf;
  Col<T> rc, pc, hr, hp;
  uint8_t zf0, zf1;
  T zr0, zr1, zq0, zq1;
};

// The own column (independent of the neighbour table) ...
template <typename T>
__device__ __forceinline__ void spmv_load_own(const PcgArgs& a, int hw, int lane, const T* r,
                                              const T* pold, SpmvIn<T>& in) {
  const HalfLeaf h = half_pos(hw, lane);
  const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
  in.f = ldflags(a.flags, o);
  ldcol(r, o, in.rc);
  ldcol(pold, o, in.pc);
}

// ... and the halo column and z faces, addressed through the face slots.
// ZD: z-face neighbours read from the vectors (large systems) instead of the
// published planes.
//
// A missing neighbour (no leaf, or a leaf without PCG
// unknowns) reads slot n_pleaf instead, which the setup zeroes (flags, r,
// both p and their z-face planes) and no kernel writes during the solve, so
// the loads need no validity branch.  The particle-leaf capacity keeps that
// slot.
__device__ __forceinline__ unsigned slot_or_null(int slot, int n_pleaf) {
  return unsigned(slot >= 0 && slot < n_pleaf ? slot : n_pleaf);
}
template <typename T, bool ZD>
__device__ __forceinline__ void spmv_load_halo(const PcgArgs& a, int hw, int lane, const int fs[6],
                                               const T* r, const T* pold, int qold,
                                               SpmvIn<T>& in) {
  const HalfLeaf h = half_pos(hw, lane);
  int hslot, hvox;
  halo_col(h, fs, hslot, hvox);
  static_assert(std::is_same<T, float>::value, "the pipelined kernels take fp32 vectors");
  const unsigned hb = slot_or_null(hslot, a.n_pleaf) * 512u + unsigned(hvox);
  in.hf = ldflags(a.flags, hb);
  ldcol(r, hb, in.hr);
  ldcol(pold, hb, in.hp);
  const unsigned z0 = slot_or_null(fs[4], a.n_pleaf), z1 = slot_or_null(fs[5], a.n_pleaf);
  if constexpr (ZD) {
    const unsigned c0 = z0 * 512u + unsigned(h.c) + 7u, c1 = z1 * 512u + unsigned(h.c);
    in.zf0 = ldv(a.flags + c0);
    in.zf1 = ldv(a.flags + c1);
    in.zr0 = ldv(r + c0);
    in.zr1 = ldv(r + c1);
    in.zq0 = ldv(pold + c0);
    in.zq1 = ldv(pold + c1);
  } else {
    const T* zf = static_cast<const T*>(a.zf);
    const unsigned zo0 = z0 * 384u + 64u + unsigned(h.fidx), zo1 = z1 * 384u + unsigned(h.fidx);
    in.zf0 = ldv(a.zff + (z0 * 128u + 64u + unsigned(h.fidx)));
    in.zf1 = ldv(a.zff + (z1 * 128u + unsigned(h.fidx)));
    in.zr0 = ldv(zf + zo0);
    in.zr1 = ldv(zf + zo1);
    in.zq0 = ldv(zf + zo0 + 128 * qold);
    in.zq1 = ldv(zf + zo1 + 128 * qold);
  }
}

template <typename T, bool ZD>
__device__ __forceinline__ void spmv_load(const PcgArgs& a, int hw, int lane, const int fs[6],
                                          const T* r, const T* pold, int qold, SpmvIn<T>& in) {
  spmv_load_own<T>(a, hw, lane, r, pold, in);
  spmv_load_halo<T, ZD>(a, hw, lane, fs, r, pold, qold, in);
}

template <typename T, int DM, bool ZD>
__global__ void __launch_bounds__(kHotThreads, 4) k_pcg_spmv_pl(const __grid_constant__ PcgArgs a) {
  __shared__ Tile<T> tiles[kHotThreads / 32];
  __shared__ DiagInv<T> tab[16];
  __shared__ HeadStage<2, PartT<DM>> hs;
  const int par = a.par;
  const T* r = static_cast<const T*>(a.r);
  const T* pold = static_cast<const T*>(par ? a.p0 : a.p1);
  T* pnew = static_cast<T*>(par ? a.p1 : a.p0);
  const int qold = 1 + (par ^ 1), qnew = 1 + par;
  const int lane = threadIdx.x & 31;
  const int wpb = kHotThreads / 32;
  const int nhw = 2 * a.n_pleaf, hstride = gridDim.x * wpb;
  int hw = blockIdx.x * wpb + (threadIdx.x >> 5);
  fill_diag_table<T>(tab);
  SpmvIn<T> cur;
  int nbl = -1;
  int fs[6];
  // before the wait: the neighbour table, flags and p_{j-1} (written by the
  // spmv two launches back) of the first half leaf
  if (hw < nhw) {
    const int nb0 = face_slot_lane(a.nbr, hw >> 1, lane);
    const HalfLeaf h = half_pos(hw, lane);
    const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
    cur.f = ldflags(a.flags, o);
    ldcol(pold, o, cur.pc);
    nbl = hw + hstride < nhw ? face_slot_lane(a.nbr, (hw + hstride) >> 1, lane) : -1;
    face_slots(nb0, fs);
  }
  pdl_wait();
  pdl_trigger();
  if (hw < nhw) {
    const HalfLeaf h = half_pos(hw, lane);
    ldcol(r, unsigned(h.s) * 512u + unsigned(h.c), cur.rc);
    spmv_load_halo<T, ZD>(a, hw, lane, fs, r, pold, qold, cur);
  }
  head_issue<DM, 2>(hs, a, 0);
  const HotHead head = spmv_head<DM>(hs, a);
  if (head.done) return;
  const T beta = T(head.s);
  Tile<T>& tile = tiles[threadIdx.x >> 5];
  Dot<DM> dp;
  while (hw < nhw) {
    const int hn = hw + hstride;
    SpmvIn<T> nxt;
    if (hn < nhw) {
      int fs[6];
      face_slots(nbl, fs);
      spmv_load<T, ZD>(a, hn, lane, fs, r, pold, qold, nxt);
      nbl = hn + hstride < nhw ? face_slot_lane(a.nbr, (hn + hstride) >> 1, lane) : -1;
    }
    const HalfLeaf h = half_pos(hw, lane);
    Col<T> P, H;
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      P.v[z] = pnew_of<T>(tab, fbyte(cur.f, z), cur.rc.v[z], cur.pc.v[z], beta);
      H.v[z] = pnew_of<T>(tab, fbyte(cur.hf, z), cur.hr.v[z], cur.hp.v[z], beta);
    }
    const T zm = pnew_of<T>(tab, cur.zf0, cur.zr0, cur.zq0, beta);
    const T zp = pnew_of<T>(tab, cur.zf1, cur.zr1, cur.zq1, beta);
    const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
    stcol(pnew, o, P);
    if constexpr (!ZD) {  // publish the z faces for the neighbours
      T* zw = static_cast<T*>(a.zf) + (unsigned(h.s) * 384u + 128u * unsigned(qnew) + unsigned(h.fidx));
      zw[0] = P.v[0];
      zw[64] = P.v[7];
    }
    __syncwarp();
    st_col_sh(tile, h.lx + 1, h.cy + 1, P);
    if (h.lx != 2) st_col_sh(tile, h.tx, h.ty, H);
    __syncwarp();
    Col<T> ap;
    stencil_col<T>(tile, tab, h.lx, h.cy, P, cur.f, zm, zp, ap);
#pragma unroll
    for (int z = 0; z < 8; ++z) dp.add(P.v[z], ap.v[z]);
    cur = nxt;
    hw = hn;
  }
  PartT<DM> v[1] = {dp.pvalue()};
  put_partials<DM, 1>(a, kPartPAp, v);
}


// ---- bulk-copy (TMA) staged spmv for large systems --------------------------------
// A half leaf's own r, p_{j-1} and flags are 1 KB + 1 KB + 256 B, contiguous.
// Lane 0 of each warp copies them into a ring of kStages shared-memory stages
// with cp.async.bulk (the SM's copy engine: no registers, no load/store-unit
// slots), kStages - 1 half leaves ahead; an mbarrier per stage counts the
// bytes in.  The halo column and the z faces (32 B and 4 B per lane,
// scattered) are loaded into registers one half leaf ahead, as in
// k_pcg_spmv_pl.  The ring keeps twice the register kernel's own-column
// bytes in flight per warp, but it measured slower at every size (spmv per
// launch: 25.4 vs 21.4 us at 256^3, 83 vs 65 us at 512^3, 480 vs 350 us at
// 1024^3): the ring's shared memory leaves the SM little L1 for the halo
// and z-face loads, and the stage adds a shared-memory round trip.  It is
// opt-in (FSIM_PCG_TMA=1) and gives bit-identical solves.
//
// Every wait is bounded (kStagePolls).  A wait that gives up records
// FSIM_ERR_TIMEOUT in PcgScalars::wait_err, issues the stage's withheld copy
// if there is one, and waits again with a long bound, so that no copy is in
// flight into shared memory when the CTA exits.  PcgArgs::withhold (tests
// only) makes CTA 0's first stage hold back its flags copy, and that stage's
// wait gives up after kHeldPolls: the wait runs out without a fault, and the
// solve still completes with the right values.
constexpr int kStages = 4;
constexpr unsigned kStagePolls = 1u << 22;  // bound of a stage wait
constexpr unsigned kHeldPolls = 256;        // the test's withheld stage (it cannot fill)
constexpr unsigned kDrainPolls = 1u << 26;  // second, long bound after a wait gave up

struct SpmvStage {
  float r[256];
  float p[256];
  uint8_t f[256];
};
// the stage ring is dynamic shared memory (above the 48 KB static limit with
// the kernel's static tiles and head stage)
constexpr size_t kTmaDynSmem = size_t(kHotThreads / 32) * kStages * sizeof(SpmvStage);

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
      ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, unsigned parity, unsigned polls) {
  for (unsigned i = 0; i < polls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Lane 0: copy half leaf hw's own columns into stage st (the flags copy held
// back when `hold`).
__device__ __forceinline__ void spmv_stage_issue(const PcgArgs& a, int hw, const float* r,
                                                 const float* pold, SpmvStage& st,
                                                 uint64_t* bar, bool hold) {
  const int64_t o = int64_t(hw >> 1) * 512 + (hw & 1) * 256;
  mbar_expect_tx(bar, 2u * 1024u + 256u);
  bulk_g2s(st.r, r + o, 1024u, bar);
  bulk_g2s(st.p, pold + o, 1024u, bar);
  if (!hold) bulk_g2s(st.f, a.flags + o, 256u, bar);
}

// Lane 0: the bounded wait on stage q (phase parity ph), with the recovery
// above; the warp learns the outcome by a shuffle.
// held: this stage's flags copy was withheld (the test's first stage only).
__device__ __forceinline__ void stage_wait(const PcgArgs& a, int lane, uint64_t* bar,
                                           unsigned ph, bool* held, int hw, SpmvStage& st) {
  const unsigned polls = (held && *held) ? kHeldPolls : kStagePolls;
  if (lane == 0 && !mbar_wait_n(bar, ph, polls)) {
    atomicExch(&a.sc->wait_err, unsigned(FSIM_ERR_TIMEOUT));
    if (held && *held) {  // the test's withheld copy: complete the stage now
      const int64_t o = int64_t(hw >> 1) * 512 + (hw & 1) * 256;
      bulk_g2s(st.f, a.flags + o, 256u, bar);
      *held = false;
    }
    if (!mbar_wait_n(bar, ph, kDrainPolls)) atomicExch(&a.sc->wait_err, unsigned(FSIM_ERR_CUDA));
  }
  __syncwarp();
}

template <int DM, bool ZD>
__global__ void __launch_bounds__(kHotThreads, 4) k_pcg_spmv_tma(const __grid_constant__ PcgArgs a) {
  pdl_wait();  // reads its predecessor's r from the first copy on
  pdl_trigger();
  using T = float;
  __shared__ Tile<T> tiles[kHotThreads / 32];
  __shared__ DiagInv<T> tab[16];
  __shared__ HeadStage<2, PartT<DM>> hs;
  extern __shared__ __align__(128) unsigned char tma_ring[];  // kTmaDynSmem bytes
  __shared__ __align__(8) uint64_t bars[kHotThreads / 32][kStages];
  const int par = a.par;
  const T* r = static_cast<const T*>(a.r);
  const T* pold = static_cast<const T*>(par ? a.p0 : a.p1);
  T* pnew = static_cast<T*>(par ? a.p1 : a.p0);
  const int qold = 1 + (par ^ 1), qnew = 1 + par;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int wpb = kHotThreads / 32;
  const int nhw = 2 * a.n_pleaf, hstride = gridDim.x * wpb;
  const int hw0 = blockIdx.x * wpb + w;
  SpmvStage* stg = reinterpret_cast<SpmvStage*>(tma_ring) + w * kStages;
  uint64_t* bar = bars[w];
  bool held = a.withhold && blockIdx.x == 0 && w == 0 && hw0 < nhw;  // lane 0's copy only
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < kStages; ++q) mbar_init(&bar[q], 1u);
    fence_async_smem();
  }
  __syncwarp();
  if (lane == 0) {
    for (int q = 0; q < kStages - 1; ++q) {
      const int hq = hw0 + q * hstride;
      if (hq < nhw) spmv_stage_issue(a, hq, r, pold, stg[q], &bar[q], held && q == 0);
    }
  }
  head_issue<DM, 2>(hs, a, 0);
  fill_diag_table<T>(tab);
  SpmvIn<T> cur;  // halo and z faces only (rc, pc, f come from the stage)
  int nbl = -1;
  if (hw0 < nhw) {
    int fs[6];
    face_slots(face_slot_lane(a.nbr, hw0 >> 1, lane), fs);
    nbl = hw0 + hstride < nhw ? face_slot_lane(a.nbr, (hw0 + hstride) >> 1, lane) : -1;
    spmv_load_halo<T, ZD>(a, hw0, lane, fs, r, pold, qold, cur);
  }
  const HotHead head = spmv_head<DM>(hs, a);
  if (head.done) {
    // no work: drain the copies already issued before leaving
    for (int q = 0; q < kStages - 1; ++q)
      if (hw0 + q * hstride < nhw)
        stage_wait(a, lane, &bar[q], 0u, q == 0 ? &held : nullptr, hw0 + q * hstride, stg[q]);
    return;
  }
  const T beta = T(head.s);
  Tile<T>& tile = tiles[w];
  Dot<DM> dp;
  int k = 0;
  for (int hw = hw0; hw < nhw; hw += hstride, ++k) {
    // keep kStages - 1 half leaves in flight: refill the stage read last time
    {
      const int hq = hw + (kStages - 1) * hstride;
      const int q = (k + kStages - 1) % kStages;
      if (lane == 0 && hq < nhw) spmv_stage_issue(a, hq, r, pold, stg[q], &bar[q], false);
    }
    const int hn = hw + hstride;
    SpmvIn<T> nxt;
    if (hn < nhw) {
      int fs[6];
      face_slots(nbl, fs);
      spmv_load_halo<T, ZD>(a, hn, lane, fs, r, pold, qold, nxt);
      nbl = hn + hstride < nhw ? face_slot_lane(a.nbr, (hn + hstride) >> 1, lane) : -1;
    }
    const int q = k % kStages;
    stage_wait(a, lane, &bar[q], unsigned((k / kStages) & 1), k == 0 ? &held : nullptr, hw,
               stg[q]);
    const HalfLeaf h = half_pos(hw, lane);
    {
      const float4 a0 = reinterpret_cast<const float4*>(stg[q].r)[2 * lane];
      const float4 a1 = reinterpret_cast<const float4*>(stg[q].r)[2 * lane + 1];
      const float4 b0 = reinterpret_cast<const float4*>(stg[q].p)[2 * lane];
      const float4 b1 = reinterpret_cast<const float4*>(stg[q].p)[2 * lane + 1];
      cur.f = reinterpret_cast<const uint2*>(stg[q].f)[lane];
      cur.rc.v[0] = a0.x; cur.rc.v[1] = a0.y; cur.rc.v[2] = a0.z; cur.rc.v[3] = a0.w;
      cur.rc.v[4] = a1.x; cur.rc.v[5] = a1.y; cur.rc.v[6] = a1.z; cur.rc.v[7] = a1.w;
      cur.pc.v[0] = b0.x; cur.pc.v[1] = b0.y; cur.pc.v[2] = b0.z; cur.pc.v[3] = b0.w;
      cur.pc.v[4] = b1.x; cur.pc.v[5] = b1.y; cur.pc.v[6] = b1.z; cur.pc.v[7] = b1.w;
    }
    __syncwarp();
    if (lane == 0) fence_async_smem();  // this stage's reads before its next bulk write
    Col<T> P, H;
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      P.v[z] = pnew_of<T>(tab, fbyte(cur.f, z), cur.rc.v[z], cur.pc.v[z], beta);
      H.v[z] = pnew_of<T>(tab, fbyte(cur.hf, z), cur.hr.v[z], cur.hp.v[z], beta);
    }
    const T zm = pnew_of<T>(tab, cur.zf0, cur.zr0, cur.zq0, beta);
    const T zp = pnew_of<T>(tab, cur.zf1, cur.zr1, cur.zq1, beta);
    const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
    stcol(pnew, o, P);
    if constexpr (!ZD) {  // publish the z faces for the neighbours
      T* zw = static_cast<T*>(a.zf) + (unsigned(h.s) * 384u + 128u * unsigned(qnew) + unsigned(h.fidx));
      zw[0] = P.v[0];
      zw[64] = P.v[7];
    }
    __syncwarp();
    st_col_sh(tile, h.lx + 1, h.cy + 1, P);
    if (h.lx != 2) st_col_sh(tile, h.tx, h.ty, H);
    __syncwarp();
    Col<T> ap;
    stencil_col<T>(tile, tab, h.lx, h.cy, P, cur.f, zm, zp, ap);
#pragma unroll
    for (int z = 0; z < 8; ++z) dp.add(P.v[z], ap.v[z]);
    cur.hf = nxt.hf;
    cur.hr = nxt.hr;
    cur.hp = nxt.hp;
    cur.zf0 = nxt.zf0; cur.zf1 = nxt.zf1;
    cur.zr0 = nxt.zr0; cur.zr1 = nxt.zr1;
    cur.zq0 = nxt.zq0; cur.zq1 = nxt.zq1;
  }
  PartT<DM> v[1] = {dp.pvalue()};
  put_partials<DM, 1>(a, kPartPAp, v);
}

template <typename T>
struct UpdIn {
  uint2 f;
  Col<T> P, x, r, H;
  T zm, zp;
};

template <typename T>
__device__ __forceinline__ void upd_load_own(const PcgArgs& a, int hw, int lane, const T* p,
                                             const T* x, const T* r, UpdIn<T>& in) {
  const HalfLeaf h = half_pos(hw, lane);
  const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
  in.f = ldflags(a.flags, o);
  ldcol(p, o, in.P);
  ldcol(x, o, in.x);
  ldcol(r, o, in.r);
}

template <typename T, bool ZD>
__device__ __forceinline__ void upd_load_halo(const PcgArgs& a, int hw, int lane, const int fs[6],
                                              const T* p, int qcur, UpdIn<T>& in) {
  const HalfLeaf h = half_pos(hw, lane);
  int hslot, hvox;
  halo_col(h, fs, hslot, hvox);
  static_assert(std::is_same<T, float>::value, "the pipelined kernels take fp32 vectors");
  ldcol(p, slot_or_null(hslot, a.n_pleaf) * 512u + unsigned(hvox), in.H);
  const unsigned z0 = slot_or_null(fs[4], a.n_pleaf), z1 = slot_or_null(fs[5], a.n_pleaf);
  if constexpr (ZD) {
    in.zm = ldv(p + (z0 * 512u + unsigned(h.c) + 7u));
    in.zp = ldv(p + (z1 * 512u + unsigned(h.c)));
  } else {
    const T* zfp = static_cast<const T*>(a.zf) + (128u * unsigned(qcur) + unsigned(h.fidx));
    in.zm = ldv(zfp + (z0 * 384u + 64u));
    in.zp = ldv(zfp + z1 * 384u);
  }
}

template <typename T, bool ZD>
__device__ __forceinline__ void upd_load(const PcgArgs& a, int hw, int lane, const int fs[6],
                                         const T* p, const T* x, const T* r, int qcur,
                                         UpdIn<T>& in) {
  upd_load_own<T>(a, hw, lane, p, x, r, in);
  upd_load_halo<T, ZD>(a, hw, lane, fs, p, qcur, in);
}

template <typename T, int DM, bool ZD>
__global__ void __launch_bounds__(kHotThreads, 4)
    k_pcg_update_pl(const __grid_constant__ PcgArgs a) {
  __shared__ Tile<T> tiles[kHotThreads / 32];
  __shared__ DiagInv<T> tab[16];
  __shared__ HeadStage<1, PartT<DM>> hs;
  const int par = a.par;
  const T* p = static_cast<const T*>(par ? a.p1 : a.p0);
  T* x = static_cast<T*>(a.x);
  T* r = static_cast<T*>(a.r);
  const int qcur = 1 + par;
  const int lane = threadIdx.x & 31;
  const int wpb = kHotThreads / 32;
  const int nhw = 2 * a.n_pleaf, hstride = gridDim.x * wpb;
  int hw = blockIdx.x * wpb + (threadIdx.x >> 5);
  fill_diag_table<T>(tab);
  UpdIn<T> cur;
  int nbl = -1;
  int fs[6];
  // before the wait: the neighbour table, flags, x and r (written by the
  // update two launches back) of the first half leaf
  if (hw < nhw) {
    const int nb0 = face_slot_lane(a.nbr, hw >> 1, lane);
    const HalfLeaf h = half_pos(hw, lane);
    const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
    cur.f = ldflags(a.flags, o);
    ldcol(x, o, cur.x);
    ldcol(r, o, cur.r);
    nbl = hw + hstride < nhw ? face_slot_lane(a.nbr, (hw + hstride) >> 1, lane) : -1;
    face_slots(nb0, fs);
  }
  pdl_wait();
  pdl_trigger();
  if (hw < nhw) {
    const HalfLeaf h = half_pos(hw, lane);
    ldcol(p, unsigned(h.s) * 512u + unsigned(h.c), cur.P);
    upd_load_halo<T, ZD>(a, hw, lane, fs, p, qcur, cur);
  }
  head_issue<DM, 1>(hs, a, kPartPAp);
  const HotHead head = update_head<DM>(hs, a);
  if (head.done) return;
  const T alpha = T(head.s);
  const T nalpha = -alpha;
  Tile<T>& tile = tiles[threadIdx.x >> 5];
  Dot<DM> drr, drz;
  while (hw < nhw) {
    const int hn = hw + hstride;
    UpdIn<T> nxt;
    if (hn < nhw) {
      int fs[6];
      face_slots(nbl, fs);
      upd_load<T, ZD>(a, hn, lane, fs, p, x, r, qcur, nxt);
      nbl = hn + hstride < nhw ? face_slot_lane(a.nbr, (hn + hstride) >> 1, lane) : -1;
    }
    const HalfLeaf h = half_pos(hw, lane);
    __syncwarp();
    st_col_sh(tile, h.lx + 1, h.cy + 1, cur.P);
    if (h.lx != 2) st_col_sh(tile, h.tx, h.ty, cur.H);
    __syncwarp();
    Col<T> ap;
    stencil_col<T>(tile, tab, h.lx, h.cy, cur.P, cur.f, cur.zm, cur.zp, ap);
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      const uint8_t g = fbyte(cur.f, z);
      cur.x.v[z] = tadd(tmul(alpha, cur.P.v[z]), cur.x.v[z]);
      cur.r.v[z] = tadd(tmul(nalpha, ap.v[z]), cur.r.v[z]);
      drr.add(cur.r.v[z], cur.r.v[z]);
      drz.add(cur.r.v[z], tmul(tab[g & 15].inv, cur.r.v[z]));
    }
    const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
    stcol(x, o, cur.x);
    stcol(r, o, cur.r);
    if constexpr (!ZD) {
      T* zw = static_cast<T*>(a.zf) + (unsigned(h.s) * 384u + unsigned(h.fidx));
      zw[0] = cur.r.v[0];
      zw[64] = cur.r.v[7];
    }
    cur = nxt;
    hw = hn;
  }
  PartT<DM> v[2] = {drr.pvalue(), drz.pvalue()};
  put_partials<DM, 2>(a, 0, v);
}

// ---- single-reduction CG (Chronopoulos-Gear) ----------------------------------
// Opt-in for fp32 solves (FSIM_PCG_CG1=1; use_cg1 below): one kernel per
// iteration instead of the spmv / update pair, so one grid-wide dependency
// per iteration instead of two.  With u = M r (recomputed, never stored), w = A u and
// s = A p kept as vectors, the iteration takes both of its scalars from one
// reduction, gamma_i = r_i.u_i and delta_i = w_i.u_i:
//   beta_i  = gamma_i / gamma_{i-1}                 (0 at i = 0)
//   alpha_i = gamma_i / (delta_i - beta_i gamma_i / alpha_{i-1})   (= r.z / p.Ap)
//   p_i = u_i + beta_i p_{i-1};   s_i = w_i + beta_i s_{i-1}
//   x += alpha_i p_i;   r_{i+1} = r_i - alpha_i s_i;   w_{i+1} = A M r_{i+1}
// and the partials of gamma_{i+1}, delta_{i+1} and r_{i+1}.r_{i+1} (the loop
// test of PCGDriver::Solve, common/solver_driver.cc:14-69, at the head of
// the next launch).  In exact arithmetic these are the iterates of
// common/solver.cc:297-366; the rounding differs (p.Ap is not formed
// directly), so solves agree with the reference's to the solver tolerance,
// not bitwise.
//
// w_{i+1} needs M r_{i+1} on the half leaf's halo: each lane recomputes
// r_{i+1} there from r_i, w_i, s_{i-1} with the owner's operations (so the
// owner's bits), which is why r, w and s alternate between two buffers by
// launch parity, while x and p, read only at their own cells, are updated in
// place.  The first launch of a solve (after setup) computes w_0 = A M r_0
// with alpha = beta = 0 and w, s, p, x taken as 0.  s drifts from A p in
// fp32 along its recurrence; k_pcg_cg1_s re-forms it once per pass.
// Per unknown and iteration it reads flags, x, p, r, w, s and writes x, p, r,
// w, s: 41 B, against the pair's 34 B.
constexpr int kPartCg1 = 0;  // part[] rows: gamma, delta, r.r of launch parity 0, then of parity 1

struct Cg1Head {
  int done, init;
  double alpha, beta;
};

// Head of a single-reduction launch: the predecessor's gamma, delta and r.r,
// the loop test, then alpha and beta with the CHECK_LE(., LARGE_FLOAT) tests
// of ComputeLocal2 / ComputeLocal3.  Launch parity par reads st[par ^ 1] and
// CTA 0 writes st[par].
template <int DM>
__device__ __forceinline__ Cg1Head cg1_head(HeadStage<3, PartT<DM>>& hs, Cg1Head& out,
                                            const PcgArgs& a) {
  double acc[3];
  head_sum<DM, 3>(hs, acc);
  if (threadIdx.x == 0) {
    const PcgScalars* cs = &hs.sc;
    const int par = a.par;
    const PcgIterState in = cs->st[par ^ 1];
    Cg1Head o;
    o.done = in.done;
    o.init = 0;
    o.alpha = 0.0;
    o.beta = 0.0;
    int status = in.status;
    double rr = 0.0, gamma = 0.0, delta = 0.0;
    if (!in.done && in.given) {
      o.init = 1;  // after setup: this launch forms w_0
    } else if (!in.done) {
      gamma = round_t(cs, acc[0]);
      delta = round_t(cs, acc[1]);
      rr = round_t(cs, acc[2]);
      const int i = in.iter;
      if (i >= cs->max_iter || converged(cs, rr)) {
        o.done = 1;
      } else {
        double alpha, beta = 0.0;
        if (cs->fp32) {
          const float g = float(gamma);
          float den = float(delta);
          if (i > 0) {
            const float b = __fdiv_rn(g, float(in.rz_prev));
            den = __fsub_rn(den, __fdiv_rn(__fmul_rn(b, g), float(in.alpha)));
            beta = double(b);
          }
          alpha = double(__fdiv_rn(g, den));
        } else {
          double den = delta;
          if (i > 0) {
            beta = gamma / in.rz_prev;
            den -= beta * gamma / in.alpha;
          }
          alpha = gamma / den;
        }
        if (!(beta <= 1e5) || !(alpha <= 1e5)) {
          status = FSIM_ERR_BREAKDOWN;
          o.done = 1;
        }
        o.alpha = alpha;
        o.beta = beta;
      }
    }
    if (blockIdx.x == 0) {
      PcgScalars* sc = a.sc;
      PcgIterState n = in;
      if (!in.done) {
        if (o.init) {
          n.given = 0;
          n.iter = 0;
          n.rz_prev = 0.0;
          n.alpha = 0.0;
        } else {
          sc->rr = rr;
          sc->rz = gamma;
          sc->pAp = delta;
          sc->iter = in.iter;
          sc->status = status;
          if (o.done) {
            n.done = 1;
            n.status = status;
            sc->done = 1;
          } else {
            n.rz_prev = gamma;
            n.alpha = o.alpha;
            n.iter = in.iter + 1;
            sc->rz_old = in.rz_prev;
            sc->alpha = o.alpha;
            sc->beta = o.beta;
          }
        }
      }
      sc->st[par] = n;
      if (o.done && a.cond) cudaGraphSetConditional(a.cond, 0u);
    }
    out = o;
  }
  __syncthreads();
  return out;
}

// r_{i+1} of a cell from its r_i, w_i and s_{i-1}: the owner's operations
// (s_i = w_i + beta s_{i-1}, then r_i - alpha s_i), for the halo.
template <typename T>
__device__ __forceinline__ T cg1_rnext(T r, T w, T s, T nalpha, T beta) {
  return tadd(tmul(nalpha, tadd(w, tmul(beta, s))), r);
}

template <typename T, int DM>
__global__ void __launch_bounds__(kHotThreads, 4) k_pcg_cg1(const __grid_constant__ PcgArgs a) {
  __shared__ Tile<T> tiles[kHotThreads / 32];
  __shared__ DiagInv<T> tab[16];
  __shared__ HeadStage<3, PartT<DM>> hs;
  __shared__ Cg1Head hout;
  const int par = a.par;
  const T* ra = static_cast<const T*>(par ? a.p1 : a.r);
  T* rb = static_cast<T*>(par ? a.r : a.p1);
  const T* wa = static_cast<const T*>(a.w[par]);
  T* wb = static_cast<T*>(a.w[par ^ 1]);
  const T* sa = static_cast<const T*>(a.sv[par]);
  T* sb = static_cast<T*>(a.sv[par ^ 1]);
  T* x = static_cast<T*>(a.x);
  T* p = static_cast<T*>(a.p0);
  const int lane = threadIdx.x & 31;
  const int wpb = kHotThreads / 32;
  const int nhw = 2 * a.n_pleaf, hstride = gridDim.x * wpb;
  int hw = blockIdx.x * wpb + (threadIdx.x >> 5);
  fill_diag_table<T>(tab);
  // before the wait: the neighbour table (fixed during the solve)
  int nbl = hw < nhw ? face_slot_lane(a.nbr, hw >> 1, lane) : -1;
  pdl_wait();
  pdl_trigger();
  head_issue<DM, 3>(hs, a, kPartCg1 + 3 * (par ^ 1));
  const Cg1Head head = cg1_head<DM>(hs, hout, a);
  if (head.done) return;
  const bool init = head.init != 0;
  const T alpha = T(head.alpha), nalpha = -alpha, beta = T(head.beta);
  Tile<T>& tile = tiles[threadIdx.x >> 5];
  Dot<DM> dg, dd, drr;
  for (; hw < nhw; hw += hstride) {
    const int nbl_next =
        hw + hstride < nhw ? face_slot_lane(a.nbr, (hw + hstride) >> 1, lane) : -1;
    int fs[6];
    face_slots(nbl, fs);
    nbl = nbl_next;
    const HalfLeaf h = half_pos(hw, lane);
    const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
    // own column
    const uint2 f = ldflags(a.flags, o);
    Col<T> R, W, S, P, X;
    ldcol(ra, o, R);
    ldcol(wa, o, W);
    ldcol(sa, o, S);
    ldcol(p, o, P);
    ldcol(x, o, X);
    // halo column (the zeroed null slot when there is none)
    int hslot, hvox;
    halo_col(h, fs, hslot, hvox);
    const unsigned hb = slot_or_null(hslot, a.n_pleaf) * 512u + unsigned(hvox);
    const uint2 hf = ldflags(a.flags, hb);
    Col<T> HR, HW, HS;
    ldcol(ra, hb, HR);
    ldcol(wa, hb, HW);
    ldcol(sa, hb, HS);
    // z faces: the -z leaf's z = 7 cell and the +z leaf's z = 0 cell, read
    // from the vectors (published z-face planes of r, w and s measured slower)
    const unsigned z0 = slot_or_null(fs[4], a.n_pleaf) * 512u + unsigned(h.c) + 7u;
    const unsigned z1 = slot_or_null(fs[5], a.n_pleaf) * 512u + unsigned(h.c);
    const uint8_t zg0 = ldv(a.flags + z0), zg1 = ldv(a.flags + z1);
    const T zr0 = ldv(ra + z0), zr1 = ldv(ra + z1);
    T zw0 = ldv(wa + z0), zw1 = ldv(wa + z1), zs0 = ldv(sa + z0), zs1 = ldv(sa + z1);
    if (init) {
#pragma unroll
      for (int z = 0; z < 8; ++z) W.v[z] = S.v[z] = P.v[z] = X.v[z] = HW.v[z] = HS.v[z] = T(0);
      zw0 = zw1 = zs0 = zs1 = T(0);
    }
    Col<T> U, HU;
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      const T inv = tab[fbyte(f, z) & 15].inv;
      P.v[z] = tadd(tmul(inv, R.v[z]), tmul(beta, P.v[z]));
      S.v[z] = tadd(W.v[z], tmul(beta, S.v[z]));
      X.v[z] = tadd(tmul(alpha, P.v[z]), X.v[z]);
      R.v[z] = tadd(tmul(nalpha, S.v[z]), R.v[z]);
      U.v[z] = tmul(inv, R.v[z]);
      HU.v[z] = tmul(tab[fbyte(hf, z) & 15].inv, cg1_rnext(HR.v[z], HW.v[z], HS.v[z], nalpha, beta));
    }
    const T zm = tmul(tab[zg0 & 15].inv, cg1_rnext(zr0, zw0, zs0, nalpha, beta));
    const T zp = tmul(tab[zg1 & 15].inv, cg1_rnext(zr1, zw1, zs1, nalpha, beta));
    __syncwarp();  // previous half leaf's tile reads are done
    st_col_sh(tile, h.lx + 1, h.cy + 1, U);
    if (h.lx != 2) st_col_sh(tile, h.tx, h.ty, HU);
    __syncwarp();
    Col<T> WN;
    stencil_col<T>(tile, tab, h.lx, h.cy, U, f, zm, zp, WN);
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      dg.add(R.v[z], U.v[z]);
      dd.add(WN.v[z], U.v[z]);
      drr.add(R.v[z], R.v[z]);
    }
    stcol(p, o, P);
    stcol(x, o, X);
    stcol(sb, o, S);
    stcol(rb, o, R);
    stcol(wb, o, WN);
  }
  PartT<DM> v[3] = {dg.pvalue(), dd.pvalue(), drr.pvalue()};
  put_partials<DM, 3>(a, kPartCg1 + 3 * par, v);
}

// s = A p formed directly from p (in place, so the latest p_i), into the s
// buffer that the next single-reduction launch reads (parity a.par): run
// once per graph pass (and per host-polled chunk), it resets the drift that
// the recurrence s_i = w_i + beta_i s_{i-1} accumulates in fp32.  A p is
// summed in the reference's column order, as in the pair.
template <typename T>
__global__ void __launch_bounds__(kHotThreads, 4) k_pcg_cg1_s(const __grid_constant__ PcgArgs a) {
  __shared__ Tile<T> tiles[kHotThreads / 32];
  __shared__ DiagInv<T> tab[16];
  const T* p = static_cast<const T*>(a.p0);
  T* sb = static_cast<T*>(a.sv[a.par]);
  const int lane = threadIdx.x & 31;
  const int wpb = kHotThreads / 32;
  const int nhw = 2 * a.n_pleaf, hstride = gridDim.x * wpb;
  int hw = blockIdx.x * wpb + (threadIdx.x >> 5);
  fill_diag_table<T>(tab);
  int nbl = hw < nhw ? face_slot_lane(a.nbr, hw >> 1, lane) : -1;
  pdl_wait();
  pdl_trigger();
  __syncthreads();  // the diagonal table
  Tile<T>& tile = tiles[threadIdx.x >> 5];
  for (; hw < nhw; hw += hstride) {
    const int nbl_next =
        hw + hstride < nhw ? face_slot_lane(a.nbr, (hw + hstride) >> 1, lane) : -1;
    int fs[6];
    face_slots(nbl, fs);
    nbl = nbl_next;
    const HalfLeaf h = half_pos(hw, lane);
    const unsigned o = unsigned(h.s) * 512u + unsigned(h.c);
    const uint2 f = ldflags(a.flags, o);
    Col<T> P, H;
    ldcol(p, o, P);
    int hslot, hvox;
    halo_col(h, fs, hslot, hvox);
    ldcol(p, slot_or_null(hslot, a.n_pleaf) * 512u + unsigned(hvox), H);
    const T zm = ldv(p + (slot_or_null(fs[4], a.n_pleaf) * 512u + unsigned(h.c) + 7u));
    const T zp = ldv(p + (slot_or_null(fs[5], a.n_pleaf) * 512u + unsigned(h.c)));
    __syncwarp();
    st_col_sh(tile, h.lx + 1, h.cy + 1, P);
    if (h.lx != 2) st_col_sh(tile, h.tx, h.ty, H);
    __syncwarp();
    Col<T> ap;
    stencil_col<T>(tile, tab, h.lx, h.cy, P, f, zm, zp, ap);
    stcol(sb, o, ap);
  }
}

// ---- on-chip resident loop: one persistent CTA per SM ---------------------------
// fp32 solves whose particle leaves fit on chip (by default 2 to kResLeaves
// particle leaves per SM; FSIM_PCG_RES=1 / 0 forces it on / off): one
// cooperative launch runs every iteration.  CTA c owns the contiguous slots
// [c * per, c * per + nl), per = ceil(n_pleaf / G) <= kResLeaves, and keeps
// every vector of the iteration on chip: p and the flags in shared memory,
// r and A p in tensor memory, x in tensor and shared memory (each warp owns
// up to kResHL half leaves, a lane one z-column of each).  Per iteration,
// as the reference's ComputeLocal1-3 (common/solver.cc:297-366):
//   S: p = z + beta p on the own columns (into shared memory, and the
//      columns other CTAs read into a global mirror), then A p (kept) and
//      the p.Ap partials;
//   grid barrier: every CTA sums the G partials in CTA order -> alpha;
//   U: x += alpha p, r -= alpha A p, z = M r (of the columns other CTAs read
//      also into a global mirror), the r.r and r.z partials;
//   grid barrier -> r.r, r.z, beta and the loop test.
// (One more grid barrier before the first iteration publishes the first z.)
// Stencil neighbours in the CTA's own leaves come from shared memory; those
// in other CTAs' leaves are formed as z + beta p from the mirrors of z and
// the previous p, read through L2 (the owner's operations, so the owner's
// bits; p alternates between two mirror buffers by iteration parity), by all
// 32 lanes of the warp together and handed out by warp shuffles.  A p is summed in the
// reference's column order.  The dot products are summed per thread, per
// CTA and over CTAs in fixed orders: the solve is deterministic (its
// per-thread order differs from the pair's, so the bits do too).  Thread 0
// alone runs the scalar steps (alpha, beta, the loop test) in fp64.  x and r
// are written back whole at the end.  Barrier waits are bounded (kResPolls);
// a CTA that gives up sets bar_err and every CTA leaves the loop
// (FSIM_ERR_TIMEOUT), freeing its tensor memory.
constexpr int kResWarps = 28;
constexpr int kResThreads = kResWarps * 32;
constexpr int kResHL = 4;                             // half leaves per warp
constexpr int kResLeaves = kResWarps * kResHL / 2;    // leaves per CTA
// dynamic shared memory: p and the flags of the CTA's leaves, and x of every
// warp's half leaves 1 .. kResHL - 1 (half leaf 0's x is in tensor memory)
constexpr size_t kResSmemX = size_t(kResHL - 1) * kResWarps * 256 * sizeof(float);
constexpr size_t kResSmem = size_t(kResLeaves) * 512 * (sizeof(float) + 1) + kResSmemX;
constexpr unsigned kResPolls = 1u << 22;  // about 2-4 s of L2 round trips

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier of round `round` with the CTA's NV partials: publish, arrive
// (a GPU-scope release add on one counter, after the CTA barrier that orders
// the CTA's mirror stores first), wait with acquire loads until all G CTAs
// of the round have arrived, then sum the G partials in CTA order (every CTA
// the same totals), and thread 0 runs fin(totals) before the closing CTA
// barrier.  Rows row0.. of the float partials; each phase type has
// its own rows, which a CTA can only rewrite after every CTA has passed the
// next barrier, and so has read them.  Waits are bounded: a CTA that gives
// up sets bar_err, which the others also poll.  With PcgArgs::res_withhold
// (tests) CTA 0 does not arrive at the first barrier and the limit is 256
// polls, so every CTA's wait gives up.  (Publishing each partial
// beside the round number in one 64-bit word, polled by every CTA, measured
// slower: 33.2 against 30.1 us per iteration at 256^3, and again with
// relaxed words and no fence on the p.Ap barrier, 21.8 against 16.8: the
// polling of 152 slots by every CTA costs more than the counter's second
// round trip.)
template <int NV, typename F>
__device__ __forceinline__ bool res_sync(const PcgArgs& a, float (&v)[NV], int row0,
                                         unsigned round, int* s_ok, F&& fin) {
  block_sum_p<float, NV, kResThreads>(v);  // its CTA barrier orders the CTA's stores first
  if (threadIdx.x < 32) {
    // warp 0: lane 0 publishes, arrives and waits; the warp then sums
    const int lane = threadIdx.x, G = int(gridDim.x);
    int ok = 1;
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) a.partf[(row0 + k) * a.maxb + blockIdx.x] = v[k];
      if (!(a.res_withhold && blockIdx.x == 0 && round == 1))
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;\n" ::"l"(&a.sc->bar_count) : "memory");
      const unsigned target = round * gridDim.x;
      const unsigned limit = a.res_withhold ? 256u : kResPolls;
      unsigned polls = 0;
      while (ld_acquire_gpu(&a.sc->bar_count) < target) {
        if ((++polls & 255u) == 0u &&
            (polls > limit || ld_acquire_gpu(&a.sc->bar_err) != 0u)) {
          ok = 0;
          break;
        }
      }
      if (!ok) atomicExch(&a.sc->bar_err, 1u);
      *s_ok = ok;
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    __syncwarp();  // orders lane 0's acquire before the other lanes' loads
    if (ok) {
      // lane adds partials lane, lane + 32, ... in that order; each batch's
      // loads are all issued before its adds (a zero pad adds exactly nothing)
      float x[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) x[k] = 0.f;
      for (int i0 = lane; i0 < G; i0 += 32 * 8) {
        float t[NV][8];
#pragma unroll
        for (int k = 0; k < NV; ++k)
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int i = i0 + 32 * u;
            t[k][u] = i < G ? __ldcg(a.partf + (row0 + k) * a.maxb + i) : 0.f;
          }
#pragma unroll
        for (int k = 0; k < NV; ++k)
#pragma unroll
          for (int u = 0; u < 8; ++u) x[k] = __fadd_rn(x[k], t[k][u]);
      }
      double tot[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x[k] = __fadd_rn(x[k], __shfl_down_sync(0xffffffffu, x[k], o));
        tot[k] = double(x[k]);
      }
      if (lane == 0) fin(tot);
    }
  }
  __syncthreads();
  return *s_ok != 0;
}

// Shared p of the CTA's leaves in 16-byte chunk planes: float4 element
// ((leaf * 2 + chunk) * 8 + x) * 8 + y holds the cells z = 4 chunk ..
// 4 chunk + 3 of column (x, y), so the lanes of a quarter warp (consecutive
// y) touch consecutive 16-byte words.  ps_col4 is the float4 index of chunk 0
// of a column; chunk 1 is 64 further, and the in-leaf neighbour columns are
// -8 / +8 (x) and -1 / +1 (y) away, constant offsets from the own column.
__device__ __forceinline__ int ps_col4(int leaf, int x, int y) { return (leaf * 16 + x) * 8 + y; }
__device__ __forceinline__ void ps_ld4(const float* ps, int i, Col<float>& c) {
  const float4* q = reinterpret_cast<const float4*>(ps);
  const float4 u = q[i], w = q[i + 64];
  c.v[0] = u.x; c.v[1] = u.y; c.v[2] = u.z; c.v[3] = u.w;
  c.v[4] = w.x; c.v[5] = w.y; c.v[6] = w.z; c.v[7] = w.w;
}
__device__ __forceinline__ void ps_st4(float* ps, int i, const Col<float>& c) {
  float4* q = reinterpret_cast<float4*>(ps);
  q[i] = make_float4(c.v[0], c.v[1], c.v[2], c.v[3]);
  q[i + 64] = make_float4(c.v[4], c.v[5], c.v[6], c.v[7]);
}

// The resident loop's scalar state, kept by thread 0.
struct ResScalars {
  double rr, rz, rz_old, alpha, beta, pAp;
  int status, max_iter;
  PcgRule rule;
};

// Where a neighbour of the CTA's cells lives.
struct ResFrame {
  const float* ps;       // shared p of the CTA's leaves
  const uint8_t* fsm;    // shared flags
  int L0, nl, n_pleaf;
};
__device__ __forceinline__ bool res_local(const ResFrame& fr, int slot) {
  return slot >= fr.L0 && slot < fr.L0 + fr.nl;
}

// p (current iteration) of cell (x, y, z) of leaf `slot`: from shared memory
// for the CTA's leaves, else formed from the mirrors of z and the previous p.
__device__ __forceinline__ float res_pcell(const ResFrame& fr, const PcgArgs& a,
                                           const float* pm_old, const DiagInv<float>* tab,
                                           float beta, int slot, int x, int y, int z) {
  if (res_local(fr, slot)) return fr.ps[(ps_col4(slot - fr.L0, x, y) + (z >> 2) * 64) * 4 + (z & 3)];
  const unsigned o = slot_or_null(slot, fr.n_pleaf) * 512u + unsigned(x * 64 + y * 8 + z);
  // the mirror holds z = M r (the owner's product): pnew_of's operations
  return tadd(__ldcg(static_cast<const float*>(a.r) + o), tmul(beta, __ldcg(pm_old + o)));
}

// The half leaf's faces in other CTAs' leaves (its outward x face and both
// y faces: 16 columns of 8 cells), formed by all 32 lanes in step: lane L
// forms cells 4 (L & 1) .. + 3 of face column t = L >> 1 (t < 8: the x face
// at y = t; 8 .. 11: the -y face at x = xb + t - 8; 12 .. 15: the +y face)
// from the mirrors of z and the previous p, with the owner's operations.
// Faces in the CTA's own leaves are left to shared memory (v stays 0).
__device__ __forceinline__ void res_faces(const ResFrame& fr, const PcgArgs& a, const float* pm_old,
                                          const DiagInv<float>* tab, float beta, int xb,
                                          const int fs[6], int lane, float (&v)[4]) {
  const int t = lane >> 1;
  int slot, off;
  if (t < 8) {
    slot = xb == 0 ? fs[0] : fs[1];
    off = (xb == 0 ? 7 : 0) * 64 + t * 8;
  } else if (t < 12) {
    slot = fs[2];
    off = (xb + t - 8) * 64 + 56;
  } else {
    slot = fs[3];
    off = (xb + t - 12) * 64;
  }
  off += 4 * (lane & 1);
#pragma unroll
  for (int j = 0; j < 4; ++j) v[j] = 0.f;
  if (!res_local(fr, slot)) {
    const unsigned o = slot_or_null(slot, fr.n_pleaf) * 512u + unsigned(off);
    // the mirror holds z = M r (the owner's product): pnew_of's operations
    const float4 zm = __ldcg(reinterpret_cast<const float4*>(static_cast<const float*>(a.r) + o));
    const float4 po = __ldcg(reinterpret_cast<const float4*>(pm_old + o));
    v[0] = tadd(zm.x, tmul(beta, po.x));
    v[1] = tadd(zm.y, tmul(beta, po.y));
    v[2] = tadd(zm.z, tmul(beta, po.z));
    v[3] = tadd(zm.w, tmul(beta, po.w));
  }
}
// column c of the faces formed by res_faces (lanes 2 c and 2 c + 1)
__device__ __forceinline__ void res_face_col(const float (&v)[4], int c, Col<float>& out) {
#pragma unroll
  for (int z = 0; z < 8; ++z) out.v[z] = __shfl_sync(0xffffffffu, v[z & 3], 2 * c + (z >> 2));
}

// A p on the lane's column (xb + lx, y) of leaf s (own values P), in the
// reference's column order; 0 off-fluid.  Called by all 32 lanes of the
// warp together (res_faces, res_face_col).
__device__ __forceinline__ void res_ap(const ResFrame& fr, const PcgArgs& a, const float* pm_old,
                                       const DiagInv<float>* tab, float beta, int s, int xb, int lx,
                                       int y, int lane, const int fs[6], const Col<float>& P,
                                       uint2 f, Col<float>& ap) {
  const int x = xb + lx;
  const int own = ps_col4(s - fr.L0, x, y);
  float fv[4];
  res_faces(fr, a, pm_old, tab, beta, xb, fs, lane, fv);
  // one neighbour column at a time, in the reference's order: -x, -y, -z,
  // diag, +z, +y, +x
  Col<float> nc;
#pragma unroll
  for (int z = 0; z < 8; ++z) ap.v[z] = 0.f;
  if (xb == 0) res_face_col(fv, y, nc);  // warp-uniform: the outward face is -x
  if (x > 0)
    ps_ld4(fr.ps, own - 8, nc);
  else if (res_local(fr, fs[0]))
    ps_ld4(fr.ps, ps_col4(fs[0] - fr.L0, 7, y), nc);
#pragma unroll
  for (int z = 0; z < 8; ++z) ap.v[z] = tsub(ap.v[z], nc.v[z]);
  Col<float> gy;  // the -y face column for lanes at y = 0, the +y one at y = 7
  res_face_col(fv, (y == 0 ? 8 : 12) + lx, gy);
  if (y > 0)
    ps_ld4(fr.ps, own - 1, nc);
  else if (res_local(fr, fs[2]))
    ps_ld4(fr.ps, ps_col4(fs[2] - fr.L0, x, 7), nc);
  else
    nc = gy;
#pragma unroll
  for (int z = 0; z < 8; ++z) ap.v[z] = tsub(ap.v[z], nc.v[z]);
  const float zm = res_pcell(fr, a, pm_old, tab, beta, fs[4], x, y, 7);
  const float zp = res_pcell(fr, a, pm_old, tab, beta, fs[5], x, y, 0);
#pragma unroll
  for (int z = 0; z < 8; ++z) {
    const uint8_t g = fbyte(f, z);
    const float vzm = z == 0 ? zm : P.v[(z + 7) & 7], vzp = z == 7 ? zp : P.v[(z + 1) & 7];
    ap.v[z] = tsub(ap.v[z], vzm);
    ap.v[z] = tadd(ap.v[z], tmul(tab[g & 15].d, P.v[z]));
    ap.v[z] = tsub(ap.v[z], vzp);
  }
  if (y < 7)
    ps_ld4(fr.ps, own + 1, nc);
  else if (res_local(fr, fs[3]))
    ps_ld4(fr.ps, ps_col4(fs[3] - fr.L0, x, 0), nc);
  else
    nc = gy;
#pragma unroll
  for (int z = 0; z < 8; ++z) ap.v[z] = tsub(ap.v[z], nc.v[z]);
  if (xb != 0) res_face_col(fv, y, nc);  // the outward face is +x
  if (x < 7)
    ps_ld4(fr.ps, own + 8, nc);
  else if (res_local(fr, fs[1]))
    ps_ld4(fr.ps, ps_col4(fs[1] - fr.L0, 0, y), nc);
#pragma unroll
  for (int z = 0; z < 8; ++z) {
    ap.v[z] = tsub(ap.v[z], nc.v[z]);
    if (!(fbyte(f, z) & 1)) ap.v[z] = 0.f;
  }
}

// r and A p of the CTA's cells live in tensor memory (TMEM): all 512
// columns, allocated by warp 0; warp w uses TMEM lanes 32 (w % 4) .. + 31
// (the quarter it may access), and for its half leaf k columns (w / 4) * 32
// + 8 k .. + 7 for r and the same + kResTmemAp for A p (lane L holds its
// column's 8 cells).  That leaves the registers to 28 warps, and A p, formed
// once per iteration for p.Ap, is kept for the update of r; from then to the
// next S its columns hold z = M r, formed once for r.z and p = z + beta p.  x of half leaf
// 0 takes columns kResTmemX + (w / 4) * 8 .. + 7; x of half leaves 1 .. 3
// is in shared memory.  So every vector of the iteration stays on chip, and
// x is read and written in global memory once per solve.
constexpr unsigned kResTmemCols = 512;
constexpr unsigned kResTmemVec = (kResWarps + 3) / 4 * kResHL * 8;  // columns of r or A p
constexpr unsigned kResTmemAp = kResTmemVec;
constexpr unsigned kResTmemX = 2 * kResTmemVec;
static_assert(kResTmemX + (kResWarps + 3) / 4 * 8 <= kResTmemCols, "TMEM columns");

// x of the warp's half leaf k >= 1 in shared memory: two 16-byte chunks per
// lane (cells z = 0..3 and 4..7), consecutive lanes in consecutive words
__device__ __forceinline__ void xs_ld(const float4* xs, int k, int warp, int lane, float (&v)[8]) {
  const float4 u = xs[(((k - 1) * kResWarps + warp) * 2 + 0) * 32 + lane];
  const float4 w = xs[(((k - 1) * kResWarps + warp) * 2 + 1) * 32 + lane];
  v[0] = u.x; v[1] = u.y; v[2] = u.z; v[3] = u.w;
  v[4] = w.x; v[5] = w.y; v[6] = w.z; v[7] = w.w;
}
__device__ __forceinline__ void xs_st(float4* xs, int k, int warp, int lane, const float (&v)[8]) {
  xs[(((k - 1) * kResWarps + warp) * 2 + 0) * 32 + lane] = make_float4(v[0], v[1], v[2], v[3]);
  xs[(((k - 1) * kResWarps + warp) * 2 + 1) * 32 + lane] = make_float4(v[4], v[5], v[6], v[7]);
}
__device__ __forceinline__ void tmem_ld8(unsigned t, float (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                 "=f"(v[6]), "=f"(v[7])
               : "r"(t)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_st8(unsigned t, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};\n" ::"r"(t),
               "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]),
               "f"(v[7])
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory");
}

__global__ void __launch_bounds__(kResThreads, 1) k_pcg_resident(const __grid_constant__ PcgArgs a) {
  extern __shared__ __align__(16) unsigned char res_smem[];
  float* ps = reinterpret_cast<float*>(res_smem);
  uint8_t* fsm = res_smem + size_t(kResLeaves) * 512 * sizeof(float);
  float4* xs = reinterpret_cast<float4*>(res_smem + size_t(kResLeaves) * 512 * (sizeof(float) + 1));
  __shared__ DiagInv<float> tab[16];
  __shared__ int s_ok, s_done;
  __shared__ float s_fa, s_fbeta;
  __shared__ ResScalars q;  // thread 0's
  __shared__ unsigned s_taddr;
  PcgScalars* sc = a.sc;
  const int G = int(gridDim.x);
  const int per = (a.n_pleaf + G - 1) / G;  // the host checks per <= kResLeaves
  ResFrame fr;
  fr.ps = ps;
  fr.fsm = fsm;
  fr.L0 = int(blockIdx.x) * per;
  fr.nl = max(0, min(per, a.n_pleaf - fr.L0));
  fr.n_pleaf = a.n_pleaf;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  fill_diag_table<float>(tab);
  for (int i = threadIdx.x; i < fr.nl * 512; i += kResThreads) {
    fsm[i] = a.flags[int64_t(fr.L0) * 512 + i];
    ps[i] = 0.f;  // p of iteration -1
  }
  if (warp == 0) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(&s_taddr));
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(sa),
                 "r"(kResTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tbase = s_taddr + ((32u * unsigned(warp & 3)) << 16) + unsigned(warp >> 2) * 32u;
  const unsigned txb = s_taddr + ((32u * unsigned(warp & 3)) << 16) + kResTmemX + unsigned(warp >> 2) * 8u;
  // the warp's half leaves: r and x on chip, the face slots, and which of
  // the lane's columns other CTAs read (bit k of mir: the column is on a face
  // whose neighbour leaf is in another CTA, or the leaf's -z or +z neighbour
  // is, which reads a cell of every column); only those go to the mirrors
  int nbl[kResHL];
  unsigned mir = 0;
#pragma unroll
  for (int k = 0; k < kResHL; ++k) {
    const int hl = warp + k * kResWarps;
    nbl[k] = -1;
    if (hl < 2 * fr.nl) {
      const HalfLeaf h = half_pos(2 * fr.L0 + hl, lane);
      const unsigned og = unsigned(h.s) * 512u + unsigned(h.c);
      Col<float> r0;
      ldcol(static_cast<const float*>(a.r), og, r0);
      tmem_st8(tbase + 8u * k, r0.v);
      Col<float> z0;
      {
        const uint2 f = *reinterpret_cast<const uint2*>(fsm + (hl >> 1) * 512 + h.c);
#pragma unroll
        for (int z = 0; z < 8; ++z) z0.v[z] = tmul(tab[fbyte(f, z) & 15].inv, r0.v[z]);
        tmem_st8(tbase + kResTmemAp + 8u * k, z0.v);
      }
      ldcol(static_cast<const float*>(a.x), og, r0);
      if (k == 0)
        tmem_st8(txb, r0.v);
      else
        xs_st(xs, k, warp, lane, r0.v);
      nbl[k] = face_slot_lane(a.nbr, h.s, lane);
      int fs[6];
      face_slots(nbl[k], fs);
      const bool xo = h.xb == 0 ? (h.lx == 0 && !res_local(fr, fs[0]))
                                : (h.lx == 3 && !res_local(fr, fs[1]));
      const bool yo = (h.cy == 0 && !res_local(fr, fs[2])) || (h.cy == 7 && !res_local(fr, fs[3]));
      const bool zo = !res_local(fr, fs[4]) || !res_local(fr, fs[5]);
      if (xo || yo || zo) {
        mir |= 1u << k;
        stcol(static_cast<float*>(a.r), og, z0);  // the mirror of z for the first iteration
      }
    }
  }
  tmem_wait_st();
  // Thread 0 keeps the scalar state in fp64 and runs the loop test and the
  // alpha / beta steps (GB300's FP64 pipe is narrow, and the solve's
  // settings are read once: after the barriers' acquire loads every read of
  // the scalar block is an L2 round trip); the other threads take the stop
  // flag and the fp32 alpha and beta from shared memory.
  int it = sc->iter;
  if (threadIdx.x == 0) {
    q = ResScalars{sc->rr, sc->rz, sc->rz_old, 0.0, 0.0, 0.0, sc->status, sc->max_iter, pcg_rule(sc)};
    s_done = sc->done || it >= q.max_iter || converged(q.rule, q.rr);  // PCGDriver::Solve's loop test
    s_fbeta = 0.f;
  }
  __syncthreads();
  unsigned round = 0;
  bool ok = true;
  float* x = static_cast<float*>(a.x);
  float* rmir = static_cast<float*>(a.r);  // during the loop: the mirror of z = M r
  {
    // every CTA's z mirror is written before any CTA's first stencil reads it
    float v[1] = {0.f};
    ok = res_sync<1>(a, v, 0, ++round, &s_ok, [](const double (&)[1]) {});
  }
  while (ok && !s_done) {
    float* pm_new = static_cast<float*>((it & 1) ? a.p1 : a.p0);
    const float* pm_old = static_cast<const float*>((it & 1) ? a.p0 : a.p1);
    const float fbeta = s_fbeta;
    // S: p = z + beta p on the own columns
#pragma unroll
    for (int k = 0; k < kResHL; ++k) {
      const int hl = warp + k * kResWarps;
      if (hl < 2 * fr.nl) {
        const HalfLeaf h = half_pos(2 * fr.L0 + hl, lane);
        Col<float> P;
        const int own = ps_col4(hl >> 1, h.xb + h.lx, h.cy);
        ps_ld4(ps, own, P);
        float zk[8];  // z = M r, left in the A p columns by U (or the set-up)
        tmem_ld8(tbase + kResTmemAp + 8u * k, zk);
#pragma unroll
        for (int z = 0; z < 8; ++z) P.v[z] = tadd(zk[z], tmul(fbeta, P.v[z]));  // pnew_of's operations
        ps_st4(ps, own, P);
        if ((mir >> k) & 1u) stcol(pm_new, unsigned(h.s) * 512u + unsigned(h.c), P);
      }
    }
    __syncthreads();
    Dot<0> dp;
#pragma unroll
    for (int k = 0; k < kResHL; ++k) {
      const int hl = warp + k * kResWarps;
      int fs[6];
      face_slots(nbl[k], fs);
      if (hl < 2 * fr.nl) {
        const HalfLeaf h = half_pos(2 * fr.L0 + hl, lane);
        const int ol = (hl >> 1) * 512 + h.c;
        Col<float> P, ap;
        ps_ld4(ps, ps_col4(hl >> 1, h.xb + h.lx, h.cy), P);
        const uint2 f = *reinterpret_cast<const uint2*>(fsm + ol);
        res_ap(fr, a, pm_old, tab, fbeta, h.s, h.xb, h.lx, h.cy, lane, fs, P, f, ap);
#pragma unroll
        for (int z = 0; z < 8; ++z) dp.add(P.v[z], ap.v[z]);
        tmem_st8(tbase + kResTmemAp + 8u * k, ap.v);
      }
    }
    tmem_wait_st();
    {
      float v[1] = {dp.pvalue()};
      ok = res_sync<1>(a, v, 0, ++round, &s_ok, [&](const double (&tot)[1]) {
        q.pAp = round_t(q.rule, tot[0]);
        q.alpha = q.rule.fp32 ? double(__fdiv_rn(float(q.rz), float(q.pAp))) : q.rz / q.pAp;
        s_fa = float(q.alpha);
        if (!(q.alpha <= 1e5)) {  // CHECK_LE(alpha, LARGE_FLOAT)
          q.status = FSIM_ERR_BREAKDOWN;
          s_done = 1;
        }
      });
      if (!ok || s_done) break;
    }
    // U: x += alpha p, r -= alpha A p
    const float fa = s_fa, fna = -fa;
    Dot<0> drr, drz;
#pragma unroll
    for (int k = 0; k < kResHL; ++k) {
      const int hl = warp + k * kResWarps;
      if (hl < 2 * fr.nl) {
        const HalfLeaf h = half_pos(2 * fr.L0 + hl, lane);
        const int ol = (hl >> 1) * 512 + h.c;
        const unsigned og = unsigned(h.s) * 512u + unsigned(h.c);
        Col<float> P, X, R;
        if (k == 0)
          tmem_ld8(txb, X.v);
        else
          xs_ld(xs, k, warp, lane, X.v);
        ps_ld4(ps, ps_col4(hl >> 1, h.xb + h.lx, h.cy), P);
        const uint2 f = *reinterpret_cast<const uint2*>(fsm + ol);
#pragma unroll
        for (int z = 0; z < 8; ++z) X.v[z] = tadd(tmul(fa, P.v[z]), X.v[z]);
        if (k == 0)
          tmem_st8(txb, X.v);
        else
          xs_st(xs, k, warp, lane, X.v);
        float ap[8];
        tmem_ld8(tbase + 8u * k, R.v);
        tmem_ld8(tbase + kResTmemAp + 8u * k, ap);
#pragma unroll
        for (int z = 0; z < 8; ++z) {
          const uint8_t g = fbyte(f, z);
          R.v[z] = tadd(tmul(fna, ap[z]), R.v[z]);
          drr.add(R.v[z], R.v[z]);
          ap[z] = tmul(tab[g & 15].inv, R.v[z]);  // z = M r, for r.z and the next S
          drz.add(R.v[z], ap[z]);
        }
        tmem_st8(tbase + 8u * k, R.v);
        tmem_st8(tbase + kResTmemAp + 8u * k, ap);
        if ((mir >> k) & 1u) {
          Col<float> Z;
#pragma unroll
          for (int z = 0; z < 8; ++z) Z.v[z] = ap[z];
          stcol(rmir, og, Z);
        }
      }
    }
    tmem_wait_st();
    {
      float v[2] = {drr.pvalue(), drz.pvalue()};
      ok = res_sync<2>(a, v, 1, ++round, &s_ok, [&](const double (&tot)[2]) {
        q.rr = round_t(q.rule, tot[0]);
        const double rzn = round_t(q.rule, tot[1]);
        q.beta = q.rule.fp32 ? double(__fdiv_rn(float(rzn), float(q.rz))) : rzn / q.rz;
        q.rz_old = q.rz;
        q.rz = rzn;
        s_fbeta = float(q.beta);
        if (!(q.beta <= 1e5)) {  // CHECK_LE(beta, LARGE_FLOAT)
          q.status = FSIM_ERR_BREAKDOWN;
          s_done = 1;
        } else {
          s_done = (it + 1 >= q.max_iter) || converged(q.rule, q.rr);  // the next loop test
        }
      });
      if (!ok) break;
      ++it;
    }
  }
  if (!ok && threadIdx.x == 0) q.status = FSIM_ERR_TIMEOUT;
  // x and r back to global memory; every warp is then done with TMEM, and
  // warp 0 frees it
  tmem_wait_st();
#pragma unroll
  for (int k = 0; k < kResHL; ++k) {
    const int hl = warp + k * kResWarps;
    if (hl < 2 * fr.nl) {
      const HalfLeaf h = half_pos(2 * fr.L0 + hl, lane);
      const unsigned og = unsigned(h.s) * 512u + unsigned(h.c);
      Col<float> X;
      if (k == 0)
        tmem_ld8(txb, X.v);
      else
        xs_ld(xs, k, warp, lane, X.v);
      stcol(x, og, X);
      tmem_ld8(tbase + 8u * k, X.v);
      stcol(rmir, og, X);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(s_taddr),
                 "r"(kResTmemCols)
                 : "memory");
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->iter = it;
    sc->done = 1;
    sc->status = q.status;
    sc->rr = q.rr;
    sc->rz = q.rz;
    sc->rz_old = q.rz_old;
    sc->alpha = q.alpha;
    sc->beta = q.beta;
    sc->pAp = q.pAp;
  }
}

// MIXED: x64 += d (inner solution); d is the fp32 x of the inner solve.
__global__ void k_accumulate_x64(const __grid_constant__ PcgArgs a) {
  const int64_t n = int64_t(a.n_pleaf) * 512;
  for (int64_t o = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; o < n;
       o += int64_t(gridDim.x) * blockDim.x)
    if (a.flags[o] & 1) a.x64[o] += double(a.dinner[o]);
}

// MIXED: r64 = b - A x64 in fp64; writes the fp32 rhs of the next inner
// solve into r and accumulates r64.r64 (fp64) into sc->rr.
__global__ void __launch_bounds__(kThreads) k_residual64(const __grid_constant__ PcgArgs a) {
  float* rr32 = static_cast<float*>(a.r);
  double acc = 0.0;
  for (int s = blockIdx.x; s < a.n_pleaf; s += gridDim.x) {
    const int32_t* nb = a.nbr + int64_t(s) * 27;
    for (int v = threadIdx.x; v < 512; v += kThreads) {
      const int64_t o = int64_t(s) * 512 + v;
      const uint8_t f = a.flags[o];
      if (!(f & 1)) { rr32[o] = 0.f; continue; }
      const int cx = v >> 6, cy = (v >> 3) & 7, cz = v & 7;
      double ax = double(flag_diag(f)) * a.x64[o];
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        int ux = cx, uy = cy, uz = cz;
        const int d = (q & 1) ? 1 : -1;
        if (q < 2) ux += d; else if (q < 4) uy += d; else uz += d;
        const int sx = ux < 0 ? -1 : (ux > 7 ? 1 : 0), sy = uy < 0 ? -1 : (uy > 7 ? 1 : 0),
                  sz = uz < 0 ? -1 : (uz > 7 ? 1 : 0);
        const int ns = nb[(sx + 1) * 9 + (sy + 1) * 3 + (sz + 1)];
        if (ns < 0 || ns >= a.n_pleaf) continue;
        const int64_t u = int64_t(ns) * 512 + (((ux & 7) << 6) | ((uy & 7) << 3) | (uz & 7));
        if (a.flags[u] & 1) ax -= a.x64[u];
      }
      const double res = (a.b64 ? a.b64[o] : double(a.b[o])) - ax;
      rr32[o] = float(res);
      acc += res * res;
    }
  }
  double v[1] = {acc};
  double tot[1];
  if (grid_sum<2, 1>(v, a.part, a.maxb, &a.sc->cnt_r, tot) && threadIdx.x == 0) a.sc->rr = tot[0];
}

// MIXED residual replacement: r now holds the fp32 image of the fp64 true
// residual b - A x64 and x64 has absorbed x.  x restarts at 0, the r z-face
// planes follow r, and r.r, r.z are recomputed; CG then continues with its
// search direction: beta = r'.z' / (r.z of the previous iteration), r.z =
// r'.z', and the inner stop is a further inner_tolerance drop from |r'|, but
// no lower than the outer target: iterating past tol*|b| in fp32 only
// overshoots, because the fp64 check that follows decides convergence.
__global__ void __launch_bounds__(kThreads) k_pcg_replace(const __grid_constant__ PcgArgs a) {
  float* x = static_cast<float*>(a.x);
  const float* r = static_cast<const float*>(a.r);
  Dot<1> drr, drz;
  for (int s = blockIdx.x; s < a.n_pleaf; s += gridDim.x) {
    for (int v = threadIdx.x; v < 512; v += kThreads) {
      const int64_t o = int64_t(s) * 512 + v;
      const uint8_t f = a.flags[o];
      x[o] = 0.f;
      const float rv = r[o];
      const int cz = v & 7;
      if (cz == 0 || cz == 7) {
        const int fi = (cz == 7 ? 64 : 0) + (v >> 6) * 8 + ((v >> 3) & 7);
        static_cast<float*>(a.zf)[int64_t(s) * 384 + fi] = rv;
      }
      drr.add(rv, rv);
      drz.add(rv, tmul(inv_sel<float>(f), rv));
    }
  }
  double v[2] = {drr.value(), drz.value()};
  double tot[2];
  if (grid_sum<1, 2>(v, a.part, a.maxb, &a.sc->cnt_s, tot) && threadIdx.x == 0) {
    PcgScalars* sc = a.sc;
    sc->rr = tot[0];
    sc->beta = tot[1] / sc->rz_old;
    sc->rz = tot[1];
    sc->thr = fmax(sc->tol2 * tot[0], sc->tol2_outer * sc->bb);
    sc->status = FSIM_OK;
    sc->done = (sc->iter >= sc->max_iter) ? 1 : 0;
    // the resuming spmv takes r'.r', r'.z' and beta from here
    PcgIterState o = {};
    o.rr = sc->rr;
    o.rz = sc->rz;
    o.beta = sc->beta;
    o.rz_prev = sc->rz_old;
    o.iter = sc->iter;
    o.done = sc->done;
    o.status = FSIM_OK;
    o.given = 1;
    sc->st[1] = o;
  }
}

template <typename T>
__global__ void k_to_pressure(const T* __restrict__ x, float* __restrict__ pres, int64_t n) {
  for (int64_t o = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; o < n;
       o += int64_t(gridDim.x) * blockDim.x)
    pres[o] = float(x[o]);
}

// The spmv whose own columns are staged by bulk copies (k_pcg_spmv_tma):
// opt-in, FSIM_PCG_TMA=1.
template <typename T>
bool use_tma_spmv(const fsim_sim* s, int /*n_pleaf*/) {
  return std::is_same<T, float>::value && s->use_pipe && s->tma_spmv;
}

// The hot kernel pair of a solve: the register-pipelined pair (fp32
// vectors; FSIM_PCG_TMA=1: the bulk-copy staged spmv), or the plain pair
// (fp64 vectors, or FSIM_PCG_PIPE=0).
template <typename T, int DM>
void* spmv_kernel(const fsim_sim* s, bool zd, int n_pleaf) {
  if constexpr (std::is_same<T, float>::value) {
    if (use_tma_spmv<T>(s, n_pleaf)) {
      void* fn = zd ? reinterpret_cast<void*>(k_pcg_spmv_tma<DM, true>)
                    : reinterpret_cast<void*>(k_pcg_spmv_tma<DM, false>);
      // opt in to the ring's dynamic shared memory (idempotent)
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTmaDynSmem));
      return fn;
    }
    if (s->use_pipe)
      return zd ? reinterpret_cast<void*>(k_pcg_spmv_pl<T, DM, true>)
                : reinterpret_cast<void*>(k_pcg_spmv_pl<T, DM, false>);
  }
  return reinterpret_cast<void*>(k_pcg_spmv<T, DM>);
}
// dynamic shared memory of the spmv launch
template <typename T>
size_t spmv_smem(const fsim_sim* s, int n_pleaf) {
  return use_tma_spmv<T>(s, n_pleaf) ? kTmaDynSmem : 0;
}
template <typename T, int DM>
void* update_kernel(const fsim_sim* s, bool zd) {
  if constexpr (std::is_same<T, float>::value) {
    if (s->use_pipe)
      return zd ? reinterpret_cast<void*>(k_pcg_update_pl<T, DM, true>)
                : reinterpret_cast<void*>(k_pcg_update_pl<T, DM, false>);
  }
  return reinterpret_cast<void*>(k_pcg_update<T, DM>);
}
// Large systems: the pipelined kernels read z-face neighbours from the
// vectors (L2 hits) instead of the published planes, which no longer fit in
// L2 and cost about 4 B of DRAM traffic per unknown and iteration.
template <typename T>
bool use_zdirect(const fsim_sim* s, int n_pleaf) {
  return std::is_same<T, float>::value && s->use_pipe &&
         (s->zdirect > 0 || (s->zdirect < 0 && n_pleaf > kZDirectLeaves));
}
int launch_hot(fsim_sim* s, const char* name, void* fn, int grid, PcgArgs& a,
               size_t smem = 0) {
  fsim::ProfScope ps(s, name);
  void* args[] = {&a};
  const cudaError_t e = cudaLaunchKernel(fn, dim3(unsigned(grid)), dim3(kHotThreads), args, smem,
                                         s->stream);
  s->launches++;
  if (e != cudaSuccess) return cuda_fail(s, e, name);
  return FSIM_OK;
}

// Builds and launches graph = WHILE(cond){ (spmv; update) x pass_iters } on
// the handle's stream: one pass runs pass_iters iterations of alternating
// parity (their buffers are fixed by PcgArgs::par), and kernels launched
// after the stop flag is set return at once.  The head of the kernel that
// sets the stop flag clears the condition.  Returns FSIM_OK, or
// FSIM_ERR_CUDA when the graph API refuses (the caller then polls from the
// host).  Kernel launches inside the graph are counted by the caller from
// the iteration count the solve reports.
//
// Pass length: each pass costs about 4 us of graph overhead, and the last
// pass runs up to pass - 1 iterations of launches that return at once (about
// 5 us each).  For I iterations the sum is smallest near pass = sqrt(1.7 I),
// so the pass length follows the longest graph-loop segment of the handle's
// previous solve (a MIXED solve runs several segments, and its last one is
// often short): 8 iterations up to about 150, 16 up to about 600, then 32
// (even, so that a pass leaves the launch parity where it found it).  FSIM_PCG_PASS_ITERS fixes it instead
// (an even count; an odd one would swap the p buffers of every later pass).
#ifndef FSIM_PCG_PASS_ITERS
#define FSIM_PCG_PASS_ITERS 0
#endif
static_assert(FSIM_PCG_PASS_ITERS >= 0 && FSIM_PCG_PASS_ITERS % 2 == 0,
              "FSIM_PCG_PASS_ITERS must be even: a pass must keep the launch parity");
int pass_iters_for(const fsim_sim* s) {
  if (FSIM_PCG_PASS_ITERS > 0) return FSIM_PCG_PASS_ITERS;
  const double p = std::sqrt(1.7 * double(s->pcg_last_iters));
  return p >= 32.0 ? 32 : (p >= 16.0 ? 16 : 8);
}

//
// With fn_cg1 (the single-reduction kernel) the body is pass_iters launches
// of that kernel, one per iteration, alternating parity.
template <typename T, int DM>
int run_graph_loop(fsim_sim* s, PcgArgs a, int wgrid, int par0, bool pdl, int pass_iters,
                   void* fn_cg1 = nullptr, void* fn_fix = nullptr) {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  cudaGraphConditionalHandle h = 0;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  if (e == cudaSuccess) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    a.cond = h;
    PcgArgs ap[2] = {a, a};
    ap[0].par = par0;
    ap[1].par = par0 ^ 1;
    cudaGraphNode_t prev = nullptr;
    const int nodes = fn_cg1 ? pass_iters + (fn_fix ? 1 : 0) : 2 * pass_iters;
    for (int k = 0; k < nodes && e == cudaSuccess; ++k) {
      cudaGraphNodeParams kn = {};
      kn.type = cudaGraphNodeTypeKernel;
      // the s re-forming node closes the pass with the next launch's parity, par0
      void* args[] = {&ap[fn_cg1 ? (k & 1) : ((k >> 1) & 1)]};
      kn.kernel.gridDim = dim3(unsigned(wgrid));
      kn.kernel.blockDim = dim3(unsigned(kHotThreads));
      kn.kernel.kernelParams = args;
      const bool zd = use_zdirect<T>(s, a.n_pleaf);
      if (fn_cg1) {
        kn.kernel.func = k == pass_iters ? fn_fix : fn_cg1;
        kn.kernel.sharedMemBytes = 0u;
      } else {
        kn.kernel.func = (k & 1) ? update_kernel<T, DM>(s, zd)
                                 : spmv_kernel<T, DM>(s, zd, a.n_pleaf);
        kn.kernel.sharedMemBytes = (k & 1) ? 0u : unsigned(spmv_smem<T>(s, a.n_pleaf));
      }
      cudaGraphEdgeData ed = {};
      if (pdl) {  // the successor may launch while this kernel's last CTAs finish
        ed.from_port = cudaGraphKernelNodePortProgrammatic;
        ed.type = cudaGraphDependencyTypeProgrammatic;
      }
      cudaGraphNode_t n = nullptr;
      e = cudaGraphAddNode(&n, body, prev ? &prev : nullptr, prev ? &ed : nullptr, prev ? 1 : 0,
                           &kn);
      prev = n;
    }
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(ge, s->stream);
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the (non-sticky) error of the refused call
    return FSIM_ERR_CUDA;
  }
  return FSIM_OK;
}

// Device time of an iteration loop: events on the handle's stream around it,
// read after the loop's own synchronisation; accumulated per solve.
struct LoopTimer {
  fsim_sim* s;
  bool on = false;
  explicit LoopTimer(fsim_sim* h) : s(h) {
    if (!s->ev_loop[0]) {
      if (cudaEventCreate(&s->ev_loop[0]) != cudaSuccess) s->ev_loop[0] = nullptr;
      if (cudaEventCreate(&s->ev_loop[1]) != cudaSuccess) s->ev_loop[1] = nullptr;
    }
    on = s->ev_loop[0] && s->ev_loop[1] &&
         cudaEventRecord(s->ev_loop[0], s->stream) == cudaSuccess;
  }
  void stop() {
    if (on && cudaEventRecord(s->ev_loop[1], s->stream) == cudaSuccess) {
      cudaEventSynchronize(s->ev_loop[1]);
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, s->ev_loop[0], s->ev_loop[1]) == cudaSuccess)
        s->pcg_loop_ms += double(ms);
    }
    on = false;
  }
};

// One inner solve: setup, then the iterations.  The iterations run as a CUDA
// graph whose conditional WHILE node repeats {spmv, update}; the kernel head
// that sets the stop flag clears the condition, so the whole loop runs
// without a host round trip.  The loop is bounded by the
// solve's max_iterations (the stop flag is set at that count).  If graph
// construction is not available the host launches chunks of iterations and
// polls the stop flag between them (kernels launched after it is set return
// at once).
template <typename T, int DM>
int run_inner(fsim_sim* s, PcgArgs& a, int grid, const char* nm_setup, const char* nm_spmv,
              const char* nm_upd, bool setup = true, int par0 = 0) {
  a.cond = 0;
  if (setup) FSIM_LAUNCH(s, nm_setup, (k_pcg_setup<T, DM>), grid, kThreads, 0, a);
  const int wpb = kHotThreads / 32;
  int occ_a = 1, occ_b = 1;
  const bool zd = use_zdirect<T>(s, a.n_pleaf);
  void* const fn_spmv = spmv_kernel<T, DM>(s, zd, a.n_pleaf);
  void* const fn_upd = update_kernel<T, DM>(s, zd);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_a, fn_spmv, kHotThreads,
                                                spmv_smem<T>(s, a.n_pleaf));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, fn_upd, kHotThreads, 0);
  const int resident = std::max(1, std::min(occ_a, occ_b)) * s->num_sms;
  const int wgrid = std::max(1, std::min({(2 * a.n_pleaf + wpb - 1) / wpb, resident,
                                          s->max_blocks, kMaxHotGrid}));
  const int it0 = setup ? 0 : s->h_sc->iter;  // iterations before this segment
  if (s->use_graphs && !s->profiling) {
    LoopTimer lt(s);
    int rc = FSIM_ERR_CUDA;
    // Programmatic edges pay off only for the pipelined fp32-vector kernels,
    // which prefetch before their wait; the others wait at their first
    // instruction, and their early-launched CTAs only hold SM slots (the
    // FP64 solve measured 20% slower with them).
    // (the bulk-copy spmv also waits at its first instruction)
    const bool pdl = s->use_pdl && std::is_same<T, float>::value && s->use_pipe &&
                     !use_tma_spmv<T>(s, a.n_pleaf);
    const int pass_iters = pass_iters_for(s);
    if (pdl) {
      rc = run_graph_loop<T, DM>(s, a, wgrid, par0, true, pass_iters);
      if (rc != FSIM_OK) s->use_pdl = false;  // programmatic edges refused: plain edges
    }
    if (rc != FSIM_OK) rc = run_graph_loop<T, DM>(s, a, wgrid, par0, false, pass_iters);
    if (rc == FSIM_OK) {
      lt.stop();
      FSIM_CK(s, cudaMemcpyAsync(s->h_sc, a.sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                                 s->stream));
      FSIM_CK(s, cudaStreamSynchronize(s->stream));
      // each WHILE pass launches 2 * pass_iters kernels; the stop flag is
      // set in the head of iteration n (n = iterations completed here), so
      // n / pass_iters + 1 passes ran
      const int64_t n = std::max(s->h_sc->iter - it0, 0);
      s->launches += 2 * pass_iters * (n / pass_iters + 1);
      s->pcg_seg_max = std::max(s->pcg_seg_max, int(std::min<int64_t>(n, 1 << 30)));
      if (s->h_sc->wait_err)
        return fail(s, FSIM_ERR_TIMEOUT, "PCG: a bulk-copy stage wait gave up");
      return FSIM_OK;
    }
    s->use_graphs = false;  // fall back for the rest of this handle's life
  }
  a.cond = 0;
  int chunk = 8;
  int64_t launched = par0;  // parity of the next iteration; tracks the device count
  LoopTimer lt(s);
  for (;;) {
    FSIM_CK(s, cudaMemcpyAsync(s->h_sc, a.sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                               s->stream));
    FSIM_CK(s, cudaStreamSynchronize(s->stream));
    if (s->h_sc->done) break;
    for (int c = 0; c < chunk; ++c, ++launched) {
      a.par = int(launched & 1);
      int rc = launch_hot(s, nm_spmv, fn_spmv, wgrid, a, spmv_smem<T>(s, a.n_pleaf));
      if (rc == FSIM_OK) rc = launch_hot(s, nm_upd, fn_upd, wgrid, a);
      if (rc != FSIM_OK) return rc;
    }
    if (chunk < 64) chunk *= 2;
  }
  lt.stop();
  if (s->h_sc->wait_err) return fail(s, FSIM_ERR_TIMEOUT, "PCG: a bulk-copy stage wait gave up");
  return FSIM_OK;
}

// One fp32 solve by the single-reduction iteration: setup, the launch that
// forms w_0 = A M r_0, then the iterations, as run_inner runs them (a graph
// WHILE loop, or host-polled chunks).
template <typename T, int DM>
int run_cg1(fsim_sim* s, PcgArgs& a, int grid) {
  a.cond = 0;
  FSIM_LAUNCH(s, "pcg_setup", (k_pcg_setup<T, DM>), grid, kThreads, 0, a);
  void* const fn = reinterpret_cast<void*>(k_pcg_cg1<T, DM>);
  void* const fn_fix = reinterpret_cast<void*>(k_pcg_cg1_s<T>);
  const int wpb = kHotThreads / 32;
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kHotThreads, 0);
  const int wgrid = std::max(1, std::min({(2 * a.n_pleaf + wpb - 1) / wpb,
                                          std::max(1, occ) * s->num_sms, s->max_blocks,
                                          kMaxHotGrid}));
  a.par = 0;
  int rc = launch_hot(s, "pcg_cg1", fn, wgrid, a);
  if (rc != FSIM_OK) return rc;
  if (s->use_graphs && !s->profiling) {
    LoopTimer lt(s);
    const int pass_iters = pass_iters_for(s);
    rc = FSIM_ERR_CUDA;
    if (s->use_pdl) {
      rc = run_graph_loop<T, DM>(s, a, wgrid, 1, true, pass_iters, fn, fn_fix);
      if (rc != FSIM_OK) s->use_pdl = false;
    }
    if (rc != FSIM_OK) rc = run_graph_loop<T, DM>(s, a, wgrid, 1, false, pass_iters, fn, fn_fix);
    if (rc == FSIM_OK) {
      lt.stop();
      FSIM_CK(s, cudaMemcpyAsync(s->h_sc, a.sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                                 s->stream));
      FSIM_CK(s, cudaStreamSynchronize(s->stream));
      // one launch per iteration and one s re-forming launch per pass; the
      // stop is set in the head of launch n
      const int64_t n = std::max(s->h_sc->iter, 0);
      s->launches += (pass_iters + 1) * (n / pass_iters + 1);
      s->pcg_seg_max = std::max(s->pcg_seg_max, int(std::min<int64_t>(n, 1 << 30)));
      return FSIM_OK;
    }
    s->use_graphs = false;
  }
  // host-polled: chunks of the graph's pass length, so that s is re-formed
  // after the same iterations and the solve is bitwise the graph loop's
  a.cond = 0;
  const int chunk = pass_iters_for(s);
  int64_t launched = 1;
  LoopTimer lt(s);
  for (;;) {
    FSIM_CK(s, cudaMemcpyAsync(s->h_sc, a.sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                               s->stream));
    FSIM_CK(s, cudaStreamSynchronize(s->stream));
    if (s->h_sc->done) break;
    for (int c = 0; c < chunk; ++c, ++launched) {
      a.par = int(launched & 1);
      if ((rc = launch_hot(s, "pcg_cg1", fn, wgrid, a)) != FSIM_OK) return rc;
    }
    a.par = int(launched & 1);  // the next launch's s buffer
    if ((rc = launch_hot(s, "pcg_cg1_s", fn_fix, wgrid, a)) != FSIM_OK) return rc;
  }
  lt.stop();
  return FSIM_OK;
}

// One fp32 solve by the resident loop: setup, then one cooperative launch of
// one CTA per SM that runs every iteration.  FSIM_ERR_CUDA when the launch is
// refused (the caller then runs the pair).
int run_resident(fsim_sim* s, PcgArgs& a, int grid) {
  void* const fn = reinterpret_cast<void*>(k_pcg_resident);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kResSmem)) !=
      cudaSuccess) {
    cudaGetLastError();
    return FSIM_ERR_CUDA;
  }
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kResThreads, kResSmem);
  if (occ < 1) return FSIM_ERR_CUDA;
  a.cond = 0;
  FSIM_LAUNCH(s, "pcg_setup", (k_pcg_setup<float, 0>), grid, kThreads, 0, a);
  LoopTimer lt(s);
  {
    fsim::ProfScope ps(s, "pcg_resident");
    void* args[] = {&a};
    const cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(unsigned(s->num_sms)),
                                                      dim3(unsigned(kResThreads)), args, kResSmem,
                                                      s->stream);
    s->launches++;
    if (e != cudaSuccess) return cuda_fail(s, e, "pcg_resident");
  }
  lt.stop();
  FSIM_CK(s, cudaMemcpyAsync(s->h_sc, a.sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  if (s->h_sc->bar_err) return fail(s, FSIM_ERR_TIMEOUT, "PCG: a resident-loop barrier gave up");
  return FSIM_OK;
}
// The resident loop takes fp32 solves whose particle leaves fit (at most
// kResLeaves per SM) and are many enough to amortise its fixed cost per
// iteration (two grid barriers, about 7.6 us in all): from kResMinLeaves per
// SM.  Measured per iteration against the pair: 20.95 against 32.1 us at
// 256^3 (55 leaves per SM), 9.0 against 12.45 at 128^3 (7.6), 7.9 against
// 6.5-7.0 at 64^3 (about one leaf per SM); the two meet near two leaves per
// SM.  FSIM_PCG_RES=0 / 1 turns it off / on wherever it fits.
constexpr int kResMinLeaves = 2;
bool use_resident(const fsim_sim* s, int precision) {
  if (precision != FSIM_PREC_FP32 || s->pcg_res == 0) return false;
  const int64_t n = s->n_pleaf, sms = s->num_sms;
  if (n > int64_t(kResLeaves) * sms) return false;
  return s->pcg_res > 0 || n >= int64_t(kResMinLeaves) * sms;
}

// fp32 solves take the single-reduction iteration on request (FSIM_PCG_CG1=1).
// It saves one launch's fixed cost per iteration (5.1 against 7.0 us per
// iteration at 64^3, 9.9 against 12.5 at 128^3) but moves 41 B per unknown
// against the pair's 34, which spill from L2 on larger systems (35.3 against
// 32.1 us at 256^3).  Its recurrence for s costs accuracy on smooth systems
// even with s re-formed once per pass: on the first step of the 64^3
// sphere-drop replay its pressure lands 1.22e-5 from the oracle's, against
// the pair's 6.3e-6, so the pair stays the default.
bool use_cg1(const fsim_sim* s, int precision) {
  return precision == FSIM_PREC_FP32 && s->pcg_cg1 == 1;
}

int ensure_pcg_vectors(fsim_sim* s, int precision) {
  const size_t n = size_t(s->cap_pleaf) * 512;
  if (use_cg1(s, precision) && !s->cgw[0]) {
    for (int b = 0; b < 2; ++b) {
      FSIM_CK(s, cudaMalloc(&s->cgw[b], n * sizeof(float)));
      FSIM_CK(s, cudaMalloc(&s->cgs[b], n * sizeof(float)));
    }
  }
  if (precision == FSIM_PREC_MIXED && !s->x64) FSIM_CK(s, cudaMalloc(&s->x64, n * sizeof(double)));
  if (precision == FSIM_PREC_FP64 && !s->r64) {
    if (!s->x64) FSIM_CK(s, cudaMalloc(&s->x64, n * sizeof(double)));
    FSIM_CK(s, cudaMalloc(&s->r64, n * sizeof(double)));
    FSIM_CK(s, cudaMalloc(&s->p64[0], n * sizeof(double)));
    FSIM_CK(s, cudaMalloc(&s->p64[1], n * sizeof(double)));
    FSIM_CK(s, cudaMalloc(&s->zface64, size_t(s->cap_pleaf) * 384 * sizeof(double)));
  }
  return FSIM_OK;
}

}  // namespace

int pcg_solve(fsim_sim* s, const fsim_pcg_params* prm, fsim_pcg_stats* st, const double* b64) {
  if (!prm) return fail(s, FSIM_ERR_INVALID, "pcg params missing");
  if (prm->mode < 0 || prm->mode > 2 || prm->precision < 0 || prm->precision > 2)
    return fail(s, FSIM_ERR_INVALID, "bad pcg mode/precision");
  // the vectors hold the particle leaves and the zeroed null slot past them
  if (int64_t(s->cap_pleaf) < int64_t(s->n_pleaf) + 1)
    return fail(s, FSIM_ERR_STATE, "PCG vectors not sized for the leaf topology");
  int rc = ensure_pcg_vectors(s, prm->precision);
  if (rc) return rc;
  s->pcg_loop_ms = 0.0;
  s->pcg_seg_max = 0;
  const int grid = std::max(1, std::min(s->n_pleaf, s->max_blocks));
  PcgArgs a;
  memset(&a, 0, sizeof(a));
  a.n_pleaf = s->n_pleaf;
  a.maxb = s->max_blocks;
  a.nbr = s->d_nbr;
  a.marker = s->marker;
  a.b = s->div;
  a.b64 = b64;
  a.flags = s->flags;
  a.sc = s->d_sc;
  a.part = s->d_part;
  a.partf = s->d_partf;
  a.zf = s->zface;
  a.zff = s->zflags;
  a.p0 = s->p[0];
  a.p1 = s->p[1];
  a.r = s->r;
  a.x = s->pres;
  a.x64 = s->x64;
  a.dinner = s->pres;
  a.init_r = 1;
  a.withhold = s->tma_withhold;
  s->tma_withhold = 0;  // a test's withheld copy applies to one solve
  a.res_withhold = s->res_withhold;
  s->res_withhold = 0;  // and a withheld barrier arrival too

  PcgScalars h;
  memset(&h, 0, sizeof(h));
  h.mode = prm->mode;
  h.max_iter = prm->max_iterations;
  h.fp32 = (prm->precision == FSIM_PREC_FP32);
  h.thr = prm->threshold;
  h.tol2 = prm->tolerance * prm->tolerance;
  int total_it = 0, refinements = 1;
  int64_t n_rows = 0;
  double final_rr = 0.0, bb = 0.0;
  int status = FSIM_OK;
  const int64_t nvec = int64_t(s->n_pleaf) * 512;

  if (prm->precision == FSIM_PREC_FP32 || prm->precision == FSIM_PREC_FP64) {
    if (prm->precision == FSIM_PREC_FP64) {
      a.x = s->x64;
      a.r = s->r64;
      a.p0 = s->p64[0];
      a.p1 = s->p64[1];
      a.zf = s->zface64;
    }
    *s->h_sc = h;
    FSIM_CK(s, cudaMemcpyAsync(s->d_sc, s->h_sc, sizeof(PcgScalars), cudaMemcpyHostToDevice,
                               s->stream));
    if (use_resident(s, prm->precision)) {
      rc = run_resident(s, a, grid);
      if (rc == FSIM_ERR_CUDA) {  // cooperative launch refused: the pair
        cudaGetLastError();
        s->pcg_res = 0;
        *s->h_sc = h;
        FSIM_CK(s, cudaMemcpyAsync(s->d_sc, s->h_sc, sizeof(PcgScalars), cudaMemcpyHostToDevice,
                                   s->stream));
        rc = run_inner<float, 0>(s, a, grid, "pcg_setup", "pcg_spmv", "pcg_update");
      }
    } else if (use_cg1(s, prm->precision)) {
      for (int b = 0; b < 2; ++b) {
        a.w[b] = s->cgw[b];
        a.sv[b] = s->cgs[b];
      }
      rc = run_cg1<float, 0>(s, a, grid);
    } else if (prm->precision == FSIM_PREC_FP32)
      rc = run_inner<float, 0>(s, a, grid, "pcg_setup", "pcg_spmv", "pcg_update");
    else
      rc = run_inner<double, 2>(s, a, grid, "pcg_setup_f64", "pcg_spmv_f64", "pcg_update_f64");
    if (rc) return rc;
    total_it = s->h_sc->iter;
    n_rows = int64_t(s->h_sc->n_rows);
    final_rr = s->h_sc->rr;
    bb = s->h_sc->bb;
    status = s->h_sc->status;
    if (status == FSIM_OK && prm->mode == FSIM_PCG_RELATIVE && !(final_rr <= s->h_sc->thr))
      status = FSIM_ERR_NOT_CONVERGED;
    if (prm->precision == FSIM_PREC_FP64)
      FSIM_LAUNCH(s, "pcg_to_pressure", k_to_pressure<double>,
                  unsigned(std::min<int64_t>((nvec + 255) / 256, 4096)), 256, 0, s->x64, s->pres,
                  nvec);
  } else {
    // MIXED: fp32 Jacobi-PCG with exact dots, and fp64 residual replacement
    // (reliable updates): each time the recursive residual has dropped by
    // inner_tolerance, x is folded into x64, r is replaced by the fp32 image
    // of the fp64 true residual b - A x64, and CG continues with its search
    // direction.  The solve stops when the fp64 true residual meets the
    // tolerance.
    if (nvec > 0) FSIM_CK(s, cudaMemsetAsync(s->x64, 0, size_t(nvec) * sizeof(double), s->stream));
    PcgScalars hi = h;
    hi.mode = FSIM_PCG_RELATIVE;
    hi.tol2 = prm->inner_tolerance * prm->inner_tolerance;
    const double tol2 = prm->tolerance * prm->tolerance;
    hi.tol2_outer = tol2;
    refinements = 0;
    const int max_ref = std::max(1, prm->max_refinements);
    *s->h_sc = hi;
    FSIM_CK(s, cudaMemcpyAsync(s->d_sc, s->h_sc, sizeof(PcgScalars), cudaMemcpyHostToDevice,
                               s->stream));
    a.init_r = 1;
    rc = run_inner<float, 1>(s, a, grid, "pcg_setup_mixed", "pcg_spmv_mixed", "pcg_update_mixed");
    if (rc) return rc;
    // b.b: the first setup's r.r with r = b, accumulated exactly
    bb = s->h_sc->bb;
    n_rows = int64_t(s->h_sc->n_rows);
    for (;;) {
      ++refinements;
      total_it = s->h_sc->iter;
      if (s->h_sc->status != FSIM_OK) { status = s->h_sc->status; break; }
      FSIM_LAUNCH(s, "pcg_accumulate_x64", k_accumulate_x64,
                  unsigned(std::min<int64_t>((nvec + 255) / 256, 4096)), 256, 0, a);
      FSIM_LAUNCH(s, "pcg_residual_f64", k_residual64, grid, kThreads, 0, a);
      FSIM_CK(s, cudaMemcpyAsync(s->h_sc, s->d_sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                                 s->stream));
      FSIM_CK(s, cudaStreamSynchronize(s->stream));
      final_rr = s->h_sc->rr;
      if (final_rr <= tol2 * bb) break;
      if (s->h_sc->iter >= prm->max_iterations || refinements >= max_ref) break;
      FSIM_LAUNCH(s, "pcg_replace_residual", k_pcg_replace, grid, kThreads, 0, a);
      rc = run_inner<float, 1>(s, a, grid, "pcg_setup_mixed", "pcg_spmv_mixed", "pcg_update_mixed",
                               false, s->h_sc->iter & 1);
      if (rc) return rc;
    }
    if (status == FSIM_OK && !(final_rr <= tol2 * bb)) status = FSIM_ERR_NOT_CONVERGED;
    FSIM_LAUNCH(s, "pcg_to_pressure", k_to_pressure<double>,
                unsigned(std::min<int64_t>((nvec + 255) / 256, 4096)), 256, 0, s->x64, s->pres,
                nvec);
  }
  if (s->pcg_seg_max > 0) s->pcg_last_iters = s->pcg_seg_max;
  if (st) {
    st->iterations = total_it;
    st->refinements = refinements;
    st->n_rows = int32_t(n_rows);
    st->status = status;
    st->rr = final_rr;
    st->bb = bb;
    st->loop_ms = s->pcg_loop_ms;
  }
  return FSIM_OK;
}

}  // namespace fsim
