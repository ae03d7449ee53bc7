// k_g2p.cu -- grid-to-particle FLIP/PIC blend.
//
// Restates FlipSimulation::UpdateParticlesFromGrid (common/flip_simulation.cc:
// 1025-1091), InterpolateComponent<D> (:1095-1166) and
// UpdateSingleParticleFromGrid (:1179-1189).  One CTA per particle leaf
// stages the 10^3 node halo of the velocity and of the velocity update in
// shared memory (the reference copies the same halo per leaf).  The two
// VectorGrid::ExtrapolateToBoundary calls (common/vector_grid.cc:302-381)
// are applied while staging: a ghost-layer node reads its tangential
// components from the source node the six ordered passes would copy from.
// Each particle then interpolates v and dv (z, then y, then x lerps) and
// writes vel = v + flip*((dv + vel) - v) and grid_velocity = v.
#include "fsim_internal.cuh"

namespace fsim {

namespace {

struct G2PArgs {
  float* part;
  int64_t cap;
  const uint32_t* keys;
  const int32_t* leaf_id;
  const int32_t* nbr;
  const uint2* leaf_range;
  const float* vel;
  const float* vold;
  const uint32_t* vel_on;
  const uint32_t* vold_on;
  LeafMap lm;
  float flip;
};

__device__ __forceinline__ int side(int t) { return t < 0 ? -1 : (t > 7 ? 1 : 0); }

__device__ __forceinline__ float lerp_ref(float a, float b, float w) {
  return __fadd_rn(a, __fmul_rn(w, __fsub_rn(b, a)));
}

__global__ void __launch_bounds__(256) k_g2p(const __grid_constant__ G2PArgs a) {
  __shared__ float hv[3][1000];
  __shared__ float hd[3][1000];
  __shared__ int nb[27];
  const int s = blockIdx.x;
  const int tid = threadIdx.x;
  if (tid < 27) nb[tid] = a.nbr[int64_t(s) * 27 + tid];
  int lx, ly, lz;
  leaf_coords(a.lm, uint32_t(a.leaf_id[s]), lx, ly, lz);
  const int org[3] = {lx * 8, ly * 8, lz * 8};
  __syncthreads();
  const int* n = a.lm.n;
  for (int h = tid; h < 1000; h += 256) {
    const int c[3] = {org[0] - 1 + h / 100, org[1] - 1 + (h / 10) % 10, org[2] - 1 + h % 10};
#pragma unroll
    for (int D = 0; D < 3; ++D) {
      int src[3];
      ghost_source(n, D, c, src);
      const int ns = nb[(side(src[0] - org[0]) + 1) * 9 + (side(src[1] - org[1]) + 1) * 3 +
                        (side(src[2] - org[2]) + 1)];
      float v = 0.f, d = 0.f;
      if (ns >= 0) {
        const int sv = ((src[0] & 7) << 6) | ((src[1] & 7) << 3) | (src[2] & 7);
        const int64_t base = int64_t(ns) * 1536 + D * 512 + sv;
        if ((a.vel_on[int64_t(ns) * 16 + (sv >> 5)] >> (sv & 31)) & 1u) v = a.vel[base];
        if ((a.vold_on[int64_t(ns) * 16 + (sv >> 5)] >> (sv & 31)) & 1u) d = a.vold[base];
      }
      hv[D][h] = v;
      hd[D][h] = d;
    }
  }
  __syncthreads();
  const uint2 lr = a.leaf_range[s];
  const int64_t cap = a.cap;
  float* P = a.part;
  for (uint32_t q = lr.x + tid; q < lr.y; q += 256) {
    const uint32_t key = a.keys[q];
    if (key == kDeadKey) continue;
    const float p[3] = {P[q], P[cap + q], P[2 * cap + q]};
    // the cell the particle is binned in (as the reference's per-cell list)
    const int vx = int(key & 511u);
    const int cc[3] = {org[0] + (vx >> 6), org[1] + ((vx >> 3) & 7), org[2] + (vx & 7)};
    float pv[3] = {P[3 * cap + q], P[4 * cap + q], P[5 * cap + q]};
    float vi[3], di[3];
#pragma unroll
    for (int D = 0; D < 3; ++D) {
      float lo[3] = {float(cc[0]), float(cc[1]), float(cc[2])};
      int st[3] = {cc[0] - org[0] + 1, cc[1] - org[1] + 1, cc[2] - org[2] + 1};
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        if (ax == D) continue;
        lo[ax] = __fadd_rn(lo[ax], 0.5f);
        if (p[ax] < lo[ax]) { lo[ax] = __fsub_rn(lo[ax], 1.0f); st[ax] -= 1; }
      }
      const float w0 = __fsub_rn(p[0], lo[0]), w1 = __fsub_rn(p[1], lo[1]),
                  w2 = __fsub_rn(p[2], lo[2]);
      const int b = (st[0] * 10 + st[1]) * 10 + st[2];
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        const float* B = f == 0 ? hv[D] : hd[D];
        const float v000 = B[b], v001 = B[b + 1], v010 = B[b + 10], v011 = B[b + 11];
        const float v100 = B[b + 100], v101 = B[b + 101], v110 = B[b + 110], v111 = B[b + 111];
        const float v00 = lerp_ref(v000, v001, w2), v01 = lerp_ref(v010, v011, w2);
        const float v10 = lerp_ref(v100, v101, w2), v11 = lerp_ref(v110, v111, w2);
        const float v0 = lerp_ref(v00, v01, w1), v1 = lerp_ref(v10, v11, w1);
        const float r = lerp_ref(v0, v1, w0);
        if (f == 0) vi[D] = r; else di[D] = r;
      }
    }
#pragma unroll
    for (int D = 0; D < 3; ++D) {
      const float blend = __fmul_rn(a.flip, __fsub_rn(__fadd_rn(di[D], pv[D]), vi[D]));
      P[(3 + D) * cap + q] = __fadd_rn(vi[D], blend);
      P[(6 + D) * cap + q] = vi[D];
    }
  }
}

}  // namespace

int launch_g2p(fsim_sim* s) {
  G2PArgs a;
  a.part = s->part[s->cur];
  a.cap = s->cap_p;
  a.keys = s->keys[0];
  a.leaf_id = s->d_leaf_id;
  a.nbr = s->d_nbr;
  a.leaf_range = s->d_leaf_range;
  a.vel = s->vel;
  a.vold = s->vold;
  a.vel_on = s->vel_on;
  a.vold_on = s->vold_on;
  a.lm = s->lm;
  a.flip = s->cfg.flip_factor;
  FSIM_LAUNCH(s, "g2p", k_g2p, s->n_pleaf, 256, 0, a);
  return FSIM_OK;
}

}  // namespace fsim
